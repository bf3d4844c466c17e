"""Stage parameters with the reference's semantics (host side, Python mirror).

``read_ini`` follows get_Simfast21_params (Input_variables.c:16-141): one
``key = value`` per line, ``#`` lines and empty lines skipped, a line without
``=`` or without a value is an error, unknown keys are ignored.  ``derive``
applies the unit conversions of Input_variables.c:119-134.  ``radii`` and
``nmax`` give the radius list of get_HIIbubbles.c:192,298-461 and the
discrete-ball radius used by the sphere window (:366) and the painting
(:443-447), computed in double exactly as the reference does.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

PI = 3.1415926535897932385e0  # Input_variables.h:10


class IniError(ValueError):
    pass


def read_ini(path: str) -> dict:
    vals: dict = {}
    with open(path, "r") as f:
        for line in f:
            if not line or line[0] in "#\n":
                continue
            if "=" not in line:
                raise IniError(f"Wrong format! {line!r}")
            line = line.replace("=", " ", 1)
            parts = line.split()
            if len(parts) < 2:
                raise IniError(f"Wrong format! {line!r}")
            vals[parts[0]] = parts[1]
    return vals


def _atof(s: str) -> float:
    """C atof: longest valid numeric prefix, 0.0 if none."""
    import re
    m = re.match(r"\s*[+-]?(\d+\.?\d*([eE][+-]?\d+)?|\.\d+([eE][+-]?\d+)?|inf|nan)", s, re.I)
    return float(m.group(0)) if m else 0.0


def _atoi(s: str) -> int:
    import re
    m = re.match(r"\s*[+-]?\d+", s)
    return int(m.group(0)) if m else 0


@dataclass
class StageParams:
    nthreads: int
    zmin: float
    zmax: float
    dz: float
    L: float  # Mpc/h (after *h)
    hubble: float
    N_halo: int
    N: int
    fesc: float
    xHlim: float
    Rmax: float  # Mpc/h (after *h and the L/2 clamp)
    Nbins: int
    use_sfr: bool

    @property
    def dx(self) -> float:
        return self.L / self.N

    @property
    def dx_halo(self) -> float:
        return self.L / self.N_halo

    @property
    def dk(self) -> float:
        return 2 * PI / self.L

    @property
    def L_file(self) -> float:
        """Box length in Mpc as written in file names (global_L/global_hubble)."""
        return self.L / self.hubble


def derive(v: dict) -> StageParams:
    h = _atof(v.get("hubble", "0"))
    L = _atof(v.get("sim_length", "0")) * h
    rmax = _atof(v.get("bubble_Rmax", "0")) * h
    if rmax > L / 2.0:
        rmax = L / 2.0
    zmax = _atof(v.get("zmax", "0"))
    dz = _atof(v.get("dz", "0"))
    zmin = _atof(v.get("zmin", "0"))
    zmin = zmax - dz * float(math.ceil((zmax - zmin) / dz))
    return StageParams(
        nthreads=_atoi(v.get("nthreads", "1")),
        zmin=zmin, zmax=zmax, dz=dz, L=L, hubble=h,
        N_halo=_atoi(v.get("N_halo", "0")), N=_atoi(v.get("N_smoothed", "0")),
        fesc=_atof(v.get("fesc", "0")), xHlim=_atof(v.get("Ion_cutoff", "0")),
        Rmax=rmax, Nbins=_atoi(v.get("bubble_Nbins", "0")),
        use_sfr=(v.get("use_SFR", "F") == "T"),
    )


def radius_ratio(Rmax: float, dx: float, Nbins: int) -> float:
    """bfactor, get_HIIbubbles.c:192."""
    return math.pow(10.0, math.log10(Rmax / dx) / Nbins)


def radii(Rmax: float, dx: float, Nbins: int):
    """(list of radii in loop order, number taking the FFT branch)."""
    b = radius_ratio(Rmax, dx, Nbins)
    out = []
    R = Rmax
    while R >= 2 * dx:
        out.append(R)
        R /= b
    nfft = len(out)
    while R >= dx:
        out.append(R)
        R /= b
    return out, nfft


def nmax(R: float, dx: float) -> int:
    """Largest integer n with sqrt((double)n)*dx <= R (the ball predicate of
    get_HIIbubbles.c:366 and :447 on the squared lattice distance)."""
    if R < 0:
        return -1
    n = int(math.floor((R / dx) ** 2))
    while n >= 0 and not (math.sqrt(float(n)) * dx <= R):
        n -= 1
    while math.sqrt(float(n + 1)) * dx <= R:
        n += 1
    return n
