"""Seeded synthetic input boxes in the reference's on-disk formats.

No public dataset is involved: the boxes stand in for the outputs of the
upstream SimFast21 stages (get_nldensity.x -> ``delta/deltanl_*``,
get_SFR.x -> ``SFR/sfrd_*``) with the shapes and value distributions the
HII stage sees.

* Density: g is a Gaussian random field with P(k) ~ k^-2 (zero mean, k=0
  removed) rescaled to standard deviation sigma per cell; the lognormal
  overdensity is delta = exp(g - sigma^2/2) - 1.
* Sources: each cell hosts one halo with probability ~ exp(1.5 delta),
  normalised to a mean occupancy of 2 %; halo masses follow dN/dM ~ M^-1.9
  on [1e8, 1e12] Msun (inverse CDF).  The SFRD box is the per-cell sum of
  sfr(M, z) = Rion(M, z)/Qion(z) divided by dx^3, i.e. get_SFR.c:119-131 with
  N_halo = N_smoothed (cloud-in-cell at integer positions deposits into one
  cell and smooth_box is the identity), scaled by SOURCE_SCALE.
* Redshift series: g_z = g D(z)/D(z_ref) with the reference's growth factor
  getGrowth (auxiliary.c:223-266), sigma_z scaled the same way.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np

try:  # multi-threaded FFTs for the large boxes when scipy is present
    import scipy.fft as _fft
    _FFT_KW = {"workers": -1}
except Exception:  # pragma: no cover
    _fft = np.fft
    _FFT_KW = {}

V_NORM = 1.0e45
# Star-formation normalisation of the synthetic SFRD boxes.  With 2 % one-halo
# occupancy the raw sfr(M, z) sum ionises the whole box for any zeta >= 3 at
# z = 8; scaling it by 1/50 makes zeta in [10, 100] span partially ionised
# boxes (about 15 % ionised at zeta = 10, 45 % at 30, 95 % at 100).
SOURCE_SCALE = 0.02


def rion(mass: np.ndarray, z: float) -> np.ndarray:
    """Ionisation rate of a halo, user_functions.c:40-47 (float mass input)."""
    m = np.asarray(mass, dtype=np.float32).astype(np.float64)
    c1, c2, c3, c4 = 1.575e39, 9.367608e07, 0.44, 2.27044695e00
    t1 = c1 * m * (1.0 + z) ** c4
    t2 = (m / c2) ** c3
    t3 = np.exp(-((c2 / m) ** 3.0))
    return t1 * t2 * t3 / V_NORM


def qion(z: float) -> float:
    """user_functions.c:84-88."""
    return 10.0 ** (2.05707274e-02 * z + 5.29944413e01) / V_NORM


def hubble_rate(z, omega_m=0.27, omega_l=0.73, h=0.71):
    """Hz, auxiliary.c:223-225 (units s^-1)."""
    H0 = 3.24078e-18
    return h * H0 * np.sqrt(omega_m * (1.0 + z) ** 3 + omega_l)


def growth(z: float, omega_m=0.27, omega_l=0.73, h=0.71) -> float:
    """Linear growth getGrowth(z) = H(z)/H(0) I(z)/I(0) with the midpoint sum
    I(z) = dz sum (1+z')/(H(z')/H0)^3 over z' in [z, z+100) (auxiliary.c:242-266)."""
    dz = 0.001

    def integral(zz):
        zs = zz + dz / 2.0 + dz * np.arange(int(round(100.0 / dz)))
        hz = hubble_rate(zs, omega_m, omega_l, h) / hubble_rate(0.0, omega_m, omega_l, h)
        return float(np.sum((1.0 + zs) / hz ** 3) * dz)

    return float(hubble_rate(z, omega_m, omega_l, h) / hubble_rate(0.0, omega_m, omega_l, h)
                 * integral(z) / integral(0.0))


def gaussian_field(N: int, seed: int, slope: float = -2.0) -> np.ndarray:
    """Unit-variance GRF on an N^3 periodic grid with P(k) ~ k^slope."""
    rng = np.random.default_rng(seed)
    white = rng.standard_normal((N, N, N))
    wk = _fft.rfftn(white, **_FFT_KW)
    del white
    k0 = np.fft.fftfreq(N) * N
    k2 = np.fft.rfftfreq(N) * N
    kk = k0[:, None, None] ** 2 + k0[None, :, None] ** 2 + k2[None, None, :] ** 2
    amp = np.zeros_like(kk)
    nz = kk > 0
    amp[nz] = kk[nz] ** (slope / 4.0)  # sqrt(P) = k^(slope/2)
    wk *= amp
    del amp
    g = _fft.irfftn(wk, s=(N, N, N), axes=(0, 1, 2), **_FFT_KW)
    g -= g.mean()
    g /= g.std()
    return g


def lognormal_delta(g_unit: np.ndarray, sigma: float) -> np.ndarray:
    g = sigma * g_unit
    return (np.exp(g - 0.5 * sigma * sigma) - 1.0).astype(np.float32)


def halo_masses(n: int, rng: np.random.Generator, m1=1e8, m2=1e12, slope=-1.9):
    a = slope + 1.0  # -0.9
    u = rng.random(n)
    lo, hi = m1 ** a, m2 ** a
    return (lo + u * (hi - lo)) ** (1.0 / a)


def host_probability(delta: np.ndarray, occupancy: float = 0.02) -> np.ndarray:
    """p = min(c exp(1.5 delta), 1) with c chosen (bisection on log c) so that
    mean(p) equals the target occupancy; the clip keeps the heavy lognormal
    tail from swallowing the normalisation.  Boxes above 2^21 cells solve for
    c on a fixed strided subsample."""
    w = np.exp(1.5 * delta.astype(np.float64))
    flat = w.ravel()
    sub = flat if flat.size <= (1 << 21) else flat[:: flat.size // (1 << 21)]
    lo, hi = -80.0, 80.0
    for _ in range(60):
        mid = 0.5 * (lo + hi)
        if np.minimum(np.exp(mid) * sub, 1.0).mean() < occupancy:
            lo = mid
        else:
            hi = mid
    w *= np.exp(0.5 * (lo + hi))
    np.minimum(w, 1.0, out=w)
    return w


def sfrd_box(delta: np.ndarray, z: float, L: float, seed: int,
             occupancy: float = 0.02) -> np.ndarray:
    """SFRD box [Msun/(Mpc/h)^3/yr] of one-halo-per-cell sources (get_SFR.c:119-131)."""
    N = delta.shape[0]
    rng = np.random.default_rng(seed)
    p = host_probability(delta, occupancy)
    host = rng.random(delta.shape) < p
    n = int(host.sum())
    mass = halo_masses(n, rng).astype(np.float32)
    sfr = rion(mass, z) / qion(z)
    dx = L / N
    box = np.zeros(delta.shape, dtype=np.float32)
    box[host] = (SOURCE_SCALE * sfr / dx ** 3).astype(np.float32)
    return box


def halo_catalogue(delta: np.ndarray, seed: int, occupancy: float = 0.02,
                   n_halo: int | None = None):
    """Halo catalogue (Halo_t {float Mass,x,y,z}, auxiliary.h:13-17) in units of
    fine cells of an n_halo^3 grid; positions are jittered inside the host cell."""
    N = delta.shape[0]
    nh = n_halo or N
    rng = np.random.default_rng(seed)
    p = host_probability(delta, occupancy)
    host = np.argwhere(rng.random(delta.shape) < p)
    mass = halo_masses(len(host), rng)
    scale = nh / N
    pos = (host + rng.random(host.shape)) * scale
    cat = np.zeros(len(host), dtype=[("Mass", "<f4"), ("x", "<f4"), ("y", "<f4"), ("z", "<f4")])
    cat["Mass"] = mass
    cat["x"], cat["y"], cat["z"] = pos[:, 0], pos[:, 1], pos[:, 2]
    return cat


@dataclass
class Workload:
    """One HII-stage workload: box, cosmology and bubble parameters."""

    N: int
    L: float  # Mpc/h
    zs: list
    zeta: float = 30.0
    Rmax: float = 50.0  # Mpc/h
    factor: float = 1.1
    hubble: float = 0.71
    seed: int = 1234
    sigma: float = 0.8
    z_ref: float = 8.0
    Nbins: int = field(default=0)

    def __post_init__(self):
        if not self.Nbins:
            dx = self.L / self.N
            rmax = min(self.Rmax, self.L / 2.0)
            self.Nbins = max(1, int(round(math.log(rmax / dx) / math.log(self.factor))))


def make_boxes(w: Workload, z: float, g_unit: np.ndarray | None = None):
    """(delta, sfrd) float32 boxes for redshift z."""
    if g_unit is None:
        g_unit = gaussian_field(w.N, w.seed)
    sig = w.sigma
    if abs(z - w.z_ref) > 1e-9:
        sig = w.sigma * growth(z) / growth(w.z_ref)
    delta = lognormal_delta(g_unit, sig)
    sfrd = sfrd_box(delta, z, w.L, w.seed + 7919 + int(round(z * 1000)))
    return delta, sfrd


def ini_text(w: Workload, zmin: float, zmax: float, dz: float, nthreads: int = 8,
             use_sfr: bool = True, n_halo: int | None = None) -> str:
    """simfast21.ini with the keys the HII stage reads (Input_variables.c:46-90).
    Lengths are written in Mpc (the file's units); the stage multiplies by h."""
    return "\n".join([
        "# synthetic workload for the HII-bubble stage",
        f"nthreads = {nthreads}",
        f"zmax = {zmax!r}",
        f"zmin = {zmin!r}",
        f"dz = {dz!r}",
        f"sim_length = {w.L / w.hubble!r}",
        f"N_halo = {n_halo or w.N}",
        f"N_smoothed = {w.N}",
        "omega_matter = 0.27",
        "omega_baryon = 0.046",
        "omega_lambda = 0.73",
        f"hubble = {w.hubble!r}",
        f"fesc = {w.zeta!r}",
        "Ion_cutoff = 0.999",
        f"bubble_Rmax = {w.Rmax / w.hubble!r}",
        f"bubble_Nbins = {w.Nbins}",
        f"use_SFR = {'T' if use_sfr else 'F'}",
        "",
    ])


def redshift_list(zmin: float, zmax: float, dz: float):
    """The redshifts the stage visits: zmin re-snapped as Input_variables.c:133,
    then repeated addition as get_HIIbubbles.c:206."""
    zmin = zmax - dz * float(math.ceil((zmax - zmin) / dz))
    zs = []
    z = zmin
    while z < zmax + dz / 10:
        zs.append(z)
        z += dz
    return zs


def box_name(kind: str, z: float, N: int, L_mpc: float) -> str:
    """File names of get_HIIbubbles.c:209,263,480 (%.3f, %ld, %.1f)."""
    sub = {"delta": "delta/deltanl", "sfrd": "SFR/sfrd", "xHII": "Ionization/xHII"}[kind]
    return f"{sub}_z{z:.3f}_N{N}_L{L_mpc:.1f}.dat"


def write_base_dir(base: str, w: Workload, zmin: float, zmax: float, dz: float,
                   nthreads: int = 8):
    """Write simfast21.ini plus delta/SFR boxes for every visited redshift.
    Returns the list of redshifts."""
    os.makedirs(os.path.join(base, "delta"), exist_ok=True)
    os.makedirs(os.path.join(base, "SFR"), exist_ok=True)
    with open(os.path.join(base, "simfast21.ini"), "w") as f:
        f.write(ini_text(w, zmin, zmax, dz, nthreads))
    L_file = (w.L / w.hubble) * w.hubble / w.hubble  # global_L/global_hubble
    g = gaussian_field(w.N, w.seed)
    zs = redshift_list(zmin, zmax, dz)
    for z in zs:
        delta, sfrd = make_boxes(w, z, g)
        delta.tofile(os.path.join(base, box_name("delta", z, w.N, L_file)))
        sfrd.tofile(os.path.join(base, box_name("sfrd", z, w.N, L_file)))
    return zs


def make_boxes_torch(N: int, L: float, z: float, seed: int, device="cuda", sigma: float = 0.8,
                     occupancy: float = 0.02):
    """The same generators on the GPU with torch (for large timing boxes, e.g.
    1024^3, where the numpy path would dominate the run): returns float32
    CUDA tensors (delta, sfrd).  Same distributions, not the same numbers as
    make_boxes."""
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    white = torch.randn((N, N, N), generator=g, device=device, dtype=torch.float32)
    wk = torch.fft.rfftn(white)
    del white
    f = torch.fft.fftfreq(N, d=1.0 / N, device=device)
    h = torch.arange(N // 2 + 1, device=device, dtype=torch.float32)
    kk = f[:, None, None] ** 2 + f[None, :, None] ** 2 + h[None, None, :] ** 2
    amp = torch.where(kk > 0, kk.clamp(min=1e-30) ** (-0.5), torch.zeros_like(kk))
    wk *= amp
    del amp, kk
    gr = torch.fft.irfftn(wk, s=(N, N, N))
    del wk
    gr -= gr.mean()
    gr /= gr.std()
    delta = torch.exp(sigma * gr - 0.5 * sigma * sigma) - 1.0
    del gr
    w = torch.exp(1.5 * delta.double().flatten()[:: max(1, N ** 3 // (1 << 21))])
    lo, hi = -80.0, 80.0
    for _ in range(60):
        mid = 0.5 * (lo + hi)
        if float(torch.clamp(math.exp(mid) * w, max=1.0).mean()) < occupancy:
            lo = mid
        else:
            hi = mid
    p = torch.clamp(math.exp(0.5 * (lo + hi)) * torch.exp(1.5 * delta), max=1.0)
    host = torch.rand((N, N, N), generator=g, device=device) < p
    del p
    n = int(host.sum())
    u = torch.rand(n, generator=g, device=device, dtype=torch.float64)
    a = -0.9
    m = (1e8 ** a + u * (1e12 ** a - 1e8 ** a)) ** (1.0 / a)
    m32 = m.float().double()
    c1, c2, c3, c4 = 1.575e39, 9.367608e07, 0.44, 2.27044695e00
    rion = c1 * m32 * (1.0 + z) ** c4 * (m32 / c2) ** c3 * torch.exp(-((c2 / m32) ** 3.0)) / V_NORM
    sfr = rion / qion(z)
    dx = L / N
    sfrd = torch.zeros((N, N, N), device=device, dtype=torch.float32)
    sfrd[host] = (SOURCE_SCALE * sfr / dx ** 3).float()
    return delta.float().contiguous(), sfrd


# ---- halo finder (get_halos.c) ---------------------------------------------
@dataclass
class HaloWorkload:
    """A base directory for the halo finder: a seeded Gaussian z = 0 linear
    density box (unit-variance field with P(k) ~ k^slope times sigma) and the
    simfast21.ini keys get_halos.c reads (Input_variables.c:46-90)."""
    N: int
    L_mpc: float          # sim_length (Mpc); the code works in Mpc/h = L_mpc * hubble
    sigma: float = 3.0    # rms of the z = 0 cell-scale density
    seed: int = 1
    hubble: float = 0.7
    subgrid: bool = False
    Mmin: float = 1e8
    dlm: float = 0.2
    slope: float = -2.0   # P(k) ~ k^slope of the Gaussian field
    smooth: int = 0       # > 0: the integer field of hash_field instead (that many box passes)

    def density(self) -> np.ndarray:
        if self.smooth > 0:
            return hash_field(self.N, self.seed, self.smooth, self.sigma)
        return (gaussian_field(self.N, self.seed, self.slope) * self.sigma).astype(np.float32)


def _splitmix64(x: np.ndarray) -> np.ndarray:
    z = x + np.uint64(0x9E3779B97F4A7C15)
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def hash_field(N: int, seed: int, passes: int, sigma: float) -> np.ndarray:
    """A density box that every machine reproduces bit for bit: integer white
    noise in [-512, 512) from the splitmix64 hash of (seed, cell), smoothed by
    `passes` rounds of the periodic 3-point box sum along each axis (integer
    arithmetic, |values| < 2^24), times the power of two that brings its rms
    closest to sigma (so the float32 values are exact).  Smoothing moves power
    to large scales, which gives the halo finder large spheres."""
    if passes > 3:
        raise ValueError("at most 3 smoothing passes keep the sums below 2^24")
    t = np.arange(N ** 3, dtype=np.uint64) + np.uint64(seed) * np.uint64(N ** 3)
    w = ((_splitmix64(t) >> np.uint64(54)).astype(np.int64) - 512).reshape(N, N, N)
    for _ in range(passes):
        for ax in range(3):
            w = w + np.roll(w, 1, ax) + np.roll(w, -1, ax)
    rms = float(np.sqrt(np.mean(w.astype(np.float64) ** 2)))
    k = int(round(math.log2(rms / sigma)))
    return (w.astype(np.float32) * np.float32(2.0 ** -k)).astype(np.float32)


def halo_ini_text(w: HaloWorkload, zmin: float, zmax: float, dz: float, nthreads: int = 8) -> str:
    return "\n".join([
        "# synthetic workload for the halo finder",
        f"nthreads = {nthreads}",
        f"zmax = {zmax!r}",
        f"zmin = {zmin!r}",
        f"dz = {dz!r}",
        f"sim_length = {w.L_mpc!r}",
        f"N_halo = {w.N}",
        f"N_smoothed = {max(w.N // 2, 16)}",
        "omega_matter = 0.27",
        "omega_baryon = 0.046",
        "omega_lambda = 0.73",
        f"hubble = {w.hubble!r}",
        "spectral_index = 0.96",
        "sigma8 = 0.81",
        "critical_overdensity = 1.68",
        "STa = 0.73",
        "STb = 0.34",
        "STc = 0.81",
        f"Use_subgrid = {'T' if w.subgrid else 'F'}",
        f"halo_Mmin = {w.Mmin!r}",
        f"halo_dlm = {w.dlm!r}",
        "",
    ])


def halo_density_name(N: int, L_mpc: float) -> str:
    """get_halos.c:128 (%ld, %.1f of L/h in Mpc)."""
    return f"delta/delta_z0_N{N}_L{L_mpc:.1f}.dat"


def halo_catalogue_name(z: float, N: int, L_mpc: float) -> str:
    """get_halos.c:173, 180 (%.3f, %ld, %.1f)."""
    return f"Halos/halo_z{z:.3f}_N{N}_L{L_mpc:.1f}.dat.catalog"


def halo_redshifts(zmin: float, zmax: float, dz: float):
    """The redshifts get_halos.c visits (:169): zmin re-snapped as
    Input_variables.c:133, then zmax downwards by repeated subtraction."""
    zmin = zmax - dz * float(math.ceil((zmax - zmin) / dz))
    zs = []
    z = zmax
    while z > zmin - dz / 10:
        zs.append(z)
        z -= dz
    return zs


def write_halo_base_dir(base: str, w: HaloWorkload, zmin: float, zmax: float, dz: float, nthreads: int = 8):
    os.makedirs(os.path.join(base, "delta"), exist_ok=True)
    with open(os.path.join(base, "simfast21.ini"), "w") as f:
        f.write(halo_ini_text(w, zmin, zmax, dz, nthreads))
    d = w.density()
    d.tofile(os.path.join(base, halo_density_name(w.N, w.L_mpc)))
    return d
