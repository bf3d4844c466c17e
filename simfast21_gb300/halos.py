"""Host-side Python mirror of the halo finder over the C-ABI
(include/sf21_halos.h).

``HaloFinder`` wraps one sf21_halo context: construct it with the parameters
get_halos.c reads (simfast21.ini, Input_variables.c:46-134), give it the
z = 0 density box once (``set_density``, get_halos.c:127-138), then call
``find_z`` per redshift (the loop body, :178-379).  Catalogues are numpy
structured arrays with the reference's records (Halo_t: Mass, x, y, z as
float32) in the reference's order.  There is no CPU fallback: without
libsf21hii.so or without a GPU the calls raise.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import hii

HALO_DTYPE = np.dtype([("Mass", "<f4"), ("x", "<f4"), ("y", "<f4"), ("z", "<f4")])

# Every entry point declared in include/sf21_halos.h.
EXPORTS = [
    "sf21_halo_schedule", "sf21_halo_create", "sf21_halo_destroy", "sf21_halo_last_error",
    "sf21_halo_set_density", "sf21_halo_set_density_device", "sf21_halo_find_z", "sf21_halo_fetch",
    "sf21_halo_catalogue_device", "sf21_halo_counts", "sf21_halo_rng_get", "sf21_halo_rng_set",
    "sf21_halo_candidates", "sf21_halo_field",
]


class HaloConfig(ctypes.Structure):
    _fields_ = [("N_halo", ctypes.c_long), ("L", ctypes.c_double), ("hubble", ctypes.c_double),
                ("omega_m", ctypes.c_double), ("omega_b", ctypes.c_double), ("omega_lambda", ctypes.c_double),
                ("sigma8", ctypes.c_double), ("n_index", ctypes.c_double), ("delta_c", ctypes.c_double),
                ("STa", ctypes.c_double), ("STb", ctypes.c_double), ("STc", ctypes.c_double),
                ("halo_Mmin", ctypes.c_double), ("halo_dlm", ctypes.c_double), ("use_subgrid", ctypes.c_int),
                ("device", ctypes.c_int)]


class HaloMass(ctypes.Structure):
    _fields_ = [("M", ctypes.c_double), ("R", ctypes.c_double), ("dndm", ctypes.c_double),
                ("dcmz", ctypes.c_double), ("active", ctypes.c_int), ("nc", ctypes.c_int)]


_ready = False


def load_library():
    global _ready
    L = hii.load_library()
    if not _ready:
        vp = ctypes.c_void_p
        C = ctypes.POINTER(HaloConfig)
        L.sf21_halo_schedule.argtypes = [C, ctypes.c_double, ctypes.POINTER(HaloMass), ctypes.c_int]
        L.sf21_halo_create.argtypes = [C, ctypes.POINTER(vp)]
        L.sf21_halo_destroy.argtypes = [vp]
        L.sf21_halo_last_error.argtypes = [vp]
        L.sf21_halo_last_error.restype = ctypes.c_char_p
        L.sf21_halo_set_density.argtypes = [vp, vp]
        L.sf21_halo_set_density_device.argtypes = [vp, vp, vp]
        L.sf21_halo_find_z.argtypes = [vp, ctypes.c_double, ctypes.POINTER(ctypes.c_long)]
        L.sf21_halo_fetch.argtypes = [vp, vp, ctypes.c_long, ctypes.c_long]
        L.sf21_halo_catalogue_device.argtypes = [vp]
        L.sf21_halo_catalogue_device.restype = vp
        L.sf21_halo_counts.argtypes = [vp, ctypes.POINTER(ctypes.c_long), ctypes.c_int]
        L.sf21_halo_rng_get.argtypes = [vp, ctypes.POINTER(ctypes.c_uint32)]
        L.sf21_halo_rng_set.argtypes = [vp, ctypes.POINTER(ctypes.c_uint32)]
        L.sf21_halo_candidates.argtypes = [vp, ctypes.c_int, vp]
        L.sf21_halo_field.argtypes = [vp, ctypes.c_double, ctypes.c_int, vp]
        _ready = True
    return L


def parse_ini(text: str) -> dict:
    """key -> first token of the value, as Input_variables.c:38-43 reads it."""
    out = {}
    for line in text.splitlines():
        if not line or line[0] == "#" or "=" not in line:
            continue
        k, v = line.split("=", 1)
        toks = v.split()
        out[k.strip()] = toks[0] if toks else ""
    return out


def config_from_ini(ini: dict, device: int = 0) -> HaloConfig:
    h = float(ini["hubble"])
    return HaloConfig(N_halo=int(ini["N_halo"]), L=float(ini["sim_length"]) * h, hubble=h,
                      omega_m=float(ini["omega_matter"]), omega_b=float(ini["omega_baryon"]),
                      omega_lambda=float(ini["omega_lambda"]), sigma8=float(ini["sigma8"]),
                      n_index=float(ini["spectral_index"]), delta_c=float(ini["critical_overdensity"]),
                      STa=float(ini["STa"]), STb=float(ini["STb"]), STc=float(ini["STc"]),
                      halo_Mmin=float(ini["halo_Mmin"]), halo_dlm=float(ini["halo_dlm"]),
                      use_subgrid=1 if ini.get("Use_subgrid", "F") == "T" else 0, device=device)


def schedule(cfg: HaloConfig, z: float) -> list:
    L = load_library()
    buf = (HaloMass * 4096)()
    n = L.sf21_halo_schedule(ctypes.byref(cfg), z, buf, 4096)
    if n < 0:
        raise hii.HIIError(-n, L.sf21_halo_last_error(None).decode())
    return [dict(M=m.M, R=m.R, dndm=m.dndm, dcmz=m.dcmz, active=bool(m.active), nc=m.nc) for m in buf[:n]]


class HaloFinder:
    """One GPU halo-finder context (sf21_halo_create)."""

    def __init__(self, cfg: HaloConfig):
        self._L = load_library()
        self.cfg = cfg
        self.N = cfg.N_halo
        h = ctypes.c_void_p()
        rc = self._L.sf21_halo_create(ctypes.byref(cfg), ctypes.byref(h))
        if rc:
            raise hii.HIIError(rc, self._L.sf21_halo_last_error(None).decode())
        self._h = h

    def _check(self, rc: int):
        if rc:
            raise hii.HIIError(rc, self._L.sf21_halo_last_error(self._h).decode())

    def set_density(self, delta_z0: np.ndarray):
        d = np.ascontiguousarray(delta_z0, np.float32)
        if d.size != self.N ** 3:
            raise ValueError(f"density box must hold {self.N}^3 cells")
        self._check(self._L.sf21_halo_set_density(self._h, d.ctypes.data))

    def find_z(self, z: float) -> np.ndarray:
        n = ctypes.c_long(0)
        self._check(self._L.sf21_halo_find_z(self._h, z, ctypes.byref(n)))
        out = np.empty(n.value, HALO_DTYPE)
        if n.value:
            self._check(self._L.sf21_halo_fetch(self._h, out.ctypes.data, 0, n.value))
        return out

    def counts(self) -> np.ndarray:
        buf = (ctypes.c_long * 4100)()
        n = self._L.sf21_halo_counts(self._h, buf, 4100)
        return np.array(buf[:n], np.int64)

    def rng(self) -> np.ndarray:
        st = (ctypes.c_uint32 * 3)()
        self._check(self._L.sf21_halo_rng_get(self._h, st))
        return np.array(st[:], np.uint32)

    def set_rng(self, state=None):
        if state is None:
            self._check(self._L.sf21_halo_rng_set(self._h, None))
        else:
            st = (ctypes.c_uint32 * 3)(*[int(v) for v in state])
            self._check(self._L.sf21_halo_rng_set(self._h, st))

    def candidates(self, m: int) -> np.ndarray:
        out = np.empty(self.N ** 3 // 32, np.uint32)
        self._check(self._L.sf21_halo_candidates(self._h, m, out.ctypes.data))
        return out

    def field(self, z: float, m: int) -> np.ndarray:
        out = np.empty(self.N ** 3, np.float32)
        self._check(self._L.sf21_halo_field(self._h, z, m, out.ctypes.data))
        return out.reshape((self.N,) * 3)

    def close(self):
        if getattr(self, "_h", None):
            self._L.sf21_halo_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
