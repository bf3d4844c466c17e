"""ctypes front end of the halo-finder restatement (oracle/halo_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by bench.py's CPU-baseline leg, never by the product package.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import oracle as _o

HALO_EXE = os.path.join(_o.HERE, "_ref", "get_halos.x")  # get_halos.c, built by make ref
HALO_DTYPE = np.dtype([("Mass", "<f4"), ("x", "<f4"), ("y", "<f4"), ("z", "<f4")])


class HParams(ctypes.Structure):
    _fields_ = [
        ("N", ctypes.c_long), ("L", ctypes.c_double), ("hubble", ctypes.c_double),
        ("omega_m", ctypes.c_double), ("omega_b", ctypes.c_double), ("omega_l", ctypes.c_double),
        ("sig8", ctypes.c_double), ("n_index", ctypes.c_double), ("delta_c", ctypes.c_double),
        ("STa", ctypes.c_double), ("STb", ctypes.c_double), ("STc", ctypes.c_double),
        ("Mmin", ctypes.c_double), ("dlm", ctypes.c_double), ("use_sgrid", ctypes.c_int),
        ("nthreads", ctypes.c_int),
    ]


class HMass(ctypes.Structure):
    _fields_ = [("M", ctypes.c_double), ("R", ctypes.c_double), ("dndm", ctypes.c_double),
                ("dcmz", ctypes.c_double), ("active", ctypes.c_int)]


_done = False


def lib():
    global _done
    L = _o.lib()
    if not _done:
        P = ctypes.POINTER(HParams)
        d = ctypes.c_double
        vp = ctypes.c_void_p
        L.sf21o_halo_schedule.argtypes = [P, d, ctypes.POINTER(HMass), ctypes.c_int]
        L.sf21o_halo_field.argtypes = [P, d, vp, ctypes.c_int, vp]
        L.sf21o_halo_find_z.argtypes = [P, d, vp, vp, ctypes.c_long, ctypes.POINTER(ctypes.c_ulong), vp, vp]
        L.sf21o_halo_find_z.restype = ctypes.c_long
        L.sf21o_taus_seed.argtypes = [ctypes.c_ulong, ctypes.POINTER(ctypes.c_ulong)]
        for fn in ("sf21o_h_growth", "sf21o_h_sigma"):
            getattr(L, fn).argtypes = [P, d]
            getattr(L, fn).restype = d
        L.sf21o_h_mass_function.argtypes = [P, d, d]
        L.sf21o_h_mass_function.restype = d
        L.sf21o_h_bias.argtypes = [P, d, d]
        L.sf21o_h_bias.restype = d
        L.sf21o_qk15_nodes.argtypes = [ctypes.c_int]
        L.sf21o_qk15_nodes.restype = ctypes.POINTER(ctypes.c_double)
        _done = True
    return L


def params_from_ini(ini: dict, nthreads: int | None = None) -> HParams:
    """HParams from a parsed simfast21.ini (key -> string), as
    Input_variables.c:46-134 derives them."""
    h = float(ini["hubble"])
    return HParams(N=int(ini["N_halo"]), L=float(ini["sim_length"]) * h, hubble=h,
                   omega_m=float(ini["omega_matter"]), omega_b=float(ini["omega_baryon"]),
                   omega_l=float(ini["omega_lambda"]), sig8=float(ini["sigma8"]),
                   n_index=float(ini["spectral_index"]), delta_c=float(ini["critical_overdensity"]),
                   STa=float(ini["STa"]), STb=float(ini["STb"]), STc=float(ini["STc"]),
                   Mmin=float(ini["halo_Mmin"]), dlm=float(ini["halo_dlm"]),
                   use_sgrid=1 if ini.get("Use_subgrid", "F") == "T" else 0,
                   nthreads=nthreads or os.cpu_count() or 1)


def parse_ini(text: str) -> dict:
    out = {}
    for line in text.splitlines():
        if not line or line[0] in "#\n" or "=" not in line:
            continue
        k, v = line.split("=", 1)
        out[k.strip()] = v.split()[0] if v.split() else ""
    return out


def schedule(p: HParams, z: float):
    buf = (HMass * 256)()
    n = lib().sf21o_halo_schedule(ctypes.byref(p), z, buf, 256)
    return [dict(M=m.M, R=m.R, dndm=m.dndm, dcmz=m.dcmz, active=bool(m.active)) for m in buf[:min(n, 256)]]


def field(p: HParams, z: float, delta_z0: np.ndarray, m: int) -> np.ndarray:
    d = np.ascontiguousarray(delta_z0, np.float32)
    out = np.empty(p.N ** 3, np.float32)
    if lib().sf21o_halo_field(ctypes.byref(p), z, d.ctypes.data, m, out.ctypes.data):
        raise RuntimeError("oracle sf21o_halo_field failed")
    return out.reshape((p.N,) * 3)


def taus_seed(seed: int = 0) -> np.ndarray:
    st = (ctypes.c_ulong * 3)()
    lib().sf21o_taus_seed(seed, st)
    return np.array(st[:], np.uint64)


def find_z(p: HParams, z: float, delta_z0: np.ndarray, rng: np.ndarray | None = None, masks=None,
           cap: int | None = None):
    """(catalogue as a HALO_DTYPE array, per-mass counts, rng state after)."""
    d = np.ascontiguousarray(delta_z0, np.float32)
    st = (ctypes.c_ulong * 3)(*[int(v) for v in (taus_seed(0) if rng is None else rng)])
    nm = len(schedule(p, z))
    counts = np.zeros(nm + 1, np.int64)
    mptr = None
    keep = []
    if masks is not None:
        arr = (ctypes.c_void_p * nm)()
        for m in range(nm):
            if masks[m] is not None:
                a = np.ascontiguousarray(masks[m], np.uint32)
                keep.append(a)
                arr[m] = a.ctypes.data
        mptr = ctypes.cast(arr, ctypes.c_void_p)
        keep.append(arr)
    cap = cap if cap is not None else max(1 << 16, 8 * p.N ** 3)
    out = np.empty(cap, HALO_DTYPE)
    n = lib().sf21o_halo_find_z(ctypes.byref(p), z, d.ctypes.data, out.ctypes.data, cap, st, mptr,
                                counts.ctypes.data)
    if n < 0:
        raise RuntimeError(f"oracle sf21o_halo_find_z failed ({n})")
    if n > cap:
        raise RuntimeError(f"catalogue of {n} halos exceeds the buffer ({cap})")
    return out[:n].copy(), counts, np.array(st[:], np.uint64)


def read_catalogue(path: str) -> np.ndarray:
    """A get_halos.c catalogue file: int64 count, then {Mass, x, y, z} float32."""
    raw = open(path, "rb").read()
    n = int(np.frombuffer(raw[:8], np.int64)[0])
    cat = np.frombuffer(raw[8:], HALO_DTYPE)
    if len(cat) != n:
        raise ValueError(f"{path}: header says {n} halos, file holds {len(cat)}")
    return cat
