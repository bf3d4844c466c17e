"""ctypes front end of the CPU restatement (oracle/hii_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by bench.py's CPU-baseline leg, never by the product package.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libsf21oracle.so")
REF_EXE = os.path.join(HERE, "_ref", "get_HIIbubbles.x")
PK_EXE = os.path.join(HERE, "_ref", "power3d_f.x")  # tools/power3d_f.c, built by make ref
T21_EXE = os.path.join(HERE, "_ref", "t21.x")  # t21.c, built by make ref


class _Params(ctypes.Structure):
    _fields_ = [
        ("N", ctypes.c_long), ("N_halo", ctypes.c_long), ("L", ctypes.c_double),
        ("hubble", ctypes.c_double), ("Rmax", ctypes.c_double),
        ("Nbins", ctypes.c_int), ("fesc", ctypes.c_double),
        ("nthreads", ctypes.c_int), ("max_radii", ctypes.c_int),
    ]


def build() -> None:
    """Compile the restatement (make -C oracle)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        f = ctypes.c_void_p
        L.sf21o_run_z_sfr.argtypes = [ctypes.POINTER(_Params), ctypes.c_double, f, f, f, f, f, f, f,
                                      ctypes.POINTER(ctypes.c_double)]
        L.sf21o_run_z_rion.argtypes = [ctypes.POINTER(_Params), ctypes.c_double, f, f, f, f, f, f,
                                       ctypes.POINTER(ctypes.c_double)]
        L.sf21o_time_radii.argtypes = [ctypes.POINTER(_Params), ctypes.c_double, f, f, f, ctypes.c_int,
                                       ctypes.POINTER(ctypes.c_double), f]
        L.sf21o_filtered.argtypes = [ctypes.POINTER(_Params), f, f, ctypes.c_double, f, f]
        L.sf21o_halo_source.argtypes = [ctypes.POINTER(_Params), ctypes.c_double, ctypes.c_long, f, f]
        L.sf21o_halo_smoothed.argtypes = [ctypes.POINTER(_Params), ctypes.c_double, ctypes.c_long, f, f]
        L.sf21o_sfrd_box.argtypes = [ctypes.POINTER(_Params), ctypes.c_double, ctypes.c_long, f, f,
                                     ctypes.POINTER(ctypes.c_double)]
        L.sf21o_radii.argtypes = [ctypes.POINTER(_Params), ctypes.POINTER(ctypes.c_double),
                                  ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
        for fn in ("sf21o_Rrec", "sf21o_Rion"):
            getattr(L, fn).argtypes = [ctypes.c_float, ctypes.c_double, ctypes.POINTER(_Params)]
            getattr(L, fn).restype = ctypes.c_double
        for fn in ("sf21o_G_H", "sf21o_XHI", "sf21o_Qion", "sf21o_W_filter"):
            getattr(L, fn).argtypes = [ctypes.c_double]
            getattr(L, fn).restype = ctypes.c_double
        _lib = L
    return _lib


def params(N, L, hubble, Rmax, Nbins, fesc, nthreads=None, N_halo=None, max_radii=0):
    return _Params(N=N, N_halo=N_halo or N, L=L, hubble=hubble, Rmax=Rmax, Nbins=Nbins,
                   fesc=fesc, nthreads=nthreads or os.cpu_count() or 1, max_radii=max_radii)


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def run_z_sfr(p: _Params, z: float, delta: np.ndarray, sfrd: np.ndarray, extras: bool = False):
    """xHII (and optionally fresid, rec0, ion0, fill0) for one redshift."""
    N3 = p.N ** 3
    delta = np.ascontiguousarray(delta, dtype=np.float32)
    sfrd = np.ascontiguousarray(sfrd, dtype=np.float32)
    x = np.empty(N3, np.float32)
    ex = [np.empty(N3, np.float32) for _ in range(4)] if extras else [None] * 4
    neutral = ctypes.c_double(0.0)
    rc = lib().sf21o_run_z_sfr(ctypes.byref(p), z, _ptr(delta), _ptr(sfrd), _ptr(x),
                               *[_ptr(e) for e in ex], ctypes.byref(neutral))
    if rc:
        raise RuntimeError(f"oracle sf21o_run_z_sfr failed ({rc})")
    shp = (p.N,) * 3
    out = {"xhii": x.reshape(shp), "neutral": neutral.value}
    if extras:
        for k, e in zip(("fresid", "rec0", "ion0", "fill0"), ex):
            out[k] = e.reshape(shp)
    return out


def time_radii(p: _Params, z: float, delta: np.ndarray, sfrd: np.ndarray, ridx):
    """(front seconds, [seconds per listed radius index]) of the restatement:
    the prologue, fill and forward transforms once, then each radius's loop
    body on its own (the CPU-baseline sample)."""
    delta = np.ascontiguousarray(delta, dtype=np.float32)
    sfrd = np.ascontiguousarray(sfrd, dtype=np.float32)
    idx = np.ascontiguousarray(ridx, dtype=np.int32)
    t = np.zeros(len(idx), np.float64)
    front = ctypes.c_double(0.0)
    rc = lib().sf21o_time_radii(ctypes.byref(p), z, _ptr(delta), _ptr(sfrd), _ptr(idx), len(idx),
                                ctypes.byref(front), _ptr(t))
    if rc:
        raise RuntimeError(f"oracle sf21o_time_radii failed ({rc})")
    return front.value, [float(v) for v in t]


def run_z_rion(p: _Params, z: float, delta: np.ndarray, rion_box: np.ndarray):
    N3 = p.N ** 3
    delta = np.ascontiguousarray(delta, dtype=np.float32)
    rion_box = np.ascontiguousarray(rion_box, dtype=np.float32)
    x = np.empty(N3, np.float32)
    neutral = ctypes.c_double(0.0)
    rc = lib().sf21o_run_z_rion(ctypes.byref(p), z, _ptr(delta), _ptr(rion_box), _ptr(x),
                                None, None, None, ctypes.byref(neutral))
    if rc:
        raise RuntimeError(f"oracle sf21o_run_z_rion failed ({rc})")
    return {"xhii": x.reshape((p.N,) * 3), "neutral": neutral.value}


def filtered(p: _Params, rec0: np.ndarray, ion0: np.ndarray, R: float):
    """The reference's FP32 filtered fields at radius R (unnormalised)."""
    N3 = p.N ** 3
    a = np.ascontiguousarray(rec0, dtype=np.float32)
    b = np.ascontiguousarray(ion0, dtype=np.float32)
    ro = np.empty(N3, np.float32)
    io = np.empty(N3, np.float32)
    if lib().sf21o_filtered(ctypes.byref(p), _ptr(a), _ptr(b), R, _ptr(ro), _ptr(io)):
        raise RuntimeError("oracle sf21o_filtered failed")
    return ro.reshape((p.N,) * 3), io.reshape((p.N,) * 3)


def halo_source(p: _Params, z: float, cat: np.ndarray) -> np.ndarray:
    out = np.empty(p.N ** 3, np.float32)
    cat = np.ascontiguousarray(cat)
    rc = lib().sf21o_halo_source(ctypes.byref(p), z, len(cat), _ptr(cat), _ptr(out))
    if rc:
        raise RuntimeError(f"oracle sf21o_halo_source failed ({rc})")
    return out.reshape((p.N,) * 3)


def halo_smoothed(p: _Params, z: float, cat: np.ndarray) -> np.ndarray:
    """CIC + smooth_box of Rion(M, z) (get_HIIbubbles.c:233-253), before :258."""
    out = np.empty(p.N ** 3, np.float32)
    cat = np.ascontiguousarray(cat)
    rc = lib().sf21o_halo_smoothed(ctypes.byref(p), z, len(cat), _ptr(cat), _ptr(out))
    if rc:
        raise RuntimeError(f"oracle sf21o_halo_smoothed failed ({rc})")
    return out.reshape((p.N,) * 3)


def sfrd_box(p: _Params, z: float, cat: np.ndarray):
    """SFRD box and its average (get_SFR.c:104-146): p.N = N_smoothed,
    p.N_halo the catalogue's grid, p.L in Mpc/h."""
    out = np.empty(p.N ** 3, np.float32)
    cat = np.ascontiguousarray(cat)
    mean = ctypes.c_double(0.0)
    rc = lib().sf21o_sfrd_box(ctypes.byref(p), z, len(cat), _ptr(cat), _ptr(out), ctypes.byref(mean))
    if rc:
        raise RuntimeError(f"oracle sf21o_sfrd_box failed ({rc})")
    return out.reshape((p.N,) * 3), mean.value


def radii(p: _Params):
    buf = (ctypes.c_double * 512)()
    nf = ctypes.c_int(0)
    n = lib().sf21o_radii(ctypes.byref(p), buf, 512, ctypes.byref(nf))
    return [buf[i] for i in range(n)], nf.value
