"""Host-side Python mirror of the HII stage over the C-ABI (include/sf21_hii.h).

``FilterBank`` wraps one sf21_hii context: construct it with the box and the
parameter sets (what get_HIIbubbles.c:98-194 sets up), then call ``run_z``
per redshift (the loop body, :215-477).  Arrays are numpy float32 boxes in C
order, or device pointers (``run_z_device``).  There is no CPU fallback:
without libsf21hii.so or without a GPU the calls raise.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libsf21hii.so")

SF21_SRC_SFRD = 0
SF21_SRC_RION = 1

_STATUS = {0: "SF21_OK", 1: "SF21_E_ARG", 2: "SF21_E_ALLOC", 3: "SF21_E_CUDA",
           4: "SF21_E_TIMEOUT", 5: "SF21_E_UNSUPPORTED"}

# Every entry point declared in include/sf21_hii.h.
EXPORTS = [
    "sf21_hii_create", "sf21_hii_destroy", "sf21_hii_last_error", "sf21_hii_run_z",
    "sf21_hii_run_z_device", "sf21_hii_radii", "sf21_hii_prologue", "sf21_hii_filtered",
    "sf21_hii_first_hit", "sf21_hii_run_z_plain_device", "sf21_hii_criterion", "sf21_hii_criterion_device",
    "sf21_hii_vjp", "sf21_hii_vjp_device", "sf21_hii_path", "sf21_hii_check", "sf21_hii_halo_source",
    "sf21_hii_run_z_halos", "sf21_hii_profile", "sf21_hii_profile_read", "sf21_hii_profile_name",
    "sf21_hii_halo_source_noalloc", "sf21_hii_power_spectrum", "sf21_hii_power_spectrum_device",
    "sf21_t21_run_z", "sf21_hii_set_wait_limit", "sf21_hii_inject_alloc_failure", "sf21_hii_batch_radii",
]


NPATH = 8  # radius pipelines (FilterBank.path)


class HIIError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{_STATUS.get(code, code)}: {msg}")
        self.code = code


class _Set(ctypes.Structure):
    _fields_ = [("fesc", ctypes.c_double), ("Rmax", ctypes.c_double), ("Nbins", ctypes.c_int)]


class T21Cosmo(ctypes.Structure):
    _fields_ = [("omega_m", ctypes.c_double), ("omega_b", ctypes.c_double), ("omega_lambda", ctypes.c_double),
                ("vel_comp", ctypes.c_int)]


class _Config(ctypes.Structure):
    _fields_ = [("N", ctypes.c_long), ("N_halo", ctypes.c_long), ("L", ctypes.c_double),
                ("hubble", ctypes.c_double), ("device", ctypes.c_int), ("nsets", ctypes.c_int),
                ("sets", ctypes.POINTER(_Set)), ("kmax", ctypes.c_int), ("path", ctypes.c_int),
                ("graph", ctypes.c_int)]


_lib = None


def load_library(path: str = LIB_PATH):
    """Load libsf21hii.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise OSError(f"{path} not found: build it with simfast21_gb300.build.build()")
    L = ctypes.CDLL(path)
    vp, dp, fp = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_void_p
    L.sf21_hii_create.argtypes = [ctypes.POINTER(_Config), ctypes.POINTER(ctypes.c_void_p)]
    L.sf21_hii_destroy.argtypes = [vp]
    L.sf21_hii_last_error.argtypes = [vp]
    L.sf21_hii_last_error.restype = ctypes.c_char_p
    L.sf21_hii_run_z.argtypes = [vp, ctypes.c_double, ctypes.c_int, fp, fp, fp, dp]
    L.sf21_hii_run_z_device.argtypes = [vp, ctypes.c_double, ctypes.c_int, vp, vp, vp, vp]
    L.sf21_hii_radii.argtypes = [vp, ctypes.c_int, dp, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
    L.sf21_hii_prologue.argtypes = [vp, ctypes.c_double, ctypes.c_int, fp, fp, ctypes.c_int, fp, fp, fp]
    L.sf21_hii_filtered.argtypes = [vp, ctypes.c_double, ctypes.c_int, fp, fp, ctypes.c_int,
                                    ctypes.c_int, fp, fp]
    L.sf21_hii_first_hit.argtypes = [vp, ctypes.c_double, ctypes.c_int, fp, fp, ctypes.c_int, fp]
    L.sf21_hii_run_z_plain_device.argtypes = [vp, ctypes.c_double, ctypes.c_int, vp, vp, ctypes.c_int, vp, vp]
    L.sf21_hii_criterion.argtypes = [vp, ctypes.c_double, ctypes.c_int, fp, fp, ctypes.c_int, fp, fp]
    L.sf21_hii_criterion_device.argtypes = [vp, ctypes.c_double, ctypes.c_int, vp, vp, ctypes.c_int, vp, vp, vp]
    L.sf21_hii_vjp.argtypes = [vp, ctypes.c_double, ctypes.c_int, fp, fp, ctypes.c_int, fp, fp, fp, dp]
    L.sf21_hii_vjp_device.argtypes = [vp, ctypes.c_double, ctypes.c_int, vp, vp, ctypes.c_int, vp, vp, vp, dp, vp]
    L.sf21_hii_path.argtypes = [vp, dp, ctypes.c_int]
    L.sf21_hii_halo_source.argtypes = [vp, ctypes.c_double, ctypes.c_long, vp, fp]
    L.sf21_hii_run_z_halos.argtypes = [vp, ctypes.c_double, fp, ctypes.c_long, vp, fp, dp]
    L.sf21_hii_halo_source_noalloc.argtypes = [ctypes.c_double, ctypes.c_long, ctypes.c_long, ctypes.c_long,
                                               vp, vp, vp]
    L.sf21_hii_power_spectrum.argtypes = [vp, fp, ctypes.c_int, ctypes.c_double, dp, dp, ctypes.c_int]
    L.sf21_hii_power_spectrum_device.argtypes = [vp, vp, ctypes.c_int, ctypes.c_double, dp, dp, ctypes.c_int, vp]
    L.sf21_t21_run_z.argtypes = [vp, ctypes.POINTER(T21Cosmo), ctypes.c_double, fp, fp, fp, fp, fp, fp, dp, dp]
    L.sf21_hii_check.argtypes = [vp]
    L.sf21_hii_set_wait_limit.argtypes = [vp, ctypes.c_uint]
    L.sf21_hii_inject_alloc_failure.argtypes = [ctypes.c_long]
    L.sf21_hii_batch_radii.argtypes = [vp]
    L.sf21_hii_profile.argtypes = [vp, ctypes.c_int]
    L.sf21_hii_profile_read.argtypes = [vp, dp, ctypes.POINTER(ctypes.c_long), ctypes.c_int]
    L.sf21_hii_profile_name.argtypes = [ctypes.c_int]
    L.sf21_hii_profile_name.restype = ctypes.c_char_p
    _lib = L
    return L


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def _f32(a, n3):
    a = np.ascontiguousarray(a, dtype=np.float32)
    if a.size != n3:
        raise ValueError(f"box has {a.size} elements, expected {n3}")
    return a


def inject_alloc_failure(n: int) -> None:
    """Test hook: the n-th device allocation of any context from now fails
    once (0 disarms)."""
    rc = load_library().sf21_hii_inject_alloc_failure(int(n))
    if rc != 0:
        raise HIIError(rc, "bad count")


def halo_source_noalloc(z: float, N_halo: int, N_smoothed: int, nhalos: int, halos_ptr: int, out_ptr: int,
                        stream: int = 0) -> None:
    """Halo source box with no device allocation (device pointers; enqueues on
    stream).  Limited to N_halo <= 128 and nhalos <= 16384."""
    L = load_library()
    rc = L.sf21_hii_halo_source_noalloc(z, N_halo, N_smoothed, nhalos, ctypes.c_void_p(halos_ptr or None),
                                        ctypes.c_void_p(out_ptr or None), ctypes.c_void_p(stream or None))
    if rc != 0:
        raise HIIError(rc, L.sf21_hii_last_error(None).decode())


@dataclass
class ParamSet:
    fesc: float
    Rmax: float  # Mpc/h, clamped to L/2 by the caller (Input_variables.c:124)
    Nbins: int


class FilterBank:
    """One GPU context for a box size and a list of parameter sets."""

    def __init__(self, N: int, L: float, hubble: float, sets, N_halo: int = 0, device: int = 0,
                 kmax: int = 0, path: int = 0, graph: bool = True):
        self._lib = load_library()
        self.N = int(N)
        self.n3 = self.N ** 3
        self.sets = [s if isinstance(s, ParamSet) else ParamSet(*s) for s in sets]
        arr = (_Set * len(self.sets))(*[_Set(s.fesc, s.Rmax, s.Nbins) for s in self.sets])
        self._arr = arr
        cfg = _Config(N=self.N, N_halo=N_halo or self.N, L=L, hubble=hubble, device=device,
                      nsets=len(self.sets), sets=arr, kmax=kmax, path=path, graph=0 if graph else -1)
        h = ctypes.c_void_p()
        rc = self._lib.sf21_hii_create(ctypes.byref(cfg), ctypes.byref(h))
        if rc != 0:
            raise HIIError(rc, self._lib.sf21_hii_last_error(None).decode())
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._lib.sf21_hii_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != 0:
            raise HIIError(rc, self._lib.sf21_hii_last_error(self._h).decode())

    def path(self):
        """(pipeline in use: 1 = three axis passes, 2 = plane clusters,
        3 = TMA-pipelined ky pass, 4 = TMA-pipelined ky and kx passes, and over
        column-block-major work boxes 5 = three axis passes, 6 = TMA ky pass,
        7 = TMA ky and kx passes, 8 = c-axis pass + one persistent ky/kx
        launch through L2; {pipeline: tuned ms of one batch})."""
        ms = (ctypes.c_double * NPATH)()
        p = self._lib.sf21_hii_path(self._h, ms, NPATH)
        return p, {i + 1: ms[i] for i in range(NPATH)}

    def batch_radii(self) -> int:
        """Radii per spectrum read (K) in use (fixed by kmax or tuned)."""
        return int(self._lib.sf21_hii_batch_radii(self._h))

    def check(self):
        """Raise if a bounded device wait expired since the last check."""
        self._check(self._lib.sf21_hii_check(self._h))

    def set_wait_limit(self, polls: int):
        """Polls per bounded device wait of the TMA-pipelined passes (0 =
        default); lowering it makes the waits run out on an ordinary launch."""
        self._check(self._lib.sf21_hii_set_wait_limit(self._h, int(polls)))

    def radii(self, s: int = 0):
        buf = (ctypes.c_double * 512)()
        nf = ctypes.c_int(0)
        n = self._lib.sf21_hii_radii(self._h, s, buf, 512, ctypes.byref(nf))
        if n < 0:
            raise HIIError(-n, "bad set index")
        return [buf[i] for i in range(n)], nf.value

    def run_z(self, z: float, delta, src, src_kind: int = SF21_SRC_SFRD, out=None):
        """xHII boxes (nsets, N, N, N) and neutral fractions (nsets,).  `out`:
        an optional C-contiguous float32 array of that shape to write into
        (e.g. pinned host memory)."""
        d = _f32(delta, self.n3)
        s = _f32(src, self.n3)
        shape = (len(self.sets), self.N, self.N, self.N)
        if out is None:
            out = np.empty(shape, np.float32)
        elif out.shape != shape or out.dtype != np.float32 or not out.flags["C_CONTIGUOUS"]:
            raise ValueError(f"out must be a C-contiguous float32 array of shape {shape}")
        neutral = (ctypes.c_double * len(self.sets))()
        self._check(self._lib.sf21_hii_run_z(self._h, z, src_kind, _ptr(d), _ptr(s), _ptr(out), neutral))
        return out, np.array(neutral[:], dtype=np.float64)

    def run_z_device(self, z: float, delta_ptr: int, src_ptr: int, xhii_ptr: int,
                     src_kind: int = SF21_SRC_SFRD, stream: int = 0):
        """Device-resident variant: raw device pointers (e.g. torch tensor
        .data_ptr()); enqueues on `stream` (0 = the context's own stream)."""
        self._check(self._lib.sf21_hii_run_z_device(self._h, z, src_kind, ctypes.c_void_p(delta_ptr),
                                                    ctypes.c_void_p(src_ptr), ctypes.c_void_p(xhii_ptr),
                                                    ctypes.c_void_p(stream or None)))

    def run_z_plain_device(self, z: float, delta_ptr: int, src_ptr: int, xhii_ptr: int, s: int = 0,
                           src_kind: int = SF21_SRC_SFRD, stream: int = 0):
        """Plain one-radius-per-launch form of set s (device pointers)."""
        self._check(self._lib.sf21_hii_run_z_plain_device(self._h, z, src_kind, ctypes.c_void_p(delta_ptr),
                                                          ctypes.c_void_p(src_ptr), s, ctypes.c_void_p(xhii_ptr),
                                                          ctypes.c_void_p(stream or None)))

    # ---- power spectrum (tools/power3d_f.c) ----------------------------------
    def power_spectrum(self, box, dl: float, flag: int = 0):
        """(k, P(k)) of an N^3 float box as tools/power3d_f.c computes it
        (flag: 0 top hat, 1 Bartlett, 2 Welch window)."""
        b = _f32(box, self.n3)
        cap = 2 * self.N
        k = (ctypes.c_double * cap)()
        P = (ctypes.c_double * cap)()
        n = self._lib.sf21_hii_power_spectrum(self._h, _ptr(b), flag, dl, k, P, cap)
        if n < 0:
            self._check(-n)
        return np.array(k[:n]), np.array(P[:n])

    def power_spectrum_device(self, box_ptr: int, dl: float, flag: int = 0, stream: int = 0):
        """The same for a device box (pointer); returns after the stream finished."""
        cap = 2 * self.N
        k = (ctypes.c_double * cap)()
        P = (ctypes.c_double * cap)()
        n = self._lib.sf21_hii_power_spectrum_device(self._h, ctypes.c_void_p(box_ptr), flag, dl, k, P, cap,
                                                     ctypes.c_void_p(stream or None))
        if n < 0:
            self._check(-n)
        return np.array(k[:n]), np.array(P[:n])

    # ---- 21-cm brightness temperature (t21.c) -------------------------------
    def t21(self, z: float, delta, xhii, omega_m=0.27, omega_b=0.046, omega_lambda=0.73, vel_comp=3,
            xc=None, xalpha=None, tempx=None):
        """(T_b box in K, mean T_b, mean TS or None) for one redshift; the spin
        boxes xc, xalpha, tempx all given (Lya/X-rays) or all None."""
        d = _f32(delta, self.n3)
        x = _f32(xhii, self.n3)
        spin = [None if a is None else _f32(a, self.n3) for a in (xc, xalpha, tempx)]
        out = np.empty((self.N,) * 3, np.float32)
        m_tb, m_ts = ctypes.c_double(0), ctypes.c_double(0)
        cosmo = T21Cosmo(omega_m, omega_b, omega_lambda, vel_comp)
        self._check(self._lib.sf21_t21_run_z(self._h, ctypes.byref(cosmo), z, _ptr(d), _ptr(x),
                                             *[_ptr(a) for a in spin], _ptr(out), ctypes.byref(m_tb),
                                             ctypes.byref(m_ts)))
        return out, m_tb.value, (m_ts.value if xc is not None else None)

    # ---- halo-catalogue source (use_SFR = F) ---------------------------------
    def halo_source(self, z: float, catalogue: np.ndarray) -> np.ndarray:
        """Rion box (CIC + smooth_box, before *(dx_s/dx_h)^3*fesc) from records
        with fields Mass, x, y, z (float32)."""
        cat = np.ascontiguousarray(catalogue)
        assert cat.dtype.itemsize == 16
        out = np.empty((self.N,) * 3, np.float32)
        self._check(self._lib.sf21_hii_halo_source(self._h, z, len(cat), cat.ctypes.data_as(ctypes.c_void_p),
                                                   _ptr(out)))
        return out

    def run_z_halos(self, z: float, delta, catalogue: np.ndarray):
        """xHII boxes and neutral fractions from a density box and a halo catalogue."""
        d = _f32(delta, self.n3)
        cat = np.ascontiguousarray(catalogue)
        out = np.empty((len(self.sets), self.N, self.N, self.N), np.float32)
        neutral = (ctypes.c_double * len(self.sets))()
        self._check(self._lib.sf21_hii_run_z_halos(self._h, z, _ptr(d), len(cat),
                                                   cat.ctypes.data_as(ctypes.c_void_p), _ptr(out), neutral))
        return out, np.array(neutral[:], dtype=np.float64)

    # ---- differentiable criterion -------------------------------------------
    def criterion(self, z: float, delta, src, s: int = 0, src_kind: int = SF21_SRC_SFRD):
        """(C, argmax) boxes of set s; the argmax is kept as the vjp checkpoint."""
        d = _f32(delta, self.n3)
        sr = _f32(src, self.n3)
        C = np.empty((self.N,) * 3, np.float32)
        A = np.empty((self.N,) * 3, np.uint8)
        self._check(self._lib.sf21_hii_criterion(self._h, z, src_kind, _ptr(d), _ptr(sr), s, _ptr(C), _ptr(A)))
        return C, A

    def vjp(self, z: float, delta, src, dC, s: int = 0, src_kind: int = SF21_SRC_SFRD):
        """(dL/d delta, dL/d src, dL/d fesc) for the cotangent dC = dL/dC."""
        d = _f32(delta, self.n3)
        sr = _f32(src, self.n3)
        g = _f32(dC, self.n3)
        gd = np.empty((self.N,) * 3, np.float32)
        gs = np.empty((self.N,) * 3, np.float32)
        gz = ctypes.c_double(0.0)
        self._check(self._lib.sf21_hii_vjp(self._h, z, src_kind, _ptr(d), _ptr(sr), s, _ptr(g), _ptr(gd),
                                           _ptr(gs), ctypes.byref(gz)))
        return gd, gs, gz.value

    def criterion_device(self, z, delta_ptr, src_ptr, C_ptr, A_ptr, s=0, src_kind=SF21_SRC_SFRD, stream=0):
        self._check(self._lib.sf21_hii_criterion_device(
            self._h, z, src_kind, ctypes.c_void_p(delta_ptr), ctypes.c_void_p(src_ptr), s,
            ctypes.c_void_p(C_ptr), ctypes.c_void_p(A_ptr), ctypes.c_void_p(stream or None)))

    def vjp_device(self, z, delta_ptr, src_ptr, dC_ptr, gd_ptr, gs_ptr, s=0, src_kind=SF21_SRC_SFRD, stream=0,
                   want_zeta=True):
        gz = ctypes.c_double(0.0)
        self._check(self._lib.sf21_hii_vjp_device(
            self._h, z, src_kind, ctypes.c_void_p(delta_ptr), ctypes.c_void_p(src_ptr), s,
            ctypes.c_void_p(dC_ptr), ctypes.c_void_p(gd_ptr or None), ctypes.c_void_p(gs_ptr or None),
            ctypes.byref(gz) if want_zeta else None, ctypes.c_void_p(stream or None)))
        return gz.value

    def prologue(self, z: float, delta, src, s: int = 0, src_kind: int = SF21_SRC_SFRD):
        d = _f32(delta, self.n3)
        sr = _f32(src, self.n3)
        shp = (self.N,) * 3
        rec0, fres, fill0 = (np.empty(shp, np.float32) for _ in range(3))
        self._check(self._lib.sf21_hii_prologue(self._h, z, src_kind, _ptr(d), _ptr(sr), s,
                                                _ptr(rec0), _ptr(fres), _ptr(fill0)))
        return rec0, fres, fill0

    def filtered(self, z: float, delta, src, ridx: int, s: int = 0, src_kind: int = SF21_SRC_SFRD):
        d = _f32(delta, self.n3)
        sr = _f32(src, self.n3)
        shp = (self.N,) * 3
        rec, ion = np.empty(shp, np.float32), np.empty(shp, np.float32)
        self._check(self._lib.sf21_hii_filtered(self._h, z, src_kind, _ptr(d), _ptr(sr), s, ridx,
                                                _ptr(rec), _ptr(ion)))
        return rec, ion

    def first_hit(self, z: float, delta, src, s: int = 0, src_kind: int = SF21_SRC_SFRD):
        d = _f32(delta, self.n3)
        sr = _f32(src, self.n3)
        rc = np.empty((self.N,) * 3, np.uint8)
        self._check(self._lib.sf21_hii_first_hit(self._h, z, src_kind, _ptr(d), _ptr(sr), s, _ptr(rc)))
        return rc

    # ---- measurement hooks -------------------------------------------------
    def profile(self, enable: bool = True):
        """Start (and reset) per-kernel CUDA-event timing on the launch stream."""
        self._check(self._lib.sf21_hii_profile(self._h, 1 if enable else 0))

    def profile_read(self):
        """{kernel kind: (total ms, launches)} since profile(True)."""
        ms = (ctypes.c_double * 32)()
        n = (ctypes.c_long * 32)()
        k = self._lib.sf21_hii_profile_read(self._h, ms, n, 32)
        if k < 0:
            self._check(-k)
        return {self._lib.sf21_hii_profile_name(i).decode(): (ms[i], n[i]) for i in range(k)}
