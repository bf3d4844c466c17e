"""Host-side Python mirror of the star-formation-rate stage over the C-ABI
(include/sf21_sfr.h).

``SFRBox`` wraps one sf21_sfr context: construct it with the grid sizes and
the box side get_SFR.c reads (N_halo, N_smoothed, L in Mpc/h), then call
``box(z, catalogue)`` per redshift (the loop body of get_SFR.c:104-146) for
the SFRD box in Msun/(Mpc/h)^3/yr and its average.  Catalogues are numpy
structured arrays of Halo_t records (``halos.HALO_DTYPE``).  There is no CPU
fallback: without libsf21hii.so or without a GPU the calls raise.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import hii
from .halos import HALO_DTYPE

# Every entry point declared in include/sf21_sfr.h.
EXPORTS = ["sf21_sfr_create", "sf21_sfr_destroy", "sf21_sfr_last_error", "sf21_sfr_box", "sf21_sfr_box_device"]


class SFRConfig(ctypes.Structure):
    _fields_ = [("N_halo", ctypes.c_long), ("N_smoothed", ctypes.c_long), ("L", ctypes.c_double),
                ("device", ctypes.c_int)]


_ready = False


def load_library():
    global _ready
    L = hii.load_library()
    if not _ready:
        vp = ctypes.c_void_p
        L.sf21_sfr_create.argtypes = [ctypes.POINTER(SFRConfig), ctypes.POINTER(vp)]
        L.sf21_sfr_destroy.argtypes = [vp]
        L.sf21_sfr_last_error.argtypes = [vp]
        L.sf21_sfr_last_error.restype = ctypes.c_char_p
        L.sf21_sfr_box.argtypes = [vp, ctypes.c_double, ctypes.c_long, vp, vp, ctypes.POINTER(ctypes.c_double)]
        L.sf21_sfr_box_device.argtypes = [vp, ctypes.c_double, ctypes.c_long, vp, vp, vp]
        _ready = True
    return L


class SFRBox:
    """One GPU star-formation-rate context (sf21_sfr_create)."""

    def __init__(self, N_halo: int, N_smoothed: int, L: float, device: int = 0):
        self._L = load_library()
        self.cfg = SFRConfig(N_halo, N_smoothed, L, device)
        self.N = N_smoothed
        h = ctypes.c_void_p()
        rc = self._L.sf21_sfr_create(ctypes.byref(self.cfg), ctypes.byref(h))
        if rc:
            raise hii.HIIError(rc, self._L.sf21_sfr_last_error(None).decode())
        self._h = h

    def _check(self, rc: int):
        if rc:
            raise hii.HIIError(rc, self._L.sf21_sfr_last_error(self._h).decode())

    def box(self, z: float, catalogue: np.ndarray):
        """(SFRD box N_smoothed^3 float32, its average as get_SFR.c:141-145)."""
        cat = np.ascontiguousarray(catalogue)
        if cat.dtype != HALO_DTYPE:
            cat = cat.astype(HALO_DTYPE)
        out = np.empty((self.N,) * 3, np.float32)
        mean = ctypes.c_double(0.0)
        self._check(self._L.sf21_sfr_box(self._h, z, len(cat), cat.ctypes.data if len(cat) else None,
                                         out.ctypes.data, ctypes.byref(mean)))
        return out, mean.value

    def box_device(self, z: float, nhalos: int, halos_dev: int, out_dev: int, stream: int = 0):
        """Device pointers in and out, enqueued on stream (no wait)."""
        self._check(self._L.sf21_sfr_box_device(self._h, z, nhalos, halos_dev or None, out_dev, stream or None))

    def close(self):
        if getattr(self, "_h", None):
            self._L.sf21_sfr_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
