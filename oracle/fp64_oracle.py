"""FP64 oracle of the HII filter bank (numpy).  TEST INFRASTRUCTURE ONLY.

Restates get_HIIbubbles.c:290-462 in float64 from the float32 prologue boxes
(the recombination-rate box rec0 of :222 and the ionisation-rate box ion0 of
:273): forward r2c, the top-hat filter W_filter (auxiliary.c:350-359) at
every radius, the unnormalised c2r (x N^3, like FFTW), and the centre test of
:339-348.  Instead of the reference's FP32 convolution / painting it applies
the exact integer dilation (every cell within the discrete ball of radius R,
min-image metric, of a centre at R) -- the set the reference's threshold at
:391-392 selects whenever its FP32 rounding stays below 0.01 of a count.

``bands`` classifies each (voxel, radius) decision by how far the criterion
is from its threshold: h/d within ``tol`` (relative) of 1, or a sign test on
a field value within ``field_tol`` of the field's max |value| of 0, makes
the decision uncertain and either answer is acceptable.  From the certain and the
possible centres it builds the lowest and highest first-hit radius index per
voxel and the dilations of both, which bound every FP32 realisation (GPU or
CPU) of the stage.
"""
from __future__ import annotations

import math

import numpy as np

from simfast21_gb300 import params as P

try:  # multi-threaded pocketfft when scipy is present
    import scipy.fft as _fft
    _KW = {"workers": -1}
except Exception:  # pragma: no cover
    _fft = np.fft
    _KW = {}


def w_filter(x: np.ndarray) -> np.ndarray:
    """auxiliary.c:350-359 in float64."""
    x = np.asarray(x, dtype=np.float64)
    out = np.empty_like(x)
    small = x < 0.03
    xs = x[small]
    out[small] = 3.0 * (1.0 / 3.0 - xs * xs * 1.0 / 30.0)
    xl = x[~small]
    out[~small] = 3.0 * (-(np.cos(xl) - (np.sin(xl) / xl)) / xl / xl)
    return out


def kmag(N: int, dk: float) -> np.ndarray:
    """dk * sqrt(indi^2 + indj^2 + p^2) on the r2c half grid (:308-317)."""
    f = np.fft.fftfreq(N) * N
    p = np.arange(N // 2 + 1, dtype=np.float64)
    n2 = f[:, None, None] ** 2 + f[None, :, None] ** 2 + p[None, None, :] ** 2
    return dk * np.sqrt(n2)


def filtered_fields(rec0, ion0, R: float, dk: float):
    """float64 (rec_R, ion_R), unnormalised like the reference's c2r."""
    N = rec0.shape[0]
    K = kmag(N, dk)
    W = w_filter(K * R)
    fr = _fft.rfftn(rec0.astype(np.float64), **_KW)
    fi = _fft.rfftn(ion0.astype(np.float64), **_KW)
    s = (N, N, N)
    n3 = float(N) ** 3
    return (_fft.irfftn(fr * W, s=s, axes=(0, 1, 2), **_KW) * n3,
            _fft.irfftn(fi * W, s=s, axes=(0, 1, 2), **_KW) * n3)


def dilate(v: np.ndarray) -> np.ndarray:
    """max over x of v(x) - n(x, y) (n = squared min-image lattice distance);
    v < 0 means no centre.  Returns the boolean 'ionised' box (>= 0)."""
    N = v.shape[0]
    vmax = int(v.max())
    if vmax < 0:
        return np.zeros(v.shape, bool)
    W = min(N // 2, int(math.isqrt(vmax)))
    cur = v.astype(np.int64)
    for ax in range(3):
        best = cur.copy()
        for d in range(1, W + 1):
            dd = d * d
            best = np.maximum(best, np.roll(cur, d, axis=ax) - dd)
            best = np.maximum(best, np.roll(cur, -d, axis=ax) - dd)
        cur = np.maximum(best, -1)
    return cur >= 0


def bands(rec0, ion0, radii, dx: float, dk: float, tol: float = 1e-5, field_tol: float = 1e-6,
          keep_fields: bool = False):
    """Certain / possible first-hit radius indices and dilations.

    A centre decision (h > 0 and (d <= 0 or h/d >= 1), :339-348) is evaluated
    over every realisation within the tolerances: h and d each within
    field_tol * max|field| of the float64 value (the FP32 rounding of any
    transform, the reference's FFTW one included), and the ratio h/d within
    tol (relative) of its threshold 1.  `certain` holds for all of them,
    `possible` for at least one.

    Returns dict with rc_lo (index of the first certain centre, 255 = none),
    rc_hi (first possible centre), ionised_lo, ionised_hi (bool boxes),
    n_band (number of (voxel, radius) decisions that are possible but not
    certain) and, if keep_fields, the float64 filtered fields per radius."""
    rc_lo = np.full(rec0.shape, 255, np.uint8)
    rc_hi = np.full(rec0.shape, 255, np.uint8)
    n_band = 0
    fields = []
    for i, R in enumerate(radii):
        d, h = filtered_fields(rec0, ion0, R, dk)
        if keep_fields:
            fields.append((d, h))
        eh = field_tol * float(np.abs(h).max())
        ed = field_tol * float(np.abs(d).max())
        possible = (h + eh > 0) & ((d - ed <= 0) | (h + eh >= (d - ed) * (1.0 - tol)))
        certain = (h - eh > 0) & ((d + ed <= 0) | (h - eh >= (d + ed) * (1.0 + tol)))
        n_band += int((possible & ~certain).sum())
        rc_lo[(rc_lo == 255) & certain] = i
        rc_hi[(rc_hi == 255) & possible] = i
    nmax = np.array([P.nmax(R, dx) for R in radii] + [-1], dtype=np.int64)
    v_lo = nmax[np.minimum(rc_lo.astype(np.int64), len(radii))]
    v_hi = nmax[np.minimum(rc_hi.astype(np.int64), len(radii))]
    out = {"rc_lo": rc_lo, "rc_hi": rc_hi, "ionised_lo": dilate(v_lo), "ionised_hi": dilate(v_hi),
           "n_band": n_band}
    if keep_fields:
        out["fields"] = fields
    return out


def finish(ionised: np.ndarray, fill0: np.ndarray, fresid: np.ndarray) -> np.ndarray:
    """xHII from a dilation: 1 inside bubbles, the single-cell fill elsewhere,
    capped by 1 - fresid in double (:466-471)."""
    x = np.where(ionised, np.float32(1.0), fill0).astype(np.float32)
    om = 1.0 - fresid.astype(np.float64)
    return np.where(x.astype(np.float64) > om, om.astype(np.float32), x).astype(np.float32)
