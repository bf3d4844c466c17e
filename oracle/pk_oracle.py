"""CPU restatement of the reference's power-spectrum tool (TEST INFRASTRUCTURE
ONLY: the checker of the GPU power spectrum and its timed CPU baseline).

Follows tools/power3d_f.c step by step:
  * window per axis (wind(), :205-211): 1 (flag 0), Bartlett (1), Welch (2),
    the product of the three factors in double, left to right;
  * wsum = sum of the squared window (:121-128);
  * windowed box (float)(value * window) (:134-156);
  * r2c transform in single precision (:163-171, FFTW float);
  * k of each half-spectrum cell from the signed indices and the per-axis dk,
    bin round(k / dk) with dk the largest per-axis dk (:83-87, :174-188);
  * power (float) re^2 + im^2 summed per bin in double; P = sum / count /
    wsum * dl^3, empty bins count 1 (:190-194).
Pinned against the reference tool's own output on the golden fixtures
(tests/golden/pk_*.npz, tests/test_pk_oracle.py).
"""
from __future__ import annotations

import math

import numpy as np
import scipy.fft as sfft


def axis_window(n: int, flag: int) -> np.ndarray:
    x = np.arange(n, dtype=np.float64)
    m = float(n - 1)
    if flag == 1:
        return 1.0 - np.abs(x - m / 2.0) / m * 2.0
    if flag == 2:
        return 1.0 - ((x - m / 2.0) / m * 2.0) ** 2
    return np.ones(n)


def power_spectrum(box: np.ndarray, dl: float, flag: int = 0, workers: int = -1):
    """(k, P) as printed by power3d_f for a float32 box of shape (N1, N2, N3)."""
    n1, n2, n3 = box.shape
    w1, w2, w3 = (axis_window(n, flag) for n in (n1, n2, n3))
    w = (w1[:, None, None] * w2[None, :, None]) * w3[None, None, :]
    wsum = float(np.sum(w * w))
    mw = (box.astype(np.float64) * w).astype(np.float32)
    F = sfft.rfftn(mw, workers=workers)  # complex64
    dk1, dk2, dk3 = (2.0 * math.pi / (n * dl) for n in (n1, n2, n3))
    dk = max(dk1, dk2, dk3)
    nk = int(round(math.sqrt((n1 // 2) ** 2 + (n2 // 2) ** 2 + (n3 // 2) ** 2))) + 1
    i = np.arange(n1)
    j = np.arange(n2)
    p = np.arange(n3 // 2 + 1)
    ii = np.where(i > n1 // 2, i - n1, i).astype(np.float64)
    jj = np.where(j > n2 // 2, j - n2, j).astype(np.float64)
    k = np.sqrt((ii[:, None, None] * dk1) ** 2 + (jj[None, :, None] * dk2) ** 2 +
                (p[None, None, :] * dk3) ** 2)
    idx = np.floor(k / dk + 0.5).astype(np.int64).ravel()  # C round() for k >= 0
    re = F.real.astype(np.float32)
    im = F.imag.astype(np.float32)
    pw = (re * re + im * im).astype(np.float64).ravel()
    sums = np.bincount(idx, weights=pw, minlength=nk)[:nk]
    cnt = np.bincount(idx, minlength=nk)[:nk].astype(np.float64)
    cnt[cnt == 0] = 1.0
    P = sums / cnt / wsum * dl ** 3
    return np.arange(nk) * dk, P, wsum
