"""FP64 tolerance bands of the HII filter bank in torch.  TEST INFRASTRUCTURE ONLY.

The same arithmetic as ``fp64_oracle.bands`` (float64 r2c of the prologue
boxes, the top-hat filter of auxiliary.c:350-359 at every radius, the
unnormalised c2r, the centre test of get_HIIbubbles.c:339-348 evaluated over
every realisation within the tolerances, exact integer dilation), written
with torch so that it runs on a CUDA device at the box sizes the filter bank
is measured on (512^3 and up), where numpy would take minutes per radius
set.  Float64 on the GPU is used here only, as the checker; the product path
computes in float32.  On the CPU (torch's float64 FFT) it reproduces
``fp64_oracle.bands`` exactly, which ``tests/test_fp64_oracle.py`` checks.
"""
from __future__ import annotations

import math

import numpy as np
import torch

from simfast21_gb300 import params as P


def w_filter(x: torch.Tensor) -> torch.Tensor:
    """auxiliary.c:350-359 in float64 (same expression order as the numpy form)."""
    small = x < 0.03
    xs = torch.where(small, torch.ones_like(x), x)
    big = 3.0 * (-(torch.cos(xs) - (torch.sin(xs) / xs)) / xs / xs)
    return torch.where(small, 3.0 * (1.0 / 3.0 - x * x * 1.0 / 30.0), big)


def kmag(N: int, dk: float, device) -> torch.Tensor:
    """dk * sqrt(indi^2 + indj^2 + p^2) on the r2c half grid (:308-317)."""
    f = torch.from_numpy(np.fft.fftfreq(N) * N).to(device)
    p = torch.arange(N // 2 + 1, dtype=torch.float64, device=device)
    n2 = f[:, None, None] ** 2 + f[None, :, None] ** 2 + p[None, None, :] ** 2
    return dk * torch.sqrt(n2)


def dilate(v: torch.Tensor) -> torch.Tensor:
    """max over x of v(x) - n(x, y) >= 0 (n = squared min-image lattice
    distance; v < 0: no centre), by three separable max-plus passes."""
    N = v.shape[0]
    vmax = int(v.max().item())
    if vmax < 0:
        return torch.zeros(v.shape, dtype=torch.bool, device=v.device)
    W = min(N // 2, math.isqrt(vmax))
    cur = v.to(torch.int32)
    for ax in range(3):
        best = cur.clone()
        for d in range(1, W + 1):
            dd = d * d
            torch.maximum(best, torch.roll(cur, d, dims=ax) - dd, out=best)
            torch.maximum(best, torch.roll(cur, -d, dims=ax) - dd, out=best)
        cur = torch.clamp_min(best, -1)
    return cur >= 0


class Bands:
    """Forward spectra of one (rec0, ion0) pair, kept on the device, and the
    bands of any radius list against them."""

    def __init__(self, rec0: np.ndarray, ion0: np.ndarray, dk: float, device="cuda"):
        self.N = rec0.shape[0]
        self.dev = torch.device(device)
        self.dk = dk
        self.fr = torch.fft.rfftn(torch.from_numpy(np.ascontiguousarray(rec0)).to(self.dev, torch.float64))
        self.fi = torch.fft.rfftn(torch.from_numpy(np.ascontiguousarray(ion0)).to(self.dev, torch.float64))
        self.k = kmag(self.N, dk, self.dev)

    def fields(self, R: float):
        """float64 (rec_R, ion_R), unnormalised like the reference's c2r."""
        N = self.N
        W = w_filter(self.k * R)
        n3 = float(N) ** 3
        d = torch.fft.irfftn(self.fr * W, s=(N, N, N)) * n3
        h = torch.fft.irfftn(self.fi * W, s=(N, N, N)) * n3
        return d, h

    def bands(self, radii, dx: float, tol: float = 1e-5, field_tol: float = 1e-6):
        """As fp64_oracle.bands: rc_lo / rc_hi (first certain / possible centre
        index, 255 = none), ionised_lo / ionised_hi (device bool boxes), n_band."""
        shape = (self.N,) * 3
        rc_lo = torch.full(shape, 255, dtype=torch.uint8, device=self.dev)
        rc_hi = torch.full(shape, 255, dtype=torch.uint8, device=self.dev)
        n_band = 0
        for i, R in enumerate(radii):
            d, h = self.fields(R)
            eh = field_tol * float(h.abs().max().item())
            ed = field_tol * float(d.abs().max().item())
            possible = (h + eh > 0) & ((d - ed <= 0) | (h + eh >= (d - ed) * (1.0 - tol)))
            certain = (h - eh > 0) & ((d + ed <= 0) | (h - eh >= (d + ed) * (1.0 + tol)))
            n_band += int((possible & ~certain).sum().item())
            rc_lo[(rc_lo == 255) & certain] = i
            rc_hi[(rc_hi == 255) & possible] = i
            del d, h, possible, certain
        nmax = torch.tensor([P.nmax(R, dx) for R in radii] + [-1], dtype=torch.int32, device=self.dev)
        n = len(radii)
        v_lo = nmax[torch.clamp_max(rc_lo.long(), n)]
        v_hi = nmax[torch.clamp_max(rc_hi.long(), n)]
        return {"rc_lo": rc_lo, "rc_hi": rc_hi, "ionised_lo": dilate(v_lo), "ionised_hi": dilate(v_hi),
                "n_band": n_band}


def finish(ionised: torch.Tensor, fill0: np.ndarray, fresid: np.ndarray) -> torch.Tensor:
    """xHII from a dilation (as fp64_oracle.finish): 1 inside bubbles, the
    single-cell fill elsewhere, capped by 1 - fresid in double (:466-471)."""
    dev = ionised.device
    f0 = torch.from_numpy(np.ascontiguousarray(fill0)).to(dev)
    x = torch.where(ionised, torch.ones_like(f0), f0)
    om = 1.0 - torch.from_numpy(np.ascontiguousarray(fresid)).to(dev).double()
    return torch.where(x.double() > om, om.float(), x)
