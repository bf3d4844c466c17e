"""CPU restatement of the reference's 21-cm brightness-temperature stage
(TEST INFRASTRUCTURE ONLY: the checker of the GPU form and its timed CPU
baseline).  Follows t21.c:114-255 for one redshift, in double precision as
the reference computes it:
  * spin-temperature factor (:121-161): 1 when Lya/X-rays are off or z is
    below Zminsfr; else x = xc + xalpha, t = x / (1 + x), t *= 1 - Tcmb/TK,
    TS accumulates Tcmb / (1 - t);
  * line-of-sight velocity gradient (:163-209): FFT of the density, times
    k_axis^2 / k^2 (axis Vel_comp: 1 -> first index, 2 -> second, else the
    third; 0 at k = 0), inverse FFT, times -dg/dt / L^3 / H(z) dx^3 / D(z),
    clamped to [-0.5, 1];
  * T_b = 23e-3 (1 + delta) t / (1 + dv) (0.7/h) (Omega_b h^2 / 0.02)
    sqrt(0.15 / Omega_m / h^2 (1 + z) / 10) (1 - xHII) (:215-235);
  * its mean over the box (:243-246).
Growth, dg/dt and H(z) as auxiliary.c:224-291 (iterated sums in double).
Pinned against the reference's own t21.c output (tests/golden/t21_*.npz).
"""
from __future__ import annotations

import math

import numpy as np

H0 = 3.24078e-18      # h/sec, Input_variables.h:108
TCMB0 = 2.725         # K, t21.c:25
MAXCUT, MINCUT = 1.0, -0.5  # t21.c:26-27


class Cosmo:
    def __init__(self, omega_m, omega_b, omega_l, hubble):
        self.om, self.ob, self.ol, self.h = omega_m, omega_b, omega_l, hubble

    def Hz(self, z):  # auxiliary.c:224-226
        return self.h * H0 * math.sqrt(self.om * (1. + z) * (1. + z) * (1. + z) + self.ol)

    def int_growth(self, zz):  # auxiliary.c:243-257, the loop as written
        dz = 0.001
        intg = 0.
        hz0 = self.Hz(0.)
        z = zz + dz / 2.
        while z < zz + 100.:
            hub = self.Hz(z) / hz0
            intg += (1. + z) / hub / hub / hub
            z += dz
        return intg * dz

    def growth(self, z):  # auxiliary.c:262-266
        return self.Hz(z) / self.Hz(0) * self.int_growth(z) / self.int_growth(0.)

    def dgrowth_dt(self, z):  # auxiliary.c:285-291 with dzdt = -H(z)(1+z)
        dz = 1e-3
        return (self.growth(z + dz / 2.) - self.growth(z - dz / 2.)) / dz * (-self.Hz(z) * (1.0 + z))


def t21_box(z, delta, xhii, L, cosmo: Cosmo, vel_comp=3, xc=None, xalpha=None, tempx=None):
    """(T_b float32 box, mean T_b, mean TS or None) for one redshift; L in Mpc/h."""
    N = delta.shape[0]
    n3 = N ** 3
    dx = L / N
    dk = 2 * math.pi / L
    ts_mean = None
    if xc is not None:
        tcmb = TCMB0 * (1. + z)
        t = xc.astype(np.float64)
        xtot = xalpha.astype(np.float64) + t
        t = xtot / (1. + xtot)
        t = t * (1. - tcmb / tempx.astype(np.float64))
        ts_mean = float(np.sum(tcmb / (1. - t))) / n3
    else:
        t = np.ones(delta.shape)
    F = np.fft.rfftn(delta.astype(np.float64))
    i = np.arange(N)
    ind = np.where(i > N // 2, i - N, i).astype(np.float64)
    p = np.arange(N // 2 + 1).astype(np.float64)
    kk2 = (dk * np.sqrt(ind[:, None, None] ** 2 + ind[None, :, None] ** 2 + p[None, None, :] ** 2)) ** 2
    if vel_comp == 1:
        ka2 = (dk * ind[:, None, None]) ** 2 * np.ones_like(kk2)
    elif vel_comp == 2:
        ka2 = (dk * ind[None, :, None]) ** 2 * np.ones_like(kk2)
    else:
        ka2 = (dk * p[None, None, :]) ** 2 * np.ones_like(kk2)
    with np.errstate(invalid="ignore", divide="ignore"):
        g = np.where(kk2 > 0, ka2 / kk2, 0.0)
    dv = np.fft.irfftn(F * g, s=delta.shape, axes=(0, 1, 2)) * n3  # unnormalised c2r
    growth = cosmo.growth(z)
    dgdt = cosmo.dgrowth_dt(z)
    hubz = cosmo.Hz(z)
    dv = -dgdt * dv / L / L / L / hubz * dx * dx * dx / growth
    dv = np.where(dv > MAXCUT, MAXCUT, np.where(dv < MINCUT, MINCUT, dv))
    h = cosmo.h
    t = (23.0 / 1000. * (1. + delta.astype(np.float64)) * t / (1. + 1. * dv) * (0.7 / h) *
         (cosmo.ob * h * h / 0.02) * math.sqrt((0.15 / cosmo.om / h / h) * (1. + z) / 10.))
    t = t * (1. - xhii.astype(np.float64))
    return t.astype(np.float32), float(np.sum(t)) / n3, ts_mean
