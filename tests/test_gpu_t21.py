"""GPU 21-cm brightness temperature (sf21_t21_run_z, kernels_t21.cu) against
the reference's t21.c: its output boxes and printed means on the golden
fixtures, the oracle restatement (oracle/t21_oracle.py) on a 128^3 box for
each velocity axis, and the sf21_t21 drop-in on a base directory.  The GPU
computes in float, the reference in double: boxes agree within 1e-5 of the
box's max |T_b|, means within 1e-5 relative."""
import os
import subprocess

import numpy as np
import pytest

from helpers import GOLDEN
from oracle import t21_oracle as T
from simfast21_gb300 import synth

pytestmark = pytest.mark.gpu

TOL = 1e-5
COSMO = dict(omega_m=0.27, omega_b=0.046, omega_lambda=0.73)


def _bank(H, N, L):
    return H.FilterBank(N, L, 0.71, [(1.0, L / 4, 1)], kmax=1, path=1)


@pytest.mark.parametrize("name", ["t21_n32.npz", "t21_n32_lya.npz"])
def test_t21_matches_reference(hii, name):
    g = np.load(os.path.join(GOLDEN, name))
    N, L = g["delta_9"].shape[0], 25.0
    lya = bool(g["lya"])
    av = [float(x.split()[1]) for x in str(g["t21_av_txt"]).splitlines()]
    ts = [float(x.split()[1]) for x in str(g["TS_av_txt"]).splitlines()] if lya else []
    fb = _bank(hii, N, L)
    for n, z in enumerate((9.0, 8.0, 7.0)):
        spin = {}
        if lya and z > 8.0 - 0.1:
            spin = dict(xc=g[f"xc_{z:.0f}"], xalpha=g[f"xalpha_{z:.0f}"], tempx=g[f"tempx_{z:.0f}"])
        tb, m, tsm = fb.t21(z, g[f"delta_{z:.0f}"], g[f"xhii_{z:.0f}"], vel_comp=int(g["vel_comp"]), **COSMO, **spin)
        ref = g[f"tb_{z:.0f}"].reshape(tb.shape)
        assert np.abs(tb - ref).max() <= TOL * np.abs(ref).max()
        assert abs(m - av[n]) <= TOL * abs(av[n])
        if spin:
            assert abs(tsm - ts[n]) <= TOL * abs(ts[n])


@pytest.mark.parametrize("vel_comp,N", [(1, 128), (2, 128), (3, 128), (3, 120)])  # 120: radix-2/3/5 transforms
def test_t21_matches_oracle_128(hii, vel_comp, N):
    L, z = 100.0 * N / 128, 8.0
    delta = synth.lognormal_delta(synth.gaussian_field(N, 808), 0.8).astype(np.float32)
    xhii = np.clip(np.random.default_rng(9).random(delta.shape) * 1.6 - 0.3, 0, 1).astype(np.float32)
    fb = _bank(hii, N, L)
    tb, m, _ = fb.t21(z, delta, xhii, vel_comp=vel_comp, **COSMO)
    ref, mref, _ = T.t21_box(z, delta, xhii, L, T.Cosmo(0.27, 0.046, 0.73, 0.71), vel_comp)
    err = np.abs(tb - ref).max() / np.abs(ref).max()
    print(f"vel_comp {vel_comp}: max |dT_b| / max |T_b| = {err:.2e}")
    assert err <= TOL
    assert abs(m - mref) <= TOL * abs(mref)


def test_t21_drop_in_executable(hii, tmp_path):
    from simfast21_gb300 import build
    build.build()
    g = np.load(os.path.join(GOLDEN, "t21_n32_lya.npz"))
    base = str(tmp_path)
    N, Lmpc = 32, 25.0 / 0.71
    with open(os.path.join(base, "simfast21.ini"), "w") as f:
        f.write(str(g["ini"]))
    for d in ("delta", "Ionization", "Output_text_files", "x_c", "Lya", "xrays"):
        os.makedirs(os.path.join(base, d), exist_ok=True)
    for z in (9.0, 8.0, 7.0):
        tag = f"z{z:.3f}_N{N}_L{Lmpc:.1f}.dat"
        g[f"delta_{z:.0f}"].tofile(os.path.join(base, "delta", "deltanl_" + tag))
        g[f"xhii_{z:.0f}"].tofile(os.path.join(base, "Ionization", "xHII_" + tag))
        g[f"xc_{z:.0f}"].tofile(os.path.join(base, "x_c", "xc_" + tag))
        g[f"xalpha_{z:.0f}"].tofile(os.path.join(base, "Lya", "xalpha_" + tag))
        g[f"tempx_{z:.0f}"].tofile(os.path.join(base, "xrays", "TempX_" + tag))
    r = subprocess.run([build.T21_DRIVER, base], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    for z in (9.0, 8.0, 7.0):
        tag = f"z{z:.3f}_N{N}_L{Lmpc:.1f}.dat"
        ours = np.fromfile(os.path.join(base, "deltaTb", "deltaTb_" + tag), dtype=np.float32)
        ref = g[f"tb_{z:.0f}"]
        assert np.abs(ours - ref).max() <= TOL * np.abs(ref).max()
    for fn, key in ((f"t21_av_N{N}_L{Lmpc:.1f}.dat", "t21_av_txt"), (f"TS_av_N{N}_L{Lmpc:.1f}.dat", "TS_av_txt")):
        ours = open(os.path.join(base, "Output_text_files", fn)).read().splitlines()
        ref = str(g[key]).splitlines()
        assert len(ours) == len(ref)
        for a, b in zip(ours, ref):
            za, va = a.split()
            zb, vb = b.split()
            assert za == zb
            assert abs(float(va) - float(vb)) <= TOL * abs(float(vb))
    # a second run skips the existing boxes and appends nothing new
    r = subprocess.run([build.T21_DRIVER, base], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "already exists" in r.stdout
