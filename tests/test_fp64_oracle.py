"""The exact dilation of the FP64 oracle against the reference algorithm."""
import numpy as np

from helpers import load_golden, oracle_params
from oracle import fp64_oracle as F
from simfast21_gb300 import params as P


def test_dilate_matches_brute_force():
    rng = np.random.default_rng(3)
    N = 12
    v = np.full((N, N, N), -1, np.int64)
    idx = rng.integers(0, N, size=(6, 3))
    vals = rng.integers(0, 30, size=6)
    for (a, b, c), val in zip(idx, vals):
        v[a, b, c] = val
    got = F.dilate(v)
    ax = np.arange(N)
    dmin = lambda u, w: np.minimum(np.abs(u - w), N - np.abs(u - w))
    want = np.zeros((N, N, N), bool)
    for (a, b, c), val in zip(idx, vals):
        n = dmin(ax, a)[:, None, None] ** 2 + dmin(ax, b)[None, :, None] ** 2 + dmin(ax, c)[None, None, :] ** 2
        want |= n <= val
    assert np.array_equal(got, want)


def test_exact_dilation_reproduces_reference(oracle_lib):
    """On every voxel whose outcome no near-threshold decision can change, the
    reference's FP32 FFT convolution and painting give the exact dilation."""
    O = oracle_lib
    g = load_golden("hii_n64_sfr.npz")
    sp = g["params"]
    p = oracle_params(O, sp)
    out = O.run_z_sfr(p, float(g["zs"][0]), g["delta_0"], g["sfrd_0"], extras=True)
    radii, _ = P.radii(sp.Rmax, sp.dx, sp.Nbins)
    b = F.bands(out["rec0"], out["ion0"], radii, sp.dx, sp.dk)
    lo = F.finish(b["ionised_lo"], out["fill0"], out["fresid"])
    hi = F.finish(b["ionised_hi"], out["fill0"], out["fresid"])
    x = g["xHII_0"]
    assert np.all((x == lo) | (x == hi))
    # uncertain outcomes come from centre decisions the FP32 rounding of any
    # transform can flip: h/d within 1e-5 of 1, or the sign of a filtered
    # field within 1e-6 of its max at the smallest radii (R < 1.5 dx), where
    # the top-hat ringing drives the filtered recombination rate below zero
    certain = b["ionised_lo"] == b["ionised_hi"]
    assert certain.mean() > 0.98


def test_nmax_definition():
    dx = 0.7
    for R in (0.7, 1.0, 1.39, 2.1, 7.77, 30.0):
        n = P.nmax(R, dx)
        assert np.sqrt(float(n)) * dx <= R and not (np.sqrt(float(n + 1)) * dx <= R)


def test_torch_bands_equal_numpy_bands(oracle_lib):
    """The torch form of the bands (run on the GPU at the measured box sizes)
    gives the numpy form's first-hit bounds, dilations and finished boxes, here
    on the CPU with torch's float64 FFT."""
    import torch
    from oracle import fp64_torch as T
    O = oracle_lib
    g = load_golden("hii_n32_sfr.npz")
    sp = g["params"]
    out = O.run_z_sfr(oracle_params(O, sp), float(g["zs"][0]), g["delta_0"], g["sfrd_0"], extras=True)
    radii, _ = P.radii(sp.Rmax, sp.dx, sp.Nbins)
    want = F.bands(out["rec0"], out["ion0"], radii, sp.dx, sp.dk)
    got = T.Bands(out["rec0"], out["ion0"], sp.dk, device="cpu").bands(radii, sp.dx)
    for k in ("rc_lo", "rc_hi", "ionised_lo", "ionised_hi"):
        assert np.array_equal(got[k].numpy(), want[k]), k
    assert got["n_band"] == want["n_band"]
    for k in ("ionised_lo", "ionised_hi"):
        x_np = F.finish(want[k], out["fill0"], out["fresid"])
        x_t = T.finish(got[k], out["fill0"], out["fresid"]).numpy()
        assert np.array_equal(x_np.view(np.uint32), x_t.view(np.uint32))
    v = torch.full((12, 12, 12), -1, dtype=torch.int32)
    v[1, 2, 3], v[7, 11, 0] = 9, 20
    assert np.array_equal(T.dilate(v).numpy(), F.dilate(v.numpy().astype(np.int64)))
