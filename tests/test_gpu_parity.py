"""Parity of the CUDA library (through its C-ABI) with the oracle.

* prologue boxes bit-exact with the CPU restatement (which is byte-identical
  to the reference's own get_HIIbubbles.c on the golden fixtures);
* filtered fields within 1e-5 of the field's max |value| of the FP64 oracle;
* first-hit radius inside the FP64 oracle's certain/possible bounds;
* xHII bit-identical with the reference's output on every voxel whose outcome
  no centre decision within 1e-5 relative of the threshold can change; the
  remaining (band) voxels equal one of the two admissible outcomes.
"""
import numpy as np
import pytest

from helpers import load_golden, oracle_params
from oracle import fp64_oracle as F
from simfast21_gb300 import params as P, synth

pytestmark = pytest.mark.gpu

TOL_BAND = 1e-5   # relative distance of h/d from 1 (the parity bar's tolerance band)
TOL_FIELD = 1e-5  # filtered fields, relative to the field's max |value|


def _bank(H, sp, sets=None):
    sets = sets or [(sp.fesc, sp.Rmax, sp.Nbins)]
    return H.FilterBank(sp.N, sp.L, sp.hubble, sets, N_halo=sp.N_halo)


def _case(name):
    g = load_golden(name)
    return g, g["params"]


@pytest.mark.parametrize("name", ["hii_n32_sfr.npz", "hii_n64_sfr.npz", "hii_n40_sfr.npz"])
def test_prologue_bit_exact(hii, oracle_lib, name):
    g, sp = _case(name)
    fb = _bank(hii, sp)
    p = oracle_params(oracle_lib, sp)
    for i, z in enumerate(g["zs"]):
        rec0, fres, fill0 = fb.prologue(float(z), g[f"delta_{i}"], g[f"sfrd_{i}"])
        ref = oracle_lib.run_z_sfr(p, float(z), g[f"delta_{i}"], g[f"sfrd_{i}"], extras=True)
        for got, want in ((rec0, ref["rec0"]), (fres, ref["fresid"]), (fill0, ref["fill0"])):
            assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_filtered_fields_vs_fp64(hii, oracle_lib):
    g, sp = _case("hii_n64_sfr.npz")
    fb = _bank(hii, sp)
    z = float(g["zs"][0])
    ref = oracle_lib.run_z_sfr(oracle_params(oracle_lib, sp), z, g["delta_0"], g["sfrd_0"], extras=True)
    radii, nf = fb.radii()
    for ridx in sorted({0, nf // 2, nf - 1, nf, len(radii) - 1}):
        rec, ion = fb.filtered(z, g["delta_0"], g["sfrd_0"], ridx)
        d64, h64 = F.filtered_fields(ref["rec0"], ref["ion0"], radii[ridx], sp.dk)
        assert np.abs(rec - d64).max() <= TOL_FIELD * np.abs(d64).max()
        assert np.abs(ion - h64).max() <= TOL_FIELD * np.abs(h64).max()


def _bounds(oracle_lib, sp, z, delta, sfrd):
    ref = oracle_lib.run_z_sfr(oracle_params(oracle_lib, sp), z, delta, sfrd, extras=True)
    radii, _ = P.radii(sp.Rmax, sp.dx, sp.Nbins)
    b = F.bands(ref["rec0"], ref["ion0"], radii, sp.dx, sp.dk, tol=TOL_BAND)
    lo = F.finish(b["ionised_lo"], ref["fill0"], ref["fresid"])
    hi = F.finish(b["ionised_hi"], ref["fill0"], ref["fresid"])
    return ref, b, lo, hi


@pytest.mark.parametrize("name", ["hii_n32_sfr.npz", "hii_n64_sfr.npz", "hii_n40_sfr.npz"])
def test_xhii_matches_reference_outside_band(hii, oracle_lib, name):
    g, sp = _case(name)
    fb = _bank(hii, sp)
    xhi_ref = [float(v) for v in str(g["x_HI_txt"]).split()][::-1]
    for i, z in enumerate(g["zs"]):
        z = float(z)
        x, neutral = fb.run_z(z, g[f"delta_{i}"], g[f"sfrd_{i}"])
        x = x[0]
        ref_x = g[f"xHII_{i}"]
        _, b, lo, hi = _bounds(oracle_lib, sp, z, g[f"delta_{i}"], g[f"sfrd_{i}"])
        certain = b["ionised_lo"] == b["ionised_hi"]
        assert np.array_equal(x[certain].view(np.uint32), ref_x[certain].view(np.uint32))
        assert np.all((x == lo) | (x == hi))
        n_diff = int((x != ref_x).sum())
        assert n_diff <= int((~certain).sum())
        if n_diff == 0:
            assert "%f" % neutral[0] == "%f" % xhi_ref[i]


@pytest.mark.parametrize("name", ["hii_n32_sfr.npz", "hii_n64_sfr.npz", "hii_n40_sfr.npz"])
def test_first_hit_within_bounds(hii, oracle_lib, name):
    g, sp = _case(name)
    fb = _bank(hii, sp)
    z = float(g["zs"][0])
    rc = fb.first_hit(z, g["delta_0"], g["sfrd_0"])
    _, b, _, _ = _bounds(oracle_lib, sp, z, g["delta_0"], g["sfrd_0"])
    # possible centres come first: rc_hi <= rc <= rc_lo (255 = never)
    assert np.all(b["rc_hi"] <= rc) and np.all(rc <= b["rc_lo"])


def test_xhii_128_vs_cpu_restatement(hii, oracle_lib):
    """Plain-method box (128^3, L=100 Mpc/h, zeta=30, z=8, Rmax=50, factor 1.1)."""
    w = synth.Workload(N=128, L=100.0, zs=[8.0], zeta=30.0, Rmax=50.0, factor=1.1, seed=1235)
    delta, sfrd = synth.make_boxes(w, 8.0)
    sp = P.StageParams(nthreads=8, zmin=8.0, zmax=8.0, dz=1.0, L=100.0, hubble=0.71, N_halo=128, N=128,
                       fesc=30.0, xHlim=0.999, Rmax=50.0, Nbins=w.Nbins, use_sfr=True)
    fb = _bank(hii, sp)
    x, neutral = fb.run_z(8.0, delta, sfrd)
    ref, b, lo, hi = _bounds(oracle_lib, sp, 8.0, delta, sfrd)
    certain = b["ionised_lo"] == b["ionised_hi"]
    assert np.array_equal(x[0][certain].view(np.uint32), ref["xhii"][certain].view(np.uint32))
    assert np.all((x[0] == lo) | (x[0] == hi))


def test_parameter_sets_share_one_transform(hii):
    """A multi-set context gives each set exactly its single-set result."""
    w = synth.Workload(N=64, L=50.0, zs=[7.0], zeta=30.0, Rmax=25.0, factor=1.05, seed=9)
    delta, sfrd = synth.make_boxes(w, 7.0)
    sets = [(12.0, 10.0, 20), (30.0, 20.0, 33), (80.0, 25.0, 41)]
    fb = hii.FilterBank(64, 50.0, 0.71, sets)
    x_all, n_all = fb.run_z(7.0, delta, sfrd)
    for s, st in enumerate(sets):
        one = hii.FilterBank(64, 50.0, 0.71, [st])
        x1, n1 = one.run_z(7.0, delta, sfrd)
        assert np.array_equal(x_all[s].view(np.uint32), x1[0].view(np.uint32))
        assert n_all[s] == n1[0]


def test_halo_catalogue_branch(hii, oracle_lib):
    g, sp = _case("hii_n32_halo.npz")
    p = oracle_params(oracle_lib, sp)
    z = float(g["zs"][0])
    smoothed = oracle_lib.halo_smoothed(p, z, g["catalogue"])
    fb = _bank(hii, sp)
    x, _ = fb.run_z(z, g["delta_0"], smoothed, src_kind=hii.SF21_SRC_RION)
    ref_x = g["xHII_0"]
    rion = oracle_lib.halo_source(p, z, g["catalogue"])
    ref = oracle_lib.run_z_sfr  # noqa: F841  (kept for symmetry)
    o = oracle_lib.run_z_rion(p, z, g["delta_0"], rion)
    assert np.array_equal(o["xhii"].view(np.uint32), ref_x.view(np.uint32))
    # GPU vs reference outside the band
    radii, _ = P.radii(sp.Rmax, sp.dx, sp.Nbins)
    rec0, fres, fill0 = fb.prologue(z, g["delta_0"], smoothed, src_kind=hii.SF21_SRC_RION)
    b = F.bands(rec0, rion, radii, sp.dx, sp.dk, tol=TOL_BAND)
    certain = b["ionised_lo"] == b["ionised_hi"]
    assert np.array_equal(x[0][certain].view(np.uint32), ref_x[certain].view(np.uint32))


@pytest.mark.parametrize("name", ["hii_n64_sfr.npz", "hii_n40_sfr.npz"])
def test_plain_form_matches_reference(hii, oracle_lib, name):
    """The plain one-radius-per-launch form (reference structure: FP32 FFT
    convolution with the sphere, painting for R < 2 dx) through the C-ABI."""
    import torch
    g, sp = _case(name)
    fb = _bank(hii, sp)
    z = float(g["zs"][0])
    d = torch.from_numpy(g["delta_0"]).cuda()
    s = torch.from_numpy(g["sfrd_0"]).cuda()
    out = torch.empty_like(d)
    fb.run_z_plain_device(z, d.data_ptr(), s.data_ptr(), out.data_ptr())
    torch.cuda.synchronize()
    x = out.cpu().numpy()
    _, b, lo, hi = _bounds(oracle_lib, sp, z, g["delta_0"], g["sfrd_0"])
    certain = b["ionised_lo"] == b["ionised_hi"]
    assert np.array_equal(x[certain].view(np.uint32), g["xHII_0"][certain].view(np.uint32))
    assert np.all((x == lo) | (x == hi))


@pytest.mark.parametrize("N,L", [(64, 50.0), (128, 100.0), (256, 150.0)])
def test_radius_pipelines_agree(hii, N, L):
    """The radius pipelines -- three axis passes, the cluster plane pass
    (filter + kz + ky in distributed shared memory), the TMA-pipelined
    persistent strided passes, and the same over column-block-major work
    boxes -- run the same arithmetic: identical outputs."""
    w = synth.Workload(N=N, L=L, zs=[8.0], zeta=40.0, Rmax=L / 2, factor=1.1, seed=21)
    delta, sfrd = synth.make_boxes(w, 8.0)
    sets = [(40.0, L / 2, w.Nbins), (15.0, L / 5, 20)]
    paths = range(1, hii.NPATH + 1)
    banks = {p: hii.FilterBank(N, L, 0.71, sets, path=p) for p in paths}
    ref_x, ref_n = banks[1].run_z(8.0, delta, sfrd)
    for p in paths[1:]:
        assert banks[p].path()[0] == p
        x, n = banks[p].run_z(8.0, delta, sfrd)
        assert np.array_equal(ref_x.view(np.uint32), x.view(np.uint32)), p
        for s in range(len(sets)):
            assert np.array_equal(banks[1].first_hit(8.0, delta, sfrd, s), banks[p].first_hit(8.0, delta, sfrd, s))
    for p in paths:
        banks[p].check()


def test_halo_source_on_gpu_bit_exact(hii, oracle_lib):
    """CIC of Rion + smooth_box on the GPU equals the reference's serial loop
    (get_HIIbubbles.c:233-253) bit for bit; the end-to-end halo branch matches
    the reference's xHII outside the band."""
    g, sp = _case("hii_n32_halo.npz")
    p = oracle_params(oracle_lib, sp)
    z = float(g["zs"][0])
    fb = _bank(hii, sp)
    got = fb.halo_source(z, g["catalogue"])
    want = oracle_lib.halo_smoothed(p, z, g["catalogue"])
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    x, neutral = fb.run_z_halos(z, g["delta_0"], g["catalogue"])
    rion = oracle_lib.halo_source(p, z, g["catalogue"])
    rec0, _, _ = fb.prologue(z, g["delta_0"], want, src_kind=hii.SF21_SRC_RION)
    radii, _ = P.radii(sp.Rmax, sp.dx, sp.Nbins)
    b = F.bands(rec0, rion, radii, sp.dx, sp.dk, tol=TOL_BAND)
    certain = b["ionised_lo"] == b["ionised_hi"]
    assert np.array_equal(x[0][certain].view(np.uint32), g["xHII_0"][certain].view(np.uint32))


def test_halo_source_larger_catalogue(hii, oracle_lib):
    """64^3 box from a 128^3 CIC grid (smoothing factor 2), many halos per cell."""
    N, Nh, L = 64, 128, 50.0
    w = synth.Workload(N=N, L=L, zs=[7.5], zeta=0.5, Rmax=L / 2, factor=1.1, seed=55)
    g = synth.gaussian_field(N, 55)
    delta = synth.lognormal_delta(g, 0.8)
    cat = synth.halo_catalogue(delta, 56, occupancy=0.05, n_halo=Nh)
    p = oracle_lib.params(N, L, 0.71, L / 2, w.Nbins, 0.5, N_halo=Nh)
    fb = hii.FilterBank(N, L, 0.71, [(0.5, L / 2, w.Nbins)], N_halo=Nh)
    got = fb.halo_source(7.5, cat)
    want = oracle_lib.halo_smoothed(p, 7.5, cat)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_filtered_fields_cufft_crosscheck(hii, oracle_lib):
    """cuFFT as a cross-check only: at 256^3 the library's filtered fields and
    the same filter applied with cuFFT in complex64 are compared with the FP64
    fields; the library's error stays within the 1e-5 bound and within a small
    factor of cuFFT's own FP32 error."""
    import torch
    N, L, z = 256, 200.0, 8.0
    w = synth.Workload(N=N, L=L, zs=[z], zeta=30.0, Rmax=60.0, factor=1.05, seed=4321)
    delta, sfrd = synth.make_boxes(w, z)
    fb = hii.FilterBank(N, L, 0.71, [(30.0, 60.0, w.Nbins)])
    p = oracle_lib.params(N, L, 0.71, 60.0, w.Nbins, 30.0, max_radii=1)  # prologue + one radius
    ex = oracle_lib.run_z_sfr(p, z, delta, sfrd, extras=True)
    rec0, ion0 = ex["rec0"], ex["ion0"]
    radii, nf = fb.radii()
    dk = 2 * P.PI / L
    f = torch.fft.fftfreq(N, d=1.0 / N, device="cuda")
    h = torch.arange(N // 2 + 1, device="cuda", dtype=torch.float32)
    kmag = dk * torch.sqrt(f[:, None, None] ** 2 + f[None, :, None] ** 2 + h[None, None, :] ** 2)
    R0 = torch.fft.rfftn(torch.from_numpy(rec0).cuda())
    H0 = torch.fft.rfftn(torch.from_numpy(ion0).cuda())
    for ridx in (0, nf // 2, nf - 1):
        R = radii[ridx]
        rec, ion = fb.filtered(z, delta, sfrd, ridx)
        d64, h64 = F.filtered_fields(rec0, ion0, R, dk)
        x = (kmag * R).double()
        W = torch.where(x < 0.03, 1.0 - x * x / 10.0, 3.0 * (torch.sin(x) - x * torch.cos(x)) / x.clamp(min=1e-30) ** 3)
        W = W.float()
        rc = (torch.fft.irfftn(R0 * W, s=(N, N, N)) * N ** 3).cpu().numpy()
        hc = (torch.fft.irfftn(H0 * W, s=(N, N, N)) * N ** 3).cpu().numpy()
        for ours, cu, ref in ((rec, rc, d64), (ion, hc, h64)):
            scale = np.abs(ref).max()
            e_ours = np.abs(ours - ref).max() / scale
            e_cu = np.abs(cu - ref).max() / scale
            print(f"R={R:.3f}: library {e_ours:.2e}, cuFFT {e_cu:.2e} (of max |field|)")
            assert e_ours <= TOL_FIELD
            assert e_ours <= 4.0 * e_cu + 1e-7


@pytest.mark.parametrize("kind", ["no_sources", "saturated", "uniform_density"])
def test_edge_boxes(hii, oracle_lib, kind):
    """Degenerate inputs against the CPU restatement (byte-identical to the
    reference on the fixtures): no sources (no centre anywhere), sources so
    strong that every cell is a centre at the largest radius, and a uniform
    density box with sparse sources."""
    g, sp = _case("hii_n32_sfr.npz")
    z = float(g["zs"][0])
    delta = np.ascontiguousarray(g["delta_0"], np.float32)
    sfrd = np.ascontiguousarray(g["sfrd_0"], np.float32)
    if kind == "no_sources":
        sfrd = np.zeros_like(sfrd)
    elif kind == "saturated":
        sfrd = (sfrd + 1.0) * np.float32(1e3)
    else:
        delta = np.zeros_like(delta)
    fb = _bank(hii, sp)
    x, neutral = fb.run_z(z, delta, sfrd)
    _, b, lo, hi = _bounds(oracle_lib, sp, z, delta, sfrd)
    certain = b["ionised_lo"] == b["ionised_hi"]
    ref = oracle_lib.run_z_sfr(oracle_params(oracle_lib, sp), z, delta, sfrd)["xhii"]
    assert np.array_equal(x[0][certain].view(np.uint32), ref[certain].view(np.uint32))
    assert np.all((x[0] == lo) | (x[0] == hi))
    if kind == "no_sources":
        assert not np.any(x[0] == 1.0)
    if kind == "saturated":
        assert np.mean(x[0] > 0.5) > 0.99


def test_filtered_fields_600_vs_fp64(hii):
    """The reference's default N_smoothed = 600 (the shared-memory 2-3-5
    transforms with a compile-time plan): filtered fields at the largest and
    the smallest FFT-branch radius against float64 transforms of the same
    prologue outputs (rec0 from the library, bit-exact with the reference;
    ion0 = sfrd dx^3 Qion(z) fesc, get_HIIbubbles.c:273)."""
    N, L, h, z, fesc = 600, 106.5, 0.71, 7.0, 30.0
    w = synth.Workload(N=N, L=L, zs=[z], seed=4242)
    delta, sfrd = synth.make_boxes(w, z)
    fb = hii.FilterBank(N, L, h, [(fesc, 35.5, 109)])
    rec0, _, _ = fb.prologue(z, delta, sfrd)
    dx = L / N
    qion = 10.0 ** (2.05707274e-02 * z + 5.29944413e+01) / 1e45
    ion0 = sfrd.astype(np.float64) * dx * dx * dx * qion * fesc
    radii, nf = fb.radii()
    for ridx in (0, nf - 1):
        rec, ion = fb.filtered(z, delta, sfrd, ridx)
        d64, h64 = F.filtered_fields(rec0, ion0, radii[ridx], 2 * np.pi / L)
        e_rec = np.abs(rec - d64).max() / np.abs(d64).max()
        e_ion = np.abs(ion - h64).max() / np.abs(h64).max()
        print(f"600^3 R={radii[ridx]:.3f}: rec {e_rec:.2e}, ion {e_ion:.2e} (of max |field|)")
        assert e_rec <= TOL_FIELD and e_ion <= TOL_FIELD
    fb.close()
