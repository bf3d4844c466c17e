"""Parity at the sizes the filter bank is measured on, through the C-ABI.

* The batched configuration (512^3, L = 300 Mpc/h, z = 7, 64 parameter sets
  with uneven radius counts, the benchmark's seeded boxes): the sets with the
  smallest, the median and the largest Rmax, from the 64-set device run
  (``sf21_hii_run_z_device``, CUDA graph) and from the host-buffer run
  (``sf21_hii_run_z``) of a context holding only those sets.  Both runs give
  the same bits; xHII is bit-identical with the oracle on every voxel whose
  outcome no decision within the tolerance band can change, the remaining
  voxels hold one of the two admissible values, and the first-hit radius lies
  within the FP64 bounds (get_HIIbubbles.c:298-471).
* The prologue at 512^3 on wide-range densities and sources: rec0, fresid
  and the single-cell fill bit-identical with the oracle, including the
  voxels that the fixed-point fast paths hand to the exact chains.
* The device entry point's CUDA graph: captured, replayed, updated across
  redshifts, input buffers and output buffers, and with the graph off or
  per-kernel timing on -- bit-identical with the host-buffer entry point.
* The plain GPU drop-in configuration (256^3, 20 redshifts from 12 to 6):
  every redshift against the oracle.

The oracle here is the CPU restatement's prologue (byte-identical to the
reference's build on the golden fixtures) with the FP64 bands computed by
``oracle/fp64_torch.py`` on the GPU (float64; the checker only).
"""
import numpy as np
import pytest
import torch

from bench import workload
from helpers import oracle_params
from oracle import fp64_torch as T
from simfast21_gb300 import params as P, synth

pytestmark = pytest.mark.gpu

TOL_BAND = 1e-5   # relative distance of h/d from 1 (the parity bar's tolerance band)


def _prologue(O, N, L, hubble, st, z, delta, sfrd):
    """rec0, ion0, fresid and the single-cell fill of one set from the CPU
    restatement (prologue only: no radius loop)."""
    fesc, Rmax, Nbins = st
    p = O.params(N, L, hubble, Rmax, Nbins, fesc, max_radii=-1)
    return O.run_z_sfr(p, z, delta, sfrd, extras=True)


def _check(x, ex, radii, dx, dk, rc=None):
    """x: device xHII box of one set.  Returns (band voxels, voxels that
    differ from the low bound, the certain-outcome mask on the host)."""
    b = T.Bands(ex["rec0"], ex["ion0"], dk).bands(radii, dx, tol=TOL_BAND)
    lo = T.finish(b["ionised_lo"], ex["fill0"], ex["fresid"])
    hi = T.finish(b["ionised_hi"], ex["fill0"], ex["fresid"])
    certain = b["ionised_lo"] == b["ionised_hi"]
    xi = x.view(torch.int32)
    assert torch.equal(xi[certain], lo.view(torch.int32)[certain])
    assert bool(((x == lo) | (x == hi)).all())
    if rc is not None:
        r = torch.from_numpy(rc).to(x.device)
        assert bool((b["rc_hi"] <= r).all()) and bool((r <= b["rc_lo"]).all())
    return int((~certain).sum().item()), int((x != lo).sum().item()), certain.cpu().numpy()


def test_batched512_sets_match_oracle(hii, oracle_lib):
    w = workload("batched512")
    N, L, z, h, sets = w["N"], w["L"], w["z"], w["hubble"], w["sets"]
    dx, dk = L / N, 2 * P.PI / L
    delta, sfrd = synth.make_boxes(synth.Workload(N=N, L=L, zs=[z], seed=w["seed"]), z)
    fb = hii.FilterBank(N, L, h, sets)
    d_delta = torch.from_numpy(delta).cuda()
    d_src = torch.from_numpy(sfrd).cuda()
    xs = torch.full((len(sets), N, N, N), float("nan"), dtype=torch.float32, device="cuda")
    fb.run_z_device(z, d_delta.data_ptr(), d_src.data_ptr(), xs.data_ptr())
    torch.cuda.synchronize()
    fb.check()
    order = np.argsort([s[1] for s in sets], kind="stable")
    pick = [int(order[0]), int(order[len(order) // 2]), int(order[-1])]
    sub = hii.FilterBank(N, L, h, [sets[i] for i in pick])
    xh, neutral = sub.run_z(z, delta, sfrd)
    sub.close()
    for j, s in enumerate(pick):
        radii, nf = fb.radii(s)
        assert torch.equal(xs[s].view(torch.int32), torch.from_numpy(xh[j]).cuda().view(torch.int32)), s
        ex = _prologue(oracle_lib, N, L, h, sets[s], z, delta, sfrd)
        rc = fb.first_hit(z, delta, sfrd, s)
        n_band, n_diff, _ = _check(xs[s], ex, radii, dx, dk, rc)
        x64 = xs[s].double()
        assert abs(neutral[j] - float((1.0 - x64).mean().item())) < 1e-9
        print(f"set {s}: zeta {sets[s][0]:.2f}, Rmax {sets[s][1]:.2f}, {len(radii)} radii ({nf} FFT), "
              f"band voxels {n_band}, differences from the low bound {n_diff}")
    fb.close()


@pytest.mark.parametrize("z", [7.0, 11.5])
def test_prologue_512_bit_exact_wide_inputs(hii, oracle_lib, z):
    """The prologue's fixed-point fast paths and their exact fallbacks
    (get_HIIbubbles.c:216-225, 272-274) on a 512^3 box of widely spread
    inputs. 1 + d is log-uniform over [2^-20, 2^20], plus the edge values
    d = -1, -1 + 2^-24 and 0. Sources are log-uniform over 60 binades, one
    in eight zero. The fast paths decline about one input in 2^21 (values
    within 2^-46 of a float rounding midpoint), so the box sends some tens
    of voxels per path through the exact soft-double chains (counted on the
    host for these inputs: Rrec 32 and 46, the residual-fraction product 27
    and 48, XHI's division 38 and 35, the source product 0 and 26 voxels at
    z = 7 and 11.5). rec0, fresid and the single-cell fill box must be
    bit-identical with the CPU restatement on every voxel."""
    w = workload("batched512")
    N, L, h = w["N"], w["L"], w["hubble"]
    n3 = N ** 3
    rng = np.random.default_rng(int(z * 10))
    one_d = np.exp2(rng.uniform(-20.0, 20.0, n3))
    delta = (one_d - 1.0).astype(np.float32)
    delta[:3] = [-1.0, np.float32(-1.0 + 2.0 ** -24), 0.0]
    sfrd = np.exp2(rng.uniform(-40.0, 20.0, n3)).astype(np.float32)
    sfrd[rng.random(n3) < 0.125] = 0.0
    delta, sfrd = delta.reshape((N,) * 3), sfrd.reshape((N,) * 3)
    st = w["sets"][0]
    fb = hii.FilterBank(N, L, h, [st])
    rec0, fres, fill0 = fb.prologue(z, delta, sfrd)
    fb.close()
    ex = _prologue(oracle_lib, N, L, h, st, z, delta, sfrd)
    for name, got, want in (("rec0", rec0, ex["rec0"]), ("fresid", fres, ex["fresid"]),
                            ("fill0", fill0, ex["fill0"])):
        g, wv = got.reshape(-1).view(np.uint32), np.asarray(want).reshape(-1).view(np.uint32)
        bad = np.flatnonzero(g != wv)
        assert bad.size == 0, (name, bad[:8], delta.reshape(-1)[bad[:8]], sfrd.reshape(-1)[bad[:8]])


def _two_inputs(N, L):
    w1 = synth.Workload(N=N, L=L, zs=[7.0], zeta=30.0, Rmax=L / 4, factor=1.05, seed=31)
    w2 = synth.Workload(N=N, L=L, zs=[8.5], zeta=30.0, Rmax=L / 4, factor=1.05, seed=32)
    return [(7.0,) + synth.make_boxes(w1, 7.0), (8.5,) + synth.make_boxes(w2, 8.5)]


def test_device_entry_graph_replay_and_update(hii):
    """run_z_device with its graph (capture, replay, cudaGraphExecUpdate when
    the redshift or a buffer changes), without it, and with per-kernel timing
    on: every call bit-identical with run_z on the same inputs."""
    N, L = 128, 80.0
    sets = [(15.0, 10.0, 30), (40.0, 20.0, 44), (90.0, 30.0, 52)]
    cases = _two_inputs(N, L)
    ref_bank = hii.FilterBank(N, L, 0.71, sets, graph=False)
    refs = [ref_bank.run_z(z, d, s)[0] for z, d, s in cases]
    ref_bank.close()
    dev = [(torch.from_numpy(d).cuda(), torch.from_numpy(s).cuda()) for _, d, s in cases]
    spare = (torch.empty_like(dev[0][0]), torch.empty_like(dev[0][1]))
    outs = [torch.empty((len(sets), N, N, N), dtype=torch.float32, device="cuda") for _ in range(2)]
    # (case, input buffers, output buffer): capture, replay, z + inputs change,
    # output changes, a copy of case 1's data in other buffers, back to the start
    calls = [(0, 0, 0), (0, 0, 0), (1, 1, 1), (1, 1, 0), (1, "spare", 1), (0, 0, 1), (0, 0, 0)]
    for mode in ("graph", "no_graph", "profiled"):
        fb = hii.FilterBank(N, L, 0.71, sets, graph=(mode != "no_graph"))
        if mode == "profiled":
            fb.profile(True)
        for case, inp, out in calls:
            z = cases[case][0]
            if inp == "spare":
                spare[0].copy_(dev[case][0])
                spare[1].copy_(dev[case][1])
                d, s = spare
            else:
                d, s = dev[inp]
            outs[out].fill_(float("nan"))
            torch.cuda.synchronize()
            fb.run_z_device(z, d.data_ptr(), s.data_ptr(), outs[out].data_ptr())
            torch.cuda.synchronize()
            got = outs[out].cpu().numpy()
            assert np.array_equal(got.view(np.uint32), refs[case].view(np.uint32)), (mode, case, inp, out)
        if mode == "profiled":
            prof = fb.profile_read()
            assert prof["inv_cols_a_test"][1] > 0
        fb.check()
        fb.close()


def test_device_entry_on_a_caller_stream(hii):
    """Enqueued on the caller's stream: the graph is captured for that stream
    and the result waits for nothing else."""
    N, L = 64, 50.0
    sets = [(30.0, 12.0, 30), (60.0, 20.0, 40)]
    (z, d, s), _ = _two_inputs(N, L)
    fb = hii.FilterBank(N, L, 0.71, sets)
    ref, _ = fb.run_z(z, d, s)
    st = torch.cuda.Stream()
    dd, ds = torch.from_numpy(d).cuda(), torch.from_numpy(s).cuda()
    out = torch.empty((len(sets), N, N, N), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    for _ in range(2):
        with torch.cuda.stream(st):
            out.fill_(float("nan"))
            fb.run_z_device(z, dd.data_ptr(), ds.data_ptr(), out.data_ptr(), stream=st.cuda_stream)
        st.synchronize()
        assert np.array_equal(out.cpu().numpy().view(np.uint32), ref.view(np.uint32))
    fb.close()


def test_xhii_256_every_redshift(hii, oracle_lib):
    """Plain GPU drop-in configuration: 256^3, L = 200 Mpc/h, zeta = 30, Rmax =
    60 Mpc/h, factor 1.05, density scaled by the linear growth factor over 20
    redshifts from 12 to 6.  Every redshift against the oracle outside the
    band (FP64 bands + restatement prologue); the first and the last also
    against the full CPU restatement of the radius loops."""
    zs = [12.0 - 6.0 * i / 19 for i in range(20)]
    w = synth.Workload(N=256, L=200.0, zs=zs, zeta=30.0, Rmax=60.0, factor=1.05, seed=1236, z_ref=8.0)
    sp = P.StageParams(nthreads=16, zmin=6.0, zmax=12.0, dz=6.0 / 19, L=200.0, hubble=0.71, N_halo=256, N=256,
                       fesc=30.0, xHlim=0.999, Rmax=60.0, Nbins=w.Nbins, use_sfr=True)
    fb = hii.FilterBank(sp.N, sp.L, sp.hubble, [(sp.fesc, sp.Rmax, sp.Nbins)])
    radii, _ = fb.radii()
    g_unit = synth.gaussian_field(w.N, w.seed)
    total_band = 0
    for i, z in enumerate(zs):
        delta, sfrd = synth.make_boxes(w, z, g_unit)
        x, nf = fb.run_z(z, delta, sfrd)
        ex = _prologue(oracle_lib, sp.N, sp.L, sp.hubble, (sp.fesc, sp.Rmax, sp.Nbins), z, delta, sfrd)
        n_band, n_diff, certain = _check(torch.from_numpy(x[0]).cuda(), ex, radii, sp.dx, sp.dk)
        total_band += n_band
        assert 0.0 <= nf[0] <= 1.0
        if i in (0, len(zs) - 1):
            ref = oracle_lib.run_z_sfr(oracle_params(oracle_lib, sp), z, delta, sfrd)["xhii"]
            n_ref = int((x[0] != ref).sum())
            assert np.array_equal(x[0][certain].view(np.uint32), ref[certain].view(np.uint32))
            print(f"z={z:.3f}: differences from the full restatement {n_ref}")
        print(f"z={z:.3f}: neutral {nf[0]:.6f}, band voxels {n_band}, differences from the low bound {n_diff}")
    fb.close()


def test_xhii_600_matches_oracle(hii, oracle_lib):
    """The reference's default side N_smoothed = 600 (the 2-3-5 transform
    family: shared-memory row passes and the register-resident 24 x 25
    column passes), one parameter set at L = 106.5 Mpc/h, z = 7: xHII
    bit-identical with the oracle outside the band, the first hit within the
    FP64 bounds."""
    N, L, z, h = 600, 106.5, 7.0, 0.71
    st = (30.0, 35.5, 109)
    delta, sfrd = synth.make_boxes(synth.Workload(N=N, L=L, zs=[z], seed=4242), z)
    fb = hii.FilterBank(N, L, h, [st])
    x, _ = fb.run_z(z, delta, sfrd)
    radii, nf = fb.radii()
    rc = fb.first_hit(z, delta, sfrd)
    ex = _prologue(oracle_lib, N, L, h, st, z, delta, sfrd)
    n_band, n_diff, _ = _check(torch.from_numpy(x[0]).cuda(), ex, radii, L / N, 2 * P.PI / L, rc)
    print(f"600^3: {len(radii)} radii ({nf} FFT), band voxels {n_band}, differences from the low bound {n_diff}")
    fb.close()
