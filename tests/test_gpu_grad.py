"""The hand-written adjoint of the criterion C(x) = max_R ion_R / rec_R
against FP64 central finite differences (differentiation configuration:
256^3, L = 200 Mpc/h, z = 8, zeta = 30, Rmax = 60 Mpc/h, factor 1.05).

Loss = sum_x w(x) C(x) + sum_bins (P_C(k) - P_target(k))^2 with w ~ U[0,1]
(seeded) and P_target the binned power of a second seeded run's criterion
(bins as tools/power3d_f.c:182-186: round(|k|/dk) over the r2c half grid).
The gradient comes from the library's adjoint through the torch.autograd
wrapper; the finite differences are FP64 on the GPU (allowed only here and in
the FP64 oracle): the filtered fields of every radius are held in float64 and
a one-voxel perturbation of the density or source box moves them by the
perturbation times the filter's real-space kernel, rolled to that voxel --
exact for this linear step -- after which C and the loss are re-evaluated in
float64.  Voxels are taken away from argmax ties (the top two ratios at the
voxel differ by more than 2 %).
"""
import math

import numpy as np
import pytest

from simfast21_gb300 import params as P, synth

pytestmark = pytest.mark.gpu

N, L, Z, ZETA, RMAX, FACTOR = 256, 200.0, 8.0, 30.0, 60.0, 1.05
H_REL = 1e-3
NVOX = 1000


def _power(C, kbin, nbins):
    import torch
    Ck = torch.fft.rfftn(C)
    p = (Ck.real ** 2 + Ck.imag ** 2).reshape(-1)
    s = torch.zeros(nbins, dtype=p.dtype, device=p.device).index_add_(0, kbin, p)
    cnt = torch.zeros(nbins, dtype=p.dtype, device=p.device).index_add_(0, kbin, torch.ones_like(p))
    return s / cnt.clamp(min=1) / float(C.numel())


def _bins(device):
    import torch
    f = torch.fft.fftfreq(N, d=1.0 / N, device=device, dtype=torch.float64)
    h = torch.arange(N // 2 + 1, device=device, dtype=torch.float64)
    kk = torch.sqrt(f[:, None, None] ** 2 + f[None, :, None] ** 2 + h[None, None, :] ** 2)
    kb = torch.round(kk).long().reshape(-1)
    return kb, int(kb.max().item()) + 1


def _rrec64(od, z, hubble):
    """Rrec (user_functions.c:58-65) in float64 without the float rounding."""
    rec1 = 1.e-24 * 9.84815696 * (1.0 + z) ** 5.06773134
    rec2 = (od / 1.76105133) ** 0.81722878
    rec3 = (rec2 / (1. + rec2)) ** 4.
    dvv = (L * 3.0857e24 / N / hubble / (1. + z)) ** 3.0
    return rec1 * rec3 * dvv / 1.e45


@pytest.fixture(scope="module")
def setup(hii):
    import torch
    torch.manual_seed(0)
    w = synth.Workload(N=N, L=L, zs=[Z], zeta=ZETA, Rmax=RMAX, factor=FACTOR, seed=4321)
    delta, sfrd = synth.make_boxes(w, Z)
    w2 = synth.Workload(N=N, L=L, zs=[Z], zeta=ZETA, Rmax=RMAX, factor=FACTOR, seed=8765)
    delta2, sfrd2 = synth.make_boxes(w2, Z)
    fb = hii.FilterBank(N, L, 0.71, [(ZETA, RMAX, w.Nbins)])
    dev = torch.device("cuda")
    kbin, nb = _bins(dev)
    # target power from the second run
    C2, _ = fb.criterion(Z, delta2, sfrd2)
    Pt = _power(torch.from_numpy(C2).to(dev, torch.float64), kbin, nb)
    wts = torch.from_numpy(np.random.default_rng(99).random((N, N, N))).to(dev)
    return dict(fb=fb, delta=delta, sfrd=sfrd, kbin=kbin, nb=nb, Pt=Pt, wts=wts, w=w, dev=dev)


def _loss(C, S):
    P_ = _power(C, S["kbin"], S["nb"])
    return (S["wts"] * C).sum() + ((P_ - S["Pt"]) ** 2).sum()


def test_vjp_matches_fp64_finite_differences(setup, hii):
    import torch
    from simfast21_gb300.autograd import Criterion
    S = setup
    fb, dev = S["fb"], S["dev"]
    d = torch.from_numpy(S["delta"]).to(dev).contiguous()
    s = torch.from_numpy(S["sfrd"]).to(dev).contiguous()
    zeta_t = torch.tensor(ZETA, dtype=torch.float64, device=dev, requires_grad=True)
    d.requires_grad_(True)
    s.requires_grad_(True)
    C = Criterion.apply(d, s, zeta_t, fb, Z, 0)
    loss = _loss(C.double(), S)
    loss.backward()
    gd = d.grad.double()
    gs = s.grad.double()
    gz = float(zeta_t.grad)

    # ---- FP64 reference fields from the library's (bit-exact) prologue ----
    rec0, _, _ = fb.prologue(Z, S["delta"], S["sfrd"])
    sp_dx = L / N
    m = sp_dx ** 3 * synth.qion(Z)          # SFRD -> Rion multiplier (:273)
    h1 = (S["sfrd"].astype(np.float64) * m).astype(np.float32)
    radii, nf = P.radii(RMAX, sp_dx, S["w"].Nbins)
    radii = radii[:nf]  # the criterion runs over the FFT-branch radii (R >= 2 dx)
    dk = 2 * P.PI / L
    f = torch.fft.fftfreq(N, d=1.0 / N, device=dev, dtype=torch.float64)
    h = torch.arange(N // 2 + 1, device=dev, dtype=torch.float64)
    kmag = dk * torch.sqrt(f[:, None, None] ** 2 + f[None, :, None] ** 2 + h[None, None, :] ** 2)
    R0 = torch.fft.rfftn(torch.from_numpy(rec0).to(dev, torch.float64))
    H0 = torch.fft.rfftn(torch.from_numpy(h1).to(dev, torch.float64))
    n3 = float(N) ** 3
    recs, hs, ks = [], [], []
    for R in radii:
        x = kmag * R
        W = torch.where(x < 0.03, 1.0 - x * x / 10.0, 3.0 * (torch.sin(x) - x * torch.cos(x)) / x.clamp(min=1e-30) ** 3)
        recs.append(torch.fft.irfftn(R0 * W, s=(N, N, N)) * n3)
        hs.append(torch.fft.irfftn(H0 * W, s=(N, N, N)) * n3)
        ks.append(torch.fft.irfftn(W.to(torch.complex128), s=(N, N, N)) * n3)

    def crit(drec=None, dh=None, v=None):
        best = torch.full((N, N, N), -math.inf, dtype=torch.float64, device=dev)
        top2 = torch.full((N, N, N), -math.inf, dtype=torch.float64, device=dev)
        for i in range(len(radii)):
            r, hh = recs[i], hs[i]
            if v is not None:
                kr = torch.roll(ks[i], shifts=v, dims=(0, 1, 2))
                if drec:
                    r = r + drec * kr
                if dh:
                    hh = hh + dh * kr
            ratio = torch.where(r > 0, ZETA * hh / r, torch.full_like(r, -math.inf))
            top2 = torch.maximum(top2, torch.minimum(best, ratio))
            best = torch.maximum(best, ratio)
        Cx = torch.where(torch.isinf(best), torch.zeros_like(best), best)
        return Cx, top2

    C64, top2 = crit()
    # the FP32 criterion agrees with the FP64 one
    dC = (C64 - C.detach().double()).abs()
    print(f"criterion: max |C| {float(C64.abs().max()):.4g}, max |C32 - C64| {float(dC.max()):.3e}, "
          f"max relative {float((dC / C64.abs().clamp(min=1e-30)).max()):.3e}")
    assert float(dC.max()) <= 1e-4 * float(C64.abs().max())
    gap = ((C64 - top2) / C64.abs().clamp(min=1e-30)).cpu().numpy()
    rng = np.random.default_rng(7)
    cand = np.argwhere(gap > 0.02)
    picks = cand[rng.choice(len(cand), size=NVOX, replace=False)]
    rel_d, rel_s = [], []
    dflat, sflat = S["delta"], S["sfrd"]
    for (a, b, c) in picks:
        v = (int(a), int(b), int(c))
        # density: rec0 moves through Rrec(1 + delta)
        dv = float(dflat[a, b, c])
        hstep = H_REL * max(abs(dv), 1e-3)
        base = _rrec64(1.0 + dv, Z, 0.71)
        Lp = float(_loss(crit(drec=_rrec64(1.0 + dv + hstep, Z, 0.71) - base, v=v)[0], S))
        Lm = float(_loss(crit(drec=_rrec64(1.0 + dv - hstep, Z, 0.71) - base, v=v)[0], S))
        fd = (Lp - Lm) / (2 * hstep)
        rel_d.append((float(gd[v]), fd))
        # source: ion1 moves linearly with the SFRD cell
        sv = float(sflat[a, b, c])
        sstep = H_REL * max(abs(sv), float(np.abs(sflat).mean()))
        Lp = float(_loss(crit(dh=sstep * m, v=v)[0], S))
        Lm = float(_loss(crit(dh=-sstep * m, v=v)[0], S))
        rel_s.append((float(gs[v]), (Lp - Lm) / (2 * sstep)))
    # zeta: C is linear in zeta at fixed argmax
    Lp = float(_loss(C64 * (1 + H_REL), S))
    Lm = float(_loss(C64 * (1 - H_REL), S))
    fdz = (Lp - Lm) / (2 * H_REL * ZETA)

    def stats(pairs):
        g = np.array(pairs)
        scale = np.abs(g[:, 1]).max()
        err = np.abs(g[:, 0] - g[:, 1]) / (np.abs(g[:, 1]) + 1e-3 * scale)
        return np.median(err), np.quantile(err, 0.95), err.max()

    md, q95d, mxd = stats(rel_d)
    ms, q95s, mxs = stats(rel_s)
    print(f"delta: median {md:.2e} q95 {q95d:.2e} max {mxd:.2e}; src: median {ms:.2e} q95 {q95s:.2e} "
          f"max {mxs:.2e}; zeta adj {gz:.6e} fd {fdz:.6e}")
    assert md < 1e-3 and q95d < 2e-2
    assert ms < 1e-3 and q95s < 2e-2
    assert abs(gz - fdz) <= 1e-3 * abs(fdz)
