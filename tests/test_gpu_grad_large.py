"""The checkpointed backward at the large-box configuration: 1024^3, L = 500
Mpc/h, z = 7, zeta = 30, Rmax = 80 Mpc/h, radius factor 1.12, four radii per
spectrum read, seeded synthetic boxes.  The forward pass keeps only the
per-voxel argmax radius (uint8); the VJP recomputes the filtered fields.

* Filtered fields at the largest and the smallest FFT-branch radius within
  1e-5 of the field's max |value| of float64 transforms of the library's
  (bit-exact) prologue boxes.
* The criterion C(x) = max_R ion_R / rec_R against float64 on a 48^3 window.
* The VJP of the loss sum_{x in window} w(x) C(x) (w ~ U[0,1], seeded) with
  respect to density, source and zeta against float64 central finite
  differences (h = 1e-3 relative) at 100 voxels of the window away from
  argmax ties.  A one-voxel perturbation moves every radius's filtered fields
  by the step times the filter's real-space kernel centred on that voxel
  (exact for this linear step), so the finite differences need the float64
  fields on the window and the kernels on the window's offsets only.
* Device memory held during the forward and backward passes is reported.

Float64 on the GPU is used here only, as the checker.
"""
import math

import numpy as np
import pytest
import torch

from simfast21_gb300 import params as P, synth

pytestmark = pytest.mark.gpu

N, L, Z, ZETA, RMAX, FACTOR, SEED = 1024, 500.0, 7.0, 30.0, 80.0, 1.12, 5555
KMAX = 4
WIN = 48
W0 = (400, 600, 300)  # window corner
NVOX = 100
H_REL = 1e-3
TOL_FIELD = 1e-5


def _w_filter(x):
    small = x < 0.03
    xs = torch.where(small, torch.ones_like(x), x)
    big = 3.0 * (-(torch.cos(xs) - (torch.sin(xs) / xs)) / xs / xs)
    return torch.where(small, 3.0 * (1.0 / 3.0 - x * x / 30.0), big)


def _rrec64(od, hubble=0.71):
    """Rrec (user_functions.c:58-65) in float64 without the float rounding."""
    rec1 = 1.e-24 * 9.84815696 * (1.0 + Z) ** 5.06773134
    rec2 = (od / 1.76105133) ** 0.81722878
    rec3 = (rec2 / (1. + rec2)) ** 4.
    dvv = (L * 3.0857e24 / N / hubble / (1. + Z)) ** 3.0
    return rec1 * rec3 * dvv / 1.e45


def test_checkpointed_vjp_1024(hii):
    dev = torch.device("cuda")
    nb = max(1, int(round(math.log(RMAX / (L / N)) / math.log(FACTOR))))
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    delta, sfrd = synth.make_boxes_torch(N, L, Z, SEED, device="cuda")
    fb = hii.FilterBank(N, L, 0.71, [(ZETA, RMAX, nb)], kmax=KMAX)
    radii, nf = fb.radii()
    C = torch.empty_like(delta)
    A = torch.empty(delta.shape, dtype=torch.uint8, device=dev)
    g = torch.zeros_like(delta)
    rng = np.random.default_rng(99)
    wts = torch.from_numpy(rng.random((WIN,) * 3)).to(dev)
    sl = tuple(slice(w, w + WIN) for w in W0)
    g[sl] = wts.float()
    gd = torch.empty_like(delta)
    gs = torch.empty_like(delta)
    fb.criterion_device(Z, delta.data_ptr(), sfrd.data_ptr(), C.data_ptr(), A.data_ptr())
    torch.cuda.synchronize()
    free_fwd = torch.cuda.mem_get_info()[0]
    gz = fb.vjp_device(Z, delta.data_ptr(), sfrd.data_ptr(), g.data_ptr(), gd.data_ptr(), gs.data_ptr())
    torch.cuda.synchronize()
    free_bwd = torch.cuda.mem_get_info()[0]
    fb.check()
    print(f"1024^3: {len(radii)} radii ({nf} FFT branch), device memory in use: forward "
          f"{(free0 - free_fwd) / 1e9:.1f} GB, after the VJP {(free0 - free_bwd) / 1e9:.1f} GB")
    h_delta, h_sfrd = delta.cpu().numpy(), sfrd.cpu().numpy()
    rec0, _, _ = fb.prologue(Z, h_delta, h_sfrd)
    fields32 = {}
    for ridx in (0, nf - 1):
        fields32[ridx] = fb.filtered(Z, h_delta, h_sfrd, ridx)
    C_win = C[sl].double()
    A_win = A[sl].clone()
    gd_h, gs_h = gd.cpu(), gs.cpu()
    fb.close()
    del C, A, g, gd, gs, delta, sfrd
    torch.cuda.empty_cache()

    # ---- float64 fields from the library's prologue boxes ----
    dx = L / N
    m = dx ** 3 * synth.qion(Z)  # SFRD -> Rion multiplier (:273)
    h1 = (h_sfrd.astype(np.float64) * m).astype(np.float32)
    dk = 2 * P.PI / L
    f = torch.fft.fftfreq(N, d=1.0 / N, device=dev, dtype=torch.float64)
    hh = torch.arange(N // 2 + 1, device=dev, dtype=torch.float64)
    kmag = dk * torch.sqrt(f[:, None, None] ** 2 + f[None, :, None] ** 2 + hh[None, None, :] ** 2)
    del f, hh
    R0 = torch.fft.rfftn(torch.from_numpy(rec0).to(dev, torch.float64))
    H0 = torch.fft.rfftn(torch.from_numpy(h1).to(dev, torch.float64))
    n3 = float(N) ** 3
    D = WIN - 1  # offsets of the kernel needed: -D..D on each axis
    kidx = torch.from_numpy(np.r_[N - D:N, 0:D + 1]).to(dev)
    recs, hs, ks = [], [], []
    for i, R in enumerate(radii[:nf]):
        W = _w_filter(kmag * R)
        r = torch.fft.irfftn(R0 * W, s=(N, N, N)) * n3
        h = torch.fft.irfftn(H0 * W, s=(N, N, N)) * n3
        if i in fields32:
            for ours, ref in zip(fields32[i], (r, h * ZETA)):  # the hook's ion_R includes zeta
                err = float((torch.from_numpy(ours).to(dev).double() - ref).abs().max())
                scale = float(ref.abs().max())
                print(f"R={R:.3f}: filtered field error {err / scale:.2e} of max |field|")
                assert err <= TOL_FIELD * scale
        recs.append(r[sl].clone())
        hs.append(h[sl].clone())
        kfull = torch.fft.irfftn(W.to(torch.complex128), s=(N, N, N)) * n3
        ks.append(kfull.index_select(0, kidx).index_select(1, kidx).index_select(2, kidx).clone())
        del W, r, h, kfull
    del R0, H0, kmag
    torch.cuda.empty_cache()

    def crit(v=None, drec=0.0, dh=0.0):
        best = torch.full((WIN,) * 3, -math.inf, dtype=torch.float64, device=dev)
        top2 = torch.full_like(best, -math.inf)
        for i in range(nf):
            r, h = recs[i], hs[i]
            if v is not None:
                # kernel value at x - v for x in the window: offset index (x - v) + D
                o = [D - (v[a] - W0[a]) for a in range(3)]
                kr = ks[i][o[0]:o[0] + WIN, o[1]:o[1] + WIN, o[2]:o[2] + WIN]
                r = r + drec * kr
                h = h + dh * kr
            ratio = torch.where(r > 0, ZETA * h / r, torch.full_like(r, -math.inf))
            top2 = torch.maximum(top2, torch.minimum(best, ratio))
            best = torch.maximum(best, ratio)
        return torch.where(torch.isinf(best), torch.zeros_like(best), best), top2

    C64, top2 = crit()
    dC = (C64 - C_win).abs()
    print(f"criterion on the window: max |C| {float(C64.abs().max()):.4g}, max |C32 - C64| {float(dC.max()):.3e}")
    assert float(dC.max()) <= 1e-4 * float(C64.abs().max())
    loss = lambda Cx: float((wts * Cx).sum())
    gap = ((C64 - top2) / C64.abs().clamp(min=1e-30)).cpu().numpy()
    cand = np.argwhere(gap > 0.02)
    picks = cand[np.random.default_rng(7).choice(len(cand), size=NVOX, replace=False)]
    rel_d, rel_s = [], []
    for p in picks:
        v = tuple(int(p[a]) + W0[a] for a in range(3))
        dv = float(h_delta[v])
        hstep = H_REL * max(abs(dv), 1e-3)
        base = _rrec64(1.0 + dv)
        Lp = loss(crit(v, drec=_rrec64(1.0 + dv + hstep) - base)[0])
        Lm = loss(crit(v, drec=_rrec64(1.0 + dv - hstep) - base)[0])
        rel_d.append((float(gd_h[v]), (Lp - Lm) / (2 * hstep)))
        sv = float(h_sfrd[v])
        sstep = H_REL * max(abs(sv), float(np.abs(h_sfrd[sl]).mean()))
        Lp = loss(crit(v, dh=sstep * m)[0])
        Lm = loss(crit(v, dh=-sstep * m)[0])
        rel_s.append((float(gs_h[v]), (Lp - Lm) / (2 * sstep)))
    fdz = loss(C64) / ZETA  # C is linear in zeta at fixed argmax

    def stats(pairs):
        a = np.array(pairs)
        scale = np.abs(a[:, 1]).max()
        err = np.abs(a[:, 0] - a[:, 1]) / (np.abs(a[:, 1]) + 1e-3 * scale)
        return np.median(err), np.quantile(err, 0.95), err.max()

    md, q95d, mxd = stats(rel_d)
    ms, q95s, mxs = stats(rel_s)
    print(f"delta: median {md:.2e} q95 {q95d:.2e} max {mxd:.2e}; src: median {ms:.2e} q95 {q95s:.2e} "
          f"max {mxs:.2e}; zeta adj {gz:.6e} fd {fdz:.6e}; argmax checkpoint range {int(A_win.min())}.."
          f"{int(A_win.max())}")
    assert md < 1e-3 and q95d < 2e-2
    assert ms < 1e-3 and q95s < 2e-2
    assert abs(gz - fdz) <= 1e-3 * abs(fdz)
