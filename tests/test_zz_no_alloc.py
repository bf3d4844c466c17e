"""sf21_hii_halo_source_noalloc: the halo source box with its scratch in the
library's fixed device array instead of cudaMalloc'd memory.  Checked through
the C-ABI against the context entry point sf21_hii_halo_source (same kernels,
so bit for bit) on consecutive calls, and its size limits."""
import numpy as np
import pytest

from simfast21_gb300 import synth

pytestmark = pytest.mark.gpu

N, NH, L, Z = 64, 128, 50.0, 7.5
MAX_HALOS = 16384


def _catalogue(seed):
    delta = synth.lognormal_delta(synth.gaussian_field(N, seed), 0.8)
    cat = synth.halo_catalogue(delta, seed + 1, occupancy=0.04, n_halo=NH)
    return cat[:MAX_HALOS]


def _device(cat):
    import torch
    return torch.from_numpy(np.ascontiguousarray(cat).view(np.float32).reshape(-1, 4).copy()).cuda()


def test_noalloc_matches_context_entry_on_consecutive_calls(hii):
    import torch
    fb = hii.FilterBank(N, L, 0.71, [(0.5, L / 2, 20)], N_halo=NH)
    cats = [_catalogue(55), _catalogue(77), _catalogue(55)]
    free_after = []
    for cat in cats:
        want = fb.halo_source(Z, cat)
        d_cat = _device(cat)
        out = torch.full((N, N, N), float("nan"), device="cuda")
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        hii.halo_source_noalloc(Z, NH, N, len(cat), d_cat.data_ptr(), out.data_ptr())
        torch.cuda.synchronize()
        free_after.append((free_before, torch.cuda.mem_get_info()[0]))
        got = out.cpu().numpy()
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    # nothing allocated on the device by the calls after the first (the first
    # may load the library's module image, which holds the array)
    for before, after in free_after[1:]:
        assert after == before
    # an empty catalogue leaves a zero box (the fine grid is cleared per call)
    out = torch.full((N, N, N), float("nan"), device="cuda")
    hii.halo_source_noalloc(Z, NH, N, 0, 0, out.data_ptr())
    torch.cuda.synchronize()
    assert not out.any().item()
    fb.close()


def test_noalloc_rejects_sizes_beyond_its_scratch(hii):
    import torch
    cat = np.zeros(MAX_HALOS + 1, dtype=[("Mass", "<f4"), ("x", "<f4"), ("y", "<f4"), ("z", "<f4")])
    cat["Mass"] = 1e10
    d_cat = _device(cat)
    out = torch.zeros((N, N, N), device="cuda")
    with pytest.raises(hii.HIIError, match="no-alloc halo source limited"):
        hii.halo_source_noalloc(Z, NH, N, MAX_HALOS + 1, d_cat.data_ptr(), out.data_ptr())
    with pytest.raises(hii.HIIError, match="no-alloc halo source limited"):
        hii.halo_source_noalloc(Z, 256, N, 10, d_cat.data_ptr(), out.data_ptr())
    with pytest.raises(hii.HIIError):
        hii.halo_source_noalloc(Z, 32, N, 10, d_cat.data_ptr(), out.data_ptr())
