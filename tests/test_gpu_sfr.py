"""The star-formation-rate stage on the GPU (include/sf21_sfr.h) against the
reference's own get_SFR.c outputs (tests/golden/sfr_*.npz) and the CPU
restatement: the SFRD boxes bit for bit, the sfrd_av text lines character
for character, and the drop-in driver's files byte for byte."""
import os
import subprocess

import numpy as np
import pytest

from helpers import load_golden

pytestmark = pytest.mark.gpu

FIXTURES = ["sfr_n32.npz", "sfr_n48_lya.npz"]


def _ctx(hii, sp):
    from simfast21_gb300 import sfr
    return sfr.SFRBox(sp.N_halo, sp.N, sp.L)


@pytest.mark.parametrize("name", FIXTURES)
def test_sfrd_boxes_match_reference(hii, name):
    g = load_golden(name)
    sp = g["params"]
    s = _ctx(hii, sp)
    written = [float(z) for z in g["zs_written"]]
    lines = []
    for i, z in enumerate(g["zs"]):
        z = float(z)
        if z not in written:
            continue
        box, mean = s.box(z, g[f"catalogue_{i}"])
        assert np.array_equal(box.view(np.uint32), g[f"sfrd_{i}"].view(np.uint32)), f"z={z}"
        lines.append("%f %.8E" % (z, mean))
    assert lines == str(g["sfrd_av_txt"]).splitlines()
    s.close()


@pytest.mark.parametrize("name", FIXTURES)
def test_driver_matches_reference_files(hii, tmp_path, name):
    """sf21_get_SFR (drop-in for get_SFR.x) on the fixture's base directory:
    the same SFR/sfrd_* files and the same sfrd_av text file."""
    from simfast21_gb300 import build
    g = load_golden(name)
    sp = g["params"]
    base = str(tmp_path)
    os.makedirs(os.path.join(base, "Halos"))
    open(os.path.join(base, "simfast21.ini"), "w").write(str(g["ini"]))
    Lf = sp.L_file
    Nh = int(g["N_halo"])
    for i, z in enumerate(g["zs"]):
        cat = g[f"catalogue_{i}"]
        with open(os.path.join(base, f"Halos/halonl_z{float(z):.3f}_N{Nh}_L{Lf:.1f}.dat.catalog"), "wb") as f:
            np.array([len(cat)], np.int64).tofile(f)
            cat.tofile(f)
    r = subprocess.run([build.SFR_DRIVER, base], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    for i, z in enumerate(g["zs"]):
        path = os.path.join(base, f"SFR/sfrd_z{float(z):.3f}_N{sp.N}_L{Lf:.1f}.dat")
        if f"sfrd_{i}" in g:
            assert open(path, "rb").read() == g[f"sfrd_{i}"].tobytes(), z
        else:
            assert not os.path.exists(path), z
    txt = open(os.path.join(base, "Output_text_files", f"sfrd_av_N{sp.N}_L{Lf:.1f}.dat")).read()
    assert txt == str(g["sfrd_av_txt"])
    assert r.stdout.count("Writing SFRD file...") == len(g["zs_written"])


def _random_catalogue(n, N_halo, seed, edges=True, discrete=False):
    from simfast21_gb300.halos import HALO_DTYPE
    rng = np.random.default_rng(seed)
    cat = np.zeros(n, HALO_DTYPE)
    if discrete:  # the halo finder's masses: a schedule of 10^(0.2 k) steps
        cat["Mass"] = (1e8 * 10.0 ** (0.2 * rng.integers(0, 21, n))).astype(np.float32)
    else:
        cat["Mass"] = (10.0 ** rng.uniform(7.5, 12.5, n)).astype(np.float32)
    for ax in ("x", "y", "z"):
        cat[ax] = (rng.random(n) * N_halo).astype(np.float32)
    if edges and n >= 64:
        # positions on cell faces, at 0 and at N_halo (wrapped by check_borders,
        # auxiliary.c:537-544), just below N_halo, and many halos in one cell
        # (a long serial chain)
        cat["x"][:8] = [0.0, float(N_halo), np.nextafter(np.float32(N_halo), np.float32(0)), 1.0, 2.5, 0.5, 3.0, 7.0]
        cat["y"][8:16] = 0.0
        cat["z"][16:24] = float(N_halo)
        cat["x"][24:64] = 5.25
        cat["y"][24:64] = 6.75
        cat["z"][24:64] = 7.5
    return cat


@pytest.mark.parametrize("N_halo,N,n,z,discrete", [(128, 64, 200_000, 9.0, False), (128, 64, 200_000, 9.0, True),
                                                    (96, 96, 50_000, 7.5, False), (100, 48, 30_000, 6.0, True),
                                                    (81, 27, 20_000, 7.0, True), (64, 32, 0, 8.0, False),
                                                    (64, 16, 1, 8.0, False)])
def test_sfrd_vs_restatement(hii, oracle_lib, N_halo, N, n, z, discrete):
    """Catalogues with edge positions, one crowded cell, distinct or schedule
    masses, equal grids (block side 1), block sides that do not divide or
    whose cube is not a power of two (3^3), an empty and a one-halo
    catalogue, against the CPU restatement bit for bit."""
    O = oracle_lib
    L = 40.0
    p = O.params(N, L, 0.71, L / 2, 10, 30.0, N_halo=N_halo)
    cat = _random_catalogue(n, N_halo, seed=N_halo * 7 + n, discrete=discrete)
    want, wmean = O.sfrd_box(p, z, cat)
    from simfast21_gb300 import sfr
    s = sfr.SFRBox(N_halo, N, L)
    got, gmean = s.box(z, cat)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    assert gmean == wmean
    if n == 0:
        assert not np.any(got)
    s.close()


def test_sfrd_full_size_and_device_entry(hii, oracle_lib):
    """512^3 catalogue grid smoothed to 256^3 with 2 M halos (host entry)
    against the restatement; the device entry on the same catalogue gives the
    same bits; the total SFR is conserved up to float rounding."""
    import torch
    from simfast21_gb300 import sfr
    O = oracle_lib
    N_halo, N, L, z = 512, 256, 200.0, 8.0
    cat = _random_catalogue(2_000_000, N_halo, seed=99)
    p = O.params(N, L, 0.71, L / 2, 10, 30.0, N_halo=N_halo, nthreads=os.cpu_count() or 1)
    want, wmean = O.sfrd_box(p, z, cat)
    s = sfr.SFRBox(N_halo, N, L)
    got, gmean = s.box(z, cat)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    assert gmean == wmean
    d_cat = torch.from_numpy(cat.view(np.uint8).copy()).cuda()
    d_out = torch.empty(N ** 3, dtype=torch.float32, device="cuda")
    st = torch.cuda.current_stream()
    s.box_device(z, len(cat), d_cat.data_ptr(), d_out.data_ptr(), st.cuda_stream)
    torch.cuda.synchronize()
    assert np.array_equal(d_out.cpu().numpy().view(np.uint32), want.reshape(-1).view(np.uint32))
    # size-independent check: the cloud-in-cell weights of a halo sum to 1, so
    # the box integral (sfrd x dx_halo^3 x block volume) is the catalogue's
    # total sfr = sum Rion(M, z) / Qion(z) (user_functions.c:40-47, 71-88)
    M = cat["Mass"].astype(np.float64)
    rion = 1.575e39 * M * (1.0 + z) ** 2.27044695 * (M / 9.367608e7) ** 0.44 * np.exp(-(9.367608e7 / M) ** 3) / 1e45
    exact = float(rion.sum() / O.lib().sf21o_Qion(z))
    integral = float(got.astype(np.float64).sum()) * (L / N_halo) ** 3 * (N_halo // N) ** 3
    assert exact > 0 and abs(integral - exact) <= 1e-4 * exact
    s.close()
