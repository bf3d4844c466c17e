"""The sf21_hii executable as a drop-in for get_HIIbubbles.x: same base
directory in, same files out (xHII boxes byte-identical with the reference's
outside the 1e-5 criterion band, same x_HI and zsim text)."""
import os
import subprocess

import numpy as np
import pytest

from helpers import load_golden, oracle_params
from oracle import fp64_oracle as F
from simfast21_gb300 import params as P, synth

pytestmark = pytest.mark.gpu


def _write_base(tmp, g, sfr=True):
    base = str(tmp)
    with open(os.path.join(base, "simfast21.ini"), "w") as f:
        f.write(str(g["ini"]))
    sp = g["params"]
    os.makedirs(os.path.join(base, "delta"), exist_ok=True)
    os.makedirs(os.path.join(base, "SFR" if sfr else "Halos"), exist_ok=True)
    for i, z in enumerate(g["zs"]):
        z = float(z)
        g[f"delta_{i}"].tofile(os.path.join(base, synth.box_name("delta", z, sp.N, sp.L_file)))
        if sfr:
            g[f"sfrd_{i}"].tofile(os.path.join(base, synth.box_name("sfrd", z, sp.N, sp.L_file)))
        else:
            name = f"Halos/halonl_z{z:.3f}_N{sp.N_halo}_L{sp.L_file:.1f}.dat.catalog"
            with open(os.path.join(base, name), "wb") as f:
                np.array([len(g["catalogue"])], dtype=np.int64).tofile(f)
                g["catalogue"].tofile(f)
    return base


def _run_driver(hii, base):
    from simfast21_gb300 import build
    build.build()
    r = subprocess.run([build.DRIVER, base], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


@pytest.mark.parametrize("name", ["hii_n32_sfr.npz", "hii_n64_sfr.npz", "hii_n40_sfr.npz"])
def test_driver_sfr_branch(hii, oracle_lib, tmp_path, name):
    g = load_golden(name)
    sp = g["params"]
    base = _write_base(tmp_path, g)
    _run_driver(hii, base)
    radii, _ = P.radii(sp.Rmax, sp.dx, sp.Nbins)
    p = oracle_params(oracle_lib, sp)
    identical = True
    for i, z in enumerate(g["zs"]):
        z = float(z)
        x = np.fromfile(os.path.join(base, synth.box_name("xHII", z, sp.N, sp.L_file)), np.float32)
        x = x.reshape((sp.N,) * 3)
        ref = oracle_lib.run_z_sfr(p, z, g[f"delta_{i}"], g[f"sfrd_{i}"], extras=True)
        b = F.bands(ref["rec0"], ref["ion0"], radii, sp.dx, sp.dk)
        certain = b["ionised_lo"] == b["ionised_hi"]
        assert np.array_equal(x[certain].view(np.uint32), g[f"xHII_{i}"][certain].view(np.uint32))
        identical &= np.array_equal(x.view(np.uint32), g[f"xHII_{i}"].view(np.uint32))
    xhi = open(os.path.join(base, "Output_text_files", f"x_HI_N{sp.N}_L{sp.L_file:.1f}.dat")).read()
    if identical:
        assert xhi.split() == str(g["x_HI_txt"]).split()
    zsim = open(os.path.join(base, "Output_text_files", "zsim.txt")).read().split()
    assert [float(v) for v in zsim] == sorted([float(f"{z:.6f}") for z in g["zs"]], reverse=True)


def test_driver_halo_branch(hii, oracle_lib, tmp_path):
    g = load_golden("hii_n32_halo.npz")
    sp = g["params"]
    base = _write_base(tmp_path, g, sfr=False)
    _run_driver(hii, base)
    z = float(g["zs"][0])
    x = np.fromfile(os.path.join(base, synth.box_name("xHII", z, sp.N, sp.L_file)), np.float32)
    x = x.reshape((sp.N,) * 3)
    p = oracle_params(oracle_lib, sp)
    rion = oracle_lib.halo_source(p, z, g["catalogue"])
    out = oracle_lib.run_z_rion(p, z, g["delta_0"], rion)
    assert np.array_equal(out["xhii"].view(np.uint32), g["xHII_0"].view(np.uint32))
    radii, _ = P.radii(sp.Rmax, sp.dx, sp.Nbins)
    fb = hii.FilterBank(sp.N, sp.L, sp.hubble, [(sp.fesc, sp.Rmax, sp.Nbins)], N_halo=sp.N_halo)
    smoothed = oracle_lib.halo_smoothed(p, z, g["catalogue"])
    rec0, _, _ = fb.prologue(z, g["delta_0"], smoothed, src_kind=hii.SF21_SRC_RION)
    b = F.bands(rec0, rion, radii, sp.dx, sp.dk)
    certain = b["ionised_lo"] == b["ionised_hi"]
    assert np.array_equal(x[certain].view(np.uint32), g["xHII_0"][certain].view(np.uint32))
