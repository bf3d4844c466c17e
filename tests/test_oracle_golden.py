"""The CPU restatement (oracle/hii_oracle.c) against the reference's own
outputs (tests/golden, produced by the reference's get_HIIbubbles.c)."""
import os

import numpy as np
import pytest

from helpers import load_golden, oracle_params


@pytest.mark.parametrize("name", ["hii_n32_sfr.npz", "hii_n64_sfr.npz", "hii_n40_sfr.npz"])
def test_port_matches_reference_sfr(oracle_lib, name):
    O = oracle_lib
    g = load_golden(name)
    sp = g["params"]
    p = oracle_params(O, sp)
    xhi_ref = [float(v) for v in str(g["x_HI_txt"]).split()]
    neutrals = []
    for i, z in enumerate(g["zs"]):
        out = O.run_z_sfr(p, float(z), g[f"delta_{i}"], g[f"sfrd_{i}"])
        ref = g[f"xHII_{i}"]
        assert out["xhii"].view(np.uint32).tolist() == ref.view(np.uint32).tolist() or \
            np.array_equal(out["xhii"].view(np.uint32), ref.view(np.uint32)), f"z={z}"
        neutrals.append(out["neutral"])
    # x_HI file: highest redshift first, %lf (get_HIIbubbles.c:527)
    assert ["%f" % v for v in reversed(neutrals)] == ["%f" % v for v in xhi_ref]


def test_port_matches_reference_halo_branch(oracle_lib):
    O = oracle_lib
    g = load_golden("hii_n32_halo.npz")
    sp = g["params"]
    p = oracle_params(O, sp)
    z = float(g["zs"][0])
    rion = O.halo_source(p, z, g["catalogue"])
    out = O.run_z_rion(p, z, g["delta_0"], rion)
    assert np.array_equal(out["xhii"].view(np.uint32), g["xHII_0"].view(np.uint32))
    assert "%f" % out["neutral"] == "%f" % float(str(g["x_HI_txt"]).split()[0])


def test_radius_schedule_matches_params(oracle_lib):
    from simfast21_gb300 import params as P
    O = oracle_lib
    for name in ("hii_n32_sfr.npz", "hii_n64_sfr.npz"):
        sp = load_golden(name)["params"]
        R_c, nf_c = O.radii(oracle_params(O, sp))
        R_py, nf_py = P.radii(sp.Rmax, sp.dx, sp.Nbins)
        assert R_c == R_py and nf_c == nf_py


def _ref_exe():
    from oracle import oracle as O
    return O.REF_EXE


@pytest.mark.skipif(not os.path.exists(_ref_exe()), reason="the reference's own build (oracle/_ref) is not present")
def test_port_matches_reference_build_directly(oracle_lib, tmp_path):
    """Where the reference's own executable was built (oracle/_ref, from its
    sources by oracle/Makefile), run it on a fresh base dir."""
    import subprocess
    from simfast21_gb300 import params as P, synth
    O = oracle_lib
    w = synth.Workload(N=32, L=30.0, zs=[], zeta=45.0, Rmax=12.0, factor=1.07, seed=77)
    base = str(tmp_path)
    zs = synth.write_base_dir(base, w, 6.5, 7.5, 0.5, nthreads=2)
    subprocess.run([O.REF_EXE, base], check=True, capture_output=True)
    sp = P.derive(P.read_ini(os.path.join(base, "simfast21.ini")))
    p = oracle_params(O, sp)
    for z in zs:
        d = np.fromfile(os.path.join(base, synth.box_name("delta", z, 32, sp.L_file)), np.float32)
        s = np.fromfile(os.path.join(base, synth.box_name("sfrd", z, 32, sp.L_file)), np.float32)
        ref = np.fromfile(os.path.join(base, synth.box_name("xHII", z, 32, sp.L_file)), np.float32)
        out = O.run_z_sfr(p, z, d, s)
        assert np.array_equal(out["xhii"].ravel().view(np.uint32), ref.view(np.uint32))


@pytest.mark.parametrize("name", ["sfr_n32.npz", "sfr_n48_lya.npz"])
def test_port_matches_reference_sfrd(oracle_lib, name):
    """The restatement of get_SFR.c against the reference's own SFRD boxes and
    its sfrd_av text lines ("%f %.8E", get_SFR.c:146)."""
    O = oracle_lib
    g = load_golden(name)
    sp = g["params"]
    p = oracle_params(O, sp)
    written = [float(z) for z in g["zs_written"]]
    lines = []
    for i, z in enumerate(g["zs"]):
        z = float(z)
        if z not in written:
            assert f"sfrd_{i}" not in g
            continue
        box, mean = O.sfrd_box(p, z, g[f"catalogue_{i}"])
        assert np.array_equal(box.view(np.uint32), g[f"sfrd_{i}"].view(np.uint32)), f"z={z}"
        lines.append("%f %.8E" % (z, mean))
    assert lines == str(g["sfrd_av_txt"]).splitlines()
