"""Host-side parameter semantics (Input_variables.c:16-141)."""
import math

import pytest

from simfast21_gb300 import params as P, synth


def test_ini_roundtrip(tmp_path):
    w = synth.Workload(N=64, L=50.0, zs=[], zeta=30.0, Rmax=60.0, factor=1.05)
    f = tmp_path / "simfast21.ini"
    f.write_text(synth.ini_text(w, 6.0, 12.0, 6.0 / 19.0))
    sp = P.derive(P.read_ini(str(f)))
    assert sp.N == 64 and sp.use_sfr and sp.fesc == 30.0
    assert abs(sp.L - 50.0) < 1e-12
    assert sp.Rmax == sp.L / 2.0  # clamp (Input_variables.c:124)
    # zmin re-snap (Input_variables.c:133)
    dz = 6.0 / 19.0
    assert sp.zmin == 12.0 - dz * float(math.ceil((12.0 - 6.0) / dz))


def test_ini_rejects_lines_without_value(tmp_path):
    f = tmp_path / "simfast21.ini"
    f.write_text("N_smoothed\n")
    with pytest.raises(P.IniError):
        P.read_ini(str(f))


def test_redshift_list_is_repeated_addition():
    zs = synth.redshift_list(6.0, 12.0, 6.0 / 19.0)
    assert len(zs) == 20 and abs(zs[-1] - 12.0) < 1e-9
    z = zs[0]
    for i in range(1, len(zs)):
        z += 6.0 / 19.0
        assert zs[i] == z


def test_radius_counts_of_the_benchmark_configs():
    # 128^3, L=100, Rmax=50, factor 1.1 -> 37 FFT-branch + 7 small radii
    R, nf = P.radii(50.0, 100.0 / 128, 44)
    assert (nf, len(R) - nf) == (37, 7)
