"""Host behaviour of the drop-in executables that needs no GPU: usage text and
exit codes, a missing simfast21.ini, get_SFR.c's early exit when neither SFR
nor Lya/X-ray boxes are wanted (get_SFR.c:51), and a loud failure (exit 1,
the library's message) where the GPU is needed -- never a CPU fallback."""
import os
import subprocess

import pytest

from conftest import gpu_available


@pytest.fixture(scope="module")
def drivers():
    from simfast21_gb300 import build
    build.build()
    return build


def _run(exe, *args):
    return subprocess.run([exe, *args], capture_output=True, text=True, timeout=120)


@pytest.mark.parametrize("attr", ["DRIVER", "HALO_DRIVER", "SFR_DRIVER", "T21_DRIVER"])
def test_usage_without_arguments(drivers, attr):
    r = _run(getattr(drivers, attr))
    assert r.returncode == 1
    assert "base_dir" in r.stdout or "work_dir" in r.stdout


@pytest.mark.parametrize("attr", ["DRIVER", "HALO_DRIVER", "SFR_DRIVER", "T21_DRIVER"])
def test_missing_ini(drivers, attr, tmp_path):
    r = _run(getattr(drivers, attr), str(tmp_path))
    assert r.returncode == 1


def _ini(tmp_path, use_sfr, lya):
    text = "\n".join(["nthreads = 2", "zmax = 8.0", "zmin = 7.0", "dz = 1.0", "sim_length = 25.0",
                      "N_halo = 64", "N_smoothed = 32", "hubble = 0.7", f"use_SFR = {use_sfr}",
                      f"use_Lya_xrays = {lya}", "Zminsfr = 7.5", ""])
    (tmp_path / "simfast21.ini").write_text(text)


def test_sfr_driver_early_exit(drivers, tmp_path):
    _ini(tmp_path, "F", "F")
    r = _run(drivers.SFR_DRIVER, str(tmp_path))
    assert r.returncode == 0
    assert "no need to calculate SFR" in r.stdout
    assert not (tmp_path / "SFR").exists()


def test_sfr_driver_fails_loudly_without_gpu(drivers, tmp_path):
    if gpu_available():
        pytest.skip("GPU present")
    _ini(tmp_path, "T", "F")
    os.makedirs(tmp_path / "Halos")
    r = _run(drivers.SFR_DRIVER, str(tmp_path))
    assert r.returncode == 1
    assert "sf21_get_SFR:" in r.stdout
    assert not any((tmp_path / "SFR").glob("sfrd_*"))
