"""Host-side helpers of bench.py (no GPU): every named workload resolves and is
described, the synthetic catalogue has the Halo_t layout, and the argument
parser accepts the documented flags."""
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


@pytest.fixture(scope="module")
def bench():
    sys.path.insert(0, ROOT)
    import bench as B
    return B


@pytest.mark.parametrize("name", ["batched512", "batched256", "single512", "single256", "single600", "plain128"])
def test_workloads_resolve(bench, name):
    w = bench.workload(name)
    assert w["name"] == name and w["N"] > 0 and len(w["sets"]) >= 1
    assert isinstance(bench.describe(w), str) and str(w["N"]) in bench.describe(w)
    assert bench.total_radii(w) > 0


def test_sfr_catalogue_layout(bench):
    from simfast21_gb300.halos import HALO_DTYPE
    cat = bench.sfr_catalogue(10000, 64, seed=1)
    assert cat.dtype == HALO_DTYPE and len(cat) == 10000
    assert len(np.unique(cat["Mass"])) <= 21  # the halo finder's mass schedule
    for ax in ("x", "y", "z"):
        assert cat[ax].min() >= 0.0 and cat[ax].max() <= 64.0


def test_flags_parse():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--help"], capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0
    for flag in ("--gpus", "--steps", "--warmup", "--impl", "--workload", "--no-600", "--sfr-only", "--halos-only"):
        assert flag in r.stdout
