"""The C-ABI library builds, loads and exports every declared entry point;
without a GPU its calls fail loudly instead of falling back to the CPU."""
import os
import re

import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def declared_symbols():
    syms = []
    for f in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if f.endswith(".h"):
            text = open(os.path.join(ROOT, "include", f)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            syms += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(sf21_\w+)\s*\(", text, flags=re.M)
    return sorted(set(syms))


@pytest.fixture(scope="module")
def lib():
    from simfast21_gb300 import build, hii
    build.build()
    return hii.load_library()


def test_exports_every_declared_symbol(lib):
    from simfast21_gb300 import halos, hii, sfr
    syms = declared_symbols()
    assert len(syms) >= 12
    for s in syms:
        assert hasattr(lib, s), s
    assert sorted(hii.EXPORTS + halos.EXPORTS + sfr.EXPORTS) == syms


def test_no_cpu_fallback_without_gpu(lib):
    from conftest import gpu_available
    from simfast21_gb300 import hii
    if gpu_available():
        pytest.skip("GPU present")
    with pytest.raises(hii.HIIError) as e:
        hii.FilterBank(32, 25.0, 0.71, [(30.0, 12.5, 29)])
    assert e.value.code == 3  # SF21_E_CUDA
    from simfast21_gb300 import sfr
    with pytest.raises(hii.HIIError) as e:
        sfr.SFRBox(64, 32, 25.0)
    assert e.value.code == 3


def test_rejects_unsupported_box(lib):
    from simfast21_gb300 import hii
    with pytest.raises(hii.HIIError) as e:
        hii.FilterBank(56, 150.0, 0.71, [(30.0, 60.0, 50)])  # 56 = 8 x 7: no radix-7 transforms
    assert e.value.code == 5  # SF21_E_UNSUPPORTED
