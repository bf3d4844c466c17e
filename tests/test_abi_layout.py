"""The ctypes mirrors of the C-ABI structures (hii.py, halos.py, sfr.py) have
the sizes and field offsets of the structures declared in include/*.h, as the
host C compiler lays them out."""
import ctypes
import os
import shutil
import subprocess

import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def _mirrors():
    from simfast21_gb300 import halos, hii, sfr
    return {
        "sf21_hii_set": hii._Set,
        "sf21_hii_config": hii._Config,
        "sf21_t21_cosmo": hii.T21Cosmo,
        "sf21_halo_config": halos.HaloConfig,
        "sf21_halo_mass": halos.HaloMass,
        "sf21_sfr_config": sfr.SFRConfig,
    }


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "sf21_hii.h"', '#include "sf21_halos.h"',
             '#include "sf21_sfr.h"', "int main(void) {"]
    for name, st in _mirrors().items():
        lines.append(f'  printf("{name} size %zu\\n", sizeof({name}));')
        for f in st._fields_:
            lines.append(f'  printf("{name} {f[0]} %zu\\n", offsetof({name}, {f[0]}));')
    lines.append('  printf("sf21_halo_rec size %zu\\n", sizeof(sf21_halo_rec));')
    lines += ["  return 0;", "}"]
    d = tmp_path_factory.mktemp("layout")
    src, exe = d / "layout.c", d / "layout"
    src.write_text("\n".join(lines) + "\n")
    subprocess.run([cc, "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    res = {}
    for line in out.splitlines():
        s, k, v = line.split()
        res[(s, k)] = int(v)
    return res


@pytest.mark.parametrize("name", ["sf21_hii_set", "sf21_hii_config", "sf21_t21_cosmo", "sf21_halo_config",
                                  "sf21_halo_mass", "sf21_sfr_config"])
def test_struct_layout_matches_header(c_layout, name):
    st = _mirrors()[name]
    assert ctypes.sizeof(st) == c_layout[(name, "size")]
    for f in st._fields_:
        assert getattr(st, f[0]).offset == c_layout[(name, f[0])], f[0]


def test_halo_record_is_halo_t(c_layout):
    from simfast21_gb300.halos import HALO_DTYPE
    assert HALO_DTYPE.itemsize == c_layout[("sf21_halo_rec", "size")] == 16
