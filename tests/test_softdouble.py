"""The integer soft-double routines of the GPU prologue against the host's
native IEEE double unit (compiled as host C++)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ not available")
    exe = str(tmp_path_factory.mktemp("sd") / "softdouble_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off",
                    "-I", os.path.join(ROOT, "simfast21_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "native", "softdouble_check.cpp"), "-o", exe],
                   check=True)
    return exe


def test_basic_ops_bit_exact(checker):
    r = subprocess.run([checker, "300000", "12345"], capture_output=True, text=True, check=True)
    stats = {l.split()[0]: list(map(int, l.split()[1:])) for l in r.stdout.strip().splitlines()}
    for op in ("add", "sub", "mul", "div", "div_c", "sqrt", "to_float", "from_float", "pow4_exact", "sqrt_fast"):
        n, bad, _ = stats[op]
        assert n > 0 and bad == 0, (op, stats[op])
    # pow is correctly rounded; libm pow may misround near ties by 1 ulp,
    # never more, and the float rounding of the prologue hides it.
    for op in ("pow", "pow4", "pow3", "exp"):
        n, bad, maxulp = stats[op]
        assert maxulp <= 1 and bad < n * 0.005, (op, stats[op])
    assert stats["pow_then_float"][1] == 0


def test_uniform_products_bit_exact(tmp_path):
    """sg_dmul.h, the subgrid's double products of taus uniforms in integer
    arithmetic, against the CPU's double multiply (chains of up to 13
    factors, including uniforms with few significant bits)."""
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "dmul_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off",
                    "-I", os.path.join(ROOT, "simfast21_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "native", "dmul_check.cpp"), "-o", exe], check=True)
    r = subprocess.run([exe, "400000", "7"], capture_output=True, text=True)
    cases, bad = map(int, r.stdout.split())
    assert cases > 1_000_000 and bad == 0, r.stdout + r.stderr


def test_prologue_fast_paths_match_exact_chains(tmp_path):
    """prologue_fast.h, the prologue's fast paths, against the exact
    soft-double chains they stand in for.  Rrec is checked on every float in
    [0.5, 2) and on sampled densities at six redshifts and four boxes; the
    residual-fraction and source products and XHI on the same sweeps.  Each
    fast path must return the exact chain's float whenever it returns.  On
    realistic inputs it must decline (guard band) for about one input in
    2^21 only."""
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "prologue_fast_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off",
                    "-I", os.path.join(ROOT, "simfast21_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "native", "prologue_fast_check.cpp"), "-o", exe], check=True)
    r = subprocess.run([exe, "40000", "31"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    stats = {l.split()[0]: list(map(int, l.split()[1:])) for l in r.stdout.strip().splitlines()
             if not l.startswith("#")}
    assert stats["rrec_exhaustive"][0] == (1 << 24)
    for name, (n, bad, fallback) in stats.items():
        assert n > 0 and bad == 0, (name, stats[name], r.stdout)
        if name != "rrec_wide":  # wide exponents include results below the float range
            assert fallback <= max(8, n * 1e-5), (name, stats[name])
