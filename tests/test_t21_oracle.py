"""The 21-cm brightness-temperature oracle (oracle/t21_oracle.py) against the
reference's own t21.c output on the golden fixtures: T_b boxes within 1e-5
of the box's max |T_b| (both compute in double; the FFTs differ at the
1e-15 level and the output is float), the mean T_b and mean TS as printed."""
import os

import numpy as np
import pytest

from helpers import GOLDEN
from oracle import t21_oracle as T


def _cosmo():
    return T.Cosmo(0.27, 0.046, 0.73, 0.71)


@pytest.mark.parametrize("name", ["t21_n32.npz", "t21_n32_lya.npz"])
def test_t21_oracle_matches_reference(name):
    g = np.load(os.path.join(GOLDEN, name))
    N = g["delta_9"].shape[0]
    L = 25.0
    lya = bool(g["lya"])
    av = [float(x.split()[1]) for x in str(g["t21_av_txt"]).splitlines()]
    ts = [float(x.split()[1]) for x in str(g["TS_av_txt"]).splitlines()] if lya else []
    for n, z in enumerate((9.0, 8.0, 7.0)):
        use = lya and z > 8.0 - 0.1
        tb, mean, tsm = T.t21_box(z, g[f"delta_{z:.0f}"], g[f"xhii_{z:.0f}"], L, _cosmo(), int(g["vel_comp"]),
                                  *((g[f"xc_{z:.0f}"], g[f"xalpha_{z:.0f}"], g[f"tempx_{z:.0f}"]) if use
                                    else (None, None, None)))
        ref = g[f"tb_{z:.0f}"].reshape(tb.shape)
        assert np.abs(tb - ref).max() <= 1e-5 * np.abs(ref).max()
        assert abs(mean - av[n]) <= 1e-7 * abs(av[n])
        if use:
            assert abs(tsm - ts[n]) <= 1e-7 * abs(ts[n])
