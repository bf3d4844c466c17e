"""The power-spectrum oracle (oracle/pk_oracle.py) against the reference's
own tools/power3d_f.c output on the golden fixtures: same number of bins, k
to the printed precision, P(k) within 1e-5 relative (the tool prints 7
significant digits; its FFT and ours round differently at the 1e-7 level)."""
import numpy as np
import pytest

from helpers import GOLDEN  # noqa: F401  (fixture directory)
from oracle import pk_oracle as K

import os


@pytest.mark.parametrize("name", ["pk_n32.npz", "pk_n64.npz"])
def test_pk_oracle_matches_reference_tool(name):
    g = np.load(os.path.join(GOLDEN, name))
    box, dl = g["box"], float(g["dl"])
    for f in g["flags"]:
        k, P, _ = K.power_spectrum(box, dl, int(f))
        kr, Pr = g[f"k_{f}"], g[f"P_{f}"]
        assert len(k) == len(kr)
        assert np.abs(k - kr).max() <= 5e-7 + 1e-12
        assert np.max(np.abs(P - Pr) / np.abs(Pr)) <= 1e-5
