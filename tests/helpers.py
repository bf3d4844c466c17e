"""Shared helpers for the tests (golden fixtures, oracle parameters)."""
import io
import os

import numpy as np

from simfast21_gb300 import params as P

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_golden(name):
    z = np.load(os.path.join(GOLDEN, name), allow_pickle=False)
    d = {k: z[k] for k in z.files}
    ini = str(d["ini"])
    vals = {}
    for line in io.StringIO(ini):
        if not line or line[0] in "#\n" or "=" not in line:
            continue
        k, v = line.replace("=", " ", 1).split()[:2]
        vals[k] = v
    d["params"] = P.derive(vals)
    return d


def oracle_params(O, sp, nthreads=None):
    return O.params(sp.N, sp.L, sp.hubble, sp.Rmax, sp.Nbins, sp.fesc, nthreads=nthreads,
                    N_halo=sp.N_halo)
