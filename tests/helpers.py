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


def load_halo_golden(name):
    """A halos_*.npz fixture with its density box: stored, or rebuilt from the
    recipe (synth.hash_field reproduces the same bits on every machine)."""
    from simfast21_gb300 import synth
    z = np.load(os.path.join(GOLDEN, name), allow_pickle=False)
    d = {k: z[k] for k in z.files}
    d["ini"] = str(d["ini"])
    if "delta" not in d:
        w = synth.HaloWorkload(N=int(d["N"]), L_mpc=float(d["L_mpc"]), sigma=float(d["sigma"]), seed=int(d["seed"]),
                               smooth=int(d["smooth"]), slope=float(d["slope"]))
        d["delta"] = w.density()
    d["delta"] = np.ascontiguousarray(d["delta"], np.float32).reshape((int(d["N"]),) * 3)
    return d


HALO_CASES = ["halos_n64.npz", "halos_n128_dense.npz", "halos_n64_sgrid.npz", "halos_n96.npz", "halos_n120_sgrid.npz"]
