"""Generate the golden fixtures of the HII stage from the reference itself.

Runs the reference's own get_HIIbubbles.c, compiled unmodified from its
sources by ``make -C oracle ref`` (against the FFTW-API shim and a GSL stub),
on seeded synthetic base directories, and stores inputs and outputs as
compressed .npz files next to this script:

  hii_n32_sfr.npz   N=32,  L=25 Mpc/h, z = 7, 8 (SFR boxes, use_SFR = T)
  hii_n64_sfr.npz   N=64,  L=50 Mpc/h, z = 8
  hii_n32_halo.npz  N=32 (N_halo=64), L=25 Mpc/h, z = 8 (halo catalogue, use_SFR = F)
  hii_n40_sfr.npz   N=40 (not a power of two), L=31.25 Mpc/h, z = 7, 8
  pk_n32.npz        power3d_f on a 32^3 lognormal box, dl = 0.75, window flags 0, 1, 2
  pk_n64.npz        power3d_f on a 64^3 lognormal box, dl = 1.5, Bartlett window
  t21_n32.npz       t21.c on 32^3 boxes, z = 9, 8, 7, Lya/X-rays off, Vel_comp 3
  t21_n32_lya.npz   the same with Lya/X-rays on (Zminsfr = 8), Vel_comp 1
  halos_n64.npz     get_halos.c, 64^3, L=40 Mpc, z = 8, 7, 6, no subgrid
  halos_n128_dense.npz  get_halos.c, 128^3 smoothed integer-hash field (nc up
                    to 8), L=100 Mpc, z = 2, 1: tens of thousands of halos
  halos_n64_sgrid.npz  get_halos.c, 64^3 integer-hash field, L=40 Mpc, z = 8, 7,
                    subgrid on (halo_Mmin 1e9)
  halos_n96.npz     get_halos.c, 96^3 (not a power of two) integer-hash field,
                    L=60 Mpc, z = 3, 2
  halos_n120_sgrid.npz  get_halos.c, 120^3 integer-hash field, L=60 Mpc, z = 6,
                    subgrid on
  sfr_n32.npz       get_SFR.c, N_halo=64 -> N_smoothed=32, L=25 Mpc/h, z = 8, 7
                    (use_SFR = T)
  sfr_n48_lya.npz   get_SFR.c, N_halo=100 -> N_smoothed=48 (a block side that
                    does not divide), use_SFR = F with Lya/X-rays on (Zminsfr
                    = 9 of z = 10, 9, 8)
The integer-hash boxes (synth.hash_field) are rebuilt bit for bit from their
recipe on any machine and are not stored.

Each holds the ini values, the input boxes per redshift, the xHII boxes the
reference wrote, and its x_HI text output.  Needs the reference sources (only
in the build container): REF_DIR or SF21_REF_DIR names their tree, as for
``make -C oracle ref``; the GPU tests read the committed .npz files.
Usage: SF21_REF_DIR=<tree> python tests/golden/make_golden.py [case-prefix ...]   (default: all)
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from simfast21_gb300 import params as P  # noqa: E402
from simfast21_gb300 import synth  # noqa: E402


def run_ref(base: str):
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
    r = subprocess.run([O.REF_EXE, base], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stdout + r.stderr)
    return r.stdout


def case_sfr(name: str, N: int, L: float, zmin: float, zmax: float, seed: int):
    w = synth.Workload(N=N, L=L, zs=[], zeta=30.0, Rmax=L / 2, factor=1.1, seed=seed)
    base = tempfile.mkdtemp(prefix="sf21gold_")
    try:
        zs = synth.write_base_dir(base, w, zmin, zmax, 1.0, nthreads=4)
        log = run_ref(base)
        sp = P.derive(P.read_ini(os.path.join(base, "simfast21.ini")))
        out = {"ini": open(os.path.join(base, "simfast21.ini")).read(), "zs": np.array(zs)}
        for i, z in enumerate(zs):
            for kind in ("delta", "sfrd", "xHII"):
                out[f"{kind}_{i}"] = np.fromfile(os.path.join(base, synth.box_name(kind, z, N, sp.L_file)),
                                                 np.float32).reshape(N, N, N)
        xhi = open(os.path.join(base, "Output_text_files", f"x_HI_N{N}_L{sp.L_file:.1f}.dat")).read()
        out["x_HI_txt"] = xhi
        out["stdout"] = log
        np.savez_compressed(os.path.join(HERE, name), **out)
        print(name, "z =", zs, "x_HI =", xhi.split())
    finally:
        shutil.rmtree(base)


def case_halo(name: str, N: int, N_halo: int, L: float, z: float, seed: int):
    w = synth.Workload(N=N, L=L, zs=[z], zeta=0.6, Rmax=L / 2, factor=1.1, seed=seed)
    base = tempfile.mkdtemp(prefix="sf21gold_")
    try:
        os.makedirs(os.path.join(base, "delta"))
        os.makedirs(os.path.join(base, "Halos"))
        with open(os.path.join(base, "simfast21.ini"), "w") as f:
            f.write(synth.ini_text(w, z, z, 1.0, nthreads=4, use_sfr=False, n_halo=N_halo))
        sp = P.derive(P.read_ini(os.path.join(base, "simfast21.ini")))
        g = synth.gaussian_field(N, seed)
        delta = synth.lognormal_delta(g, w.sigma)
        cat = synth.halo_catalogue(delta, seed + 1, n_halo=N_halo)
        delta.tofile(os.path.join(base, synth.box_name("delta", z, N, sp.L_file)))
        cname = f"Halos/halonl_z{z:.3f}_N{N_halo}_L{sp.L_file:.1f}.dat.catalog"
        with open(os.path.join(base, cname), "wb") as f:
            np.array([len(cat)], dtype=np.int64).tofile(f)
            cat.tofile(f)
        log = run_ref(base)
        xhii = np.fromfile(os.path.join(base, synth.box_name("xHII", z, N, sp.L_file)), np.float32)
        xhi = open(os.path.join(base, "Output_text_files", f"x_HI_N{N}_L{sp.L_file:.1f}.dat")).read()
        np.savez_compressed(os.path.join(HERE, name), ini=open(os.path.join(base, "simfast21.ini")).read(),
                            zs=np.array([z]), delta_0=delta, catalogue=cat,
                            xHII_0=xhii.reshape(N, N, N), x_HI_txt=xhi, stdout=log)
        print(name, "halos", len(cat), "x_HI =", xhi.split())
    finally:
        shutil.rmtree(base)


def case_pk(name: str, N: int, dl: float, seed: int, flags=(0, 1, 2)):
    """The reference's power-spectrum tool (tools/power3d_f.c, built by
    ``make -C oracle ref``) on a seeded lognormal density box: input box and,
    per window flag, the printed output (text, k and P columns)."""
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
    box = synth.lognormal_delta(synth.gaussian_field(N, seed), 0.8).astype(np.float32)
    tmp = tempfile.mkdtemp(prefix="sf21pk_")
    try:
        path = os.path.join(tmp, "box.dat")
        box.tofile(path)
        out = {"box": box, "dl": np.float64(dl), "flags": np.array(flags)}
        for f in flags:
            r = subprocess.run([O.PK_EXE, "4", str(N), str(N), str(N), repr(dl), str(f), path, "4"],
                               capture_output=True, text=True, check=True)
            rows = [ln.split() for ln in r.stdout.splitlines() if ln and not ln.startswith("#")]
            out[f"text_{f}"] = r.stdout.replace(path, "box.dat")
            out[f"k_{f}"] = np.array([float(x[0]) for x in rows])
            out[f"P_{f}"] = np.array([float(x[1]) for x in rows])
        np.savez_compressed(os.path.join(HERE, name), **out)
    finally:
        shutil.rmtree(tmp)


def case_t21(name: str, N: int, L: float, seed: int, vel_comp: int, lya: bool):
    """The reference's t21.c (built by ``make -C oracle ref``) on a seeded base
    directory: density and xHII boxes for z = 9, 8, 7 and, with Lya/X-rays on
    (Zminsfr = 8, so z = 9 and 8 use them), x_c, x_alpha and T_K boxes.
    Stores the inputs, the deltaTb boxes and the two text outputs."""
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
    w = synth.Workload(N=N, L=L, zs=[], zeta=30.0, Rmax=L / 2, factor=1.1, seed=seed)
    base = tempfile.mkdtemp(prefix="sf21t21_")
    rng = np.random.default_rng(seed)
    try:
        ini = synth.ini_text(w, 7.0, 9.0, 1.0, nthreads=4)
        ini += f"Vel_comp = {vel_comp}\nuse_Lya_xrays = {'T' if lya else 'F'}\nZminsfr = 8.0\n"
        with open(os.path.join(base, "simfast21.ini"), "w") as f:
            f.write(ini)
        for d in ("delta", "Ionization", "Output_text_files", "x_c", "Lya", "xrays"):
            os.makedirs(os.path.join(base, d), exist_ok=True)
        out = {"ini": ini, "zs": np.array([9.0, 8.0, 7.0]), "vel_comp": np.int64(vel_comp), "lya": np.int64(lya)}
        g = synth.gaussian_field(N, seed)
        Lmpc = L / w.hubble
        for z in (9.0, 8.0, 7.0):
            delta = synth.lognormal_delta(g, 0.8 * synth.growth(z) / synth.growth(8.0)).astype(np.float32)
            xhii = np.clip(rng.random(delta.shape) * 1.6 - 0.3, 0.0, 1.0).astype(np.float32)
            tag = f"z{z:.3f}_N{N}_L{Lmpc:.1f}.dat"
            delta.tofile(os.path.join(base, "delta", "deltanl_" + tag))
            xhii.tofile(os.path.join(base, "Ionization", "xHII_" + tag))
            out[f"delta_{z:.0f}"] = delta
            out[f"xhii_{z:.0f}"] = xhii
            if lya:
                xc = (rng.random(delta.shape) * 0.5).astype(np.float32)
                xa = (rng.random(delta.shape) * 2.0).astype(np.float32)
                tk = (10.0 + rng.random(delta.shape) * 500.0).astype(np.float32)
                xc.tofile(os.path.join(base, "x_c", "xc_" + tag))
                xa.tofile(os.path.join(base, "Lya", "xalpha_" + tag))
                tk.tofile(os.path.join(base, "xrays", "TempX_" + tag))
                out[f"xc_{z:.0f}"], out[f"xalpha_{z:.0f}"], out[f"tempx_{z:.0f}"] = xc, xa, tk
        r = subprocess.run([O.T21_EXE, base], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(r.stdout + r.stderr)
        for z in (9.0, 8.0, 7.0):
            tag = f"z{z:.3f}_N{N}_L{Lmpc:.1f}.dat"
            out[f"tb_{z:.0f}"] = np.fromfile(os.path.join(base, "deltaTb", "deltaTb_" + tag), dtype=np.float32)
        txt = os.path.join(base, "Output_text_files")
        out["t21_av_txt"] = open(os.path.join(txt, f"t21_av_N{N}_L{Lmpc:.1f}.dat")).read()
        out["TS_av_txt"] = open(os.path.join(txt, f"TS_av_N{N}_L{Lmpc:.1f}.dat")).read()
        np.savez_compressed(os.path.join(HERE, name), **out)
    finally:
        shutil.rmtree(base)


def case_halos(name: str, w, zmin: float, zmax: float, dz: float, keep_full: int = 20000):
    """The reference's get_halos.c (built by ``make -C oracle ref``) on a
    seeded z = 0 density box.  Stores the ini, the box, and per redshift the
    halo count, the SHA-256 of the catalogue records, the per-mass counts the
    reference prints (:281, :320) and the records themselves (all of them up
    to keep_full, else the first 4096)."""
    import hashlib
    import re
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
    base = tempfile.mkdtemp(prefix="sf21halo_")
    try:
        delta = synth.write_halo_base_dir(base, w, zmin, zmax, dz, nthreads=4)
        r = subprocess.run([os.path.join(ROOT, "oracle", "_ref", "get_halos.x"), base], capture_output=True,
                           text=True)
        if r.returncode != 0:
            raise RuntimeError(r.stdout + r.stderr)
        zs = synth.halo_redshifts(zmin, zmax, dz)
        ini = open(os.path.join(base, "simfast21.ini")).read()
        out = {"ini": ini, "zs": np.array(zs), "stdout": r.stdout, "N": np.int64(w.N), "L_mpc": np.float64(w.L_mpc),
               "sigma": np.float64(w.sigma), "seed": np.int64(w.seed), "smooth": np.int64(w.smooth),
               "slope": np.float64(w.slope)}
        if w.smooth == 0:  # a Gaussian field is stored; synth.hash_field boxes are rebuilt from the recipe
            out["delta"] = delta
        blocks = r.stdout.split("+++++++++++++++++++++++++++ z = ")[1:]
        for i, z in enumerate(zs):
            raw = open(os.path.join(base, synth.halo_catalogue_name(z, w.N, w.L_mpc)), "rb").read()
            n = int(np.frombuffer(raw[:8], np.int64)[0])
            recs = np.frombuffer(raw[8:], dtype=[("Mass", "<f4"), ("x", "<f4"), ("y", "<f4"), ("z", "<f4")])
            assert len(recs) == n
            out[f"count_{i}"] = np.int64(n)
            out[f"sha_{i}"] = hashlib.sha256(raw[8:]).hexdigest()
            mc = re.findall(r"Number of halos for M=([0-9.E+-]+): (\d+)", blocks[i])
            out[f"masscounts_{i}"] = np.array([[float(m), float(c)] for m, c in mc])
            cell = re.findall(r"Number of halos found in cell size cycle: (\d+)", blocks[i])
            out[f"cellcount_{i}"] = np.int64(cell[0]) if cell else np.int64(-1)
            out[f"cat_{i}"] = recs.copy() if n <= keep_full else recs[:4096].copy()
            print(name, "z =", z, "halos", n)
        np.savez_compressed(os.path.join(HERE, name), **out)
    finally:
        shutil.rmtree(base)


def case_sfrd(name: str, N: int, N_halo: int, L: float, zmin: float, zmax: float, seed: int,
              use_sfr: bool = True, zminsfr: float | None = None):
    """The reference's star-formation-rate stage (get_SFR.c, built by
    ``make -C oracle ref``) on seeded halo catalogues, one per redshift."""
    w = synth.Workload(N=N, L=L, zs=[], zeta=30.0, Rmax=L / 2, factor=1.1, seed=seed)
    base = tempfile.mkdtemp(prefix="sf21gold_")
    try:
        os.makedirs(os.path.join(base, "Halos"))
        ini = synth.ini_text(w, zmin, zmax, 1.0, nthreads=4, use_sfr=use_sfr, n_halo=N_halo)
        if zminsfr is not None:
            ini += f"use_Lya_xrays = T\nZminsfr = {zminsfr!r}\n"
        with open(os.path.join(base, "simfast21.ini"), "w") as f:
            f.write(ini)
        sp = P.derive(P.read_ini(os.path.join(base, "simfast21.ini")))
        g = synth.gaussian_field(N, seed)
        delta = synth.lognormal_delta(g, w.sigma)
        zs = synth.halo_redshifts(zmin, zmax, 1.0)
        out = {"ini": ini, "zs": np.array(zs), "N_halo": N_halo}
        for i, z in enumerate(zs):
            cat = synth.halo_catalogue(delta, seed + 10 + i, n_halo=N_halo)
            with open(os.path.join(base, f"Halos/halonl_z{z:.3f}_N{N_halo}_L{sp.L_file:.1f}.dat.catalog"), "wb") as f:
                np.array([len(cat)], dtype=np.int64).tofile(f)
                cat.tofile(f)
            out[f"catalogue_{i}"] = cat
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
        r = subprocess.run([os.path.join(ROOT, "oracle", "_ref", "get_SFR.x"), base], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(r.stdout + r.stderr)
        zrun = [z for z in zs if z > (zminsfr if zminsfr is not None else zmin) - 0.1]
        out["zs_written"] = np.array(zrun)
        for i, z in enumerate(zs):
            path = os.path.join(base, f"SFR/sfrd_z{z:.3f}_N{N}_L{sp.L_file:.1f}.dat")
            if os.path.exists(path):
                out[f"sfrd_{i}"] = np.fromfile(path, np.float32).reshape(N, N, N)
        out["sfrd_av_txt"] = open(os.path.join(base, "Output_text_files",
                                               f"sfrd_av_N{N}_L{sp.L_file:.1f}.dat")).read()
        out["stdout"] = r.stdout
        np.savez_compressed(os.path.join(HERE, name), **out)
        print(name, "z =", zs, "halos", [len(out[f"catalogue_{i}"]) for i in range(len(zs))],
              out["sfrd_av_txt"].split())
    finally:
        shutil.rmtree(base)


CASES = {
    "hii_n32_sfr": lambda: case_sfr("hii_n32_sfr.npz", 32, 25.0, 7.0, 8.0, seed=101),
    "hii_n64_sfr": lambda: case_sfr("hii_n64_sfr.npz", 64, 50.0, 8.0, 8.0, seed=202),
    "hii_n32_halo": lambda: case_halo("hii_n32_halo.npz", 32, 64, 25.0, 8.0, seed=303),
    "hii_n40_sfr": lambda: case_sfr("hii_n40_sfr.npz", 40, 31.25, 7.0, 8.0, seed=131),
    "pk_n32": lambda: case_pk("pk_n32.npz", 32, 0.75, seed=404),
    "pk_n64": lambda: case_pk("pk_n64.npz", 64, 1.5, seed=505, flags=(1,)),
    "t21_n32": lambda: case_t21("t21_n32.npz", 32, 25.0, seed=606, vel_comp=3, lya=False),
    "t21_n32_lya": lambda: case_t21("t21_n32_lya.npz", 32, 25.0, seed=707, vel_comp=1, lya=True),
    "halos_n64": lambda: case_halos("halos_n64.npz", synth.HaloWorkload(N=64, L_mpc=40.0, sigma=3.0, seed=808),
                                    6.0, 8.0, 1.0),
    "halos_n128_dense": lambda: case_halos("halos_n128_dense.npz",
                                           synth.HaloWorkload(N=128, L_mpc=100.0, sigma=4.0, seed=7, smooth=3),
                                           1.0, 2.0, 1.0),
    "halos_n96": lambda: case_halos("halos_n96.npz",
                                    synth.HaloWorkload(N=96, L_mpc=60.0, sigma=3.0, seed=1111, smooth=2),
                                    2.0, 3.0, 1.0),
    "halos_n120_sgrid": lambda: case_halos("halos_n120_sgrid.npz",
                                           synth.HaloWorkload(N=120, L_mpc=60.0, sigma=3.0, seed=1212, smooth=1,
                                                              subgrid=True, Mmin=1e9),
                                           6.0, 6.0, 1.0),
    "halos_n64_sgrid": lambda: case_halos("halos_n64_sgrid.npz",
                                          synth.HaloWorkload(N=64, L_mpc=40.0, sigma=3.0, seed=1010, smooth=1,
                                                             subgrid=True, Mmin=1e9),
                                          7.0, 8.0, 1.0),
    "sfr_n32": lambda: case_sfrd("sfr_n32.npz", 32, 64, 25.0, 7.0, 8.0, seed=1313),
    "sfr_n48_lya": lambda: case_sfrd("sfr_n48_lya.npz", 48, 100, 30.0, 8.0, 10.0, seed=1414, use_sfr=False,
                                     zminsfr=9.0),
}


if __name__ == "__main__":
    want = sys.argv[1:]
    for key, fn in CASES.items():
        if not want or any(key.startswith(w) for w in want):
            fn()

