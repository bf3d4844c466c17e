"""Benchmark of the HII-bubble filter bank (one JSON line on rank 0).

Workload (default): the batched form at 512^3 -- L = 300 Mpc/h, one
redshift z = 7, 64 efficiency / Rmax parameter sets (zeta log-uniform on
[10, 100], Rmax uniform on [10, 60] Mpc/h, radius factor 1.05, so radius
counts are uneven), seeded synthetic density and SFRD boxes.  A step is one
full stage pass: prologue, shared forward transform, every set's radius loop,
dilation, fill and cap, giving 64 xHII boxes.

metric: voxel*radii/s = N^3 * (radii summed over the sets) / step time.
value : device-resident inputs, CUDA events on the launch stream; the timed
        steps are the production path (one CUDA graph launch per step); the
        per-kernel split comes from a separate event-instrumented step.
e2e   : the same through the host-buffer C-ABI call sf21_hii_run_z (pinned
        host inputs copied in, 64 xHII boxes copied out into pinned host
        memory while the next set computes, neutral fractions summed on the
        host) -- the reference-facing path.
--impl reference: the CPU restatement of get_HIIbubbles.c (oracle/, FFTW-API
        shim, OpenMP on all host cores) timed on bounded samples of the
        workload (the front of a redshift and a spread of radii of the median
        set) and extrapolated to the whole workload (CpuSampler).
Multi-GPU (torchrun): independent replicas (each rank runs the full
workload on its GPU; scaling "weak"), barrier + max over ranks.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from simfast21_gb300 import params as P  # noqa: E402
from simfast21_gb300 import synth  # noqa: E402


# ---------------------------------------------------------------------------
METRIC = "HII filter-bank voxel*radii/s"


def workload(name: str, rank: int = 0):
    """(N, L, z, sets, seed, label) of a named workload.  Under torchrun each
    rank is one replica with its own parameter sets (the batched workloads
    draw them from a rank-dependent seed): per-GPU work is fixed, units
    differ between ranks (weak scaling, no collective on the data path)."""
    h = 0.71
    if name == "batched512":
        N, L, z, seed = 512, 300.0, 7.0, 1236
        rng = np.random.default_rng(seed + 7919 * rank)
        zetas = np.exp(rng.uniform(np.log(10.0), np.log(100.0), 64))
        rmaxs = rng.uniform(10.0, 60.0, 64)
    elif name == "batched256":
        N, L, z, seed = 256, 150.0, 7.0, 1236
        rng = np.random.default_rng(seed + 7919 * rank)
        zetas = np.exp(rng.uniform(np.log(10.0), np.log(100.0), 16))
        rmaxs = rng.uniform(5.0, 30.0, 16)
    elif name == "single512":
        N, L, z, seed = 512, 300.0, 7.0, 1236
        zetas, rmaxs = np.array([30.0]), np.array([35.0])
    elif name == "single256":
        N, L, z, seed = 256, 150.0, 7.0, 1236
        zetas, rmaxs = np.array([30.0]), np.array([30.0])
    elif name == "single600":  # the reference's default N_smoothed (2-3-5 transforms)
        N, L, z, seed = 600, 150.0 * h, 7.0, 1236
        zetas, rmaxs = np.array([30.0]), np.array([50.0 * h])
    elif name == "plain128":
        N, L, z, seed = 128, 100.0, 8.0, 1234
        zetas, rmaxs = np.array([30.0]), np.array([50.0])
    else:
        raise SystemExit(f"unknown workload {name}")
    dx = L / N
    sets = []
    for zt, rm in zip(zetas, rmaxs):
        # ini values are in Mpc (bubble_Rmax = Rmax/h); the stage multiplies by h
        rmax = min((rm / h) * h, L / 2.0)
        factor = 1.1 if name == "plain128" else 1.05
        nb = max(1, int(round(math.log(rmax / dx) / math.log(factor))))
        sets.append((float(zt), float(rmax), nb))
    return dict(N=N, L=L, z=z, hubble=h, sets=sets, seed=seed, name=name)


def reduce_across_ranks(ms: float, units: float, device):
    """(max of ms, sum of units) over the ranks of the default process group
    (identity without one): the job's step time and the units all ranks
    processed in it."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return ms, units
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    u = torch.tensor([units], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t.item()), float(u.item())


def describe(w):
    return {"batched512": "HII filter bank, batched: 512^3, L=300 Mpc/h, z=7, 64 sets "
                          "(zeta log-U[10,100], Rmax U[10,60] Mpc/h, factor 1.05)",
            "batched256": "HII filter bank, batched: 256^3, L=150 Mpc/h, z=7, 16 sets",
            "single256": "HII filter bank: 256^3, L=150 Mpc/h, z=7, 1 set (zeta=30, Rmax=30 Mpc/h, factor 1.05)",
            "single512": "HII filter bank: 512^3, L=300 Mpc/h, z=7, 1 set (zeta=30, Rmax=35 Mpc/h, factor 1.05)",
            "single600": "HII filter bank: 600^3 (the reference's default N_smoothed, 2-3-5 transforms), "
                         "L=106.5 Mpc/h, z=7, 1 set (zeta=30, Rmax=35.5 Mpc/h, factor 1.05)",
            "plain128": "HII filter bank: 128^3, L=100 Mpc/h, z=8, zeta=30, Rmax=50, factor 1.1"}[w["name"]]


def total_radii(w):
    return sum(len(P.radii(s[1], w["L"] / w["N"], s[2])[0]) for s in w["sets"])


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for i, n in enumerate(names):
                if len(r) > 5 + i and r[5 + i].lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "samples": len(self.rows), "reasons": sorted(reasons)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ---------------------------------------------------------------------------
class CpuSampler:
    """The CPU restatement of get_HIIbubbles.c (oracle/, FFTW-API shim with
    the project's own FFT -- FFTW is absent on both machines -- OpenMP on the
    host cores) timed on a bounded sample of the workload and extrapolated
    to all of it.  The sampled set is the one with the median radius count;
    the sample radii are four of its FFT-branch radii (largest, two middle,
    smallest) and two of its small-R radii.  Each step times the front of a
    redshift (prologue, source conversion, fill, both forward transforms)
    and two of the sample radii in turn.  The reference runs one parameter
    set per process, so it pays the front per set:
    t_set = t_front + n_fft(set) * mean t_fft + n_small(set) * mean t_small,
    and the rate is N^3 * (all radii) / (sum of t_set over the sets)."""

    def __init__(self, w, nthreads: int):
        from oracle import oracle as O
        O.build()
        self.O, self.w, self.nthreads = O, w, nthreads
        N, dx = w["N"], w["L"] / w["N"]
        self.counts = []
        for zt, rmax, nb in w["sets"]:
            R, nf = P.radii(rmax, dx, nb)
            self.counts.append((nf, len(R) - nf))
        order = sorted(range(len(w["sets"])), key=lambda i: sum(self.counts[i]))
        self.set = order[len(order) // 2]
        nf, ns = self.counts[self.set]
        self.idx = [0, nf // 3, (2 * nf) // 3, nf - 1] + ([nf, nf + ns - 1] if ns else [])
        self.nfft = nf
        self.delta, self.sfrd = synth.make_boxes(synth.Workload(N=N, L=w["L"], zs=[w["z"]], seed=w["seed"]),
                                                 w["z"])
        self.t_front, self.t_r = [], {i: [] for i in self.idx}
        self.k = 0

    def step(self) -> float:
        """One bounded sample; returns its wall seconds."""
        zt, rmax, nb = self.w["sets"][self.set]
        p = self.O.params(self.w["N"], self.w["L"], self.w["hubble"], rmax, nb, zt, nthreads=self.nthreads)
        pick = [self.idx[(2 * self.k + j) % len(self.idx)] for j in range(2)]
        self.k += 1
        t0 = time.perf_counter()
        front, tr = self.O.time_radii(p, self.w["z"], self.delta, self.sfrd, pick)
        dt = time.perf_counter() - t0
        self.t_front.append(front)
        for i, t in zip(pick, tr):
            self.t_r[i].append(t)
        return dt

    def estimate(self):
        """(voxel*radii/s of the whole workload, details)."""
        tf = float(np.mean(self.t_front))
        fft = [np.mean(v) for i, v in self.t_r.items() if v and i < self.nfft]
        small = [np.mean(v) for i, v in self.t_r.items() if v and i >= self.nfft]
        t_fft = float(np.mean(fft))
        t_small = float(np.mean(small)) if small else t_fft
        total = sum(tf + nf * t_fft + ns * t_small for nf, ns in self.counts)
        units = float(self.w["N"]) ** 3 * sum(nf + ns for nf, ns in self.counts)
        return units / total, {"front_s": tf, "fft_radius_s": t_fft, "small_radius_s": t_small,
                               "workload_s_extrapolated": total}

    def describe(self, n_steps: int) -> str:
        nf, ns = self.counts[self.set]
        return (f"extrapolated: {n_steps} samples of set {self.set} ({nf}+{ns} radii) of the {self.w['N']}^3 "
                f"workload, each the front of a redshift (prologue, fill, forward transforms) plus two of the "
                f"radius indices {self.idx}; rate = N^3 * all radii / sum over sets of (front + radii x mean "
                f"radius time); FFT = the project's FFTW-API shim, not FFTW")


def run_reference(args, w, rank):
    if rank != 0:
        return
    ncpu = os.cpu_count() or 1
    cs = CpuSampler(w, ncpu)
    for _ in range(args.warmup):
        cs.step()
    cs.t_front.clear()
    for v in cs.t_r.values():
        v.clear()
    times = [cs.step() for _ in range(max(args.steps, 3))]
    v, detail = cs.estimate()
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v,
        "unit": "voxel*radii/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * float(np.mean(times)), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": describe(w), "form": "one parameter set per process (reference structure)",
                   "flush": "inputs larger than L2"},
        "cpu_baseline": {"value": v, "unit": "voxel*radii/s", "cores": ncpu, "kind": "port",
                         "sample": cs.describe(len(times)), **detail},
        "e2e": {"value": v, "unit": "voxel*radii/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


# radius pipelines of the library (FilterBank.path): short and long names
PIPELINES = {
    1: ("three_pass", "three axis passes"),
    2: ("plane", "cluster plane pass + kx pass"),
    3: ("tma_ky", "three axis passes, ky pass TMA-pipelined"),
    4: ("tma_ky_kx", "three axis passes, ky and kx passes TMA-pipelined"),
    5: ("cb_three_pass", "column-block-major work boxes, three axis passes"),
    6: ("cb_tma_ky", "column-block-major work boxes, ky pass TMA-pipelined"),
    7: ("cb_tma_ky_kx", "column-block-major work boxes, ky and kx passes TMA-pipelined"),
    8: ("cb_fused_l2", "column-block-major work boxes, c-axis pass + one persistent ky/kx launch through L2"),
}


# ---------------------------------------------------------------------------
def grad_metrics(N, L, z, zeta, rmax, factor, seed, stream, dev, kmax=0):
    """Forward criterion and VJP times (CUDA events on the launch stream) and
    device memory held by the context during them."""
    import torch
    from simfast21_gb300 import hii
    free0, _ = torch.cuda.mem_get_info()
    delta, sfrd = synth.make_boxes_torch(N, L, z, seed, device="cuda")
    nb = max(1, int(round(math.log(rmax / (L / N)) / math.log(factor))))
    fb = hii.FilterBank(N, L, 0.71, [(zeta, rmax, nb)], device=dev, kmax=kmax)
    C = torch.empty_like(delta)
    A = torch.empty(delta.shape, dtype=torch.uint8, device="cuda")
    g = torch.rand(delta.shape, device="cuda", dtype=torch.float32)
    gd = torch.empty_like(delta)
    gs = torch.empty_like(delta)
    sptr = stream.cuda_stream

    def fwd():
        fb.criterion_device(z, delta.data_ptr(), sfrd.data_ptr(), C.data_ptr(), A.data_ptr(), stream=sptr)

    def bwd():
        fb.vjp_device(z, delta.data_ptr(), sfrd.data_ptr(), g.data_ptr(), gd.data_ptr(), gs.data_ptr(),
                      stream=sptr, want_zeta=False)

    fwd()
    bwd()
    torch.cuda.synchronize()
    e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    reps = 2
    e[0].record(stream)
    for _ in range(reps):
        fwd()
    e[1].record(stream)
    for _ in range(reps):
        bwd()
    e[2].record(stream)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    fms = e[0].elapsed_time(e[1]) / reps
    bms = e[1].elapsed_time(e[2]) / reps
    nr = len(fb.radii(0)[0])
    nf = fb.radii(0)[1]
    fb.close()
    del delta, sfrd, C, A, g, gd, gs
    torch.cuda.empty_cache()
    return {"N": N, "radii_fft_branch": nf, "radii": nr, "fwd_ms": fms, "bwd_ms": bms, "bwd_over_fwd": bms / fms,
            "device_bytes_in_use": int(free0 - free1),
            "checkpoint": "uint8 argmax radius per voxel; filtered fields recomputed"}


def halo_metrics(rank: int, with_cpu: bool, N: int = 512, z: float = 7.0, reps: int = 3):
    """Halo finder of get_halos.c on a seeded Gaussian z = 0 density box
    (P(k) ~ k^-2, rms 4 per cell), L = 100 Mpc at 512^3 (the same cell size at
    other N), default halo keys with the subgrid cycle on: device time per
    redshift, end to end with the catalogue copied to host memory, and the CPU
    restatement at 256^3."""
    import ctypes

    from simfast21_gb300 import halos
    L_mpc = 100.0 * N / 512
    w = synth.HaloWorkload(N=N, L_mpc=L_mpc, sigma=4.0, seed=11, subgrid=True)
    ini = synth.halo_ini_text(w, z, z, 1.0)
    d = w.density()
    hf = halos.HaloFinder(halos.config_from_ini(halos.parse_ini(ini)))
    t0 = time.perf_counter()
    hf.set_density(d)
    dens_ms = (time.perf_counter() - t0) * 1e3
    n = ctypes.c_long(0)
    L = hf._L
    dev, e2e = [], []
    for r in range(reps + 1):
        hf.set_rng(None)
        t0 = time.perf_counter()
        hf._check(L.sf21_halo_find_z(hf._h, z, ctypes.byref(n)))
        t1 = time.perf_counter()
        out = np.empty(n.value, halos.HALO_DTYPE)
        hf._check(L.sf21_halo_fetch(hf._h, out.ctypes.data, 0, n.value))
        t2 = time.perf_counter()
        if r:  # first call: warm-up (allocations)
            dev.append((t1 - t0) * 1e3)
            e2e.append((t2 - t0) * 1e3)
    counts = hf.counts()
    hf.close()
    ms, ms_e2e = float(np.median(dev)), float(np.median(e2e))
    res = {"N": N, "L_mpc": L_mpc, "z": z, "subgrid": True, "halos": int(n.value),
           "excursion_set_halos": int(counts[:-2].sum()), "cell_cycle_halos": int(counts[-2]),
           "subgrid_halos": int(counts[-1]), "set_density_ms": dens_ms, "ms_per_redshift": ms,
           "cells_per_s": N ** 3 / (ms / 1e3), "e2e_ms_per_redshift": ms_e2e,
           "e2e_cells_per_s": N ** 3 / (ms_e2e / 1e3), "d2h_bytes": int(n.value) * 16}
    if rank == 0 and with_cpu:
        from oracle import halo as OH
        Nc = 256
        wc = synth.HaloWorkload(N=Nc, L_mpc=L_mpc * Nc / N, sigma=4.0, seed=11, subgrid=True)
        pc = OH.params_from_ini(OH.parse_ini(synth.halo_ini_text(wc, z, z, 1.0)))
        dc = wc.density()
        t0 = time.perf_counter()
        OH.find_z(pc, z, dc, OH.taus_seed(0))
        cpu_s = time.perf_counter() - t0
        res["cpu_baseline"] = {"value": Nc ** 3 / cpu_s, "unit": "cells/s", "cores": os.cpu_count() or 1,
                               "kind": "port", "sample": f"restatement of get_halos.c (FFTW-API shim, OpenMP "
                                                         f"filter loop, serial overlap and subgrid loops) at "
                                                         f"{Nc}^3, same cell size and parameters, {cpu_s:.1f} s"}
    return res


def sfr_catalogue(n: int, N_halo: int, seed: int):
    """Seeded Halo_t catalogue with the halo finder's mass structure: masses
    on its schedule (halo_Mmin = 1e8 Msun, halo_dlm = 0.2, up to 1e12: 21
    distinct values), abundance falling as dn/dlnM ~ M^-0.9; uniform positions
    in N_halo cells."""
    from simfast21_gb300.halos import HALO_DTYPE
    rng = np.random.default_rng(seed)
    cat = np.empty(n, HALO_DTYPE)
    sched = 1e8 * 10.0 ** (0.2 * np.arange(21))
    p = sched ** -0.9
    cat["Mass"] = sched[rng.choice(len(sched), size=n, p=p / p.sum())].astype(np.float32)
    for ax in ("x", "y", "z"):
        cat[ax] = (rng.random(n, dtype=np.float32) * np.float32(N_halo)).astype(np.float32)
    return cat


def sfr_metrics(rank: int, with_cpu: bool, N_halo: int = 1200, N: int = 600, n_halos: int = 20_000_000,
                z: float = 8.0, reps: int = 3):
    """Star-formation-rate stage of get_SFR.c at the reference's default grids
    (N_halo 1200 -> N_smoothed 600, L = 150 Mpc, h = 0.7) on a seeded
    catalogue: device time per redshift with the catalogue resident (CUDA
    events on the launching stream), end to end through sf21_sfr_box (host
    catalogue in, host box out), and the CPU restatement on the same inputs."""
    import torch

    from simfast21_gb300 import sfr
    L = 150.0 * 0.7
    cat = sfr_catalogue(n_halos, N_halo, seed=2024)
    s = sfr.SFRBox(N_halo, N, L)
    d_cat = torch.from_numpy(cat.view(np.uint8)).cuda()
    d_out = torch.empty(N ** 3, dtype=torch.float32, device="cuda")
    st = torch.cuda.current_stream()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    dev = []
    for r in range(reps + 1):
        torch.cuda.synchronize()
        ev0.record(st)
        s.box_device(z, n_halos, d_cat.data_ptr(), d_out.data_ptr(), st.cuda_stream)
        ev1.record(st)
        torch.cuda.synchronize()
        if r:
            dev.append(ev0.elapsed_time(ev1))
    host_out = np.empty((N,) * 3, np.float32)
    e2e = []
    L_ = s._L
    for r in range(reps + 1):
        t0 = time.perf_counter()
        s._check(L_.sf21_sfr_box(s._h, z, n_halos, cat.ctypes.data, host_out.ctypes.data, None))
        if r:
            e2e.append((time.perf_counter() - t0) * 1e3)
    s.close()
    ms, ms_e2e = float(np.median(dev)), float(np.median(e2e))
    res = {"N_halo": N_halo, "N_smoothed": N, "halos": n_halos, "z": z, "ms_per_redshift": ms,
           "halos_per_s": n_halos / (ms / 1e3), "e2e_ms_per_redshift": ms_e2e,
           "e2e_halos_per_s": n_halos / (ms_e2e / 1e3), "h2d_bytes": 16 * n_halos, "d2h_bytes": 4 * N ** 3}
    if rank == 0 and with_cpu:
        from oracle import oracle as O
        p = O.params(N, L, 0.7, L / 2, 10, 30.0, N_halo=N_halo, nthreads=os.cpu_count() or 1)
        t0 = time.perf_counter()
        O.sfrd_box(p, z, cat)
        cpu_s = time.perf_counter() - t0
        res["cpu_baseline"] = {"value": n_halos / cpu_s, "unit": "halos/s", "cores": os.cpu_count() or 1,
                               "kind": "port", "sample": f"restatement of get_SFR.c (serial CIC, OpenMP "
                                                         f"smooth_box, serial mean), same catalogue and grids, "
                                                         f"{cpu_s:.1f} s"}
    return res


def hii600_metrics(reps: int = 3):
    """The HII stage at the reference's default N_smoothed = 600 (2-3-5
    transforms; workload single600): device time per redshift with CUDA
    events on the launching stream, per-kernel split, and end to end through
    sf21_hii_run_z with host boxes."""
    import torch
    from simfast21_gb300 import hii
    w = workload("single600")
    N = w["N"]
    delta, sfrd = synth.make_boxes(synth.Workload(N=N, L=w["L"], zs=[w["z"]], seed=w["seed"]), w["z"])
    fb = hii.FilterBank(N, w["L"], w["hubble"], w["sets"])
    R = sum(len(fb.radii(s)[0]) for s in range(len(w["sets"])))
    d_delta = torch.from_numpy(delta).cuda()
    d_src = torch.from_numpy(sfrd).cuda()
    d_x = torch.empty((len(w["sets"]), N, N, N), dtype=torch.float32, device="cuda")
    stream = torch.cuda.Stream()
    sptr = stream.cuda_stream

    def step():
        fb.run_z_device(w["z"], d_delta.data_ptr(), d_src.data_ptr(), d_x.data_ptr(), stream=sptr)

    for _ in range(3):
        step()
    torch.cuda.synchronize()
    fb.profile(True)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(reps):
        step()
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / reps
    prof = fb.profile_read()
    fb.profile(False)
    t0 = time.perf_counter()
    fb.run_z(w["z"], delta, sfrd)
    e2e_ms = (time.perf_counter() - t0) * 1e3
    fb.close()
    del d_delta, d_src, d_x
    return {"workload": describe(w), "radii": R, "ms_per_redshift": ms,
            "voxel_radii_per_s": N ** 3 * R / (ms / 1e3), "e2e_ms_per_redshift": e2e_ms,
            "kernels_ms_per_redshift": {k: round(v[0] / reps, 3) for k, v in prof.items() if v[1] > 0}}


def run_ours(args, w, rank, world):
    import torch
    from simfast21_gb300 import build as B
    from simfast21_gb300 import hii

    B.build()
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    N = w["N"]
    n3 = N ** 3
    nsets = len(w["sets"])
    delta, sfrd = synth.make_boxes(synth.Workload(N=N, L=w["L"], zs=[w["z"]], seed=w["seed"]), w["z"])
    fb = hii.FilterBank(N, w["L"], w["hubble"], w["sets"], device=dev, kmax=args.kmax, path=args.path)
    path, tuned = fb.path()
    R_total = sum(len(fb.radii(s)[0]) for s in range(nsets))
    units = float(n3) * R_total
    d_delta = torch.from_numpy(delta).cuda()
    d_src = torch.from_numpy(sfrd).cuda()
    d_x = torch.empty((nsets, N, N, N), dtype=torch.float32, device="cuda")
    # a dedicated stream: the library's kernels and the timing events share it
    stream = torch.cuda.Stream()
    sptr = stream.cuda_stream

    def step():
        fb.run_z_device(w["z"], d_delta.data_ptr(), d_src.data_ptr(), d_x.data_ptr(), stream=sptr)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    torch.cuda.synchronize()
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    # timed region: the production path (one CUDA graph launch per step, no
    # per-kernel events)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            step()
        ev1.record(stream)
        torch.cuda.synchronize()
    barrier()
    ms = ev0.elapsed_time(ev1) / args.steps
    # per-kernel breakdown from separate, event-instrumented steps (the graph
    # is bypassed while timing is on)
    prof_steps = 1
    fb.profile(True)
    for _ in range(prof_steps):
        step()
    torch.cuda.synchronize()
    prof = fb.profile_read()
    fb.profile(False)
    ms, job_units = reduce_across_ranks(ms, units, "cuda")
    value = job_units / (ms / 1e3)

    # e2e through the host-buffer C-ABI call
    h_delta = torch.from_numpy(delta).pin_memory().numpy()
    h_src = torch.from_numpy(sfrd).pin_memory().numpy()
    h_out = torch.empty((nsets, N, N, N), dtype=torch.float32, pin_memory=True).numpy()
    e2e_steps = max(1, min(args.steps, 2))
    fb.run_z(w["z"], h_delta, h_src, out=h_out)  # warm (allocates nothing new)
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        x, neutral = fb.run_z(w["z"], h_delta, h_src, out=h_out)
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    barrier()
    e2e_s, _ = reduce_across_ranks(e2e_s, units, "cuda")
    e2e_val = job_units / e2e_s

    # roofline of the dominant kernel kind (largest device-time share)
    hbm, peak_kind = peaks()
    steps = prof_steps
    kinds = {k: v for k, v in prof.items() if v[1] > 0}
    dom = max(kinds, key=lambda k: kinds[k][0])
    dom_ms, dom_n = kinds[dom]
    per_launch_ms = dom_ms / dom_n
    # algorithmic bytes per launch (complex64 boxes: 8 B per voxel)
    nbatch = kinds.get("inv_cols_a_test", kinds.get("inv_cols_ba_fused", (0, 1)))[1] / steps
    K_avg = R_total / nbatch
    alg = {
        "inv_rows_filter": n3 * 8.0 * (1 + K_avg),      # spectrum read once, K boxes written
        "inv_cols_b": n3 * 16.0 * K_avg,                 # K boxes read + written
        "inv_cols_a_test": n3 * (8.0 * K_avg + 2.0),     # K boxes read, first-hit byte r/w
        "inv_cols_ba_fused": n3 * (8.0 * K_avg + 2.0),   # K boxes read from DRAM (ky), kx through L2
        "inv_plane_filter": n3 * 8.0 * (1 + K_avg),      # spectrum read once, K boxes written
    }.get(dom, None)
    achieved = alg / (per_launch_ms / 1e3) / 1e9 if alg else None
    # DRAM traffic per launch (dram__bytes_read + dram__bytes_write) from the
    # ncu capture of the same kernels at 512^3, K = 8, per voxel*radius
    # (profiles/radius_kernels_cb_single512.md), scaled to this launch's radii
    traffic_b = {"inv_cols_b": 15.94, "inv_cols_a_test": 8.00, "inv_rows_filter": 8.94}.get(dom)
    traffic = traffic_b * n3 * K_avg if (traffic_b and path >= 5) else None
    # whole radius pipeline against the 16 B per voxel*radius algorithmic traffic
    pipe_ms = sum(kinds.get(k, (0, 0))[0] for k in ("inv_rows_filter", "inv_cols_b", "inv_cols_a_test",
                                                     "inv_plane_filter", "inv_cols_ba_fused"))
    pipe_gbs = 16.0 * units * steps / (pipe_ms / 1e3) / 1e9 if pipe_ms else None

    # the plain one-radius-per-launch form on one parameter set (same box)
    d_plain = torch.empty((N, N, N), dtype=torch.float32, device="cuda")
    plain_set = 0
    fb.run_z_plain_device(w["z"], d_delta.data_ptr(), d_src.data_ptr(), d_plain.data_ptr(), s=plain_set, stream=sptr)
    torch.cuda.synchronize()
    p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    p0.record(stream)
    fb.run_z_plain_device(w["z"], d_delta.data_ptr(), d_src.data_ptr(), d_plain.data_ptr(), s=plain_set, stream=sptr)
    p1.record(stream)
    torch.cuda.synchronize()
    plain_ms = p0.elapsed_time(p1)
    plain_units = float(n3) * len(fb.radii(plain_set)[0])
    plain = {"value": plain_units / (plain_ms / 1e3), "unit": "voxel*radii/s", "ms": plain_ms,
             "set": plain_set, "radii": len(fb.radii(plain_set)[0]),
             "batched_per_set_speedup": (units / (ms / 1e3)) / (plain_units / (plain_ms / 1e3))}
    del d_plain

    # differentiation: criterion forward and hand-written VJP (bwd/fwd),
    # 256^3 (L=200, z=8, zeta=30, Rmax=60, factor 1.05) and, unless --no-grad-large,
    # 1024^3 (L=500, z=7, Rmax=80, factor 1.12) with peak HBM
    grad = None
    if not args.no_grad:
        del d_x
        torch.cuda.synchronize()
        grad = {"box256": grad_metrics(256, 200.0, 8.0, 30.0, 60.0, 1.05, 4321, stream, dev)}
        if not args.no_grad_large:
            grad["box1024"] = grad_metrics(1024, 500.0, 7.0, 30.0, 80.0, 1.12, 5555, stream, dev, kmax=4)

    # power spectrum of the density box (tools/power3d_f.c, Bartlett window):
    # the library's GPU form (device box in, binned P(k) on the host) and,
    # as its CPU baseline, the restatement of the tool on the host cores
    pk = None
    if not args.no_pk:
        dl = w["L"] / N
        fb.power_spectrum_device(d_delta.data_ptr(), dl, 1, stream=sptr)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        reps = 3
        for _ in range(reps):
            fb.power_spectrum_device(d_delta.data_ptr(), dl, 1, stream=sptr)
        pk_ms = (time.perf_counter() - t0) / reps * 1e3
        pk = {"N": N, "window": "Bartlett", "gpu_ms": pk_ms,
              "gpu_voxels_per_s": n3 / (pk_ms / 1e3)}
        if rank == 0 and not args.no_cpu_baseline:
            from oracle import pk_oracle as K
            t0 = time.perf_counter()
            K.power_spectrum(delta, dl, 1)
            cpu_ms = (time.perf_counter() - t0) * 1e3
            pk["cpu_baseline"] = {"ms": cpu_ms, "cores": os.cpu_count() or 1, "kind": "port",
                                  "sample": "restatement of tools/power3d_f.c (numpy/scipy float32 FFT), "
                                            "same box"}

    # 21-cm brightness temperature of the density box with set 0's xHII
    # (t21.c, Lya/X-rays off): host boxes in and out through sf21_t21_run_z,
    # and the restatement of t21.c (double, numpy) on the host as its baseline
    t21 = None
    if not args.no_pk:
        xh = np.ascontiguousarray(x[0])
        fb.t21(w["z"], delta, xh)
        t0 = time.perf_counter()
        fb.t21(w["z"], delta, xh)
        g_ms = (time.perf_counter() - t0) * 1e3
        t21 = {"N": N, "gpu_ms_host_buffers": g_ms}
        if rank == 0 and not args.no_cpu_baseline:
            from oracle import t21_oracle as T
            t0 = time.perf_counter()
            T.t21_box(w["z"], delta, xh, w["L"], T.Cosmo(0.27, 0.046, 0.73, w["hubble"]), 3)
            t21["cpu_baseline"] = {"ms": (time.perf_counter() - t0) * 1e3, "cores": os.cpu_count() or 1,
                                   "kind": "port", "sample": "restatement of t21.c (numpy, double), same boxes"}

    # excursion-set halo finder (get_halos.c) through the C-ABI: one redshift
    # of a 512^3 box per call, the catalogue left on the device (value) or
    # fetched to host memory (e2e); the restatement of get_halos.c on the host
    # cores at 256^3 (the same generator and parameters) as its baseline
    halo = None
    if not args.no_halos:
        halo = halo_metrics(rank, not args.no_cpu_baseline)

    # star-formation-rate stage (get_SFR.c) at the reference's default grids
    sfr_res = None
    if not args.no_halos:
        sfr_res = sfr_metrics(rank, not args.no_cpu_baseline)

    # the HII stage at the reference's default 600^3 (2-3-5 transforms)
    hii600 = None
    if not args.no_600:
        try:
            hii600 = hii600_metrics()
        except Exception as e:  # reported in the line, never fatal to the headline measurement
            hii600 = {"error": str(e)[:300]}

    # CPU baseline (rank 0 only): the restatement on the host cores, a
    # bounded sample extrapolated to the workload
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        ncpu = os.cpu_count() or 1
        cs = CpuSampler(w, ncpu)
        n_cpu = 3
        t_cpu = sum(cs.step() for _ in range(n_cpu))
        v, detail = cs.estimate()
        cpu = {"value": v, "unit": "voxel*radii/s", "cores": ncpu, "kind": "port",
               "sample": cs.describe(n_cpu) + f"; {t_cpu:.1f} s of samples", **detail}

    launches = int(sum(v[1] for v in kinds.values()) // steps)
    if rank == 0:
        out = {
            "metric": METRIC,
            "value": value, "unit": "voxel*radii/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded lognormal density + SFRD boxes)",
            "config": {"workload": describe(w), "form": "batched (one shared forward transform, "
                       "one CUDA graph per step)", "N": N, "sets": nsets, "radii_total": R_total,
                       "pipeline": PIPELINES[path][1], "batch_radii": fb.batch_radii(),
                       "tuned_batch_ms": {PIPELINES[p][0]: tuned[p] for p in PIPELINES},
                       "flush": "inputs larger than L2 (every box >= 537 MB)"},
            "e2e": {"value": e2e_val, "unit": "voxel*radii/s",
                    "h2d_bytes_per_step": 2 * 4 * n3, "d2h_bytes_per_step": nsets * 4 * n3},
            "gpu_launches": launches,
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm,
                         "unit": "GB/s", "frac": (achieved / hbm) if achieved else None,
                         "peak_source": peak_kind, "traffic": traffic,
                         "traffic_source": "ncu capture, 512^3 K=8, scaled per launch" if traffic else None,
                         "pipeline_16B_per_voxel_radius_gbs": pipe_gbs,
                         "pipeline_frac": (pipe_gbs / hbm) if pipe_gbs else None,
                         "step_16B_per_voxel_radius_frac": value / world * 16.0 / (hbm * 1e9)},
            "kernels_ms_per_step": {k: round(v[0] / steps, 3) for k, v in kinds.items()},
            "kernels_source": f"{prof_steps} separate step(s) with CUDA events around each launch",
            "clocks": clk.summary(),
            "plain_gpu": plain,
            "differentiation": grad,
            "power_spectrum": pk,
            "t21": t21,
            "halo_finder": halo,
            "sfr": sfr_res,
            "hii_600": hii600,
            "cpu_baseline": cpu,
        }
        print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="batched512")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--kmax", type=int, default=0, help="radii per spectrum read (0 = library default)")
    ap.add_argument("--no-grad", action="store_true", help="skip the bwd/fwd measurement")
    ap.add_argument("--no-pk", action="store_true", help="skip the power-spectrum and 21-cm measurements")
    ap.add_argument("--no-halos", action="store_true",
                    help="skip the halo-finder and star-formation-rate measurements")
    ap.add_argument("--halos-only", type=int, default=0, metavar="N",
                    help="run only the halo-finder measurement at N^3 and print it (profiling entry point)")
    ap.add_argument("--no-600", action="store_true", help="skip the 600^3 (reference default size) HII measurement")
    ap.add_argument("--sfr-only", action="store_true",
                    help="run only the star-formation-rate measurement and print it (profiling entry point)")
    ap.add_argument("--no-grad-large", action="store_true", help="skip fwd+bwd at 1024^3 (peak HBM)")
    ap.add_argument("--path", type=int, default=0,
                    help="radius pipeline: 0 = tuned, else one of PIPELINES")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.halos_only:
        from simfast21_gb300 import build as B
        B.build()
        print(json.dumps({"halo_finder": halo_metrics(rank, not args.no_cpu_baseline, N=args.halos_only)}))
        return
    if args.sfr_only:
        from simfast21_gb300 import build as B
        B.build()
        print(json.dumps({"sfr": sfr_metrics(rank, not args.no_cpu_baseline)}))
        return
    w = workload(args.workload, rank)
    if args.impl == "reference":
        run_reference(args, w, rank)
        return
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    run_ours(args, w, rank, world)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
