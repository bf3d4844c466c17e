"""Failure paths, made without faulting, trapping or hanging the GPU.

* A bounded device wait that runs out: the TMA-pipelined passes' polls are
  lowered (sf21_hii_set_wait_limit) until they expire on an ordinary launch;
  each block records the error, drains its own copies and returns.  The run
  reports SF21_E_TIMEOUT and the context then runs cleanly.
* A device allocation that fails (sf21_hii_inject_alloc_failure): create and
  the first-use allocations return SF21_E_ALLOC and leave no device memory
  behind.
* The drop-in executable's file errors (get_HIIbubbles.c:209-211, :236-238,
  :263-265): a truncated density box, a missing SFR box and a truncated halo
  catalogue end the run with exit code 1 and the reference's message.
"""
import os
import subprocess

import numpy as np
import pytest
import torch

from helpers import load_golden
from simfast21_gb300 import synth

pytestmark = pytest.mark.gpu

SF21_E_ALLOC, SF21_E_TIMEOUT = 2, 4


def _boxes(N, L, seed=5):
    w = synth.Workload(N=N, L=L, zs=[7.5], zeta=40.0, Rmax=L / 4, factor=1.1, seed=seed)
    return synth.make_boxes(w, 7.5)


@pytest.mark.parametrize("path", [6, 7, 3, 8])
def test_wait_timeout_is_reported_and_the_context_recovers(hii, path):
    N, L = 128, 80.0
    sets = [(40.0, 20.0, 30)]
    delta, sfrd = _boxes(N, L)
    ref = hii.FilterBank(N, L, 0.71, sets, path=5)
    want, _ = ref.run_z(7.5, delta, sfrd)
    ref.close()
    fb = hii.FilterBank(N, L, 0.71, sets, path=path)
    fb.set_wait_limit(1)
    with pytest.raises(hii.HIIError) as ei:
        fb.run_z(7.5, delta, sfrd)
    assert ei.value.code == SF21_E_TIMEOUT
    fb.check()  # the flag was cleared by the report
    fb.set_wait_limit(0)
    got, _ = fb.run_z(7.5, delta, sfrd)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    # the device entry point: the error surfaces at the next check
    d, s = torch.from_numpy(delta).cuda(), torch.from_numpy(sfrd).cuda()
    out = torch.empty((1, N, N, N), device="cuda")
    fb.set_wait_limit(1)
    fb.run_z_device(7.5, d.data_ptr(), s.data_ptr(), out.data_ptr())
    with pytest.raises(hii.HIIError) as ei:
        fb.check()
    assert ei.value.code == SF21_E_TIMEOUT
    fb.set_wait_limit(0)
    fb.run_z_device(7.5, d.data_ptr(), s.data_ptr(), out.data_ptr())
    fb.check()
    assert np.array_equal(out.cpu().numpy().view(np.uint32), want.view(np.uint32))
    fb.close()


def _free():
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info()[0]


def test_allocation_failures_leave_nothing_behind(hii):
    N, L = 64, 50.0
    sets = [(30.0, 12.0, 30), (60.0, 20.0, 40)]
    delta, sfrd = _boxes(N, L)
    fb = hii.FilterBank(N, L, 0.71, sets)  # loads the modules, fills the tuning cache
    want, _ = fb.run_z(7.5, delta, sfrd)
    fb.close()
    base = _free()
    k = 1
    try:
        while True:
            hii.inject_alloc_failure(k)
            try:
                fb = hii.FilterBank(N, L, 0.71, sets)
            except hii.HIIError as e:
                assert e.code == SF21_E_ALLOC, str(e)
                assert _free() == base, k
                k += 1
                continue
            break
    finally:
        hii.inject_alloc_failure(0)
    assert k > 10  # every allocation of create was met once
    # first-use allocations of the host-buffer entry point (second staging box)
    hii.inject_alloc_failure(1)
    try:
        with pytest.raises(hii.HIIError) as ei:
            fb.run_z(7.5, delta, sfrd)
        assert ei.value.code == SF21_E_ALLOC
    finally:
        hii.inject_alloc_failure(0)
    got, _ = fb.run_z(7.5, delta, sfrd)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    fb.close()
    assert _free() == base


def _base_dir(tmp_path, name, sfr=True):
    from test_gpu_driver import _write_base
    g = load_golden(name)
    return _write_base(tmp_path, g, sfr=sfr), g


def _run(base):
    from simfast21_gb300 import build
    build.build()
    return subprocess.run([build.DRIVER, base], capture_output=True, text=True, timeout=300)


def test_driver_truncated_density_box(hii, tmp_path):
    base, g = _base_dir(tmp_path, "hii_n32_sfr.npz")
    sp = g["params"]
    path = os.path.join(base, synth.box_name("delta", float(g["zs"][0]), sp.N, sp.L_file))
    data = open(path, "rb").read()
    with open(path, "wb") as f:
        f.write(data[: len(data) - 4])
    r = _run(base)
    assert r.returncode == 1
    assert "Error reading deltanl file" in r.stdout


def test_driver_missing_sfr_box(hii, tmp_path):
    base, g = _base_dir(tmp_path, "hii_n32_sfr.npz")
    sp = g["params"]
    os.remove(os.path.join(base, synth.box_name("sfrd", float(g["zs"][0]), sp.N, sp.L_file)))
    r = _run(base)
    assert r.returncode == 1
    assert "Error reading SFR file" in r.stdout


def test_driver_truncated_halo_catalogue(hii, tmp_path):
    base, g = _base_dir(tmp_path, "hii_n32_halo.npz", sfr=False)
    sp = g["params"]
    z = float(g["zs"][0])
    path = os.path.join(base, f"Halos/halonl_z{z:.3f}_N{sp.N_halo}_L{sp.L_file:.1f}.dat.catalog")
    data = open(path, "rb").read()
    with open(path, "wb") as f:
        f.write(data[: 8 + 16 * 3 + 5])  # the count says more records than follow
    r = _run(base)
    assert r.returncode == 1
    assert "Error reading halo catalogue" in r.stdout
