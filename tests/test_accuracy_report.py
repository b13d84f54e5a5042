"""Accuracy of the device path against the FP64 oracle on the benchmark configurations: the
64x64x512 cell over its whole run (4 passes x 200 fixed split steps, lens mirror), and four
split steps of the 256x256x2048 and 512x512x1024 cells.  Each case prints one line: the relative
L2 error of the output field, of its power spectrum sum_xy |A(x, y, omega)|^2, and the
difference between the device's and the oracle's relative energy change (plasma absorption
makes the physical energy change nonzero).  Run with -s to see the lines."""
import json

import numpy as np
import pytest

import oracle
from mpc_gb300 import inputs

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _power_spectrum(A, p):
    import torch
    F = torch.fft.fft(torch.from_numpy(A.reshape(p.Nt, p.Ny * p.Nx)).cuda(), dim=0)
    return (F.abs() ** 2).sum(dim=1).cpu().numpy()


def _compare(cfg, nsteps, label):
    from mpc_gb300.capi import Propagator
    p, A = inputs.make_cell(cfg)
    o = oracle.Oracle(p)
    o.calibrate(A)
    e0 = float(np.sum(np.abs(A) ** 2))
    ref = A.copy()
    st = o.new_state()
    o.run_fixed(ref, st, nsteps)
    with Propagator(p.copy(variant=-1)) as prop:
        prop.upload(A)
        prop.run_fixed(nsteps)
        got = prop.download()
    change = float(np.sum(np.abs(ref) ** 2)) / e0 - 1
    res = {"case": label, "grid": [p.Nx, p.Ny, p.Nt], "split_steps": nsteps,
           "field_rel_l2": _rel(got, ref),
           "spectrum_rel_l2": _rel(_power_spectrum(got, p), _power_spectrum(ref, p)),
           "energy_drift": (float(np.sum(np.abs(got) ** 2)) / e0 - 1) - change,
           "oracle_energy_change": change}
    print(json.dumps(res), flush=True)
    return res


def test_cell64_whole_run(gpu_lib):
    """The 64x64x512 cell, 0.2 mJ, 4 passes of 200 fixed steps with the lens mirror: 800 split
    steps, within 1e-4 of the FP64 run (the precision target of the long runs)."""
    cfg = inputs.config1()
    r = _compare(cfg, cfg.passes * cfg.steps_per_pass, "cell64 whole run")
    assert r["field_rel_l2"] < 1e-4 and r["spectrum_rel_l2"] < 1e-4 and abs(r["energy_drift"]) < 5e-5


@pytest.mark.parametrize("name", ["config2", "config3"])
def test_large_cells_four_steps(gpu_lib, name):
    """Four split steps of the 256x256x2048 cell and of the plasma-dominated 512x512x1024 cell:
    the split-step tolerance."""
    cfg = getattr(inputs, name)()
    r = _compare(cfg, 4, f"{name} 4 steps")
    assert r["field_rel_l2"] < 1e-5 and r["spectrum_rel_l2"] < 1e-5 and abs(r["energy_drift"]) < 1e-6
