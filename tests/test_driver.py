"""The C run driver (mpc_gb300/driver/mpc_run.c, in place of the reference's MPC.c) and the
input generator: reference file formats, adaptive stepping against the FP64 oracle's loop, and
checkpoint / resume."""
import os
import subprocess

import numpy as np
import pytest

from mpc_gb300 import build, inputs
from mpc_gb300.params import BOUNCE_LENS, MPCParams, read_field


def _cell(**kw):
    base = dict(Nx=32, Ny=32, Nt=256, window_xy=4e-3, window_t=2e-12, energy=2e-3, fwhm=150e-15, pressure=2.0,
                cav=0.05, passes=2, steps_per_pass=5, def_err=3e-4, Ab_M=0.9)
    base.update(kw)
    return inputs.cell64(**base)


def test_generator_writes_reference_layout(tmp_path):
    cfg = _cell()
    d = str(tmp_path / "data")
    p = inputs.write_run(cfg, d, nrun=3)
    N = p.Nx * p.Ny * p.Nt
    assert os.path.getsize(d + "0003/param.bin") == 12 + 8 * (2 + p.Nt + 3 + p.Ny) + 4 + 8 * p.Nt + 16 + 4 + 48 \
        + 8 * p.Ny + 32 + 9
    assert os.path.getsize(os.path.join(d, "datar.bin")) == 8 * N
    q = MPCParams.read(d + "0003/param.bin")
    assert q.dims == p.dims and q.gas == p.gas and np.array_equal(q.betas, p.betas) and q.Esig == p.Esig
    _, A = inputs.make_cell(cfg)
    assert np.array_equal(read_field(os.path.join(d, "datar.bin"), os.path.join(d, "datai.bin"), p.dims), A)


def _driver():
    path = build.build_driver()
    assert os.path.exists(path)
    return path


def test_driver_usage_and_missing_inputs(tmp_path):
    """Argument errors exit 2, missing files exit 1, before any GPU work."""
    exe = _driver()
    r = subprocess.run([exe, "-x"], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr
    r = subprocess.run([exe, "-d", str(tmp_path / "nothing")], capture_output=True, text=True)
    assert r.returncode == 1 and "param.bin" in r.stderr
    r = subprocess.run([exe, "-m", "lens"], capture_output=True, text=True)
    assert r.returncode == 1 and "ROC" in r.stderr


def _records(path, n):
    a = np.fromfile(path, dtype=np.float64)
    assert a.size % n == 0
    return a.reshape(-1, n)


@pytest.mark.gpu
def test_driver_adaptive_matches_oracle(gpu_lib, tmp_path):
    """mpc_run's adaptive loop (lens mirrors) against the FP64 oracle running MPC.c's loop with
    the same corrections: every accepted step's record, the step sizes, and the final field."""
    import oracle
    cfg = _cell(bounce=BOUNCE_LENS)
    d = str(tmp_path / "data")
    p = inputs.write_run(cfg, d)
    r = subprocess.run([_driver(), "-d", d, "-m", "lens", "-R", str(cfg.roc)], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    run = d + "0000"
    _, A = inputs.make_cell(cfg)
    o = oracle.Oracle(p)
    o.calibrate(A)
    st = o.new_state()
    C1, C2 = np.empty_like(A), np.empty_like(A)
    dz_rec, temps = [], []
    while st.z < p.dist:
        o.double_step(A, C1, C2, st)
        if st.bad:
            continue
        dz_rec.append(st.dzz)
        temps.append(o.diag(A)[0])
    other = np.loadtxt(os.path.join(run, "other.bin")).reshape(-1, 2)
    assert len(other) == len(dz_rec) >= 4
    assert np.allclose(other[:, 1], np.round(dz_rec, 6), atol=1e-6)
    temp = _records(os.path.join(run, "temp.bin"), p.Nt)
    assert len(temp) == len(dz_rec) and len(_records(os.path.join(run, "bp1.bin"), p.Nx)) == len(dz_rec)
    assert np.linalg.norm(temp[-1] - temps[-1]) / np.linalg.norm(temps[-1]) < 1e-4
    out = np.fromfile(os.path.join(run, "out.bin"), dtype=np.complex128)
    assert np.linalg.norm(out - A) / np.linalg.norm(A) < 1e-4
    assert os.path.exists(os.path.join(run, "resdata.bin")) and os.path.exists(os.path.join(run, "bp1.bin.bak"))


@pytest.mark.gpu
def test_driver_resume_continues_the_run(gpu_lib, tmp_path):
    """Fixed steps in chunks of 2: a run resumed (-r) from its last checkpoint ends with the
    same field and the same diagnostic records as the uninterrupted run."""
    cfg = _cell(steps_per_pass=20, passes=4)           # 80 steps = 40 chunks: checkpoints at 0, 10, 20, 30
    d = str(tmp_path / "data")
    p = inputs.write_run(cfg, d)
    exe = _driver()
    run = d + "0000"
    r = subprocess.run([exe, "-d", d, "-f", "2"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    full = {f: open(os.path.join(run, f), "rb").read() for f in ("out.bin", "temp.bin", "bp1.bin", "other.bin")}
    resparam = open(os.path.join(run, "resparam.bin"), "rb").read()
    assert len(resparam) == 8 + 8 + 4 + 8 + 4
    nstep = int(np.frombuffer(resparam[-4:], dtype=np.int32)[0])
    assert nstep == 31                                  # the checkpoint at chunk 30 stores 30 + 1
    r = subprocess.run([exe, "-d", d, "-f", "2", "-r"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    out0 = np.frombuffer(full["out.bin"], dtype=np.complex128)
    out1 = np.fromfile(os.path.join(run, "out.bin"), dtype=np.complex128)
    assert np.linalg.norm(out1 - out0) / np.linalg.norm(out0) < 1e-5
    t0 = np.frombuffer(full["temp.bin"], dtype=np.float64).reshape(-1, p.Nt)
    t1 = _records(os.path.join(run, "temp.bin"), p.Nt)
    assert t1.shape == t0.shape == (40, p.Nt)
    assert np.array_equal(t1[:31], t0[:31])             # restored from the checkpoint copies
    assert np.linalg.norm(t1 - t0) / np.linalg.norm(t0) < 1e-5
