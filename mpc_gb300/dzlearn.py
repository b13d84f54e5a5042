"""Learned step-size control: training pairs from step-doubling runs, training on the GPU,
and evaluation against plain step doubling.

The reference chooses dz by step doubling (MPC.c:269-383, propagation.c:616-677): every
accepted advance of 2h costs three split steps (one of 2h, two of h) plus the comparison.  The
learned controller instead predicts the next step from 16 features of the field and state
(mpc_features) with a small network (mpc_mlp_*, trained and run by this project's kernels) and
takes plain split steps of that length; a step-doubling check every few steps measures the
local error and falls back to step doubling when it exceeds the tolerance.

Training pairs come from batched step-doubling runs of cells drawn from the high-intensity,
plasma-dominated distribution (argon, 0.5-3 mJ, 1-3 bar, 80-200 fs): features before an
attempt -> target = log(d / Cav), where d = 2 h (tol / err)^(1/3) is the largest advance whose
step-doubling error estimate meets the tolerance (the local error of a second-order step grows
as h^3).

  python -m mpc_gb300.dzlearn collect --cells 64 --rounds 1600 --out pairs.npz
  python -m mpc_gb300.dzlearn train --data pairs.npz --out controller.npz
  python -m mpc_gb300.dzlearn eval --model controller.npz --cells 4 --grid 256,256,2048 --passes 2
"""
from __future__ import annotations

import json
import math
import os
import time

import numpy as np

from . import inputs

DEFAULT_MODEL = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "dz_controller.npz")


def controller_cells(seed: int, n: int, grid=(64, 64, 512), passes: int = 1, steps_per_pass: int = 50,
                     def_err: float = 1e-5) -> list:
    """Cells of the controller's training / evaluation distribution on a given grid: argon,
    energy log-uniform 0.5-3 mJ, pressure U(1, 3) bar, FWHM U(80, 200) fs, 0.3 mm beam."""
    Nx, Ny, Nt = grid
    out = []
    for i in range(n):
        u = ((inputs.splitmix64(seed + i, 3) >> np.uint64(11)).astype(np.float64) + 0.5) / 9007199254740992.0
        energy = 10 ** (math.log10(0.5e-3) + u[0] * (math.log10(3e-3) - math.log10(0.5e-3)))
        out.append(inputs.CellConfig(Nx=Nx, Ny=Ny, Nt=Nt, window_xy=4e-3 * Nx / 64 if Nx <= 128 else 8e-3,
                                     window_t=2e-12 * max(1, Nt // 1024), beam_w=0.3e-3, energy=energy,
                                     pressure=1.0 + 2.0 * u[1], fwhm=(80 + 120 * u[2]) * 1e-15, seed=seed + i,
                                     passes=passes, steps_per_pass=steps_per_pass, def_err=def_err))
    return out


def dz_target(h: float, err: float, def_err: float, cav: float) -> float:
    """log(d / Cav) of the largest advance d = 2 h (tol / err)^(1/3) meeting the tolerance."""
    return math.log(2.0 * h * (def_err / max(err, 1e-30)) ** (1.0 / 3.0) / cav)


def collect(cfgs: list, rounds: int, variant: int = -1):
    """Run the cells by batched step doubling for `rounds` rounds (or until all finish) and
    return (X, y): the features before each attempt and that attempt's target."""
    from .capi import Batch, Propagator
    props = []
    for cfg in cfgs:
        p, A = inputs.make_cell(cfg)
        prop = Propagator(p.copy(variant=variant))
        prop.upload(A, calibrate=True)
        props.append(prop)
    X, Y = [], []
    with Batch(props) as batch:
        for r in range(rounds):
            feats = [prop.features() for prop in props]
            for prop in props:
                prop.step_stats(reset=True)
            hs = [prop.state().dzz for prop in props]
            bad, err = batch.step_double()
            if (bad < 0).all():
                break
            if r == 0:
                continue   # no step statistics before the first attempt
            for i, prop in enumerate(props):
                if bad[i] >= 0 and err[i] > 0:
                    X.append(feats[i])
                    Y.append(dz_target(hs[i], float(err[i]), prop.p.def_err, prop.p.Cav))
    for prop in props:
        prop.close()
    return np.asarray(X, dtype=np.float32), np.asarray(Y, dtype=np.float32)


def fit(X, y, epochs: int = 60, batch: int = 256, lr: float = 2e-3, seed: int = 0):
    """Train a fresh network on (X, y) with per-feature normalisation; returns (mlp, loss)."""
    from .capi import MLP
    mean = X.mean(0)
    std = X.std(0)
    std = np.where(std > 1e-3, std, 1.0).astype(np.float32)
    mlp = MLP(seed)
    mlp.set_normalization(mean, std, float(y.mean()), float(max(y.std(), 1e-3)))
    loss = mlp.train(X, y, epochs=epochs, batch=batch, lr=lr, seed=seed)
    return mlp, loss


def save(mlp, path: str, **meta) -> None:
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    np.savez(path, weights=mlp.weights, norm=mlp.normalization(), meta=json.dumps(meta))


def load(path: str = DEFAULT_MODEL):
    from .capi import MLP
    d = np.load(path)
    mlp = MLP(0)
    norm = d["norm"]
    mlp.set_normalization(norm[:16], norm[16:32], float(norm[32]), float(norm[33]))
    mlp.weights = d["weights"]
    return mlp


def _cell(cfg):
    return cfg if isinstance(cfg, tuple) else inputs.make_cell(cfg)


def run_plain(cfg, variant: int = -1, def_err: float | None = None, land: bool = False):
    """Plain step doubling to dist: (field, executed split steps, seconds).  cfg: a CellConfig
    or its (params, field) from inputs.make_cell; land: end attempts on the mirror planes (the
    reference steps across them and applies the bounce after the attempt)."""
    from .capi import Propagator
    p, A = _cell(cfg)
    if def_err is not None:
        p = p.copy(def_err=def_err)
    p = p.copy(land_mirrors=int(land))
    with Propagator(p.copy(variant=variant)) as prop:
        prop.upload(A, calibrate=True)
        prop.sync()
        t = time.perf_counter()
        attempts = 0
        while prop.state().z < p.dist * (1 - 1e-12):
            prop.step_double()
            attempts += 1
        prop.sync()
        dt = time.perf_counter() - t
        return prop.download(), 3 * attempts, dt


def run_learned(cfg, mlp, safety: float = 0.9, check_every: int = 8, fallback_len: int = 4, variant: int = -1,
                hold: int = 1):
    """The learned controller to dist: (field, statistics, seconds).  Its own steps land on the
    mirror planes, and so do its step-doubling checks and fallbacks; one prediction serves `hold`
    consecutive steps."""
    from .capi import Propagator
    p, A = _cell(cfg)
    p = p.copy(land_mirrors=1)
    with Propagator(p.copy(variant=variant)) as prop:
        prop.upload(A, calibrate=True)
        prop.sync()
        t = time.perf_counter()
        st = prop.run_learned(mlp, safety=safety, check_every=check_every, fallback_len=fallback_len, hold=hold)
        prop.sync()
        dt = time.perf_counter() - t
        return prop.download(), st, dt


def run_reference(cfg, steps_per_pass: int, variant: int = -1):
    """Fixed steps of Cav / steps_per_pass to dist (each mirror bounce exactly on its plane): the
    converged solution the step-size controllers are measured against.  (A step-doubling run at a
    tolerance near the ~1e-7 rounding floor of its complex64 error estimate cannot serve: it
    shrinks dz to dzmin.)"""
    from .capi import Propagator
    p, A = _cell(cfg)
    p = p.copy(dzz=p.Cav / steps_per_pass)
    with Propagator(p.copy(variant=variant)) as prop:
        prop.upload(A, calibrate=True)
        n = int(round(p.dist / p.dzz))
        prop.run_fixed(n)
        return prop.download(), n


def evaluate(cfgs: list, mlp, ref_steps_per_pass: int = 2000, safeties=(0.9,), plain_tols=(), **kw) -> list[dict]:
    """Per cell: end-field relative L2 error against a fine fixed-step run, executed steps and
    wall time of plain step doubling (as the reference: bounces after the attempt that crosses a
    mirror plane; and landing on the planes, at the cell's tolerance and at each of plain_tols)
    and of the learned controller at each safety factor.  The err_learned / steps_learned /
    seconds_learned keys are the first safety's."""
    rows = []
    for cfg in cfgs:
        cfg = _cell(cfg)
        ref, n_ref = run_reference(cfg, ref_steps_per_pass)
        nr = np.linalg.norm(ref)
        plain, n_plain, t_plain = run_plain(cfg)
        landed, n_landed, t_landed = run_plain(cfg, land=True)
        row = dict(err_plain=float(np.linalg.norm(plain - ref) / nr), steps_plain=int(n_plain), seconds_plain=t_plain,
                   err_plain_landing=float(np.linalg.norm(landed - ref) / nr), steps_plain_landing=int(n_landed),
                   seconds_plain_landing=t_landed, ref_steps=int(n_ref), learned={}, plain_landing_tol={})
        for tol in plain_tols:
            f_t, n_t, t_t = run_plain(cfg, def_err=tol, land=True)
            row["plain_landing_tol"][tol] = dict(err=float(np.linalg.norm(f_t - ref) / nr), steps=int(n_t), seconds=t_t)
        for sf in safeties:
            learned, st, t_learned = run_learned(cfg, mlp, safety=sf, **kw)
            row["learned"][sf] = dict(err=float(np.linalg.norm(learned - ref) / nr), steps=int(st["executed_steps"]),
                                      seconds=t_learned, checks=st["checks"], check_failures=st["check_failures"],
                                      fallback_attempts=st["fallback_attempts"])
        first = row["learned"][safeties[0]]
        row.update(err_learned=first["err"], steps_learned=first["steps"], seconds_learned=first["seconds"],
                   speedup=t_plain / first["seconds"], speedup_vs_landing=t_landed / first["seconds"],
                   checks=first["checks"], check_failures=first["check_failures"],
                   fallback_attempts=first["fallback_attempts"])
        rows.append(row)
    return rows


def main(argv=None) -> int:
    import argparse
    ap = argparse.ArgumentParser(description="learned step-size control")
    sub = ap.add_subparsers(dest="cmd", required=True)
    c = sub.add_parser("collect")
    c.add_argument("--cells", type=int, default=64)
    c.add_argument("--rounds", type=int, default=1600)
    c.add_argument("--seed", type=int, default=2000)
    c.add_argument("--grid", default="64,64,512")
    c.add_argument("--out", required=True)
    t = sub.add_parser("train")
    t.add_argument("--data", required=True)
    t.add_argument("--epochs", type=int, default=60)
    t.add_argument("--out", default=DEFAULT_MODEL)
    e = sub.add_parser("eval")
    e.add_argument("--model", default=DEFAULT_MODEL)
    e.add_argument("--cells", type=int, default=4)
    e.add_argument("--seed", type=int, default=1000)
    e.add_argument("--grid", default="256,256,2048")
    e.add_argument("--passes", type=int, default=8)
    e.add_argument("--safety", default="0.9", help="comma-separated safety factors of the learned controller")
    e.add_argument("--ref-steps", type=int, default=2000, help="fixed steps per pass of the reference run")
    e.add_argument("--plain-tol", default="", help="comma-separated extra tolerances of plain step doubling (landing)")
    e.add_argument("--hold", type=int, default=1, help="consecutive steps per network prediction")
    a = ap.parse_args(argv)
    if a.cmd == "collect":
        grid = tuple(int(v) for v in a.grid.split(","))
        cfgs = controller_cells(a.seed, a.cells, grid, passes=8)
        t0 = time.perf_counter()
        X, y = collect(cfgs, a.rounds)
        np.savez(a.out, X=X, y=y)
        print(json.dumps(dict(pairs=len(y), seconds=time.perf_counter() - t0, grid=grid, cells=a.cells)))
    elif a.cmd == "train":
        d = np.load(a.data)
        X, y = d["X"], d["y"]
        rng = np.random.default_rng(0)
        idx = rng.permutation(len(y))
        nval = max(1, len(y) // 10)
        va, tr = idx[:nval], idx[nval:]
        t0 = time.perf_counter()
        mlp, loss = fit(X[tr], y[tr], epochs=a.epochs)
        pred = mlp.predict(X[va])
        rmse = float(np.sqrt(np.mean((pred - y[va]) ** 2)))
        save(mlp, a.out, pairs=int(len(y)), train_loss=loss, val_rmse_log=rmse)
        print(json.dumps(dict(pairs=len(y), train_loss=loss, val_rmse_log_dz=rmse, seconds=time.perf_counter() - t0)))
    else:
        grid = tuple(int(v) for v in a.grid.split(","))
        cfgs = controller_cells(a.seed, a.cells, grid, passes=a.passes, steps_per_pass=400)
        safeties = tuple(float(v) for v in a.safety.split(","))
        plain_tols = tuple(float(v) for v in a.plain_tol.split(",") if v)
        rows = evaluate(cfgs, load(a.model), ref_steps_per_pass=a.ref_steps, safeties=safeties, plain_tols=plain_tols,
                        hold=a.hold)
        summary = dict(cells=len(rows), grid=grid, passes=a.passes,
                       plain=dict(max_err=max(r["err_plain"] for r in rows), seconds=sum(r["seconds_plain"] for r in rows)),
                       plain_landing=dict(max_err=max(r["err_plain_landing"] for r in rows),
                                          seconds=sum(r["seconds_plain_landing"] for r in rows)),
                       learned={str(sf): dict(max_err=max(r["learned"][sf]["err"] for r in rows),
                                              seconds=sum(r["learned"][sf]["seconds"] for r in rows))
                                for sf in safeties},
                       plain_landing_tol={str(t): dict(max_err=max(r["plain_landing_tol"][t]["err"] for r in rows),
                                                       seconds=sum(r["plain_landing_tol"][t]["seconds"] for r in rows))
                                          for t in plain_tols})
        print(json.dumps(dict(summary=summary, rows=[{k: ({str(a): b for a, b in v.items()} if isinstance(v, dict) else v)
                                                      for k, v in r.items()} for r in rows])))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
