"""Batched parameter sweep: many independent multipass cells of mixed grid shapes on one GPU
(one batch, one CUDA graph per call) or sharded whole-cell over several ranks.

The reference runs one cell per process (MPC.c); a sweep is many such runs.  Here a rank
takes a share of the cells (balanced by N * steps, whole cells, no data exchange between
ranks), creates one context per cell (the autotuner picks each grid shape's kernel variant
once), and advances all its cells together:
  fixed dz:  mpc_batch_run_fixed, one graph per pass of every cell;
  adaptive:  mpc_batch_step_double, one graph per round of step-doubling attempts (MPC.c:269-383
             per cell) until every cell has reached its dist.
Throughput counts every executed split step (3 per attempt in adaptive mode) of every grid
point: grid-point-steps/s.

  python -m mpc_gb300.sweep [--cells 64] [--fixed] [--passes P] [--steps-per-pass S]
  torchrun --nproc-per-node N -m mpc_gb300.sweep ...   (cells sharded over N ranks)
"""
from __future__ import annotations

import json
import os
import time

import numpy as np

from . import inputs


def cell_cost(cfg: inputs.CellConfig) -> float:
    """Work of one cell: grid points x split steps at the initial dz."""
    return float(cfg.Nx * cfg.Ny * cfg.Nt) * cfg.passes * cfg.steps_per_pass


def shard(cfgs: list, world: int, rank: int) -> list[int]:
    """Indices of the cells rank `rank` runs: longest-processing-time-first assignment of whole
    cells to the least loaded rank (ties to the lower rank), deterministic on every rank."""
    order = sorted(range(len(cfgs)), key=lambda i: (-cell_cost(cfgs[i]), i))
    load = [0.0] * world
    owner = [0] * len(cfgs)
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        owner[i] = r
        load[r] += cell_cost(cfgs[i])
    return [i for i in range(len(cfgs)) if owner[i] == rank]


def run_cells(cfgs: list, adaptive: bool = True, variant: int = -1, max_rounds: int = 100000) -> dict:
    """Run the given cells to their dist on the current GPU as one batch; return statistics and
    the final device states."""
    from .capi import Batch, Propagator
    props, n_pts = [], []
    for cfg in cfgs:
        p, A = inputs.make_cell(cfg)
        prop = Propagator(p.copy(variant=variant))
        prop.upload(A, calibrate=True)
        props.append(prop)
        n_pts.append(p.N)
    for prop in props:
        prop.sync()
    batch = Batch(props)
    t0 = time.perf_counter()
    executed = np.zeros(len(props))
    rounds = attempts = accepted = 0
    if adaptive:
        while rounds < max_rounds:
            bad, err = batch.step_double()
            live = bad >= 0
            if not live.any():
                break
            rounds += 1
            attempts += int(live.sum())
            accepted += int((bad == 0).sum())
            executed += 3 * live
    else:
        # whole passes: every cell has the same number of fixed steps per pass
        per_pass = {cfg.steps_per_pass for cfg in cfgs}
        passes = {cfg.passes for cfg in cfgs}
        if len(per_pass) != 1 or len(passes) != 1:
            raise ValueError("fixed-dz batches need one steps_per_pass and one passes for all cells")
        spp, npass = per_pass.pop(), passes.pop()
        for _ in range(npass):
            batch.run_fixed(spp)
            rounds += 1
        executed[:] = spp * npass
    for prop in props:
        prop.sync()
    dt = time.perf_counter() - t0
    states = [prop.state() for prop in props]
    pt_steps = float(np.dot(executed, n_pts))
    out = dict(cells=len(cfgs), seconds=dt, pt_steps=pt_steps, value=pt_steps / dt if dt > 0 else 0.0,
               rounds=rounds, attempts=attempts, accepted=accepted, graphs=batch.stats(),
               z=[s.z for s in states], dzz=[s.dzz for s in states],
               variants={f"{p.p.Nx}x{p.p.Ny}x{p.p.Nt}": p.variant_info()["variant"] for p in props})
    batch.close()
    for prop in props:
        prop.close()
    return out


def main(argv=None) -> int:
    import argparse
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--cells", type=int, default=64)
    ap.add_argument("--seed", type=int, default=100)
    ap.add_argument("--fixed", action="store_true", help="fixed dz (default: adaptive step doubling)")
    ap.add_argument("--passes", type=int, default=None)
    ap.add_argument("--steps-per-pass", type=int, default=None)
    a = ap.parse_args(argv)
    cfgs = inputs.sweep_cells(a.seed, a.cells)
    for c in cfgs:
        if a.passes:
            c.passes = a.passes
        if a.steps_per_pass:
            c.steps_per_pass = a.steps_per_pass
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("gloo")
    mine = shard(cfgs, world, rank)
    res = run_cells([cfgs[i] for i in mine], adaptive=not a.fixed)
    res["rank"] = rank
    if dist is not None:
        gathered = [None] * world
        dist.all_gather_object(gathered, res)
        dist.destroy_process_group()
    else:
        gathered = [res]
    if rank == 0:
        secs = max(r["seconds"] for r in gathered)
        pts = sum(r["pt_steps"] for r in gathered)
        print(json.dumps({"metric": "grid-point-steps/s", "value": pts / secs, "unit": "grid-point-steps/s",
                          "workload": f"sweep of {a.cells} cells (seed {a.seed}), "
                                      f"{'fixed dz' if a.fixed else 'adaptive step doubling'}",
                          "ranks": world, "seconds": secs, "pt_steps": pts,
                          "attempts": sum(r["attempts"] for r in gathered),
                          "accepted": sum(r["accepted"] for r in gathered),
                          "graphs": sum(r["graphs"]["graphs"] for r in gathered),
                          "graph_nodes": sum(r["graphs"]["nodes"] for r in gathered),
                          "variants": gathered[0]["variants"]}))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
