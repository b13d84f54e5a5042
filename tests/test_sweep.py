"""Batched sweeps: whole-cell sharding over ranks (CPU, gloo) and batches of cells run as one
CUDA graph per call against the same cells run one by one (GPU)."""
import os
import socket

import numpy as np
import pytest

from mpc_gb300 import inputs, sweep


def test_shard_covers_every_cell_once_and_balances():
    cfgs = inputs.sweep_cells(100, 64)
    costs = [sweep.cell_cost(c) for c in cfgs]
    for world in (1, 2, 3, 4, 8):
        parts = [sweep.shard(cfgs, world, r) for r in range(world)]
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(cfgs)))
        loads = [sum(costs[i] for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(costs)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    cfgs = inputs.sweep_cells(100, 64)
    mine = sweep.shard(cfgs, world, rank)
    gathered = [None] * world
    dist.all_gather_object(gathered, {"rank": rank, "cells": mine, "seconds": 1.0 + rank})
    dist.destroy_process_group()
    q.put((rank, gathered))


def test_shard_agrees_across_gloo_ranks():
    """Two ranks compute their shares independently; the gathered shares partition the sweep
    and both ranks see the same result (the aggregation of the sweep's main())."""
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got[0] == got[1]
    cells = sorted(i for r in got[0] for i in r["cells"])
    assert cells == list(range(64))
    assert max(r["seconds"] for r in got[0]) == 2.0


def _small_cells():
    return [inputs.cell64(Nx=16, Ny=16, Nt=64, window_xy=2e-3, window_t=1e-12, energy=0.3e-3, steps_per_pass=10,
                           passes=1, seed=5),
            inputs.cell64(Nx=32, Ny=32, Nt=256, window_xy=4e-3, window_t=2e-12, energy=1e-3, steps_per_pass=10,
                           passes=1, seed=6, pressure=2.0),
            inputs.cell64(Nx=64, Ny=64, Nt=512, steps_per_pass=10, passes=1, seed=7)]


@pytest.mark.gpu
def test_batch_run_fixed_matches_cells_one_by_one(gpu_lib):
    from mpc_gb300.capi import Batch, Propagator
    cells = [inputs.make_cell(c) for c in _small_cells()]
    single = []
    for p, A in cells:
        with Propagator(p) as prop:
            prop.upload(A, calibrate=True)
            prop.run_fixed(7)
            single.append(prop.download())
    props = [Propagator(p) for p, _ in cells]
    for prop, (p, A) in zip(props, cells):
        prop.upload(A, calibrate=True)
    with Batch(props) as b:
        b.run_fixed(7)
        assert b.stats()["graphs"] == 1 and b.stats()["nodes"] >= 3 * 14
    for prop, ref in zip(props, single):
        assert prop.state().nstep == 7
        got = prop.download()
        assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-7
        prop.close()


@pytest.mark.gpu
def test_batch_step_double_matches_cells_one_by_one(gpu_lib):
    from mpc_gb300.capi import Batch, Propagator
    cells = [inputs.make_cell(c) for c in _small_cells()]
    single = []
    for p, A in cells:
        with Propagator(p) as prop:
            prop.upload(A, calibrate=True)
            rec = [prop.step_double() for _ in range(4)]
            single.append((rec, prop.download(), prop.state().z))
    props = [Propagator(p) for p, _ in cells]
    for prop, (p, A) in zip(props, cells):
        prop.upload(A, calibrate=True)
    with Batch(props) as b:
        recs = [b.step_double() for _ in range(4)]
        assert b.stats()["graphs"] == 4
    for i, (prop, (rec, ref, z)) in enumerate(zip(props, single)):
        assert [int(r[0][i]) for r in recs] == [r["bad"] for r in rec]
        assert [r[1][i] for r in recs] == pytest.approx([r["err"] for r in rec], rel=1e-12)
        assert prop.state().z == z
        got = prop.download()
        assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-7
        prop.close()


@pytest.mark.gpu
def test_batch_cells_match_the_oracle(gpu_lib):
    """Every cell of a batch against the FP64 oracle (not only against itself run alone): 7 fixed
    split steps in one graph, then 4 step-doubling attempts as batch rounds, with the oracle's
    accept/reject decisions, step sizes and z (propagation.c:111-372, 616-677; MPC.c:269-383)."""
    import oracle
    from mpc_gb300.capi import Batch, Propagator
    cells = []
    for c in _small_cells():
        c.passes = 4                 # room for the 7 fixed steps and the 4 attempts
        p, A = inputs.make_cell(c)
        o = oracle.Oracle(p)
        o.calibrate(A)
        cells.append((p, A, o))
    props = [Propagator(p) for p, _, _ in cells]
    refs, states = [], []
    for prop, (p, A, o) in zip(props, cells):
        prop.upload(A)
        ref = A.copy()
        st = o.new_state()
        o.run_fixed(ref, st, 7)
        refs.append(ref)
        states.append(st)
    try:
        with Batch(props) as b:
            b.run_fixed(7)
            for prop, ref in zip(props, refs):
                got = prop.download()
                assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-5
            scratch = [(np.empty_like(r), np.empty_like(r)) for r in refs]
            for _ in range(4):
                bad, err = b.step_double()
                for i, ((p, A, o), ref, st, (C1, C2)) in enumerate(zip(cells, refs, states, scratch)):
                    assert bad[i] >= 0          # no cell has finished its distance yet
                    o.double_step(ref, C1, C2, st)
                    assert int(bad[i]) == st.bad
                    assert abs(err[i] / st.err - 1) < 0.05
                    s = props[i].state()
                    assert s.dzz == pytest.approx(st.dzz, rel=1e-12) and s.z == pytest.approx(st.z, rel=1e-12, abs=1e-15)
        for prop, ref in zip(props, refs):
            got = prop.download()
            assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-5
    finally:
        for prop in props:
            prop.close()


@pytest.mark.gpu
def test_sweep_runs_every_cell_to_its_distance(gpu_lib):
    cfgs = _small_cells()
    for c in cfgs:
        c.cav = 0.05
        c.def_err = 1e-4
    res = sweep.run_cells(cfgs, adaptive=True)
    assert res["z"] == pytest.approx([c.passes * c.cav for c in cfgs], rel=1e-12)
    assert res["graphs"]["graphs"] == res["rounds"] and res["attempts"] >= res["accepted"] > 0
    assert res["value"] > 0
