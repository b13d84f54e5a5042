"""The allocation-free nonlinear step (mpc_nonlinear_noalloc), for callers that cannot allocate
device memory (code under another library's no-allocation promise, processes whose device memory
is owned by a pool handed out at start-up, hosts with a fixed device-memory budget).

The checker is the FP64 oracle's nonlinear operator: with no dispersion and no diffraction
(betas = 0, wr = 0, alpha = 0) the oracle's split step L(dz/2) N(dz) L(dz/2) has identity linear
half steps and returns N(dz) alone (propagation.c:164-327, plasma.c:118-245).  The first test
also runs the context-based entry point (mpc_ssfmprop) on the same field and compares the two
device results.  Two calls in a row are checked, the second on the first's output, at the
one-step tolerance of the other parity tests (1e-5 relative L2).  This file is collected last so
that a run stopping at the first failure has run everything else.
"""
import numpy as np
import pytest

import oracle
from mpc_gb300 import inputs

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _cell(Nx, Ny, Nt):
    # the 32x32x256 cell's sample spacings, 3 mJ, 120 fs, argon 3 bar (strong ionization)
    cfg = inputs.cell64(Nx=Nx, Ny=Ny, Nt=Nt, window_xy=4e-3 * Nx / 32, window_t=2e-12 * Nt / 256, energy=3e-3,
                         fwhm=120e-15, pressure=3.0, beam_w=0.3e-3)
    p, A = inputs.make_cell(cfg)
    p = p.copy(betas=np.zeros(p.Nt), wr=np.zeros(p.Ny), alpha=0.0)
    o = oracle.Oracle(p)
    o.calibrate(A)
    return p, A, o


def _two_calls(p, A, o, also_ssfmprop=False):
    torch = pytest.importorskip("torch")
    from mpc_gb300.capi import Propagator, nonlinear_noalloc
    dz = p.dzz
    torch.cuda.init()
    dev = torch.from_numpy(A.astype(np.complex64)).to("cuda")
    stream = torch.cuda.current_stream().cuda_stream
    ref = A.copy()
    ctx_field = A.copy()
    prop = Propagator(p) if also_ssfmprop else None
    try:
        for call in range(2):
            o.ssfmprop(ref, dz, 1, 0.0, p.puls_e)
            rc = nonlinear_noalloc(p, dev.data_ptr(), dz, stream)
            assert rc == 0, f"call {call}: status {rc}"
            torch.cuda.synchronize()
            got = dev.cpu().numpy().astype(np.complex128)
            assert np.isfinite(got).all()
            assert rel(got, ref) < 1e-5, f"call {call}: {rel(got, ref):.3e} against the FP64 oracle"
            if prop is not None:
                prop.ssfmprop(ctx_field, dz, 1, 0.0, p.puls_e)
                assert rel(got, ctx_field) < 1e-5, f"call {call}: against mpc_ssfmprop"
    finally:
        if prop is not None:
            prop.close()
    assert rel(ref, A) > 1e-4      # the step changed the field


def test_nonlinear_noalloc_matches_oracle_and_ssfmprop_twice(gpu_lib):
    """32x32x256 (a grid the context-based path compiles): against the FP64 oracle and against
    mpc_ssfmprop, two calls in a row."""
    p, A, o = _cell(32, 32, 256)
    _two_calls(p, A, o, also_ssfmprop=True)


@pytest.mark.parametrize("Nt", [64, 512, 1024, 2048])
def test_nonlinear_noalloc_every_length(gpu_lib, Nt):
    """The other compiled t lengths (tiles of 256, 32, 16 and 8 pencils) on a 16x16 grid, against
    the FP64 oracle, two calls in a row."""
    p, A, o = _cell(16, 16, Nt)
    _two_calls(p, A, o)


def test_nonlinear_noalloc_rejects_oversize(gpu_lib):
    torch = pytest.importorskip("torch")
    from mpc_gb300.capi import nonlinear_noalloc
    p, _ = inputs.make_cell(inputs.cell64(Nx=16, Ny=16, Nt=64))
    big = p.copy(dims=(16, 16, 4096), w=np.zeros(4096), betas=np.zeros(4096))
    host = np.full(16 * 16 * 4096, 1 + 2j, dtype=np.complex64)
    buf = torch.from_numpy(host).to("cuda")       # a copy, no torch kernel
    # Nt beyond the static scratch: MPC_ERR_SHAPE, returned before anything is queued
    assert nonlinear_noalloc(big, buf.data_ptr(), 1e-3, torch.cuda.current_stream().cuda_stream) == 2
    torch.cuda.synchronize()
    assert np.array_equal(buf.cpu().numpy(), host)
