"""The allocation-free nonlinear step (mpc_nonlinear_noalloc), for callers that cannot
allocate device memory, against the context-based entry point.

mpc_ssfmprop applies L(dz/2) N(dz) L(dz/2); with no dispersion and no diffraction
(betas = 0, wr = 0, alpha = 0) the linear half steps are the identity and it returns N(dz)
alone, which is what mpc_nonlinear_noalloc computes.  Two calls in a row are compared, the
second on the first's output, with the one-step tolerance of the other parity tests.  This
file is collected last so that a run stopping at the first failure has run everything else.
"""
import numpy as np
import pytest

from mpc_gb300 import inputs

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_nonlinear_noalloc_matches_ssfmprop_twice(gpu_lib):
    torch = pytest.importorskip("torch")
    import oracle
    from mpc_gb300.capi import Propagator, nonlinear_noalloc

    cfg = inputs.config1(Nx=32, Ny=32, Nt=256, window_xy=4e-3, window_t=2e-12, energy=3e-3, fwhm=120e-15,
                         pressure=3.0, beam_w=0.3e-3)
    p, A = inputs.make_cell(cfg)
    p = p.copy(betas=np.zeros(p.Nt), wr=np.zeros(p.Ny), alpha=0.0)
    oracle.Oracle(p).calibrate(A)
    dz = p.dzz
    torch.cuda.init()
    dev = torch.from_numpy(A.astype(np.complex64)).to("cuda")
    stream = torch.cuda.current_stream().cuda_stream
    ref = A.copy()
    with Propagator(p) as prop:
        for call in range(2):
            prop.ssfmprop(ref, dz, 1, 0.0, p.puls_e)
            rc = nonlinear_noalloc(p, dev.data_ptr(), dz, stream)
            assert rc == 0, f"call {call}: status {rc}"
            torch.cuda.synchronize()
            got = dev.cpu().numpy().astype(np.complex128)
            assert np.isfinite(got).all()
            assert rel(got, ref) < 1e-5, f"call {call}"
    assert rel(ref, A) > 1e-4      # the step changed the field


def test_nonlinear_noalloc_rejects_oversize(gpu_lib):
    torch = pytest.importorskip("torch")
    from mpc_gb300.capi import nonlinear_noalloc
    p, _ = inputs.make_cell(inputs.config1(Nx=16, Ny=16, Nt=64))
    big = p.copy(dims=(16, 16, 4096), w=np.zeros(4096), betas=np.zeros(4096))
    host = np.full(16 * 16 * 4096, 1 + 2j, dtype=np.complex64)
    buf = torch.from_numpy(host).to("cuda")       # a copy, no torch kernel
    # Nt beyond the static scratch: MPC_ERR_SHAPE, returned before anything is queued
    assert nonlinear_noalloc(big, buf.data_ptr(), 1e-3, torch.cuda.current_stream().cuda_stream) == 2
    torch.cuda.synchronize()
    assert np.array_equal(buf.cpu().numpy(), host)
