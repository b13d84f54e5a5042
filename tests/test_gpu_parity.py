"""Parity of the CUDA path (through the C ABI of libmpc_gpu.so) against the FP64 CPU oracle.

Tolerances: the device field is complex64 with FP32 FFTs; one split step reproduces the
FP64 oracle to a relative L2 error of ~1e-6, so single-step checks use 1e-5 and runs of
hundreds of steps 1e-4 (the accuracy target for the full 256^2 x 2048 run).  FP64 device
routines (ADK) are checked to 1e-12.
"""
import numpy as np
import pytest

import oracle
from mpc_gb300 import inputs
from mpc_gb300.params import BOUNCE_LENS, BOUNCE_SIGNFLIP

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def small_cell(**kw):
    base = dict(Nx=32, Ny=32, Nt=256, window_xy=4e-3, window_t=2e-12, energy=0.5e-3, steps_per_pass=50)
    base.update(kw)
    p, A = inputs.make_cell(inputs.cell64(**base))
    o = oracle.Oracle(p)
    o.calibrate(A)
    return p, A, o


@pytest.mark.parametrize("shape", [(16, 16, 64), (32, 32, 256), (64, 64, 512)])
def test_linearstep(gpu_lib, shape):
    from mpc_gb300.capi import Propagator
    Nx, Ny, Nt = shape
    p, A, o = small_cell(Nx=Nx, Ny=Ny, Nt=Nt, window_t=2e-12 * Nt / 256)
    rng = np.random.default_rng(1)
    A = A + 0.1 * np.abs(A).max() * (rng.standard_normal(A.size) + 1j * rng.standard_normal(A.size))
    dz = 0.01
    eD = o.expD0(dz)
    eR, _ = o.calcexpR(Nx, 1, 0.0, dz / 2)
    ref = A.copy()
    oracle.lib().or_linearstep(oracle._p(ref.view(np.float64)), Nx, Ny, Nt, oracle._p(eD.view(np.float64)),
                               oracle._p(eR.view(np.float64)), oracle._p(eR.view(np.float64)))
    with Propagator(p) as prop:
        got = A.copy()
        prop.linearstep(got, eD, eR)
    assert rel(got, ref) < 1e-5


def test_calcexpR(gpu_lib):
    from mpc_gb300.capi import Propagator
    p, A, o = small_cell()
    with Propagator(p) as prop:
        for z, sm in [(0.1, 1), (0.6, 1), (0.6, -1), (1.2, -1)]:
            ref, sm_ref = o.calcexpR(p.Nx, sm, z, 1.25e-3)
            got, sm_got = prop.calcexpR(sm, z, 1.25e-3)
            assert sm_got == sm_ref
            assert np.abs(got - ref).max() < 2e-7


GASES = ["Argon", "Helium", "Neon", "Air", "Nitrogen", "Xenon", "Krypton"]


@pytest.mark.parametrize("gas", GASES)
def test_ADK_fp64(gpu_lib, gas):
    """ADK rates of both stages on the device (FP64) for every gas of plasma.c:4-115."""
    from mpc_gb300.capi import Propagator
    p, A, o = small_cell(gas=gas)
    E = np.geomspace(1e-4, 0.5, 257)
    with Propagator(p) as prop:
        r1, r2 = prop.ADK(E)
    I1, I2 = oracle.ionizpot(gas)
    Iion = np.array([I1, I2]) / 27.21
    nq = np.array([1 / np.sqrt(2 * Iion[0]), 2 / np.sqrt(2 * Iion[1])])
    from math import gamma
    Cnl = np.array([np.sqrt(2 ** (2 * n) / (n * gamma(n + 1) * gamma(n))) for n in nq])
    e1, e2 = oracle.ADK(E, Cnl, [1, 1], nq, [0, 0], Iion)
    assert rel(r1, e1) < 1e-12 and rel(r2, e2) < 1e-12


@pytest.mark.parametrize("gas", GASES)
def test_ioniz_every_gas(gpu_lib, gas):
    """Free-electron density and collision time of every gas (ionization potentials, atom
    densities and cross-sections of plasma.c:4-115) against the oracle."""
    from mpc_gb300.capi import Propagator
    p, A, o = small_cell(gas=gas, energy=3e-3, fwhm=100e-15, pressure=2.0, beam_w=0.3e-3)
    tau, fe = o.ioniz(A)
    with Propagator(p) as prop:
        t_g, f_g = prop.ioniz(A)
    print(f"ioniz {gas}: tau_c rel L2 {rel(t_g, tau):.3e}, fe_sp rel L2 {rel(f_g, fe):.3e}")
    # measured on GB300: tau_c <= 8e-8, fe_sp <= 1.9e-7 (FP32 within 32-sample chunks, FP64 carries)
    assert rel(t_g, tau) < 1e-6 and fe.max() > 0 and rel(f_g, fe) < 1e-6


def test_ioniz(gpu_lib):
    from mpc_gb300.capi import Propagator
    p, A, o = small_cell(energy=3e-3, fwhm=120e-15, pressure=3.0, beam_w=0.3e-3)
    tau_ref, fe_ref = o.ioniz(A)
    with Propagator(p) as prop:
        tau, fe = prop.ioniz(A)
    print(f"ioniz argon 3 bar: tau_c rel L2 {rel(tau, tau_ref):.3e}, fe_sp rel L2 {rel(fe, fe_ref):.3e}, "
          f"max fe_sp {fe_ref.max():.3e}")
    assert rel(tau, tau_ref) < 1e-6
    assert fe_ref.max() > 0
    assert rel(fe, fe_ref) < 1e-6


def test_pinned_host_buffers_move_by_sm_copies(gpu_lib):
    """Upload, download and the reference-signature step through page-locked host buffers take the
    SM copy kernel (one more launch per transfer) and give the same bits as pageable buffers (the
    copy engine path)."""
    from mpc_gb300.capi import PinnedArray, Propagator
    p, A, o = small_cell()
    pin_in, pin_out = PinnedArray(p.N), PinnedArray(p.N)
    with Propagator(p) as prop:
        n0 = prop.launch_count()
        prop.upload(A)
        n1 = prop.launch_count()
        ref = prop.download()
        n2 = prop.launch_count()
        pin_in.array[:] = A
        prop.upload(pin_in.array)
        n3 = prop.launch_count()
        prop.download(pin_out.array)
        n4 = prop.launch_count()
        assert (n3 - n2) == (n1 - n0) + 1 and (n4 - n3) == (n2 - n1) + 1
        assert np.array_equal(pin_out.array, ref)
        # one reference-signature step on a pageable and on a pinned copy of the same field
        B = ref.copy()
        prop.ssfmprop(B, p.dzz, 1, 0.0, p.puls_e)
        pin_in.array[:] = ref
        prop.ssfmprop(pin_in.array, p.dzz, 1, 0.0, p.puls_e)
        assert np.array_equal(pin_in.array, B)
    pin_in.free()
    pin_out.free()


@pytest.mark.parametrize("plasm,sst", [(1, 1), (0, 1), (1, 0), (0, 0)])
def test_ssfmprop_one_step(gpu_lib, plasm, sst):
    from mpc_gb300.capi import Propagator
    p, A, o = small_cell(energy=3e-3, fwhm=120e-15, pressure=3.0, beam_w=0.3e-3, plasm=plasm, sst_on=sst)
    ref = A.copy()
    r_or = o.ssfmprop(ref, p.dzz, 1, 0.0, p.puls_e, change=1)
    with Propagator(p) as prop:
        got = A.copy()
        r_gpu = prop.ssfmprop(got, p.dzz, 1, 0.0, p.puls_e, change=1)
    assert rel(got, ref) < 1e-5
    assert rel(r_gpu["BP1"], r_or["BP1"]) < 1e-5 and rel(r_gpu["BP2"], r_or["BP2"]) < 1e-5
    assert np.allclose(r_gpu["y1"], r_or["y1"], rtol=1e-6) and r_gpu["signmem"] == r_or["signmem"]


@pytest.mark.parametrize("bounce", [BOUNCE_LENS, BOUNCE_SIGNFLIP])
def test_run_fixed_two_passes(gpu_lib, bounce):
    """100 fixed steps (2 passes of 50, mirror bounce between them) on 32x32x256."""
    from mpc_gb300.capi import Propagator
    p, A, o = small_cell(energy=2e-3, fwhm=150e-15, pressure=2.0, bounce=bounce, steps_per_pass=50)
    o2 = oracle.Oracle(p)
    ref = A.copy()
    st = o2.new_state()
    o2.run_fixed(ref, st, 100)
    with Propagator(p) as prop:
        prop.upload(A)
        prop.run_fixed(100)
        got = prop.download()
        s = prop.state()
    assert s.nstep == 100 and abs(s.z - st.z) < 1e-12
    assert rel(got, ref) < 1e-4
    # spectrum
    assert rel(np.abs(np.fft.fft(got.reshape(p.Nt, -1), axis=0)), np.abs(np.fft.fft(ref.reshape(p.Nt, -1), axis=0))) < 1e-4


def test_diag(gpu_lib):
    from mpc_gb300.capi import Propagator
    p, A, o = small_cell()
    with Propagator(p) as prop:
        prop.upload(A)
        temp, spec, BP1, BP2 = prop.diag()
        energy = prop.energy()
    t_ref, s_ref, b1, b2 = o.diag(A)
    assert rel(temp, t_ref) < 1e-6 and rel(spec, s_ref) < 1e-6
    assert rel(BP1, b1) < 1e-6 and rel(BP2, b2) < 1e-6
    assert abs(energy / o.energy(A) - 1) < 1e-6


def test_setStep(gpu_lib):
    from mpc_gb300.capi import Propagator
    p, A, o = small_cell()
    rng = np.random.default_rng(3)
    for scale in (1e-7, 1e-5, 3e-5, 1e-3):
        C1 = A.copy()
        C2 = A + scale * np.abs(A).max() * rng.standard_normal(A.size)
        y = np.array([0.0, 1e-3, 0, 0])
        ref = oracle.setStep(1e-3, C1, C2, p.def_err, p.dzmin, y, y)
        with Propagator(p) as prop:
            got = prop.setStep(1e-3, C1, C2, y, y)
        assert got[1] == ref[1] and abs(got[0] - ref[0]) < 1e-15 and abs(got[2] / ref[2] - 1) < 1e-12


def test_energy_conservation_no_plasma(gpu_lib):
    """Kerr + SST + dispersion + diffraction, alpha = 0, no plasma: energy is invariant."""
    from mpc_gb300.capi import Propagator
    p, A, o = small_cell(plasm=0, energy=2e-3)
    with Propagator(p) as prop:
        prop.upload(A)
        e0 = prop.energy()
        prop.run_fixed(100)
        e1 = prop.energy()
    # the exponential integrator of the self-steepening term changes the energy at O(dz^2);
    # the device run reproduces the FP64 oracle's own drift
    ref = A.copy()
    st = o.new_state()
    o.run_fixed(ref, st, 100)
    drift_ref = o.energy(ref) / o.energy(A) - 1
    assert abs(drift_ref) < 5e-5
    assert abs((e1 / e0 - 1) - drift_ref) < 1e-6


def test_create_destroy_leaves_no_pending_error(gpu_lib):
    """The library shares the CUDA runtime (libcudart.so) with its caller, so a failed runtime
    call inside it would surface in the caller's next CUDA call; a context's whole life must
    leave no error pending."""
    import ctypes

    from mpc_gb300.capi import Propagator
    cudart = ctypes.CDLL("libcudart.so.13")      # the instance the library already loaded
    cudart.cudaGetLastError.restype = ctypes.c_int
    cudart.cudaGetLastError()
    p, A = inputs.make_cell(inputs.cell64(Nx=32, Ny=32, Nt=256))
    with Propagator(p) as prop:
        prop.ssfmprop(A.copy(), p.dzz, 1, 0.0, p.puls_e, change=1)
    assert cudart.cudaGetLastError() == 0


@pytest.mark.parametrize("grid,bounce", [((64, 64, 512), False), ((128, 128, 1024), False), ((256, 256, 512), False),
                                         ((256, 256, 2048), False), ((512, 512, 1024), False),
                                         ((128, 128, 1024), True), ((256, 256, 512), True), ((256, 256, 2048), True)])
def test_kernel_variants_agree(gpu_lib, grid, bounce):
    """Every compiled kernel variant of a grid (device layout, tile and launch shapes) gives the
    same field after 6 split steps; an index past the last variant is rejected; the
    autotuner (variant = -1) picks one of them.  With `bounce`, the cell is 5 steps long at the
    same step length, so the sixth step crosses the mirror: the plane sweep's lens form
    (linear step, lens phase, linear step) runs in every variant."""
    from mpc_gb300.capi import MPCError, Propagator
    Nx, Ny, Nt = grid
    extra = dict(cav=0.5 / 400 * 5, steps_per_pass=5, bounce=BOUNCE_LENS) if bounce else {}
    cfg = inputs.cell256(Nx=Nx, Ny=Ny, Nt=Nt, window_xy=8e-3 * Nx / 256, window_t=4e-12 * Nt / 2048, **extra)
    p0, A = inputs.make_cell(cfg)
    ref = None
    v = 0
    while True:
        try:
            prop = Propagator(p0.copy(variant=v))
        except MPCError:
            break
        with prop:
            assert prop.variant_info()["variant"] == v
            prop.upload(A, calibrate=True)
            prop.run_fixed(6)
            out = prop.download()
        if ref is None:
            ref = out
        else:
            # same-chunk variants agree bit for bit; 16-sample chunks differ by FP32 composition
            # (~1e-7 per step), with margin for the stronger field after the lens
            assert np.linalg.norm(out - ref) / np.linalg.norm(ref) < (2e-6 if bounce else 1e-6), v
        v += 1
    assert v >= 2
    with Propagator(p0.copy(variant=-1)) as prop:
        assert 0 <= prop.variant_info()["variant"] < v


@pytest.mark.parametrize("grid", [(128, 128, 1024), (512, 512, 1024)])
def test_step_double_variants_agree(gpu_lib, grid):
    """Step-doubling attempts write their trial fields to other buffers than the one they read
    (the plane sweep out of place); every kernel variant of the grid, cluster or strip plane
    sweep, gives the same decisions, step sizes and fields (all with 32-sample chunks: the same
    arithmetic)."""
    from mpc_gb300.capi import MPCError, Propagator
    Nx, Ny, Nt = grid
    cfg = inputs.cell256(Nx=Nx, Ny=Ny, Nt=Nt, window_xy=8e-3 * Nx / 256, window_t=4e-12 * Nt / 2048, def_err=1e-5)
    p0, A = inputs.make_cell(cfg)
    ref = None
    v = 0
    while True:
        try:
            prop = Propagator(p0.copy(variant=v))
        except MPCError:
            break
        with prop:
            prop.upload(A, calibrate=True)
            rec = [prop.step_double() for _ in range(2)]
            s = prop.state()
            out = (rec, s.z, s.dzz, s.nstep, prop.download())
        if ref is None:
            ref = out
        else:
            assert [r["bad"] for r in out[0]] == [r["bad"] for r in ref[0]], v
            assert [r["err"] for r in out[0]] == pytest.approx([r["err"] for r in ref[0]], rel=1e-6), v
            assert out[1:4] == pytest.approx(ref[1:4], rel=1e-12), v
            assert np.linalg.norm(out[4] - ref[4]) / np.linalg.norm(ref[4]) < 1e-6, v
        v += 1
    assert v >= 2


@pytest.mark.parametrize("bounce", [BOUNCE_LENS, BOUNCE_SIGNFLIP])
def test_step_double_matches_oracle(gpu_lib, bounce):
    """Adaptive step-doubling attempts (MPC.c:269-383) on the device field against the
    oracle's, until the pulse has crossed a mirror plane: the same accept/reject decisions,
    step sizes, z, mirror bounces and loss, beam sizes, and the field within the multi-step
    tolerance."""
    from mpc_gb300.capi import Propagator
    p, A, o = small_cell(energy=2e-3, fwhm=150e-15, pressure=2.0, bounce=bounce, steps_per_pass=4, Ab_M=0.9,
                         def_err=3e-4)
    o2 = oracle.Oracle(p)
    ref = A.copy()
    C1 = np.empty_like(ref)
    C2 = np.empty_like(ref)
    st = o2.new_state()
    decisions = []
    with Propagator(p) as prop:
        prop.upload(A)
        for k in range(80):
            if st.z > p.Cav + 2 * st.dzz:
                break
            o2.double_step(ref, C1, C2, st)
            r = prop.step_double(profiles=True)
            s = prop.state()
            decisions.append(r["bad"])
            assert r["bad"] == st.bad, k
            assert abs(r["err"] / st.err - 1) < 0.05, (k, r["err"], st.err)
            assert s.dzz == pytest.approx(st.dzz, rel=1e-12) and s.z == pytest.approx(st.z, rel=1e-12, abs=1e-15)
            assert s.nstep == st.nstep and s.attempts == st.attempts and s.signmem == st.signmem
            assert s.puls_e == pytest.approx(st.puls_e, rel=1e-12)
            # beam sizes from C2's profiles: crossing positions on the r grid, profile values
            assert list(s.y1)[:2] == list(st.y1)[:2] and list(s.y2)[:2] == list(st.y2)[:2], k
            assert list(s.y1)[2:] == pytest.approx(list(st.y1)[2:], rel=1e-4)
            assert s.bps1 == pytest.approx(st.bps1, rel=1e-12) and r["BP1"].max() > 0
        got = prop.download()
    assert 0 in decisions and 1 in decisions          # both branches exercised
    assert st.z > p.Cav                                # at least one mirror bounce
    assert st.puls_e < p.puls_e                        # the mirror loss was applied
    assert rel(got, ref) < 1e-4


def test_mirror_bounce_lens(gpu_lib):
    import ctypes as C

    from mpc_gb300.capi import Propagator
    p, A, o = small_cell(bounce=BOUNCE_LENS, Ab_M=0.95)
    ref = A.copy()
    L = oracle.lib()
    cd = C.POINTER(C.c_double)
    L.or_mirror_lens.argtypes = [cd, C.c_int, C.c_int, C.c_int, cd, C.c_double, C.c_double]
    r = np.ascontiguousarray(p.r, dtype=np.float64)
    L.or_mirror_lens(oracle._p(ref.view(np.float64)), p.Nx, p.Ny, p.Nt, oracle._p(r), p.k0, p.roc)
    with Propagator(p) as prop:
        prop.upload(A)
        prop.mirror_bounce(BOUNCE_LENS)
        got = prop.download()
        assert prop.state().puls_e == pytest.approx(p.puls_e * 0.95, rel=1e-12)
    assert rel(got, ref) < 1e-5


def test_step_of_many_lengths_matches_oracle(gpu_lib):
    """mpc_step with 120 different lengths (the phase-table cache is recycled on the way) follows
    the oracle's split steps of the same lengths."""
    from mpc_gb300.capi import Propagator
    p, A, o = small_cell(Nx=16, Ny=16, Nt=64, window_xy=2e-3, window_t=1e-12, energy=0.3e-3)
    lengths = p.dzz * 0.2 * (1.0 + 0.01 * np.arange(120))
    assert lengths.sum() < p.Cav                       # no mirror plane on the way
    ref = A.copy()
    z, sm = 0.0, 1
    for dz in lengths:
        sm = o.ssfmprop(ref, float(dz), sm, z, p.puls_e)["signmem"]
        z += dz
    with Propagator(p) as prop:
        prop.upload(A)
        for dz in lengths:
            prop.step(float(dz))
        got = prop.download()
        assert prop.state().z == pytest.approx(z, rel=1e-12) and prop.state().nstep == len(lengths)
    assert rel(got, ref) < 1e-4


def test_error_paths_return_status_and_leave_the_context_usable(gpu_lib):
    """Errors come back as status codes with a message (the reference prints and exits or
    carries on): unsupported grid, Nx != Ny, a variant past the last, calls before a field is
    uploaded, null arguments, a non-positive step; afterwards the context still works."""
    from mpc_gb300.capi import ERRORS, MPCError, Propagator
    lib = gpu_lib
    p, A, o = small_cell()
    assert lib.mpc_shape_supported(48, 48, 300) == 0 and lib.mpc_shape_supported(p.Nx, p.Ny, p.Nt) == 1
    for bad, code in ((p.copy(dims=(48, 48, 300), betas=np.zeros(300), w=np.zeros(300), wr=np.zeros(48),
                                  r=np.zeros(48)), "MPC_ERR_SHAPE"),
                      (p.copy(dims=(32, 16, 256), wr=np.zeros(16), r=np.zeros(16)), "MPC_ERR_SHAPE"),
                      (p.copy(variant=99), "MPC_ERR_ARG"),
                      (p.copy(variant=-2), "MPC_ERR_ARG")):
        with pytest.raises(MPCError, match=code):
            Propagator(bad)
    with Propagator(p) as prop:
        for call in (lambda: prop.run_fixed(3), lambda: prop.download(), lambda: prop.step_double(),
                     lambda: prop.step(1e-3), lambda: prop.energy()):
            with pytest.raises(MPCError, match="MPC_ERR_STATE"):
                call()
        assert lib.mpc_run_fixed(None, 1) == 1                       # MPC_ERR_ARG
        assert lib.mpc_ssfmprop(prop.h, None, 1, 0.01, None, 0.0, None, None, None, None, None, None, None, 0) == 1
        assert b"null" in lib.mpc_last_error()
        prop.upload(A)
        with pytest.raises(MPCError, match="MPC_ERR_ARG"):
            prop.step(0.0)
        with pytest.raises(MPCError, match="MPC_ERR_ARG"):
            prop.mirror_bounce(7)
        prop.run_fixed(2)                                            # still usable
        assert prop.state().nstep == 2 and np.isfinite(prop.download()).all()
    assert set(ERRORS.values()) >= {"MPC_ERR_ARG", "MPC_ERR_SHAPE", "MPC_ERR_STATE"}


def test_features_match_numpy_moments(gpu_lib):
    """The step-size features' moments pass (FP32 runs, FP64 across) against numpy moments of
    the downloaded field: pulse energy, spectral width and centroid (Parseval over t), beam
    widths in x and y (the grid positions r)."""
    from mpc_gb300.capi import Propagator
    p, A, o = small_cell(Nx=64, Ny=64, Nt=512, window_t=4e-12)
    with Propagator(p) as prop:
        prop.upload(A)
        prop.run_fixed(3)
        f = prop.features()
        got = prop.download()
    HBAR = 1.054560652926899e-34
    Nt, Ny, Nx = p.Nt, p.Ny, p.Nx
    F = np.fft.fft(got.reshape(Nt, Ny, Nx), axis=0)
    P = (np.abs(F) ** 2).sum(axis=(1, 2))
    w = np.asarray(p.w)[(np.arange(Nt) + Nt // 2) % Nt]
    E = P.sum()
    wm = (w * P).sum() / E
    ws = np.sqrt((w * w * P).sum() / E - wm ** 2)
    I = (np.abs(got.reshape(Nt, Ny, Nx)) ** 2).sum(axis=0)
    r = np.asarray(p.r)
    Ex = I.sum(axis=0)
    Ey = I.sum(axis=1)
    xm = (r[:Nx] * Ex).sum() / Ex.sum()
    xs = np.sqrt((r[:Nx] ** 2 * Ex).sum() / Ex.sum() - xm ** 2)
    ym = (r[:Ny] * Ey).sum() / Ey.sum()
    ys = np.sqrt((r[:Ny] ** 2 * Ey).sum() / Ey.sum() - ym ** 2)
    energy = np.sum(np.abs(got) ** 2) * p.dr ** 2 * p.deltat * HBAR * p.w0
    window = Nx * p.dr
    assert f[4] == pytest.approx(np.log10(energy), abs=1e-5)
    assert f[5] == pytest.approx(ws / p.w0 * 1e2, rel=1e-4)
    assert f[6] == pytest.approx(wm / p.w0 * 1e2, abs=1e-4 * ws / p.w0 * 1e2)
    assert f[7] == pytest.approx(xs / window, rel=1e-4)
    assert f[8] == pytest.approx(ys / window, rel=1e-4)


def test_bounded_wait_runs_out_and_reports_timeout(gpu_lib):
    """The device-side waits are bounded: a probe kernel waits on an mbarrier that nothing
    completes, gives up after about a second and leaves its code in the context's error word;
    the host reads it as MPC_ERR_TIMEOUT and clears it, and the context keeps working (a fixed
    run afterwards matches one on a fresh context)."""
    import time

    from mpc_gb300.capi import Propagator
    lib = gpu_lib
    p, A, o = small_cell()
    with Propagator(p) as prop:
        prop.upload(A)
        t0 = time.time()
        assert lib.mpc_wait_limit_check(prop.h) == 9                 # MPC_ERR_TIMEOUT
        assert 0.2 < time.time() - t0 < 30
        assert b"wait" in lib.mpc_last_error()
        assert lib.mpc_sync(prop.h) == 0                             # reported once, then cleared
        prop.run_fixed(3)
        got = prop.download()
    with Propagator(p) as prop:
        prop.upload(A)
        prop.run_fixed(3)
        ref = prop.download()
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("grid", [(128, 128, 1024), (256, 256, 512), (256, 256, 2048)])
def test_production_grids_match_oracle(gpu_lib, grid):
    """Two split steps on the sweep's and the benchmark's grids (autotuned kernel variant,
    lens mirror, SST + ADK + plasma) against the FP64 oracle: the split-step tolerance."""
    from mpc_gb300.capi import Propagator
    Nx, Ny, Nt = grid
    cfg = inputs.cell256(Nx=Nx, Ny=Ny, Nt=Nt, window_xy=8e-3 * Nx / 256, window_t=4e-12 * Nt / 2048,
                         energy=1e-3, bounce=BOUNCE_LENS)
    p, A = inputs.make_cell(cfg)
    o = oracle.Oracle(p)
    o.calibrate(A)
    ref = A.copy()
    st = o.new_state()
    o.run_fixed(ref, st, 2)
    with Propagator(p.copy(variant=-1)) as prop:
        prop.upload(A)
        prop.run_fixed(2)
        got = prop.download()
    assert rel(got, ref) < 1e-5


def test_step_double_landing_on_mirror_planes(gpu_lib):
    """With land_mirrors, an attempt that would cross a mirror plane ends on it: some accepted
    state sits exactly on z = Cav, the run still reaches the next pass, and a later attempt
    does not shrink merely because the landing step was short."""
    from mpc_gb300.capi import Propagator
    p, A, o = small_cell(energy=1e-3, steps_per_pass=6, def_err=1e-3)
    with Propagator(p.copy(land_mirrors=1)) as prop:
        prop.upload(A)
        zs = []
        while prop.state().z < 1.5 * p.Cav and len(zs) < 200:
            if prop.step_double()["bad"] == 0:
                zs.append(prop.state().z)
        assert any(abs(z - p.Cav) < 1e-12 for z in zs), zs
        assert zs[-1] >= 1.5 * p.Cav and np.isfinite(prop.download()).all()
