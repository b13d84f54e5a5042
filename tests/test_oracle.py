"""Known-answer tests of the FP64 oracle (the reference ships none, so these pin the
restated physics): FFT vs numpy, analytic Gaussian-beam diffraction and GDD broadening,
exact SPM phase, energy conservation, spectral derivative, ADK closed form, forward
ionization prefix, O(dz^3) local error of the split step with Richardson gaining an order,
and the mirror lens against ABCD Gaussian-beam propagation."""
import math

import numpy as np
import pytest

import oracle
from mpc_gb300 import inputs
from mpc_gb300.params import BOUNCE_LENS, BOUNCE_SIGNFLIP


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("dims", [(16, 8, 32), (64, 64, 8), (4, 4, 2048)])
def test_fft_vs_numpy(dims):
    rng = np.random.default_rng(0)
    Nx, Ny, Nt = dims
    A = rng.standard_normal(Nx * Ny * Nt) + 1j * rng.standard_normal(Nx * Ny * Nt)
    for ax, npax in ((0, 2), (1, 1), (2, 0)):
        for sign in (-1, 1):
            B = A.copy()
            oracle.fft_axis(B, dims, ax, sign)
            f = np.fft.fft if sign < 0 else (lambda x, axis: np.fft.ifft(x, axis=axis) * x.shape[axis])
            ref = f(A.reshape(Nt, Ny, Nx), axis=npax).reshape(-1)
            assert rel(B, ref) < 1e-13


def linear_cell(**kw):
    cfg = inputs.cell64(**{**dict(Nx=64, Ny=64, Nt=64, window_t=2e-12, noise=0.0, sst_on=0, plasm=0), **kw})
    p, A = inputs.make_cell(cfg)
    return cfg, p, A


def test_diffraction_gaussian_beam():
    """No dispersion or nonlinearity: the beam follows A = g exp(-r^2 s),
    s = 1/(w0^2 (1 + i z/zR)), g = 1/(1 + i z/zR), zR = k0 w0^2/2."""
    cfg, p, A = linear_cell(Nt=4, window_t=2e-12, fwhm=1e-9, bounce=BOUNCE_SIGNFLIP)
    p = p.copy(gamma2=0.0, betas=np.zeros(p.Nt))
    o = oracle.Oracle(p)
    st = o.new_state()
    st.dzz = 0.05
    o.run_fixed(A, st, 8)   # z = 0.4 m < Cav: diffraction sign +1 all along
    z = 0.4
    zR = p.k0 * cfg.beam_w ** 2 / 2
    q = 1 + 1j * z / zR
    x = p.r
    r2 = x[None, :] ** 2 + x[:, None] ** 2
    tprof = np.exp(-2 * math.log(2) * ((np.arange(p.Nt) - p.Nt // 2) * p.deltat / cfg.fwhm) ** 2)
    ref = (tprof[:, None, None] * (np.exp(-r2 / (cfg.beam_w ** 2 * q)) / q)[None]).reshape(-1)
    # the periodic 4 mm window truncates the continuous solution's tails at the 1e-6 level
    assert rel(A, ref) < 1e-5


def test_dispersion_gdd_broadening():
    """Only beta2: A = T0/sqrt(T0^2 - i beta2 z) exp(-t^2 / (2 (T0^2 - i beta2 z)))."""
    cfg, p, A = linear_cell(Nx=4, Ny=4, Nt=512, window_t=4e-12, window_xy=1.0, beam_w=1e6, fwhm=150e-15,
                            bounce=BOUNCE_SIGNFLIP)
    beta2 = 2e-26
    p = p.copy(gamma2=0.0, betas=beta2 / 2 * p.w ** 2, wr=np.zeros(p.Ny))
    o = oracle.Oracle(p)
    st = o.new_state()
    st.dzz = 0.05
    o.run_fixed(A, st, 8)
    z = 0.4
    T0 = cfg.fwhm / (2 * math.sqrt(math.log(2)))
    t = (np.arange(p.Nt) - p.Nt // 2) * p.deltat
    Q = T0 ** 2 - 1j * beta2 * z
    ref_t = T0 / np.sqrt(Q) * np.exp(-t ** 2 / (2 * Q))
    got = A.reshape(p.Nt, p.Ny, p.Nx)[:, 1, 1]
    scale = got[p.Nt // 2] / ref_t[p.Nt // 2]      # transverse factor (flat to 1e-12)
    assert abs(abs(scale) - 1) < 1e-9
    assert rel(got, ref_t) < 1e-9


def test_spm_phase_exact():
    """Kerr only on a transversely flat field: |A| invariant, phase = gamma2 |A|^2 z."""
    cfg, p, A = linear_cell(Nx=8, Ny=8, Nt=128, window_xy=1.0, beam_w=1e6, fwhm=300e-15, bounce=BOUNCE_SIGNFLIP)
    p = p.copy(betas=np.zeros(p.Nt))
    o = oracle.Oracle(p)
    o.calibrate(A)
    A0 = A.copy()
    st = o.new_state()
    st.dzz = 0.01
    o.run_fixed(A, st, 10)
    assert np.allclose(np.abs(A), np.abs(A0), rtol=1e-12, atol=1e-12 * np.abs(A0).max())
    ph = np.angle(A / A0)
    expect = np.angle(np.exp(1j * p.gamma2 * np.abs(A0) ** 2 * 0.1))
    m = np.abs(A0) > 1e-3 * np.abs(A0).max()
    assert np.abs(ph[m] - expect[m]).max() < 1e-9


@pytest.mark.parametrize("sst", [0, 1])
def test_energy_conserved_without_plasma(sst):
    cfg = inputs.cell64(Nx=32, Ny=32, Nt=128, window_t=1e-12, energy=1e-3, plasm=0, sst_on=sst, steps_per_pass=20)
    p, A = inputs.make_cell(cfg)
    o = oracle.Oracle(p)
    o.calibrate(A)
    e0 = o.energy(A)
    st = o.new_state()
    o.run_fixed(A, st, 30)
    drift = abs(o.energy(A) / e0 - 1)
    assert drift < (1e-12 if sst == 0 else 1e-5)


def test_plasma_absorbs_energy():
    cfg = inputs.cell64(Nx=32, Ny=32, Nt=128, window_t=1e-12, energy=3e-3, fwhm=100e-15, beam_w=0.15e-3,
                         pressure=3.0, steps_per_pass=20)
    p, A = inputs.make_cell(cfg)
    o = oracle.Oracle(p)
    o.calibrate(A)
    e0 = o.energy(A)
    st = o.new_state()
    o.run_fixed(A, st, 5)
    assert o.energy(A) < e0 * (1 - 1e-9)


def test_sst_derivative_of_gaussian():
    """dA = IFFT(-i w FFT A)/Nt equals -dA/dt of a Gaussian; sst built from it
    (propagation.c:215-233)."""
    cfg, p, A = linear_cell(Nx=4, Ny=4, Nt=1024, window_t=4e-12, window_xy=1.0, beam_w=1e6, fwhm=200e-15)
    o = oracle.Oracle(p)
    sst = o.sst(A)
    T = cfg.fwhm / math.sqrt(2 * math.log(2)) / math.sqrt(2)   # A = exp(-t^2/(2 T^2)) * 1
    t = (np.arange(p.Nt) - p.Nt // 2) * p.deltat
    a = A.reshape(p.Nt, -1)[:, 5]
    dA_dt = -t / T ** 2 * a
    dA = -dA_dt
    ref = p.gamma2 / p.w0 * (2 * dA * np.conj(a) + a * np.conj(dA))
    assert rel(sst.reshape(p.Nt, -1)[:, 5], ref) < 1e-10


def test_adk_closed_form():
    """Rates of both argon stages against an independent numpy evaluation of the ADK formula."""
    E = np.geomspace(1e-3, 1.0, 50)
    Iion = np.array([15.75962, 27.62967]) / 27.21
    nq = np.array([1 / math.sqrt(2 * Iion[0]), 2 / math.sqrt(2 * Iion[1])])
    Cnl = np.array([math.sqrt(2 ** (2 * n) / (n * math.gamma(n + 1) * math.gamma(n))) for n in nq])
    r1, r2 = oracle.ADK(E, Cnl, [1, 1], nq, [0, 0], Iion)
    for r, s in ((r1, 0), (r2, 1)):
        F0 = (2 * Iion[s]) ** 1.5
        w = Cnl[s] ** 2 * math.sqrt(6 / math.pi) * Iion[s] * (2 * F0 / E) ** (2 * nq[s] - 1.5) * np.exp(-2 * F0 / (3 * E))
        np.testing.assert_allclose(r, w, rtol=1e-12)
    # argon at 1e14 W/cm^2: about 1e-3 of the atoms ionized per 100 fs (order of magnitude)
    F = math.sqrt(2 * 377 * 1e18) * 0.89 / 5.14220642e11
    rate = oracle.ADK(np.array([F]), Cnl, [1, 1], nq, [0, 0], Iion)[0][0] / 2.4188843265e-17
    assert 1e8 < rate < 1e13


def test_ionization_grows_forward_in_time():
    """Corrected prefix (A15): the free-electron density is non-decreasing along t on axis
    (the scan runs from the leading edge); as written it runs from the trailing edge."""
    cfg = inputs.cell64(Nx=16, Ny=16, Nt=256, window_t=1e-12, energy=3e-3, fwhm=80e-15, beam_w=0.1e-3,
                         pressure=3.0, noise=0.0)
    p, A = inputs.make_cell(cfg)
    o = oracle.Oracle(p)
    o.calibrate(A)
    axis = p.Ny // 2 * p.Nx + p.Nx // 2

    def ions_on_axis(orc):
        tau, fe = orc.ioniz(A)
        assert np.isfinite(fe).all()
        tau = tau.reshape(p.Nt, -1)[:, axis]
        k4 = (p.w0 / 299792458.0) / (p.n0 * p.rho_c) * p.w0
        sigma = k4 * tau / (1 + p.w0 ** 2 * tau ** 2)       # plasma.c:211
        return fe.reshape(p.Nt, -1)[:, axis] / sigma

    ions = ions_on_axis(o)
    assert ions[0] == 0.0 and ions[-1] > 1e-9                  # grows from the leading edge
    assert np.all(np.diff(ions) >= -1e-15 * ions.max())        # and never decreases
    ions_w = ions_on_axis(oracle.Oracle(p, ion_forward=0))
    assert ions_w[1] > 0.5 * ions.max() and ions_w[-1] < 1e-3 * ions.max()   # as written: time reversed


def test_step_doubling_order():
    """Local error of the symmetric split step is O(dz^3): halving dz divides the
    step-doubling error estimate by ~8; Richardson's (4 C2 - C1)/3 is closer to a
    fine-step reference than C2."""
    cfg = inputs.cell64(Nx=16, Ny=16, Nt=128, window_t=1e-12, window_xy=2e-3, energy=2e-3, beam_w=0.2e-3,
                         plasm=0, sst_on=0, steps_per_pass=4)
    p, A = inputs.make_cell(cfg)
    p = p.copy(def_err=1.0)          # accept every attempt
    o = oracle.Oracle(p)
    o.calibrate(A)
    errs = []
    for dz in (0.02, 0.01):
        st = o.new_state()
        st.dzz = dz
        B, C1, C2 = A.copy(), np.zeros_like(A), np.zeros_like(A)
        o.double_step(B, C1, C2, st)
        errs.append(st.err)
    assert 5.5 < errs[0] / errs[1] < 10.5
    # Richardson vs a fine reference over 2*dz
    dz = 0.02
    st = o.new_state()
    st.dzz = dz
    B, C1, C2 = A.copy(), np.zeros_like(A), np.zeros_like(A)
    o.double_step(B, C1, C2, st)
    ref = A.copy()
    s2 = o.new_state()
    s2.dzz = 2 * dz / 64
    o.run_fixed(ref, s2, 64)
    assert rel(B, ref) < 0.25 * rel(C2, ref)


def test_lens_mode_vs_abcd():
    """Linear propagation through the cell with the mirror lens at each bounce follows the
    ABCD law for the Gaussian q parameter (free space L, then thin lens f = R/2)."""
    cfg = inputs.cell64(Nx=128, Ny=128, Nt=4, window_xy=8e-3, window_t=2e-12, fwhm=1e-9, noise=0.0, sst_on=0,
                         plasm=0, steps_per_pass=25, bounce=BOUNCE_LENS, roc=0.3, cav=0.5, beam_w=0.5e-3)
    p, A = inputs.make_cell(cfg)
    p = p.copy(gamma2=0.0, betas=np.zeros(p.Nt))
    o = oracle.Oracle(p)
    st = o.new_state()
    lam = 2 * math.pi / p.k0
    q = 1j * math.pi * cfg.beam_w ** 2 / lam          # flat phase at the mirror plane
    x = p.r
    for n_pass in range(3):
        o.run_fixed(A, st, 25)
        q = q + cfg.cav                                 # free space
        q = q / (1 - q / (cfg.roc / 2))                 # thin lens f = R/2 (after the pass)
        w_abcd = math.sqrt(-lam / (math.pi * (1 / q).imag))
        I = np.abs(A.reshape(p.Nt, p.Ny, p.Nx)[0]) ** 2
        w_num = 2 * math.sqrt((I * x[None, :] ** 2).sum() / I.sum())
        assert abs(w_num / w_abcd - 1) < 2e-3
