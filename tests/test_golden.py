"""The oracle's restatement pinned against vectors produced by the reference's own code
(tests/golden/reference_vectors.npz, made by tests/golden/make_golden.py from
oracle/_ref/libmpcref.so, which compiles plasma.c and propagation.c's host functions)."""
import math
import os

import numpy as np
import pytest

import oracle

HERE = os.path.dirname(os.path.abspath(__file__))
G = np.load(os.path.join(HERE, "golden", "reference_vectors.npz"))
GASES = ["Argon", "Helium", "Neon", "Air", "Nitrogen", "Xenon", "Krypton"]


def test_gas_tables_exact():
    for i, g in enumerate(GASES):
        I1, I2 = oracle.ionizpot(g)
        Na, sg = oracle.Natoms(g)
        assert (I1, I2) == (G["gas_I1"][i], G["gas_I2"][i])
        assert Na == pytest.approx(G["gas_Natm"][i], rel=1e-15) and sg == G["gas_sigma"][i]


@pytest.mark.parametrize("which", ["corrected", "as_written"])
def test_adk(which):
    E = G["adk_E"]
    r1, r2 = oracle.ADK(E, G[f"adk_{which}_Cnl"], [1.0, 1.0], G[f"adk_{which}_nq"], [0.0, 0.0], G["adk_Iion"])
    np.testing.assert_allclose(r1, G[f"adk_{which}_r1"], rtol=1e-13, atol=0)
    np.testing.assert_allclose(r2, G[f"adk_{which}_r2"], rtol=1e-13, atol=0)


class _P:
    pass


def test_ioniz_as_written():
    """plasma.c:118-245 as written: descending prefix, ve with w[k], n*_0 from Iion[1]."""
    Nx, Ny, Nt = (int(v) for v in G["ioniz_dims"])
    w0, dt, rho_c, rho_nt, n0 = G["ioniz_scalars"]
    p = _P()
    p.dims = (Nx, Ny, Nt)
    p.betas = np.zeros(Nt); p.wr = np.zeros(Ny); p.w = G["ioniz_w"]; p.r = np.zeros(Ny)
    for k, v in dict(dist=1, dzz=1, alpha=0, Cav=1, k0=1, sst_on=0, gamma2=0, w0=w0, plasm=1, deltat=dt, rho_c=rho_c,
                     rho_nt=rho_nt, n0=n0, puls_e=1, Ab_M=1, dr=1, def_err=1, dzmin=1, Esig=1, gas="Argon").items():
        setattr(p, k, v)
    o = oracle.Oracle(p, ion_forward=0, ion_nq=0, ve_omega0=0)
    tau, fe = o.ioniz(G["ioniz_A"].copy())
    np.testing.assert_allclose(tau, G["ioniz_tau"], rtol=1e-12)
    np.testing.assert_allclose(fe, G["ioniz_fe"], rtol=1e-10, atol=1e-12 * np.abs(G["ioniz_fe"]).max())
    assert np.abs(G["ioniz_fe"]).max() > 0


def test_calcexpR_as_written():
    wr = G["expR_wr"]
    N = wr.size
    p = _P()
    p.dims = (N, N, 4)
    p.betas = np.zeros(4); p.wr = wr; p.w = np.zeros(4); p.r = np.zeros(N)
    for k, v in dict(dist=1, dzz=1, alpha=0, Cav=0.5, k0=2 * math.pi / 1030e-9, sst_on=0, gamma2=0, w0=1, plasm=0,
                     deltat=1, rho_c=1, rho_nt=1, n0=1, puls_e=1, Ab_M=1, dr=1, def_err=1, dzmin=1, Esig=1,
                     gas="Argon").items():
        setattr(p, k, v)
    o = oracle.Oracle(p, diffr_phase=0, diffr_fftorder=0, diffr_center=0)
    for i, (z, sm) in enumerate(G["expR_cases"]):
        tab, s = o.calcexpR(N, int(sm), z, 1.25e-3 / 2)
        np.testing.assert_allclose(tab, G["expR_tab"][i], rtol=1e-14)
        assert s == G["expR_signmem"][i]


def test_fftshift_axis0():
    """or_expD0's swap of halves equals the reference's fftshift(axis 0)."""
    v = G["shift_in"]
    n = v.size
    np.testing.assert_array_equal(np.concatenate([v[n // 2:], v[:n // 2]]), G["shift_out"])


def test_calc1oes():
    r = G["c1_r"]
    for BP, bps, y in zip(G["c1_BP"], G["c1_bps"], G["c1_y"]):
        v, yy = oracle.calc1oes(BP, r)
        assert v == bps
        np.testing.assert_array_equal(yy, y)


def test_library_calc1oes_matches_reference_vectors():
    """The library's own host-side calc1oes (mpc_calc1oes, the beam-size search used after every
    accepted step) against the vectors generated from the reference's code; no GPU call."""
    from mpc_gb300 import build, capi
    build.build()
    r = G["c1_r"]
    for BP, bps, y in zip(G["c1_BP"], G["c1_bps"], G["c1_y"]):
        v, yy = capi.calc1oes(BP, r)
        assert v == bps
        np.testing.assert_array_equal(yy, y)


def test_setStep():
    C1 = G["ss_C1"]
    noise = G["ss_noise"]
    for (rel, dzz, dzmin, ycap), (dz_ref, bad_ref, err_ref) in zip(G["ss_in"], G["ss_out"]):
        C2 = C1 + rel * noise
        y = np.array([0, ycap, 0, 0.0])
        dz, bad, err = oracle.setStep(dzz, C1.copy(), C2, 1e-5, dzmin, y, y)
        assert bad == bad_ref and dz == pytest.approx(dz_ref, rel=1e-15)
        assert err == pytest.approx(err_ref, rel=1e-12)


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(HERE), "oracle", "_ref", "libmpcref.so")),
                    reason="reference sources not compiled here")
def test_vectors_reproduce_from_reference():
    """When the reference is mounted, the fixture regenerates bit for bit from its code."""
    import ctypes as C
    import sys
    sys.path.insert(0, os.path.join(HERE, "golden"))
    import make_golden
    lib = make_golden.load()
    E = G["adk_E"]
    r1 = np.zeros_like(E); r2 = np.zeros_like(E)
    args = [np.ascontiguousarray(G[k]) for k in ("adk_corrected_Cnl",)] + [np.array([1.0, 1.0])] + \
        [G["adk_corrected_nq"], np.zeros(2), G["adk_Iion"]]
    lib.ref_ADK(E.size, make_golden._p(r1), make_golden._p(r2), *(make_golden._p(np.ascontiguousarray(a, dtype=np.float64))
                                                                   for a in args), make_golden._p(E))
    np.testing.assert_array_equal(r1, G["adk_corrected_r1"])
    a = C.c_double(0); b = C.c_double(0)
    lib.ref_ionizpot(b"Argon", C.byref(a), C.byref(b))
    assert a.value == G["gas_I1"][0]
    # ioniz as written, on the stored pulse
    Nx, Ny, Nt = (int(v) for v in G["ioniz_dims"])
    w0, dt, rho_c, rho_nt, n0 = (float(v) for v in G["ioniz_scalars"])
    A = np.ascontiguousarray(G["ioniz_A"])
    w = np.ascontiguousarray(G["ioniz_w"])
    tau = np.zeros(A.size); fe = np.zeros(A.size)
    lib.ref_ioniz(make_golden._p(A.view(np.float64)), Nx, Ny, Nt, w0, dt, b"Argon", rho_c, make_golden._p(w), rho_nt,
                  n0, make_golden._p(tau), make_golden._p(fe), float(G["adk_Iion"][1]))
    np.testing.assert_array_equal(tau, G["ioniz_tau"])
    np.testing.assert_array_equal(fe, G["ioniz_fe"])
