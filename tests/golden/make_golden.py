"""Generate golden vectors from the reference's own code (oracle/_ref/libmpcref.so).

The reference ships no tests or fixtures.  oracle/build_ref.sh compiles the parts of it that
build on their own -- plasma.c (ionizpot, Natoms, ADK, ioniz) and the host functions calcexpR,
fftshift (axis 0), calc1oes and setStep of propagation.c -- and this script runs them on
seeded inputs and stores inputs and outputs in tests/golden/reference_vectors.npz.  The
oracle's as-written switches are checked against these vectors by tests/test_golden.py
(which also runs without the reference mounted).

    bash oracle/build_ref.sh && python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes as C
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
LIB = os.path.join(ROOT, "oracle", "_ref", "libmpcref.so")
OUT = os.path.join(HERE, "reference_vectors.npz")
GASES = ["Argon", "Helium", "Neon", "Air", "Nitrogen", "Xenon", "Krypton"]
HBAR = 1.054560652926899e-34


def _p(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def load():
    lib = C.CDLL(LIB)
    d = C.POINTER(C.c_double)
    lib.ref_ionizpot.argtypes = [C.c_char_p, d, d]
    lib.ref_Natoms.argtypes = [C.c_char_p, d, d]
    lib.ref_ADK.argtypes = [C.c_long, d, d, d, d, d, d, d, d]
    lib.ref_ioniz.argtypes = [d, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_char_p, C.c_double, d,
                              C.c_double, C.c_double, d, d, C.c_double]
    lib.ref_calcexpR.argtypes = [d, C.POINTER(C.c_int), C.c_double, C.c_double, C.c_double, C.c_double, d, C.c_int,
                                 C.c_int]
    lib.ref_fftshift0.argtypes = [d, C.c_int]
    lib.ref_calc1oes.argtypes = [d, C.c_int, d, d, d]
    lib.ref_setStep.argtypes = [C.c_long, d, d, d, C.c_double, C.c_double, d, d, C.POINTER(C.c_int), d]
    return lib


def ion_field(Nx=8, Ny=8, Nt=64, peak=2e18, seed=7):
    """Gaussian pulse whose peak intensity |A|^2 hbar w0 is `peak` W/m^2, plus noise."""
    lam = 1030e-9
    w0 = 2 * math.pi * 299792458.0 / lam
    rng = np.random.default_rng(seed)
    x = (np.arange(Nx) - Nx / 2 + 0.5) / (Nx / 4)
    t = (np.arange(Nt) - Nt / 2 + 0.5) / (Nt / 6)
    g = np.exp(-t[:, None, None] ** 2 - x[None, :, None] ** 2 - x[None, None, :] ** 2)
    amp = math.sqrt(peak / (HBAR * w0))
    A = amp * g * (1 + 0.05 * rng.standard_normal(g.shape)) * np.exp(1j * rng.uniform(0, 2 * np.pi, g.shape))
    return A.reshape(-1).astype(np.complex128), w0


def main():
    if not os.path.exists(LIB):
        sys.exit(f"{LIB} missing: run oracle/build_ref.sh first")
    lib = load()
    out = {}
    # gas tables
    I1 = np.zeros(len(GASES)); I2 = np.zeros(len(GASES)); Na = np.zeros(len(GASES)); sg = np.zeros(len(GASES))
    for i, g in enumerate(GASES):
        a, b = C.c_double(0), C.c_double(0)
        lib.ref_ionizpot(g.encode(), C.byref(a), C.byref(b))
        I1[i], I2[i] = a.value, b.value
        lib.ref_Natoms(g.encode(), C.byref(a), C.byref(b))
        Na[i], sg[i] = a.value, b.value
    out.update(gas_I1=I1, gas_I2=I2, gas_Natm=Na, gas_sigma=sg)
    # ADK on a field grid for two constant sets (argon corrected, argon as written in ioniz)
    E = np.geomspace(2e-3, 0.6, 97)
    Iion = np.array([15.75962, 27.62967]) / 27.21
    sets = {}
    nq_c = np.array([1 / math.sqrt(2 * Iion[0]), 2 / math.sqrt(2 * Iion[1])])
    sets["corrected"] = nq_c
    sets["as_written"] = np.array([(2 * Iion[1]) ** -0.5, 2 / math.sqrt(2 * Iion[1])])
    for name, nq in sets.items():
        Cnl = np.array([math.sqrt(2 ** (2 * n) / (n * math.gamma(n + 1) * math.gamma(n))) for n in nq])
        r1 = np.zeros_like(E); r2 = np.zeros_like(E)
        args = [np.ascontiguousarray(v, dtype=np.float64) for v in (Cnl, [1.0, 1.0], nq, [0.0, 0.0], Iion)]
        lib.ref_ADK(E.size, _p(r1), _p(r2), *(_p(a) for a in args), _p(E))
        out[f"adk_{name}_Cnl"] = args[0]; out[f"adk_{name}_nq"] = args[2]
        out[f"adk_{name}_r1"] = r1; out[f"adk_{name}_r2"] = r2
    out["adk_E"] = E; out["adk_Iion"] = Iion
    # ioniz as written on a small pulse
    Nx, Ny, Nt = 8, 8, 64
    A, w0 = ion_field(Nx, Ny, Nt)
    dt = 4e-15
    w = 2 * np.pi * (np.arange(Nt) - Nt // 2) / (Nt * dt)
    rho_nt = 2.0 * 1.784e3 * 6.02214e23 / 39.941
    rho_c = 8.8541878128e-12 * 9.1094e-31 * w0 ** 2 / 1.602e-19 ** 2
    tau = np.zeros(A.size); fe = np.zeros(A.size)
    lib.ref_ioniz(_p(A.view(np.float64)), Nx, Ny, Nt, w0, dt, b"Argon", rho_c, _p(w), rho_nt, 1.0, _p(tau), _p(fe),
                  Iion[1])
    out.update(ioniz_A=A, ioniz_dims=np.array([Nx, Ny, Nt]), ioniz_w=w,
               ioniz_scalars=np.array([w0, dt, rho_c, rho_nt, 1.0]), ioniz_tau=tau, ioniz_fe=fe)
    # calcexpR as written (real exponent, centred order)
    N = 32
    dx = 4e-3 / N
    wr = 2 * np.pi * (np.arange(N) - N // 2) / (N * dx)
    cases = [(0.1, 1), (0.6, 1), (0.6, -1), (1.2, 1), (1.2, -1)]
    tabs = np.zeros((len(cases), N), dtype=np.complex128)
    signs = np.zeros(len(cases), dtype=np.int64)
    for i, (z, sm) in enumerate(cases):
        s = C.c_int(sm)
        lib.ref_calcexpR(_p(tabs[i].view(np.float64)), C.byref(s), z, 0.5, 2 * math.pi / 1030e-9, 1.25e-3 / 2, _p(wr),
                         N, N)
        signs[i] = s.value
    out.update(expR_cases=np.array(cases, dtype=np.float64), expR_wr=wr, expR_tab=tabs, expR_signmem=signs)
    # fftshift axis 0
    v = (np.arange(16) + 1j * np.arange(16) ** 2).astype(np.complex128)
    sh = v.copy()
    lib.ref_fftshift0(_p(sh.view(np.float64)), 16)
    out.update(shift_in=v, shift_out=sh)
    # calc1oes on Gaussian and noisy profiles
    rng = np.random.default_rng(11)
    r = (np.arange(64) - 32) * 62.5e-6
    bps = []
    ys = []
    BPs = []
    for k in range(6):
        wbeam = (0.3 + 0.15 * k) * 1e-3
        BP = np.exp(-2 * (r - 1e-4 * (k - 3)) ** 2 / wbeam ** 2) * (1 + 0.02 * rng.standard_normal(64))
        vald = C.c_double(0); y = np.zeros(4)
        lib.ref_calc1oes(_p(BP), 64, _p(r), C.byref(vald), _p(y))
        BPs.append(BP); bps.append(vald.value); ys.append(y)
    out.update(c1_r=r, c1_BP=np.array(BPs), c1_bps=np.array(bps), c1_y=np.array(ys))
    # setStep over its branches
    n = 4096
    C1 = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex128)
    res = []
    noise = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    ins = []
    for rel in (3e-5, 1.5e-5, 0.7e-5, 0.2e-5, 1e-7):
        C2 = C1 + rel * noise
        for (dzz, dzmin, ycap) in ((1e-3, 1e-7, 1.0), (1e-3, 1e-3, 1.0), (1e-3, 1e-7, 1e-6)):
            d = C.c_double(dzz); bad = C.c_int(0); err = C.c_double(0)
            y1 = np.array([0, ycap, 0, 0.0]); y2 = y1.copy()
            lib.ref_setStep(n, C.byref(d), _p(C1.view(np.float64)), _p(C2.view(np.float64)), 1e-5, dzmin, _p(y1),
                            _p(y2), C.byref(bad), C.byref(err))
            ins.append([rel, dzz, dzmin, ycap]); res.append([d.value, bad.value, err.value])
    out.update(ss_C1=C1, ss_noise=noise, ss_in=np.array(ins), ss_out=np.array(res))
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
