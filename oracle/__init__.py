"""ctypes wrappers of the FP64 oracles: the CPU restatement (oracle/mpc_oracle.c) and its
FP64 GPU counterpart (oracle/mpc_oracle64.cu, cuFFT Z2Z plus FP64 kernels) for whole runs of the
large cells.

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and by bench.py's
cpu_baseline / reference arm, as the checker and the CPU baseline.  The product package
never imports it.  build() compiles liboracle.so with gcc (OpenMP, -ffp-contract=off so
x86 and Arm hosts round alike) and liboracle64.so with nvcc (--fmad=false, linked against
liboracle.so for the phase tables, the beam-size search and the step rule).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
SRC = os.path.join(HERE, "mpc_oracle.c")
HDR = os.path.join(HERE, "mpc_oracle.h")
LIB64 = os.path.join(BUILD, "liboracle64.so")
SRC64 = os.path.join(HERE, "mpc_oracle64.cu")
HDR64 = os.path.join(HERE, "mpc_oracle64.h")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class or_params(C.Structure):
    _fields_ = [("Nx", C.c_int), ("Ny", C.c_int), ("Nt", C.c_int), ("dist", C.c_double), ("dzz", C.c_double),
                ("betas", _dp), ("alpha", C.c_double), ("Cav", C.c_double), ("k0", C.c_double), ("wr", _dp),
                ("sst_on", C.c_int), ("w", _dp), ("gamma2", C.c_double), ("w0", C.c_double), ("plasm", C.c_int),
                ("deltat", C.c_double), ("rho_c", C.c_double), ("rho_nt", C.c_double), ("n0", C.c_double),
                ("puls_e", C.c_double), ("Ab_M", C.c_double), ("r", _dp), ("dr", C.c_double),
                ("def_err", C.c_double), ("dzmin", C.c_double), ("Esig", C.c_double), ("gas", C.c_char * 16),
                ("roc", C.c_double)]


SWITCHES = ["diffr_phase", "diffr_fftorder", "diffr_center", "plasma_imag", "nl_apply", "ion_forward", "ion_nq",
            "ve_omega0", "energy_both", "mirror_loss", "z_advance_used", "sigma_limit", "bounce_lens"]


class or_switches(C.Structure):
    _fields_ = [(n, C.c_int) for n in SWITCHES]


class or_state(C.Structure):
    _fields_ = [("z", C.c_double), ("dzz", C.c_double), ("err", C.c_double), ("puls_e", C.c_double),
                ("bps1", C.c_double), ("bps2", C.c_double), ("signmem", C.c_int), ("bad", C.c_int),
                ("nstep", C.c_int), ("attempts", C.c_int), ("y1", C.c_double * 4), ("y2", C.c_double * 4)]


def build(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(SRC), os.path.getmtime(HDR)):
        return LIB
    cmd = ["gcc", "-O3", "-fopenmp", "-fcx-limited-range", "-ffp-contract=off", "-fPIC", "-shared", "-std=gnu11",
           "-o", LIB, SRC, "-lm"]
    subprocess.run(cmd, check=True)
    return LIB


def _nvcc() -> str:
    import shutil
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def build64(force: bool = False) -> str:
    """liboracle64.so: the FP64 GPU oracle for sm_103a, linked against liboracle.so."""
    build(force)
    deps = [SRC64, HDR64, HDR, LIB]
    if not force and os.path.exists(LIB64) and os.path.getmtime(LIB64) >= max(os.path.getmtime(d) for d in deps):
        return LIB64
    cmd = [_nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "--fmad=false",
           "-Xcompiler", "-fPIC,-ffp-contract=off", "-shared", "-o", LIB64, SRC64, f"-L{BUILD}", "-l:liboracle.so",
           "-Xlinker", "-rpath,$ORIGIN", "-lcufft"]
    subprocess.run(cmd, check=True)
    return LIB64


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        L = _lib
        cd = C.POINTER(C.c_double)
        L.or_default_switches.argtypes = [C.POINTER(or_switches)]
        L.or_set_threads.argtypes = [C.c_int]
        L.or_fft_axis.argtypes = [cd, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
        L.or_expD0.argtypes = [cd, C.c_int, C.c_double, C.c_double, cd]
        L.or_calcexpR.argtypes = [cd, C.c_int, C.c_int, _ip, C.c_double, C.c_double, C.c_double, C.c_double, cd,
                                  C.POINTER(or_switches)]
        L.or_linearstep.argtypes = [cd, C.c_int, C.c_int, C.c_int, cd, cd, cd]
        L.or_sst.argtypes = [cd, C.c_int, C.c_int, C.c_int, cd, C.c_double, C.c_double, cd]
        L.or_ionizpot.argtypes = [C.c_char_p, cd, cd]
        L.or_Natoms.argtypes = [C.c_char_p, cd, cd]
        L.or_ADK.argtypes = [cd, cd, C.c_long, cd, cd, cd, cd, cd, cd]
        L.or_ioniz.argtypes = [cd, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_char_p, C.c_double, cd,
                               C.c_double, C.c_double, cd, cd, C.POINTER(or_switches)]
        L.or_calc1oes.argtypes = [cd, C.c_int, cd, cd, cd]
        L.or_beam_profiles.argtypes = [cd, C.c_int, C.c_int, C.c_int, cd, cd]
        L.or_ssfmprop.argtypes = [cd, C.POINTER(or_params), C.c_double, _ip, C.c_double, cd, cd, cd, cd, cd, cd, cd,
                                  C.c_int, C.POINTER(or_switches)]
        L.or_setStep.argtypes = [C.c_long, cd, cd, cd, C.c_double, C.c_double, cd, cd, _ip, cd]
        L.or_diag.argtypes = [cd, C.c_int, C.c_int, C.c_int, cd, cd]
        L.or_calibrate.argtypes = [cd, C.c_long, C.c_double, C.c_double, C.POINTER(or_switches)]
        L.or_mirror_lens.argtypes = [cd, C.c_int, C.c_int, C.c_int, cd, C.c_double, C.c_double]
        L.or_run_fixed.argtypes = [cd, C.POINTER(or_params), C.POINTER(or_state), C.c_int, C.POINTER(or_switches)]
        L.or_double_step.argtypes = [cd, cd, cd, C.POINTER(or_params), C.POINTER(or_state), C.POINTER(or_switches)]
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(_dp)


def switches(**kw) -> or_switches:
    s = or_switches()
    lib().or_default_switches(C.byref(s))
    for k, v in kw.items():
        setattr(s, k, int(v))
    return s


def set_threads(n: int) -> None:
    lib().or_set_threads(int(n))


class Oracle:
    """Holds the parameter record (any object with the param.bin fields) for the C calls."""

    def __init__(self, p, **sw):
        self.p = p
        self._keep = [np.ascontiguousarray(x, dtype=np.float64) for x in (p.betas, p.wr, p.w, p.r)]
        op = or_params()
        op.Nx, op.Ny, op.Nt = (int(d) for d in p.dims)
        op.dist, op.dzz = p.dist, p.dzz
        op.betas, op.wr, op.w, op.r = (_p(x) for x in self._keep)
        op.alpha, op.Cav, op.k0 = p.alpha, p.Cav, p.k0
        op.sst_on, op.gamma2, op.w0, op.plasm = p.sst_on, p.gamma2, p.w0, p.plasm
        op.deltat, op.rho_c, op.rho_nt, op.n0 = p.deltat, p.rho_c, p.rho_nt, p.n0
        op.puls_e, op.Ab_M, op.dr, op.def_err, op.dzmin, op.Esig = p.puls_e, p.Ab_M, p.dr, p.def_err, p.dzmin, p.Esig
        op.gas = p.gas.encode("ascii")
        op.roc = getattr(p, "roc", 0.0)
        self.op = op
        if "bounce_lens" not in sw:
            sw["bounce_lens"] = int(getattr(p, "bounce_mode", 0) == 1)
        self.sw = switches(**sw)
        self.L = lib()

    def new_state(self) -> or_state:
        st = or_state()
        st.z = 0.0
        st.dzz = self.p.dzz
        st.puls_e = self.p.puls_e
        st.signmem = 1
        return st

    def calibrate(self, A: np.ndarray) -> None:
        self.L.or_calibrate(_p(A.view(np.float64)), A.size, self.p.puls_e, self.p.Esig, C.byref(self.sw))

    def ssfmprop(self, A: np.ndarray, dzz: float, signmem: int, z: float, puls_e: float, change: int = 0):
        sm = C.c_int(signmem)
        pe = C.c_double(puls_e)
        BP1 = np.zeros(self.p.dims[0])
        BP2 = np.zeros(self.p.dims[1])
        y1 = np.zeros(4)
        y2 = np.zeros(4)
        b1 = C.c_double(0)
        b2 = C.c_double(0)
        self.L.or_ssfmprop(_p(A.view(np.float64)), C.byref(self.op), dzz, C.byref(sm), z, C.byref(pe), _p(BP1), _p(BP2),
                           _p(y1), _p(y2), C.byref(b1), C.byref(b2), change, C.byref(self.sw))
        return dict(signmem=sm.value, puls_e=pe.value, BP1=BP1, BP2=BP2, y1=y1, y2=y2, bps1=b1.value, bps2=b2.value)

    def run_fixed(self, A: np.ndarray, st: or_state, nsteps: int) -> None:
        self.L.or_run_fixed(_p(A.view(np.float64)), C.byref(self.op), C.byref(st), nsteps, C.byref(self.sw))

    def double_step(self, A: np.ndarray, C1: np.ndarray, C2: np.ndarray, st: or_state) -> None:
        self.L.or_double_step(_p(A.view(np.float64)), _p(C1.view(np.float64)), _p(C2.view(np.float64)), C.byref(self.op),
                              C.byref(st), C.byref(self.sw))

    def ioniz(self, A: np.ndarray):
        n = A.size
        tau = np.zeros(n)
        fe = np.zeros(n)
        Nx, Ny, Nt = (int(d) for d in self.p.dims)
        self.L.or_ioniz(_p(A.view(np.float64)), Nx, Ny, Nt, self.p.w0, self.p.deltat, self.p.gas.encode(), self.p.rho_c,
                        _p(self._keep[2]), self.p.rho_nt, self.p.n0, _p(tau), _p(fe), C.byref(self.sw))
        return tau, fe

    def sst(self, A: np.ndarray) -> np.ndarray:
        out = np.zeros_like(A)
        Nx, Ny, Nt = (int(d) for d in self.p.dims)
        self.L.or_sst(_p(A.view(np.float64)), Nx, Ny, Nt, _p(self._keep[2]), self.p.gamma2, self.p.w0,
                      _p(out.view(np.float64)))
        return out

    def diag(self, A: np.ndarray):
        Nx, Ny, Nt = (int(d) for d in self.p.dims)
        temp = np.zeros(Nt)
        spec = np.zeros(Nt)
        self.L.or_diag(_p(A.view(np.float64)), Nx, Ny, Nt, _p(temp), _p(spec))
        BP1 = np.zeros(Nx)
        BP2 = np.zeros(Ny)
        self.L.or_beam_profiles(_p(A.view(np.float64)), Nx, Ny, Nt, _p(BP1), _p(BP2))
        return temp, spec, BP1, BP2

    def energy(self, A: np.ndarray) -> float:
        HBAR = 1.054560652926899e-34
        return float(np.sum(np.abs(A) ** 2) * self.p.dr ** 2 * self.p.deltat * HBAR * self.p.w0)

    def calcexpR(self, n: int, signmem: int, z: float, dzh: float):
        out = np.zeros(n, dtype=np.complex128)
        sm = C.c_int(signmem)
        self.L.or_calcexpR(_p(out.view(np.float64)), n, int(self.p.dims[1]), C.byref(sm), z, self.p.Cav, self.p.k0, dzh,
                           _p(self._keep[1]), C.byref(self.sw))
        return out, sm.value

    def expD0(self, dzz: float) -> np.ndarray:
        Nt = int(self.p.dims[2])
        out = np.zeros(Nt, dtype=np.complex128)
        self.L.or_expD0(_p(out.view(np.float64)), Nt, dzz, self.p.alpha, _p(self._keep[0]))
        return out


def fft_axis(A: np.ndarray, dims, axis: int, sign: int) -> None:
    lib().or_fft_axis(_p(A.view(np.float64)), int(dims[0]), int(dims[1]), int(dims[2]), axis, sign)


def ADK(E: np.ndarray, C_nl, f_lm, nq, mq, Ei):
    E = np.ascontiguousarray(E, dtype=np.float64)
    r1 = np.zeros_like(E)
    r2 = np.zeros_like(E)
    arrs = [np.ascontiguousarray(x, dtype=np.float64) for x in (C_nl, f_lm, nq, mq, Ei)]
    lib().or_ADK(_p(r1), _p(r2), E.size, *(_p(a) for a in arrs), _p(E))
    return r1, r2


def ionizpot(gas: str):
    a = C.c_double(0)
    b = C.c_double(0)
    lib().or_ionizpot(gas.encode(), C.byref(a), C.byref(b))
    return a.value, b.value


def Natoms(gas: str):
    a = C.c_double(0)
    b = C.c_double(0)
    lib().or_Natoms(gas.encode(), C.byref(a), C.byref(b))
    return a.value, b.value


def calc1oes(BP: np.ndarray, r: np.ndarray):
    BP = np.ascontiguousarray(BP, dtype=np.float64)
    r = np.ascontiguousarray(r, dtype=np.float64)
    v = C.c_double(0)
    y = np.zeros(4)
    lib().or_calc1oes(_p(BP), BP.size, _p(r), C.byref(v), _p(y))
    return v.value, y


def setStep(dzz: float, C1: np.ndarray, C2: np.ndarray, def_err: float, dzmin: float, y1, y2):
    d = C.c_double(dzz)
    bad = C.c_int(0)
    err = C.c_double(0)
    y1 = np.ascontiguousarray(y1, dtype=np.float64)
    y2 = np.ascontiguousarray(y2, dtype=np.float64)
    lib().or_setStep(C1.size, C.byref(d), _p(C1.view(np.float64)), _p(C2.view(np.float64)), def_err, dzmin, _p(y1), _p(y2),
                     C.byref(bad), C.byref(err))
    return d.value, bad.value, err.value


# ---- FP64 GPU oracle -------------------------------------------------------------------
_lib64 = None


def lib64() -> C.CDLL:
    global _lib64
    if _lib64 is None:
        _lib64 = C.CDLL(build64())
        L = _lib64
        cd = C.POINTER(C.c_double)
        L.or64_last_error.restype = C.c_char_p
        L.or64_create.argtypes = [C.POINTER(C.c_void_p), C.POINTER(or_params), C.POINTER(or_switches)]
        L.or64_destroy.argtypes = [C.c_void_p]
        L.or64_upload.argtypes = [C.c_void_p, cd]
        L.or64_download.argtypes = [C.c_void_p, cd]
        L.or64_ssfmprop.argtypes = [C.c_void_p, C.c_double, _ip, C.c_double, cd, cd, cd, cd, cd, cd, cd, C.c_int]
        L.or64_run_fixed.argtypes = [C.c_void_p, C.POINTER(or_state), C.c_int]
        L.or64_double_step.argtypes = [C.c_void_p, C.POINTER(or_state), C.c_double, C.c_int, _ip, cd]
        L.or64_energy.argtypes = [C.c_void_p, cd]
    return _lib64


class Oracle64(Oracle):
    """The FP64 GPU oracle on the current CUDA device, holding the field (complex128) there.
    Same parameter record and switches as Oracle; the field stays on the device between calls."""

    def __init__(self, p, **sw):
        super().__init__(p, **sw)
        self.L64 = lib64()
        self.ctx = C.c_void_p()
        if self.L64.or64_create(C.byref(self.ctx), C.byref(self.op), C.byref(self.sw)) != 0:
            raise RuntimeError(f"or64_create: {self.L64.or64_last_error().decode()}")

    def _ck(self, rc: int, what: str) -> None:
        if rc != 0:
            raise RuntimeError(f"{what}: {self.L64.or64_last_error().decode()}")

    def close(self) -> None:
        if self.ctx:
            self.L64.or64_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, A: np.ndarray) -> None:
        A = np.ascontiguousarray(A, dtype=np.complex128)
        self._ck(self.L64.or64_upload(self.ctx, _p(A.view(np.float64))), "upload")

    def download(self) -> np.ndarray:
        out = np.empty(int(np.prod(self.p.dims)), dtype=np.complex128)
        self._ck(self.L64.or64_download(self.ctx, _p(out.view(np.float64))), "download")
        return out

    def ssfmprop_dev(self, dzz: float, signmem: int, z: float, puls_e: float, change: int = 0):
        sm = C.c_int(signmem)
        pe = C.c_double(puls_e)
        BP1 = np.zeros(self.p.dims[0])
        BP2 = np.zeros(self.p.dims[1])
        y1 = np.zeros(4)
        y2 = np.zeros(4)
        b1 = C.c_double(0)
        b2 = C.c_double(0)
        self._ck(self.L64.or64_ssfmprop(self.ctx, dzz, C.byref(sm), z, C.byref(pe), _p(BP1), _p(BP2), _p(y1), _p(y2),
                                        C.byref(b1), C.byref(b2), change), "ssfmprop")
        return dict(signmem=sm.value, puls_e=pe.value, BP1=BP1, BP2=BP2, y1=y1, y2=y2, bps1=b1.value, bps2=b2.value)

    def run_fixed_dev(self, st: or_state, nsteps: int) -> None:
        self._ck(self.L64.or64_run_fixed(self.ctx, C.byref(st), nsteps), "run_fixed")

    def double_step_dev(self, st: or_state, dz_used: float = 0.0, force: int = -1):
        """One attempt on the resident field; returns (own_bad, own_err) of this oracle's rule."""
        ob = C.c_int(0)
        oe = C.c_double(0)
        self._ck(self.L64.or64_double_step(self.ctx, C.byref(st), dz_used, force, C.byref(ob), C.byref(oe)),
                 "double_step")
        return ob.value, oe.value

    def energy_dev(self) -> float:
        e = C.c_double(0)
        self._ck(self.L64.or64_energy(self.ctx, C.byref(e)), "energy")
        return e.value
