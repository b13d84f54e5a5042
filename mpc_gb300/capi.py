"""ctypes binding of libmpc_gpu.so (include/mpc_gpu.h) and a Python mirror of the
reference's propagation.h / plasma.h entry points on top of it.

The library must have been built (mpc_gb300.build.build()); loading fails loudly if it is
absent -- there is no CPU fallback for any propagator call.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .params import MPCParams

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("MPC_GPU_LIB", os.path.join(_HERE, "libmpc_gpu.so"))

MPC_OK = 0
ERRORS = {1: "MPC_ERR_ARG", 2: "MPC_ERR_SHAPE", 3: "MPC_ERR_CUDA", 4: "MPC_ERR_NOMEM", 5: "MPC_ERR_NONFINITE",
          6: "MPC_ERR_STATE", 7: "MPC_ERR_IO", 8: "MPC_ERR_UNSUPPORTED", 9: "MPC_ERR_TIMEOUT"}

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_fp = C.POINTER(C.c_float)


class c_mpc_params(C.Structure):
    _fields_ = [("dims", C.c_int * 3), ("dist", C.c_double), ("dzz", C.c_double), ("betas", _dp),
                ("alpha", C.c_double), ("Cav", C.c_double), ("k0", C.c_double), ("wr", _dp),
                ("sst_on", C.c_int), ("w", _dp), ("gamma2", C.c_double), ("w0", C.c_double),
                ("plasm", C.c_int), ("deltat", C.c_double), ("rho_c", C.c_double), ("rho_nt", C.c_double),
                ("n0", C.c_double), ("puls_e", C.c_double), ("Ab_M", C.c_double), ("r", _dp),
                ("dr", C.c_double), ("def_err", C.c_double), ("dzmin", C.c_double), ("Esig", C.c_double),
                ("gas", C.c_char * 9), ("bounce_mode", C.c_int), ("roc", C.c_double),
                ("variant", C.c_int), ("land_mirrors", C.c_int)]


class c_mpc_state(C.Structure):
    _fields_ = [("z", C.c_double), ("dzz", C.c_double), ("err", C.c_double), ("puls_e", C.c_double),
                ("bps1", C.c_double), ("bps2", C.c_double), ("signmem", C.c_int), ("bad", C.c_int),
                ("nstep", C.c_int), ("attempts", C.c_int), ("y1", C.c_double * 4), ("y2", C.c_double * 4)]


# name -> (restype, argtypes); every entry point of include/mpc_gpu.h
SIGNATURES = {
    "mpc_version": (C.c_char_p, []),
    "mpc_last_error": (C.c_char_p, []),
    "mpc_shape_supported": (C.c_int, [C.c_int, C.c_int, C.c_int]),
    "mpc_create": (C.c_int, [C.POINTER(C.c_void_p), C.POINTER(c_mpc_params)]),
    "mpc_destroy": (C.c_int, [C.c_void_p]),
    "mpc_ssfmprop": (C.c_int, [C.c_void_p, _dp, C.c_int, C.c_double, _ip, C.c_double, _dp, _dp, _dp, _dp, _dp,
                               _dp, _dp, C.c_int]),
    "mpc_linearstep": (C.c_int, [C.c_void_p, _dp, _dp, _dp]),
    "mpc_calcexpR": (C.c_int, [C.c_void_p, _dp, _ip, C.c_double, C.c_double]),
    "mpc_ioniz": (C.c_int, [C.c_void_p, _dp, _dp, _dp]),
    "mpc_ADK": (C.c_int, [C.c_void_p, C.c_long, _dp, _dp, _dp]),
    "mpc_calc1oes": (C.c_int, [_dp, C.c_int, _dp, _dp, _dp]),
    "mpc_setStep": (C.c_int, [C.c_void_p, _dp, _dp, _dp, _dp, _dp, _ip, _dp]),
    "mpc_field_upload": (C.c_int, [C.c_void_p, _dp, C.c_int]),
    "mpc_field_download": (C.c_int, [C.c_void_p, _dp]),
    "mpc_get_state": (C.c_int, [C.c_void_p, C.POINTER(c_mpc_state)]),
    "mpc_set_state": (C.c_int, [C.c_void_p, C.POINTER(c_mpc_state)]),
    "mpc_run_fixed": (C.c_int, [C.c_void_p, C.c_int]),
    "mpc_step_double": (C.c_int, [C.c_void_p, _dp, _dp, _ip, _dp]),
    "mpc_mirror_bounce": (C.c_int, [C.c_void_p, C.c_int]),
    "mpc_diag": (C.c_int, [C.c_void_p, _dp, _dp, _dp, _dp]),
    "mpc_energy": (C.c_int, [C.c_void_p, _dp]),
    "mpc_sync": (C.c_int, [C.c_void_p]),
    "mpc_host_alloc": (C.c_int, [C.POINTER(C.c_void_p), C.c_size_t]),
    "mpc_host_free": (C.c_int, [C.c_void_p]),
    "mpc_stream_handle": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "mpc_launch_count": (C.c_long, [C.c_void_p]),
    "mpc_variant_info": (C.c_int, [C.c_void_p, _ip, _ip]),
    "mpc_profile": (C.c_int, [C.c_void_p, C.c_int]),
    "mpc_kernel_times": (C.c_int, [C.c_void_p, _dp, C.POINTER(C.c_long), _dp, C.POINTER(C.c_long)]),
    "mpc_wait_limit_check": (C.c_int, [C.c_void_p]),
    "mpc_nonlinear_noalloc": (C.c_int, [C.POINTER(c_mpc_params), C.c_void_p, C.c_double, C.c_void_p]),
    "mpc_batch_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.POINTER(C.c_void_p)]),
    "mpc_batch_destroy": (C.c_int, [C.c_void_p]),
    "mpc_batch_run_fixed": (C.c_int, [C.c_void_p, C.c_int]),
    "mpc_batch_step_double": (C.c_int, [C.c_void_p, _ip, _dp]),
    "mpc_batch_stats": (C.c_int, [C.c_void_p, C.POINTER(C.c_long), C.POINTER(C.c_long)]),
    "mpc_step": (C.c_int, [C.c_void_p, C.c_double]),
    "mpc_step_stats": (C.c_int, [C.c_void_p, _fp, C.c_int]),
    "mpc_features": (C.c_int, [C.c_void_p, _fp]),
    "mpc_mlp_num_weights": (C.c_int, []),
    "mpc_mlp_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_ulonglong]),
    "mpc_mlp_destroy": (C.c_int, [C.c_void_p]),
    "mpc_mlp_set_normalization": (C.c_int, [C.c_void_p, _fp, _fp, C.c_float, C.c_float]),
    "mpc_mlp_get_normalization": (C.c_int, [C.c_void_p, _fp]),
    "mpc_mlp_get_weights": (C.c_int, [C.c_void_p, _fp]),
    "mpc_mlp_set_weights": (C.c_int, [C.c_void_p, _fp]),
    "mpc_mlp_loss_grad": (C.c_int, [C.c_void_p, _fp, _fp, C.c_int, _fp, _fp]),
    "mpc_mlp_train": (C.c_int, [C.c_void_p, _fp, _fp, C.c_int, C.c_int, C.c_int, C.c_float, C.c_ulonglong, _fp]),
    "mpc_mlp_predict": (C.c_int, [C.c_void_p, _fp, C.c_int, _fp]),
    "mpc_mlp_predict1": (C.c_int, [C.c_void_p, _fp, _fp]),
    "mpc_run_learned": (C.c_int, [C.c_void_p, C.c_void_p, C.c_double, C.c_int, C.c_int, C.c_void_p]),
    "mpc_run_learned_hold": (C.c_int, [C.c_void_p, C.c_void_p, C.c_double, C.c_int, C.c_int, C.c_int, C.c_void_p]),
}

_fp = C.POINTER(C.c_float)
NFEATURES = 16


class c_mpc_learned_stats(C.Structure):
    _fields_ = [("steps", C.c_int), ("checks", C.c_int), ("check_failures", C.c_int),
                ("fallback_attempts", C.c_int), ("executed_steps", C.c_long), ("dz_min", C.c_double),
                ("dz_max", C.c_double)]

_lib = None


def load(path: str = LIB_PATH) -> C.CDLL:
    """Load libmpc_gpu.so and declare every entry point; raises if the library is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with mpc_gb300.build.build() (needs nvcc)")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


class MPCError(RuntimeError):
    pass


def _check(rc: int, what: str) -> None:
    if rc != MPC_OK:
        msg = _lib.mpc_last_error().decode() if _lib else ""
        raise MPCError(f"{what}: {ERRORS.get(rc, rc)}: {msg}")


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_dp)


def _c128(a: np.ndarray) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.complex128)
    return a


class Propagator:
    """One device context: a grid, its tables and the device-resident field."""

    def __init__(self, p: MPCParams):
        self.lib = load()
        self.p = p
        self._keep = [np.ascontiguousarray(x, dtype=np.float64) for x in (p.betas, p.wr, p.w, p.r)]
        cp = c_mpc_params()
        cp.dims[:] = list(p.dims)
        cp.dist, cp.dzz = p.dist, p.dzz
        cp.betas, cp.wr, cp.w, cp.r = (_ptr(x) for x in self._keep)
        cp.alpha, cp.Cav, cp.k0 = p.alpha, p.Cav, p.k0
        cp.sst_on, cp.gamma2, cp.w0, cp.plasm = p.sst_on, p.gamma2, p.w0, p.plasm
        cp.deltat, cp.rho_c, cp.rho_nt, cp.n0 = p.deltat, p.rho_c, p.rho_nt, p.n0
        cp.puls_e, cp.Ab_M, cp.dr, cp.def_err, cp.dzmin, cp.Esig = p.puls_e, p.Ab_M, p.dr, p.def_err, p.dzmin, p.Esig
        cp.gas = p.gas.encode("ascii")[:8]
        cp.bounce_mode, cp.roc = p.bounce_mode, p.roc
        cp.variant = p.variant
        cp.land_mirrors = p.land_mirrors
        self._cp = cp
        h = C.c_void_p()
        _check(self.lib.mpc_create(C.byref(h), C.byref(cp)), "mpc_create")
        self.h = h

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.mpc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- reference entry points ----------------------------------------------------
    def ssfmprop(self, A: np.ndarray, dzz: float, signmem: int, z: float, puls_e: float, change: int = 0,
                 sst_on: int | None = None):
        """propagation.c:111 on a host complex128 field (modified in place).
        Returns dict(signmem, puls_e, BP1, BP2, y1, y2, bps1, bps2)."""
        assert A.dtype == np.complex128 and A.flags.c_contiguous and A.size == self.p.N
        sm = C.c_int(signmem)
        pe = C.c_double(puls_e)
        BP1 = np.zeros(self.p.Nx)
        BP2 = np.zeros(self.p.Ny)
        y1 = np.zeros(4)
        y2 = np.zeros(4)
        b1 = C.c_double(0)
        b2 = C.c_double(0)
        rc = self.lib.mpc_ssfmprop(self.h, A.ctypes.data_as(_dp), self.p.sst_on if sst_on is None else sst_on, dzz,
                                   C.byref(sm), z, C.byref(pe), _ptr(BP1), _ptr(BP2), _ptr(y1), _ptr(y2),
                                   C.byref(b1), C.byref(b2), change)
        _check(rc, "mpc_ssfmprop")
        return dict(signmem=sm.value, puls_e=pe.value, BP1=BP1, BP2=BP2, y1=y1, y2=y2, bps1=b1.value, bps2=b2.value)

    def linearstep(self, A: np.ndarray, exp_D0: np.ndarray, expR: np.ndarray) -> None:
        e0 = _c128(exp_D0)
        er = _c128(expR)
        _check(self.lib.mpc_linearstep(self.h, A.ctypes.data_as(_dp), e0.ctypes.data_as(_dp), er.ctypes.data_as(_dp)),
               "mpc_linearstep")

    def calcexpR(self, signmem: int, z: float, dzz: float):
        out = np.zeros(self.p.Nx, dtype=np.complex128)
        sm = C.c_int(signmem)
        _check(self.lib.mpc_calcexpR(self.h, out.ctypes.data_as(_dp), C.byref(sm), z, dzz), "mpc_calcexpR")
        return out, sm.value

    def ioniz(self, A: np.ndarray):
        A = _c128(A)
        tau = np.zeros(self.p.N)
        fe = np.zeros(self.p.N)
        _check(self.lib.mpc_ioniz(self.h, A.ctypes.data_as(_dp), _ptr(tau), _ptr(fe)), "mpc_ioniz")
        return tau, fe

    def ADK(self, E: np.ndarray):
        E = np.ascontiguousarray(E, dtype=np.float64)
        r1 = np.zeros_like(E)
        r2 = np.zeros_like(E)
        _check(self.lib.mpc_ADK(self.h, E.size, _ptr(E), _ptr(r1), _ptr(r2)), "mpc_ADK")
        return r1, r2

    def setStep(self, dzz: float, C1: np.ndarray, C2: np.ndarray, y1, y2):
        d = C.c_double(dzz)
        bad = C.c_int(0)
        err = C.c_double(0)
        y1 = np.ascontiguousarray(y1, dtype=np.float64)
        y2 = np.ascontiguousarray(y2, dtype=np.float64)
        _check(self.lib.mpc_setStep(self.h, C.byref(d), _c128(C1).ctypes.data_as(_dp), _c128(C2).ctypes.data_as(_dp),
                                    _ptr(y1), _ptr(y2), C.byref(bad), C.byref(err)), "mpc_setStep")
        return d.value, bad.value, err.value

    # ---- device-resident field ------------------------------------------------------
    def upload(self, A: np.ndarray, calibrate: bool = False) -> None:
        A = _c128(A)
        _check(self.lib.mpc_field_upload(self.h, A.ctypes.data_as(_dp), int(calibrate)), "mpc_field_upload")

    def download(self, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty(self.p.N, dtype=np.complex128)
        _check(self.lib.mpc_field_download(self.h, out.ctypes.data_as(_dp)), "mpc_field_download")
        return out

    def state(self) -> c_mpc_state:
        st = c_mpc_state()
        _check(self.lib.mpc_get_state(self.h, C.byref(st)), "mpc_get_state")
        return st

    def set_state(self, st: c_mpc_state) -> None:
        _check(self.lib.mpc_set_state(self.h, C.byref(st)), "mpc_set_state")

    def run_fixed(self, nsteps: int) -> None:
        _check(self.lib.mpc_run_fixed(self.h, nsteps), "mpc_run_fixed")

    def step_double(self, profiles: bool = False):
        """One adaptive step-doubling attempt on the device field (MPC.c:269-383).
        Returns dict(bad, err[, BP1, BP2])."""
        bad = C.c_int(0)
        err = C.c_double(0)
        BP1 = np.zeros(self.p.Nx) if profiles else None
        BP2 = np.zeros(self.p.Ny) if profiles else None
        _check(self.lib.mpc_step_double(self.h, _ptr(BP1) if profiles else None, _ptr(BP2) if profiles else None,
                                        C.byref(bad), C.byref(err)), "mpc_step_double")
        out = dict(bad=bad.value, err=err.value)
        if profiles:
            out.update(BP1=BP1, BP2=BP2)
        return out

    def step(self, dzz: float) -> None:
        """One split step of length dzz on the device field at state.z (mirror bounces crossed applied)."""
        _check(self.lib.mpc_step(self.h, float(dzz)), "mpc_step")

    def step_stats(self, reset: bool = False) -> np.ndarray:
        out = np.zeros(4, dtype=np.float32)
        _check(self.lib.mpc_step_stats(self.h, out.ctypes.data_as(_fp), int(reset)), "mpc_step_stats")
        return out

    def features(self) -> np.ndarray:
        f = np.zeros(NFEATURES, dtype=np.float32)
        _check(self.lib.mpc_features(self.h, f.ctypes.data_as(_fp)), "mpc_features")
        return f

    def run_learned(self, mlp: "MLP", safety: float = 0.9, check_every: int = 8, fallback_len: int = 4,
                    hold: int = 1) -> dict:
        st = c_mpc_learned_stats()
        _check(self.lib.mpc_run_learned_hold(self.h, mlp.h, float(safety), int(check_every), int(fallback_len),
                                             int(hold), C.byref(st)), "mpc_run_learned_hold")
        return {k: getattr(st, k) for k, _ in st._fields_}

    def mirror_bounce(self, mode: int) -> None:
        _check(self.lib.mpc_mirror_bounce(self.h, int(mode)), "mpc_mirror_bounce")

    def diag(self):
        temp = np.zeros(self.p.Nt)
        spec = np.zeros(self.p.Nt)
        BP1 = np.zeros(self.p.Nx)
        BP2 = np.zeros(self.p.Ny)
        _check(self.lib.mpc_diag(self.h, _ptr(temp), _ptr(spec), _ptr(BP1), _ptr(BP2)), "mpc_diag")
        return temp, spec, BP1, BP2

    def energy(self) -> float:
        e = C.c_double(0)
        _check(self.lib.mpc_energy(self.h, C.byref(e)), "mpc_energy")
        return e.value

    def sync(self) -> None:
        _check(self.lib.mpc_sync(self.h), "mpc_sync")

    def variant_info(self) -> dict:
        """The kernel variant this context runs and its launch shapes."""
        v = C.c_int(0)
        info = (C.c_int * 10)()
        _check(self.lib.mpc_variant_info(self.h, C.byref(v), info), "mpc_variant_info")
        keys = ("P", "SLO", "CL", "PB", "PT", "pencil_ctas", "plane_clusters", "pencil_threads", "LD", "PL")
        return dict(variant=v.value, **dict(zip(keys, list(info))))

    def launch_count(self) -> int:
        return int(self.lib.mpc_launch_count(self.h))

    def stream_handle(self) -> int:
        h = C.c_void_p()
        _check(self.lib.mpc_stream_handle(self.h, C.byref(h)), "mpc_stream_handle")
        return int(h.value or 0)

    def profile(self, on: bool) -> None:
        _check(self.lib.mpc_profile(self.h, int(on)), "mpc_profile")

    def kernel_times(self):
        pm, pl = C.c_double(0), C.c_double(0)
        npn, npl = C.c_long(0), C.c_long(0)
        _check(self.lib.mpc_kernel_times(self.h, C.byref(pm), C.byref(npn), C.byref(pl), C.byref(npl)),
               "mpc_kernel_times")
        return dict(pencil_ms=pm.value, n_pencil=npn.value, plane_ms=pl.value, n_plane=npl.value)


def _f32(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float32)
    if shape is not None and a.shape != shape:
        raise ValueError(f"expected shape {shape}, got {a.shape}")
    return a


class MLP:
    """The learned controller's network (16 -> 64 -> 64 -> 1, SiLU) on the GPU."""

    def __init__(self, seed: int = 0):
        self.lib = load()
        h = C.c_void_p()
        _check(self.lib.mpc_mlp_create(C.byref(h), C.c_ulonglong(seed)), "mpc_mlp_create")
        self.h = h
        self.nw = int(self.lib.mpc_mlp_num_weights())

    def set_normalization(self, mean, std, y_mean: float, y_std: float) -> None:
        m, s = _f32(mean, (NFEATURES,)), _f32(std, (NFEATURES,))
        _check(self.lib.mpc_mlp_set_normalization(self.h, m.ctypes.data_as(_fp), s.ctypes.data_as(_fp),
                                                  float(y_mean), float(y_std)), "mpc_mlp_set_normalization")

    def normalization(self) -> np.ndarray:
        out = np.zeros(2 * NFEATURES + 2, dtype=np.float32)
        _check(self.lib.mpc_mlp_get_normalization(self.h, out.ctypes.data_as(_fp)), "mpc_mlp_get_normalization")
        return out

    @property
    def weights(self) -> np.ndarray:
        w = np.zeros(self.nw, dtype=np.float32)
        _check(self.lib.mpc_mlp_get_weights(self.h, w.ctypes.data_as(_fp)), "mpc_mlp_get_weights")
        return w

    @weights.setter
    def weights(self, w) -> None:
        w = _f32(w, (self.nw,))
        _check(self.lib.mpc_mlp_set_weights(self.h, w.ctypes.data_as(_fp)), "mpc_mlp_set_weights")

    def loss_grad(self, X, y):
        X, y = _f32(X), _f32(y)
        g = np.zeros(self.nw, dtype=np.float32)
        loss = np.zeros(1, dtype=np.float32)
        _check(self.lib.mpc_mlp_loss_grad(self.h, X.ctypes.data_as(_fp), y.ctypes.data_as(_fp), len(y),
                                          g.ctypes.data_as(_fp), loss.ctypes.data_as(_fp)), "mpc_mlp_loss_grad")
        return float(loss[0]), g

    def train(self, X, y, epochs: int = 20, batch: int = 256, lr: float = 1e-3, seed: int = 0) -> float:
        X, y = _f32(X), _f32(y)
        loss = np.zeros(1, dtype=np.float32)
        _check(self.lib.mpc_mlp_train(self.h, X.ctypes.data_as(_fp), y.ctypes.data_as(_fp), len(y), int(epochs),
                                      int(batch), float(lr), C.c_ulonglong(seed), loss.ctypes.data_as(_fp)),
               "mpc_mlp_train")
        return float(loss[0])

    def predict(self, X) -> np.ndarray:
        X = _f32(X)
        y = np.zeros(len(X), dtype=np.float32)
        _check(self.lib.mpc_mlp_predict(self.h, X.ctypes.data_as(_fp), len(X), y.ctypes.data_as(_fp)),
               "mpc_mlp_predict")
        return y

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.mpc_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Many cells (Propagators, any grid shapes) run call by call as one CUDA graph each."""

    def __init__(self, cells: list[Propagator]):
        self.lib = load()
        self.cells = list(cells)
        arr = (C.c_void_p * len(self.cells))(*[c.h.value for c in self.cells])
        h = C.c_void_p()
        _check(self.lib.mpc_batch_create(C.byref(h), len(self.cells), arr), "mpc_batch_create")
        self.h = h

    def run_fixed(self, nsteps: int) -> None:
        _check(self.lib.mpc_batch_run_fixed(self.h, int(nsteps)), "mpc_batch_run_fixed")

    def step_double(self):
        """One adaptive attempt of every unfinished cell: (bad[n], err[n]); bad = -1 when finished."""
        n = len(self.cells)
        bad = np.zeros(n, dtype=np.int32)
        err = np.zeros(n)
        _check(self.lib.mpc_batch_step_double(self.h, bad.ctypes.data_as(_ip), _ptr(err)), "mpc_batch_step_double")
        return bad, err

    def stats(self):
        g, nn = C.c_long(0), C.c_long(0)
        _check(self.lib.mpc_batch_stats(self.h, C.byref(g), C.byref(nn)), "mpc_batch_stats")
        return dict(graphs=g.value, nodes=nn.value)

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.mpc_batch_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PinnedArray:
    """A page-locked host complex128 buffer (cudaMallocHost) viewed as a numpy array."""

    def __init__(self, n: int):
        self.lib = load()
        self.ptr = C.c_void_p()
        _check(self.lib.mpc_host_alloc(C.byref(self.ptr), 16 * n), "mpc_host_alloc")
        buf = (C.c_double * (2 * n)).from_address(self.ptr.value)
        self.array = np.frombuffer(buf, dtype=np.complex128, count=n)

    def free(self) -> None:
        if self.ptr:
            self.array = None
            self.lib.mpc_host_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def calc1oes(BP: np.ndarray, r: np.ndarray):
    lib = load()
    BP = np.ascontiguousarray(BP, dtype=np.float64)
    r = np.ascontiguousarray(r, dtype=np.float64)
    v = C.c_double(0)
    y = np.zeros(4)
    _check(lib.mpc_calc1oes(_ptr(BP), BP.size, _ptr(r), C.byref(v), _ptr(y)), "mpc_calc1oes")
    return v.value, y


def nonlinear_noalloc(p: MPCParams, A_dev_ptr: int, dz: float, stream: int = 0) -> int:
    """Apply the nonlinear step in place to a complex64 field already in device memory
    (address A_dev_ptr, real space, reference layout, physical units) without allocating
    device memory: for callers that cannot call cudaMalloc.  The work is queued on `stream`
    (a cudaStream_t as an integer); returns the MPC status code."""
    lib = load()
    keep = [np.ascontiguousarray(x, dtype=np.float64) for x in (p.betas, p.wr, p.w, p.r)]
    cp = c_mpc_params()
    cp.dims[:] = list(p.dims)
    cp.betas, cp.wr, cp.w, cp.r = (_ptr(x) for x in keep)
    cp.sst_on, cp.gamma2, cp.w0, cp.plasm = p.sst_on, p.gamma2, p.w0, p.plasm
    cp.deltat, cp.rho_c, cp.rho_nt, cp.n0 = p.deltat, p.rho_c, p.rho_nt, p.n0
    cp.gas = p.gas.encode("ascii")[:8]
    return int(lib.mpc_nonlinear_noalloc(C.byref(cp), C.c_void_p(A_dev_ptr), dz, C.c_void_p(stream)))
