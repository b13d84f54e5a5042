"""mpc_gb300: a GB300 (sm_103a) split-step Fourier propagator for nonlinear pulse
propagation in gas-filled multipass cells, a drop-in for the hot path of kmecseki/MPC.

The compute runs in libmpc_gpu.so (hand-written CUDA behind the C ABI of
include/mpc_gpu.h); this package holds its ctypes binding, the param.bin record and a
seeded input generator.
"""
from .params import BOUNCE_LENS, BOUNCE_SIGNFLIP, MPCParams, read_field, write_field  # noqa: F401

__all__ = ["MPCParams", "BOUNCE_LENS", "BOUNCE_SIGNFLIP", "read_field", "write_field", "Propagator", "load"]


def __getattr__(name):
    if name in ("Propagator", "load", "MPCError", "calc1oes"):
        from . import capi
        return getattr(capi, name)
    raise AttributeError(name)
