"""The linear step with cuFFT and a separate multiply, timed beside this library's sweeps.

A cuFFT implementation of the reference's linear step (propagation.c:3-108) on the device is
three library calls: a 3-D complex-to-complex FFT over (t, y, x), one pointwise multiply by
D(omega) Ry(ky) Rx(kx), and the inverse FFT.  This module times that with cuFFT (through
torch.fft, complex64, the same 256x256x2048 field) and prints it beside the library's own
per-launch times of the plane sweep (the x and y transforms with their factors) and the pencil
sweep (the t transforms fused with the nonlinear step).  cuFFT serves only as the
comparison here; the library never calls it.

  python cufft_compare.py [--grid 256,256,2048] [--reps 20]

The plane sweep's time covers its kernels together (two strip passes in the default variant).
"""
from __future__ import annotations

import json
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def time_cufft_linear(Nx: int, Ny: int, Nt: int, reps: int = 20) -> dict:
    import torch
    dev = torch.device("cuda")
    g = torch.Generator(device=dev).manual_seed(0)
    A = torch.randn((Nt, Ny, Nx), dtype=torch.complex64, device=dev, generator=g)
    D = torch.exp(1j * torch.linspace(0, 3, Nt, device=dev, dtype=torch.float32)).to(torch.complex64)
    Ry = torch.exp(1j * torch.linspace(0, 2, Ny, device=dev, dtype=torch.float32)).to(torch.complex64)
    Rx = torch.exp(1j * torch.linspace(0, 1, Nx, device=dev, dtype=torch.float32)).to(torch.complex64)
    fac = D[:, None, None] * Ry[None, :, None] * Rx[None, None, :] / (Nx * Ny * Nt)

    def step(x):
        X = torch.fft.fftn(x, dim=(0, 1, 2))
        X.mul_(fac)
        return torch.fft.ifftn(X, dim=(0, 1, 2), norm="forward")

    def fft_only(x):
        return torch.fft.fftn(x, dim=(0, 1, 2))

    out = {}
    for name, fn in (("fft3d_ms", fft_only), ("linear_step_ms", step)):
        for _ in range(3):
            fn(A)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn(A)
        e1.record()
        e1.synchronize()
        out[name] = e0.elapsed_time(e1) / reps
    return out


def time_library(Nx: int, Ny: int, Nt: int, steps: int = 20, **physics) -> dict:
    from mpc_gb300 import inputs
    from mpc_gb300.capi import Propagator
    cfg = inputs.cell256(Nx=Nx, Ny=Ny, Nt=Nt, window_xy=8e-3 * Nx / 256, window_t=4e-12 * Nt / 2048, **physics)
    p, A = inputs.make_cell(cfg)
    with Propagator(p.copy(variant=-1)) as prop:
        prop.upload(A, calibrate=True)
        prop.run_fixed(4)
        prop.profile(True)
        prop.run_fixed(steps)
        kt = prop.kernel_times()
        prop.profile(False)
    return {"plane_sweep_ms": kt["plane_ms"] / kt["n_plane"], "pencil_sweep_ms": kt["pencil_ms"] / kt["n_pencil"]}


def main(argv=None) -> int:
    import argparse
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--grid", default="256,256,2048")
    ap.add_argument("--reps", type=int, default=20)
    a = ap.parse_args(argv)
    Nx, Ny, Nt = (int(v) for v in a.grid.split(","))
    lib = time_library(Nx, Ny, Nt)
    kerr = time_library(Nx, Ny, Nt, plasm=0, sst_on=0)
    cu = time_cufft_linear(Nx, Ny, Nt, a.reps)
    print(json.dumps({"grid": [Nx, Ny, Nt], "dtype": "complex64", "cufft": cu,
                      "library_full_step": lib, "library_full_step_ms": sum(lib.values()),
                      "library_kerr_only_step": kerr, "library_kerr_only_step_ms": sum(kerr.values()),
                      "note": "cufft multiply reads a materialised 3-D factor"}))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
