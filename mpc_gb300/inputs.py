"""Seeded synthetic inputs in the reference's formats (param.bin + datar/datai.bin).

The reference reads these from an external preprocessor that is not part of it
(MPC.c:76-203).  This module writes the same record from physical settings:
  grids      x_i = (i - Nx/2) dx, t_k = (k - Nt/2) dt, w_k = 2 pi (k - Nt/2)/(Nt dt),
             wr_m = 2 pi (m - Ny/2)/(Ny dx)  (centred, the reference fftshifts them);
  dispersion betas_k = beta2/2 w_k^2, beta2 = 20 fs^2/mm per bar;
  Kerr       gamma2 = n2 k0 hbar w0, n2 = 1e-23 m^2/W per bar, so that gamma2 |A|^2 = n2 k0 I
             with I = |A|^2 hbar w0 (the convention of plasma.c:135);
  gas        rho_nt = p * Natm(gas) with the density formula of plasma.c:61-115,
             rho_c = eps0 me w0^2 / e^2, n0 = 1;
  field      Gaussian in x,y (1/e^2 intensity radius) and t (intensity FWHM), flat phase,
             plus complex Gaussian noise of relative amplitude 1e-4 (splitmix64 + Box-Muller);
             Esig = sum |A|^2 dx dy dt hbar w0 of that seed, so MPC.c's calibration
             A *= sqrt(puls_e/Esig) gives the configured pulse energy.
The benchmark workloads of the multipass-cell study are the named cells below (cell64, cell256,
cell512, by their transverse grid); the data are synthetic stand-ins with the stated shapes and
distributions.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

from .params import BOUNCE_LENS, BOUNCE_SIGNFLIP, MPCParams

C0 = 299792458.0
HBAR = 1.054560652926899e-34
ME = 9.1094e-31
EL0 = 1.602e-19
EPS0 = 8.8541878128e-12
NAVO = 6.02214e23
# number density at 1 bar and molar data of plasma.c:61-115
_GAS_DENS = {"Argon": (1.784e3, 39.941), "Helium": (0.166e3, 4.002602), "Neon": (0.9002e3, 20.1797),
             "Air": (1.205e3, 28.97), "Nitrogen": (1.65e3, 14.0067), "Xenon": (5.86e3, 5.761),
             "Krypton": (3.749e3, 83.798)}


def natm(gas: str) -> float:
    dens, M = _GAS_DENS[gas]
    return dens * NAVO / M


# ---- splitmix64 + Box-Muller --------------------------------------------------------------
_GOLD = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed: int, n: int) -> np.ndarray:
    """First n outputs of the splitmix64 sequence started at `seed` (uint64)."""
    with np.errstate(over="ignore"):
        z = np.uint64(seed & 0xFFFFFFFFFFFFFFFF) + _GOLD * (np.arange(1, n + 1, dtype=np.uint64))
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def gaussian_noise(seed: int, n: int) -> np.ndarray:
    """n complex samples with independent N(0, 1/2) real and imaginary parts."""
    u = splitmix64(seed, 2 * n)
    u = ((u >> np.uint64(11)).astype(np.float64) + 0.5) * (1.0 / 9007199254740992.0)
    u1, u2 = u[0::2], u[1::2]
    rad = np.sqrt(-2.0 * np.log(u1))
    return (rad * np.cos(2 * np.pi * u2) + 1j * rad * np.sin(2 * np.pi * u2)) / math.sqrt(2.0)


@dataclasses.dataclass
class CellConfig:
    Nx: int = 64
    Ny: int = 64
    Nt: int = 512
    window_xy: float = 4e-3       # m
    window_t: float = 2e-12       # s
    beam_w: float = 0.5e-3        # 1/e^2 intensity radius, m
    fwhm: float = 250e-15         # intensity FWHM, s
    lam0: float = 1030e-9
    energy: float = 0.2e-3        # J
    noise: float = 1e-4
    seed: int = 0
    gas: str = "Argon"
    pressure: float = 1.0         # bar
    n2_per_bar: float = 1e-23
    beta2_per_bar: float = 20e-30 / 1e-3   # 20 fs^2/mm in s^2/m
    cav: float = 0.5
    roc: float = 0.3
    passes: int = 4
    steps_per_pass: int = 200
    def_err: float = 1e-5
    dzmin: float = 1e-7
    sst_on: int = 1
    plasm: int = 1
    bounce: int = BOUNCE_LENS
    Ab_M: float = 1.0


def make_cell(cfg: CellConfig) -> tuple[MPCParams, np.ndarray]:
    """(parameters, seed field A[t, y, x] complex128, un-normalised) for one cell."""
    Nx, Ny, Nt = cfg.Nx, cfg.Ny, cfg.Nt
    dx = cfg.window_xy / Nx
    dt = cfg.window_t / Nt
    x = (np.arange(Nx) - Nx // 2) * dx
    y = (np.arange(Ny) - Ny // 2) * dx
    t = (np.arange(Nt) - Nt // 2) * dt
    w = 2 * np.pi * (np.arange(Nt) - Nt // 2) / (Nt * dt)
    wr = 2 * np.pi * (np.arange(Ny) - Ny // 2) / (Ny * dx)
    k0 = 2 * np.pi / cfg.lam0
    w0 = 2 * np.pi * C0 / cfg.lam0
    beta2 = cfg.beta2_per_bar * cfg.pressure
    betas = beta2 / 2 * w ** 2
    n2 = cfg.n2_per_bar * cfg.pressure
    gamma2 = n2 * k0 * HBAR * w0
    rho_nt = cfg.pressure * natm(cfg.gas)
    rho_c = EPS0 * ME * w0 ** 2 / EL0 ** 2
    gx = np.exp(-(x / cfg.beam_w) ** 2)
    gy = np.exp(-(y / cfg.beam_w) ** 2)
    gt = np.exp(-2 * math.log(2) * (t / cfg.fwhm) ** 2)
    A = gt[:, None, None] * gy[None, :, None] * gx[None, None, :]
    A = A.astype(np.complex128)
    if cfg.noise > 0:
        A += cfg.noise * gaussian_noise(cfg.seed, A.size).reshape(A.shape)
    Esig = float(np.sum(np.abs(A) ** 2) * dx * dx * dt * HBAR * w0)
    r = y.copy()
    p = MPCParams(dims=(Nx, Ny, Nt), dist=cfg.passes * cfg.cav, dzz=cfg.cav / cfg.steps_per_pass,
                  betas=betas, alpha=0.0, Cav=cfg.cav, k0=k0, wr=wr, sst_on=cfg.sst_on, w=w,
                  gamma2=gamma2, w0=w0, plasm=cfg.plasm, deltat=dt, rho_c=rho_c, rho_nt=rho_nt,
                  n0=1.0, puls_e=cfg.energy, Ab_M=cfg.Ab_M, r=r, dr=dx, def_err=cfg.def_err,
                  dzmin=cfg.dzmin, Esig=Esig, gas=cfg.gas, bounce_mode=cfg.bounce, roc=cfg.roc)
    return p, A.reshape(-1)


# ---- the named workloads -------------------------------------------------------------
def cell64(**kw) -> CellConfig:
    """64x64 over 4 mm, 512 over 2 ps, 0.2 mJ, argon 1 bar, 4 passes x 200 fixed steps."""
    return CellConfig(**{**dict(Nx=64, Ny=64, Nt=512, window_xy=4e-3, window_t=2e-12, energy=0.2e-3,
                                seed=0, passes=4, steps_per_pass=200), **kw})


def cell256(**kw) -> CellConfig:
    """256x256 over 8 mm, 2048 over 4 ps, 1.0 mJ, 8 passes x 400 fixed steps."""
    return CellConfig(**{**dict(Nx=256, Ny=256, Nt=2048, window_xy=8e-3, window_t=4e-12, energy=1.0e-3,
                                seed=1, passes=8, steps_per_pass=400), **kw})


def cell512(**kw) -> CellConfig:
    """512x512 over 8 mm, 1024 over 2 ps, 3 mJ, 120 fs, argon 3 bar, 12 passes, adaptive 1e-5."""
    return CellConfig(**{**dict(Nx=512, Ny=512, Nt=1024, window_xy=8e-3, window_t=2e-12, energy=3e-3,
                                fwhm=120e-15, pressure=3.0, seed=2, passes=12, steps_per_pass=400,
                                def_err=1e-5), **kw})


def sweep_cells(seed: int = 100, n: int = 64) -> list[CellConfig]:
    """Batched sweep: energy log-uniform 0.1-2 mJ, pressure U(0.5, 3) bar, FWHM U(100, 300) fs;
    half the cells 128x128x1024 (4 mm, 2 ps), half 256x256x512 (8 mm, 2 ps); 6 passes."""
    out = []
    for i in range(n):
        u = ((splitmix64(seed + i, 3) >> np.uint64(11)).astype(np.float64) + 0.5) / 9007199254740992.0
        energy = 10 ** (math.log10(0.1e-3) + u[0] * (math.log10(2e-3) - math.log10(0.1e-3)))
        pressure = 0.5 + 2.5 * u[1]
        fwhm = (100 + 200 * u[2]) * 1e-15
        if i < n // 2:
            shape = dict(Nx=128, Ny=128, Nt=1024, window_xy=4e-3, window_t=2e-12)
        else:
            shape = dict(Nx=256, Ny=256, Nt=512, window_xy=8e-3, window_t=2e-12)
        out.append(CellConfig(**shape, energy=energy, pressure=pressure, fwhm=fwhm, seed=seed + i,
                              passes=6, steps_per_pass=400))
    return out


def write_run(cfg: CellConfig, datadir: str, nrun: int = 0) -> MPCParams:
    """Write one cell's inputs in the reference's layout: datadir/datar.bin and datai.bin (the
    seed field) and datadir%04d/param.bin (MPC.c:73-77, 159-168)."""
    import os

    from .params import write_field
    p, A = make_cell(cfg)
    run = f"{datadir}{nrun:04d}"
    os.makedirs(run, exist_ok=True)
    os.makedirs(datadir, exist_ok=True)
    p.write(os.path.join(run, "param.bin"))
    write_field(os.path.join(datadir, "datar.bin"), os.path.join(datadir, "datai.bin"), A)
    return p


def main(argv=None) -> int:
    """python -m mpc_gb300.inputs --cell 64 --datadir DIR [--nrun N] [--set key=value ...]"""
    import argparse
    ap = argparse.ArgumentParser(description="write param.bin, datar.bin and datai.bin for one cell")
    ap.add_argument("--cell", type=int, default=64, choices=[64, 256, 512],
                    help="64: 64x64x512, 256: 256x256x2048, 512: 512x512x1024 (adaptive)")
    ap.add_argument("--datadir", required=True, help="run directory prefix (the field goes here, "
                                                     "param.bin into DATADIR%%04d)")
    ap.add_argument("--nrun", type=int, default=0)
    ap.add_argument("--set", action="append", default=[], metavar="KEY=VALUE",
                    help="override a cell field, e.g. --set Nx=32 --set energy=1e-3")
    a = ap.parse_args(argv)
    kw = {}
    for item in a.set:
        k, v = item.split("=", 1)
        if k not in CellConfig.__dataclass_fields__:
            ap.error(f"unknown cell field {k}")
        typ = type(getattr(CellConfig(), k))
        kw[k] = typ(float(v)) if typ in (int, float) else typ(v)
    cfg = {64: cell64, 256: cell256, 512: cell512}[a.cell](**kw)
    p = write_run(cfg, a.datadir, a.nrun)
    print(f"wrote {a.datadir}{a.nrun:04d}/param.bin and {a.datadir}/datar.bin, datai.bin: "
          f"{p.Nx}x{p.Ny}x{p.Nt}, dist {p.dist} m, dzz {p.dzz} m")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
