"""Run parameters of the split-step propagator: the param.bin record of kmecseki/MPC.

param.bin is read field by field with fread in MPC.c:77,180-203, native byte order, no
padding:  int dims[3]; double dist, dzz; double betas[Nt]; double alpha, Cav, k0;
double wr[Ny]; int sst_on; double w[Nt]; double gamma2, w0; int plasm; double deltat,
rho_c, rho_nt, n0, puls_e, Ab_M; double r[Ny]; double dr, def_err, dzmin, Esig;
char gas[9].  Fields and units are those of the reference; bounce_mode and roc describe
the mirror, which the reference models only as a diffraction sign flip and which
param.bin therefore does not carry; variant picks among the compiled kernel variants of a
grid (speed only).
"""
from __future__ import annotations

import dataclasses
import struct

import numpy as np

BOUNCE_SIGNFLIP = 0
BOUNCE_LENS = 1


@dataclasses.dataclass
class MPCParams:
    dims: tuple[int, int, int]
    dist: float
    dzz: float
    betas: np.ndarray
    alpha: float
    Cav: float
    k0: float
    wr: np.ndarray
    sst_on: int
    w: np.ndarray
    gamma2: float
    w0: float
    plasm: int
    deltat: float
    rho_c: float
    rho_nt: float
    n0: float
    puls_e: float
    Ab_M: float
    r: np.ndarray
    dr: float
    def_err: float
    dzmin: float
    Esig: float
    gas: str
    bounce_mode: int = BOUNCE_SIGNFLIP
    roc: float = 0.0
    variant: int = 0          # compiled kernel variant of the grid (0 default, -1 autotune)
    land_mirrors: int = 0     # step doubling ends attempts on mirror planes (0: as the reference)

    @property
    def Nx(self) -> int:
        return int(self.dims[0])

    @property
    def Ny(self) -> int:
        return int(self.dims[1])

    @property
    def Nt(self) -> int:
        return int(self.dims[2])

    @property
    def N(self) -> int:
        return self.Nx * self.Ny * self.Nt

    def copy(self, **changes) -> "MPCParams":
        d = dataclasses.asdict(self)
        for k in ("betas", "wr", "w", "r"):
            d[k] = np.array(d[k], dtype=np.float64)
        d.update(changes)
        return MPCParams(**d)

    # ---- param.bin ------------------------------------------------------------------
    def to_bytes(self) -> bytes:
        Nx, Ny, Nt = self.dims
        out = [struct.pack("=3i", Nx, Ny, Nt), struct.pack("=2d", self.dist, self.dzz)]
        out.append(np.asarray(self.betas, dtype="=f8").tobytes())
        out.append(struct.pack("=3d", self.alpha, self.Cav, self.k0))
        out.append(np.asarray(self.wr, dtype="=f8").tobytes())
        out.append(struct.pack("=i", self.sst_on))
        out.append(np.asarray(self.w, dtype="=f8").tobytes())
        out.append(struct.pack("=2d", self.gamma2, self.w0))
        out.append(struct.pack("=i", self.plasm))
        out.append(struct.pack("=6d", self.deltat, self.rho_c, self.rho_nt, self.n0, self.puls_e, self.Ab_M))
        out.append(np.asarray(self.r, dtype="=f8").tobytes())
        out.append(struct.pack("=4d", self.dr, self.def_err, self.dzmin, self.Esig))
        g = self.gas.encode("ascii")[:8]
        out.append(g + b"\0" * (9 - len(g)))
        return b"".join(out)

    @classmethod
    def from_bytes(cls, buf: bytes, bounce_mode: int = BOUNCE_SIGNFLIP, roc: float = 0.0) -> "MPCParams":
        off = 0

        def take(fmt):
            nonlocal off
            v = struct.unpack_from(fmt, buf, off)
            off += struct.calcsize(fmt)
            return v

        def arr(n):
            nonlocal off
            a = np.frombuffer(buf, dtype="=f8", count=n, offset=off).copy()
            off += 8 * n
            return a

        Nx, Ny, Nt = take("=3i")
        if min(Nx, Ny, Nt) <= 0:
            raise ValueError(f"param.bin: invalid dims {Nx}x{Ny}x{Nt}")
        dist, dzz = take("=2d")
        betas = arr(Nt)
        alpha, Cav, k0 = take("=3d")
        wr = arr(Ny)
        (sst_on,) = take("=i")
        w = arr(Nt)
        gamma2, w0 = take("=2d")
        (plasm,) = take("=i")
        deltat, rho_c, rho_nt, n0, puls_e, Ab_M = take("=6d")
        r = arr(Ny)
        dr, def_err, dzmin, Esig = take("=4d")
        if len(buf) < off + 9:
            raise ValueError("param.bin: truncated record")
        gas = buf[off:off + 9].split(b"\0", 1)[0].decode("ascii")
        return cls((Nx, Ny, Nt), dist, dzz, betas, alpha, Cav, k0, wr, sst_on, w, gamma2, w0, plasm,
                   deltat, rho_c, rho_nt, n0, puls_e, Ab_M, r, dr, def_err, dzmin, Esig, gas,
                   bounce_mode, roc)

    def write(self, path: str) -> None:
        with open(path, "wb") as f:
            f.write(self.to_bytes())

    @classmethod
    def read(cls, path: str, **kw) -> "MPCParams":
        with open(path, "rb") as f:
            return cls.from_bytes(f.read(), **kw)


def write_field(prefix_r: str, prefix_i: str, A: np.ndarray) -> None:
    """datar.bin / datai.bin: N raw doubles each, x fastest, t slowest (MPC.c:159-168)."""
    np.ascontiguousarray(A.real, dtype="=f8").tofile(prefix_r)
    np.ascontiguousarray(A.imag, dtype="=f8").tofile(prefix_i)


def read_field(path_r: str, path_i: str, dims) -> np.ndarray:
    n = int(np.prod(dims))
    re = np.fromfile(path_r, dtype="=f8", count=n)
    im = np.fromfile(path_i, dtype="=f8", count=n)
    if re.size != n or im.size != n:
        raise ValueError("field files shorter than Nx*Ny*Nt doubles")
    return (re + 1j * im).astype(np.complex128)
