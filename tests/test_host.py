"""Host-side logic that needs no GPU: the param.bin record, the seeded input generator, the
position->frequency tables of the in-place FFT sweeps, and the C ABI library's exports."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from mpc_gb300 import inputs
from mpc_gb300.params import MPCParams, read_field, write_field

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_param_bin_roundtrip(tmp_path):
    p, A = inputs.make_cell(inputs.cell64(Nx=16, Ny=16, Nt=32))
    path = tmp_path / "param.bin"
    p.write(str(path))
    raw = path.read_bytes()
    # exact size of the record MPC.c reads field by field
    Nx, Ny, Nt = p.dims
    assert len(raw) == 3 * 4 + 2 * 8 + Nt * 8 + 3 * 8 + Ny * 8 + 4 + Nt * 8 + 2 * 8 + 4 + 6 * 8 + Ny * 8 + 4 * 8 + 9
    q = MPCParams.read(str(path), bounce_mode=p.bounce_mode, roc=p.roc)
    for f in ("dims", "dist", "dzz", "alpha", "Cav", "k0", "sst_on", "gamma2", "w0", "plasm", "deltat", "rho_c",
              "rho_nt", "n0", "puls_e", "Ab_M", "dr", "def_err", "dzmin", "Esig", "gas"):
        assert getattr(q, f) == getattr(p, f), f
    for f in ("betas", "wr", "w", "r"):
        np.testing.assert_array_equal(getattr(q, f), getattr(p, f))
    write_field(str(tmp_path / "datar.bin"), str(tmp_path / "datai.bin"), A)
    B = read_field(str(tmp_path / "datar.bin"), str(tmp_path / "datai.bin"), p.dims)
    np.testing.assert_array_equal(A, B)


def test_param_bin_rejects_truncated():
    p, _ = inputs.make_cell(inputs.cell64(Nx=16, Ny=16, Nt=32))
    with pytest.raises(Exception):
        MPCParams.from_bytes(p.to_bytes()[:-20])


def test_splitmix64_known_values():
    # splitmix64 reference outputs for seed 0 (Vigna's reference implementation)
    v = inputs.splitmix64(0, 3)
    assert [int(x) for x in v] == [0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4, 0x06C45D188009454F]


def test_generator_deterministic_and_calibrated():
    p1, A1 = inputs.make_cell(inputs.cell64(Nx=16, Ny=16, Nt=32, seed=5))
    p2, A2 = inputs.make_cell(inputs.cell64(Nx=16, Ny=16, Nt=32, seed=5))
    np.testing.assert_array_equal(A1, A2)
    _, A3 = inputs.make_cell(inputs.cell64(Nx=16, Ny=16, Nt=32, seed=6))
    assert not np.array_equal(A1, A3)
    HBAR = 1.054560652926899e-34
    E = np.sum(np.abs(A1) ** 2) * p1.dr ** 2 * p1.deltat * HBAR * p1.w0
    assert E == pytest.approx(p1.Esig, rel=1e-12)
    noise = inputs.gaussian_noise(1, 200000)
    assert abs(np.mean(np.abs(noise) ** 2) - 1) < 0.02


def test_sweep_distribution():
    cells = inputs.sweep_cells()
    assert len(cells) == 64
    e = np.array([c.energy for c in cells])
    pr = np.array([c.pressure for c in cells])
    fw = np.array([c.fwhm for c in cells])
    assert e.min() >= 0.1e-3 and e.max() <= 2e-3 and pr.min() >= 0.5 and pr.max() <= 3 and fw.min() >= 100e-15
    assert sum(c.Nx == 128 for c in cells) == 32 and sum(c.Nt == 512 for c in cells) == 32


def _freq_of_pos(N):
    """Python statement of the in-place DIF sweep with radices 16...16, r_last, run on
    delta functions: which frequency ends up at which position."""
    radix, span = [], []
    L = N
    while L > 1:
        R = 16 if L >= 16 else L
        radix.append(R)
        span.append(L // R)
        L //= R
    x = np.eye(N, dtype=np.complex128)
    for s, R in enumerate(radix):
        Ls = span[s] * R
        out = x.copy()
        for b in range(N // Ls):
            for j in range(span[s]):
                idx = b * Ls + j + span[s] * np.arange(R)
                v = x[idx]
                y = np.fft.fft(v, axis=0)
                y *= np.exp(-2j * np.pi * j * np.arange(R) / Ls)[:, None]
                out[idx] = y
        x = out
    # row = position, column = input index; X[pos] = sum_n x_n W^(n f) identifies f
    f = []
    for pos in range(N):
        ph = np.angle(x[pos, 1]) if N > 1 else 0.0
        f.append(int(round(-ph * N / (2 * np.pi))) % N)
        np.testing.assert_allclose(x[pos], np.exp(-2j * np.pi * np.arange(N) * f[-1] / N), atol=1e-9)
    return f


@pytest.mark.parametrize("N", [8, 64, 128, 512, 2048])
def test_position_frequency_table(N):
    """The closed form the library uses (pos = sum span_s k_s, freq = sum k_s prod r_<s)
    matches a direct simulation of the DIF sweep."""
    radix, span = [], []
    L = N
    while L > 1:
        R = 16 if L >= 16 else L
        radix.append(R)
        span.append(L // R)
        L //= R
    closed = []
    for pos in range(N):
        rem, freq, mult = pos, 0, 1
        for s in range(len(radix)):
            k = rem // span[s]
            rem -= k * span[s]
            freq += k * mult
            mult *= radix[s]
        closed.append(freq)
    if N <= 512:
        assert closed == _freq_of_pos(N)
    assert sorted(closed) == list(range(N))


def _compiled_variants():
    """(Nx, Ny, Nt, SLO, PT, TP, CH, LD, PL, PMB) of every Shape<...>::ops() entry of the shape lists."""
    import glob
    import re
    out = []
    for f in sorted(glob.glob(os.path.join(ROOT, "mpc_gb300", "csrc", "mpc_shapes_*.cu"))):
        for m in re.finditer(r"Shape<([\d,\s]+)>::ops\(\)", open(f).read()):
            v = [int(x) for x in m.group(1).split(",")]
            v += [0, 512, 16384, 32, 1, 1, 0][len(v) - 3:]
            out.append(tuple(v))
    return out


SHAPES = _compiled_variants()


def _shape_cfg(NX, NY, NT, SLO_=0, PT=512, TP=16384, CH=32, LD=1, PL=1, PMB=0):
    """Tile and cluster parameters, as mpc_shapes.cuh derives them."""
    P = TP // NT
    SLO = SLO_ if SLO_ > 0 else (16 // P if P < 16 else 1)
    plane_b = NX * NY * 8
    plb = 131072 * PT // 512
    if PL >= 2:
        CL, PB = 1, 1
    elif SLO == 2:
        CL, PB = plane_b * 2 // plb, 2
    elif plane_b > plb:
        CL, PB = plane_b // plb, 1
    else:
        CL, PB = 1, min(plb // plane_b, NT)
    return P, SLO, CL, PB


def _views(*variant):
    """Python statement of the shared-memory views of mpc_kernels.cuh:
    (name, N, NLINES, at(pos, line), size)."""
    NX, NY, NT = variant[:3]
    P, SLO, CL, PB = _shape_cfg(*variant)
    if P < 16:
        SH = 3 if P < 8 else 4
        pen = lambda pos, l: pos * P + l + P * ((pos >> SH) + (pos >> 5))  # noqa: E731
        psize = NT * P + P * ((NT >> SH) + NT // 32)
    else:
        pen = lambda pos, l: pos * P + l  # noqa: E731
        psize = NT * P
    CX, RY = NX // CL, NY // CL
    RS = CX + 1
    RSZ = PB * RY * RS
    row = lambda x, l: (x // CX) * RSZ + l * RS + (x % CX)  # noqa: E731

    def col(y, l):
        pl, xl = divmod(l, CX)
        return (y // RY) * RSZ + (pl * RY + (y % RY)) * RS + xl

    if variant[8] in (2, 3):   # two-pass plane: column strips (line = column) and row strips (line = row)
        plb = 131072 * variant[4] // 512
        CXS, RYS = plb // (NY * 8), plb // (NX * 8)
        if variant[8] >= 3:    # the y pass staged by TMA: 16-column strips, 256 threads
            CXS = 16
        return [("pencil", NT, P, pen, psize), ("strip_y", NY, CXS, lambda y, l: y * CXS + l, NY * CXS),
                ("strip_x", NX, RYS, lambda x, l: l * (NX + 1) + x, RYS * (NX + 1))]
    return [("pencil", NT, P, pen, psize), ("row", NX, PB * RY, row, CL * RSZ), ("col", NY, PB * CX, col, CL * RSZ)]


def test_variant_list_parsed():
    assert (256, 256, 2048, 0, 512, 16384, 32, 1, 1, 0) in SHAPES and (256, 256, 2048, 1, 256, 16384, 16, 1, 1, 0) in SHAPES
    assert (256, 256, 2048, 1, 256, 8192, 32, 0, 1, 0) in SHAPES and (512, 512, 1024, 1, 256, 16384, 32, 1, 2, 0) in SHAPES
    assert (256, 256, 2048, 1, 128, 8192, 32, 0, 2, 5) in SHAPES
    assert (256, 256, 2048, 1, 128, 8192, 32, 0, 3, 0) in SHAPES
    assert len({v[:3] for v in SHAPES}) >= 7


def _wavefronts(addrs):
    """Shared-memory wavefronts of one warp-wide 8-byte access (32 four-byte banks)."""
    rows = {}
    for a in addrs:
        for w in (2 * a, 2 * a + 1):
            rows.setdefault(w % 32, set()).add(w // 32)
    return max(len(r) for r in rows.values())


def _warp_tail(N, NL, NTH):
    """mpc_fft.cuh WarpTail: whether the span-1 stage keeps each warp on the sub-transforms of
    the stage before, and its (line, butterfly) of pass u for thread tid."""
    LL = N
    while LL > 16:
        LL //= 16
    L2, NW, PPS = 16 * LL, NTH // 32, max(1, 16 // LL)
    ok = (N > L2 and NTH % 32 == 0 and NL * LL == 32 and 16 % LL == 0 and (N // 16 * NL) % NTH == 0
          and (N // L2) % NW == 0 and (N // LL * NL) % NTH == 0 and (N // LL * NL) // NTH == (N // L2) // NW * PPS)

    def item(tid, u):
        w, lane = tid >> 5, tid & 31
        sub = w + NW * (u // PPS)
        i = (u % PPS) * 32 + lane
        return i % NL, sub * 16 + i // NL
    return ok, LL, L2, item


@pytest.mark.parametrize("shape", SHAPES)
def test_pencil_view_bank_conflict_free(shape):
    """Every FFT stage of the pencil tile and the CH-sample t walk of the nonlinear step take
    the minimum two wavefronts per warp access (no bank conflicts); the span-1 stage with the
    warp-local mapping where it applies."""
    name, N, P, at, size = _views(*shape)[0]
    CH = shape[6]
    nthr = N * P // CH
    ok, LL, _, item = _warp_tail(N, P, nthr)
    L = N
    while L > 1:
        R = 16 if L >= 16 else L
        S = L // R
        if ok and S == 1:
            for w in range(nthr // 32):
                for u in range(N // R * P // nthr):
                    for q in range(R):
                        addrs = []
                        for tid in range(32 * w, 32 * w + 32):
                            line, g = item(tid, u)
                            addrs.append(at(g * L + q, line))
                        assert _wavefronts(addrs) <= 2, (shape, L, w, u, q)
        else:
            for w0 in range(0, min(N // R * P, nthr), 32):
                for q in range(R):
                    addrs = []
                    for idx in range(w0, w0 + 32):
                        line, g = idx % P, idx // P
                        addrs.append(at((g // S) * L + g % S + S * q, line))
                    assert _wavefronts(addrs) <= 2, (shape, L, w0, q)
        L //= R
    for w0 in range(0, min(nthr, 256), 32):
        for i in range(CH):
            assert _wavefronts([at(CH * (t // P) + i, t % P) for t in range(w0, w0 + 32)]) <= 2, (shape, i)


@pytest.mark.parametrize("N,NL,NTH", [(2048, 4, 256), (1024, 8, 256), (2048, 8, 512), (512, 32, 512)])
def test_warp_tail_mapping(N, NL, NTH):
    """Where the warp-local tail applies, its span-1 stage visits every (line, butterfly) once
    and each warp works only inside the sub-transforms it wrote in the stage before (so a warp
    barrier between the two stages suffices); the 2048-point, 4-pencil, 256-thread tile uses it."""
    ok, LL, L2, item = _warp_tail(N, NL, NTH)
    assert ok == ((N, NL, NTH) in [(2048, 4, 256), (1024, 8, 256)])
    if not ok:
        return
    TOT = N // LL * NL
    seen = set()
    for tid in range(NTH):
        w = tid >> 5
        # stage L2 (radix 16, span LL), default mapping: the sub-transforms this warp wrote
        mine = {((tid + u * NTH) // NL // LL) for u in range(N // 16 * NL // NTH)}
        for u in range(TOT // NTH):
            line, g = item(tid, u)
            assert 0 <= line < NL and 0 <= g < N // LL
            seen.add((line, g))
            assert g * LL // L2 in mine, (tid, u)
        assert all(b % (NTH // 32) == w for b in mine)
    assert len(seen) == TOT


def _xsw(x, l):
    """Byte offset of element (row l, x) in the TMA x pass's swizzled unit (mpc_kernels.cuh xsw_offset)."""
    return ((x >> 4) << 11) + (l << 7) + ((((x & 15) >> 1) ^ (l & 7)) << 4) + ((x & 1) << 3)


def _wavefronts_bytes(accesses):
    """Wavefronts of one warp-wide access given (thread, byte offset, width): threads are served
    128 bytes at a time (half-warps for 8-byte, quarter-warps for 16-byte accesses); within a
    phase every distinct 4-byte word of a bank costs one wavefront."""
    width = accesses[0][2]
    per = 128 // width
    total = 0
    for g in range(0, len(accesses), per):
        banks = {}
        for _, off, w in accesses[g:g + per]:
            for wd in range(off // 4, (off + w) // 4):
                banks.setdefault(wd % 32, set()).add(wd)
        total += max(len(v) for v in banks.values())
    return total


def test_tma_x_swizzle_is_a_permutation_and_conflict_free():
    """The TMA x pass's unit layout (16 boxes of 16 rows x 128 B with the 128-byte swizzle) covers
    the 32 KB unit once, and its three passes over a unit take the minimum wavefronts per warp
    access: the span-16 stages (8-byte accesses, 16 butterflies j of a row per half-warp) and
    the span-1 pass (16-byte pairs, 8 rows per quarter-warp)."""
    offs = sorted(_xsw(x, l) for l in range(16) for x in range(256))
    assert offs == list(range(0, 32768, 8))
    for w0 in range(0, 256, 32):               # span-16 stages: item -> (j = item & 15, l = item >> 4)
        for q in range(16):
            acc = [(t, _xsw((t & 15) + 16 * q, t >> 4), 8) for t in range(w0, w0 + 32)]
            assert _wavefronts_bytes(acc) == 2, (w0, q)
    for w0 in range(0, 256, 32):               # span-1 pass: item -> (l = item & 15, b = item >> 4)
        for c in range(8):
            acc = [(t, (((t >> 4) << 11) + ((t & 15) << 7) + ((c ^ ((t & 15) & 7)) << 4)), 16) for t in range(w0, w0 + 32)]
            assert _wavefronts_bytes(acc) == 4, (w0, c)


@pytest.mark.parametrize("shape", [v for v in SHAPES if v[8] in (2, 3, 4)])
def test_strip_views_bank_conflict_free(shape):
    """The two-pass plane's strip views: every FFT stage (lines fastest across a warp, as the
    stage loops take them) reads and writes with the minimum two wavefronts per warp access."""
    for name, N, NL, at, size in _views(*shape)[1:]:
        L = N
        while L > 1:
            R = 16 if L >= 16 else L
            S = L // R
            for w0 in range(0, min(N // R * NL, shape[4]), 32):
                for q in range(R):
                    addrs = [at(((idx // NL) // S) * L + (idx // NL) % S + S * q, idx % NL) for idx in range(w0, w0 + 32)]
                    assert _wavefronts(addrs) <= 2, (shape, name, L, w0, q)
            L //= R


@pytest.mark.parametrize("shape", SHAPES)
def test_fft_views_stage_separable_and_in_bounds(shape):
    """The FFT stages address a butterfly as at(base) + at(S q) - at(0) (mpc_fft.cuh); check
    that this equals at(base + S q) for every view, stage and butterfly, that every address
    is inside the view's shared-memory buffer, and that the view is one-to-one."""
    for name, N, NL, at, size in _views(*shape):
        if name == "pencil":   # the walk offsets of the nonlinear step equal at(t0 + i) - at(t0)
            CH = shape[6]
            for t0 in range(0, N, CH):
                for i in range(CH):
                    assert at(t0 + i, 0) - at(t0, 0) == at(i, 0) - at(0, 0), (t0, i)
        seen = set()
        for pos in range(N):
            for l in range(NL):
                a = at(pos, l)
                assert 0 <= a < size, (name, pos, l)
                seen.add(a)
        assert len(seen) == N * NL, name
        L = N
        while L > 1:
            R = 16 if L >= 16 else L
            S = L // R
            for b in range(N // L):
                for j in range(S):
                    base = b * L + j
                    for l in (0, 1, NL - 1):
                        for q in range(R):
                            assert at(base + S * q, l) == at(base, l) + at(S * q, 0) - at(0, 0), (name, L, b, j, l, q)
            L //= R


def _header_symbols():
    with open(os.path.join(ROOT, "include", "mpc_gpu.h")) as f:
        txt = f.read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(mpc_[a-z0-9_A-Z]+)\s*\(", txt)))


def test_capi_library_exports_every_header_symbol():
    """libmpc_gpu.so loads without a GPU and exports every entry point of include/mpc_gpu.h;
    no compute call is made here."""
    from mpc_gb300 import build, capi
    lib_path = build.build()
    lib = C.CDLL(lib_path)
    syms = _header_symbols()
    assert len(syms) >= 25
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    assert set(syms) <= set(capi.SIGNATURES), set(syms) - set(capi.SIGNATURES)
    lib.mpc_version.restype = C.c_char_p
    assert b"sm_103a" in lib.mpc_version()
    lib.mpc_shape_supported.argtypes = [C.c_int] * 3
    assert lib.mpc_shape_supported(256, 256, 2048) == 1
    assert lib.mpc_shape_supported(100, 100, 100) == 0


def test_context_without_a_gpu_fails_loudly():
    """With no usable GPU, creating a context returns an error status with the CUDA reason
    (raised as MPCError by the binding): there is no CPU fallback in the product."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from mpc_gb300 import build, capi, inputs
    build.build()
    p, _ = inputs.make_cell(inputs.cell64(Nx=16, Ny=16, Nt=64))
    with pytest.raises(capi.MPCError, match="mpc_create: MPC_ERR_CUDA"):
        capi.Propagator(p)


def _tw_stage_offset(N, L):
    """Python statement of tw_stage_offset (mpc_fft.cuh): entries before the stage of sub-length L."""
    off, M = 0, N
    while M != L:
        R = 16 if M >= 16 else M
        off += M - M // R
        M //= R
    return off


@pytest.mark.parametrize("N", sorted({v[0] for v in SHAPES} | {v[2] for v in SHAPES}))
def test_staged_twiddle_layout(N):
    """The shared-memory twiddle table of a length-N transform in staged order
    (stage_twiddles): stage L, factor k, butterfly j at tw_stage_offset(N, L) + (k-1) S + j holds
    W_N^(j k N/L); the stages fill fewer than N entries, each entry once; and a warp's reads of
    one factor k, lines fastest as the stage loops take them, need at most one wavefront for
    P >= 4 lines (the natural-order table needed up to 8 at the middle stage of N = 2048)."""
    seen = {}
    L = N
    while L > 1:
        R = 16 if L >= 16 else L
        S = L // R
        off = _tw_stage_offset(N, L)
        if S > 1:
            for k in range(1, R):
                for j in range(S):
                    i = off + (k - 1) * S + j
                    assert i not in seen and 0 <= i < N
                    seen[i] = (j * k * (N // L)) % N
            for P in (4, 8):
                for w0 in range(0, N // R * P, 32):
                    for k in range(1, R):
                        words = set()
                        for idx in range(w0, min(w0 + 32, N // R * P)):
                            j = (idx // P) % S
                            a = off + (k - 1) * S + j
                            words |= {2 * a, 2 * a + 1}
                        per_bank = {}
                        for w in words:
                            per_bank.setdefault(w % 32, set()).add(w // 32)
                        assert max(len(r) for r in per_bank.values()) <= 1, (N, L, P, k)
        L //= R
    # the span-1 stage (the last, sub-length L_min <= 16) has no twiddles: the stages before it
    # fill N - L_min entries (a telescoping sum of L - L/R)
    L_min = N
    while L_min > 16:
        L_min //= 16
    assert len(seen) == _tw_stage_offset(N, L_min) == N - L_min
