"""Device sorts and COO -> HiCOO conversion: bit-exact against the reference's
own outputs (tests/golden) and against the oracle on larger inputs; HiCOO
MTTKRP within the MTTKRP tolerance."""
import ctypes as C
import os

import numpy as np
import pytest

import oracle as O
import sptol_gb300 as S
from conftest import golden, rel_fro

pytestmark = pytest.mark.gpu


def _tensor(g, key_i="inds", key_v="vals"):
    ndims = [int(x) for x in g["ndims"]]
    return ndims, S.Tensor.from_arrays(ndims, g[key_i], g[key_v])


@pytest.mark.parametrize("case", ["sort_3d", "sort_4d"])
def test_sort_golden(case):
    g = golden(case)
    ndims, t = _tensor(g)
    S.lib().sptSparseTensorSortIndex(t.ptr(), 1, 1)
    i, v = t.arrays()
    assert np.array_equal(i, g["lex_inds"]) and np.array_equal(v, g["lex_vals"])
    assert t.sortorder == list(range(len(ndims)))
    ndims, t = _tensor(g)
    order = np.ascontiguousarray(g["order"], np.uint32)
    S.lib().sptSparseTensorSortIndexCustomOrder(t.ptr(), order.ctypes.data_as(C.POINTER(C.c_uint32)), 1, 1)
    i, v = t.arrays()
    assert np.array_equal(i, g["custom_inds"]) and np.array_equal(v, g["custom_vals"])
    assert t.sortorder == [int(x) for x in order]


def test_sort_large_against_oracle():
    rng = np.random.default_rng(9)
    ndims = [3000, 70000, 257, 5]
    n = 400000
    inds = np.unique(np.stack([rng.integers(0, d, n + n // 4) for d in ndims]).astype(np.uint32), axis=1)
    inds = inds[:, rng.permutation(inds.shape[1])[:n]]
    vals = rng.random(inds.shape[1], dtype=np.float32)
    for order in ([0, 1, 2, 3], [2, 3, 0, 1]):
        t = S.Tensor.from_arrays(ndims, inds, vals)
        o = np.ascontiguousarray(order, np.uint32)
        S.lib().sptSparseTensorSortIndexCustomOrder(t.ptr(), o.ctypes.data_as(C.POINTER(C.c_uint32)), 1, 1)
        p = O.sort_lex(inds, order)
        i, v = t.arrays()
        assert np.array_equal(i, inds[:, p]) and np.array_equal(v, vals[p])


def _check_hicoo(h, g, n):
    a = h.arrays()
    N = len(a["binds"])
    assert np.array_equal(a["kptr"], g["kptr"])
    assert np.array_equal(a["cptr"], g["cptr"])
    assert np.array_equal(a["bptr"], g["bptr"])
    assert np.array_equal(np.stack(a["binds"]), g["binds"])
    assert np.array_equal(np.stack(a["einds"]), g["einds"])
    assert np.array_equal(np.array(a["nkiters"], np.uint32), g["nkiters"])
    klen = np.array([len(r) for m in range(N) for r in a["kschr"][m]], np.uint32)
    assert np.array_equal(klen, g["kschr_len"])
    kflat = np.concatenate([r for m in range(N) for r in a["kschr"][m]]).astype(np.uint32)
    assert np.array_equal(kflat, g["kschr"])
    assert h.max_nnzb == int(g["max_nnzb"])


@pytest.mark.parametrize("case", ["hicoo_3d_small", "hicoo_3d_skew", "hicoo_4d"])
def test_hicoo_golden(case):
    g = golden(case)
    ndims, t = _tensor(g)
    h = S.HiCOO(t, int(g["sb"]), int(g["sk"]))
    i, v = t.arrays()
    assert np.array_equal(i, g["sorted_inds"]) and np.array_equal(v, g["sorted_vals"])
    _check_hicoo(h, g, t.nnz)
    a = h.arrays()
    assert np.array_equal(a["values"], g["sorted_vals"])
    if "out0" in g.files:
        rank = int(g["rank"])
        N = len(ndims)
        mats = [S.Matrix.from_array(g["mat%d" % m][:, :rank]) for m in range(N)] + [S.Matrix(max(ndims), rank)]
        for mode in range(N):
            out = S.mttkrp_hicoo(h, mats, mode)
            assert rel_fro(out, g["out%d" % mode][:, :rank]) <= 1e-5


def test_hicoo_skewed_against_oracle():
    """A power-law tensor large enough for many kernels and chunks."""
    spec = S.GenSpec()
    spec.seed = 5
    spec.nmodes = 3
    for m, d in enumerate([2_000_000, 1_000_000, 20_000]):
        spec.ndims[m] = d
    spec.coord_dist[0] = spec.coord_dist[1] = S.DIST_ZIPF
    spec.zipf_s[0] = spec.zipf_s[1] = 1.2
    spec.count = 600_000
    spec.value_dist = S.VAL_LOGNORMAL
    t = S.Tensor.generate(spec)
    ndims = t.ndims
    inds, vals = t.arrays()
    p = O.sort_hicoo(inds, 17)
    oh = O.hicoo_build(ndims, inds[:, p], 7, 17)
    h = S.HiCOO(t, 7, 17)
    i2, v2 = t.arrays()
    assert np.array_equal(i2, inds[:, p]) and np.array_equal(v2, vals[p])
    _check_hicoo(h, oh, t.nnz)
    rank = 16
    mats = S.new_factors(ndims, rank, seed=4)
    facs = [m.array()[: ndims[k]].copy() for k, m in enumerate(mats[:3])]
    for mode in range(3):
        out = S.mttkrp_hicoo(h, mats, mode)
        ref = O.mttkrp(ndims, i2, v2, facs, rank, mode, precision="f64")
        assert rel_fro(out, ref) <= 1e-5


@pytest.mark.parametrize("rank,sb", [(64, 8), (5, 4)])
def test_hicoo_window_kernel_4d_skewed_against_oracle(rank, sb):
    """Order 4, power-law modes (hot output windows split over many CTAs),
    the widest tile (2^8 rows x 64) and an odd rank with small blocks."""
    spec = S.GenSpec()
    spec.seed = 8
    spec.nmodes = 4
    for m, d in enumerate([300_000, 5_000, 40_000, 300]):
        spec.ndims[m] = d
    spec.coord_dist[0] = spec.coord_dist[2] = S.DIST_ZIPF
    spec.zipf_s[0] = spec.zipf_s[2] = 1.3
    spec.count = 400_000
    spec.value_dist = S.VAL_UPM1
    t = S.Tensor.generate(spec)
    ndims = t.ndims
    h = S.HiCOO(t, sb, sb + 6)
    i2, v2 = t.arrays()
    mats = S.new_factors(ndims, rank, seed=6)
    facs = [m.array()[: ndims[k]].copy() for k, m in enumerate(mats[:4])]
    for mode in range(4):
        out = S.mttkrp_hicoo(h, mats, mode)
        ref = O.mttkrp(ndims, i2, v2, facs, rank, mode, precision="f64")
        assert rel_fro(out, ref) <= 1e-5, (mode, rel_fro(out, ref))


def test_morton_sort_matches_oracle_within_kernels():
    rng = np.random.default_rng(2)
    ndims = [5000, 3000, 700]
    n = 50000
    inds = np.unique(np.stack([rng.integers(0, d, 2 * n) for d in ndims]).astype(np.uint32), axis=1)
    inds = inds[:, rng.permutation(inds.shape[1])[:n]]
    vals = rng.random(inds.shape[1], dtype=np.float32)
    t = S.Tensor.from_arrays(ndims, inds, vals)
    assert S.lib().sptSparseTensorMixedOrder(t.ptr(), 4, 9, 1) == 0
    p = O.sort_hicoo(inds, 9)
    i, v = t.arrays()
    assert np.array_equal(i, inds[:, p])


def test_empty_tensor_conversion():
    t = S.Tensor.from_arrays([10, 10, 10], np.zeros((3, 0), np.uint32), np.zeros(0, np.float32))
    h = S.HiCOO(t, 2, 3)
    a = h.arrays()
    assert list(a["kptr"]) == [0, 1] and list(a["bptr"]) == [0, 0] and list(a["cptr"]) == [0, 1]


def _skewed3(count, seed):
    spec = S.GenSpec()
    spec.seed = seed
    spec.nmodes = 3
    for m, d in enumerate([900_000, 400_000, 9_000]):
        spec.ndims[m] = d
    spec.coord_dist[0] = spec.coord_dist[1] = S.DIST_ZIPF
    spec.zipf_s[0] = spec.zipf_s[1] = 1.2
    spec.count = count
    spec.value_dist = S.VAL_UPM1
    return S.Tensor.generate(spec)


@pytest.mark.parametrize("rank", [5, 16, 32, 64, 128])
def test_hicoo_window_kernel_3d_every_worker_width(rank):
    """Order 3 decodes 32 schedule positions per warp; worker widths 2..32
    lanes (ranks 5..128), power-law output windows split over many CTAs."""
    t = _skewed3(500_000, 21)
    ndims = t.ndims
    h = S.HiCOO(t, 7, 17)
    i2, v2 = t.arrays()
    mats = S.new_factors(ndims, rank, seed=9)
    facs = [m.array()[: ndims[k]].copy() for k, m in enumerate(mats[:3])]
    for mode in range(3):
        out = S.mttkrp_hicoo(h, mats, mode)
        ref = O.mttkrp(ndims, i2, v2, facs, rank, mode, precision="f64")
        assert rel_fro(out, ref) <= 1e-5, (mode, rel_fro(out, ref))


@pytest.mark.parametrize("sb", [4, 8])
def test_hicoo_window_kernel_3d_block_sizes(sb):
    """Order 3 with 16- and 256-row windows: the heavy windows' shared-memory
    tile covers every window size the format allows (2^sb <= 256)."""
    t = _skewed3(500_000, 23)
    ndims = t.ndims
    h = S.HiCOO(t, sb, 17)
    i2, v2 = t.arrays()
    rank = 32
    mats = S.new_factors(ndims, rank, seed=10)
    facs = [m.array()[: ndims[k]].copy() for k, m in enumerate(mats[:3])]
    for mode in range(3):
        out = S.mttkrp_hicoo(h, mats, mode)
        ref = O.mttkrp(ndims, i2, v2, facs, rank, mode, precision="f64")
        assert rel_fro(out, ref) <= 1e-5, (mode, rel_fro(out, ref))


def test_hicoo_empty_blocks_in_a_caller_hicoo():
    """A caller's HiCOO may hold empty blocks (repeated bptr entries), alone,
    in a run of 100, inside windows and as windows of their own; the result is
    that of the same nonzeros without them."""
    t = _skewed3(200_000, 22)
    ndims = t.ndims
    h = S.HiCOO(t, 7, 17)
    A = h.arrays()
    i2, v2 = t.arrays()
    rng = np.random.default_rng(23)
    bptr = A["bptr"]
    nb = len(bptr) - 1
    at = np.sort(np.concatenate([rng.integers(0, nb + 1, 300), np.full(100, nb // 2)]))
    src = np.minimum(at, nb - 1)
    nbptr = np.insert(bptr, at, bptr[at]).astype(np.uint64)
    nbinds = []
    for m in range(3):
        fill = A["binds"][m][src].copy()
        fresh = rng.random(len(at)) < 0.5
        fill[fresh] = rng.integers(0, (ndims[m] + 127) // 128, int(fresh.sum()))
        nbinds.append(np.insert(A["binds"][m], at, fill).astype(np.uint32))
    assert np.array_equal(np.diff(nbptr)[np.diff(nbptr) > 0], np.diff(bptr))
    s2, keep = _caller_hicoo(h, nbptr, nbinds)
    rank = 16
    mats = S.new_factors(ndims, rank, seed=24)
    facs = [m.array()[: ndims[k]].copy() for k, m in enumerate(mats[:3])]
    for mode in range(3):
        assert _mttkrp_raw(s2, mats, mode) == 0
        out = mats[3].array()[: ndims[mode], :rank].copy()
        ref = O.mttkrp(ndims, i2, v2, facs, rank, mode, precision="f64")
        assert rel_fro(out, ref) <= 1e-5, (mode, rel_fro(out, ref))
    del keep


def _caller_hicoo(h, bptr, binds):
    """A HiCOO struct of the caller's own arrays: h's element indices and
    values, the given bptr and block indices (kept alive by the caller)."""
    s2 = S.HiCOOS()
    s2.nmodes = h.s.nmodes
    s2.sortorder = h.s.sortorder
    s2.ndims = h.s.ndims
    s2.nnz = h.s.nnz
    s2.sb_bits, s2.sk_bits, s2.sc_bits = h.s.sb_bits, h.s.sk_bits, h.s.sc_bits
    s2.bptr = S.NnzIndexVector(len(bptr), len(bptr), bptr.ctypes.data_as(S.u64p))
    bv = (S.BlockIndexVector * len(binds))(
        *[S.BlockIndexVector(len(b), len(b), b.ctypes.data_as(S.u32p)) for b in binds])
    s2.binds = C.cast(bv, C.POINTER(S.BlockIndexVector))
    s2.einds = h.s.einds
    s2.values = h.s.values
    return s2, (bv, bptr, binds)


def _mttkrp_raw(s2, mats, mode):
    N = int(s2.nmodes)
    order, op = S._u32([mode] + [(mode + i) % N for i in range(1, N)])
    mats[N].s.nrows = int(s2.ndims[mode])
    return S.lib().sptMTTKRPHiCOO(C.byref(s2), S._mat_array(mats), op, mode)


def test_inconsistent_block_pointers_are_rejected_then_a_valid_call():
    """bptr decreasing somewhere, not starting at 0 or not ending at nnz: the
    call fails (checked on the device before the schedule or a kernel uses
    bptr); the same tensor with its own bptr then gives the right result."""
    t = _skewed3(50_000, 25)
    ndims = t.ndims
    h = S.HiCOO(t, 7, 17)
    A = h.arrays()
    i2, v2 = t.arrays()
    rank = 8
    mats = S.new_factors(ndims, rank, seed=26)
    binds = [b.astype(np.uint32) for b in A["binds"]]
    good = A["bptr"].astype(np.uint64)
    nb = len(good) - 1
    bad_variants = []
    b1 = good.copy(); b1[nb // 2] = b1[nb // 2 + 1] + 5; bad_variants.append(b1)   # decreasing
    b2 = good.copy(); b2[0] = 1; bad_variants.append(b2)                         # does not start at 0
    b3 = good.copy(); b3[nb] = good[nb] + 1000; bad_variants.append(b3)          # runs past nnz
    for bp in bad_variants:
        s2, keep = _caller_hicoo(h, bp, binds)
        for mode in range(3):
            assert _mttkrp_raw(s2, mats, mode) == 3
        del keep
    s2, keep = _caller_hicoo(h, good, binds)
    facs = [m.array()[: ndims[k]].copy() for k, m in enumerate(mats[:3])]
    for mode in range(3):
        assert _mttkrp_raw(s2, mats, mode) == 0
        ref = O.mttkrp(ndims, i2, v2, facs, rank, mode, precision="f64")
        assert rel_fro(mats[3].array()[: ndims[mode], :rank], ref) <= 1e-5
    del keep


@pytest.mark.parametrize("order", [3, 4])
def test_rank_matrix_hicoo_entry_points(order):
    """sptMTTKRPHiCOO_MatrixTiling and the OpenMP-named Scheduled / Reduce
    forms take sptRankMatrix factors and output; every mode against FP64."""
    if order == 3:
        t = _skewed3(60_000, 31)
    else:
        spec = S.GenSpec()
        spec.seed = 32
        spec.nmodes = 4
        for m, d in enumerate([3000, 700, 2000, 90]):
            spec.ndims[m] = d
        spec.count = 60_000
        spec.value_dist = S.VAL_UPM1
        t = S.Tensor.generate(spec)
    ndims = t.ndims
    N = len(ndims)
    h = S.HiCOO(t, 7, 12)
    i2, v2 = t.arrays()
    rank = 24
    rng = np.random.default_rng(33)
    facs = [rng.uniform(-1, 1, (d, rank)).astype(np.float32) for d in ndims]
    rmats = [S.RankMatrix.from_array(f) for f in facs] + [S.RankMatrix(max(ndims), rank)]
    copies = [S.RankMatrix(max(ndims), rank) for _ in range(2)]
    arr = (C.POINTER(S.RankMatrixS) * (N + 1))(*[C.pointer(m.s) for m in rmats])
    carr = (C.POINTER(S.RankMatrixS) * 2)(*[C.pointer(m.s) for m in copies])
    L = S.lib()
    pad = [np.pad(f, ((0, 0), (0, rmats[0].s.stride - rank))) for f in facs]
    for mode in range(N):
        order_, op = S._u32([mode] + [(mode + i) % N for i in range(1, N)])
        rmats[N].s.nrows = ndims[mode]
        ref = O.mttkrp(ndims, i2, v2, pad, rank, mode, precision="f64")
        for name, call in (
                ("MatrixTiling", lambda: L.sptMTTKRPHiCOO_MatrixTiling(h.ptr(), arr, op, mode)),
                ("Omp", lambda: L.sptOmpMTTKRPHiCOO_MatrixTiling(h.ptr(), arr, op, mode, 4)),
                ("Scheduled", lambda: L.sptOmpMTTKRPHiCOO_MatrixTiling_Scheduled(h.ptr(), arr, op, mode, 4, 0)),
                ("Reduce", lambda: L.sptOmpMTTKRPHiCOO_MatrixTiling_Scheduled_Reduce(h.ptr(), arr, carr, op, mode,
                                                                                    2, 0))):
            rmats[N].array()[:] = 7.0
            assert call() == 0, name
            out = rmats[N].array()[: ndims[mode], :rank]
            assert rel_fro(out, ref) <= 1e-5, (name, mode)
            assert not rmats[N].array()[: ndims[mode], rank:].any(), name


def test_dump_hicoo(tmp_path):
    """sptDumpSparseTensorHiCOO (sptensor/hicoo/dump.c:28-72): every array of
    the converted tensor, in the reference's text layout."""
    libc = C.CDLL(None)
    libc.fopen.restype = C.c_void_p
    libc.fopen.argtypes = [C.c_char_p, C.c_char_p]
    libc.fclose.argtypes = [C.c_void_p]
    rng = np.random.default_rng(21)
    ndims = [70, 40, 33]
    inds = np.stack([rng.integers(0, d, 500) for d in ndims]).astype(np.uint32)
    vals = rng.uniform(0, 1, 500).astype(np.float32)
    h = S.HiCOO(S.Tensor.from_arrays(ndims, inds, vals), 3, 5)
    A = h.arrays()
    path = str(tmp_path / "h.txt")
    fp = libc.fopen(path.encode(), b"w")
    rc = S.lib().sptDumpSparseTensorHiCOO(h.ptr(), fp)
    libc.fclose(fp)
    assert rc == 0

    def lst(tag, fmt, xs):
        return "%s length: %d\n" % (tag, len(xs)) + "".join((fmt % x) + "\t" for x in xs) + "\n"

    exp = "3\n70 40 33\nnkiters:\n" + lst("sptIndex array", "%u", A["nkiters"]) + "kschr:\n"
    for m in range(3):
        exp += "mode %d\n" % m + "".join(lst("sptIndexVector", "%u", v.tolist()) for v in A["kschr"][m])
    for name in ("kptr", "cptr", "bptr"):
        exp += name + ":\n" + lst("sptNnzIndexVector", "%u", A[name].tolist())
    exp += "binds:\n" + "".join(lst("sptBlockIndexVector", "%u", b.tolist()) for b in A["binds"])
    exp += "einds:\n" + "".join(lst("sptElementIndexVector", "%u", e.tolist()) for e in A["einds"])
    exp += "values:\n" + lst("sptValueVector", "%f", [float(v) for v in A["values"]])
    assert open(path).read() == exp
    h.free()


C2_DIMS = [4_000_000, 2_000_000, 25_000]
C2_NNZ = int(float(os.environ.get("SPTGB_C2_NNZ", "100000000")))


@pytest.mark.parametrize("nnz", [C2_NNZ], ids=lambda n: "nnz%d" % n)
def test_power_law_full_size_sorts_and_hicoo_bit_exact(nnz):
    """The 100M-nonzero power-law tensor (4,000,000 x 2,000,000 x 25,000,
    Zipf(1.2) on modes 0 and 1, lognormal values): the device HiCOO order and
    every HiCOO array (blocks 2^7, kernels 2^17: kptr, kschr, nkiters, cptr,
    bptr, binds, einds, values), the lexicographic sort and each mode's
    custom-order sort (the mode first, the others ascending) are equal bit
    for bit to the oracle's (sort.c:410-585, hicoo/convert.c:300-497).
    SPTGB_C2_NNZ sets the size (default the full 1e8)."""
    import time
    spec = S.GenSpec()
    spec.seed = 20261203
    spec.nmodes = 3
    for m, d in enumerate(C2_DIMS):
        spec.ndims[m] = d
    spec.coord_dist[0] = spec.coord_dist[1] = S.DIST_ZIPF
    spec.zipf_s[0] = spec.zipf_s[1] = 1.2
    spec.count = nnz
    spec.merge_duplicates = 0
    spec.value_dist = S.VAL_LOGNORMAL
    t0 = time.time()
    g = S.Tensor.generate(spec)
    ndims = g.ndims
    assert g.nnz == nnz
    # the generator emits lexicographic order: shuffle so that every sort has work to do
    shuf = np.random.default_rng(7).permutation(g.nnz)
    inds, vals = g.arrays()
    g.free()
    inds, vals = np.ascontiguousarray(inds[:, shuf]), vals[shuf]
    del shuf
    t = S.Tensor.from_arrays(ndims, inds, vals)
    h = S.HiCOO(t, 7, 17)
    i2, v2 = t.arrays()
    p = O.sort_hicoo(inds, 17)
    assert np.array_equal(i2, inds[:, p]) and np.array_equal(v2, vals[p])
    del i2, v2
    oh = O.hicoo_build(ndims, inds[:, p], 7, 17)
    _check_hicoo(h, oh, t.nnz)
    assert np.array_equal(h.arrays()["values"], vals[p])
    nb = len(oh["bptr"]) - 1
    del oh, p
    h.free()
    t.free()
    for order in ([0, 1, 2], [1, 0, 2], [2, 0, 1]):
        x = S.Tensor.from_arrays(ndims, inds, vals)
        o = np.ascontiguousarray(order, np.uint32)
        if order == [0, 1, 2]:
            S.lib().sptSparseTensorSortIndex(x.ptr(), 1, 1)
        else:
            S.lib().sptSparseTensorSortIndexCustomOrder(x.ptr(), o.ctypes.data_as(C.POINTER(C.c_uint32)), 1, 1)
        q = O.sort_lex(inds, order)
        xi, xv = x.arrays()
        assert np.array_equal(xi, inds[:, q]) and np.array_equal(xv, vals[q]), order
        assert x.sortorder == order
        x.free()
    print("nnz %d  %d HiCOO blocks  bit-exact HiCOO + 3 lexicographic orders in %.1f s"
          % (nnz, nb, time.time() - t0))
