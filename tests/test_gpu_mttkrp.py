"""COO MTTKRP on the GPU through the drop-in C API, against the reference's
own outputs (tests/golden) and the oracle.

Tolerance: relative Frobenius error <= 1e-5 against the reference's
sequential FP32 sptMTTKRP (the required tolerance); against the FP64 oracle
where the reference's own FP32 summation error would dominate.
"""
import numpy as np
import pytest

import oracle as O
import sptol_gb300 as S
from conftest import golden, rel_fro

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _mats(g, N, rank):
    return [S.Matrix.from_array(g["mat%d" % m][:, :rank]) for m in range(N)]


def _with_out(mats, ndims, rank):
    return mats + [S.Matrix(max(ndims), rank)]


@pytest.mark.parametrize("case", ["mttkrp_3d_r16", "mttkrp_3d_r17", "mttkrp_4d_r8"])
@pytest.mark.parametrize("entry", ["sptMTTKRP", "sptCudaMTTKRP", "sptOmpMTTKRP_Lock"])
def test_golden_all_modes(case, entry):
    g = golden(case)
    ndims = [int(x) for x in g["ndims"]]
    rank = int(g["rank"])
    N = len(ndims)
    t = S.Tensor.from_arrays(ndims, g["inds"], g["vals"])
    mats = _with_out(_mats(g, N, rank), ndims, rank)
    for mode in range(N):
        out = S.mttkrp(t, mats, mode, entry=entry)
        assert rel_fro(out, g["out%d" % mode][:, :rank]) <= TOL, (case, mode)
        # padding columns of the output stay zero, as the reference's memset leaves them
        assert not mats[N].array()[: ndims[mode], rank:].any()


def test_unsorted_input_and_mats_order():
    g = golden("mttkrp_4d_r8")
    ndims = [int(x) for x in g["ndims"]]
    rank = int(g["rank"])
    rng = np.random.default_rng(5)
    p = rng.permutation(g["vals"].shape[0])
    inds, vals = g["inds"][:, p], g["vals"][p]
    t = S.Tensor.from_arrays(ndims, inds, vals)
    mats = _with_out(_mats(g, 4, rank), ndims, rank)
    facs = [g["mat%d" % m] for m in range(4)]
    for mode in range(4):
        order = [mode] + [m for m in (3, 2, 1, 0) if m != mode]
        out = S.mttkrp(t, mats, mode, mats_order=order)
        ref = O.mttkrp(ndims, inds, vals, facs, rank, mode, order=order)
        assert rel_fro(out, ref) <= TOL


def test_empty_single_and_heavy_row():
    ndims = [7, 5, 3]
    rank = 8
    rng = np.random.default_rng(7)
    facs = [rng.random((d, 8), dtype=np.float32) for d in ndims]
    mats = _with_out([S.Matrix.from_array(f) for f in facs], ndims, rank)
    # empty tensor: every output row is zero
    t0 = S.Tensor.from_arrays(ndims, np.zeros((3, 0), np.uint32), np.zeros(0, np.float32))
    mats[3].array()[:] = 1.0
    out = S.mttkrp(t0, mats, 1)
    assert out.shape == (5, rank) and not out.any()
    # one nonzero
    t1 = S.Tensor.from_arrays(ndims, np.array([[6], [4], [2]], np.uint32), np.array([2.0], np.float32))
    out = S.mttkrp(t1, mats, 0)
    exp = np.zeros((7, rank), np.float32)
    exp[6] = 2.0 * facs[1][4] * facs[2][2]
    assert np.allclose(out, exp, rtol=1e-6)
    # every nonzero in one output row, long enough to span many work units
    big = [3, 4000, 64]
    n = 150000
    inds = np.stack([np.full(n, 1), rng.integers(0, big[1], n), rng.integers(0, big[2], n)]).astype(np.uint32)
    vals = rng.random(n, dtype=np.float32)
    bf = [rng.random((d, 16), dtype=np.float32) for d in big]
    bm = _with_out([S.Matrix.from_array(f) for f in bf], big, 16)
    tb = S.Tensor.from_arrays(big, inds, vals)
    out = S.mttkrp(tb, bm, 0)
    ref = O.mttkrp(big, inds, vals, [np.pad(f, ((0, 0), (0, 0))) for f in bf], 16, 0, precision="f64")
    assert rel_fro(out, ref) <= TOL
    assert not out[0].any() and not out[2].any()


def test_shape_mismatch_is_an_error():
    ndims = [4, 3, 2]
    t = S.Tensor.from_arrays(ndims, np.zeros((3, 1), np.uint32), np.ones(1, np.float32))
    mats = [S.Matrix(4, 8), S.Matrix(3, 8), S.Matrix(5, 8), S.Matrix(4, 8)]
    with pytest.raises(S.SptError) as e:
        S.mttkrp(t, mats, 0)
    assert e.value.code == 2


def test_out_of_range_coordinate_is_rejected():
    ndims = [4, 3, 2]
    t = S.Tensor.from_arrays(ndims, np.array([[3], [3], [1]], np.uint32), np.ones(1, np.float32))
    mats = [S.Matrix(4, 8), S.Matrix(3, 8), S.Matrix(2, 8), S.Matrix(4, 8)]
    with pytest.raises(S.SptError) as e:
        S.mttkrp(t, mats, 0)
    assert e.value.code == 3


@pytest.mark.parametrize("N", [3, 4])
@pytest.mark.parametrize("entry", ["sptMTTKRP", "sptCudaMTTKRP"])
def test_out_of_range_in_every_mode_then_a_valid_call(N, entry):
    """A coordinate at its mode size, in the output mode or in a multiplied
    mode, sorted or not, fails the call; the next valid call is exact."""
    rng = np.random.default_rng(40 + N)
    ndims = [300, 200, 100, 50][:N]
    nnz = 5000
    inds = np.stack([rng.integers(0, d, nnz) for d in ndims]).astype(np.uint32)
    vals = rng.uniform(-1, 1, nnz).astype(np.float32)
    facs = [rng.uniform(-1, 1, (d, 8)).astype(np.float32) for d in ndims]
    mats = [S.Matrix.from_array(f) for f in facs] + [S.Matrix(max(ndims), 8)]
    for bad_mode in range(N):
        for where in (0, nnz // 2, nnz - 1):
            bad = inds.copy()
            bad[bad_mode, where] = ndims[bad_mode]
            t = S.Tensor.from_arrays(ndims, bad, vals)
            for mode in range(N):
                with pytest.raises(S.SptError) as e:
                    S.mttkrp(t, mats, mode, entry=entry)
                assert e.value.code == 3, (bad_mode, where, mode)
    t = S.Tensor.from_arrays(ndims, inds, vals)
    for mode in range(N):
        out = S.mttkrp(t, mats, mode, entry=entry)
        assert rel_fro(out, O.mttkrp(ndims, inds, vals, facs, 8, mode)) <= TOL


def test_unsorted_order3_records_through_the_permutation():
    """Order 3, nonzeros in random order: the sort overlaps the uploads and
    whole records are gathered through the permutation; every mode and a
    non-default mats_order match the oracle."""
    g = golden("mttkrp_3d_r16")
    ndims = [int(x) for x in g["ndims"]]
    rank = int(g["rank"])
    p = np.random.default_rng(6).permutation(g["vals"].shape[0])
    inds, vals = g["inds"][:, p], g["vals"][p]
    t = S.Tensor.from_arrays(ndims, inds, vals)
    mats = _with_out(_mats(g, 3, rank), ndims, rank)
    facs = [g["mat%d" % m] for m in range(3)]
    for mode in range(3):
        for order in ([mode] + [m for m in (0, 1, 2) if m != mode], [mode] + [m for m in (2, 1, 0) if m != mode]):
            out = S.mttkrp(t, mats, mode, mats_order=order, entry="sptCudaMTTKRP")
            ref = O.mttkrp(ndims, inds, vals, facs, rank, mode, order=order)
            assert rel_fro(out, ref) <= TOL


def _c1_tensor():
    spec = S.GenSpec()
    spec.seed = 0
    spec.nmodes = 3
    for m in range(3):
        spec.ndims[m] = 1024
    spec.count = 1_000_000
    spec.merge_duplicates = 1
    spec.value_dist = S.VAL_U01
    return S.Tensor.generate(spec)


def test_uniform_1m_full_size_against_reference_summary_and_oracle():
    """The 1024^3 / 1,000,000-draw tensor, rank 16, every mode."""
    g = golden("uniform_1m_summary")
    t = _c1_tensor()
    assert t.nnz == int(g["nnz"])
    inds, vals = t.arrays()
    ndims = [1024] * 3
    mats = S.new_factors(ndims, 16, seed=1)
    facs = [m.array()[:1024].copy() for m in mats[:3]]
    rows = g["sample_rows"]
    for mode in range(3):
        out = S.mttkrp(t, mats, mode, entry="sptCudaMTTKRP").astype(np.float64)
        ref = O.mttkrp(ndims, inds, vals, facs, 16, mode)
        f64 = O.mttkrp(ndims, inds, vals, facs, 16, mode, precision="f64")
        assert rel_fro(out, ref) <= TOL
        assert rel_fro(out, f64) <= TOL
        assert abs(np.linalg.norm(out) - float(g["norm%d" % mode])) <= 1e-5 * float(g["norm%d" % mode])
        assert rel_fro(out[rows], g["rows%d" % mode]) <= TOL


POWERLAW_NNZ = int(float(__import__("os").environ.get("SPTGB_POWERLAW_NNZ", "100000000")))


@pytest.mark.parametrize("nnz", [POWERLAW_NNZ], ids=lambda n: "nnz%d" % n)
def test_power_law_against_fp64(nnz):
    """The 4,000,000 x 2,000,000 x 25,000 power-law tensor (Zipf(1.2) on
    modes 0 and 1, lognormal values), rank 32: ours against the FP64 oracle
    within 1e-5 for every mode, and the reference-order sequential FP32 sum
    against FP64 reported beside it (its error on the hot rows is why this
    tensor is adjudicated against FP64).  SPTGB_POWERLAW_NNZ sets the size
    (default the full 100000000)."""
    dims = [4_000_000, 2_000_000, 25_000]
    spec = S.GenSpec()
    spec.seed = 20261203
    spec.nmodes = 3
    for m, d in enumerate(dims):
        spec.ndims[m] = d
    spec.coord_dist[0] = spec.coord_dist[1] = S.DIST_ZIPF
    spec.zipf_s[0] = spec.zipf_s[1] = 1.2
    spec.count = nnz
    spec.merge_duplicates = 0
    spec.value_dist = S.VAL_LOGNORMAL
    t = S.Tensor.generate(spec)
    inds, vals = t.arrays()
    mats = S.new_factors(dims, 32, seed=1)
    facs = [m.array()[: dims[k]].copy() for k, m in enumerate(mats[:3])]
    for mode in range(3):
        out = S.mttkrp(t, mats, mode, entry="sptCudaMTTKRP").astype(np.float64)
        f64 = O.mttkrp(dims, inds, vals, facs, 32, mode, precision="f64_omp")
        seq = O.mttkrp(dims, inds, vals, facs, 32, mode)
        ours, theirs = rel_fro(out, f64), rel_fro(seq, f64)
        print("nnz %d mode %d  ours vs FP64 %.2e  reference-order FP32 vs FP64 %.2e  ours vs reference order %.2e"
              % (nnz, mode, ours, theirs, rel_fro(out, seq)))
        assert ours <= TOL


@pytest.mark.parametrize("ndims", [[700, 500], [40, 30, 20, 10, 9], [12, 11, 10, 9, 8, 7], [6, 5, 5, 4, 4, 3, 3, 2]])
@pytest.mark.parametrize("entry", ["sptMTTKRP", "sptCudaMTTKRP"])
def test_orders_2_5_6_8_against_fp64(ndims, entry):
    """Orders other than 3 and 4 run the generic segmented kernel (runtime
    number of product modes): every mode, a non-default mats_order."""
    rng = np.random.default_rng(len(ndims))
    n = 20000
    inds = np.unique(np.stack([rng.integers(0, d, 2 * n) for d in ndims]).astype(np.uint32), axis=1)
    inds = inds[:, rng.permutation(inds.shape[1])[:n]]
    vals = rng.uniform(-1, 1, inds.shape[1]).astype(np.float32)
    t = S.Tensor.from_arrays(ndims, inds, vals)
    rank = 12
    N = len(ndims)
    mats = S.new_factors(ndims, rank, seed=N)
    facs = [mats[m].array()[: ndims[m]].copy() for m in range(N)]
    for mode in range(N):
        order = [mode] + [m for m in reversed(range(N)) if m != mode]
        out = S.mttkrp(t, mats, mode, mats_order=order, entry=entry)
        ref = O.mttkrp(ndims, inds, vals, facs, rank, mode, order=order, precision="f64")
        assert rel_fro(out, ref) <= TOL, (ndims, mode)


@pytest.mark.parametrize("shuffled,rank", [(False, 16), (True, 16), (True, 17), (False, 64)])
def test_chunked_result_copy_with_a_row_across_chunks(shuffled, rank):
    """Order 3, >= 4M nonzeros through the host-buffer entry: the kernel runs
    in unit ranges and finished rows are copied back while later ranges run.
    One row holds ~30% of the nonzeros, so it crosses range boundaries;
    every mode against the FP64 oracle."""
    rng = np.random.default_rng(77)
    n = 4_500_000
    ndims = [3000, 2500, 400]
    r0 = rng.integers(0, ndims[0], n)
    r0[rng.random(n) < 0.3] = 1500
    inds = np.stack([r0, rng.integers(0, ndims[1], n), rng.integers(0, ndims[2], n)]).astype(np.uint32)
    order = np.lexsort(inds[::-1])
    if shuffled:
        order = rng.permutation(n)
    inds = np.ascontiguousarray(inds[:, order])
    vals = rng.uniform(-1, 1, n).astype(np.float32)
    t = S.Tensor.from_arrays(ndims, inds, vals)
    mats = [S.Matrix.from_array(rng.uniform(-1, 1, (d, rank)).astype(np.float32)) for d in ndims]
    mats.append(S.Matrix(max(ndims), rank))
    facs = [m.array()[: ndims[k]].copy() for k, m in enumerate(mats[:3])]   # stride-padded rows
    for mode in range(3):
        out = S.mttkrp(t, mats, mode, entry="sptCudaMTTKRP")
        ref = O.mttkrp(ndims, inds, vals, facs, rank, mode, precision="f64_omp")
        assert rel_fro(out, ref) <= TOL, mode
        # padding columns of the output stay zero
        assert not mats[3].array()[: ndims[mode], rank:].any()


@pytest.mark.parametrize("n,rank,shuffled", [(30_000, 16, False), (30_000, 20, True), (4_200_000, 16, True),
                                            (4_200_000, 64, False)])
@pytest.mark.parametrize("entry", ["sptMTTKRP", "sptCudaMTTKRP"])
def test_order4_records(n, rank, shuffled, entry):
    """Order 4 through the host-buffer entries: 16-byte records {row, a, b, c}
    in the caller's product order, values in their own array permuted with
    them when the input is not sorted by the output mode; >= 4M nonzeros also
    runs the row-range result copy.  Every mode, a rotated and a reversed
    mats_order, against the FP64 oracle."""
    rng = np.random.default_rng(n + rank)
    ndims = [700, 500, 300, 60]
    inds = np.stack([rng.integers(0, d, n) for d in ndims]).astype(np.uint32)
    inds[0, rng.random(n) < 0.2] = 123                      # one heavy row in mode 0
    order = rng.permutation(n) if shuffled else np.lexsort(inds[::-1])
    inds = np.ascontiguousarray(inds[:, order])
    vals = rng.uniform(-1, 1, n).astype(np.float32)
    t = S.Tensor.from_arrays(ndims, inds, vals)
    mats = [S.Matrix.from_array(rng.uniform(-1, 1, (d, rank)).astype(np.float32)) for d in ndims]
    mats.append(S.Matrix(max(ndims), rank))
    facs = [m.array()[: ndims[k]].copy() for k, m in enumerate(mats[:4])]
    for mode in range(4):
        others = [(mode + i) % 4 for i in range(1, 4)]
        for mo in ([mode] + others, [mode] + others[::-1]):
            out = S.mttkrp(t, mats, mode, mats_order=mo, entry=entry)
            ref = O.mttkrp(ndims, inds, vals, facs, rank, mode, precision="f64_omp")
            assert rel_fro(out, ref) <= TOL, (mode, mo)
            assert not mats[4].array()[: ndims[mode], rank:].any()


def test_pinned_host_buffers_give_the_same_result():
    """sptgbPinSparseTensor / sptgbPinMatrix: the host-buffer entry on page-
    locked caller arrays returns the same result as on pageable ones (within
    1e-6: a row spread over three or more work units is summed with float
    atomics in whatever order they land); pinning twice and unpinning what is
    not pinned are errors."""
    import ctypes as C
    rng = np.random.default_rng(5)
    ndims = [400, 300, 200]
    n = 50_000
    inds = np.stack([rng.integers(0, d, n) for d in ndims]).astype(np.uint32)
    vals = rng.uniform(-1, 1, n).astype(np.float32)
    t = S.Tensor.from_arrays(ndims, inds, vals)
    mats = [S.Matrix.from_array(rng.uniform(0, 1, (d, 16)).astype(np.float32)) for d in ndims]
    mats.append(S.Matrix(max(ndims), 16))
    plain = [S.mttkrp(t, mats, m, entry="sptCudaMTTKRP") for m in range(3)]
    L = S.lib()
    assert L.sptgbPinSparseTensor(t.ptr()) == 0
    for m in mats:
        assert L.sptgbPinMatrix(C.byref(m.s)) == 0
    try:
        assert L.sptgbPinSparseTensor(t.ptr()) != 0          # already pinned
        for mode in range(3):
            assert rel_fro(S.mttkrp(t, mats, mode, entry="sptCudaMTTKRP"), plain[mode]) <= 1e-6
    finally:
        assert L.sptgbUnpinSparseTensor(t.ptr()) == 0
        for m in mats:
            assert L.sptgbUnpinMatrix(C.byref(m.s)) == 0
    assert L.sptgbUnpinMatrix(C.byref(mats[0].s)) != 0      # not pinned any more
    S.lib().sptClearLastError()
