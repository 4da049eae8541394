"""The reference's dense ALS helpers on caller matrices, on the GPU:
sptMatrixDotMulSeqTriangle (bit-exact FP32, same product order),
sptMatrixSolveNormals, sptMatrix2Norm / sptMatrixMaxNorm / GetFinalLambda and
the fit and its parts, against numpy restatements of matrix.c / ktensor.c."""
import ctypes as C

import numpy as np
import pytest

import sptol_gb300 as S
from conftest import rel_fro

pytestmark = pytest.mark.gpu


def _arr(mats):
    return (C.POINTER(S.MatrixS) * len(mats))(*[C.pointer(m.s) for m in mats])


def _grams(rng, N, rank, upper_only=True):
    gs = []
    for _ in range(N):
        a = rng.uniform(0, 1, (rng.integers(rank + 5, 4 * rank + 5), rank)).astype(np.float32)
        g = (a.T.astype(np.float64) @ a).astype(np.float32)
        if upper_only:
            g[np.tril_indices(rank, -1)] = np.float32(7e3)   # never read
        gs.append(g)
    return gs


@pytest.mark.parametrize("N,rank,mode", [(3, 16, 0), (3, 24, 2), (4, 64, 1)])
def test_dot_mul_seq_triangle_bitexact(N, rank, mode):
    rng = np.random.default_rng(N * 100 + rank)
    gs = _grams(rng, N, rank)
    mats = [S.Matrix.from_array(g) for g in gs] + [S.Matrix(rank, rank)]
    assert S.lib().sptMatrixDotMulSeqTriangle(mode, N, _arr(mats)) == 0
    exp = np.ones((rank, rank), np.float32)
    for m in range(1, N):
        pm = (mode + m) % N
        for i in range(rank):
            exp[i, i:] = exp[i, i:] * gs[pm][i, i:]
    exp = np.triu(exp) + np.triu(exp, 1).T
    assert np.array_equal(mats[N].array()[:rank, :rank], exp)


@pytest.mark.parametrize("N,rank,mode", [(3, 16, 1), (4, 32, 3), (3, 5, 0), (3, 8, 2), (4, 12, 1), (3, 24, 1),
                                         (3, 64, 2), (4, 48, 0)])
def test_solve_normals(N, rank, mode):
    """Every row-tile class of the solve (256 / 128 / 64 / 32 rows for ranks
    <= 8 / 16 / 32 / 64), with ranks that divide the block (one column per
    thread) and ranks that do not."""
    rng = np.random.default_rng(7 + rank)
    gs = _grams(rng, N, rank)
    mats = [S.Matrix.from_array(g) for g in gs] + [S.Matrix(rank, rank)]
    rhs_a = rng.uniform(-1, 1, (500, rank)).astype(np.float32)
    rhs = S.Matrix.from_array(rhs_a)
    assert S.lib().sptMatrixSolveNormals(mode, N, _arr(mats), C.byref(rhs.s)) == 0
    up = [np.triu(g.astype(np.float64)) for g in gs]
    full = [u + np.triu(u, 1).T for u in up]
    H = np.ones((rank, rank))
    for m in range(1, N):
        H *= full[(mode + m) % N]
    X = np.linalg.solve(H, rhs_a.astype(np.float64).T).T
    assert rel_fro(rhs.array()[:500, :rank], X) <= 1e-5
    # aTa[N] holds the Hadamard, as sptMatrixDotMulSeqTriangle leaves it
    assert rel_fro(mats[N].array()[:rank, :rank], H) <= 1e-6


@pytest.mark.parametrize("N,rank,mode,zero_col", [(3, 16, 1, 5), (4, 32, 3, 0)])
def test_solve_normals_exactly_singular_leaves_rows(N, rank, mode, zero_col):
    """Exactly singular Hadamard (a zero row and column in one Gram): the
    rows come back unsolved, bit for bit, as the reference's sgesv_ fallback
    leaves them (pinned in tests/test_oracle_dense.py)."""
    rng = np.random.default_rng(11 + rank)
    gs = _grams(rng, N, rank)
    k = (mode + 1) % N
    gs[k][zero_col, :] = 0.0
    gs[k][:, zero_col] = 0.0
    mats = [S.Matrix.from_array(g) for g in gs] + [S.Matrix(rank, rank)]
    rhs_a = rng.uniform(-1, 1, (300, rank)).astype(np.float32)
    rhs = S.Matrix.from_array(rhs_a)
    assert S.lib().sptMatrixSolveNormals(mode, N, _arr(mats), C.byref(rhs.s)) == 0
    assert np.array_equal(rhs.array()[:300, :rank], rhs_a)


def test_norms_and_final_lambda():
    rng = np.random.default_rng(3)
    rank = 20
    a = rng.uniform(-2, 3, (3000, rank)).astype(np.float32)
    L = S.lib()
    m = S.Matrix.from_array(a)
    lam = np.zeros(rank, np.float32)
    assert L.sptMatrix2Norm(C.byref(m.s), lam.ctypes.data_as(S.f32p)) == 0
    n2 = np.sqrt((a.astype(np.float64) ** 2).sum(0))
    assert np.allclose(lam, n2, rtol=1e-6)
    assert np.allclose(m.array()[:3000, :rank], a / n2, rtol=1e-6)
    m = S.Matrix.from_array(a)
    assert L.sptMatrixMaxNorm(C.byref(m.s), lam.ctypes.data_as(S.f32p)) == 0
    mx = np.maximum(np.maximum(a.max(0), 0), 1)
    assert np.array_equal(lam, mx.astype(np.float32))
    assert np.allclose(m.array()[:3000, :rank], a / mx, rtol=1e-6)
    # GetFinalLambda: lambda *= the 2-norms of every factor
    fs = [rng.uniform(0, 1, (n, rank)).astype(np.float32) for n in (700, 500, 90)]
    ms = [S.Matrix.from_array(f) for f in fs]
    lam = rng.uniform(1, 2, rank).astype(np.float32)
    exp = lam.astype(np.float64).copy()
    for f in fs:
        exp *= np.sqrt((f.astype(np.float64) ** 2).sum(0))
    L.GetFinalLambda(rank, 3, _arr(ms), lam.ctypes.data_as(S.f32p))
    assert np.allclose(lam, exp, rtol=1e-5)


def test_fit_and_parts():
    rng = np.random.default_rng(5)
    ndims = [60, 50, 40]
    rank = 8
    inds = np.stack([rng.integers(0, d, 3000) for d in ndims]).astype(np.uint32)
    vals = rng.uniform(0, 1, 3000).astype(np.float32)
    t = S.Tensor.from_arrays(ndims, inds, vals)
    facs = [rng.uniform(0, 1, (d, rank)).astype(np.float32) for d in ndims]
    lam = rng.uniform(0.5, 2, rank).astype(np.float32)
    mats = [S.Matrix.from_array(f) for f in facs] + [S.Matrix(max(ndims), rank)]
    # mats[N]: the last mode's MTTKRP output
    out = S.mttkrp(t, mats, 2)
    grams = [f.astype(np.float64).T @ f for f in facs]
    ata = [S.Matrix.from_array(g.astype(np.float32)) for g in grams] + [S.Matrix(rank, rank)]
    L = S.lib()
    lp = lam.ctypes.data_as(S.f32p)
    # ||K||^2 from the (row j, column i), j >= i, entries, as ktensor.c:126-168
    tmp = np.ones((rank, rank), np.float64)
    for g in grams:
        tmp *= g.astype(np.float32)
    nk = sum(tmp[i, i] * lam[i] * lam[i] for i in range(rank)) + \
        2 * sum(tmp[j, i] * lam[i] * lam[j] for i in range(rank) for j in range(i + 1, rank))
    got = L.sptKruskalTensorFrobeniusNormSquared(3, lp, _arr(ata))
    assert abs(got - nk) <= 1e-5 * abs(nk)
    inner = float((facs[2].astype(np.float64) * out.astype(np.float64)).sum(0) @ lam)
    got_inner = L.sptSparseKruskalTensorInnerProduct(3, lp, _arr(mats))
    assert abs(got_inner - inner) <= 1e-5 * abs(inner)
    nx = float((vals.astype(np.float64) ** 2).sum())
    res = nx + nk - 2 * inner
    exp_fit = 1 - (np.sqrt(res) if res > 0 else res) / np.sqrt(nx)
    fit = L.sptKruskalTensorFit(t.ptr(), lp, _arr(mats), _arr(ata))
    assert abs(fit - exp_fit) <= 1e-5


def _rarr(mats):
    return (C.POINTER(S.RankMatrixS) * len(mats))(*[C.pointer(m.s) for m in mats])


def test_rank_forms_match_matrix_forms():
    """rankmatrix.c / rankmatrix_solver.c / rankktensor.c: the sptRankMatrix
    forms give the sptMatrix forms' results bit for bit."""
    rng = np.random.default_rng(11)
    N, rank, mode = 3, 16, 1
    L = S.lib()
    gs = _grams(rng, N, rank)
    m = [S.Matrix.from_array(g) for g in gs] + [S.Matrix(rank, rank)]
    rm = [S.RankMatrix.from_array(g) for g in gs] + [S.RankMatrix(rank, rank)]
    assert L.sptMatrixDotMulSeqTriangle(mode, N, _arr(m)) == 0
    assert L.sptRankMatrixDotMulSeqTriangle(mode, N, _rarr(rm)) == 0
    assert np.array_equal(m[N].array()[:rank, :rank], rm[N].array()[:rank, :rank])
    rhs_a = rng.uniform(-1, 1, (300, rank)).astype(np.float32)
    rhs, rrhs = S.Matrix.from_array(rhs_a), S.RankMatrix.from_array(rhs_a)
    assert L.sptMatrixSolveNormals(mode, N, _arr(m), C.byref(rhs.s)) == 0
    assert L.sptRankMatrixSolveNormals(mode, N, _rarr(rm), C.byref(rrhs.s)) == 0
    assert np.array_equal(rhs.array()[:300, :rank], rrhs.array()[:300, :rank])
    a = rng.uniform(-2, 3, (2000, rank)).astype(np.float32)
    for f, rf in (("sptMatrix2Norm", "sptRankMatrix2Norm"), ("sptMatrixMaxNorm", "sptRankMatrixMaxNorm")):
        x, rx = S.Matrix.from_array(a), S.RankMatrix.from_array(a)
        l1, l2 = np.zeros(rank, np.float32), np.zeros(rank, np.float32)
        assert getattr(L, f)(C.byref(x.s), l1.ctypes.data_as(S.f32p)) == 0
        assert getattr(L, rf)(C.byref(rx.s), l2.ctypes.data_as(S.f32p)) == 0
        assert np.array_equal(l1, l2)
        assert np.array_equal(x.array()[:2000, :rank], rx.array()[:2000, :rank])
    fs = [rng.uniform(0, 1, (n, rank)).astype(np.float32) for n in (70, 50, 90)]
    lam1 = rng.uniform(1, 2, rank).astype(np.float32)
    lam2 = lam1.copy()
    L.GetFinalLambda(rank, 3, _arr([S.Matrix.from_array(f) for f in fs]), lam1.ctypes.data_as(S.f32p))
    L.GetRankFinalLambda(rank, 3, _rarr([S.RankMatrix.from_array(f) for f in fs]), lam2.ctypes.data_as(S.f32p))
    assert np.array_equal(lam1, lam2)


def test_fit_hicoo_matches_coo_fit():
    """sptKruskalTensorFitHiCOO (rankktensor.c:101-119) against
    sptKruskalTensorFit on the same tensor and factors."""
    rng = np.random.default_rng(12)
    ndims = [300, 200, 150]
    rank = 8
    inds = np.stack([rng.integers(0, d, 20000) for d in ndims]).astype(np.uint32)
    vals = rng.uniform(0, 1, 20000).astype(np.float32)
    t = S.Tensor.from_arrays(ndims, inds, vals)
    facs = [rng.uniform(0, 1, (d, rank)).astype(np.float32) for d in ndims]
    lam = rng.uniform(0.5, 2, rank).astype(np.float32)
    mats = [S.Matrix.from_array(f) for f in facs] + [S.Matrix(max(ndims), rank)]
    out = S.mttkrp(t, mats, 2)
    rmats = [S.RankMatrix.from_array(f) for f in facs] + [S.RankMatrix.from_array(
        np.vstack([out, np.zeros((max(ndims) - ndims[2], rank), np.float32)]))]
    grams = [(f.astype(np.float64).T @ f).astype(np.float32) for f in facs]
    ata = [S.Matrix.from_array(g) for g in grams] + [S.Matrix(rank, rank)]
    rata = [S.RankMatrix.from_array(g) for g in grams] + [S.RankMatrix(rank, rank)]
    L = S.lib()
    lp = lam.ctypes.data_as(S.f32p)
    fit = L.sptKruskalTensorFit(t.ptr(), lp, _arr(mats), _arr(ata))
    h = S.HiCOO(t, 4, 6)
    fit_h = L.sptKruskalTensorFitHiCOO(h.ptr(), lp, _rarr(rmats), _rarr(rata))
    assert abs(fit - fit_h) <= 1e-9 + 1e-6 * abs(fit)
    assert L.sptKruskalTensorFrobeniusNormSquaredRank(3, lp, _rarr(rata)) == \
        L.sptKruskalTensorFrobeniusNormSquared(3, lp, _arr(ata))
    h.free()
