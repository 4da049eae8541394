"""The formulas the GPU tests of the dense CP-ALS helpers check against
(tests/test_gpu_dense_api.py) pinned to the reference's own functions, built
from its sources: sptMatrixDotMulSeqTriangle (matrix.c:341-386) bit for bit,
sptMatrix2Norm / sptMatrixMaxNorm (matrix.c:390-554), and the parts of
sptKruskalTensorFit (ktensor.c:126-257).  CPU only."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.skipif(not O.ref_available(), reason="reference sources not present")


def _grams(rng, N, rank):
    gs = []
    for _ in range(N):
        a = rng.uniform(0, 1, (rank + 9, rank)).astype(np.float32)
        gs.append((a.T.astype(np.float64) @ a).astype(np.float32))
    return gs


@pytest.mark.parametrize("N,rank,mode", [(3, 16, 0), (3, 24, 2), (4, 64, 1), (5, 8, 4)])
def test_dot_mul_seq_triangle_formula(N, rank, mode):
    rng = np.random.default_rng(N * 100 + rank)
    gs = _grams(rng, N, rank)
    for g in gs:
        g[np.tril_indices(rank, -1)] = np.float32(7e3)     # the lower triangle is never read
    got = O.ref_dotmul_triangle(gs, mode)
    exp = np.ones((rank, rank), np.float32)
    for m in range(1, N):
        pm = (mode + m) % N
        for i in range(rank):
            exp[i, i:] = exp[i, i:] * gs[pm][i, i:]
    exp = np.triu(exp) + np.triu(exp, 1).T
    assert np.array_equal(got, exp)


def test_column_norm_formulas():
    rng = np.random.default_rng(3)
    a = rng.uniform(-2, 3, (3000, 20)).astype(np.float32)
    na, lam = O.ref_colnorm(a, use_max=False)
    n2 = np.sqrt((a.astype(np.float64) ** 2).sum(0))
    assert np.allclose(lam, n2, rtol=1e-5)
    assert np.allclose(na, a / n2, rtol=1e-5)
    na, lam = O.ref_colnorm(a, use_max=True)
    mx = np.maximum(a.max(0), 1).astype(np.float32)          # signed column maximum, at least 1
    assert np.array_equal(lam, mx)
    assert np.allclose(na, a / mx, rtol=1e-6)
    # every column below 1: the divisor stays 1
    small = rng.uniform(-1, 0.5, (100, 8)).astype(np.float32)
    na, lam = O.ref_colnorm(small, use_max=True)
    assert np.array_equal(lam, np.ones(8, np.float32)) and np.array_equal(na, small)


def test_kruskal_norm_and_inner_product_formulas():
    rng = np.random.default_rng(5)
    ndims = [60, 50, 40]
    rank = 8
    facs = [rng.uniform(0, 1, (d, rank)).astype(np.float32) for d in ndims]
    lam = rng.uniform(0.5, 2, rank).astype(np.float32)
    grams = [(f.astype(np.float64).T @ f).astype(np.float32) for f in facs]
    tmp = np.ones((rank, rank), np.float64)
    for g in grams:
        tmp *= g
    nk = sum(tmp[i, i] * lam[i] * lam[i] for i in range(rank)) + \
        2 * sum(tmp[j, i] * lam[i] * lam[j] for i in range(rank) for j in range(i + 1, rank))
    got = O.ref_kruskal_normsq(grams, lam)
    assert abs(got - nk) <= 1e-5 * abs(nk)
    mout = rng.uniform(0, 3, (ndims[2], rank)).astype(np.float32)
    inner = float((facs[2].astype(np.float64) * mout.astype(np.float64)).sum(0) @ lam)
    got = O.ref_kruskal_inner(facs, mout, lam)
    assert abs(got - inner) <= 1e-5 * abs(inner)


@pytest.mark.parametrize("N,rank,mode", [(3, 16, 1), (4, 32, 3)])
def test_solve_normals_formula(N, rank, mode):
    """X G = rhs with G the Hadamard of the other Grams (upper triangles
    mirrored): the reference's FP32 Cholesky solve against the FP64 formula
    the GPU test uses, within the GPU test's own 1e-5 (condition numbers ~60-70)."""
    rng = np.random.default_rng(7 + rank)
    gs = _grams(rng, N, rank)
    rhs = rng.uniform(-1, 1, (500, rank)).astype(np.float32)
    got = O.ref_solve_normals(gs, mode, rhs)
    full = [np.triu(g.astype(np.float64)) + np.triu(g.astype(np.float64), 1).T for g in gs]
    H = np.ones((rank, rank))
    for m in range(1, N):
        H *= full[(mode + m) % N]
    X = np.linalg.solve(H, rhs.astype(np.float64).T).T
    err = np.linalg.norm(got - X) / np.linalg.norm(X)
    assert err <= 1e-5, err


@pytest.mark.parametrize("N,rank,mode,zero_col", [(3, 16, 1, 5), (4, 32, 3, 0)])
def test_solve_normals_exactly_singular_leaves_rows(N, rank, mode, zero_col):
    """A Gram with a zero row and column (a factor column that is all zero)
    makes the Hadamard exactly singular: the reference's spotrf_ fails, its
    sgesv_ fallback meets an exactly zero pivot and returns with the
    right-hand sides untouched, so sptMatrixSolveNormals leaves the rows as
    they came in.  The device solve and the oracle restate that."""
    rng = np.random.default_rng(11 + rank)
    gs = _grams(rng, N, rank)
    k = (mode + 1) % N
    gs[k][zero_col, :] = 0.0
    gs[k][:, zero_col] = 0.0
    rhs = rng.uniform(-1, 1, (300, rank)).astype(np.float32)
    got = O.ref_solve_normals(gs, mode, rhs)
    assert np.array_equal(got, rhs)
