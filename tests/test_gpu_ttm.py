"""Sparse tensor times matrix on the GPU (sptSparseTensorMulMatrix) against
the oracle's restatement of the reference (sort at mode, fibers, products
accumulated in nonzero order with separate roundings): fiber coordinates and
values bit-exact; the input tensor left sorted at `mode` as the reference
leaves it; the semi-sparse result converted back to COO."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
import sptol_gb300 as S

pytestmark = pytest.mark.gpu


def _tensor(ndims, n, seed):
    rng = np.random.default_rng(seed)
    inds = np.unique(np.stack([rng.integers(0, d, 2 * n) for d in ndims]).astype(np.uint32), axis=1)
    inds = inds[:, rng.permutation(inds.shape[1])[:n]]
    vals = rng.uniform(-1, 1, inds.shape[1]).astype(np.float32)
    return inds, vals


def _ttm(ndims, inds, vals, U, mode, entry="sptSparseTensorMulMatrix", claim_sorted=False):
    t = S.Tensor.from_arrays(ndims, inds, vals)
    if not claim_sorted:   # sortorder as a loaded tensor has it (all zero): the call sorts
        for m in range(len(ndims)):
            t.s.sortorder[m] = 0
    um = S.Matrix.from_array(U)
    y = S.SemiSparseS()
    rc = getattr(S.lib(), entry)(C.byref(y), t.ptr(), C.byref(um.s), mode)
    return rc, t, y


@pytest.mark.parametrize("ndims,n", [([40, 30, 20], 8000), ([12, 10, 9, 8], 6000)])
@pytest.mark.parametrize("ncols", [5, 16, 40, 130])
def test_ttm_bit_exact_every_mode(ndims, n, ncols):
    inds, vals = _tensor(ndims, n, len(ndims) * 100 + ncols)
    N = len(ndims)
    for mode in range(N):
        rng = np.random.default_rng(mode + ncols)
        U = rng.uniform(-1, 1, (ndims[mode], ncols)).astype(np.float32)
        rc, t, y = _ttm(ndims, inds, vals, U, mode, "sptCudaSparseTensorMulMatrix" if mode % 2 else
                        "sptSparseTensorMulMatrix")
        assert rc == 0
        fib, Y, p = O.ttm(ndims, inds, vals, U, mode)
        nf = Y.shape[0]
        assert y.nnz == nf and y.mode == mode and y.stride == ((ncols - 1) // 8 + 1) * 8
        for m in range(N):
            if m != mode:
                got = np.ctypeslib.as_array(y.inds[m].data, shape=(nf,))
                assert np.array_equal(got, fib[m])
        vals_y = np.ctypeslib.as_array(y.values.values, shape=(nf, y.stride))[:, :ncols]
        assert np.array_equal(vals_y.view(np.uint32), Y.view(np.uint32))
        i2, v2 = t.arrays()                      # X is left sorted with `mode` last
        assert np.array_equal(i2, inds[:, p]) and np.array_equal(v2, vals[p])
        S.lib().sptFreeSemiSparseTensor(C.byref(y))


def test_semi_sparse_to_sparse_and_errors():
    ndims = [30, 20, 10]
    inds, vals = _tensor(ndims, 3000, 7)
    U = np.random.default_rng(8).uniform(-1, 1, (20, 6)).astype(np.float32)
    U[3] = 0.0                                    # zero rows give zero entries, dropped below
    rc, t, y = _ttm(ndims, inds, vals, U, 1)
    assert rc == 0
    fib, Y, _ = O.ttm(ndims, inds, vals, U, 1)
    out = S.Tensor()
    assert S.lib().sptSemiSparseTensorToSparseTensor(C.byref(out.s), C.byref(y), 1e-3) == 0
    out._owned = True
    keep = np.abs(Y.astype(np.float64)) >= 1e-3
    f_i, c_j = np.nonzero(keep)
    exp = np.stack([fib[0][f_i], c_j.astype(np.uint32), fib[2][f_i]])
    order = np.lexsort(exp[::-1])
    i2, v2 = out.arrays()
    assert np.array_equal(i2, exp[:, order])
    assert np.array_equal(v2, Y[f_i, c_j][order])
    S.lib().sptFreeSemiSparseTensor(C.byref(y))
    bad = np.zeros((7, 3), np.float32)            # U rows != ndims[mode]
    rc, _, _ = _ttm(ndims, inds, vals, bad, 0)
    assert rc != 0


def test_last_mode_with_identity_sortorder_is_not_resorted():
    """sptSparseTensorSortIndexAtMode(X, N-1, force=0) does nothing when
    X->sortorder already reads 0..N-1 (sort.c:588-617), which is what
    sptNewSparseTensor sets: the fibers are then runs in the given order,
    exactly as the reference forms them."""
    ndims = [20, 15, 10]
    inds, vals = _tensor(ndims, 1500, 21)
    U = np.random.default_rng(22).uniform(-1, 1, (10, 4)).astype(np.float32)
    rc, t, y = _ttm(ndims, inds, vals, U, 2, claim_sorted=True)
    assert rc == 0
    fib, Y, _ = O.ttm(ndims, inds, vals, U, 2, sort=False)
    nf = Y.shape[0]
    assert y.nnz == nf
    vals_y = np.ctypeslib.as_array(y.values.values, shape=(nf, y.stride))[:, :4]
    assert np.array_equal(vals_y.view(np.uint32), Y.view(np.uint32))
    i2, _ = t.arrays()
    assert np.array_equal(i2, inds)
    S.lib().sptFreeSemiSparseTensor(C.byref(y))
