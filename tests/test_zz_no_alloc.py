"""The entry point that computes ||X||^2 without allocating device memory,
for callers that cannot allocate (their device memory belongs to another
allocator, or cudaMalloc per call is too costly for them): two calls in a row
through the C-ABI must agree with the allocating SparseTensorFrobeniusNormSquared,
and tensors past its fixed staging capacity must be rejected.

This file is collected last so that a run stopping at the first failure has
run every other test first."""
import ctypes as C

import numpy as np
import pytest

import sptol_gb300 as S

pytestmark = pytest.mark.gpu
LIMIT = 4 * 1024 * 1024


def _entry():
    L = S.lib()
    f = L.sptgbSparseTensorFrobeniusNormSquaredNoAlloc
    f.restype = C.c_int
    f.argtypes = [C.POINTER(S.SparseTensorS), C.POINTER(C.c_double), C.c_void_p]
    return f


def _tensor(n, seed):
    rng = np.random.default_rng(seed)
    ndims = [5000, 4000, 3000]
    inds = np.stack([rng.integers(0, d, n) for d in ndims]).astype(np.uint32)
    vals = rng.standard_normal(n).astype(np.float32)
    return S.Tensor.from_arrays(ndims, inds, vals), vals


def test_no_alloc_matches_allocating_entry_point_twice():
    f = _entry()
    for n, seed in ((3_000_000, 1), (123_457, 2)):   # the second call is smaller than the first
        t, vals = _tensor(n, seed)
        got = C.c_double()
        assert f(t.ptr(), C.byref(got), None) == 0
        ref = S.lib().SparseTensorFrobeniusNormSquared(t.ptr())
        assert got.value == pytest.approx(ref, rel=1e-12)
        # FP32 squares summed in FP64, as the reference's SparseTensorFrobeniusNormSquared
        assert got.value == pytest.approx(float((vals * vals).astype(np.float64).sum()), rel=1e-12)


def test_no_alloc_empty_tensor_and_caller_stream():
    """nnz = 0 gives 0.0 (the partial slots are rewritten, not left from the
    previous call), and a caller-created stream works like the default one."""
    import torch
    f = _entry()
    t, vals = _tensor(200_000, 4)
    got = C.c_double()
    assert f(t.ptr(), C.byref(got), None) == 0 and got.value > 0.0
    empty, _ = _tensor(0, 5)
    got0 = C.c_double(-1.0)
    assert f(empty.ptr(), C.byref(got0), None) == 0
    assert got0.value == 0.0
    stream = torch.cuda.Stream()
    got1 = C.c_double()
    assert f(t.ptr(), C.byref(got1), C.c_void_p(stream.cuda_stream)) == 0
    assert got1.value == pytest.approx(float((vals * vals).astype(np.float64).sum()), rel=1e-12)


def test_no_alloc_rejects_more_values_than_its_scratch_holds():
    f = _entry()
    t, _ = _tensor(LIMIT + 1, 3)
    got = C.c_double(-1.0)
    assert f(t.ptr(), C.byref(got), None) == 3
    assert got.value == -1.0
