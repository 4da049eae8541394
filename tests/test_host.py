"""Host-side logic of the library that needs no GPU: containers, argument
checks and their error codes, mode-order helpers, the seeded generator."""
import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest

import sptol_gb300 as S
from conftest import ROOT


def test_matrix_stride_and_vectors():
    m = S.Matrix(5, 17)
    assert m.s.stride == 24 and m.s.cap == 5
    m0 = S.Matrix(0, 8)
    assert m0.s.cap == 1 and m0.s.stride == 8
    t = S.Tensor.from_arrays([3, 4], np.array([[0, 2], [3, 1]], np.uint32), np.array([1.5, 2.5], np.float32))
    i, v = t.arrays()
    assert t.nnz == 2 and list(i[1]) == [3, 1] and list(v) == [1.5, 2.5]
    assert t.sortorder == [0, 1]


def test_shape_errors_return_codes_before_any_device_work():
    L = S.lib()
    t = S.Tensor.from_arrays([4, 3, 2], np.zeros((3, 1), np.uint32), np.ones(1, np.float32))
    bad_cols = [S.Matrix(4, 8), S.Matrix(3, 16), S.Matrix(2, 8), S.Matrix(4, 8)]
    with pytest.raises(S.SptError) as e:
        S.mttkrp(t, bad_cols, 0)
    assert e.value.code == 2
    bad_rows = [S.Matrix(4, 8), S.Matrix(3, 8), S.Matrix(7, 8), S.Matrix(4, 8)]
    with pytest.raises(S.SptError) as e:
        S.mttkrp(t, bad_rows, 0, entry="sptCudaMTTKRP")
    assert e.value.code == 2
    reason = C.c_char_p()
    assert L.sptGetLastError(None, None, None, C.byref(reason)) == 2
    assert b"nrows" in reason.value
    L.sptClearLastError()
    assert L.sptGetLastError(None, None, None, None) == 0


def _best(ndims, mode):
    L = S.lib()
    L.sptGetBestModeOrder.argtypes = [C.POINTER(C.c_uint32), C.c_uint32, C.POINTER(C.c_uint32), C.c_uint32]
    L.sptGetWorstModeOrder.argtypes = L.sptGetBestModeOrder.argtypes
    nd = np.array(ndims, np.uint32)
    out = np.zeros(len(ndims), np.uint32)
    L.sptGetBestModeOrder(out.ctypes.data_as(C.POINTER(C.c_uint32)), mode, nd.ctypes.data_as(C.POINTER(C.c_uint32)),
                          len(ndims))
    worst = np.zeros(len(ndims), np.uint32)
    L.sptGetWorstModeOrder(worst.ctypes.data_as(C.POINTER(C.c_uint32)), mode,
                           nd.ctypes.data_as(C.POINTER(C.c_uint32)), len(ndims))
    return list(out), list(worst)


def test_mode_orders():
    # mode first, then increasing sizes (sort.c:193-227)
    assert _best([40, 10, 30], 0)[0] == [0, 1, 2]
    assert _best([40, 10, 30], 2)[0] == [2, 1, 0]
    # decreasing sizes with the mode moved last (sort.c:239-274)
    assert _best([40, 10, 30], 1)[1] == [0, 2, 1]


def _spec(seed=1, count=50_000, merge=0, val=S.VAL_LOGNORMAL):
    s = S.GenSpec()
    s.seed = seed
    s.nmodes = 3
    for m, d in enumerate([3000, 2000, 50]):
        s.ndims[m] = d
    s.coord_dist[0] = s.coord_dist[1] = S.DIST_ZIPF
    s.zipf_s[0] = s.zipf_s[1] = 1.2
    s.count = count
    s.merge_duplicates = merge
    s.value_dist = val
    return s


def test_generator_exact_unique_count_sorted_and_skewed():
    t = S.Tensor.generate(_spec())
    i, v = t.arrays()
    assert t.nnz == 50_000
    key = (i[0].astype(np.int64) * 2000 + i[1]) * 50 + i[2]
    assert (np.diff(key) > 0).all()       # lexicographically sorted, no duplicates
    assert (i[0] < 3000).all() and (i[1] < 2000).all() and (i[2] < 50).all()
    c = np.bincount(i[0], minlength=3000)
    assert c[0] > 20 * c[100:].mean()     # Zipf head
    assert (v > 0).all()
    t2 = S.Tensor.generate(_spec())
    assert np.array_equal(t2.arrays()[0], i) and np.array_equal(t2.arrays()[1], v)
    t3 = S.Tensor.generate(_spec(seed=2))
    assert not np.array_equal(t3.arrays()[0], i)


def test_generator_merge_mode_sums_duplicates():
    s = _spec(count=200_000, merge=1, val=S.VAL_U01)
    t = S.Tensor.generate(s)
    i, v = t.arrays()
    assert t.nnz < 200_000
    assert abs(v.astype(np.float64).sum() / 200_000 - 0.5) < 0.01


def test_generator_wide_keys_beyond_64_bits():
    """4 modes of 100,000 (68 coordinate bits): 128-bit keys, same contract."""
    dims = [100_000, 99_000, 70_000, 65_000]
    s = S.GenSpec()
    s.seed = 9
    s.nmodes = 4
    for m, d in enumerate(dims):
        s.ndims[m] = d
    s.count = 20_000
    s.merge_duplicates = 0
    s.value_dist = S.VAL_U01
    t = S.Tensor.generate(s)
    i, v = t.arrays()
    assert t.nnz == 20_000
    assert all((i[m] < dims[m]).all() for m in range(4))
    order = np.lexsort(i[::-1])
    assert (order == np.arange(len(order))).all()          # lexicographically sorted
    k = np.stack(i, 1)
    assert (np.abs(np.diff(k, axis=0)).sum(1) > 0).all()   # no duplicates
    assert (i[3] > 40_000).any() and (i[0] > 80_000).any()
    t2 = S.Tensor.generate(s)
    assert np.array_equal(t2.arrays()[0], i) and np.array_equal(t2.arrays()[1], v)
    s.merge_duplicates = 1
    with pytest.raises(S.SptError):
        S.Tensor.generate(s)


def test_generator_independent_of_thread_count():
    code = ("import sys; sys.path.insert(0, %r); sys.path.insert(0, %r); import hashlib, sptol_gb300 as S;"
            "from test_host import _spec; t = S.Tensor.generate(_spec(count=200000));"
            "i, v = t.arrays(); print(hashlib.sha1(i.tobytes() + v.tobytes()).hexdigest())"
            % (ROOT, os.path.join(ROOT, "tests")))
    outs = []
    for threads in ("1", "3"):
        env = dict(os.environ, OMP_NUM_THREADS=threads, PYTHONPATH=ROOT)
        outs.append(subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True,
                                   check=True).stdout.strip())
    assert outs[0] == outs[1]


def test_mode_orders_equal_the_reference():
    """sptGetBestModeOrder / sptGetWorstModeOrder (sort.c:193-233) against the
    reference library built from its sources, over random shapes with ties."""
    import oracle as O
    if not O.ref_available():
        pytest.skip("reference sources not present")
    R = O.ref()
    rng = np.random.default_rng(4)
    for lib in (R, S.lib()):
        for f in (lib.sptGetBestModeOrder, lib.sptGetWorstModeOrder):
            f.argtypes = [C.POINTER(C.c_uint32), C.c_uint32, C.POINTER(C.c_uint32), C.c_uint32]
    for _ in range(200):
        N = int(rng.integers(2, 9))
        nd = rng.integers(1, 6, N).astype(np.uint32)            # small sizes: many ties
        mode = int(rng.integers(0, N))
        outs = []
        for lib in (R, S.lib()):
            for f in (lib.sptGetBestModeOrder, lib.sptGetWorstModeOrder):
                o = np.zeros(N, np.uint32)
                f(o.ctypes.data_as(C.POINTER(C.c_uint32)), mode, nd.ctypes.data_as(C.POINTER(C.c_uint32)), N)
                outs.append(list(o))
        assert outs[:2] == outs[2:], (list(nd), mode, outs)
