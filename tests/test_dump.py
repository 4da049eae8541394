"""Text writers in the reference's formats (sptensor/dump.c:29-52,
matrix/dump.c:34-50, ktensor/dump.c:24-51); host only, no GPU."""
import ctypes as C

import numpy as np
import pytest

import sptol_gb300 as S

_libc = C.CDLL(None)
_libc.fopen.restype = C.c_void_p
_libc.fopen.argtypes = [C.c_char_p, C.c_char_p]
_libc.fclose.argtypes = [C.c_void_p]


def _write(tmp_path, fn):
    path = str(tmp_path / "out.txt")
    fp = _libc.fopen(path.encode(), b"w")
    rc = fn(fp)
    _libc.fclose(fp)
    assert rc == 0
    return open(path).read()


def test_dump_sparse_tensor(tmp_path):
    inds = np.array([[0, 2, 1], [3, 0, 1], [4, 4, 0]], np.uint32)
    vals = np.array([1.5, -0.25, 1e-7], np.float32)
    t = S.Tensor.from_arrays([3, 4, 5], inds, vals)
    text = _write(tmp_path, lambda fp: S.lib().sptDumpSparseTensor(t.ptr(), 1, fp))
    exp = "3\n3 4 5\n"
    for x in range(3):
        exp += "".join("%u\t" % (inds[m, x] + 1) for m in range(3)) + "%f\n" % float(vals[x])
    assert text == exp


def test_dump_matrix(tmp_path):
    a = np.array([[1.0, 2.345, -3.0], [0.004, 5.0, 6.5]], np.float32)
    m = S.Matrix.from_array(a)
    text = _write(tmp_path, lambda fp: S.lib().sptDumpMatrix(C.byref(m.s), fp))
    exp = "2 x 3 matrix\n" + "".join("".join("%.2f\t" % float(v) for v in row) + "\n" for row in a) + "\n"
    assert text == exp


def _lines(tag, fmt, xs):
    return "%s length: %d\n" % (tag, len(xs)) + "".join((fmt % x) + "\t" for x in xs) + "\n"


def test_dump_arrays(tmp_path):
    L = S.lib()
    a = np.array([7, 0, 4294967295, 12], np.uint32)
    text = _write(tmp_path, lambda fp: L.sptDumpIndexArray(a.ctypes.data_as(S.u32p), len(a), fp))
    assert text == _lines("sptIndex array", "%u", a.tolist())
    b = np.array([1 << 40, 3], np.uint64)
    text = _write(tmp_path, lambda fp: L.sptDumpNnzIndexArray(b.ctypes.data_as(S.u64p), len(b), fp))
    assert text == _lines("sptNnzIndex array", "%u", b.tolist())
    text = _write(tmp_path, lambda fp: L.sptDumpIndexArray(a.ctypes.data_as(S.u32p), 0, fp))
    assert text == "sptIndex array length: 0\n\n"


def test_dump_rank_matrix(tmp_path):
    a = np.array([[1.0, -2.345, 3.0], [0.004, 5.0, 6.5], [9, 8, 7]], np.float32)
    m = S.RankMatrix.from_array(a)
    text = _write(tmp_path, lambda fp: S.lib().sptDumpRankMatrix(C.byref(m.s), fp))
    exp = "3 x 3 matrix\n" + "".join("".join("%.2f\t" % float(v) for v in row) + "\n" for row in a) + "\n"
    assert text == exp


def _ktensor_text(nmodes, rank, ndims, fit, lam, facs):
    exp = "nmodes: %d, rank: %d\n" % (nmodes, rank) + " ".join(str(d) for d in ndims) + "\n"
    exp += "fit: %f\nlambda:\n" % fit + "".join("%f " % float(lam[m]) for m in range(nmodes))
    exp += "Factor matrices:\n"
    for f in facs:
        exp += "%d x %d matrix\n" % f.shape + "".join("".join("%.2f\t" % float(v) for v in row) + "\n"
                                                  for row in f) + "\n"
    return exp


@pytest.mark.parametrize("rank_form", [False, True])
def test_dump_kruskal(tmp_path, rank_form):
    L = S.lib()
    ndims = np.array([3, 2, 4], np.uint32)
    rank = 4
    rng = np.random.default_rng(1)
    facs = [rng.uniform(-1, 1, (int(d), rank)).astype(np.float32) for d in ndims]
    lam = np.array([1.25, -0.5, 3.0, 2.0], np.float32)
    mk = S.RankMatrix if rank_form else S.Matrix
    mats = [mk.from_array(f) for f in facs]
    P = type(C.pointer(mats[0].s))
    arr = (P * 4)(*[C.pointer(m.s) for m in mats])        # factors[nmodes] left NULL
    K = S.RankKruskalS if rank_form else S.KruskalS
    k = K(3, rank, ndims.ctypes.data_as(S.u32p), lam.ctypes.data_as(S.f32p), 0.8125, arr)
    fn = L.sptDumpRankKruskalTensor if rank_form else L.sptDumpKruskalTensor
    text = _write(tmp_path, lambda fp: fn(C.byref(k), fp))
    # one lambda entry per mode, as the reference prints
    assert text == _ktensor_text(3, rank, ndims, 0.8125, lam, facs)


def _ref_or_skip():
    import oracle as O
    if not O.ref_available():
        pytest.skip("reference sources not present")
    return O


@pytest.mark.parametrize("start", [0, 1])
def test_dump_tensor_and_matrix_equal_the_reference_bytes(tmp_path, start):
    """The writers against the reference's own sptDumpSparseTensor /
    sptDumpMatrix / sptDump*Array on the same objects, byte for byte."""
    O = _ref_or_skip()
    rng = np.random.default_rng(11 + start)
    ndims = [9, 7, 5]
    inds = np.stack([rng.integers(0, d, 40) for d in ndims]).astype(np.uint32)
    vals = (rng.standard_normal(40) * 10.0 ** rng.integers(-4, 5, 40)).astype(np.float32)
    t = S.Tensor.from_arrays(ndims, inds, vals)
    mine = _write(tmp_path, lambda fp: S.lib().sptDumpSparseTensor(t.ptr(), start, fp))
    ref_path = str(tmp_path / "ref_t.txt")
    O.ref_dump_tensor(ndims, inds, vals, start, ref_path)
    assert mine == open(ref_path).read()
    a = (rng.standard_normal((6, 11)) * 10.0 ** rng.integers(-3, 4, (6, 11))).astype(np.float32)
    m = S.Matrix.from_array(a)
    mine = _write(tmp_path, lambda fp: S.lib().sptDumpMatrix(C.byref(m.s), fp))
    O.ref_dump_matrix(a, ref_path)
    assert mine == open(ref_path).read()
    ia = rng.integers(0, 2**32, 13, dtype=np.uint64).astype(np.uint32)
    nb = rng.integers(0, 2**63, 5, dtype=np.uint64)
    L = S.lib()
    mine = _write(tmp_path, lambda fp: L.sptDumpIndexArray(ia.ctypes.data_as(S.u32p), len(ia), fp) or
                  L.sptDumpNnzIndexArray(nb.ctypes.data_as(S.u64p), len(nb), fp))
    O.ref_dump_arrays(ia, nb, ref_path)
    assert mine == open(ref_path).read()


def test_hicoo_status_equals_the_reference(tmp_path):
    """sptSparseTensorStatusHiCOO (hicoo/status.c:28-118) of one HiCOO
    container printed by both libraries, line for line: sizes, storage,
    schedule per mode, block-size statistics and the suggested parameters."""
    O = _ref_or_skip()
    R, L = O.ref(), S.lib()
    H = C.POINTER(S.HiCOOS)
    for lib in (R, L):
        lib.sptNewSparseTensorHiCOO.argtypes = [H, C.c_uint32, S.u32p, C.c_uint64, C.c_uint8, C.c_uint8, C.c_uint8]
        lib.sptSparseTensorStatusHiCOO.argtypes = [H, C.c_void_p]
        lib.sptSparseTensorStatusHiCOO.restype = None
    L.sptFreeSparseTensorHiCOO.argtypes = [H]
    rng = np.random.default_rng(5)
    ndims, nnz, sb, sk, sc = [300, 200, 100], 1000, 3, 6, 10
    h = S.HiCOOS()
    nd = (C.c_uint32 * 3)(*ndims)
    assert L.sptNewSparseTensorHiCOO(C.byref(h), 3, nd, nnz, sb, sk, sc) == 0
    sizes = []
    while sum(sizes) < nnz:
        sizes.append(int(min(rng.integers(1, 12), nnz - sum(sizes))))
    pos = 0
    assert L.sptAppendNnzIndexVector(C.byref(h.bptr), 0) == 0
    for n in sizes:
        pos += n
        assert L.sptAppendNnzIndexVector(C.byref(h.bptr), pos) == 0
    for m in range(3):
        for _ in sizes:
            assert L.sptAppendBlockIndexVector(C.byref(h.binds[m]), int(rng.integers(0, ndims[m] >> sb))) == 0
        for i in range((ndims[m] + (1 << sk) - 1) >> sk):
            for _ in range(int(rng.integers(0, 4))):
                assert L.sptAppendIndexVector(C.byref(h.kschr[m][i]), int(rng.integers(0, 50))) == 0
        h.nkiters[m] = int(rng.integers(1, 9))
    for v in (0, 17, len(sizes)):
        assert L.sptAppendNnzIndexVector(C.byref(h.kptr), v) == 0
        assert L.sptAppendNnzIndexVector(C.byref(h.cptr), v) == 0
    mine = _write(tmp_path, lambda fp: L.sptSparseTensorStatusHiCOO(C.byref(h), fp) or 0)
    ref = _write(tmp_path, lambda fp: R.sptSparseTensorStatusHiCOO(C.byref(h), fp) or 0)
    L.sptFreeSparseTensorHiCOO(C.byref(h))
    assert mine == ref and "Nnzb: Max=" in mine
