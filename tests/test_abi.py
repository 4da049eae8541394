"""The C-ABI boundary without a GPU: the library loads, exports every function
include/*.h declares, and its struct layouts equal the reference's."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

import oracle as O
import sptol_gb300 as S
from conftest import ROOT

HEADERS = [os.path.join(ROOT, "include", h) for h in ("ParTI.h", "sptgb.h")]


def declared_functions():
    names = set()
    for h in HEADERS:
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*[A-Za-z_][\w\s\*]*?\b([A-Za-z_]\w*)\s*\(", src, flags=re.M):
            name = m.group(1)
            if name in ("if", "for", "while", "return", "sizeof", "defined"):
                continue
            names.add(name)
    return sorted(names)


def test_library_loads_and_exports_every_declared_symbol():
    L = S.lib()
    names = declared_functions()
    assert len(names) > 60
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


LAYOUT_PROBE = r"""
#include <stdio.h>
#include <stddef.h>
#include <ParTI.h>
#define P(T) printf(#T " %zu\n", sizeof(T));
#define O(T, f) printf(#T "." #f " %zu\n", offsetof(T, f));
int main(void) {
  P(sptIndexVector) P(sptValueVector) P(sptNnzIndexVector) P(sptElementIndexVector)
  P(sptMatrix) P(sptRankMatrix) P(sptSparseTensor) P(sptSparseTensorHiCOO) P(sptKruskalTensor)
  O(sptSparseTensor, nnz) O(sptSparseTensor, inds) O(sptSparseTensor, values)
  O(sptMatrix, stride) O(sptMatrix, values)
  O(sptSparseTensorHiCOO, sb_bits) O(sptSparseTensorHiCOO, sc_bits) O(sptSparseTensorHiCOO, kptr)
  O(sptSparseTensorHiCOO, kschr) O(sptSparseTensorHiCOO, nkiters) O(sptSparseTensorHiCOO, cptr)
  O(sptSparseTensorHiCOO, knnzs) O(sptSparseTensorHiCOO, bptr) O(sptSparseTensorHiCOO, binds)
  O(sptSparseTensorHiCOO, einds) O(sptSparseTensorHiCOO, values)
  O(sptKruskalTensor, lambda) O(sptKruskalTensor, fit) O(sptKruskalTensor, factors)
  P(sptRankKruskalTensor) O(sptRankKruskalTensor, rank) O(sptRankKruskalTensor, lambda)
  O(sptRankKruskalTensor, fit) O(sptRankKruskalTensor, factors)
  O(sptRankMatrix, ncols) O(sptRankMatrix, cap) O(sptRankMatrix, stride) O(sptRankMatrix, values)
  P(sptMutexPool) O(sptMutexPool, nlocks) O(sptMutexPool, padsize) O(sptMutexPool, locks)
  return 0;
}
"""


def layout(include_dir, extra=()):
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "p.c")
        exe = os.path.join(d, "p")
        open(src, "w").write(LAYOUT_PROBE)
        subprocess.run(["gcc", "-std=gnu99", "-I", include_dir] + list(extra) + [src, "-o", exe], check=True,
                       capture_output=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    return dict(l.rsplit(" ", 1) for l in out.strip().splitlines())


def test_ctypes_mirror_matches_header():
    ours = layout(os.path.join(ROOT, "include"))
    assert int(ours["sptSparseTensor"]) == C.sizeof(S.SparseTensorS)
    assert int(ours["sptMatrix"]) == C.sizeof(S.MatrixS)
    assert int(ours["sptSparseTensorHiCOO"]) == C.sizeof(S.HiCOOS)
    assert int(ours["sptKruskalTensor"]) == C.sizeof(S.KruskalS)
    assert int(ours["sptSparseTensorHiCOO.bptr"]) == S.HiCOOS.bptr.offset


@pytest.mark.skipif(not os.path.isdir(os.path.join(O.REF_TREE, "include")), reason="reference headers not present")
def test_struct_layouts_equal_reference():
    ours = layout(os.path.join(ROOT, "include"))
    ref = layout(os.path.join(O.REF_TREE, "include"), ["-DPARTI_INDEX_TYPEWIDTH=32", "-DPARTI_VALUE_TYPEWIDTH=32",
                                             "-DPARTI_ELEMENT_INDEX_TYPEWIDTH=8", "-DPARTI_USE_OPENMP", "-fopenmp"])
    assert ours == ref


def test_mutex_pool_alloc_and_free():
    """sptMutexAlloc / SptMutexAllocCustom / sptMutexFree (locks.c:21-55) need no GPU."""
    L = S.lib()

    class Pool(C.Structure):
        _fields_ = [("initialized", C.c_bool), ("nlocks", C.c_uint32), ("padsize", C.c_uint32),
                    ("locks", C.c_void_p)]
    for alloc in (lambda: L.sptMutexAlloc(), lambda: L.SptMutexAllocCustom(7, 3)):
        p = alloc()
        assert p
        pool = Pool.from_address(p)
        assert pool.initialized and pool.locks
        assert (pool.nlocks, pool.padsize) in ((1024, 16), (7, 3))
        L.sptMutexFree(p)


def test_container_growth_rules_equal_the_reference():
    """Capacities after New / Append / Resize and the matrix stride and cap
    rules, side by side with the reference library built from its sources:
    objects built by either library can be grown or freed by the other."""
    import oracle as O
    if not O.ref_available():
        pytest.skip("reference sources not present")
    R, L = O.ref(), S.lib()
    for lib in (R, L):
        lib.sptNewIndexVector.argtypes = [C.POINTER(S.IndexVector), C.c_uint64, C.c_uint64]
        lib.sptAppendIndexVector.argtypes = [C.POINTER(S.IndexVector), C.c_uint32]
        lib.sptResizeIndexVector.argtypes = [C.POINTER(S.IndexVector), C.c_uint64]
        lib.sptFreeIndexVector.argtypes = [C.POINTER(S.IndexVector)]
        lib.sptNewMatrix.argtypes = [C.POINTER(S.MatrixS), C.c_uint32, C.c_uint32]
        lib.sptFreeMatrix.argtypes = [C.POINTER(S.MatrixS)]

    def trace(lib):
        out = []
        for ln, cap in ((0, 0), (3, 1), (5, 9)):
            v = S.IndexVector()
            assert lib.sptNewIndexVector(C.byref(v), ln, cap) == 0
            out.append((v.len, v.cap))
            for k in range(37):
                assert lib.sptAppendIndexVector(C.byref(v), k) == 0
                out.append((v.len, v.cap))
            for size in (1, 0, 100, 7):
                assert lib.sptResizeIndexVector(C.byref(v), size) == 0
                out.append((v.len, v.cap))
            lib.sptFreeIndexVector(C.byref(v))
        for nr, nc in ((0, 1), (5, 7), (3, 8), (2, 9), (10, 33)):
            m = S.MatrixS()
            assert lib.sptNewMatrix(C.byref(m), nr, nc) == 0
            out.append((m.nrows, m.ncols, m.cap, m.stride))
            lib.sptFreeMatrix(C.byref(m))
        return out

    assert trace(L) == trace(R)


def test_hicoo_container_shape_equals_the_reference():
    """sptNewSparseTensorHiCOO (hicoo.c:29-129) side by side with the
    reference: the same scalar fields, vector lengths and capacities, and one
    kernel-schedule vector per kernel row of every mode, so a HiCOO tensor
    made by one library can be filled or freed by the other.  (nkiters is
    left out: the reference allocates it without initialising it, this
    library zero-fills it.)"""
    import oracle as O
    if not O.ref_available():
        pytest.skip("reference sources not present")
    R, L = O.ref(), S.lib()
    H = C.POINTER(S.HiCOOS)
    u32p = C.POINTER(C.c_uint32)
    for lib in (R, L):
        lib.sptNewSparseTensorHiCOO.argtypes = [H, C.c_uint32, u32p, C.c_uint64, C.c_uint8, C.c_uint8, C.c_uint8]
        lib.sptFreeSparseTensorHiCOO.argtypes = [H]

    def shape(lib, ndims, nnz, sb, sk, sc):
        h = S.HiCOOS()
        nd = (C.c_uint32 * len(ndims))(*ndims)
        assert lib.sptNewSparseTensorHiCOO(C.byref(h), len(ndims), nd, nnz, sb, sk, sc) == 0
        N = h.nmodes
        vec = lambda v: (int(v.len), int(v.cap))
        out = {"scalars": (N, int(h.nnz), h.sb_bits, h.sk_bits, h.sc_bits),
               "ndims": [h.ndims[m] for m in range(N)], "sortorder": [h.sortorder[m] for m in range(N)],
               "kptr": vec(h.kptr), "cptr": vec(h.cptr), "bptr": vec(h.bptr), "values": vec(h.values),
               "binds": [vec(h.binds[m]) for m in range(N)], "einds": [vec(h.einds[m]) for m in range(N)],
               "kschr": [[vec(h.kschr[m][i]) for i in range((ndims[m] + (1 << sk) - 1) >> sk)] for m in range(N)]}
        lib.sptFreeSparseTensorHiCOO(C.byref(h))
        return out

    for args in (([300, 200, 100], 1000, 3, 6, 10), ([40, 30, 20, 10], 55, 2, 4, 7), ([5, 5, 5], 0, 1, 2, 2)):
        mine, ref = shape(L, *args), shape(R, *args)
        for k in ref:
            assert mine[k] == ref[k], (args, k, mine[k], ref[k])


def test_other_containers_equal_the_reference():
    """sptNewSparseTensor, sptNewRankMatrix, sptNewKruskalTensor and
    sptNewRankKruskalTensor side by side with the reference: fields, vector
    sizes, strides and which pointers start empty.  The Kruskal tensors are
    released with this library's free functions: the reference's own
    sptFreeKruskalTensor (ktensor.c:79-89) dereferences factors[i] even when
    no factors were attached, which crashes on a fresh object."""
    import oracle as O
    if not O.ref_available():
        pytest.skip("reference sources not present")
    R, L = O.ref(), S.lib()
    u32p = C.POINTER(C.c_uint32)
    T, RM = C.POINTER(S.SparseTensorS), C.POINTER(S.RankMatrixS)
    K, RK = C.POINTER(S.KruskalS), C.POINTER(S.RankKruskalS)
    for lib in (R, L):
        lib.sptNewSparseTensor.argtypes = [T, C.c_uint32, u32p]
        lib.sptFreeSparseTensor.argtypes = [T]
        lib.sptNewRankMatrix.argtypes = [RM, C.c_uint32, C.c_uint8]
        lib.sptFreeRankMatrix.argtypes = [RM]
        lib.sptNewKruskalTensor.argtypes = [K, C.c_uint32, u32p, C.c_uint32]
        lib.sptFreeKruskalTensor.argtypes = [K]
        lib.sptNewRankKruskalTensor.argtypes = [RK, C.c_uint32, u32p, C.c_uint8]
        lib.sptFreeRankKruskalTensor.argtypes = [RK]

    def shapes(lib):
        out = []
        for ndims in ([4, 5, 6], [7, 3, 2, 9]):
            N = len(ndims)
            nd = (C.c_uint32 * N)(*ndims)
            t = S.SparseTensorS()
            assert lib.sptNewSparseTensor(C.byref(t), N, nd) == 0
            out.append(("tsr", t.nmodes, int(t.nnz), [t.sortorder[m] for m in range(N)],
                        [t.ndims[m] for m in range(N)], [(int(t.inds[m].len), int(t.inds[m].cap)) for m in range(N)],
                        (int(t.values.len), int(t.values.cap))))
            lib.sptFreeSparseTensor(C.byref(t))
            for rank in (3, 16):
                k = S.KruskalS()
                assert lib.sptNewKruskalTensor(C.byref(k), N, nd, rank) == 0
                out.append(("ktsr", k.nmodes, k.rank, [k.ndims[m] for m in range(N)], k.fit, bool(k.factors)))
                L.sptFreeKruskalTensor(C.byref(k))
                rk = S.RankKruskalS()
                assert lib.sptNewRankKruskalTensor(C.byref(rk), N, nd, rank) == 0
                out.append(("rktsr", rk.nmodes, rk.rank, [rk.ndims[m] for m in range(N)], rk.fit, bool(rk.factors)))
                L.sptFreeRankKruskalTensor(C.byref(rk))
        for nr, nc in ((0, 1), (5, 7), (3, 8), (2, 9), (10, 33)):
            m = S.RankMatrixS()
            assert lib.sptNewRankMatrix(C.byref(m), nr, nc) == 0
            out.append(("rmtx", m.nrows, m.ncols, m.cap, m.stride))
            lib.sptFreeRankMatrix(C.byref(m))
        return out

    assert shapes(L) == shapes(R)
