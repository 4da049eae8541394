"""ORACLE -- test infrastructure only.

Loads the CPU restatement of ParTI!'s MTTKRP / CP-ALS path (orc.c ->
_build/liborc.so) and, where the reference sources exist, the reference
itself (_ref/libparti_ref.so, built from its own sources by the Makefile).
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline arm use this
package; the library under sptol_gb300/ never imports it.

Arrays: coordinates are [N, nnz] uint32, values [nnz] float32, factor
matrices float32 [ndims[m], stride] with stride = rank rounded up to 8.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORC_PATH = os.path.join(HERE, "_build", "liborc.so")
REF_PATH = os.path.join(HERE, "_ref", "libparti_ref.so")
# The staged copy of the reference sources that the `ref` target compiles
# (made by `make stage` from the tree named by SPTGB_REFERENCE; git-ignored).
REF_TREE = os.path.join(HERE, "_ref", "tree")

u32p = C.POINTER(C.c_uint32)
u64p = C.POINTER(C.c_uint64)
f32p = C.POINTER(C.c_float)
f64p = C.POINTER(C.c_double)
u8p = C.POINTER(C.c_uint8)

_ORC = None
_REF = None


def build(with_ref=None):
    """Builds liborc.so, and the reference library when its sources are
    staged.  With SPTGB_REFERENCE set to a reference checkout, the sources are
    (re)staged from it first."""
    subprocess.run(["make", "-s", "-C", HERE, "orc"], check=True)
    if os.environ.get("SPTGB_REFERENCE"):
        stage_reference()
    if with_ref is None:
        with_ref = os.path.isdir(os.path.join(REF_TREE, "src"))
    if with_ref:
        if not os.path.isdir(os.path.join(REF_TREE, "src")):
            raise RuntimeError("no staged reference sources under %s: set SPTGB_REFERENCE to a reference "
                               "checkout and call oracle.stage_reference()" % REF_TREE)
        subprocess.run(["make", "-s", "-j%d" % min(16, os.cpu_count() or 4), "-C", HERE, "ref"], check=True)


def stage_reference():
    """Copies the reference sources the `ref` target needs from the checkout
    named by SPTGB_REFERENCE into oracle/_ref/tree (git-ignored)."""
    src = os.environ.get("SPTGB_REFERENCE")
    if not src:
        raise RuntimeError("SPTGB_REFERENCE is not set: it must name a reference (ParTI!) source checkout")
    subprocess.run(["make", "-s", "-C", HERE, "stage", "REF=" + src], check=True)


def stride_of(rank):
    return ((rank - 1) // 8 + 1) * 8


class HiCOOOut(C.Structure):
    _fields_ = [("nb", C.c_uint64), ("nk", C.c_uint64), ("ncptr", C.c_uint64), ("max_nnzb", C.c_uint64),
                ("bptr", u64p), ("kptr", u64p), ("cptr", u64p), ("binds", u32p), ("einds", u8p),
                ("nkiters", u32p), ("kschr_len", u32p), ("kschr", u32p)]


def orc():
    global _ORC
    if _ORC is None:
        if not os.path.exists(ORC_PATH):
            build(with_ref=False)
        L = C.CDLL(ORC_PATH)
        L.orc_sort_lex.argtypes = [C.c_uint32, C.c_uint64, C.POINTER(u32p), u32p, u64p]
        L.orc_sort_hicoo.argtypes = [C.c_uint32, C.c_uint64, C.POINTER(u32p), C.c_int, u64p]
        L.orc_hicoo_build.argtypes = [C.c_uint32, u32p, C.c_uint64, C.POINTER(u32p), C.c_int, C.c_int,
                                      C.POINTER(HiCOOOut)]
        mt = [C.c_uint32, C.c_uint64, C.POINTER(u32p), f32p, C.POINTER(f32p), C.c_uint32, C.c_uint32, u32p,
              C.c_uint32, C.c_uint32]
        L.orc_mttkrp_f32.argtypes = mt + [f32p]
        L.orc_mttkrp_f64.argtypes = mt + [f64p]
        L.orc_omp_mttkrp_f64.argtypes = mt + [f64p, C.c_int]
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_sort_keyed_check.argtypes = [C.c_uint32, C.c_uint64, C.POINTER(u32p), u32p, C.c_int]
        L.orc_ttm.restype = C.c_uint64
        L.orc_ttm.argtypes = [C.c_uint32, C.c_uint64, C.POINTER(u32p), f32p, C.c_uint32, f32p, C.c_uint32,
                              C.c_uint32, C.c_uint32, C.POINTER(u32p), f32p]
        L.orc_load_tns.argtypes = [C.c_char_p, C.c_uint32, u32p, u32p, C.c_uint64, C.POINTER(u32p), f32p, u64p]
        L.orc_omp_mttkrp_reduce.argtypes = mt + [f32p, C.c_int, f32p]
        L.orc_mttkrp_hicoo_f32.argtypes = [C.c_uint32, C.c_uint64, u64p, C.POINTER(u32p), C.POINTER(u8p), f32p,
                                           C.c_int, C.POINTER(f32p), C.c_uint32, C.c_uint32, u32p, C.c_uint32,
                                           C.c_uint32, f32p]
        L.orc_omp_mttkrp_hicoo_reduce.argtypes = [C.c_uint32, u64p, C.POINTER(u32p), C.POINTER(u8p), f32p, C.c_int,
                                                  u64p, C.c_uint32, u64p, u32p, C.c_uint32, C.POINTER(f32p),
                                                  C.c_uint32, C.c_uint32, u32p, C.c_uint32, C.c_uint32, f32p, C.c_int,
                                                  f32p]
        L.orc_cpd_als_f64.argtypes = [C.c_uint32, u32p, C.c_uint64, C.POINTER(u32p), f32p, C.c_uint32, C.c_uint32,
                                      C.c_double, C.POINTER(f32p), C.c_uint32, f32p, f64p, u32p]
        L.orc_fit_exact.argtypes = [C.c_uint32, u32p, C.c_uint64, C.POINTER(u32p), f32p, C.c_uint32,
                                    C.POINTER(f32p), C.c_uint32, f32p]
        L.orc_fit_exact.restype = C.c_double
        _ORC = L
    return _ORC


def ref_available():
    return os.path.exists(REF_PATH) or os.path.isdir(os.path.join(REF_TREE, "src"))


def ref_loadable():
    """True when the reference library is already built and loads in this
    process (a build for another machine's architecture does not)."""
    if not os.path.exists(REF_PATH):
        return False
    try:
        ref()
        return True
    except OSError:
        return False


def ref():
    """The reference library with its LAPACK calls forwarded to scipy's."""
    global _REF
    if _REF is None:
        if not os.path.exists(REF_PATH):
            build(with_ref=True)
        L = C.CDLL(REF_PATH)
        import scipy.linalg.cython_blas as cb
        import scipy.linalg.cython_lapack as cl
        get = C.pythonapi.PyCapsule_GetPointer
        get.restype = C.c_void_p
        get.argtypes = [C.py_object, C.c_char_p]
        gname = C.pythonapi.PyCapsule_GetName
        gname.restype = C.c_char_p
        gname.argtypes = [C.py_object]

        def fp(mod, name):
            cap = mod.__pyx_capi__[name]
            return get(cap, gname(cap))

        L.ref_set_lapack.argtypes = [C.c_void_p] * 4
        L.ref_set_lapack(fp(cb, "ssyrk"), fp(cl, "spotrf"), fp(cl, "spotrs"), fp(cl, "sgesv"))
        L.ref_sort.argtypes = [C.c_uint32, u32p, C.c_uint64, C.POINTER(u32p), f32p, u32p]
        L.ref_mttkrp.argtypes = [C.c_uint32, u32p, C.c_uint64, C.POINTER(u32p), f32p, C.c_uint32, C.POINTER(f32p),
                                 C.c_uint32, u32p, C.c_uint32, f32p, C.c_int, C.c_int, C.c_int, f64p]
        L.ref_hicoo.argtypes = [C.c_uint32, u32p, C.c_uint64, C.POINTER(u32p), f32p, C.c_int, C.c_int,
                                C.POINTER(HiCOOOut)]
        L.ref_mttkrp_hicoo.argtypes = [C.c_uint32, u32p, C.c_uint64, C.POINTER(u32p), f32p, C.c_int, C.c_int,
                                       C.c_uint32, C.POINTER(f32p), C.c_uint32, u32p, C.c_uint32, f32p]
        L.ref_cpd_trace.argtypes = [C.c_uint32, u32p, C.c_uint64, C.POINTER(u32p), f32p, C.c_uint32, C.c_uint32,
                                    C.POINTER(f32p), C.c_uint32, C.POINTER(f32p), f32p, f64p, C.POINTER(f32p), f32p,
                                    f64p]
        L.ref_ttm.restype = C.c_uint64
        L.ref_ttm.argtypes = [C.c_uint32, u32p, C.c_uint64, C.POINTER(u32p), f32p, C.c_uint32, f32p, C.c_uint32,
                              C.c_uint32, C.POINTER(u32p), f32p, u32p]
        L.ref_load_tns.argtypes = [C.c_char_p, C.c_uint32, u32p, u32p, C.c_uint64, C.POINTER(u32p), f32p, u64p]
        L.ref_dotmul_triangle.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32, C.POINTER(f32p), C.c_uint32, f32p]
        L.ref_colnorm.argtypes = [C.c_int, C.c_uint32, C.c_uint32, f32p, C.c_uint32, f32p]
        L.ref_kruskal_normsq.restype = C.c_double
        L.ref_kruskal_normsq.argtypes = [C.c_uint32, C.c_uint32, C.POINTER(f32p), C.c_uint32, f32p]
        L.ref_solve_normals.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32, C.POINTER(f32p), C.c_uint32, C.c_uint32,
                                        f32p]
        L.ref_dump_tensor.argtypes = [C.c_uint32, u32p, C.c_uint64, C.POINTER(u32p), f32p, C.c_uint32, C.c_char_p]
        L.ref_dump_matrix.argtypes = [C.c_uint32, C.c_uint32, f32p, C.c_uint32, C.c_char_p]
        L.ref_dump_arrays.argtypes = [u32p, C.c_uint64, u64p, C.c_uint64, C.c_char_p]
        L.ref_session_open.restype = C.c_void_p
        L.ref_session_open.argtypes = [C.c_void_p, C.c_uint32, C.c_uint64, C.c_int]
        L.ref_session_close.argtypes = [C.c_void_p]
        L.ref_session_nnz.restype = C.c_uint64
        L.ref_session_nnz.argtypes = [C.c_void_p]
        L.ref_session_ndims.argtypes = [C.c_void_p, u32p]
        L.ref_session_mttkrp.restype = C.c_double
        L.ref_session_mttkrp.argtypes = [C.c_void_p, C.c_int, C.c_uint32, f32p]
        L.ref_session_cuda_mttkrp.restype = C.c_double
        L.ref_session_cuda_mttkrp.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, f32p]
        L.ref_session_cpd.restype = C.c_double
        L.ref_session_cpd.argtypes = [C.c_void_p, C.c_uint32, C.c_int, f32p, f64p]
        L.ref_omp_cpd.restype = C.c_double
        L.ref_omp_cpd.argtypes = [C.c_uint32, u32p, C.c_uint64, C.POINTER(u32p), f32p, C.c_uint32, C.c_uint32,
                                  C.POINTER(f32p), C.c_uint32, C.c_int, f32p, f64p]
        L.ref_kruskal_inner.restype = C.c_double
        L.ref_kruskal_inner.argtypes = [C.c_uint32, C.c_uint32, u32p, C.POINTER(f32p), f32p, C.c_uint32, f32p]
        _REF = L
    return _REF


# ----------------------------------------------------------------- helpers --
def _u32(a):
    a = np.ascontiguousarray(a, dtype=np.uint32)
    return a, a.ctypes.data_as(u32p)


def _rows(arrs, ptype, dtype):
    arrs = [np.ascontiguousarray(a, dtype=dtype) for a in arrs]
    p = (ptype * len(arrs))(*[a.ctypes.data_as(ptype) for a in arrs])
    return arrs, p


def _check_mats(mats, ndims, stride):
    """The C routines read ndims[m] rows of `stride` floats from each factor."""
    for m, a in enumerate(mats):
        a = np.asarray(a)
        if a.ndim != 2 or a.shape[1] < stride or a.shape[0] < ndims[m]:
            raise ValueError("factor %d must have ndims[%d] rows of at least %d (the padded stride) columns"
                             % (m, m, stride))


def _default_order(N, mode):
    return [mode] + [(mode + i) % N for i in range(1, N)]


def sort_lex(inds, order=None):
    """Permutation sorting the nonzeros lexicographically in `order`."""
    N, n = inds.shape
    order = list(range(N)) if order is None else order
    keep, ip = _rows(list(inds), u32p, np.uint32)
    o, op = _u32(order)
    perm = np.zeros(n, np.uint64)
    orc().orc_sort_lex(N, n, ip, op, perm.ctypes.data_as(u64p))
    return perm.astype(np.int64)


def sort_keyed_check(inds, order=None, sk_bits=None):
    """True when the packed-key sort (used from 2^20 nonzeros up) and the
    comparison merge sort give one permutation: lexicographic in `order`, or
    the HiCOO order of kernel size 2^sk_bits when order is None."""
    N, n = inds.shape
    keep, ip = _rows(list(inds), u32p, np.uint32)
    if order is not None:
        o, op = _u32(order)
        return orc().orc_sort_keyed_check(N, n, ip, op, 0) == 0
    return orc().orc_sort_keyed_check(N, n, ip, None, sk_bits) == 0


def sort_hicoo(inds, sk_bits):
    N, n = inds.shape
    keep, ip = _rows(list(inds), u32p, np.uint32)
    perm = np.zeros(n, np.uint64)
    orc().orc_sort_hicoo(N, n, ip, sk_bits, perm.ctypes.data_as(u64p))
    return perm.astype(np.int64)


def _hicoo_alloc(N, n, ndims, sk_bits):
    nrows = sum((d + (1 << sk_bits) - 1) >> sk_bits for d in ndims)
    bufs = {
        "bptr": np.zeros(n + 1, np.uint64), "kptr": np.zeros(n + 1, np.uint64),
        "cptr": np.zeros(2 * n + 2, np.uint64), "binds": np.zeros(N * n, np.uint32),
        "einds": np.zeros(N * n, np.uint8), "nkiters": np.zeros(N, np.uint32),
        "kschr_len": np.zeros(nrows, np.uint32), "kschr": np.zeros(N * n, np.uint32),
    }
    o = HiCOOOut()
    for k in ("bptr", "kptr", "cptr"):
        setattr(o, k, bufs[k].ctypes.data_as(u64p))
    for k in ("binds", "nkiters", "kschr_len", "kschr"):
        setattr(o, k, bufs[k].ctypes.data_as(u32p))
    o.einds = bufs["einds"].ctypes.data_as(u8p)
    return bufs, o


def _hicoo_trim(bufs, o, N, n):
    nb, nk = int(o.nb), int(o.nk)
    return {
        "kptr": bufs["kptr"][: nk + 1].copy(), "cptr": bufs["cptr"][: int(o.ncptr)].copy(),
        "bptr": bufs["bptr"][: nb + 1].copy(), "binds": bufs["binds"][: N * nb].reshape(N, nb).copy(),
        "einds": bufs["einds"].reshape(N, n).copy(), "nkiters": bufs["nkiters"].copy(),
        "kschr_len": bufs["kschr_len"].copy(), "kschr": bufs["kschr"][: N * nk].copy(),
        "max_nnzb": int(o.max_nnzb),
    }


def hicoo_build(ndims, inds_sorted, sb_bits, sk_bits):
    """HiCOO arrays from a COO already in HiCOO order (orc_sort_hicoo)."""
    N, n = inds_sorted.shape
    keep, ip = _rows(list(inds_sorted), u32p, np.uint32)
    nd, ndp = _u32(ndims)
    bufs, o = _hicoo_alloc(N, n, ndims, sk_bits)
    orc().orc_hicoo_build(N, ndp, n, ip, sb_bits, sk_bits, C.byref(o))
    return _hicoo_trim(bufs, o, N, n)


def mttkrp(ndims, inds, vals, mats, rank, mode, order=None, precision="f32", tk=None):
    """Sequential FP32 (reference order), FP64, FP64 over threads
    ("f64_omp"), or OpenMP-reduce FP32 MTTKRP."""
    N, n = inds.shape
    order = _default_order(N, mode) if order is None else order
    stride = stride_of(rank)
    _check_mats(mats, ndims, stride)
    keep, ip = _rows(list(inds), u32p, np.uint32)
    mkeep, mp = _rows(mats, f32p, np.float32)
    v = np.ascontiguousarray(vals, np.float32)
    o, op = _u32(order)
    rows = ndims[mode]
    L = orc()
    args = [N, n, ip, v.ctypes.data_as(f32p), mp, stride, rank, op, mode, rows]
    if precision == "f64":
        out = np.zeros((rows, stride), np.float64)
        L.orc_mttkrp_f64(*args, out.ctypes.data_as(f64p))
    elif precision == "f64_omp":
        out = np.zeros((rows, stride), np.float64)
        L.orc_omp_mttkrp_f64(*args, out.ctypes.data_as(f64p), tk or os.cpu_count())
    elif precision == "omp":
        tk = tk or os.cpu_count()
        out = np.zeros((rows, stride), np.float32)
        copies = np.zeros(tk * rows * stride, np.float32)
        L.orc_omp_mttkrp_reduce(*args, out.ctypes.data_as(f32p), tk, copies.ctypes.data_as(f32p))
    else:
        out = np.zeros((rows, stride), np.float32)
        L.orc_mttkrp_f32(*args, out.ctypes.data_as(f32p))
    return out[:, :rank]


def kschr_rows(h, ndims, sk_bits, mode):
    """Kernel ids of every kernel row of `mode`, from either HiCOO layout:
    nested lists (sptSparseTensorHiCOO.kschr as read back from the library)
    or the flattened kschr_len / kschr arrays of hicoo_build."""
    if "kschr_len" not in h:
        return [np.asarray(r, np.uint32) for r in h["kschr"][mode]]
    rows = [(d + (1 << sk_bits) - 1) >> sk_bits for d in ndims]
    r0 = sum(rows[:mode])
    lens = h["kschr_len"].astype(np.int64)
    start = int(lens[:r0].sum())
    out = []
    for i in range(rows[mode]):
        ln = int(lens[r0 + i])
        out.append(h["kschr"][start:start + ln].astype(np.uint32))
        start += ln
    return out


def omp_mttkrp_hicoo_reduce(ndims, h, vals, sb_bits, mats, rank, mode, tk, ks_rows, order=None, copies=None):
    """3-D HiCOO MTTKRP as sptOmpMTTKRPHiCOO_MatrixTiling_Scheduled_Reduce
    (the kernel rows of `mode`, ks_rows = kschr_rows(...), per-thread output
    copies)."""
    N = len(ndims)
    order = _default_order(N, mode) if order is None else order
    stride = stride_of(rank)
    bk, bp = _rows(list(h["binds"]), u32p, np.uint32)
    ek, ep = _rows(list(h["einds"]), u8p, np.uint8)
    _check_mats(mats, ndims, stride)
    mkeep, mp = _rows(mats, f32p, np.float32)
    v = np.ascontiguousarray(vals, np.float32)
    bptr = np.ascontiguousarray(h["bptr"], np.uint64)
    kptr = np.ascontiguousarray(h["kptr"], np.uint64)
    rows_k = ks_rows
    ks_off = np.zeros(len(rows_k) + 1, np.uint64)
    ks_off[1:] = np.cumsum([len(r) for r in rows_k])
    ks_ids = np.ascontiguousarray(np.concatenate(rows_k) if len(rows_k) else np.zeros(0), np.uint32)
    o, op = _u32(order)
    out = np.zeros((ndims[mode], stride), np.float32)
    if copies is None or copies.size < tk * ndims[mode] * stride:
        copies = np.zeros(tk * ndims[mode] * stride, np.float32)
    orc().orc_omp_mttkrp_hicoo_reduce(N, bptr.ctypes.data_as(u64p), bp, ep, v.ctypes.data_as(f32p), sb_bits,
                                      kptr.ctypes.data_as(u64p), len(rows_k), ks_off.ctypes.data_as(u64p),
                                      ks_ids.ctypes.data_as(u32p), max((len(r) for r in rows_k), default=0), mp,
                                      stride, rank, op, mode,
                                      ndims[mode], out.ctypes.data_as(f32p), tk, copies.ctypes.data_as(f32p))
    return out[:, :rank]


def mttkrp_hicoo(ndims, h, vals, sb_bits, mats, rank, mode, order=None):
    N = len(ndims)
    order = _default_order(N, mode) if order is None else order
    stride = stride_of(rank)
    bk, bp = _rows(list(h["binds"]), u32p, np.uint32)
    ek, ep = _rows(list(h["einds"]), u8p, np.uint8)
    _check_mats(mats, ndims, stride)
    mkeep, mp = _rows(mats, f32p, np.float32)
    v = np.ascontiguousarray(vals, np.float32)
    bptr = np.ascontiguousarray(h["bptr"], np.uint64)
    o, op = _u32(order)
    out = np.zeros((ndims[mode], stride), np.float32)
    orc().orc_mttkrp_hicoo_f32(N, len(bptr) - 1, bptr.ctypes.data_as(u64p), bp, ep, v.ctypes.data_as(f32p), sb_bits,
                               mp, stride, rank, op, mode, ndims[mode], out.ctypes.data_as(f32p))
    return out[:, :rank]


def cpd_als(ndims, inds, vals, rank, niters, tol, init, tk=1):
    """FP64 CP-ALS restatement; init: list of [ndims[m], rank] float arrays.
    tk > 1 runs the MTTKRP, Gram and row solves on tk threads (per-thread
    partial sums added in thread order)."""
    N, n = inds.shape
    stride = stride_of(rank)
    facs = []
    for a in init:
        f = np.zeros((a.shape[0], stride), np.float32)
        f[:, :rank] = a
        facs.append(f)
    keep, ip = _rows(list(inds), u32p, np.uint32)
    fkeep, fp = _rows(facs, f32p, np.float32)
    nd, ndp = _u32(ndims)
    v = np.ascontiguousarray(vals, np.float32)
    lam = np.zeros(rank, np.float32)
    fits = np.full(niters, np.nan)
    done = C.c_uint32()
    orc().orc_set_threads(int(tk))
    try:
        orc().orc_cpd_als_f64(N, ndp, n, ip, v.ctypes.data_as(f32p), rank, niters, tol, fp, stride,
                              lam.ctypes.data_as(f32p), fits.ctypes.data_as(f64p), C.byref(done))
    finally:
        orc().orc_set_threads(1)
    return [f[:, :rank].copy() for f in fkeep], lam, fits, int(done.value)


def fit_exact(ndims, inds, vals, factors, lam):
    N, n = inds.shape
    rank = factors[0].shape[1]
    stride = stride_of(rank)
    facs = []
    for a in factors:
        f = np.zeros((a.shape[0], stride), np.float32)
        f[:, :rank] = a
        facs.append(f)
    keep, ip = _rows(list(inds), u32p, np.uint32)
    fkeep, fp = _rows(facs, f32p, np.float32)
    nd, ndp = _u32(ndims)
    v = np.ascontiguousarray(vals, np.float32)
    l = np.ascontiguousarray(lam, np.float32)
    return float(orc().orc_fit_exact(N, ndp, n, ip, v.ctypes.data_as(f32p), rank, fp, stride,
                                     l.ctypes.data_as(f32p)))


# ------------------------------------------------------- the reference --
def ref_sort(ndims, inds, vals, order=None):
    N, n = inds.shape
    ik, ip = _rows([r.copy() for r in inds], u32p, np.uint32)
    v = np.ascontiguousarray(vals, np.float32).copy()
    nd, ndp = _u32(ndims)
    op = None
    if order is not None:
        o, op = _u32(order)
    ref().ref_sort(N, ndp, n, ip, v.ctypes.data_as(f32p), op)
    return np.stack(ik), v


def ref_mttkrp(ndims, inds, vals, mats, rank, mode, order=None, which=0, tk=1, reps=0):
    N, n = inds.shape
    order = _default_order(N, mode) if order is None else order
    stride = stride_of(rank)
    ik, ip = _rows(list(inds), u32p, np.uint32)
    mk, mp = _rows(mats, f32p, np.float32)
    v = np.ascontiguousarray(vals, np.float32)
    nd, ndp = _u32(ndims)
    o, op = _u32(order)
    out = np.zeros((ndims[mode], stride), np.float32)
    secs = C.c_double()
    with quiet_stdout():   # the sequential sptMTTKRP prints its time
        r = ref().ref_mttkrp(N, ndp, n, ip, v.ctypes.data_as(f32p), rank, mp, stride, op, mode,
                             out.ctypes.data_as(f32p), which, tk, reps, C.byref(secs))
    assert r == 0
    return out[:, :rank], secs.value


def ref_hicoo(ndims, inds, vals, sb_bits, sk_bits):
    N, n = inds.shape
    ik, ip = _rows([r.copy() for r in inds], u32p, np.uint32)
    v = np.ascontiguousarray(vals, np.float32).copy()
    nd, ndp = _u32(ndims)
    bufs, o = _hicoo_alloc(N, n, ndims, sk_bits)
    ref().ref_hicoo(N, ndp, n, ip, v.ctypes.data_as(f32p), sb_bits, sk_bits, C.byref(o))
    return np.stack(ik), v, _hicoo_trim(bufs, o, N, n)


def ref_mttkrp_hicoo(ndims, inds, vals, sb_bits, sk_bits, mats, rank, mode, order=None):
    N, n = inds.shape
    order = _default_order(N, mode) if order is None else order
    stride = stride_of(rank)
    ik, ip = _rows([r.copy() for r in inds], u32p, np.uint32)
    mk, mp = _rows(mats, f32p, np.float32)
    v = np.ascontiguousarray(vals, np.float32)
    nd, ndp = _u32(ndims)
    o, op = _u32(order)
    out = np.zeros((ndims[mode], stride), np.float32)
    ref().ref_mttkrp_hicoo(N, ndp, n, ip, v.ctypes.data_as(f32p), sb_bits, sk_bits, rank, mp, stride, op, mode,
                           out.ctypes.data_as(f32p))
    return out[:, :rank]


def ref_cpd_trace(ndims, inds, vals, rank, niters, init):
    N, n = inds.shape
    stride = stride_of(rank)

    def padded():
        out = []
        for a in init:
            f = np.zeros((a.shape[0], stride), np.float32)
            f[:, :rank] = a
            out.append(f)
        return out

    ik, ip = _rows(list(inds), u32p, np.uint32)
    v = np.ascontiguousarray(vals, np.float32)
    nd, ndp = _u32(ndims)
    ink, inp = _rows(padded(), f32p, np.float32)
    lk, lp = _rows(padded(), f32p, np.float32)
    sk, sp = _rows(padded(), f32p, np.float32)
    lam_loop = np.zeros(rank, np.float32)
    lam_step = np.zeros(rank, np.float32)
    fits = np.zeros(niters)
    step_fit = C.c_double()
    ref().ref_cpd_trace(N, ndp, n, ip, v.ctypes.data_as(f32p), rank, niters, inp, stride, lp,
                        lam_loop.ctypes.data_as(f32p), fits.ctypes.data_as(f64p), sp, lam_step.ctypes.data_as(f32p),
                        C.byref(step_fit))
    return {
        "loop_factors": [f[:, :rank].copy() for f in lk], "loop_lambda": lam_loop, "fits": fits,
        "step_factors": [f[:, :rank].copy() for f in sk], "step_lambda": lam_step, "step_fit": step_fit.value,
    }


def load_tns(path, start_index=1):
    """The reference's text reader (load.c + collect.c) restated: returns
    (ndims, inds [N, nnz], vals) or raises ValueError with the reader's code."""
    size = os.path.getsize(path)
    cap = size // 2 + 2
    N = C.c_uint32()
    nd = (C.c_uint32 * 8)()
    arrs = [np.zeros(cap, np.uint32) for _ in range(8)]
    ptrs = (u32p * 8)(*[a.ctypes.data_as(u32p) for a in arrs])
    vals = np.zeros(cap, np.float32)
    nnz = C.c_uint64()
    rc = orc().orc_load_tns(path.encode(), start_index, C.byref(N), nd, cap, ptrs, vals.ctypes.data_as(f32p),
                            C.byref(nnz))
    if rc != 0:
        raise ValueError("reader returned %d" % rc)
    n = int(nnz.value)
    return [int(nd[m]) for m in range(N.value)], np.stack([a[:n] for a in arrs[: N.value]]), vals[:n].copy()


def _read_tns(fn, path, start_index):
    size = os.path.getsize(path)
    cap = size // 2 + 2
    N = C.c_uint32()
    nd = (C.c_uint32 * 8)()
    arrs = [np.zeros(cap, np.uint32) for _ in range(8)]
    ptrs = (u32p * 8)(*[a.ctypes.data_as(u32p) for a in arrs])
    vals = np.zeros(cap, np.float32)
    nnz = C.c_uint64()
    rc = fn(path.encode(), start_index, C.byref(N), nd, cap, ptrs, vals.ctypes.data_as(f32p), C.byref(nnz))
    if rc != 0:
        raise ValueError("reader returned %d" % rc)
    n = int(nnz.value)
    return [int(nd[m]) for m in range(N.value)], np.stack([a[:n] for a in arrs[: N.value]]), vals[:n].copy()


def _padded(a, stride):
    f = np.zeros((a.shape[0], stride), np.float32)
    f[:, : a.shape[1]] = a
    return f


def ref_dotmul_triangle(grams, mode):
    """sptMatrixDotMulSeqTriangle on R x R Grams; returns the R x R result."""
    R = grams[0].shape[1]
    st = stride_of(R)
    gk, gp = _rows([_padded(g, st) for g in grams], f32p, np.float32)
    out = np.zeros((R, st), np.float32)
    assert ref().ref_dotmul_triangle(len(grams), mode, R, gp, st, out.ctypes.data_as(f32p)) == 0
    return out[:, :R]


def ref_colnorm(A, use_max):
    """sptMatrix2Norm (use_max False) or sptMatrixMaxNorm: (normalised A, lambda)."""
    n, R = A.shape
    st = stride_of(R)
    a = _padded(A, st)
    lam = np.zeros(R, np.float32)
    assert ref().ref_colnorm(int(use_max), n, R, a.ctypes.data_as(f32p), st, lam.ctypes.data_as(f32p)) == 0
    return a[:, :R], lam


def ref_solve_normals(grams, mode, rhs):
    """sptMatrixSolveNormals: X with X G = rhs (G the Hadamard of the other Grams)."""
    R = grams[0].shape[1]
    st = stride_of(R)
    gk, gp = _rows([_padded(g, st) for g in grams], f32p, np.float32)
    b = _padded(rhs, st)
    assert ref().ref_solve_normals(len(grams), mode, R, gp, st, rhs.shape[0], b.ctypes.data_as(f32p)) == 0
    return b[:, :R]


def ref_kruskal_normsq(ata, lam):
    R = ata[0].shape[1]
    st = stride_of(R)
    ak, ap = _rows([_padded(g, st) for g in ata], f32p, np.float32)
    return ref().ref_kruskal_normsq(len(ata), R, ap, st, np.ascontiguousarray(lam, np.float32).ctypes.data_as(f32p))


def ref_kruskal_inner(facs, mout, lam):
    R = facs[0].shape[1]
    st = stride_of(R)
    fk, fp = _rows([_padded(f, st) for f in facs], f32p, np.float32)
    nd, ndp = _u32([f.shape[0] for f in facs])
    mo = _padded(mout, st)
    return ref().ref_kruskal_inner(len(facs), R, ndp, fp, mo.ctypes.data_as(f32p), st,
                                   np.ascontiguousarray(lam, np.float32).ctypes.data_as(f32p))


def ref_dump_tensor(ndims, inds, vals, start_index, path):
    ik, ip = _rows(list(inds), u32p, np.uint32)
    v = np.ascontiguousarray(vals, np.float32)
    nd, ndp = _u32(ndims)
    assert ref().ref_dump_tensor(len(ndims), ndp, inds.shape[1], ip, v.ctypes.data_as(f32p), start_index,
                                 path.encode()) == 0


def ref_dump_matrix(a, path):
    n, R = a.shape
    st = stride_of(R)
    p = _padded(a, st)
    assert ref().ref_dump_matrix(n, R, p.ctypes.data_as(f32p), st, path.encode()) == 0


def ref_dump_arrays(a, b, path):
    a = np.ascontiguousarray(a, np.uint32)
    b = np.ascontiguousarray(b, np.uint64)
    assert ref().ref_dump_arrays(a.ctypes.data_as(u32p), len(a), b.ctypes.data_as(u64p), len(b), path.encode()) == 0


def ref_load_tns(path, start_index=1):
    """The reference's own sptLoadSparseTensor (built from its sources), same
    return convention as load_tns."""
    return _read_tns(ref().ref_load_tns, path, start_index)


def ttm(ndims, inds, vals, U, mode, sort=True):
    """Sparse tensor times matrix as the reference computes it: the tensor
    sorted with `mode` last (sort=False: taken in the given order, as the
    reference does when the tensor's sortorder already says so), a dense
    fiber per run of equal coordinates in the other modes.  Returns (fiber
    coordinates [N, nfib] (row `mode` zero), Y [nfib, ncols], the
    permutation applied)."""
    N, n = inds.shape
    order = [m for m in range(N) if m != mode] + [mode]
    p = sort_lex(inds, order) if sort else np.arange(n)
    si = np.ascontiguousarray(inds[:, p])
    sv = np.ascontiguousarray(vals[p], np.float32)
    U = np.asarray(U, np.float32)
    ncols = U.shape[1]
    ustride = stride_of(ncols)
    Up = np.zeros((U.shape[0], ustride), np.float32)
    Up[:, :ncols] = U
    keep, ip = _rows(list(si), u32p, np.uint32)
    fib = [np.zeros(max(n, 1), np.uint32) for _ in range(N)]
    fp = (u32p * N)(*[f.ctypes.data_as(u32p) for f in fib])
    Y = np.zeros((max(n, 1), ustride), np.float32)
    nf = orc().orc_ttm(N, n, ip, sv.ctypes.data_as(f32p), mode, Up.ctypes.data_as(f32p), ustride, ncols, ustride,
                       fp, Y.ctypes.data_as(f32p))
    return np.stack([f[:nf] for f in fib]), Y[:nf, :ncols], p


def ref_ttm(ndims, inds, vals, U, mode):
    """The reference's own sptSparseTensorMulMatrix (tensor marked unsorted).
    Returns (fiber coordinates, Y [nfib, ncols], sorted inds, sorted vals)."""
    N, n = inds.shape
    si = [np.ascontiguousarray(a, np.uint32).copy() for a in inds]
    sp = (u32p * N)(*[a.ctypes.data_as(u32p) for a in si])
    sv = np.ascontiguousarray(vals, np.float32).copy()
    U = np.ascontiguousarray(U, np.float32)
    ncols = U.shape[1]
    fib = [np.zeros(max(n, 1), np.uint32) for _ in range(N)]
    fp = (u32p * N)(*[f.ctypes.data_as(u32p) for f in fib])
    Y = np.zeros((max(n, 1), stride_of(ncols)), np.float32)
    ys = C.c_uint32()
    nd, ndp = _u32(ndims)
    nf = ref().ref_ttm(N, ndp, n, sp, sv.ctypes.data_as(f32p), mode, U.ctypes.data_as(f32p), U.shape[0], ncols, fp,
                       Y.ctypes.data_as(f32p), C.byref(ys))
    return np.stack([f[:nf] for f in fib]), Y[:nf, :ncols], np.stack(si), sv


# ------------------------------------------------- reference timing sessions --
class quiet_stdout:
    """Sends the C library's stdout (the reference prints per-iteration
    progress lines) to stderr for the duration of a call, so that a caller's
    own stdout stays machine-readable."""

    def __enter__(self):
        import sys
        sys.stdout.flush()
        self._saved = os.dup(1)
        os.dup2(2, 1)
        return self

    def __exit__(self, *exc):
        import sys
        sys.stdout.flush()
        C.CDLL(None).fflush(None)   # the C library's buffered stdout, while fd 1 still points at stderr
        os.dup2(self._saved, 1)
        os.close(self._saved)
        return False


class capture_stdout:
    """Collects what the C library writes to stdout during a call (the
    reference prints its own phase timings) into .text."""

    def __enter__(self):
        import sys
        import tempfile
        sys.stdout.flush()
        self._f = tempfile.TemporaryFile(mode="w+b")
        self._saved = os.dup(1)
        os.dup2(self._f.fileno(), 1)
        self.text = ""
        return self

    def __exit__(self, *exc):
        C.CDLL(None).fflush(None)
        os.dup2(self._saved, 1)
        os.close(self._saved)
        self._f.seek(0)
        self.text = self._f.read().decode(errors="replace")
        self._f.close()
        return False


class RefSession:
    """The reference's own CPU MTTKRP / CP-ALS on a tensor held in the
    reference's containers (ref_harness.c, ref_session_*): the tensor is made
    by the library's seeded generator compiled into libparti_ref.so (spec: a
    ctypes structure with the layout of sptgbGenSpec), the factors U[0,1) from
    seed `fac_seed`, stream m for mode m, as sptgbFillMatrix makes them for the
    GPU.  Nothing of libParTI.so is loaded."""

    WHICH = {"seq": 0, "reduce": 1, "atomic": 2}

    def __init__(self, spec, rank, fac_seed, threads):
        L = ref()
        self.rank = rank
        self.threads = threads
        self.h = L.ref_session_open(C.byref(spec), rank, fac_seed, threads)
        if not self.h:
            raise RuntimeError("ref_session_open failed")
        self.nnz = int(L.ref_session_nnz(self.h))
        nd = np.zeros(8, np.uint32)
        L.ref_session_ndims(self.h, nd.ctypes.data_as(u32p))
        self.ndims = [int(x) for x in nd[: spec.nmodes]]

    def mttkrp(self, mode, which="reduce", out=None):
        """Seconds of one call; out (ndims[mode] x stride float32) receives M."""
        p = out.ctypes.data_as(f32p) if out is not None else None
        with quiet_stdout():
            t = ref().ref_session_mttkrp(self.h, self.WHICH[which], mode, p)
        if t < 0:
            raise RuntimeError("reference MTTKRP failed")
        return t

    def cuda_mttkrp(self, mode, impl=15, out=None):
        """The reference's sptCudaMTTKRPOneKernel: (call seconds, kernel
        seconds as the reference itself prints them), or None when the
        reference was built without CUDA."""
        p = out.ctypes.data_as(f32p) if out is not None else None
        with capture_stdout() as cap:
            t = ref().ref_session_cuda_mttkrp(self.h, mode, impl, p)
        if t == -2.0:
            return None
        if t < 0:
            raise RuntimeError("reference sptCudaMTTKRPOneKernel failed:\n" + cap.text[-2000:])
        import re
        m = re.search(r"^\[CUDA SpTns MTTKRP\]: ([0-9.eE+-]+) s$", cap.text, re.M)
        return t, (float(m.group(1)) if m else None)

    def cpd(self, niters, use_reduce=1):
        """OmpCpdAlsStep from the session's factors: (seconds, corrected fit, lambda)."""
        lam = np.zeros(self.rank, np.float32)
        fit = C.c_double()
        with quiet_stdout():
            t = ref().ref_session_cpd(self.h, niters, use_reduce, lam.ctypes.data_as(f32p), C.byref(fit))
        return t, fit.value, lam

    def close(self):
        if self.h:
            ref().ref_session_close(self.h)
            self.h = None


def ref_omp_cpd(ndims, inds, vals, rank, niters, init, tk):
    """The reference's OmpCpdAlsStep (sptOmpCpdAls with use_reduce = 1) from
    caller factors: (seconds, corrected fit, lambda)."""
    N = len(ndims)
    stride = stride_of(rank)
    nd, ndp = _u32(ndims)
    keep, ip = _rows(list(inds), u32p, np.uint32)
    v = np.ascontiguousarray(vals, np.float32)
    facs = [_padded(np.asarray(a, np.float32)[:, :rank], stride) for a in init]
    fk, fp = _rows(facs, f32p, np.float32)
    lam = np.zeros(rank, np.float32)
    fit = C.c_double()
    with quiet_stdout():
        t = ref().ref_omp_cpd(N, ndp, v.shape[0], ip, v.ctypes.data_as(f32p), rank, niters, fp, stride, tk,
                              lam.ctypes.data_as(f32p), C.byref(fit))
    return t, fit.value, lam
