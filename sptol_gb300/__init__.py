"""Host-side mirror of ParTI!'s MTTKRP / CP-ALS C API over libParTI.so.

The C library (include/ParTI.h, include/sptgb.h) is the product; this module
only binds it with ctypes so that Python callers (tests, the benchmark) use
exactly the entry points a C caller would: sptMTTKRP, sptCudaMTTKRP,
sptSparseTensorSortIndex, sptSparseTensorToHiCOO, sptMTTKRPHiCOO, sptCpdAls /
CpdAlsStep, plus the device-resident extension API.  Struct definitions mirror
include/ParTI.h field by field.  There is no Python or CPU implementation of
any operation here: a missing library raises ImportError.
"""
import ctypes as C
import os

import numpy as np

__all__ = [
    "lib", "Tensor", "Matrix", "HiCOO", "GenSpec", "mttkrp", "mttkrp_hicoo", "cpd_als",
    "new_factors", "SptError", "DIST_UNIFORM", "DIST_ZIPF", "VAL_U01", "VAL_UPM1", "VAL_LOGNORMAL",
    "VAL_PLANTED", "DeviceCoo", "DeviceHicoo", "Server", "RankMatrix", "cpd_als_hicoo",
]

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libParTI.so")

DIST_UNIFORM, DIST_ZIPF = 0, 1
VAL_U01, VAL_UPM1, VAL_LOGNORMAL, VAL_PLANTED = 0, 1, 2, 3
MAX_MODES = 8

u32p = C.POINTER(C.c_uint32)
u64p = C.POINTER(C.c_uint64)
f32p = C.POINTER(C.c_float)
u8p = C.POINTER(C.c_uint8)


class SptError(RuntimeError):
    def __init__(self, code, where):
        self.code = code
        super().__init__("%s failed with SptError 0x%x%s" % (where, code, _last_reason()))


class IndexVector(C.Structure):
    _fields_ = [("len", C.c_uint64), ("cap", C.c_uint64), ("data", u32p)]


class ValueVector(C.Structure):
    _fields_ = [("len", C.c_uint64), ("cap", C.c_uint64), ("data", f32p)]


class ElementIndexVector(C.Structure):
    _fields_ = [("len", C.c_uint64), ("cap", C.c_uint64), ("data", u8p)]


class BlockIndexVector(C.Structure):
    _fields_ = [("len", C.c_uint64), ("cap", C.c_uint64), ("data", u32p)]


class NnzIndexVector(C.Structure):
    _fields_ = [("len", C.c_uint64), ("cap", C.c_uint64), ("data", u64p)]


class SparseTensorS(C.Structure):
    _fields_ = [("nmodes", C.c_uint32), ("sortorder", u32p), ("ndims", u32p), ("nnz", C.c_uint64),
                ("inds", C.POINTER(IndexVector)), ("values", ValueVector)]


class MatrixS(C.Structure):
    _fields_ = [("nrows", C.c_uint32), ("ncols", C.c_uint32), ("cap", C.c_uint32), ("stride", C.c_uint32),
                ("values", f32p)]


class SemiSparseS(C.Structure):
    _fields_ = [("nmodes", C.c_uint32), ("ndims", u32p), ("mode", C.c_uint32), ("nnz", C.c_uint64),
                ("inds", C.POINTER(IndexVector)), ("stride", C.c_uint32), ("values", MatrixS)]


class RankMatrixS(C.Structure):
    _fields_ = [("nrows", C.c_uint32), ("ncols", C.c_uint8), ("cap", C.c_uint32), ("stride", C.c_uint8),
                ("values", f32p)]


class RankKruskalS(C.Structure):
    _fields_ = [("nmodes", C.c_uint32), ("rank", C.c_uint8), ("ndims", u32p), ("lambda_", f32p),
                ("fit", C.c_double), ("factors", C.POINTER(C.POINTER(RankMatrixS)))]


class HiCOOS(C.Structure):
    _fields_ = [("nmodes", C.c_uint32), ("sortorder", u32p), ("ndims", u32p), ("nnz", C.c_uint64),
                ("sb_bits", C.c_uint8), ("sk_bits", C.c_uint8), ("sc_bits", C.c_uint8),
                ("kptr", NnzIndexVector), ("kschr", C.POINTER(C.POINTER(IndexVector))), ("nkiters", u32p),
                ("cptr", NnzIndexVector), ("kschr_balanced", C.POINTER(C.POINTER(IndexVector))),
                ("kschr_balanced_pos", C.POINTER(C.POINTER(IndexVector))), ("nkpars", u32p),
                ("kschr_rest", C.POINTER(IndexVector)), ("knnzs", NnzIndexVector), ("bptr", NnzIndexVector),
                ("binds", C.POINTER(BlockIndexVector)), ("einds", C.POINTER(ElementIndexVector)),
                ("values", ValueVector)]


class KruskalS(C.Structure):
    _fields_ = [("nmodes", C.c_uint32), ("rank", C.c_uint32), ("ndims", u32p), ("lambda_", f32p),
                ("fit", C.c_double), ("factors", C.POINTER(C.POINTER(MatrixS)))]


class GenSpec(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("nmodes", C.c_uint32), ("ndims", C.c_uint32 * 8),
                ("coord_dist", C.c_int * 8), ("zipf_s", C.c_double * 8), ("count", C.c_uint64),
                ("merge_duplicates", C.c_int), ("value_dist", C.c_int), ("planted_rank", C.c_uint32),
                ("planted_seed", C.c_uint64), ("noise_sigma", C.c_double)]


_LIB = None


def _declare(L):
    T = C.POINTER(SparseTensorS)
    M = C.POINTER(MatrixS)
    MM = C.POINTER(M)
    H = C.POINTER(HiCOOS)
    RM = C.POINTER(RankMatrixS)
    RMM = C.POINTER(RM)
    sig = {
        "sptGetLastError": (C.c_int, [C.POINTER(C.c_char_p), C.POINTER(C.c_char_p), C.POINTER(C.c_uint),
                                      C.POINTER(C.c_char_p)]),
        "sptClearLastError": (None, []),
        "sptNewSparseTensor": (C.c_int, [T, C.c_uint32, u32p]),
        "sptFreeSparseTensor": (None, [T]),
        "sptResizeIndexVector": (C.c_int, [C.POINTER(IndexVector), C.c_uint64]),
        "sptResizeValueVector": (C.c_int, [C.POINTER(ValueVector), C.c_uint64]),
        "sptNewMatrix": (C.c_int, [M, C.c_uint32, C.c_uint32]),
        "sptFreeMatrix": (None, [M]),
        "sptMTTKRP": (C.c_int, [T, MM, u32p, C.c_uint32]),
        "sptOmpMTTKRP": (C.c_int, [T, MM, u32p, C.c_uint32, C.c_int]),
        "sptOmpMTTKRP_Lock": (C.c_int, [T, MM, u32p, C.c_uint32, C.c_int, C.c_void_p]),
        "sptMutexAlloc": (C.c_void_p, []),
        "sptMatrixDotMulSeqTriangle": (C.c_int, [C.c_uint32, C.c_uint32, MM]),
        "sptMatrixSolveNormals": (C.c_int, [C.c_uint32, C.c_uint32, MM, M]),
        "sptMatrix2Norm": (C.c_int, [M, f32p]),
        "sptMatrixMaxNorm": (C.c_int, [M, f32p]),
        "GetFinalLambda": (None, [C.c_uint32, C.c_uint32, MM, f32p]),
        "sptKruskalTensorFit": (C.c_double, [T, f32p, MM, MM]),
        "sptKruskalTensorFrobeniusNormSquared": (C.c_double, [C.c_uint32, f32p, MM]),
        "sptSparseKruskalTensorInnerProduct": (C.c_double, [C.c_uint32, f32p, MM]),
        "sptDumpSparseTensor": (C.c_int, [T, C.c_uint32, C.c_void_p]),
        "sptDumpMatrix": (C.c_int, [M, C.c_void_p]),
        "sptDumpSparseTensorHiCOO": (C.c_int, [H, C.c_void_p]),
        "sptDumpRankMatrix": (C.c_int, [RM, C.c_void_p]),
        "sptDumpRankKruskalTensor": (C.c_int, [C.POINTER(RankKruskalS), C.c_void_p]),
        "sptDumpKruskalTensor": (C.c_int, [C.POINTER(KruskalS), C.c_void_p]),
        "sptDumpIndexArray": (C.c_int, [u32p, C.c_uint64, C.c_void_p]),
        "sptDumpNnzIndexArray": (C.c_int, [u64p, C.c_uint64, C.c_void_p]),
        "sptRankMatrixDotMulSeqTriangle": (C.c_int, [C.c_uint32, C.c_uint32, RMM]),
        "sptRankMatrixSolveNormals": (C.c_int, [C.c_uint32, C.c_uint32, RMM, RM]),
        "sptRankMatrix2Norm": (C.c_int, [RM, f32p]),
        "sptRankMatrixMaxNorm": (C.c_int, [RM, f32p]),
        "GetRankFinalLambda": (None, [C.c_uint8, C.c_uint32, RMM, f32p]),
        "sptKruskalTensorFitHiCOO": (C.c_double, [H, f32p, RMM, RMM]),
        "sptKruskalTensorFrobeniusNormSquaredRank": (C.c_double, [C.c_uint32, f32p, RMM]),
        "sptSparseKruskalTensorInnerProductRank": (C.c_double, [C.c_uint32, f32p, RMM]),
        "SptMutexAllocCustom": (C.c_void_p, [C.c_uint32, C.c_uint32]),
        "sptMutexFree": (None, [C.c_void_p]),
        "sptMTTKRPHiCOO_MatrixTiling": (C.c_int, [H, C.POINTER(C.POINTER(RankMatrixS)), u32p, C.c_uint32]),
        "sptOmpMTTKRPHiCOO_MatrixTiling": (C.c_int, [H, C.POINTER(C.POINTER(RankMatrixS)), u32p, C.c_uint32,
                                                      C.c_int]),
        "sptOmpMTTKRPHiCOO_MatrixTiling_Scheduled": (C.c_int, [H, C.POINTER(C.POINTER(RankMatrixS)), u32p,
                                                                C.c_uint32, C.c_int, C.c_int]),
        "sptOmpMTTKRPHiCOO_MatrixTiling_Scheduled_Reduce": (C.c_int, [H, C.POINTER(C.POINTER(RankMatrixS)),
                                                                       C.POINTER(C.POINTER(RankMatrixS)), u32p,
                                                                       C.c_uint32, C.c_int, C.c_int]),
        "sptCudaMTTKRP": (C.c_int, [T, MM, u32p, C.c_uint32, C.c_uint32]),
        "sptSparseTensorSortIndex": (None, [T, C.c_int, C.c_int]),
        "sptSparseTensorSortIndexCustomOrder": (None, [T, u32p, C.c_int, C.c_int]),
        "sptSparseTensorSortIndexAtMode": (None, [T, C.c_uint32, C.c_int, C.c_int]),
        "sptSparseTensorSortIndexMorton": (None, [T, C.c_int, C.c_uint64, C.c_uint64, C.c_uint8, C.c_int]),
        "sptSparseTensorSortIndexRowBlock": (None, [T, C.c_int, C.c_uint64, C.c_uint64, C.c_uint8, C.c_int]),
        "sptSparseTensorMixedOrder": (C.c_int, [T, C.c_uint8, C.c_uint8, C.c_int]),
        "sptSparseTensorToHiCOO": (C.c_int, [H, u64p, T, C.c_uint8, C.c_uint8, C.c_int]),
        "sptFreeSparseTensorHiCOO": (None, [H]),
        "sptMTTKRPHiCOO": (C.c_int, [H, MM, u32p, C.c_uint32]),
        "CpdAlsStep": (C.c_double, [T, C.c_uint32, C.c_uint32, C.c_double, MM, f32p]),
        "sptCpdAls": (C.c_int, [T, C.c_uint32, C.c_uint32, C.c_double, C.POINTER(KruskalS)]),
        "sptNewKruskalTensor": (C.c_int, [C.POINTER(KruskalS), C.c_uint32, u32p, C.c_uint32]),
        "sptFreeKruskalTensor": (None, [C.POINTER(KruskalS)]),
        "SparseTensorFrobeniusNormSquared": (C.c_double, [T]),
        "sptgbVersion": (C.c_char_p, []),
        "sptgbInit": (C.c_int, [C.c_int]),
        "sptgbStream": (C.c_void_p, []),
        "sptgbLaunchCount": (C.c_uint64, []),
        "sptgbSetSeed": (None, [C.c_uint64]),
        "sptgbPinSparseTensor": (C.c_int, [T]),
        "sptgbUnpinSparseTensor": (C.c_int, [T]),
        "sptgbPinMatrix": (C.c_int, [M]),
        "sptgbUnpinMatrix": (C.c_int, [M]),
        "sptgbGenerate": (C.c_int, [T, C.POINTER(GenSpec)]),
        "sptgbFillMatrix": (C.c_int, [M, C.c_uint64, C.c_uint64, C.c_float, C.c_float]),
        "sptgbCpdAls": (C.c_int, [T, C.c_uint32, C.c_uint32, C.c_double, MM, f32p, C.POINTER(C.c_double),
                                  u32p]),
        "sptgbCooCreate": (C.c_int, [C.POINTER(C.c_void_p), T, C.c_void_p]),
        "sptgbCooPrepareMode": (C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p]),
        "sptgbCooMTTKRP": (C.c_int, [C.c_void_p, C.c_uint32, u32p, C.POINTER(C.c_void_p), C.c_uint32,
                                     C.c_uint32, C.c_void_p, C.c_void_p]),
        "sptgbCooMTTKRPBf16": (C.c_int, [C.c_void_p, C.c_uint32, u32p, C.POINTER(C.c_void_p), C.c_uint32,
                                         C.c_uint32, C.c_void_p, C.c_void_p]),
        "sptgbCooNnz": (C.c_uint64, [C.c_void_p]),
        "sptgbCooModeArrays": (C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p),
                                         C.c_void_p]),
        "sptgbCooDeviceBytes": (C.c_size_t, [C.c_void_p]),
        "sptgbCooSetTiming": (None, [C.c_void_p, C.c_int]),
        "sptgbCooLastKernelMs": (C.c_float, [C.c_void_p]),
        "sptgbCooFree": (None, [C.c_void_p]),
        "sptgbHiCOOSetTiming": (None, [C.c_int]),
        "sptSparseTensorMulMatrix": (C.c_int, [C.POINTER(SemiSparseS), T, M, C.c_uint32]),
        "sptCudaSparseTensorMulMatrix": (C.c_int, [C.POINTER(SemiSparseS), T, M, C.c_uint32]),
        "sptFreeSemiSparseTensor": (None, [C.POINTER(SemiSparseS)]),
        "sptSemiSparseTensorToSparseTensor": (C.c_int, [T, C.POINTER(SemiSparseS), C.c_float]),
        "sptNewRankMatrix": (C.c_int, [C.POINTER(RankMatrixS), C.c_uint32, C.c_uint8]),
        "sptFreeRankMatrix": (None, [C.POINTER(RankMatrixS)]),
        "sptNewRankKruskalTensor": (C.c_int, [C.POINTER(RankKruskalS), C.c_uint32, u32p, C.c_uint8]),
        "sptFreeRankKruskalTensor": (None, [C.POINTER(RankKruskalS)]),
        "sptCpdAlsHiCOO": (C.c_int, [H, C.c_uint32, C.c_uint32, C.c_double, C.POINTER(RankKruskalS)]),
        "sptgbCpdAlsHiCOO": (C.c_int, [H, C.c_uint32, C.c_uint32, C.c_double, C.POINTER(C.POINTER(RankMatrixS)),
                                       f32p, C.POINTER(C.c_double), u32p]),
        "sptgbHicooCreate": (C.c_int, [C.POINTER(C.c_void_p), H, C.c_void_p]),
        "sptgbHicooPrepareMode": (C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p]),
        "sptgbHicooMTTKRP": (C.c_int, [C.c_void_p, C.c_uint32, u32p, C.POINTER(C.c_void_p), C.c_uint32,
                                       C.c_uint32, C.c_void_p, C.c_void_p]),
        "sptgbHicooDeviceBytes": (C.c_size_t, [C.c_void_p]),
        "sptgbHicooFree": (None, [C.c_void_p]),
        "sptgbHiCOOLastKernelMs": (C.c_float, []),
        "sptgbServerCreate": (C.c_int, [C.POINTER(C.c_void_p), C.c_size_t, C.c_uint32]),
        "sptgbServerSubmit": (C.c_int, [C.c_void_p, T, C.c_uint32, C.c_uint32, MM, MM, f32p,
                                        C.POINTER(C.c_double), u64p]),
        "sptgbServerStep": (C.c_int, [C.c_void_p, u32p, u32p]),
        "sptgbServerDone": (C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
        "sptgbServerDrain": (C.c_int, [C.c_void_p]),
        "sptgbServerCompleted": (C.c_uint32, [C.c_void_p, u64p, C.c_uint32]),
        "sptgbServerBytesInUse": (C.c_size_t, [C.c_void_p]),
        "sptgbServerUnitLength": (C.c_uint32, [C.c_void_p, C.c_int]),
        "sptgbServerPersistent": (C.c_int, [C.c_void_p]),
        "sptgbServerStepKernels": (C.c_uint32, [C.c_void_p]),
        "sptgbServerSchedule": (C.c_int, [C.c_void_p, C.c_int, u32p, u32p, u32p, C.POINTER(C.c_int)]),
        "sptgbGridBarrierSelfTest": (C.c_int, [C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_uint)]),
        "sptgbServerFree": (None, [C.c_void_p]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args


def lib():
    """Loads libParTI.so (built in-tree by sptol_gb300.build)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libParTI.so is not built (%s); run sptol_gb300/build.py" % LIB_PATH)
        _LIB = C.CDLL(LIB_PATH)
        _declare(_LIB)
    return _LIB


def _last_reason():
    L = _LIB
    if L is None:
        return ""
    r = C.c_char_p()
    L.sptGetLastError(None, None, None, C.byref(r))
    return (": " + r.value.decode()) if r.value else ""


def _check(code, where):
    if code != 0:
        raise SptError(code, where)


def _u32(a):
    a = np.ascontiguousarray(a, dtype=np.uint32)
    return a, a.ctypes.data_as(u32p)


class Tensor:
    """An sptSparseTensor allocated by the library."""

    def __init__(self):
        self.s = SparseTensorS()
        self._owned = False

    @classmethod
    def from_arrays(cls, ndims, inds, vals):
        inds = np.asarray(inds)
        vals = np.ascontiguousarray(vals, dtype=np.float32)
        L = lib()
        t = cls()
        nd, ndp = _u32(ndims)
        N = len(nd)
        _check(L.sptNewSparseTensor(C.byref(t.s), N, ndp), "sptNewSparseTensor")
        t._owned = True
        n = int(vals.shape[0])
        for m in range(N):
            _check(L.sptResizeIndexVector(C.byref(t.s.inds[m]), n), "sptResizeIndexVector")
            if n:
                row = np.ascontiguousarray(inds[m], dtype=np.uint32)  # keep alive across memmove
                C.memmove(t.s.inds[m].data, row.ctypes.data, 4 * n)
        _check(L.sptResizeValueVector(C.byref(t.s.values), n), "sptResizeValueVector")
        if n:
            C.memmove(t.s.values.data, vals.ctypes.data, 4 * n)
        t.s.nnz = n
        return t

    @classmethod
    def generate(cls, spec):
        t = cls()
        _check(lib().sptgbGenerate(C.byref(t.s), C.byref(spec)), "sptgbGenerate")
        t._owned = True
        return t

    @property
    def nmodes(self):
        return int(self.s.nmodes)

    @property
    def nnz(self):
        return int(self.s.nnz)

    @property
    def ndims(self):
        return [int(self.s.ndims[m]) for m in range(self.nmodes)]

    @property
    def sortorder(self):
        return [int(self.s.sortorder[m]) for m in range(self.nmodes)]

    def inds(self, m):
        if self.nnz == 0:
            return np.zeros(0, np.uint32)
        return np.ctypeslib.as_array(self.s.inds[m].data, shape=(self.nnz,))

    def vals(self):
        if self.nnz == 0:
            return np.zeros(0, np.float32)
        return np.ctypeslib.as_array(self.s.values.data, shape=(self.nnz,))

    def arrays(self):
        """Copies: (inds [N, nnz] uint32, vals [nnz] float32)."""
        return np.stack([self.inds(m).copy() for m in range(self.nmodes)]), self.vals().copy()

    def ptr(self):
        return C.byref(self.s)

    def free(self):
        if self._owned:
            lib().sptFreeSparseTensor(C.byref(self.s))
            self._owned = False

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Matrix:
    """An sptMatrix allocated by sptNewMatrix (row-major, stride = ncols rounded up to 8)."""

    def __init__(self, nrows, ncols, zero=True):
        self.s = MatrixS()
        _check(lib().sptNewMatrix(C.byref(self.s), nrows, ncols), "sptNewMatrix")
        self._owned = True
        if zero:
            self.array()[:] = 0

    @classmethod
    def from_array(cls, a, stride_like=None):
        a = np.asarray(a, dtype=np.float32)
        m = cls(a.shape[0], a.shape[1])
        m.array()[:, : a.shape[1]] = a
        return m

    def array(self):
        """Full (cap x stride) view including padding columns."""
        s = self.s
        return np.ctypeslib.as_array(s.values, shape=(int(s.cap), int(s.stride)))

    def view(self):
        """(nrows x ncols) view."""
        return self.array()[: int(self.s.nrows), : int(self.s.ncols)]

    def free(self):
        if self._owned:
            lib().sptFreeMatrix(C.byref(self.s))
            self._owned = False

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def new_factors(ndims, rank, seed=0, lo=0.0, hi=1.0):
    """Factor matrices U[lo, hi) from the library's seeded filler, plus the
    scratch output mats[N] sized to the largest mode."""
    L = lib()
    mats = []
    for m, d in enumerate(ndims):
        M = Matrix(d, rank)
        _check(L.sptgbFillMatrix(C.byref(M.s), seed, m, lo, hi), "sptgbFillMatrix")
        mats.append(M)
    mats.append(Matrix(max(ndims), rank))
    return mats


def _mat_array(mats):
    arr = (C.POINTER(MatrixS) * len(mats))()
    for i, m in enumerate(mats):
        arr[i] = C.pointer(m.s)
    return arr


def mttkrp(tensor, mats, mode, mats_order=None, entry="sptMTTKRP", copy=True):
    """Runs the drop-in entry point `entry`; returns a copy of mats[N] rows
    [0, ndims[mode]) (copy=False: a view of mats[N] itself)."""
    L = lib()
    N = tensor.nmodes
    if mats_order is None:
        mats_order = [mode] + [(mode + i) % N for i in range(1, N)]
    order, op = _u32(mats_order)
    mats[N].s.nrows = tensor.ndims[mode]
    arr = _mat_array(mats)
    if entry == "sptMTTKRP":
        r = L.sptMTTKRP(tensor.ptr(), arr, op, mode)
    elif entry == "sptCudaMTTKRP":
        r = L.sptCudaMTTKRP(tensor.ptr(), arr, op, mode, 15)
    elif entry == "sptOmpMTTKRP":
        r = L.sptOmpMTTKRP(tensor.ptr(), arr, op, mode, 1)
    elif entry == "sptOmpMTTKRP_Lock":
        pool = L.sptMutexAlloc()
        try:
            r = L.sptOmpMTTKRP_Lock(tensor.ptr(), arr, op, mode, 4, pool)
        finally:
            L.sptMutexFree(pool)
    else:
        raise ValueError(entry)
    _check(r, entry)
    out = mats[N].array()[: tensor.ndims[mode], : int(mats[N].s.ncols)]
    return out.copy() if copy else out


class HiCOO:
    def __init__(self, tensor, sb_bits, sk_bits):
        self.s = HiCOOS()
        mx = C.c_uint64()
        _check(lib().sptSparseTensorToHiCOO(C.byref(self.s), C.byref(mx), tensor.ptr(), sb_bits, sk_bits, 1),
               "sptSparseTensorToHiCOO")
        self.max_nnzb = int(mx.value)
        self._owned = True

    def arrays(self):
        s = self.s
        N = int(s.nmodes)

        def vec(v):
            n = int(v.len)
            if n == 0:
                return np.zeros(0, dtype=np.dtype(v.data._type_))
            return np.ctypeslib.as_array(v.data, shape=(n,)).copy()

        sk = 1 << int(s.sk_bits)
        out = {
            "kptr": vec(s.kptr), "cptr": vec(s.cptr), "bptr": vec(s.bptr),
            "binds": [vec(s.binds[m]) for m in range(N)],
            "einds": [vec(s.einds[m]) for m in range(N)],
            "values": vec(s.values),
            "nkiters": [int(s.nkiters[m]) for m in range(N)],
            "kschr": [[vec(s.kschr[m][i]) for i in range((int(s.ndims[m]) + sk - 1) // sk)] for m in range(N)],
        }
        return out

    def ptr(self):
        return C.byref(self.s)

    def free(self):
        if self._owned:
            lib().sptFreeSparseTensorHiCOO(C.byref(self.s))
            self._owned = False

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def mttkrp_hicoo(h, mats, mode, mats_order=None):
    L = lib()
    N = int(h.s.nmodes)
    if mats_order is None:
        mats_order = [mode] + [(mode + i) % N for i in range(1, N)]
    order, op = _u32(mats_order)
    nd = int(h.s.ndims[mode])
    mats[N].s.nrows = nd
    _check(L.sptMTTKRPHiCOO(h.ptr(), _mat_array(mats), op, mode), "sptMTTKRPHiCOO")
    return mats[N].array()[:nd, : int(mats[N].s.ncols)].copy()


def cpd_als(tensor, rank, niters, tol, init):
    """CP-ALS from caller factors `init` (list of N arrays ndims[m] x rank).
    Returns (factors, lambda, fits per iteration, iterations run)."""
    L = lib()
    N = tensor.nmodes
    mats = [Matrix.from_array(a) for a in init] + [Matrix(max(tensor.ndims), rank)]
    lam = np.zeros(rank, np.float32)
    fits = np.zeros(niters, np.float64)
    done = C.c_uint32()
    _check(L.sptgbCpdAls(tensor.ptr(), rank, niters, tol, _mat_array(mats), lam.ctypes.data_as(f32p),
                         fits.ctypes.data_as(C.POINTER(C.c_double)), C.byref(done)), "sptgbCpdAls")
    return [mats[m].view().copy() for m in range(N)], lam, fits, int(done.value)


class DeviceCoo:
    """sptgbCoo handle: a device-resident tensor with per-mode segmented copies."""

    def __init__(self, tensor, stream=None):
        self.h = C.c_void_p()
        _check(lib().sptgbCooCreate(C.byref(self.h), tensor.ptr(), stream), "sptgbCooCreate")
        self.nmodes = tensor.nmodes

    def prepare(self, mode, stream=None):
        _check(lib().sptgbCooPrepareMode(self.h, mode, stream), "sptgbCooPrepareMode")

    def mttkrp(self, mode, mats_order, dev_ptrs, rank, stride, out_ptr, stream=None, bf16=False):
        order, op = _u32(mats_order)
        arr = (C.c_void_p * len(dev_ptrs))(*dev_ptrs)
        f = lib().sptgbCooMTTKRPBf16 if bf16 else lib().sptgbCooMTTKRP
        _check(f(self.h, mode, op, arr, rank, stride, out_ptr, stream), "sptgbCooMTTKRP")

    def mode_arrays(self, mode, stream=None):
        """Device pointers of the copy sorted by `mode`: ([inds per mode], vals)."""
        inds = (C.c_void_p * self.nmodes)()
        vals = C.c_void_p()
        _check(lib().sptgbCooModeArrays(self.h, mode, inds, C.byref(vals), stream), "sptgbCooModeArrays")
        return [int(p) for p in inds], int(vals.value)

    def set_timing(self, on):
        lib().sptgbCooSetTiming(self.h, 1 if on else 0)

    def last_ms(self):
        return float(lib().sptgbCooLastKernelMs(self.h))

    def nbytes(self):
        return int(lib().sptgbCooDeviceBytes(self.h))

    def free(self):
        if self.h:
            lib().sptgbCooFree(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def launch_count():
    return int(lib().sptgbLaunchCount())


class Server:
    """sptgbServer handle: batched / served CP-ALS under an HBM budget.

    submit() queues a job and returns its ticket; step() admits what fits and
    runs one ALS iteration of every admitted job; result() returns a finished
    job's (factors, lambda, fits).  The tensor, the initial factors and the
    result buffers of a job are kept alive here until the job is done."""

    QUEUED, DONE, FAILED = 0, 1, -1

    def __init__(self, hbm_budget, max_slots):
        self.h = C.c_void_p()
        _check(lib().sptgbServerCreate(C.byref(self.h), int(hbm_budget), int(max_slots)), "sptgbServerCreate")
        self.jobs = {}

    def submit(self, tensor, rank, niters, init, out=None):
        """init: list of N arrays (ndims[m] x rank) or Matrix objects; out:
        optional Matrix objects of the same shapes for the results."""
        N = tensor.nmodes
        ini = [a if isinstance(a, Matrix) else Matrix.from_array(a) for a in init]
        if out is None:
            out = [Matrix(int(tensor.ndims[m]), rank, zero=False) for m in range(N)]
        lam = np.zeros(rank, np.float32)
        fits = np.zeros(max(niters, 1), np.float64)
        ia, oa = _mat_array(ini), _mat_array(out)
        t = C.c_uint64()
        _check(lib().sptgbServerSubmit(self.h, tensor.ptr(), rank, niters, ia, oa, lam.ctypes.data_as(f32p),
                                       fits.ctypes.data_as(C.POINTER(C.c_double)), C.byref(t)),
               "sptgbServerSubmit")
        self.jobs[t.value] = (tensor, ini, out, lam, fits, ia, oa, niters)
        return t.value

    def step(self):
        a, q = C.c_uint32(), C.c_uint32()
        _check(lib().sptgbServerStep(self.h, C.byref(a), C.byref(q)), "sptgbServerStep")
        return int(a.value), int(q.value)

    def drain(self):
        _check(lib().sptgbServerDrain(self.h), "sptgbServerDrain")

    def state(self, ticket):
        """(state, submit time, completion time) in seconds of CLOCK_MONOTONIC."""
        a, b = C.c_double(), C.c_double()
        st = lib().sptgbServerDone(self.h, ticket, C.byref(a), C.byref(b))
        return int(st), a.value, b.value

    def completed(self, max_n=4096):
        """Tickets finished (done or failed) since the previous call."""
        buf = (C.c_uint64 * max_n)()
        n = lib().sptgbServerCompleted(self.h, buf, max_n)
        return [int(buf[i]) for i in range(n)]

    def result(self, ticket, release=True, copy=True):
        """(factors, lambda, fits) of a finished job; copy=False returns views
        of the job's own buffers."""
        st = self.state(ticket)[0]
        if st != self.DONE:
            raise RuntimeError("job %d is not done (state %d)%s" % (ticket, st, _last_reason()))
        tensor, ini, out, lam, fits, ia, oa, niters = self.jobs[ticket]
        if copy:
            res = ([m.view().copy() for m in out], lam.copy(), fits[:niters].copy())
        else:
            res = ([m.view() for m in out], lam, fits[:niters])
        if release:
            del self.jobs[ticket]
        return res

    def bytes_in_use(self):
        return int(lib().sptgbServerBytesInUse(self.h))

    def unit_length(self, group):
        return int(lib().sptgbServerUnitLength(self.h, group))

    def schedule(self, group):
        """The tuned MTTKRP schedule of a rank group: dict of unit length,
        record batch depth, blocks per SM and where it came from."""
        ul, deep, bps, src = C.c_uint32(), C.c_uint32(), C.c_uint32(), C.c_int()
        _check(lib().sptgbServerSchedule(self.h, group, C.byref(ul), C.byref(deep), C.byref(bps), C.byref(src)),
               "sptgbServerSchedule")
        return {"unit": int(ul.value), "batches": "deep" if deep.value else "shallow",
                "blocks_per_sm": int(bps.value), "source": {1: "cached", 0: "timed", -1: "no jobs"}[src.value]}

    def step_kernels(self):
        """Kernels one ALS step launches (0 before the first step)."""
        return int(lib().sptgbServerStepKernels(self.h))

    def persistent(self):
        """True when each step runs as one persistent cooperative kernel."""
        return bool(lib().sptgbServerPersistent(self.h))

    def free(self):
        if self.h:
            lib().sptgbServerFree(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class RankMatrix:
    """An sptRankMatrix allocated by sptNewRankMatrix (8-bit column count)."""

    def __init__(self, nrows, ncols):
        self.s = RankMatrixS()
        _check(lib().sptNewRankMatrix(C.byref(self.s), nrows, ncols), "sptNewRankMatrix")
        self._owned = True

    @classmethod
    def from_array(cls, a):
        a = np.asarray(a, dtype=np.float32)
        m = cls(a.shape[0], a.shape[1])
        m.array()[:, : a.shape[1]] = a
        return m

    def array(self):
        s = self.s
        return np.ctypeslib.as_array(s.values, shape=(int(s.cap), int(s.stride)))

    def view(self):
        return self.array()[: int(self.s.nrows), : int(self.s.ncols)]

    def free(self):
        if self._owned:
            lib().sptFreeRankMatrix(C.byref(self.s))
            self._owned = False

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def cpd_als_hicoo(h, rank, niters, tol, init):
    """sptgbCpdAlsHiCOO from caller factors `init` (N arrays ndims[m] x rank).
    Returns (factors, lambda, fits, iterations run)."""
    L = lib()
    N = int(h.s.nmodes)
    mats = [RankMatrix.from_array(a) for a in init]
    arr = (C.POINTER(RankMatrixS) * N)(*[C.pointer(m.s) for m in mats])
    lam = np.zeros(rank, np.float32)
    fits = np.zeros(niters, np.float64)
    done = C.c_uint32()
    _check(L.sptgbCpdAlsHiCOO(h.ptr(), rank, niters, tol, arr, lam.ctypes.data_as(f32p),
                              fits.ctypes.data_as(C.POINTER(C.c_double)), C.byref(done)), "sptgbCpdAlsHiCOO")
    return [m.view().copy() for m in mats], lam, fits, int(done.value)


class DeviceHicoo:
    """sptgbHicoo handle: HiCOO arrays resident on the device, per-mode
    output-window schedules."""

    def __init__(self, h, stream=None):
        self.h = C.c_void_p()
        _check(lib().sptgbHicooCreate(C.byref(self.h), h.ptr(), stream), "sptgbHicooCreate")
        self.nmodes = int(h.s.nmodes)

    def prepare(self, mode, stream=None):
        _check(lib().sptgbHicooPrepareMode(self.h, mode, stream), "sptgbHicooPrepareMode")

    def mttkrp(self, mode, mats_order, dev_ptrs, rank, stride, out_ptr, stream=None):
        order, op = _u32(mats_order)
        arr = (C.c_void_p * len(dev_ptrs))(*dev_ptrs)
        _check(lib().sptgbHicooMTTKRP(self.h, mode, op, arr, rank, stride, out_ptr, stream), "sptgbHicooMTTKRP")

    def nbytes(self):
        return int(lib().sptgbHicooDeviceBytes(self.h))

    def free(self):
        if self.h:
            lib().sptgbHicooFree(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass
