"""Text writers in the reference's formats (sptensor/dump.c:29-52,
matrix/dump.c:34-50, ktensor/dump.c:24-51); host only, no GPU."""
import ctypes as C

import numpy as np

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
