"""Text tensor loading on the GPU (sptLoadSparseTensor) against the oracle's
restatement of the reference reader (fscanf tokens, stop at the first token
that does not convert, zero values removed by moving the last nonzero in):
coordinates and values bit-exact.  The merged variant is checked against a
lexicographic sort with duplicates summed in file order (FP32)."""
import ctypes as C
import os

import numpy as np
import pytest

import oracle as O
import sptol_gb300 as S

pytestmark = pytest.mark.gpu
_libc = C.CDLL(None)
_libc.fopen.restype = C.c_void_p
_libc.fopen.argtypes = [C.c_char_p, C.c_char_p]
_libc.fclose.argtypes = [C.c_void_p]


def load_gpu(path, start=1, merged=False):
    L = S.lib()
    fn = L.sptgbLoadSparseTensorMerged if merged else L.sptLoadSparseTensor
    fn.argtypes = [C.POINTER(S.SparseTensorS), C.c_uint32, C.c_void_p]
    fn.restype = C.c_int
    t = S.Tensor()
    fp = _libc.fopen(path.encode(), b"r")
    rc = fn(C.byref(t.s), start, fp)
    _libc.fclose(fp)
    if rc:
        return rc, None
    t._owned = True
    return 0, t


def _fmt_value(rng, v):
    k = rng.integers(0, 7)
    if k == 0:
        return "%.6f" % v
    if k == 1:
        return "%g" % v
    if k == 2:
        return "%.3e" % v
    if k == 3:
        return "%d" % int(round(v * 100))
    if k == 4:
        return "%.25f" % v          # more than 19 significant digits: host path
    if k == 5:
        return "%.4E" % (v * 1e30)   # exponent beyond 22: host path
    return ("+%.5f" % v) if v >= 0 else ("%.5f" % v)


def _write(path, ndims, recs, rng, messy):
    seps = [" ", "\t", "  ", " \t "]
    out = ["%d\n" % len(ndims), " ".join(str(d) for d in ndims), "\n"]
    for idx, val in recs:
        toks = [str(i + 1) for i in idx] + [val]
        if messy:
            line = ""
            for t in toks:
                line += t + seps[rng.integers(0, len(seps))]
                if rng.random() < 0.1:
                    line += "\r\n"
            out.append(line + ("\r\n" if rng.random() < 0.5 else "\n"))
        else:
            out.append(" ".join(toks) + "\n")
    with open(path, "w", newline="") as f:
        f.write("".join(out))


def _records(rng, ndims, n, zero_frac=0.05, dup_frac=0.0):
    recs = []
    for _ in range(n):
        if recs and rng.random() < dup_frac:
            idx = recs[rng.integers(0, len(recs))][0]
        else:
            idx = [int(rng.integers(0, d)) for d in ndims]
        v = 0.0 if rng.random() < zero_frac else float(rng.uniform(-5, 5))
        recs.append((idx, "0" if v == 0.0 else _fmt_value(rng, v)))
    return recs


def _same(t, ref):
    nd, inds, vals = ref
    i, v = t.arrays()
    assert t.ndims == nd
    assert np.array_equal(i, inds)
    assert np.array_equal(v.view(np.uint32), vals.view(np.uint32))


@pytest.mark.parametrize("messy,chunk", [(False, None), (True, None), (True, "4096")])
def test_load_matches_reference_reader(tmp_path, messy, chunk):
    rng = np.random.default_rng(11 if messy else 12)
    ndims = [500, 300, 40, 7]
    path = str(tmp_path / "t.tns")
    _write(path, ndims, _records(rng, ndims, 20000), rng, messy)
    if chunk:
        os.environ["SPTGB_INGEST_CHUNK"] = chunk
    try:
        rc, t = load_gpu(path)
    finally:
        os.environ.pop("SPTGB_INGEST_CHUNK", None)
    assert rc == 0
    ref = O.load_tns(path)
    _same(t, ref)
    assert t.nnz > 18000          # the whole file was read (only zero values removed)


def test_bad_token_ends_the_tensor(tmp_path):
    rng = np.random.default_rng(13)
    ndims = [50, 40, 30]
    recs = _records(rng, ndims, 3000)
    recs[1700] = (recs[1700][0], "1.5zz")     # value with trailing bytes: read, then reading stops
    recs[2500] = (recs[2500][0], "abc")       # not a number
    path = str(tmp_path / "b.tns")
    _write(path, ndims, recs, rng, False)
    rc, t = load_gpu(path)
    assert rc == 0
    ref = O.load_tns(path)
    _same(t, ref)
    assert t.nnz <= 1701
    with open(path) as f:
        txt = f.read().replace("1.5zz", "1.5 5 5")   # an index token that is fine: reading continues
    with open(path, "w") as f:
        f.write(txt)
    rc, t = load_gpu(path)
    _same(t, O.load_tns(path))


def test_index_below_start_is_an_error(tmp_path):
    path = str(tmp_path / "z.tns")
    with open(path, "w") as f:
        f.write("3\n4 4 4\n1 1 1 1.0\n0 2 2 2.0\n")
    rc, _ = load_gpu(path, start=1)
    assert rc != 0
    with pytest.raises(ValueError):
        O.load_tns(path, 1)
    rc, t = load_gpu(path, start=0)
    assert rc == 0
    _same(t, O.load_tns(path, 0))


def test_empty_body_and_special_values(tmp_path):
    path = str(tmp_path / "e.tns")
    with open(path, "w") as f:
        f.write("2\n3 3\n")
    rc, t = load_gpu(path)
    assert rc == 0 and t.nnz == 0
    with open(path, "w") as f:
        f.write("2\n3 3\n1 1 inf\n2 2 -0.0\n3 3 1e-320\n1 2 0x1p-3\n2 1 1e+39\n")
    rc, t = load_gpu(path)
    assert rc == 0
    _same(t, O.load_tns(path))


def test_merged_load_sums_duplicates_in_file_order(tmp_path):
    rng = np.random.default_rng(14)
    ndims = [60, 50, 9]
    recs = _records(rng, ndims, 30000, zero_frac=0.02, dup_frac=0.3)
    path = str(tmp_path / "m.tns")
    _write(path, ndims, recs, rng, True)
    rc, t = load_gpu(path, merged=True)
    assert rc == 0
    sums = {}
    for idx, val in recs:
        k = tuple(idx)
        sums[k] = np.float32(sums.get(k, np.float32(0)) + np.float32(float.fromhex(val) if "x" in val else float(val)))
    keys = sorted(k for k, v in sums.items() if v != 0)
    i, v = t.arrays()
    assert t.nnz == len(keys)
    assert np.array_equal(i.T, np.array(keys, np.uint32))
    assert np.array_equal(v, np.array([sums[k] for k in keys], np.float32))
    assert list(t.sortorder) == [0, 1, 2]
