"""The reference's own callers of the path, compiled from the reference's
sources against include/ParTI.h alone, linked to libParTI.so and run as
separate programs:

  tests/test_cpd.c    sptLoadSparseTensor from a string, sptNewKruskalTensor,
                      sptCpdAls (rank 2, 5 iterations, tol 1e-9) and
                      sptDumpKruskalTensor (tests/test_cpd.c:24-83);
  examples/mttkrp.c   sptLoadSparseTensor, sptRandomizeMatrix factors,
                      sptSparseTensorSortIndex and the MTTKRP of every mode
                      through sptMTTKRP (-d -2), sptOmpMTTKRP_Reduce (-d -1
                      -u 1) or sptOmpMTTKRP (-d -1 -u 0), each result written
                      by sptDumpMatrix (examples/mttkrp.c:142-291);
  examples/cpd.c      sptCpdAls (-d -2) / sptOmpCpdAls (-d -1) and
                      sptDumpKruskalTensor (examples/cpd.c:107-140);
  tests/test_ttm.c    sptSparseTensorMulMatrix of a 2x2x2 tensor, converted
                      and dumped, checked by the program itself against its
                      expected text (tests/test_ttm.c:45-106);
  examples/convert_hicoo.c  sptLoadSparseTensor, sptSparseTensorToHiCOO,
                      sptSparseTensorStatusHiCOO, sptDumpSparseTensorHiCOO
                      (examples/convert_hicoo.c:79-92);
  examples/loadstore.c  sptLoadSparseTensor then sptDumpSparseTensor
                      (examples/loadstore.c:22-42).

Their printed results are checked against the oracle run from the same
initial factors, or, for the converters, against the same program built
on the reference library (oracle/_ref/libparti_ref.so) and run on the same
input: this library's sptRandomizeMatrix draws the k-th matrix of a
process from a seeded stream (SPTGB_SEED), restated here in numpy and pinned
to the library by a CPU test.  The reference sources come from the staged copy
(oracle/_ref/tree, `make -C oracle stage`); without it these tests skip."""
import os
import re
import subprocess
import sys

import numpy as np
import pytest

import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TREE = O.REF_TREE
LIBDIR = os.path.join(ROOT, "sptol_gb300", "lib")
CALLERS = {"test_cpd": "tests/test_cpd.c", "mttkrp": "examples/mttkrp.c", "cpd": "examples/cpd.c",
           "test_ttm": "tests/test_ttm.c", "convert_hicoo": "examples/convert_hicoo.c",
           "loadstore": "examples/loadstore.c"}
have_tree = pytest.mark.skipif(not all(os.path.exists(os.path.join(TREE, p)) for p in CALLERS.values()),
                               reason="reference sources not staged (make -C oracle stage)")
GAMMA = 0x9E3779B97F4A7C15
M64 = (1 << 64) - 1


def _mix64(z):
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def seeded_matrix(seed, k, nrows, ncols):
    """The k-th (0-based) matrix sptRandomizeMatrix fills in a process whose
    SPTGB_SEED is `seed`: entry (i, j) from SplitMix64 value i*ncols + j of
    the stream seed*gamma + k + 1, scaled to [-3, 3] with a sign bit."""
    base = np.uint64((seed * GAMMA + k + 1) & M64)
    with np.errstate(over="ignore"):
        idx = np.arange(1, nrows * ncols + 1, dtype=np.uint64)
        z = _mix64(base + np.uint64(GAMMA) * idx)
    v = np.float32(3.0) * ((z >> np.uint64(40)).astype(np.float64) / 16777216.0).astype(np.float32)
    v = np.where((z & np.uint64(1)) == 1, -v, v).astype(np.float32)
    return v.reshape(nrows, ncols)


def test_seeded_matrix_restatement_matches_library():
    """CPU: the numpy restatement above equals the library's
    sptRandomizeMatrix in a fresh process with SPTGB_SEED set."""
    code = ("import ctypes as C, numpy as np, sys; sys.path.insert(0, %r)\n"
            "import sptol_gb300 as S\n"
            "out = []\n"
            "for (r, c) in ((5, 3), (7, 16), (4, 9)):\n"
            "    M = S.Matrix(r, c)\n"
            "    assert S.lib().sptRandomizeMatrix(C.byref(M.s), r, c) == 0\n"
            "    out.append(M.view().copy())\n"
            "np.savez(sys.argv[1], *out)\n" % ROOT)
    path = os.path.join(ROOT, "_build_seeded_check.npz")
    try:
        env = dict(os.environ, SPTGB_SEED="12345")
        subprocess.run([sys.executable, "-c", code, path], check=True, env=env, timeout=300)
        got = np.load(path)
        for k, (r, c) in enumerate(((5, 3), (7, 16), (4, 9))):
            assert np.array_equal(got["arr_%d" % k], seeded_matrix(12345, k, r, c))
    finally:
        if os.path.exists(path):
            os.remove(path)


def _compile(name, outdir, on_reference=False):
    """The caller against include/ParTI.h and libParTI.so, or (on_reference)
    against the reference's own headers and its library built from the staged
    sources."""
    if on_reference:
        exe = os.path.join(outdir, name + "_ref")
        refdir = os.path.dirname(O.REF_PATH)
        cmd = ["gcc", "-O2", "-std=gnu99", "-fopenmp", "-D_GNU_SOURCE", "-DPARTI_USE_OPENMP",
               "-DPARTI_INDEX_TYPEWIDTH=32", "-DPARTI_VALUE_TYPEWIDTH=32", "-DPARTI_ELEMENT_INDEX_TYPEWIDTH=8",
               "-I", os.path.join(TREE, "include"), "-o", exe, os.path.join(TREE, CALLERS[name]),
               "-L", refdir, "-lparti_ref", "-Wl,-rpath," + refdir, "-lm"]
    else:
        exe = os.path.join(outdir, name)
        cmd = ["gcc", "-O2", "-std=gnu99", "-fopenmp", "-D_GNU_SOURCE", "-DPARTI_USE_OPENMP",
               "-I", os.path.join(ROOT, "include"), "-o", exe, os.path.join(TREE, CALLERS[name]),
               "-L", LIBDIR, "-lParTI", "-Wl,-rpath," + LIBDIR, "-lm"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def _run(cmd, seed, timeout=300):
    env = dict(os.environ, SPTGB_SEED=str(seed), SPTGB_QUIET="1")
    p = subprocess.run(cmd, env=env, capture_output=True, text=True, timeout=timeout)
    assert p.returncode == 0, (cmd, p.returncode, p.stdout[-2000:], p.stderr[-2000:])
    return p.stdout


def _write_tns(path, ndims, inds, vals):
    with open(path, "w") as f:
        f.write("%d\n%s\n" % (len(ndims), " ".join(str(d) for d in ndims)))
        for x in range(vals.shape[0]):
            f.write(" ".join(str(int(inds[m, x]) + 1) for m in range(len(ndims))) + " %.6f\n" % vals[x])


def _small_tensor(seed, ndims, n):
    rng = np.random.default_rng(seed)
    keys = np.unique(np.stack([rng.integers(0, d, 2 * n) for d in ndims]).astype(np.uint32), axis=1)
    keys = keys[:, rng.permutation(keys.shape[1])[:n]]
    vals = np.round(rng.random(keys.shape[1]), 6).astype(np.float32) + np.float32(0.25)
    return keys, vals


def _parse_matrices(text):
    """Blocks written by sptDumpMatrix: 'R x C matrix' then R rows."""
    mats = []
    lines = text.splitlines()
    i = 0
    while i < len(lines):
        m = re.match(r"^(\d+) x (\d+) matrix$", lines[i].strip())
        if m:
            r, c = int(m.group(1)), int(m.group(2))
            rows = [[float(x) for x in lines[i + 1 + k].split()] for k in range(r)]
            mats.append(np.array(rows, np.float64).reshape(r, c))
            i += 1 + r
        else:
            i += 1
    return mats


def _fit_line(text):
    m = re.search(r"^fit: ([-+0-9.eE]+)$", text, re.M)
    assert m, text[-2000:]
    return float(m.group(1))


@pytest.mark.gpu
@have_tree
def test_reference_test_cpd_program(tmp_path):
    """tests/test_cpd.c unmodified: its rank-2 CP-ALS of the 3x3x3 tensor
    X[i,j,k] = 3j + k + 1 ends at the oracle's fit from the same seeded
    factors (within 1e-4; the program prints six decimals)."""
    exe = _compile("test_cpd", str(tmp_path))
    seed = 31
    out = _run([exe], seed)
    fit = _fit_line(out)
    ndims = [3, 3, 3]
    ii, jj, kk = np.meshgrid(np.arange(3), np.arange(3), np.arange(3), indexing="ij")
    inds = np.stack([ii.ravel(), jj.ravel(), kk.ravel()]).astype(np.uint32)
    vals = (3 * inds[1] + inds[2] + 1).astype(np.float32)
    init = [seeded_matrix(seed, m, 3, 2) for m in range(3)]
    _, _, ofits, oit = O.cpd_als(ndims, inds, vals, 2, 5, 1e-9, init)
    assert abs(fit - ofits[oit - 1]) <= 1e-4, (fit, ofits[:oit])
    assert "nmodes: 3, rank: 2" in out


@pytest.mark.gpu
@have_tree
@pytest.mark.parametrize("flags", [["-d", "-2"], ["-d", "-1", "-u", "1", "-t", "4"], ["-d", "-1", "-u", "0", "-t", "4"]],
                         ids=["sptMTTKRP", "sptOmpMTTKRP_Reduce", "sptOmpMTTKRP"])
def test_reference_mttkrp_example(tmp_path, flags):
    """examples/mttkrp.c unmodified, every mode at rank 16: each matrix it
    dumps (two decimals) equals the oracle's FP64 MTTKRP of the same tensor
    and seeded factors to within half a unit of the last printed digit."""
    exe = _compile("mttkrp", str(tmp_path))
    ndims, rank, seed = [40, 30, 20], 16, 77
    inds, vals = _small_tensor(5, ndims, 3000)
    tns = str(tmp_path / "x.tns")
    dump = str(tmp_path / "out.txt")
    _write_tns(tns, ndims, inds, vals)
    _run([exe, "-i", tns, "-o", dump, "-r", str(rank)] + flags, seed)
    mats = _parse_matrices(open(dump).read())
    assert len(mats) == 3
    stride = O.stride_of(rank)
    facs = [np.pad(seeded_matrix(seed, m, ndims[m], rank), ((0, 0), (0, stride - rank))) for m in range(3)]
    # the tensor as the text reader stores it (values parsed as float)
    vals_read = np.array([np.float32(float("%.6f" % v)) for v in vals], np.float32)
    for mode in range(3):
        ref = O.mttkrp(ndims, inds, vals_read, facs, rank, mode, precision="f64")[:, :rank]
        got = mats[mode]
        assert got.shape == (ndims[mode], rank)
        assert np.abs(got - ref).max() <= 0.005 + 1e-4 * np.abs(ref).max(), (mode, np.abs(got - ref).max())


@pytest.mark.gpu
@have_tree
@pytest.mark.parametrize("flags", [["-d", "-2"], ["-d", "-1", "-u", "1", "-t", "4"]], ids=["sptCpdAls", "sptOmpCpdAls"])
def test_reference_cpd_example(tmp_path, flags):
    """examples/cpd.c unmodified, rank 16, 5 iterations, tol 1e-5: the fit it
    writes with sptDumpKruskalTensor equals the oracle's from the same seeded
    factors within 1e-4."""
    exe = _compile("cpd", str(tmp_path))
    ndims, rank, seed = [60, 50, 40], 16, 91
    inds, vals = _small_tensor(6, ndims, 8000)
    tns = str(tmp_path / "x.tns")
    dump = str(tmp_path / "kt.txt")
    _write_tns(tns, ndims, inds, vals)
    _run([exe, "-i", tns, "-o", dump, "-r", str(rank)] + flags, seed)
    fit = _fit_line(open(dump).read())
    vals_read = np.array([np.float32(float("%.6f" % v)) for v in vals], np.float32)
    init = [seeded_matrix(seed, m, ndims[m], rank) for m in range(3)]
    _, _, ofits, oit = O.cpd_als(ndims, inds, vals_read, rank, 5, 1e-5, init)
    assert abs(fit - ofits[oit - 1]) <= 1e-4, (fit, ofits[:oit])


have_ref_lib = pytest.mark.skipif(not os.path.exists(O.REF_PATH), reason="reference library not built (oracle.build())")


@pytest.mark.gpu
@have_tree
def test_reference_test_ttm_program(tmp_path):
    """tests/test_ttm.c unmodified: the TTM of its 2x2x2 tensor, converted to
    a sparse tensor and dumped, must equal the text the program expects; it
    exits 1 on any difference."""
    exe = _compile("test_ttm", str(tmp_path))
    p = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, (p.stdout[-2000:], p.stderr[-2000:])


def _status_lines(text):
    keep = ("DIMS=", "sb=", "nb=", "HiCOO-STORAGE=", "SCHEDULE MODE", "Nnzb:", "cb:", "median cb:", "alpha_b:",
            "Suggest", "COO-STORAGE=", "Average slice length")
    return [l.rstrip() for l in text.splitlines() if l.startswith(keep)]


@pytest.mark.gpu
@have_tree
@have_ref_lib
@pytest.mark.parametrize("bits", [(3, 5), (7, 17)], ids=["sb3_sk5", "sb7_sk17"])
def test_reference_convert_hicoo_example_matches_reference(tmp_path, bits):
    """examples/convert_hicoo.c unmodified, built on this library and on the
    reference, same input: the dumped HiCOO files are byte-identical and the
    COO and HiCOO status lines it prints are the same."""
    ndims = [300, 200, 90]
    inds, vals = _small_tensor(12, ndims, 20000)
    tns = str(tmp_path / "x.tns")
    _write_tns(tns, ndims, inds, vals)
    outs = {}
    for ref in (False, True):
        exe = _compile("convert_hicoo", str(tmp_path), on_reference=ref)
        dump = str(tmp_path / ("ref.txt" if ref else "ours.txt"))
        stdout = _run([exe, "-i", tns, "-o", dump, "-b", str(bits[0]), "-k", str(bits[1])], 1)
        outs[ref] = (open(dump, "rb").read(), _status_lines(stdout))
    assert outs[False][0] == outs[True][0]
    assert outs[False][1] == outs[True][1] and len(outs[True][1]) >= 10


@pytest.mark.gpu
@have_tree
@have_ref_lib
def test_reference_loadstore_example_matches_reference(tmp_path):
    """examples/loadstore.c unmodified, built on this library and on the
    reference: the same text file (with a zero value and a duplicated
    coordinate) is read and written back byte-identically."""
    ndims = [50, 40, 30]
    inds, vals = _small_tensor(13, ndims, 3000)
    vals[17] = 0.0
    inds[:, 25] = inds[:, 24]
    tns = str(tmp_path / "x.tns")
    _write_tns(tns, ndims, inds, vals)
    outs = []
    for ref in (False, True):
        exe = _compile("loadstore", str(tmp_path), on_reference=ref)
        out = str(tmp_path / ("ref.tns" if ref else "ours.tns"))
        _run([exe, tns, out], 1)
        outs.append(open(out, "rb").read())
    assert outs[0] == outs[1] and len(outs[0]) > 1000
