"""Pins the oracle (the C restatement in oracle/orc.c) to the reference's own
outputs stored in tests/golden: bit-exact sorts, HiCOO arrays and MTTKRP
(same summation order), CP-ALS fits within 1e-6."""
import os

import numpy as np
import pytest

import oracle as O
from conftest import golden, rel_fro


@pytest.mark.parametrize("case", ["sort_3d", "sort_4d"])
def test_sorts(case):
    g = golden(case)
    p = O.sort_lex(g["inds"])
    assert np.array_equal(g["inds"][:, p], g["lex_inds"]) and np.array_equal(g["vals"][p], g["lex_vals"])
    order = [int(x) for x in g["order"]]
    p = O.sort_lex(g["inds"], order)
    assert np.array_equal(g["inds"][:, p], g["custom_inds"])


@pytest.mark.parametrize("case", ["hicoo_3d_small", "hicoo_3d_skew", "hicoo_4d"])
def test_hicoo(case):
    g = golden(case)
    ndims = [int(x) for x in g["ndims"]]
    p = O.sort_hicoo(g["inds"], int(g["sk"]))
    si = g["inds"][:, p]
    assert np.array_equal(si, g["sorted_inds"])
    h = O.hicoo_build(ndims, si, int(g["sb"]), int(g["sk"]))
    for k in ("kptr", "cptr", "bptr", "binds", "einds", "nkiters", "kschr_len", "kschr"):
        assert np.array_equal(h[k], g[k]), k
    assert h["max_nnzb"] == int(g["max_nnzb"])
    if "out0" in g.files:
        rank = int(g["rank"])
        mats = [g["mat%d" % m] for m in range(len(ndims))]
        for mode in range(len(ndims)):
            out = O.mttkrp_hicoo(ndims, h, g["sorted_vals"], int(g["sb"]), mats, rank, mode)
            assert np.array_equal(out, g["out%d" % mode][:, :rank])
            if len(ndims) == 3:
                # the scheduled, privatised OpenMP form: one thread visits each
                # output row's kernels in the sequential order (bit-exact)
                rows = O.kschr_rows(h, ndims, int(g["sk"]), mode)
                for tk in (1, 4):
                    par = O.omp_mttkrp_hicoo_reduce(ndims, h, g["sorted_vals"], int(g["sb"]), mats, rank, mode,
                                                    tk, rows)
                    if tk == 1:
                        assert np.array_equal(par, g["out%d" % mode][:, :rank])
                    else:
                        assert rel_fro(par, g["out%d" % mode][:, :rank]) <= 1e-6


@pytest.mark.parametrize("case", ["mttkrp_3d_r16", "mttkrp_3d_r17", "mttkrp_4d_r8"])
def test_mttkrp_bitexact(case):
    g = golden(case)
    ndims = [int(x) for x in g["ndims"]]
    rank = int(g["rank"])
    mats = [g["mat%d" % m] for m in range(len(ndims))]
    for mode in range(len(ndims)):
        out = O.mttkrp(ndims, g["inds"], g["vals"], mats, rank, mode)
        assert np.array_equal(out, g["out%d" % mode][:, :rank])
        f64 = O.mttkrp(ndims, g["inds"], g["vals"], mats, rank, mode, precision="f64")
        assert rel_fro(out, f64) <= 1e-6
        omp = O.mttkrp(ndims, g["inds"], g["vals"], mats, rank, mode, precision="omp", tk=4)
        assert rel_fro(omp, f64) <= 1e-6


@pytest.mark.parametrize("case", ["cpd_3d", "cpd_4d"])
def test_cpd_fits(case):
    g = golden(case)
    ndims = [int(x) for x in g["ndims"]]
    rank, niters = int(g["rank"]), int(g["niters"])
    init = [g["init%d" % m] for m in range(len(ndims))]
    facs, lam, fits, it = O.cpd_als(ndims, g["inds"], g["vals"], rank, niters, 0.0, init)
    assert it == niters
    assert np.abs(fits - g["fits"]).max() <= 1e-6
    assert rel_fro(lam, g["lam"]) <= 1e-4
    assert abs(O.fit_exact(ndims, g["inds"], g["vals"], [g["final%d" % m] for m in range(len(ndims))], g["lam"])
               - g["fits"][-1]) <= 1e-6


def test_uniform_1m_summary_from_generator():
    """The library generator reproduces the 1024^3 tensor the summary was taken
    on, and the oracle reproduces the reference's per-mode outputs on it."""
    import sptol_gb300 as S
    g = golden("uniform_1m_summary")
    spec = S.GenSpec()
    spec.seed = 0
    spec.nmodes = 3
    for m in range(3):
        spec.ndims[m] = 1024
    spec.count = 1_000_000
    spec.merge_duplicates = 1
    spec.value_dist = S.VAL_U01
    t = S.Tensor.generate(spec)
    inds, vals = t.arrays()
    assert t.nnz == int(g["nnz"])
    ck = (inds[0].astype(np.uint64) * 1048576 * 1024 + inds[1].astype(np.uint64) * 1024 + inds[2]).sum()
    assert np.uint64(ck) == g["key_checksum"]
    assert vals.astype(np.float64).sum() == pytest.approx(float(g["val_sum"]), rel=1e-12)
    mats = [m.array()[:1024].copy() for m in S.new_factors([1024] * 3, 16, seed=1)[:3]]
    for mode in range(3):
        out = O.mttkrp([1024] * 3, inds, vals, mats, 16, mode).astype(np.float64)
        assert abs(np.linalg.norm(out) - float(g["norm%d" % mode])) <= 1e-6 * float(g["norm%d" % mode])
        assert np.array_equal(out[g["sample_rows"]], g["rows%d" % mode])


@pytest.mark.skipif(not O.ref_available(), reason="reference sources not present")
@pytest.mark.parametrize("ndims", [[70, 60, 50], [30, 25, 20, 15]])
def test_reference_library_agrees_with_oracle_on_fresh_inputs(ndims):
    rng = np.random.default_rng(99 + len(ndims))
    N = len(ndims)
    inds = np.unique(np.stack([rng.integers(0, d, 9000) for d in ndims]).astype(np.uint32), axis=1)
    inds = inds[:, rng.permutation(inds.shape[1])]
    vals = rng.random(inds.shape[1], dtype=np.float32)
    si, sv = O.ref_sort(ndims, inds, vals)
    p = O.sort_lex(inds)
    assert np.array_equal(si, inds[:, p])
    mats = [rng.random((d, 8), dtype=np.float32) for d in ndims]
    for mode in range(N):
        others = [(mode + i) % N for i in range(1, N)]
        for order in ([mode] + others, [mode] + others[::-1]):
            r, _ = O.ref_mttkrp(ndims, inds, vals, mats, 8, mode, order=order)
            assert np.array_equal(r, O.mttkrp(ndims, inds, vals, mats, 8, mode, order=order)), (mode, order)


def test_threaded_fp64_oracle_equals_sequential():
    rng = np.random.default_rng(0)
    nd = [50, 40, 30, 20]
    n = 20000
    inds = np.stack([rng.integers(0, d, n) for d in nd]).astype(np.uint32)
    vals = rng.random(n, dtype=np.float32)
    mats = [rng.random((d, 16), dtype=np.float32) for d in nd]
    for m in range(4):
        a = O.mttkrp(nd, inds, vals, mats, 16, m, precision="f64")
        b = O.mttkrp(nd, inds, vals, mats, 16, m, precision="f64_omp", tk=4)
        assert np.abs(a - b).max() <= 1e-13 * np.abs(a).max()


@pytest.mark.skipif(not os.path.isdir(os.path.join(O.REF_TREE, "src")), reason="reference sources not present")
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_ttm_oracle_equals_reference(mode):
    """The TTM restatement against the reference's own sptSparseTensorMulMatrix
    (built here from its sources): sorted tensor, fibers and values bit-exact."""
    rng = np.random.default_rng(40 + mode)
    ndims = [30, 20, 15]
    inds = np.unique(np.stack([rng.integers(0, d, 6000) for d in ndims]).astype(np.uint32), axis=1)
    inds = inds[:, rng.permutation(inds.shape[1])[:3000]]
    vals = rng.uniform(-1, 1, inds.shape[1]).astype(np.float32)
    U = rng.uniform(-1, 1, (ndims[mode], 11)).astype(np.float32)
    fib, Y, p = O.ttm(ndims, inds, vals, U, mode)
    rfib, rY, rinds, rvals = O.ref_ttm(ndims, inds, vals, U, mode)
    assert np.array_equal(inds[:, p], rinds) and np.array_equal(vals[p], rvals)
    for m in range(3):
        if m != mode:
            assert np.array_equal(fib[m], rfib[m])
    assert np.array_equal(Y.view(np.uint32), rY.view(np.uint32))


@pytest.mark.skipif(not O.ref_available(), reason="reference sources not present")
@pytest.mark.parametrize("ndims,sb,sk", [([300, 200, 100], 3, 6), ([40, 30, 20, 10], 2, 4)])
def test_reference_hicoo_agrees_with_oracle_on_fresh_inputs(ndims, sb, sk):
    """The HiCOO restatement against the reference library built from its
    sources: sort order, every conversion array and the HiCOO MTTKRP of each
    mode, bit for bit, on fresh shuffled coordinates."""
    rng = np.random.default_rng(7 + len(ndims))
    N = len(ndims)
    inds = np.unique(np.stack([rng.integers(0, d, 6000) for d in ndims]).astype(np.uint32), axis=1)
    inds = inds[:, rng.permutation(inds.shape[1])]
    vals = rng.random(inds.shape[1], dtype=np.float32)
    ri, rv, rh = O.ref_hicoo(ndims, inds, vals, sb, sk)
    p = O.sort_hicoo(inds, sk)
    assert np.array_equal(ri, inds[:, p]) and np.array_equal(rv, vals[p])
    h = O.hicoo_build(ndims, inds[:, p], sb, sk)
    for k in ("kptr", "cptr", "bptr", "binds", "einds", "nkiters", "kschr_len", "kschr"):
        assert np.array_equal(h[k], rh[k]), k
    assert h["max_nnzb"] == rh["max_nnzb"]
    mats = [rng.random((d, 8), dtype=np.float32) for d in ndims]
    for mode in range(N):
        r = O.ref_mttkrp_hicoo(ndims, inds, vals, sb, sk, mats, 8, mode)
        assert np.array_equal(r, O.mttkrp_hicoo(ndims, h, vals[p], sb, mats, 8, mode)), mode


@pytest.mark.skipif(not O.ref_available(), reason="reference sources not present")
@pytest.mark.parametrize("ndims,rank", [([60, 50, 40], 6), ([25, 20, 15, 10], 4)])
def test_reference_cpd_agrees_with_oracle_on_fresh_inputs(ndims, rank):
    """The FP64 CP-ALS restatement against the reference's own loop (built
    from its sources) from the same initial factors: the fit of every
    iteration within 1e-5 (FP64 against the reference's FP32 arithmetic)."""
    rng = np.random.default_rng(31 + len(ndims))
    inds = np.unique(np.stack([rng.integers(0, d, 4000) for d in ndims]).astype(np.uint32), axis=1)
    vals = rng.random(inds.shape[1], dtype=np.float32)
    init = [rng.random((d, rank), dtype=np.float32) for d in ndims]
    niters = 6
    ref = O.ref_cpd_trace(ndims, inds, vals, rank, niters, init)
    # the traced loop is the reference's CpdAlsStep, bit for bit
    assert all(np.array_equal(a, b) for a, b in zip(ref["loop_factors"], ref["step_factors"]))
    assert np.array_equal(ref["loop_lambda"], ref["step_lambda"])
    facs, lam, fits, it = O.cpd_als(ndims, inds, vals, rank, niters, 0.0, init)
    assert it == niters
    assert np.abs(np.asarray(fits) - ref["fits"]).max() <= 1e-5


_TNS_CASES = {
    "basic": ("3\n4 5 6\n1 1 1 1.5\n4 5 6 -2.25e-3\n2 3 1 7\n1 2 3 0.1\n", 1),
    "zeros_removed": ("3\n3 3 3\n1 1 1 0\n2 2 2 3.5\n3 3 3 0.0\n1 2 3 -0\n2 1 1 4e1\n", 1),
    "duplicates_kept": ("2\n4 4\n1 1 2.0\n1 1 3.0\n4 4 1\n1 1 2.0\n", 1),
    "zero_based": ("3\n2 2 2\n0 0 0 1\n1 1 1 2\n0 1 0 3.25\n", 0),
    "crlf_and_spaces": ("3\r\n2 3 4\r\n 1\t2  3  9.5\r\n2 3 4 1E-2 \r\n\r\n", 1),
    "four_modes": ("4\n3 4 5 6\n1 2 3 4 1\n3 4 5 6 2\n2 2 2 2 -3.5\n", 1),
    "invalid_token_ends": ("3\n3 3 3\n1 1 1 1\n2 x 2 2\n3 3 3 3\n", 1),
    "trailing_garbage_value": ("3\n3 3 3\n1 1 1 1.5zz\n2 2 2 2\n", 1),
    "empty_body": ("3\n3 3 3\n", 1),
}


@pytest.mark.skipif(not O.ref_available(), reason="reference sources not present")
@pytest.mark.parametrize("case", sorted(_TNS_CASES))
def test_reference_reader_agrees_with_oracle(tmp_path, case):
    """The text-reader restatement against the reference's own
    sptLoadSparseTensor: order, mode sizes, coordinates and values bit for
    bit (zero removal, duplicates, 0/1-based indices, the first unreadable
    token ending the tensor)."""
    text, start = _TNS_CASES[case]
    path = str(tmp_path / (case + ".tns"))
    with open(path, "w", newline="") as f:
        f.write(text)
    try:
        ref = O.ref_load_tns(path, start)
    except ValueError as e:
        with pytest.raises(ValueError) as mine:
            O.load_tns(path, start)
        assert str(mine.value) == str(e)
        return
    got = O.load_tns(path, start)
    assert got[0] == ref[0]
    assert np.array_equal(got[1], ref[1]) and np.array_equal(got[2].view(np.uint32), ref[2].view(np.uint32))


@pytest.mark.skipif(not O.ref_available(), reason="reference sources not present")
@pytest.mark.parametrize("tk", [1, 4])
def test_reduce_port_agrees_with_the_reference(tk):
    """The port of sptOmpMTTKRP_Reduce that serves as the CPU baseline where
    the reference cannot be built, against the reference's own function at
    the same thread count: bit for bit at one thread, within the FP32
    reordering of the per-thread partial sums otherwise."""
    rng = np.random.default_rng(17)
    ndims = [300, 200, 100]
    inds = np.unique(np.stack([rng.integers(0, d, 60000) for d in ndims]).astype(np.uint32), axis=1)
    vals = rng.random(inds.shape[1], dtype=np.float32)
    mats = [rng.random((d, 16), dtype=np.float32) for d in ndims]
    for mode in range(3):
        r, _ = O.ref_mttkrp(ndims, inds, vals, mats, 16, mode, which=1, tk=tk)
        p = O.mttkrp(ndims, inds, vals, mats, 16, mode, precision="omp", tk=tk)
        if tk == 1:
            assert np.array_equal(r, p), mode
        else:
            assert rel_fro(p, r) <= 1e-6, mode
