"""CP-ALS on the GPU against the reference's per-iteration fit (corrected,
from its own factors; tests/golden) and against the FP64 oracle.
Tolerance: fit within 1e-4 at every iteration."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
import sptol_gb300 as S
from conftest import golden

pytestmark = pytest.mark.gpu
FIT_TOL = 1e-4


@pytest.mark.parametrize("case", ["cpd_3d", "cpd_4d"])
def test_fit_per_iteration_matches_reference(case):
    g = golden(case)
    ndims = [int(x) for x in g["ndims"]]
    rank, niters = int(g["rank"]), int(g["niters"])
    N = len(ndims)
    t = S.Tensor.from_arrays(ndims, g["inds"], g["vals"])
    init = [g["init%d" % m] for m in range(N)]
    facs, lam, fits, it = S.cpd_als(t, rank, niters, 0.0, init)
    assert it == niters
    assert np.abs(fits - g["fits"]).max() <= FIT_TOL, (fits, g["fits"])
    # the returned model has the fit the device reported for the last iteration
    fx = O.fit_exact(ndims, g["inds"], g["vals"], facs, lam)
    assert abs(fx - fits[-1]) <= FIT_TOL
    # factors are column-normalised (GetFinalLambda)
    for f in facs:
        assert np.allclose(np.linalg.norm(f.astype(np.float64), axis=0), 1.0, atol=1e-4)


def test_planted_model_against_oracle_and_tolerance_stop():
    spec = S.GenSpec()
    spec.seed = 11
    spec.nmodes = 3
    for m, d in enumerate([5000, 3000, 400]):
        spec.ndims[m] = d
        spec.coord_dist[m] = S.DIST_ZIPF
        spec.zipf_s[m] = 1.1
    spec.count = 300_000
    spec.value_dist = S.VAL_PLANTED
    spec.planted_rank = 8
    spec.planted_seed = 12
    spec.noise_sigma = 0.01
    t = S.Tensor.generate(spec)
    ndims = t.ndims
    inds, vals = t.arrays()
    rng = np.random.default_rng(13)
    init = [rng.random((d, 8), dtype=np.float32) for d in ndims]
    facs, lam, fits, it = S.cpd_als(t, 8, 12, 0.0, init)
    ofacs, olam, ofits, oit = O.cpd_als(ndims, inds, vals, 8, 12, 0.0, init)
    assert np.abs(fits - ofits).max() <= FIT_TOL, (fits, ofits)
    # a loose tolerance stops early, at the same iteration as the oracle
    _, _, fits2, it2 = S.cpd_als(t, 8, 12, 1e-2, init)
    _, _, ofits2, oit2 = O.cpd_als(ndims, inds, vals, 8, 12, 1e-2, init)
    assert it2 == oit2 and it2 < 12
    assert np.isnan(fits2[it2:]).all()


def test_rank64_and_drop_in_entry_points():
    rng = np.random.default_rng(17)
    ndims = [400, 300, 200]
    n = 60000
    inds = np.unique(np.stack([rng.integers(0, d, 2 * n) for d in ndims]).astype(np.uint32), axis=1)[:, :n]
    vals = rng.random(inds.shape[1], dtype=np.float32)
    t = S.Tensor.from_arrays(ndims, inds, vals)
    init = [rng.random((d, 64), dtype=np.float32) for d in ndims]
    facs, lam, fits, it = S.cpd_als(t, 64, 4, 0.0, init)
    _, _, ofits, _ = O.cpd_als(ndims, inds, vals, 64, 4, 0.0, init)
    assert np.abs(fits - ofits).max() <= FIT_TOL, (fits, ofits)
    # sptCpdAls: seeded random init, result in a Kruskal tensor
    L = S.lib()
    S.lib().sptgbSetSeed(5)
    k = S.KruskalS()
    nd = np.array(ndims, np.uint32)
    assert L.sptNewKruskalTensor(C.byref(k), 3, nd.ctypes.data_as(C.POINTER(C.c_uint32)), 8) == 0
    assert L.sptCpdAls(t.ptr(), 8, 3, 0.0, C.byref(k)) == 0
    assert 0.0 < k.fit <= 1.0 + 1e-6
    f0 = np.ctypeslib.as_array(k.factors[0].contents.values, shape=(ndims[0], 8))
    assert np.isfinite(f0).all()
    L.sptFreeKruskalTensor(C.byref(k))


def test_rank_above_64_is_rejected():
    t = S.Tensor.from_arrays([4, 4, 4], np.zeros((3, 1), np.uint32), np.ones(1, np.float32))
    init = [np.ones((4, 65), np.float32)] * 3
    with pytest.raises(S.SptError) as e:
        S.cpd_als(t, 65, 1, 0.0, init)
    assert e.value.code == 3


@pytest.mark.parametrize("case", ["cpd_3d", "cpd_4d"])
def test_hicoo_cpd_fits_match_reference(case):
    """sptgbCpdAlsHiCOO (HiCOO MTTKRP inside the same loop) from the same
    initial factors: the reference's per-iteration fits within 1e-4."""
    g = golden(case)
    ndims = [int(x) for x in g["ndims"]]
    rank, niters = int(g["rank"]), int(g["niters"])
    N = len(ndims)
    t = S.Tensor.from_arrays(ndims, g["inds"], g["vals"])
    h = S.HiCOO(t, 2, 4)
    init = [g["init%d" % m] for m in range(N)]
    facs, lam, fits, it = S.cpd_als_hicoo(h, rank, niters, 0.0, init)
    assert it == niters
    assert np.abs(fits - g["fits"]).max() <= FIT_TOL, (fits, g["fits"])
    for f in facs:
        assert np.allclose(np.linalg.norm(f.astype(np.float64), axis=0), 1.0, atol=1e-4)


def test_hicoo_cpd_matches_coo_cpd_on_skewed_tensor():
    spec = S.GenSpec()
    spec.seed = 21
    spec.nmodes = 3
    for m, d in enumerate([40_000, 20_000, 3_000]):
        spec.ndims[m] = d
    spec.coord_dist[0] = spec.coord_dist[1] = S.DIST_ZIPF
    spec.zipf_s[0] = spec.zipf_s[1] = 1.2
    spec.count = 300_000
    spec.value_dist = S.VAL_U01
    t = S.Tensor.generate(spec)
    ndims = t.ndims
    rng = np.random.default_rng(22)
    init = [rng.random((d, 16), dtype=np.float32) for d in ndims]
    _, lam_c, fits_c, _ = S.cpd_als(t, 16, 6, 0.0, init)
    h = S.HiCOO(t, 7, 12)
    _, lam_h, fits_h, _ = S.cpd_als_hicoo(h, 16, 6, 0.0, init)
    assert np.abs(fits_h - fits_c).max() <= FIT_TOL, (fits_h, fits_c)


def test_drop_in_cpd_als_hicoo_fills_rank_kruskal_tensor():
    g = golden("cpd_3d")
    ndims = [int(x) for x in g["ndims"]]
    t = S.Tensor.from_arrays(ndims, g["inds"], g["vals"])
    h = S.HiCOO(t, 2, 4)
    L = S.lib()
    k = S.RankKruskalS()
    nd = (C.c_uint32 * 3)(*ndims)
    assert L.sptNewRankKruskalTensor(C.byref(k), 3, nd, 4) == 0
    assert L.sptCpdAlsHiCOO(h.ptr(), 4, 5, 0.0, C.byref(k)) == 0
    assert np.isfinite(k.fit) and 0.0 < k.fit < 1.0
    for m in range(3):
        f = k.factors[m].contents
        a = np.ctypeslib.as_array(f.values, shape=(int(f.cap), int(f.stride)))[: ndims[m], :4]
        assert np.allclose(np.linalg.norm(a.astype(np.float64), axis=0), 1.0, atol=1e-4)
    assert not k.factors[3]
    L.sptFreeRankKruskalTensor(C.byref(k))


@pytest.mark.parametrize("dims,sb", [([3000, 2000, 500], 7), ([300, 200, 100, 50], 4)])
def test_resident_hicoo_mttkrp_equals_drop_in(dims, sb):
    torch = pytest.importorskip("torch")
    spec = S.GenSpec()
    spec.seed = 31
    spec.nmodes = len(dims)
    for m, d in enumerate(dims):
        spec.ndims[m] = d
    spec.count = 100_000
    spec.value_dist = S.VAL_UPM1
    t = S.Tensor.generate(spec)
    h = S.HiCOO(t, sb, sb + 3)
    N = len(dims)
    rank = 16
    mats = S.new_factors(dims, rank, seed=3)
    dev = [torch.from_numpy(mats[m].array()[: dims[m]].copy()).cuda() for m in range(N)]
    out = torch.zeros((max(dims), 16), device="cuda")
    dh = S.DeviceHicoo(h)
    for mode in range(N):
        order = [mode] + [(mode + i) % N for i in range(1, N)]
        ref = S.mttkrp_hicoo(h, mats, mode, mats_order=order)
        dh.mttkrp(mode, order, [d.data_ptr() for d in dev], rank, 16, out.data_ptr())
        torch.cuda.synchronize()
        got = out[: dims[mode], :rank].cpu().numpy()
        assert np.abs(got - ref).max() <= 1e-5 * np.abs(ref).max()
    dh.free()


def test_order5_cpd_against_oracle():
    rng = np.random.default_rng(55)
    ndims = [30, 25, 20, 15, 10]
    n = 30000
    inds = np.unique(np.stack([rng.integers(0, d, 2 * n) for d in ndims]).astype(np.uint32), axis=1)
    inds = inds[:, rng.permutation(inds.shape[1])[:n]]
    vals = rng.random(inds.shape[1], dtype=np.float32)
    t = S.Tensor.from_arrays(ndims, inds, vals)
    init = [rng.random((d, 6), dtype=np.float32) for d in ndims]
    facs, lam, fits, it = S.cpd_als(t, 6, 5, 0.0, init)
    _, _, ofits, _ = O.cpd_als(ndims, inds, vals, 6, 5, 0.0, init)
    assert np.abs(fits - ofits).max() <= FIT_TOL, (fits, ofits)
