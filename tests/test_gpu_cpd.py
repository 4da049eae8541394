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
