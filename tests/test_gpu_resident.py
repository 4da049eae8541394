"""Device-resident extension API (sptgbCoo*): the kernels on caller device
buffers and a caller stream, FP32 and BF16 factor storage."""
import numpy as np
import pytest

import oracle as O
import sptol_gb300 as S
from conftest import rel_fro

pytestmark = pytest.mark.gpu


def _skewed(n, seed=3):
    spec = S.GenSpec()
    spec.seed = seed
    spec.nmodes = 3
    for m, d in enumerate([400_000, 200_000, 2_500]):
        spec.ndims[m] = d
    spec.coord_dist[0] = spec.coord_dist[1] = S.DIST_ZIPF
    spec.zipf_s[0] = spec.zipf_s[1] = 1.2
    spec.count = n
    spec.value_dist = S.VAL_LOGNORMAL
    return S.Tensor.generate(spec)


def test_resident_fp32_and_bf16_against_fp64_oracle():
    torch = pytest.importorskip("torch")
    t = _skewed(2_000_000)
    ndims = t.ndims
    inds, vals = t.arrays()
    rank = 32
    mats = S.new_factors(ndims, rank, seed=8)
    facs = [m.array()[: ndims[k]].copy() for k, m in enumerate(mats[:3])]
    dfac = [torch.from_numpy(f).cuda() for f in facs]
    dbf = [f.to(torch.bfloat16).contiguous() for f in dfac]
    out = torch.zeros((max(ndims), 32), device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    coo = S.DeviceCoo(t, stream=stream)
    for mode in range(3):
        order = [mode] + [(mode + i) % 3 for i in (1, 2)]
        ref64 = O.mttkrp(ndims, inds, vals, facs, rank, mode, precision="f64")
        coo.mttkrp(mode, order, [f.data_ptr() for f in dfac], rank, 32, out.data_ptr(), stream=stream)
        torch.cuda.synchronize()
        got = out[: ndims[mode]].cpu().numpy()
        assert rel_fro(got, ref64) <= 1e-5
        coo.mttkrp(mode, order, [f.data_ptr() for f in dbf], rank, 32, out.data_ptr(), stream=stream, bf16=True)
        torch.cuda.synchronize()
        got16 = out[: ndims[mode]].cpu().numpy()
        # BF16 rounding of the factors (8 significand bits): error of a sum of
        # products of two rounded factors stays below 2^-7 relative
        err = rel_fro(got16, ref64)
        assert err <= 2.0 ** -7, err
    coo.free()


def test_repeated_calls_are_deterministic_in_segments():
    torch = pytest.importorskip("torch")
    t = _skewed(300_000, seed=4)
    ndims = t.ndims
    rank = 16
    facs = [np.random.default_rng(k).random((d, 16), dtype=np.float32) for k, d in enumerate(ndims)]
    dfac = [torch.from_numpy(f).cuda() for f in facs]
    out = torch.zeros((max(ndims), 16), device="cuda")
    coo = S.DeviceCoo(t)
    res = []
    for _ in range(2):
        coo.mttkrp(1, [1, 2, 0], [f.data_ptr() for f in dfac], rank, 16, out.data_ptr())
        torch.cuda.synchronize()
        res.append(out[: ndims[1]].cpu().numpy().copy())
    # atomics touch only unit-boundary rows: results agree to FP32 rounding
    assert rel_fro(res[0], res[1]) <= 1e-6
    coo.free()
