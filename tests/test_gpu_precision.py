"""MTTKRP precision study on the 4th-order uniform tensor (10,000 x 5,000 x
2,000 x 500, values U[-1,1), factors U[0,1)), ranks 16 and 64: FP32 factors
with FP32 accumulation and BF16 factor storage with FP32 accumulation, each
against the FP64 oracle (relative Frobenius error, every mode).

Bounds: FP32 <= 1e-5 (the parity bar); BF16 <= 1e-2 (a BF16 factor entry
carries a relative rounding error of at most 2^-9 ~ 2e-3; products of three
factors and sums with cancellation stay well inside 1e-2).

The default is the full 200M-nonzero study; SPTGB_PRECISION_NNZ sets another size,
and SPTGB_PRECISION_REPORT=<file> writes the error table as JSON.
"""
import json
import os

import numpy as np
import pytest

import oracle as O
import sptol_gb300 as S
from conftest import rel_fro

pytestmark = pytest.mark.gpu
DIMS = [10_000, 5_000, 2_000, 500]
NNZ = int(float(os.environ.get("SPTGB_PRECISION_NNZ", "200000000")))
FP32_TOL = 1e-5
BF16_TOL = 1e-2
_results = []


@pytest.fixture(scope="module")
def tensor():
    spec = S.GenSpec()
    spec.seed = 303
    spec.nmodes = 4
    for m, d in enumerate(DIMS):
        spec.ndims[m] = d
        spec.coord_dist[m] = S.DIST_UNIFORM
    spec.count = NNZ
    spec.merge_duplicates = 0
    spec.value_dist = S.VAL_UPM1
    t = S.Tensor.generate(spec)
    yield t
    report = os.environ.get("SPTGB_PRECISION_REPORT")
    if report and _results:
        with open(report, "w") as f:
            json.dump({"dims": DIMS, "nnz": NNZ, "values": "U[-1,1)", "factors": "U[0,1)", "results": _results}, f,
                      indent=1)


@pytest.mark.parametrize("rank", [16, 64], ids=lambda r: "nnz%d-rank%d" % (NNZ, r))
def test_fp32_and_bf16_against_fp64_oracle(tensor, rank):
    torch = pytest.importorskip("torch")
    t = tensor
    ndims = t.ndims
    inds, vals = t.arrays()
    mats = S.new_factors(ndims, rank, seed=rank)
    facs = [mats[m].array()[: ndims[m]].copy() for m in range(4)]
    stride = facs[0].shape[1]
    d32 = [torch.from_numpy(f).cuda() for f in facs]
    d16 = [f.to(torch.bfloat16).contiguous() for f in d32]
    out = torch.zeros((max(ndims), stride), dtype=torch.float32, device="cuda")
    coo = S.DeviceCoo(t)
    coo.set_timing(True)
    for mode in range(4):
        order = [mode] + [(mode + i) % 4 for i in range(1, 4)]
        coo.prepare(mode)
        ref = O.mttkrp(ndims, inds, vals, facs, rank, mode, precision="f64_omp")
        coo.mttkrp(mode, order, [p.data_ptr() for p in d32], rank, stride, out.data_ptr())
        torch.cuda.synchronize()
        e32 = rel_fro(out[: ndims[mode], :rank].cpu().numpy(), ref)
        coo.mttkrp(mode, order, [p.data_ptr() for p in d16], rank, stride, out.data_ptr(), bf16=True)
        torch.cuda.synchronize()
        e16 = rel_fro(out[: ndims[mode], :rank].cpu().numpy(), ref)
        # kernel time of a repeated call (CUDA events around the launch)
        ms = {}
        for key, ptrs, b in (("fp32", d32, False), ("bf16", d16, True)):
            coo.mttkrp(mode, order, [p.data_ptr() for p in ptrs], rank, stride, out.data_ptr(), bf16=b)
            ms[key] = coo.last_ms()
        _results.append({"rank": rank, "mode": mode, "fp32_rel_fro": e32, "bf16_rel_fro": e16,
                         "fp32_ms": ms["fp32"], "bf16_ms": ms["bf16"]})
        print("rank %d mode %d  fp32 %.3e  bf16 %.3e  (%.3f / %.3f ms)" % (rank, mode, e32, e16, ms["fp32"],
                                                                         ms["bf16"]))
        assert e32 <= FP32_TOL, (rank, mode, e32)
        assert e16 <= BF16_TOL, (rank, mode, e16)
        assert e16 > e32
    coo.free()
