"""Batched / served CP-ALS (sptgbServer*) on the GPU.

- every job's per-iteration fit equals the reference's (tests/golden) and the
  plain sptgbCpdAls path's within 1e-4;
- a job gives the same result alone and inside a mix of jobs of other orders,
  ranks and sizes that arrive while it runs: fits within 1e-6, factors within
  a relative Frobenius error of 1e-4 (the only differences are the FP32
  summation order at unit boundaries, which depends on the autotuned unit
  length, and the order of the boundary atomics);
- admission never exceeds the HBM budget, queued jobs start when space frees,
  and a job larger than the whole budget fails alone;
- the persistent cooperative step (SPTGB_STEP=persistent, one launch per
  step) gives the default kernel sequence's results on the same jobs.
"""
import ctypes as C
import os
import time

import numpy as np
import pytest

import sptol_gb300 as S
from conftest import golden, rel_fro

pytestmark = pytest.mark.gpu
FIT_TOL = 1e-4
MIX_FIT_TOL = 1e-6
MIX_FAC_TOL = 1e-4


def make_tensor(seed, dims, nnz):
    spec = S.GenSpec()
    spec.seed = seed
    spec.nmodes = len(dims)
    for m, d in enumerate(dims):
        spec.ndims[m] = d
        spec.coord_dist[m] = S.DIST_UNIFORM
    spec.count = nnz
    spec.merge_duplicates = 0
    spec.value_dist = S.VAL_U01
    return S.Tensor.generate(spec)


def init_for(dims, rank, seed):
    rng = np.random.default_rng(seed)
    return [rng.random((d, rank), dtype=np.float32) for d in dims]


JOBS = [  # (dims, nnz, rank)
    ([300, 200, 100], 5000, 8),
    ([1000, 500, 64], 20000, 32),
    ([100, 80, 60, 40], 10000, 16),
    ([200, 100, 70, 64], 8000, 64),
    ([4000, 3000, 2000], 60000, 16),
    ([90, 5000, 70, 300], 30000, 32),
    ([64, 64, 64], 1000, 64),
    ([20000, 100, 900], 100000, 8),
]


@pytest.mark.parametrize("case", ["cpd_3d", "cpd_4d"])
def test_server_fits_match_reference(case):
    g = golden(case)
    ndims = [int(x) for x in g["ndims"]]
    rank, niters = int(g["rank"]), int(g["niters"])
    t = S.Tensor.from_arrays(ndims, g["inds"], g["vals"])
    init = [g["init%d" % m] for m in range(len(ndims))]
    srv = S.Server(1 << 30, 8)
    k = srv.submit(t, rank, niters, init)
    srv.drain()
    facs, lam, fits = srv.result(k)
    assert np.abs(fits - g["fits"]).max() <= FIT_TOL, (fits, g["fits"])
    for f in facs:
        assert np.allclose(np.linalg.norm(f.astype(np.float64), axis=0), 1.0, atol=1e-4)


def test_batched_jobs_match_plain_path():
    niters = 6
    tensors = [make_tensor(100 + i, d, n) for i, (d, n, r) in enumerate(JOBS)]
    inits = [init_for(d, r, 200 + i) for i, (d, n, r) in enumerate(JOBS)]
    srv = S.Server(4 << 30, 64)
    tickets = [srv.submit(t, r, niters, ini) for t, (d, n, r), ini in zip(tensors, JOBS, inits)]
    a, q = srv.step()
    assert a == len(JOBS) and q == 0
    srv.drain()
    for t, (d, n, r), ini, k in zip(tensors, JOBS, inits, tickets):
        facs, lam, fits = srv.result(k)
        pf, plam, pfits, it = S.cpd_als(t, r, niters, 0.0, ini)
        assert it == niters
        assert np.abs(fits - pfits).max() <= FIT_TOL, (d, r, fits, pfits)
        assert rel_fro(lam, plam) <= 1e-2, (d, r)
    assert srv.bytes_in_use() == 0
    for g in range(4):
        assert srv.unit_length(g) in (64, 128, 256, 512)
        sch = srv.schedule(g)
        assert sch["unit"] == srv.unit_length(g)
        assert sch["blocks_per_sm"] in (2, 3) and sch["batches"] in ("deep", "shallow")
        assert sch["source"] in ("timed", "cached")   # every rank group has jobs in JOBS
    assert not srv.persistent()


def test_tuned_schedules_are_reused():
    """A second server given jobs of the same kinds takes every rank group's
    MTTKRP schedule from the process cache instead of timing again."""
    tensors = [make_tensor(700 + i, d, n) for i, (d, n, r) in enumerate(JOBS)]
    inits = [init_for(d, r, 800 + i) for i, (d, n, r) in enumerate(JOBS)]
    first = S.Server(4 << 30, 64)
    for t, (d, n, r), ini in zip(tensors, JOBS, inits):
        first.submit(t, r, 2, ini)
    first.drain()
    second = S.Server(4 << 30, 64)
    for t, (d, n, r), ini in zip(tensors, JOBS, inits):
        second.submit(t, r, 2, ini)
    second.drain()
    for g in range(4):
        a, b = first.schedule(g), second.schedule(g)
        assert b["source"] == "cached", (g, a, b)
        assert (a["unit"], a["batches"], a["blocks_per_sm"]) == (b["unit"], b["batches"], b["blocks_per_sm"])


def _run_mix(step_kind, niters=5):
    old = os.environ.get("SPTGB_STEP")
    if step_kind:
        os.environ["SPTGB_STEP"] = step_kind
    else:
        os.environ.pop("SPTGB_STEP", None)
    try:
        tensors = [make_tensor(500 + i, d, n) for i, (d, n, r) in enumerate(JOBS)]
        inits = [init_for(d, r, 600 + i) for i, (d, n, r) in enumerate(JOBS)]
        srv = S.Server(4 << 30, 64)
        n0 = S.launch_count()
        tickets = [srv.submit(t, r, niters + (i % 3), ini)
                   for i, (t, (d, n, r), ini) in enumerate(zip(tensors, JOBS, inits))]
        steps = 0
        while True:
            a, q = srv.step()
            if a == 0 and q == 0:
                break
            steps += 1
        out = [srv.result(k) for k in tickets]
        launches = S.launch_count() - n0
        kind = srv.persistent()
        assert srv.step_kernels() == (1 if kind else 38)
        srv.free()
        return out, kind, launches, steps
    finally:
        if old is None:
            os.environ.pop("SPTGB_STEP", None)
        else:
            os.environ["SPTGB_STEP"] = old


def test_persistent_step_matches_kernel_sequence():
    """Same jobs, same initial factors, staggered iteration counts: the
    one-launch persistent step and the ~38-launch kernel sequence agree to
    the FP32 atomic-order tolerance, and the persistent step launches far
    fewer kernels."""
    pers, kind_p, launches_p, steps_p = _run_mix("persistent")
    seq, kind_s, launches_s, steps_s = _run_mix(None)
    assert kind_p and not kind_s
    for (f1, l1, fit1), (f2, l2, fit2), (d, n, r) in zip(pers, seq, JOBS):
        assert fit1.shape == fit2.shape
        assert np.abs(fit1 - fit2).max() <= MIX_FIT_TOL, (d, r, fit1, fit2)
        for a, b in zip(f1, f2):
            assert rel_fro(a, b) <= MIX_FAC_TOL, (d, r)
        assert rel_fro(l1, l2) <= MIX_FAC_TOL
    assert steps_p == steps_s
    assert launches_s - launches_p >= 20 * steps_p


def test_same_result_alone_and_in_mix():
    niters = 8
    probe = ([3000, 700, 120, 90], 40000, 32)
    pt = make_tensor(7, probe[0], probe[1])
    pinit = init_for(probe[0], probe[2], 8)

    alone = S.Server(2 << 30, 4)
    k = alone.submit(pt, probe[2], niters, pinit)
    alone.drain()
    f1, l1, fit1 = alone.result(k)

    others = [make_tensor(300 + i, d, n) for i, (d, n, r) in enumerate(JOBS)]
    oinit = [init_for(d, r, 400 + i) for i, (d, n, r) in enumerate(JOBS)]
    mix = S.Server(4 << 30, 16)
    for i in range(3):
        mix.submit(others[i], JOBS[i][2], niters + i, oinit[i])
    mix.step()
    mix.step()
    kp = mix.submit(pt, probe[2], niters, pinit)  # arrives while others run
    for i in range(3, 6):
        mix.submit(others[i], JOBS[i][2], 3 + i, oinit[i])
    mix.step()
    for i in range(6, len(JOBS)):
        mix.submit(others[i], JOBS[i][2], niters, oinit[i])
    mix.drain()
    f2, l2, fit2 = mix.result(kp)
    assert np.abs(fit1 - fit2).max() <= MIX_FIT_TOL, (fit1, fit2)
    for a, b in zip(f1, f2):
        assert rel_fro(b, a) <= MIX_FAC_TOL
    assert rel_fro(l2, l1) <= MIX_FAC_TOL


def test_budget_gates_admission():
    niters = 4
    dims, nnz, rank = [2000, 1500, 300], 30000, 16
    ts = [make_tensor(500 + i, dims, nnz) for i in range(6)]
    inits = [init_for(dims, rank, 600 + i) for i in range(6)]

    probe = S.Server(1 << 30, 4)
    probe.submit(ts[0], rank, niters, inits[0])
    probe.step()
    job_bytes = probe.bytes_in_use()
    assert job_bytes > 0
    probe.drain()
    assert probe.bytes_in_use() == 0

    budget = int(2.5 * job_bytes)
    srv = S.Server(budget, 16)
    ks = [srv.submit(t, rank, niters, ini) for t, ini in zip(ts, inits)]
    a, q = srv.step()
    assert (a, q) == (2, 4)
    assert srv.bytes_in_use() <= budget
    peak = 0
    while a or q:
        a, q = srv.step()
        assert a <= 2
        peak = max(peak, srv.bytes_in_use())
    assert peak <= budget
    # FIFO: the jobs finish in pairs, in submission order
    done = [srv.state(k)[2] for k in ks]
    assert done[0] <= done[2] <= done[4] and done[1] <= done[3] <= done[5]
    for t, ini, k in zip(ts, inits, ks):
        facs, lam, fits = srv.result(k)
        pf, plam, pfits, it = S.cpd_als(t, rank, niters, 0.0, ini)
        assert np.abs(fits - pfits).max() <= FIT_TOL


def test_job_larger_than_budget_fails_alone():
    small = make_tensor(900, [200, 100, 80], 3000)
    big = make_tensor(901, [50000, 20000, 3000], 400000)
    srv = S.Server(4 << 20, 4)
    kb = srv.submit(big, 32, 3, init_for([50000, 20000, 3000], 32, 1))
    ks = srv.submit(small, 8, 3, init_for([200, 100, 80], 8, 2))
    srv.drain()
    assert srv.state(kb)[0] == S.Server.FAILED
    assert srv.state(ks)[0] == S.Server.DONE
    facs, lam, fits = srv.result(ks)
    assert np.all(np.isfinite(fits))


def test_single_slot_server_serialises():
    niters = 3
    sel = [JOBS[0], JOBS[2], JOBS[6]]
    ts = [make_tensor(700 + i, d, n) for i, (d, n, r) in enumerate(sel)]
    inits = [init_for(d, r, 800 + i) for i, (d, n, r) in enumerate(sel)]
    srv = S.Server(1 << 30, 1)
    ks = [srv.submit(t, r, niters, ini) for t, (d, n, r), ini in zip(ts, sel, inits)]
    a, q = srv.step()
    assert (a, q) == (1, 2)
    srv.drain()
    for t, (d, n, r), ini, k in zip(ts, sel, inits, ks):
        facs, lam, fits = srv.result(k)
        pf, plam, pfits, it = S.cpd_als(t, r, niters, 0.0, ini)
        assert np.abs(fits - pfits).max() <= FIT_TOL


def test_grid_barrier_wait_is_bounded():
    """The persistent step's grid barrier: complete rounds pass with no error;
    a round that waits for a block the grid does not have gives up after its
    bounded wait with the error word set, the kernel returns, and the context
    stays usable."""
    L = S.lib()
    err, rounds = C.c_int(-1), C.c_uint(0)
    assert L.sptgbGridBarrierSelfTest(0, C.byref(err), C.byref(rounds)) == 0
    assert err.value == 0 and rounds.value == 8
    t0 = time.monotonic()
    assert L.sptgbGridBarrierSelfTest(1, C.byref(err), C.byref(rounds)) == 0
    assert err.value == 1 and rounds.value == 8
    assert time.monotonic() - t0 < 30.0
    t = make_tensor(9, [50, 40, 30], 2000)
    srv = S.Server(1 << 28, 2)
    k = srv.submit(t, 8, 2, init_for([50, 40, 30], 8, 10))
    srv.drain()
    assert np.all(np.isfinite(srv.result(k)[2]))


def test_rank_group_tuned_when_it_first_gets_jobs():
    """Jobs of a new rank group arriving after the first step get a tuned
    schedule of their own before their first iteration."""
    srv = S.Server(4 << 30, 16)
    t8 = make_tensor(901, [300, 200, 100], 5000)
    k8 = srv.submit(t8, 8, 6, init_for([300, 200, 100], 8, 902))
    srv.step()
    srv.step()
    assert srv.schedule(0)["source"] in ("timed", "cached")
    assert srv.schedule(3)["source"] == "no jobs"
    t64 = make_tensor(903, [200, 100, 70, 64], 8000)
    k64 = srv.submit(t64, 64, 3, init_for([200, 100, 70, 64], 64, 904))
    srv.drain()
    assert srv.schedule(3)["source"] in ("timed", "cached")
    for k in (k8, k64):
        assert np.all(np.isfinite(srv.result(k)[2]))
