#!/usr/bin/env python
"""MTTKRP throughput on the 100M-nonzero power-law tensor.

Workload (one "step" = MTTKRP of every mode, 0, 1, 2, on one GPU):
  3rd-order COO tensor 4,000,000 x 2,000,000 x 25,000 with exactly 100,000,000
  unique nonzeros; modes 0 and 1 truncated Zipf(1.2), mode 2 uniform; values
  lognormal(0,1) float32; rank 32 float32 factors U[0,1).  Seeded synthetic
  data from the library generator (sptgbGenerate).

  value   GB/s by the reference's algorithmic byte count per MTTKRP,
          nnz*(4N+4) + sum_m I_m*R*4 (src/sptensor/mttkrp_cuda_onekernel.cu:94-97),
          with tensor copies and factors resident in HBM (sptgbCoo*).
  e2e     the same metric through the drop-in C entry point sptCudaMTTKRP with
          host buffers in page-locked memory from cudaHostAlloc (a caller that
          allocates its arrays for the GPU): every call copies the tensor and
          factors to the GPU, sorts by the output mode when needed and copies
          the result back; beside it the same calls on arrays page-locked with
          cudaHostRegister (sptgbPinSparseTensor / sptgbPinMatrix).
  roofline  the segmented MTTKRP launch (output memset + k_mttkrp_rec), per
          launch duration from CUDA events on the launching stream.
  cpu_baseline  the oracle port of sptOmpMTTKRP_Reduce (all host threads) on
          a 10M-nonzero sample tensor of the same shape and distributions.
  hicoo   the same tensor as HiCOO (blocks 2^7, kernels 2^17): conversion time
          and sptMTTKRPHiCOO per mode (kernel time from CUDA events); its
          cpu_baseline is the oracle port of
          sptOmpMTTKRPHiCOO_MatrixTiling_Scheduled_Reduce (all host threads)
          on the HiCOO form of the 10M-nonzero sample.  With --hicoo4,
          hicoo.order4 adds order-4 HiCOO against the order-4 record kernel on
          two 50M-draw tensors (uniform and power-law), kernel times per mode.
  serve   the batched / served CP-ALS stream: 4,096 requests of order 3 or 4
          (50/50), mode sizes log-uniform in [64, 100,000], nnz log-uniform in
          [1e3, 1e6] (at most half the index space, unique uniform
          coordinates), values U[0,1), rank from {8,16,32,64}, 10 ALS
          iterations each, Poisson arrivals at 2,000/s, 120 GB HBM budget.
          "served" replays the arrivals through sptgbServer (continuous
          batching), "batched" submits every request at once and drains, and
          "plain" runs one sptgbCpdAls call per request (its own upload, sort
          and per-iteration launches) on a sample of the stream, back to back.
          Latency = completion - arrival; solves/s = requests / makespan.
--impl reference times that CPU implementation alone (the reference's own
library when it was built here, else the port), per step all three modes of
the sample tensor.  With torchrun each rank runs its own replica (the path
does not shard); value is the sum over ranks over the slowest rank's time.
"""
import argparse
import ctypes
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

DIMS = [4_000_000, 2_000_000, 25_000]
ZIPF = [1.2, 1.2, None]
RANK = 32
SEED = 20261203
METRIC = "MTTKRP GB/s (algorithmic bytes, all 3 modes, 100M-nnz power-law COO, rank 32)"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=300)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--nnz", type=int, default=100_000_000)
    p.add_argument("--cpu-sample", type=int, default=10_000_000)
    p.add_argument("--e2e-steps", type=int, default=20)
    p.add_argument("--skip-cpu", action="store_true")
    p.add_argument("--serve-requests", type=int, default=4096)
    p.add_argument("--plain-sample", type=int, default=256)
    p.add_argument("--serve-cpu-sample", type=int, default=32)
    p.add_argument("--skip-serve", action="store_true")
    p.add_argument("--skip-hicoo", action="store_true")
    p.add_argument("--hicoo4", action="store_true", help="also time order-4 HiCOO against order-4 COO")
    p.add_argument("--skip-registered", action="store_true")
    p.add_argument("--skip-c1", action="store_true")
    p.add_argument("--skip-cpals", action="store_true")
    p.add_argument("--cpals-nnz", type=int, default=50_000_000)
    p.add_argument("--skip-ref-gpu", action="store_true")
    return p.parse_args()


def spec_for(count, seed=SEED):
    import sptol_gb300 as S
    s = S.GenSpec()
    s.seed = seed
    s.nmodes = 3
    for m, d in enumerate(DIMS):
        s.ndims[m] = d
        if ZIPF[m]:
            s.coord_dist[m] = S.DIST_ZIPF
            s.zipf_s[m] = ZIPF[m]
        else:
            s.coord_dist[m] = S.DIST_UNIFORM
    s.count = count
    s.merge_duplicates = 0
    s.value_dist = S.VAL_LOGNORMAL
    return s


def host_link_gbs(nbytes=1 << 30, reps=3):
    """Host-to-device copy rate of this machine from page-locked memory (GB/s),
    the floor of the host-buffer path on pinned caller arrays."""
    import torch
    try:
        h = torch.ones(nbytes // 4, dtype=torch.float32).pin_memory()
        d = torch.empty(nbytes // 4, dtype=torch.float32, device="cuda")
        d.copy_(h)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            d.copy_(h)
        torch.cuda.synchronize()
        gbs = reps * nbytes / (time.perf_counter() - t0) / 1e9
        del d, h
        torch.cuda.empty_cache()
        return round(gbs, 1)
    except Exception:
        return None


def workload_config(nnz, world):
    """The workload both arms report: the 100M-nonzero power-law tensor at
    rank 32 (the reference arm times a bounded sample of it, described in its
    cpu_baseline)."""
    return {"workload": "mttkrp_powerlaw_coo_4Mx2Mx25K_100Mnnz_rank32", "dims": DIMS, "nnz": nnz,
            "zipf": ZIPF, "values": "lognormal(0,1)", "rank": RANK, "modes_per_step": 3,
            "l2": "inputs larger than L2 (1.6 GB nonzero stream per launch)",
            "parallelism": "replicas" if world > 1 else "single"}


def algo_bytes(ndims, nnz, rank):
    N = len(ndims)
    return nnz * (4 * N + 4) + sum(d * rank * 4 for d in ndims)


SERVE_RATE = 2000.0
SERVE_BUDGET = 120 * 10**9
SERVE_ITERS = 10
SERVE_SEED = 5150


def serve_stream(n, seed=SERVE_SEED):
    """The request stream: arrival time, order, mode sizes, nnz, rank."""
    rng = np.random.default_rng(seed)
    t = 0.0
    reqs = []
    for i in range(n):
        t += rng.exponential(1.0 / SERVE_RATE)
        order = 3 if rng.random() < 0.5 else 4
        dims = [int(round(math.exp(rng.uniform(math.log(64), math.log(100_000))))) for _ in range(order)]
        nnz = int(round(math.exp(rng.uniform(math.log(1e3), math.log(1e6)))))
        nnz = max(1, min(nnz, int(0.5 * math.prod(dims))))
        rank = int(rng.choice([8, 16, 32, 64]))
        reqs.append({"arrival": t, "dims": dims, "nnz": nnz, "rank": rank, "seed": seed * 100_003 + i})
    return reqs


def request_tensor(r):
    import sptol_gb300 as S
    s = S.GenSpec()
    s.seed = r["seed"]
    s.nmodes = len(r["dims"])
    for m, d in enumerate(r["dims"]):
        s.ndims[m] = d
        s.coord_dist[m] = S.DIST_UNIFORM
    s.count = r["nnz"]
    s.merge_duplicates = 0
    s.value_dist = S.VAL_U01
    return S.Tensor.generate(s)


def request_init(r):
    """Initial factors U[0,1) from the library's seeded filler."""
    import sptol_gb300 as S
    L = S.lib()
    mats = []
    for m, d in enumerate(r["dims"]):
        M = S.Matrix(d, r["rank"], zero=False)
        L.sptgbFillMatrix(ctypes.byref(M.s), r["seed"], m, 0.0, 1.0)
        mats.append(M)
    return mats


def run_plain(reqs, tensors, inits, count):
    """One sptgbCpdAls call per request, in arrival order, back to back.
    The calls overwrite inits[i] with the results."""
    import sptol_gb300 as S
    L = S.lib()
    lat, fits = [], []
    t0 = time.monotonic()
    for i in range(count):
        r = reqs[i]
        wait = r["arrival"] - (time.monotonic() - t0)
        if wait > 0:
            time.sleep(wait)
        mats = inits[i] + [S.Matrix(max(r["dims"]), r["rank"], zero=False)]
        arr = (ctypes.POINTER(S.MatrixS) * len(mats))(*[ctypes.pointer(m.s) for m in mats])
        lam = np.zeros(r["rank"], np.float32)
        f = np.zeros(SERVE_ITERS, np.float64)
        done = ctypes.c_uint32()
        rc = L.sptgbCpdAls(tensors[i].ptr(), r["rank"], SERVE_ITERS, 0.0, arr,
                           lam.ctypes.data_as(S.f32p), f.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                           ctypes.byref(done))
        if rc:
            raise RuntimeError("sptgbCpdAls failed on request %d" % i)
        lat.append(time.monotonic() - t0 - r["arrival"])
        fits.append(f)
    span = time.monotonic() - t0 - reqs[0]["arrival"]
    return {"solves_per_s": count / span, "makespan_s": span, "lat": np.array(lat), "fits": fits}


def run_served(reqs, tensors, inits, outs, poisson, keep_fits):
    """sptgbServer: requests submitted at their arrival times (poisson) or all
    at once; one ALS iteration of every admitted job per step; finished jobs
    taken from the server's completion queue."""
    import sptol_gb300 as S
    n = len(reqs)
    srv = S.Server(SERVE_BUDGET, n)
    lat = np.zeros(n)
    fits = {}
    index = {}
    i = 0
    done = 0
    active = queued = 0
    steps = 0
    n0 = S.launch_count()
    t_sub = t_step = t_poll = 0.0
    t0 = time.monotonic()
    if not poisson:
        for r_i, r in enumerate(reqs):
            index[srv.submit(tensors[r_i], r["rank"], SERVE_ITERS, inits[r_i], outs[r_i])] = r_i
        i = n
        queued = n
        t_sub = time.monotonic() - t0
    while done < n:
        now = time.monotonic() - t0
        a0 = time.monotonic()
        while poisson and i < n and reqs[i]["arrival"] <= now:
            index[srv.submit(tensors[i], reqs[i]["rank"], SERVE_ITERS, inits[i], outs[i])] = i
            i += 1
            queued += 1
        a1 = time.monotonic()
        t_sub += a1 - a0
        if active or queued:
            active, queued = srv.step()
            steps += 1
        elif i < n:
            time.sleep(max(0.0, reqs[i]["arrival"] - (time.monotonic() - t0)))
            continue
        a2 = time.monotonic()
        t_step += a2 - a1
        for k in srv.completed():
            r_i = index.pop(k)
            st, _, t_done = srv.state(k)
            if st != S.Server.DONE:
                raise RuntimeError("served request %d failed" % r_i)
            lat[r_i] = t_done - t0 - (reqs[r_i]["arrival"] if poisson else 0.0)
            f = srv.result(k, copy=False)[2]
            if r_i < keep_fits:
                fits[r_i] = f.copy()
            done += 1
        t_poll += time.monotonic() - a2
    span = time.monotonic() - t0 - (reqs[0]["arrival"] if poisson else 0.0)
    launches = S.launch_count() - n0
    units = {g: srv.schedule(g) for g in range(4)}
    persistent = srv.persistent()
    step_kernels = srv.step_kernels()
    srv.free()
    return {"solves_per_s": n / span, "makespan_s": span, "lat": lat, "fits": fits, "steps": steps,
            "launches": int(launches), "schedules": units, "persistent": persistent, "step_kernels": step_kernels,
            "host_s": {"submit": round(t_sub, 3), "step": round(t_step, 3), "poll": round(t_poll, 3)}}


def hicoo_leg(t, mats, ndims, nnz, reps):
    """HiCOO (block 2^7, kernel 2^17) conversion and sptMTTKRPHiCOO of every
    mode on the same tensor; kernel time from CUDA events around the HiCOO
    kernel (output memset included), call time around the drop-in call."""
    import sptol_gb300 as S
    L = S.lib()
    N = len(ndims)
    c0 = time.time()
    h = S.HiCOO(t, 7, 17)
    conv_s = time.time() - c0
    nb = int(h.s.bptr.len) - 1
    arr = S._mat_array(mats)
    L.sptgbHiCOOSetTiming(1)
    kern, call = [], []
    for m in range(N):
        order = (ctypes.c_uint32 * N)(*([m] + [(m + i) % N for i in range(1, N)]))
        mats[N].s.nrows = ndims[m]
        if L.sptMTTKRPHiCOO(h.ptr(), arr, order, m):
            raise RuntimeError("sptMTTKRPHiCOO failed")
        ks, cs = [], []
        for _ in range(reps):
            a = time.perf_counter()
            L.sptMTTKRPHiCOO(h.ptr(), arr, order, m)
            cs.append(time.perf_counter() - a)
            ks.append(float(L.sptgbHiCOOLastKernelMs()))
        kern.append(float(np.median(ks)))
        call.append(float(np.median(cs)) * 1e3)
    L.sptgbHiCOOSetTiming(0)
    h.free()
    # the reference's HiCOO byte count per MTTKRP: values + 1-byte element
    # indices per nonzero, bptr + block indices per block, factor rows
    hb = nnz * (4 + N) + nb * (8 + 4 * N) + sum(d * RANK * 4 for d in ndims)
    return {"sb_bits": 7, "sk_bits": 17, "blocks": nb, "convert_s": round(conv_s, 2),
            "kernel_ms_by_mode": [round(x, 4) for x in kern], "call_ms_by_mode": [round(x, 2) for x in call],
            "algorithmic_bytes_per_mttkrp": hb,
            "kernel_gbs": round(N * hb / (sum(kern) / 1e3) / 1e9, 1),
            "coo_bytes_gbs": round(N * algo_bytes(ndims, nnz, RANK) / (sum(kern) / 1e3) / 1e9, 1)}


def hicoo4_leg(reps=3):
    """Order-4 HiCOO (blocks 2^7, kernels 2^17) against the order-4 record
    kernel on the same tensors: a uniform 10K x 5K x 2K x 500 and a power-law
    2M x 1M x 50K x 500 (Zipf(1.2) in the first two modes), 50M draws each,
    values U[-1,1), rank 16.  Kernel times (output memset included) from CUDA
    events, median of `reps` calls per mode after one warm-up call."""
    import torch
    import sptol_gb300 as S
    L = S.lib()
    rank = stride = 16
    out = {}
    for name, dims, zipf in (("uniform_10Kx5Kx2Kx500", [10_000, 5_000, 2_000, 500], [0, 0, 0, 0]),
                             ("zipf_2Mx1Mx50Kx500", [2_000_000, 1_000_000, 50_000, 500], [1.2, 1.2, 0, 0])):
        spec = S.GenSpec()
        spec.seed = SEED + 4
        spec.nmodes = 4
        for m, d in enumerate(dims):
            spec.ndims[m] = d
            spec.coord_dist[m] = S.DIST_ZIPF if zipf[m] else S.DIST_UNIFORM
            spec.zipf_s[m] = zipf[m]
        spec.count = 50_000_000
        spec.value_dist = S.VAL_UPM1
        t = S.Tensor.generate(spec)
        nd = t.ndims
        mats = S.new_factors(nd, rank, seed=3)
        h = S.HiCOO(t, 7, 17)
        nb = int(h.s.bptr.len) - 1
        L.sptgbHiCOOSetTiming(1)
        hk = []
        for m in range(4):
            S.mttkrp_hicoo(h, mats, m)
            ks = []
            for _ in range(reps):
                S.mttkrp_hicoo(h, mats, m)
                ks.append(float(L.sptgbHiCOOLastKernelMs()))
            hk.append(round(float(np.median(ks)), 3))
        L.sptgbHiCOOSetTiming(0)
        h.free()
        dc = S.DeviceCoo(t)
        facs = [torch.from_numpy(mats[m].array()[: nd[m]].copy()).cuda() for m in range(4)]
        ptrs = [f.data_ptr() for f in facs]
        dout = torch.zeros((max(nd), stride), dtype=torch.float32, device="cuda")
        dc.set_timing(True)
        ck = []
        for m in range(4):
            order = [m] + [(m + j) % 4 for j in (1, 2, 3)]
            dc.prepare(m)
            dc.mttkrp(m, order, ptrs, rank, stride, dout.data_ptr())
            ks = []
            for _ in range(reps):
                dc.mttkrp(m, order, ptrs, rank, stride, dout.data_ptr())
                ks.append(dc.last_ms())
            ck.append(round(float(np.median(ks)), 3))
        dc.free()
        del facs, dout
        out[name] = {"nnz": int(t.nnz), "blocks": nb, "hicoo_kernel_ms_by_mode": hk, "coo_kernel_ms_by_mode": ck}
        t.free()
    return out


def hicoo_cpu_leg(sample_nnz, reps):
    """sptOmpMTTKRPHiCOO_MatrixTiling_Scheduled_Reduce restated (oracle) with
    all host threads on a bounded sample of the workload (HiCOO built by the
    library's conversion): GB/s on the same HiCOO byte count as the GPU leg."""
    import oracle as O
    import sptol_gb300 as S
    O.build(with_ref=False)
    threads = os.cpu_count() or 1
    t = S.Tensor.generate(spec_for(sample_nnz, seed=SEED + 1))
    mats = S.new_factors(DIMS, RANK, seed=2)
    h = S.HiCOO(t, 7, 17)
    A = h.arrays()
    nb = len(A["bptr"]) - 1
    _, vals = t.arrays()
    facs = [m.array()[: t.ndims[i]] for i, m in enumerate(mats[:3])]
    rows = [O.kschr_rows(A, t.ndims, 17, m) for m in range(3)]
    h.free()
    copies = np.zeros(threads * max(t.ndims) * mats[0].s.stride, np.float32)
    secs = []
    for r in range(reps + 1):
        t0 = time.perf_counter()
        for m in range(3):
            O.omp_mttkrp_hicoo_reduce(t.ndims, A, vals, 7, facs, RANK, m, threads, rows[m], copies=copies)
        if r > 0:
            secs.append(time.perf_counter() - t0)
    step = float(np.mean(secs))
    hb = t.nnz * 7 + nb * 20 + sum(d * RANK * 4 for d in t.ndims)
    return {"value": round(3 * hb / step / 1e9, 3), "unit": "GB/s", "cores": threads, "kind": "port",
            "sample": ("%d-nnz tensor of the same shape and distributions (%d HiCOO blocks), all 3 modes, %d reps "
                       "after 1 warm-up, sptOmpMTTKRPHiCOO_MatrixTiling_Scheduled_Reduce with %d threads"
                       % (t.nnz, nb, reps, threads)),
            "seconds_per_step": step}


def serve_cpu_leg(reqs, tensors, count):
    """The reference's sptOmpCpdAls loop (OmpCpdAlsStep, use_reduce = 1,
    every host thread) run on the stream's first `count` requests one after
    another from the same initial factors as the GPU runs: seconds per
    request (a CPU figure for context; the reference has no GPU CP-ALS)."""
    import oracle as O
    if count <= 0 or not O.ref_loadable():
        return None
    threads = os.cpu_count() or 1
    secs, fits = [], []
    for i in range(min(count, len(reqs))):
        r = reqs[i]
        init = [m.array()[: d, : r["rank"]].copy() for m, d in zip(request_init(r), r["dims"])]
        inds, vals = tensors[i].arrays()
        sec, fit, _ = O.ref_omp_cpd(r["dims"], inds, vals, r["rank"], SERVE_ITERS, init, threads)
        secs.append(sec)
        fits.append(fit)
    return {"kind": "reference", "cores": threads, "requests": len(secs),
            "solves_per_s": round(len(secs) / sum(secs), 2), "mean_s_per_request": round(float(np.mean(secs)), 4),
            "sample": "first %d requests of the stream, %d iterations each, OmpCpdAlsStep (use_reduce = 1, tol 0), "
                      "one request at a time with %d threads" % (len(secs), SERVE_ITERS, threads)}


def serve_leg(args):
    import sptol_gb300 as S
    reqs = serve_stream(args.serve_requests)
    g0 = time.time()
    tensors = [request_tensor(r) for r in reqs]
    inits = [request_init(r) for r in reqs]
    # result buffers, allocated and touched once, reused by both server runs
    outs = [[S.Matrix(d, r["rank"]) for d in r["dims"]] for r in reqs]
    gen_s = time.time() - g0
    nnz_total = sum(t.nnz for t in tensors)
    sample = min(args.plain_sample, len(reqs))
    # warm-up: library context, device buffers, kernel modules
    warm = serve_stream(4, seed=SERVE_SEED + 1)
    wt = [request_tensor(r) for r in warm]
    run_plain(warm, wt, [request_init(r) for r in warm], 2)
    run_served(warm, wt, [request_init(r) for r in warm], [[S.Matrix(d, r["rank"]) for d in r["dims"]] for r in warm],
               poisson=False, keep_fits=0)
    batched = run_served(reqs, tensors, inits, outs, poisson=False, keep_fits=sample)
    # the same batched run with each ALS step as one persistent cooperative
    # kernel instead of the kernel sequence (SPTGB_STEP=persistent)
    os.environ["SPTGB_STEP"] = "persistent"
    try:
        pers = run_served(reqs, tensors, inits, outs, poisson=False, keep_fits=sample)
    finally:
        os.environ.pop("SPTGB_STEP", None)
    served = run_served(reqs, tensors, inits, outs, poisson=True, keep_fits=sample)
    # the same arrivals as the plain run: the stream's first `sample`
    # requests, so that served and plain latencies cover one population
    prefix = run_served(reqs[:sample], tensors[:sample], inits[:sample], outs[:sample], poisson=True,
                        keep_fits=sample)
    cpu = serve_cpu_leg(reqs, tensors, args.serve_cpu_sample)
    plain = run_plain(reqs, tensors, inits, sample)   # last: overwrites inits[:sample]
    # fit agreement: requests on which the ALS iteration stays well defined in
    # both paths.  A run diverges when a fit is not finite, negative, or drops
    # by more than 0.01 (ALS fits do not decrease); that happens on requests
    # whose Gram Hadamard products are singular (rank 32-64 with a few
    # thousand nonzeros over 1e4-1e5 rows), where every arithmetic path
    # breaks down differently.
    def diverged(f):
        return (not np.all(np.isfinite(f))) or f.min() < 0.0 or (np.diff(f).min(initial=0.0) < -0.01)

    diffs, div = [], []
    for i in range(sample):
        runs = (served["fits"][i], batched["fits"][i], plain["fits"][i])
        if any(diverged(f) for f in runs):
            div.append(i)
            continue
        diffs.append(max(float(np.abs(served["fits"][i] - plain["fits"][i]).max()),
                         float(np.abs(batched["fits"][i] - plain["fits"][i]).max())))
    dfit = max(diffs) if diffs else None
    pdiff = [float(np.abs(pers["fits"][i] - batched["fits"][i]).max()) for i in range(sample) if i not in div]
    # the requests left out: the reference's own CP-ALS loop (CpdAlsStep's
    # steps through its exported pieces, corrected fit per iteration) from
    # the same initial factors, judged by the same rule
    ref_div = {}
    try:
        import oracle as O
        if O.ref_loadable():
            for i in div:
                r = reqs[i]
                init = [m.array()[:d, : r["rank"]].copy() for m, d in zip(request_init(r), r["dims"])]
                inds, vals = tensors[i].arrays()
                with O.quiet_stdout():
                    tr = O.ref_cpd_trace(r["dims"], inds, vals, r["rank"], SERVE_ITERS, init)
                ref_div[i] = {"reference_fits": [float(x) for x in tr["fits"]],
                              "reference_diverges": bool(diverged(np.asarray(tr["fits"])))}
    except Exception as e:   # informational only
        ref_div = {"error": str(e)[:200]}

    def pct(a, q):
        return round(float(np.percentile(a, q)) * 1e3, 2)

    return {
        "workload": "cpals_stream_4096req_order3or4_dims64-1e5_nnz1e3-1e6_rank8-64_10it_poisson2000_120GB"
        if len(reqs) == 4096 else "cpals_stream_%dreq" % len(reqs),
        "requests": len(reqs), "nnz_total": int(nnz_total), "iterations": SERVE_ITERS,
        "served": {"solves_per_s": round(served["solves_per_s"], 1), "p50_ms": pct(served["lat"], 50),
                   "p99_ms": pct(served["lat"], 99), "makespan_s": round(served["makespan_s"], 3),
                   "steps": served["steps"], "gpu_launches": served["launches"],
                   "kernels_per_als_step": served["step_kernels"],
                   "mttkrp_schedule_by_rank": {"<=%d" % (8 << g): v for g, v in served["schedules"].items()},
                   "persistent_step": served["persistent"],
                   "host_s": served["host_s"]},
        "batched": {"solves_per_s": round(batched["solves_per_s"], 1), "p50_ms": pct(batched["lat"], 50),
                    "p99_ms": pct(batched["lat"], 99), "makespan_s": round(batched["makespan_s"], 3),
                    "steps": batched["steps"], "gpu_launches": batched["launches"],
                    "kernels_per_als_step": batched["step_kernels"],
                    "mttkrp_schedule_by_rank": {"<=%d" % (8 << g): v for g, v in batched["schedules"].items()},
                    "persistent_step": batched["persistent"], "host_s": batched["host_s"]},
        "batched_persistent_step": {
            "solves_per_s": round(pers["solves_per_s"], 1), "makespan_s": round(pers["makespan_s"], 3),
            "steps": pers["steps"], "gpu_launches": pers["launches"], "persistent_step": pers["persistent"],
            "kernels_per_als_step": pers["step_kernels"],
            "launches_note": "gpu_launches also counts admission (sorts, packing, Grams) and retirement kernels",
            "max_fit_diff_vs_batched": max(pdiff) if pdiff else None,
            "what": "the batched run with each ALS step as one persistent cooperative kernel"},
        "plain": {"solves_per_s": round(plain["solves_per_s"], 1), "p50_ms": pct(plain["lat"], 50),
                  "p99_ms": pct(plain["lat"], 99), "makespan_s": round(plain["makespan_s"], 3),
                  "sample": "first %d requests of the same stream at their arrival times, one at a time "
                            "(latency = completion - arrival)" % sample},
        "served_same_requests_as_plain": {
            "solves_per_s": round(prefix["solves_per_s"], 1), "p50_ms": pct(prefix["lat"], 50),
            "p99_ms": pct(prefix["lat"], 99), "makespan_s": round(prefix["makespan_s"], 3),
            "steps": prefix["steps"], "gpu_launches": prefix["launches"],
            "sample": "first %d requests of the same stream at their arrival times through sptgbServer" % sample},
        "cpu_baseline": cpu,
        "served_over_plain": round(served["solves_per_s"] / plain["solves_per_s"], 2),
        "served_over_plain_same_requests": round(prefix["solves_per_s"] / plain["solves_per_s"], 2),
        "batched_over_plain": round(batched["solves_per_s"] / plain["solves_per_s"], 2),
        "fit_match": {"compared": sample, "well_posed": len(diffs), "max_diff_vs_plain": dfit, "tolerance": 1e-4,
                      "within_tolerance": int(sum(d <= 1e-4 for d in diffs)),
                      "diverged": [dict({"request": i, "dims": reqs[i]["dims"], "nnz": int(tensors[i].nnz),
                                         "rank": reqs[i]["rank"], "plain_fits": [float(x) for x in plain["fits"][i]]},
                                        **(ref_div.get(i, {}) if isinstance(ref_div, dict) else {}))
                                   for i in div]},
        "generate_s": round(gen_s, 1),
    }


class HostAllocCopy:
    """A second host copy of a tensor and its factor matrices in memory from
    cudaHostAlloc (torch's pinned allocator), described by sptSparseTensor /
    sptMatrix structures that point into it: the e2e leg's inputs allocated as
    page-locked memory instead of registered (cudaHostRegister) caller memory."""

    def __init__(self, t, mats):
        import torch
        import sptol_gb300 as S
        self.keep = []
        N, n = t.nmodes, t.nnz
        self.nmodes, self.ndims = N, t.ndims
        x = S.SparseTensorS()
        x.nmodes = N
        so = (ctypes.c_uint32 * N)(*t.sortorder)
        nd = (ctypes.c_uint32 * N)(*t.ndims)
        iv = (S.IndexVector * N)()
        for m in range(N):
            b = torch.empty(n, dtype=torch.int32, pin_memory=True)
            b.numpy()[:] = t.inds(m).view(np.int32)
            iv[m].len = iv[m].cap = n
            iv[m].data = ctypes.cast(b.data_ptr(), S.u32p)
            self.keep.append(b)
        vb = torch.empty(n, dtype=torch.float32, pin_memory=True)
        vb.numpy()[:] = t.vals()
        self.keep += [vb, so, nd, iv]
        x.sortorder = ctypes.cast(so, S.u32p)
        x.ndims = ctypes.cast(nd, S.u32p)
        x.nnz = n
        x.inds = ctypes.cast(iv, ctypes.POINTER(S.IndexVector))
        x.values.len = x.values.cap = n
        x.values.data = ctypes.cast(vb.data_ptr(), S.f32p)
        self.s = x
        self.mats = []
        for M in mats:
            cap, st = int(M.s.cap), int(M.s.stride)
            b = torch.empty(cap * st, dtype=torch.float32, pin_memory=True)
            b.numpy()[:] = np.ctypeslib.as_array(M.s.values, shape=(cap * st,))
            ms = S.MatrixS()
            ms.nrows, ms.ncols, ms.cap, ms.stride = M.s.nrows, M.s.ncols, cap, st
            ms.values = ctypes.cast(b.data_ptr(), S.f32p)
            self.keep.append(b)
            self.mats.append(ms)

    def call(self, mode, order):
        import sptol_gb300 as S
        N = self.nmodes
        self.mats[N].nrows = self.ndims[mode]
        arr = (ctypes.POINTER(S.MatrixS) * (N + 1))(*[ctypes.pointer(m) for m in self.mats])
        op = (ctypes.c_uint32 * N)(*order)
        r = S.lib().sptCudaMTTKRP(ctypes.byref(self.s), arr, op, mode, 15)
        if r:
            raise RuntimeError("sptCudaMTTKRP failed (0x%x)" % r)


C1_DIMS = [1024, 1024, 1024]
C1_DRAWS = 1_000_000
C1_RANK = 16


def c1_leg(reps):
    """The CPU-runnable reference configuration: 1024^3, 1,000,000 uniform
    draws (seed 0) with duplicates merged by summation, values U[0,1), rank-16
    factors U[0,1); mode 0 first, then every mode.  GPU: the resident kernel
    (CUDA events) and the drop-in sptMTTKRP with host buffers (wall time);
    beside them the reference's sequential sptMTTKRP (mttkrp.c:39-115) and
    sptOmpMTTKRP_Reduce with every host thread (the oracle port of the latter
    where the reference was not built).  Medians of `reps` calls after one
    warm-up call each."""
    import torch
    import oracle as O
    import sptol_gb300 as S
    spec = S.GenSpec()
    spec.seed = 0
    spec.nmodes = 3
    for m, d in enumerate(C1_DIMS):
        spec.ndims[m] = d
        spec.coord_dist[m] = S.DIST_UNIFORM
    spec.count = C1_DRAWS
    spec.merge_duplicates = 1
    spec.value_dist = S.VAL_U01
    t = S.Tensor.generate(spec)
    ndims, nnz = t.ndims, t.nnz
    stride = ((C1_RANK - 1) // 8 + 1) * 8
    mats = S.new_factors(ndims, C1_RANK, seed=1)
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream
    dfac = [torch.from_numpy(mats[m].array()[: ndims[m]].copy()).cuda() for m in range(3)]
    dout = torch.zeros((max(ndims), stride), dtype=torch.float32, device="cuda")
    coo = S.DeviceCoo(t, stream=sh)
    orders = [[m] + [(m + i) % 3 for i in (1, 2)] for m in range(3)]
    kern, call = [], []
    for m in range(3):
        coo.prepare(m, stream=sh)
        ptrs = [f.data_ptr() for f in dfac]
        ks = []
        for r in range(reps + 1):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            coo.mttkrp(m, orders[m], ptrs, C1_RANK, stride, dout.data_ptr(), stream=sh)
            b.record(stream)
            b.synchronize()
            if r:
                ks.append(a.elapsed_time(b))
        kern.append(float(np.median(ks)))
        cs = []
        for r in range(reps + 1):
            a = time.perf_counter()
            S.mttkrp(t, mats, m, mats_order=orders[m], entry="sptMTTKRP", copy=False)
            if r:
                cs.append((time.perf_counter() - a) * 1e3)
        call.append(float(np.median(cs)))
    coo.free()
    threads = os.cpu_count() or 1
    inds, vals = t.arrays()
    facs = [mats[m].array()[: ndims[m]] for m in range(3)]
    seq, red = [], []
    kind = "reference" if O.ref_loadable() else "port"
    for m in range(3):
        if kind == "reference":
            seq.append(O.ref_mttkrp(ndims, inds, vals, facs, C1_RANK, m, which=0, tk=1, reps=reps)[1] * 1e3)
            red.append(O.ref_mttkrp(ndims, inds, vals, facs, C1_RANK, m, which=1, tk=threads, reps=reps)[1] * 1e3)
        else:
            for which, dst, tk in (("f32", seq, 1), ("omp", red, threads)):
                ts = []
                for r in range(reps + 1):
                    a = time.perf_counter()
                    O.mttkrp(ndims, inds, vals, facs, C1_RANK, m, precision=which, tk=tk)
                    if r:
                        ts.append((time.perf_counter() - a) * 1e3)
                dst.append(float(np.median(ts)))
    ab = algo_bytes(ndims, nnz, C1_RANK)

    def gbs(ms):
        return [round(ab / (x / 1e3) / 1e9, 2) for x in ms]

    return {"workload": "mttkrp_uniform_coo_1024cubed_1Mdraws_merged_rank16", "nnz": nnz,
            "algorithmic_bytes_per_mttkrp": ab,
            "gpu_kernel_ms_by_mode": [round(x, 4) for x in kern], "gpu_kernel_gbs_by_mode": gbs(kern),
            "sptMTTKRP_call_ms_by_mode": [round(x, 3) for x in call], "sptMTTKRP_call_gbs_by_mode": gbs(call),
            "cpu": {"kind": kind, "cores": threads,
                    "sequential_sptMTTKRP_ms_by_mode": [round(x, 3) for x in seq],
                    "sequential_gbs_by_mode": gbs(seq),
                    "omp_reduce_ms_by_mode": [round(x, 3) for x in red], "omp_reduce_gbs_by_mode": gbs(red),
                    "omp_reduce_threads": threads},
            "reps": reps}


C4_DIMS = [500_000, 300_000, 10_000]


def cpals_leg(nnz, iters=20):
    """Full CP-ALS on the planted-model tensor 500,000 x 300,000 x 10,000
    (coordinates Zipf(1.1) in every mode, 50M unique nonzeros, values a
    planted rank-32 Kruskal model plus N(0, 0.01^2)), rank 32, 20 iterations
    from seeded U[0,1) factors.  GPU: sptgbCpdAls (the device loop behind
    sptCpdAls), wall time including upload and the per-mode device sorts.
    cpu_baseline: the reference's sptOmpCpdAls loop, OmpCpdAlsStep with
    use_reduce = 1 (cpd_omp.c:32-157), every host thread, from the same
    factors; both fits are the corrected fit of the final model."""
    import oracle as O
    import sptol_gb300 as S
    spec = S.GenSpec()
    spec.seed = 404
    spec.nmodes = 3
    for m, d in enumerate(C4_DIMS):
        spec.ndims[m] = d
        spec.coord_dist[m] = S.DIST_ZIPF
        spec.zipf_s[m] = 1.1
    spec.count = nnz
    spec.merge_duplicates = 0
    spec.value_dist = S.VAL_PLANTED
    spec.planted_rank = 32
    spec.planted_seed = 405
    spec.noise_sigma = 0.01
    g0 = time.time()
    t = S.Tensor.generate(spec)
    gen_s = time.time() - g0
    ndims = t.ndims
    rng = np.random.default_rng(406)
    init = [rng.random((d, 32), dtype=np.float32) for d in ndims]
    S.cpd_als(t, 32, 1, 0.0, init)          # context and kernel modules loaded before timing
    t0 = time.perf_counter()
    _, _, fits, it = S.cpd_als(t, 32, iters, 0.0, init)
    gpu_s = time.perf_counter() - t0
    out = {"workload": "cpals_planted_rank32_500Kx300Kx10K_zipf1.1_%dnnz_rank32_%dit" % (t.nnz, iters),
           "nnz": t.nnz, "rank": 32, "iterations": iters, "generate_s": round(gen_s, 2),
           "gpu": {"seconds": round(gpu_s, 4), "s_per_iteration": round(gpu_s / iters, 5),
                   "fit_final": float(fits[it - 1]), "entry": "sptgbCpdAls (upload, sorts and copies back included)"}}
    if O.ref_loadable():
        threads = os.cpu_count() or 1
        inds, vals = t.arrays()
        secs, fit, _ = O.ref_omp_cpd(ndims, inds, vals, 32, iters, init, threads)
        out["cpu_baseline"] = {"seconds": round(secs, 3), "s_per_iteration": round(secs / iters, 4),
                               "fit_final": fit, "kind": "reference", "cores": threads,
                               "sample": "the full tensor, %d iterations, OmpCpdAlsStep (sptOmpCpdAls loop, "
                                         "use_reduce = 1, tol 0) from the same initial factors" % iters}
        out["fit_abs_diff"] = abs(float(fits[it - 1]) - fit)
        out["gpu_over_cpu"] = round(secs / gpu_s, 1)
    return out


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def traffic_per_launch():
    """DRAM bytes per MTTKRP launch from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "mttkrp_coo_powerlaw_100m.md")
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_launch:"):
                return int(float(line.split(":")[1]))
    except Exception:
        pass
    return None


class Clocks:
    """Samples SM clocks and throttle reasons with nvidia-smi while running."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=" + self.Q, "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.gpu)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def reduce_max(value, world):
    """Max of a float over ranks (identity for a single process)."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def cpu_port_mttkrp(t, mats, threads, reps):
    """sptOmpMTTKRP_Reduce restated (oracle) on the host tensor: seconds per step."""
    import oracle as O
    inds, vals = t.arrays()
    facs = [m.array()[: t.ndims[i]] for i, m in enumerate(mats[:3])]
    best = []
    for r in range(reps + 1):
        t0 = time.perf_counter()
        for mode in range(3):
            O.mttkrp(t.ndims, inds, vals, facs, RANK, mode, precision="omp", tk=threads)
        if r > 0:
            best.append(time.perf_counter() - t0)
    return float(np.mean(best)) if best else 0.0


def cpu_leg(t, mats, reps):
    """cpu_baseline of the GPU arm: the reference's own sptOmpMTTKRP_Reduce
    (mttkrp_omp.c:401-563) with every host thread on the arm's own host copy of
    the full workload tensor, one warm-up call then `reps` timed calls per
    mode; beside it the atomic sptOmpMTTKRP (mttkrp_omp.c:125-252), one timed
    call per mode.  Where the reference was not built, the oracle port of
    sptOmpMTTKRP_Reduce instead (kind "port")."""
    import oracle as O
    threads = os.cpu_count() or 1
    inds, vals = t.arrays()
    facs = [m.array()[: t.ndims[i]] for i, m in enumerate(mats[:3])]
    atomic = None
    if O.ref_loadable():
        kind = "reference"
        secs = 0.0
        for mode in range(3):
            secs += O.ref_mttkrp(t.ndims, inds, vals, facs, RANK, mode, which=1, tk=threads, reps=reps)[1]
        asecs = []
        for mode in range(3):
            asecs.append(O.ref_mttkrp(t.ndims, inds, vals, facs, RANK, mode, which=2, tk=threads, reps=1)[1])
        bstep = 3 * algo_bytes(DIMS, t.nnz, RANK)
        atomic = {"value": round(bstep / sum(asecs) / 1e9, 3), "unit": "GB/s", "seconds_by_mode": asecs,
                  "function": "sptOmpMTTKRP (OpenMP atomics), %d threads, 1 call per mode after the Reduce "
                              "calls" % threads}
    else:
        kind = "port"
        secs = cpu_port_mttkrp(t, mats, threads, reps)
    gbs = 3 * algo_bytes(DIMS, t.nnz, RANK) / secs / 1e9
    sample = ("the full %d-nnz workload tensor, all 3 modes, %d timed calls per mode after 1 warm-up, "
              "sptOmpMTTKRP_Reduce with %d threads" % (t.nnz, reps, threads))
    return {"value": round(gbs, 3), "unit": "GB/s", "cores": threads, "kind": kind, "sample": sample,
            "seconds_per_step": secs, "nnz_per_s": 3 * t.nnz / secs, "atomic": atomic}


def reference_gpu_leg(sess, reps=2):
    """The reference's own best CUDA MTTKRP on the same tensor: sptCudaMTTKRPOneKernel
    with impl_num 15 (mttkrp_cuda_onekernel.cu:41-427; kernel
    spt_MTTKRPKernelRankSplitNnz3DOneKernel, mttkrp_cuda_kernels.cu:544-603,
    one atomicAdd per nonzero and column), built for sm_103a.  Per mode one
    warm-up call, then `reps` calls: the kernel time as the reference prints
    it (CPU timer around the launch and the synchronisation) and the time of
    the whole call (uploads of the tensor and factors, cudaMalloc/cudaFree,
    the kernel and the copy back, all from pageable memory)."""
    try:
        import torch
        if not torch.cuda.is_available():
            return None
    except Exception:
        return None
    kern, call = [], []
    for m in range(3):
        if sess.cuda_mttkrp(m) is None:
            return None
        ks, cs = [], []
        for _ in range(reps):
            c, k = sess.cuda_mttkrp(m)
            cs.append(c)
            if k is not None:
                ks.append(k)
        kern.append(float(np.median(ks)) if ks else None)
        call.append(float(np.median(cs)))
    ab = algo_bytes(sess.ndims, sess.nnz, RANK)
    return {"function": "sptCudaMTTKRPOneKernel impl 15 (spt_MTTKRPKernelRankSplitNnz3DOneKernel), sm_103a",
            "kernel_ms_by_mode": [round(k * 1e3, 3) if k is not None else None for k in kern],
            "kernel_gbs": round(3 * ab / sum(kern) / 1e9, 1) if all(k for k in kern) else None,
            "call_ms_by_mode": [round(c * 1e3, 2) for c in call],
            "call_gbs": round(3 * ab / sum(call) / 1e9, 2), "reps": reps}


def run_reference(args, world, rank):
    """--impl reference: the reference's own sptOmpMTTKRP_Reduce
    (mttkrp_omp.c:401-563) with every host thread on the full workload tensor,
    in a process that loads nothing of libParTI.so: the tensor and factors are
    made by the library's generator compiled into oracle/_ref/libparti_ref.so,
    which builds them in the reference's own containers (ref_session_*).  One
    step = MTTKRP of modes 0, 1, 2 (protocol of examples/mttkrp.c:240-274);
    `warmup` untimed steps, then `steps` timed steps.  Where the reference was
    not built, the oracle port on the tensor from libParTI.so's generator."""
    if rank != 0:
        return
    import oracle as O
    threads = os.cpu_count() or 1
    K, W = max(1, args.steps), max(0, args.warmup)
    if not O.ref_loadable():
        try:
            O.build()
        except Exception:
            pass
    g0 = time.time()
    if O.ref_loadable():
        kind = "reference"
        sess = O.RefSession(spec_for(args.nnz), RANK, 1, threads)
        nnz = sess.nnz

        def step():
            for m in range(3):
                sess.mttkrp(m, "reduce")
    else:
        import sptol_gb300 as S
        kind = "port"
        t = S.Tensor.generate(spec_for(args.nnz))
        mats = S.new_factors(DIMS, RANK, seed=1)
        inds, vals = t.arrays()
        facs = [m.array()[: t.ndims[i]] for i, m in enumerate(mats[:3])]
        nnz = t.nnz

        def step():
            for m in range(3):
                O.mttkrp(DIMS, inds, vals, facs, RANK, m, precision="omp", tk=threads)
    gen_s = time.time() - g0
    for _ in range(W):
        step()
    t0 = time.perf_counter()
    for _ in range(K):
        step()
    secs = (time.perf_counter() - t0) / K
    gbs = 3 * algo_bytes(DIMS, nnz, RANK) / secs / 1e9
    ref_gpu = reference_gpu_leg(sess) if kind == "reference" and not args.skip_ref_gpu else None
    sample = ("the full %d-nnz workload tensor, 3 modes per step, sptOmpMTTKRP_Reduce with %d threads, "
              "%d timed steps after %d warm-up steps" % (nnz, threads, K, W))
    line = {
        "metric": METRIC, "value": round(gbs, 3), "unit": "GB/s", "n_gpus": args.gpus, "steps": K,
        "warmup": W, "ms_per_step": secs * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
        "config": workload_config(nnz, args.gpus),
        "cpu_baseline": {"value": round(gbs, 3), "unit": "GB/s", "cores": threads, "kind": kind, "sample": sample},
        "e2e": {"value": round(gbs, 3), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "nnz_per_s": round(3 * nnz / secs, 1),
        "setup_s": {"generate": round(gen_s, 2)},
        "tensor_source": ("library generator linked into the reference build (reference containers)"
                          if kind == "reference" else "libParTI.so generator (reference not built)"),
        "reference_gpu": ref_gpu,
    }
    print(json.dumps(line), flush=True)


def run_ours(args, world, rank, local):
    import torch
    import sptol_gb300 as S
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    L = S.lib()
    L.sptgbInit(local)
    os.environ.setdefault("SPTGB_QUIET", "1")
    gen_t0 = time.time()
    t = S.Tensor.generate(spec_for(args.nnz))
    gen_s = time.time() - gen_t0
    ndims = t.ndims
    nnz = t.nnz
    stride = ((RANK - 1) // 8 + 1) * 8
    mats = S.new_factors(ndims, RANK, seed=1)
    dfac = [torch.from_numpy(mats[m].array()[: ndims[m]].copy()).cuda() for m in range(3)]
    dout = torch.zeros((max(ndims), stride), dtype=torch.float32, device="cuda")
    # a dedicated stream: the library kernels and the timing events share it
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sh = stream.cuda_stream
    prep_t0 = time.time()
    coo = S.DeviceCoo(t, stream=sh)
    for m in range(3):
        coo.prepare(m, stream=sh)
    torch.cuda.synchronize()
    prep_s = time.time() - prep_t0
    ptrs = [f.data_ptr() for f in dfac]
    orders = [[m] + [(m + i) % 3 for i in (1, 2)] for m in range(3)]

    def launch(mode):
        coo.mttkrp(mode, orders[mode], ptrs, RANK, stride, dout.data_ptr(), stream=sh)

    for _ in range(args.warmup):
        for m in range(3):
            launch(m)
    torch.cuda.synchronize()
    K = args.steps
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(3 * K)]
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    clocks = Clocks(local)
    clocks.start()
    time.sleep(0.3)
    barrier(world)
    torch.cuda.synchronize()
    n0 = S.launch_count()
    t_start.record(stream)
    i = 0
    for _ in range(K):
        for m in range(3):
            evs[i][0].record(stream)
            launch(m)
            evs[i][1].record(stream)
            i += 1
    t_end.record(stream)
    torch.cuda.synchronize()
    n1 = S.launch_count()
    barrier(world)
    timed_ms = t_start.elapsed_time(t_end)
    if len(clocks.rows) < 5:
        # the timed region was shorter than the sampling period: keep the same
        # kernels running for about a second more so the clock record covers them
        t1 = time.time()
        while time.time() - t1 < 1.5:
            for m in range(3):
                launch(m)
            torch.cuda.synchronize()
    clocks.stop()
    per_launch = [evs[j][0].elapsed_time(evs[j][1]) for j in range(3 * K)]
    per_mode = [float(np.mean(per_launch[m::3])) for m in range(3)]
    ms_max = reduce_max(timed_ms, world)
    bytes_step = 3 * algo_bytes(ndims, nnz, RANK)
    value = world * K * bytes_step / (ms_max / 1e3) / 1e9
    peak, peak_kind = peaks()
    launch_ms = float(np.mean(per_launch))
    achieved = algo_bytes(ndims, nnz, RANK) / (launch_ms / 1e3) / 1e9
    traffic = traffic_per_launch()

    # BF16 factor storage (FP32 accumulation) on the same resident copies:
    # reported beside the FP32 headline, same algorithmic byte formula
    d16 = [f.to(torch.bfloat16).contiguous() for f in dfac]
    p16 = [f.data_ptr() for f in d16]
    for _ in range(args.warmup):
        for m in range(3):
            coo.mttkrp(m, orders[m], p16, RANK, stride, dout.data_ptr(), stream=sh, bf16=True)
    kb = max(3, K // 4)
    ev16 = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(3 * kb)]
    torch.cuda.synchronize()
    j = 0
    for _ in range(kb):
        for m in range(3):
            ev16[j][0].record(stream)
            coo.mttkrp(m, orders[m], p16, RANK, stride, dout.data_ptr(), stream=sh, bf16=True)
            ev16[j][1].record(stream)
            j += 1
    torch.cuda.synchronize()
    pl16 = [a.elapsed_time(b) for a, b in ev16]
    bf16 = {"ms_per_launch_by_mode": [round(float(np.mean(pl16[m::3])), 4) for m in range(3)],
            "gbs_fp32_byte_formula": round(algo_bytes(ndims, nnz, RANK) / (float(np.mean(pl16)) / 1e3) / 1e9, 1),
            "rel_fro_vs_fp64": "about 2.6e-3 (4th-order precision study)"}
    del d16

    # e2e through the drop-in host-buffer API
    h2d = 0
    d2h = 0
    for m in range(3):
        h2d += nnz * 16 + sum(ndims[p] * stride * 4 for p in orders[m][1:])
        d2h += ndims[m] * stride * 4
    ke = max(1, args.e2e_steps)
    link_gbs = host_link_gbs()
    L = S.lib()

    def e2e_steps(call):
        """Two untimed steps (grow the library's device buffers), then ke
        timed steps of the three host-buffer calls: (seconds each step, mean)."""
        for _ in range(2):
            for m in range(3):
                call(m)
        barrier(world)
        each = []
        e0 = time.perf_counter()
        for _ in range(ke):
            s0 = time.perf_counter()
            for m in range(3):
                call(m)
            each.append(time.perf_counter() - s0)
        return each, reduce_max((time.perf_counter() - e0) / ke, world)

    # headline: the caller's tensor and factors live in page-locked memory
    # from cudaHostAlloc (torch's pinned allocator) -- a caller that allocates
    # its arrays for the GPU; every call copies them in and the result out
    hc = HostAllocCopy(t, mats)
    e_each, e_s = e2e_steps(lambda m: hc.call(m, orders[m]))
    del hc
    e2e = world * bytes_step / e_s / 1e9
    # the same calls on the library-allocated arrays page-locked afterwards
    # with cudaHostRegister (sptgbPinSparseTensor / sptgbPinMatrix)
    registered = None
    if world == 1 and not args.skip_registered:
        pinned = L.sptgbPinSparseTensor(t.ptr()) == 0
        pinned_mats = [m for m in mats if L.sptgbPinMatrix(ctypes.byref(m.s)) == 0]
        r_each, r_s = e2e_steps(lambda m: S.mttkrp(t, mats, m, mats_order=orders[m], entry="sptCudaMTTKRP",
                                                   copy=False))
        if pinned:
            L.sptgbUnpinSparseTensor(t.ptr())
        for m in pinned_mats:
            L.sptgbUnpinMatrix(ctypes.byref(m.s))
        S.lib().sptClearLastError()
        registered = {"value": round(bytes_step / r_s / 1e9, 2), "unit": "GB/s", "ms_per_step": round(r_s * 1e3, 2),
                      "ms_median_step": round(float(np.median(r_each)) * 1e3, 2),
                      "ms_each_step": [round(x * 1e3, 2) for x in r_each],
                      "host_memory": "cudaHostRegister" if pinned and len(pinned_mats) == len(mats) else "pageable"}

    hicoo = None
    if world == 1 and not args.skip_hicoo:
        coo.free()
        hicoo = hicoo_leg(t, mats, ndims, nnz, 3)
        if not args.skip_cpu:
            hicoo["cpu_baseline"] = hicoo_cpu_leg(args.cpu_sample, 2)
        if args.hicoo4:
            hicoo["order4"] = hicoo4_leg()

    # CP-ALS before the serve leg: after that leg (a 120 GB arena and ~10 GB of
    # request tensors allocated and freed) the first upload of this tensor
    # took 91 ms instead of 5.4 ms (SPTGB_TRACE=1), a state of the process,
    # not of the call
    cpals = None
    if world == 1 and not args.skip_cpals:
        coo.free()
        cpals = cpals_leg(args.cpals_nnz)

    serve = None
    if world == 1 and not args.skip_serve:
        coo.free()
        serve = serve_leg(args)

    c1 = None
    if world == 1 and not args.skip_c1:
        c1 = c1_leg(5)

    cpu = None
    if rank == 0 and world == 1 and not args.skip_cpu:
        cpu = cpu_leg(t, mats, 2)

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 2), "unit": "GB/s", "n_gpus": world, "steps": K,
            "warmup": args.warmup, "ms_per_step": ms_max / K, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(nnz, world),
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "traffic": traffic, "peak_kind": peak_kind,
                         "kernel": "k_mttkrp_rec (order-3 record kernel) after the output memset, one launch per mode",
                         "ms_per_launch_by_mode": [round(x, 4) for x in per_mode]},
            "e2e": {"value": round(e2e, 2), "unit": "GB/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "entry": "sptCudaMTTKRP (host buffers)", "ms_per_step": e_s * 1e3,
                    "ms_each_step": [round(x * 1e3, 2) for x in e_each],
                    "ms_median_step": round(float(np.median(e_each)) * 1e3, 2),
                    "host_memory": "cudaHostAlloc (torch pinned allocator)",
                    "host_link_h2d_gbs": link_gbs,
                    "link_floor_ms": round((h2d + d2h) / (link_gbs * 1e9) * 1e3, 2) if link_gbs else None,
                    "registered_variant": registered},
            "gpu_launches": int(n1 - n0),
            "clocks": clocks.summary(),
            "nnz_per_s": round(world * K * 3 * nnz / (ms_max / 1e3), 1),
            "setup_s": {"generate": round(gen_s, 2), "upload_and_sort_3_modes": round(prep_s, 2)},
            "cpu_baseline": cpu,
            "bf16_storage": bf16,
            "hicoo": hicoo,
            "serve": serve,
            "c1": c1,
            "cpals": cpals,
        }
        print(json.dumps(line), flush=True)
    coo.free()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def main():
    args = parse()
    world, rank, local = dist_init()
    if args.impl == "reference":
        if world > 1 and rank != 0:
            return
        run_reference(args, world, rank)
        return
    run_ours(args, world, rank, local)


if __name__ == "__main__":
    main()
