"""Generates tests/golden/*.npz from the reference library itself.

Runs ParTI!'s own code (oracle/_ref/libparti_ref.so, built from the reference
sources by oracle/Makefile) on small seeded inputs and stores inputs and
outputs:
  sort_*.npz     sptSparseTensorSortIndex / SortIndexCustomOrder results
  hicoo_*.npz    sptSparseTensorToHiCOO arrays (sorted COO, kptr, kschr,
                 nkiters, cptr, bptr, binds, einds, values, max_nnzb) and
                 sptMTTKRPHiCOO outputs
  mttkrp_*.npz   sequential sptMTTKRP outputs for every mode
  cpd_*.npz      corrected fit after every iteration of the reference's
                 CP-ALS loop, final factors and lambda (the loop is checked
                 here to end bit-for-bit where CpdAlsStep ends)
  uniform_1m_summary.npz per-mode norms, sums and sample rows of sptMTTKRP on the
                 1024^3 / 1,000,000-draw tensor of the library generator
Needs the reference sources (only present where the fixtures are made):
    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402


def unique_coords(rng, ndims, n, zipf=None):
    cols = []
    for m, d in enumerate(ndims):
        if zipf and zipf[m]:
            c = np.minimum(rng.zipf(zipf[m], size=3 * n) - 1, d - 1)
        else:
            c = rng.integers(0, d, size=3 * n)
        cols.append(c)
    u = np.unique(np.stack(cols).astype(np.uint32), axis=1)
    u = u[:, rng.permutation(u.shape[1])[:n]]
    return np.ascontiguousarray(u)


def factors(rng, ndims, rank):
    st = O.stride_of(rank)
    out = []
    for d in ndims:
        f = np.zeros((d, st), np.float32)
        f[:, :rank] = rng.random((d, rank), dtype=np.float32)
        out.append(f)
    return out


def save(name, **kw):
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **kw)
    print("wrote", name)


def sort_case(name, seed, ndims, n, order):
    rng = np.random.default_rng(seed)
    inds = unique_coords(rng, ndims, n)
    vals = rng.random(inds.shape[1], dtype=np.float32)
    si, sv = O.ref_sort(ndims, inds, vals)
    ci, cv = O.ref_sort(ndims, inds, vals, order)
    save(name, ndims=np.array(ndims, np.uint32), inds=inds, vals=vals, lex_inds=si, lex_vals=sv,
         order=np.array(order, np.uint32), custom_inds=ci, custom_vals=cv)


def hicoo_case(name, seed, ndims, n, sb, sk, rank, zipf=None, with_mttkrp=True):
    rng = np.random.default_rng(seed)
    inds = unique_coords(rng, ndims, n, zipf)
    vals = rng.random(inds.shape[1], dtype=np.float32)
    si, sv, h = O.ref_hicoo(ndims, inds, vals, sb, sk)
    kw = {}
    if with_mttkrp:
        mats = factors(rng, ndims, rank)
        outs = [O.ref_mttkrp_hicoo(ndims, inds, vals, sb, sk, mats, rank, m) for m in range(len(ndims))]
        kw = {"out%d" % m: o for m, o in enumerate(outs)}
        kw.update({"mat%d" % m: f for m, f in enumerate(mats)})
    save(name, ndims=np.array(ndims, np.uint32), inds=inds, vals=vals, sb=sb, sk=sk, rank=rank, sorted_inds=si,
         sorted_vals=sv, kptr=h["kptr"], cptr=h["cptr"], bptr=h["bptr"], binds=h["binds"], einds=h["einds"],
         nkiters=h["nkiters"], kschr_len=h["kschr_len"], kschr=h["kschr"], max_nnzb=h["max_nnzb"], **kw)


def mttkrp_case(name, seed, ndims, n, rank):
    rng = np.random.default_rng(seed)
    inds = unique_coords(rng, ndims, n)
    vals = rng.random(inds.shape[1], dtype=np.float32)
    mats = factors(rng, ndims, rank)
    kw = {}
    for m in range(len(ndims)):
        kw["out%d" % m] = O.ref_mttkrp(ndims, inds, vals, mats, rank, m)[0]
        kw["mat%d" % m] = mats[m]
    save(name, ndims=np.array(ndims, np.uint32), inds=inds, vals=vals, rank=rank, **kw)


def cpd_case(name, seed, ndims, n, rank, niters, noise):
    rng = np.random.default_rng(seed)
    inds = unique_coords(rng, ndims, n)
    A = [rng.random((d, rank)) for d in ndims]
    prod = np.ones((inds.shape[1], rank))
    for m in range(len(ndims)):
        prod *= A[m][inds[m]]
    vals = (prod.sum(1) + noise * rng.standard_normal(inds.shape[1])).astype(np.float32)
    init = [rng.random((d, rank)).astype(np.float32) for d in ndims]
    t = O.ref_cpd_trace(ndims, inds, vals, rank, niters, init)
    same = all(np.array_equal(a, b) for a, b in zip(t["loop_factors"], t["step_factors"]))
    assert same and np.array_equal(t["loop_lambda"], t["step_lambda"]), "trace loop != CpdAlsStep"
    kw = {"init%d" % m: a for m, a in enumerate(init)}
    kw.update({"final%d" % m: a for m, a in enumerate(t["loop_factors"])})
    save(name, ndims=np.array(ndims, np.uint32), inds=inds, vals=vals, rank=rank, niters=niters, fits=t["fits"],
         lam=t["loop_lambda"], **kw)


def uniform_1m_summary():
    import sptol_gb300 as S
    spec = S.GenSpec()
    spec.seed = 0
    spec.nmodes = 3
    for m in range(3):
        spec.ndims[m] = 1024
        spec.coord_dist[m] = S.DIST_UNIFORM
    spec.count = 1_000_000
    spec.merge_duplicates = 1
    spec.value_dist = S.VAL_U01
    t = S.Tensor.generate(spec)
    inds, vals = t.arrays()
    ndims = [1024] * 3
    rank = 16
    mats = [m.array()[: ndims[i]].copy() for i, m in enumerate(S.new_factors(ndims, rank, seed=1)[:3])]
    rows = np.array([0, 1, 2, 3, 511, 777, 1000, 1023])
    kw = {}
    for m in range(3):
        out = O.ref_mttkrp(ndims, inds, vals, mats, rank, m)[0].astype(np.float64)
        kw["norm%d" % m] = np.sqrt((out ** 2).sum())
        kw["sum%d" % m] = out.sum()
        kw["rows%d" % m] = out[rows]
    save("uniform_1m_summary", nnz=inds.shape[1], key_checksum=np.uint64(
        (inds[0].astype(np.uint64) * 1048576 * 1024 + inds[1].astype(np.uint64) * 1024 + inds[2]).sum()),
         val_sum=np.float64(vals.astype(np.float64).sum()), sample_rows=rows, **kw)


def main():
    sort_case("sort_3d", 11, [50, 40, 30], 3000, [2, 0, 1])
    sort_case("sort_4d", 12, [20, 15, 12, 9], 3000, [3, 1, 0, 2])
    hicoo_case("hicoo_3d_small", 21, [50, 40, 30], 3000, 2, 4, 16)
    hicoo_case("hicoo_3d_skew", 22, [300000, 200000, 2500], 20000, 7, 17, 32, zipf=[1.2, 1.2, None],
               with_mttkrp=False)
    hicoo_case("hicoo_4d", 23, [20, 15, 12, 9], 3000, 2, 3, 8)
    mttkrp_case("mttkrp_3d_r16", 31, [1024, 1024, 1024], 20000, 16)
    mttkrp_case("mttkrp_3d_r17", 32, [300, 200, 100], 5000, 17)
    mttkrp_case("mttkrp_4d_r8", 33, [40, 30, 20, 10], 5000, 8)
    cpd_case("cpd_3d", 41, [30, 25, 20], 6000, 5, 10, 0.01)
    cpd_case("cpd_4d", 42, [12, 10, 9, 8], 4000, 3, 8, 0.01)
    uniform_1m_summary()


if __name__ == "__main__":
    main()
