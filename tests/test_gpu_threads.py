"""First calls from several host threads at once.

The launchers size their grids and set kernel attributes once per process;
this runs in a fresh process so that four threads, released together, make
the first device-resident COO and HiCOO MTTKRP calls of the process
concurrently (each on its own stream and output buffers).  Every thread's
result must equal a sequential pass afterwards within FP32 summation-order
tolerance (the kernels' atomics make the last bits order-dependent)."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import sys, threading
import numpy as np
import torch
sys.path.insert(0, ROOT)
import sptol_gb300 as S

L = S.lib()
L.sptgbInit(0)
spec = S.GenSpec()
spec.seed = 31
spec.nmodes = 3
for m, d in enumerate([900_000, 400_000, 9_000]):
    spec.ndims[m] = d
spec.coord_dist[0] = spec.coord_dist[1] = S.DIST_ZIPF
spec.zipf_s[0] = spec.zipf_s[1] = 1.2
spec.count = 400_000
spec.value_dist = S.VAL_UPM1
t = S.Tensor.generate(spec)
ndims = t.ndims
h = S.HiCOO(t, 7, 17)
dh = S.DeviceHicoo(h)
dc = S.DeviceCoo(t)
for m in range(3):
    dh.prepare(m)
    dc.prepare(m)
torch.cuda.synchronize()
RANK = STRIDE = 32
T = 4
gen = torch.Generator(device="cuda").manual_seed(5)
facs = [torch.rand(ndims[m], STRIDE, device="cuda", generator=gen) for m in range(3)]
ptrs = [f.data_ptr() for f in facs]
orders = [[m] + [(m + j) % 3 for j in (1, 2)] for m in range(3)]


def new_outs():
    return {(k, m): torch.empty(ndims[m], STRIDE, device="cuda") for k in ("coo", "hicoo") for m in range(3)}


def run(outs, stream):
    for m in range(3):
        dc.mttkrp(m, orders[m], ptrs, RANK, STRIDE, outs[("coo", m)].data_ptr(), stream=stream)
        dh.mttkrp(m, orders[m], ptrs, RANK, STRIDE, outs[("hicoo", m)].data_ptr(), stream=stream)


outs = [new_outs() for _ in range(T)]
streams = [torch.cuda.Stream() for _ in range(T)]
gate = threading.Barrier(T)
errors = []


def work(i):
    try:
        gate.wait()
        run(outs[i], streams[i].cuda_stream)
    except Exception as e:
        errors.append(repr(e))


threads = [threading.Thread(target=work, args=(i,)) for i in range(T)]
for th in threads:
    th.start()
for th in threads:
    th.join()
torch.cuda.synchronize()
assert not errors, errors
ref = new_outs()
run(ref, torch.cuda.current_stream().cuda_stream)
torch.cuda.synchronize()
worst = 0.0
for i in range(T):
    for key, r in ref.items():
        d = float(torch.linalg.norm(outs[i][key] - r) / torch.linalg.norm(r))
        worst = max(worst, d)
assert worst <= 1e-6, worst
print("threads ok, worst relative difference %.2e" % worst)
"""


def test_first_mttkrp_calls_from_four_threads():
    code = "ROOT = %r\n" % ROOT + CHILD
    p = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=900)
    assert p.returncode == 0, p.stdout[-2000:] + p.stderr[-4000:]
    assert "threads ok" in p.stdout
