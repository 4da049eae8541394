"""Builds libParTI.so (host C + sm_103a CUDA) in-tree.

Sources: csrc/host/*.c (gcc, OpenMP) and csrc/cuda/*.cu (nvcc, one -gencode
for sm_103a).  Objects go to sptol_gb300/_build/, the library to
sptol_gb300/lib/libParTI.so.  Translation units compile in parallel and are
skipped when their object is newer than the source and every header.
"""
import glob
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJDIR = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libParTI.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found; set CUDA_HOME")


def _headers():
    hs = glob.glob(os.path.join(CSRC, "**", "*.h"), recursive=True)
    hs += glob.glob(os.path.join(CSRC, "**", "*.cuh"), recursive=True)
    hs += glob.glob(os.path.join(ROOT, "include", "*.h"))
    return hs


def _stale(src, obj, headers):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src, __file__] + headers)


def _run(cmd):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("build failed:\n%s\n%s" % (" ".join(cmd), p.stdout))
    return p.stdout


def build(verbose=False, jobs=None):
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    inc = ["-I", os.path.join(cuda, "include"), "-I", os.path.join(ROOT, "include")]
    os.makedirs(OBJDIR, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    headers = _headers()
    cmds = []
    objs = []
    for src in sorted(glob.glob(os.path.join(CSRC, "cuda", "*.cu"))):
        obj = os.path.join(OBJDIR, "cu_" + os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(src, obj, headers):
            cmds.append([nvcc] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                                         "-Xptxas", "-warn-spills"] + inc + ["-c", src, "-o", obj])
    for src in sorted(glob.glob(os.path.join(CSRC, "host", "*.c"))):
        obj = os.path.join(OBJDIR, "c_" + os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(src, obj, headers):
            cmds.append(["gcc", "-O2", "-fPIC", "-fopenmp", "-std=gnu11", "-Wall", "-Wno-unused-function"] + inc +
                        ["-c", src, "-o", obj])
    with ThreadPoolExecutor(max_workers=jobs or min(16, os.cpu_count() or 4)) as ex:
        for out in ex.map(_run, cmds):
            if verbose and out.strip():
                print(out)
    if cmds or not os.path.exists(LIB):
        _run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs +
             ["-Xlinker", "-Bsymbolic", "-Xcompiler", "-fopenmp", "-lgomp", "-lpthread", "-lm"])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
