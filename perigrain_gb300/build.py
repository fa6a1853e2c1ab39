"""Build the in-tree native library and executables.

    libperigrain.so   CUDA kernels (sm_103a) + engine + C ABI (include/perigrain.h,
                      include/perigrain_io.h) + HDF5 subset + driver
    bin/simulate2d    drop-in for the reference's bin/simulate2d
    bin/simulate3d    drop-in for the reference's bin/simulate3d

Every translation unit is compiled in parallel; FP arithmetic is compiled without contraction
(--fmad=false on the device, -ffp-contract=off on the host) so the FP64 path performs the
reference's operations exactly.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(ROOT, "_build", "native")
LIB = os.path.join(HERE, "libperigrain.so")
BIN = os.path.join(HERE, "bin")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["pg_kernels.cu", "pg_kernels_mixed.cu", "pg_engine.cu", "pg_snapshot.cu", "pg_bonds.cu", "pg_noalloc.cu",
              "pg_adjoint.cu", "pg_adjoint_rev.cu", "pg_grad.cu", "pg_post.cu", "pg_pack.cu"]
CXX_SOURCES = ["h5lite.cpp", "pg_io.cpp", "pg_order.cpp"]


def _nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build perigrain_gb300")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build(verbose=False, force=False):
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(BIN, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers += [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        # the mixed-precision kernels and the reverse step use FMA; everything else performs the
        # reference's exact ops
        fmad = "--fmad=true" if src in ("pg_kernels_mixed.cu", "pg_adjoint_rev.cu") else "--fmad=false"
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc] + ARCH + ["-O3", fmad, "-lineinfo", "-std=c++17",
                                         "-Xcompiler", "-fPIC,-ffp-contract=off", "-Xptxas", "-v",
                                         "-c", s, "-o", o])
    for src in CXX_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-pthread", "-ffp-contract=off", "-Wall",
                         "-c", s, "-o", o])
    logs = []
    with ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        for out in ex.map(_run, jobs):
            logs.append(out)
    if force or _stale(LIB, objs):
        logs.append(_run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart", "-lpthread"]))
    for dim in (2, 3):
        exe = os.path.join(BIN, "simulate%dd" % dim)
        src = os.path.join(CSRC, "simulate.cpp")
        if force or _stale(exe, [src, LIB]):
            logs.append(_run(["g++", "-O2", "-std=c++17", "-DPG_SIM_DIM=%d" % dim, src, "-o", exe,
                              "-L" + HERE, "-lperigrain", "-Wl,-rpath,$ORIGIN/.."]))
    if verbose:
        print("\n".join(l for l in logs if l.strip()))
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB)
