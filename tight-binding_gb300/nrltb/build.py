"""In-tree build of the native libraries (no cmake, one -gencode, parallel nvcc).

  _lib/libnrltb_gb300.so   CUDA path (sm_103a) + host readers, the product
  _lib/libnrltb_host.so    host readers only (C11), loadable without CUDA
  _lib/nrltb_static        C host driver (restates static.f), linked to the CUDA lib
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

from .abi import GPU_LIB, HOST_LIB, LIB_DIR, PKG_ROOT, REPO_ROOT

CSRC = os.path.join(PKG_ROOT, "csrc")
HOST = os.path.join(PKG_ROOT, "host")
INCLUDE = os.path.join(REPO_ROOT, "include")
OBJ = os.path.join(LIB_DIR, "obj")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
HOST_SOURCES = ["nrltb_input.c", "nrltb_qlmt.c"]
CU_SOURCES = ["nrltb_api.cu", "eig.cu", "setup.cu", "sums.cu", "refine.cu", "ozaki.cu", "gemm_tc.cu", "gemm_umma.cu", "bench_hooks.cu", "noalloc.cu"]
DRIVER = os.path.join(LIB_DIR, "nrltb_static")


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    return hs


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def build_all(force=False, verbose=False):
    os.makedirs(OBJ, exist_ok=True)
    nvcc = _nvcc()
    hdrs = _headers()
    cflags = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC]
    jobs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src.replace(".cu", ".o"))
        if force or _stale(o, [s] + hdrs):
            jobs.append([nvcc] + ARCH + cflags + ["-c", s, "-o", o])
    hos = []
    for src in HOST_SOURCES:
        hsrc = os.path.join(HOST, src)
        ho = os.path.join(OBJ, src.replace(".c", ".o"))
        hos.append(ho)
        if force or _stale(ho, [hsrc] + hdrs):
            jobs.append(["gcc", "-std=gnu11", "-O2", "-ffp-contract=off", "-fPIC", "-Wall", "-I", INCLUDE, "-c",
                         hsrc, "-o", ho])
    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, os.cpu_count() or 1))) as ex:
        list(ex.map(_run, jobs))
    objs = [os.path.join(OBJ, s.replace(".cu", ".o")) for s in CU_SOURCES] + hos
    if force or _stale(GPU_LIB, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", GPU_LIB + ".tmp"] + objs + ["-lcudart"])
        os.replace(GPU_LIB + ".tmp", GPU_LIB)
    if force or _stale(HOST_LIB, hos):
        _run(["gcc", "-shared", "-o", HOST_LIB + ".tmp"] + hos + ["-lm"])
        os.replace(HOST_LIB + ".tmp", HOST_LIB)
    dsrc = os.path.join(HOST, "nrltb_static.c")
    if os.path.exists(dsrc) and (force or _stale(DRIVER, [dsrc, GPU_LIB] + hdrs)):
        _run(["gcc", "-std=gnu11", "-O2", "-Wall", "-I", INCLUDE, dsrc, "-o", DRIVER,
              "-L", LIB_DIR, "-lnrltb_gb300", "-Wl,-rpath,$ORIGIN", "-lm"])
    if verbose:
        print("built", GPU_LIB, HOST_LIB)
    return GPU_LIB


if __name__ == "__main__":
    build_all(force="--force" in sys.argv, verbose=True)
