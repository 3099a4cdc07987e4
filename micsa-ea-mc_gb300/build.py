"""Build libmicsa.so (CUDA sm_103a + host C) and the micsa_run driver.

Outputs go to micsa-ea-mc_gb300/lib and micsa-ea-mc_gb300/bin (git-ignored).
Translation units compile in parallel; nothing here needs cmake or make.
"""
import os
import platform
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
INCLUDE = os.path.join(ROOT, "include")
OBJ = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "lib")
BIN = os.path.join(PKG, "bin")

HOST_C = ["host/micsa_rng.c", "host/micsa_model.c", "host/micsa_io.c", "host/micsa_jump.c",
          "host/micsa_jobs.c", "host/micsa_serve.c"]
CUDA = ["csrc/micsa_kernels.cu", "csrc/micsa_api.cu", "csrc/micsa_noalloc.cu"]
GENCODE = "-gencode=arch=compute_103a,code=sm_103a"


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _quadmath():
    # binary128 arithmetic: libquadmath on x86-64; native long double on AArch64
    return ["-lquadmath"] if platform.machine() in ("x86_64", "AMD64", "i686") else []


def _run(cmd):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("command failed: %s\n%s" % (" ".join(cmd), p.stdout))
    return p.stdout


def _newer(target, sources):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def _headers():
    hs = []
    for d in (INCLUDE, os.path.join(PKG, "host"), os.path.join(PKG, "csrc")):
        for f in os.listdir(d):
            if f.endswith((".h", ".cuh")):
                hs.append(os.path.join(d, f))
    return hs


def build(verbose=False, force=False):
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIB, exist_ok=True)
    os.makedirs(BIN, exist_ok=True)
    hdrs = _headers()
    inc = ["-I" + INCLUDE, "-I" + os.path.join(PKG, "host"), "-I" + os.path.join(PKG, "csrc")]
    jobs = []
    objs = []
    for src in HOST_C:
        s = os.path.join(PKG, src)
        o = os.path.join(OBJ, os.path.basename(src) + ".o")
        objs.append(o)
        if force or not _newer(o, [s] + hdrs):
            jobs.append(["gcc", "-O3", "-std=gnu11", "-ffp-contract=off", "-fPIC", "-Wall", "-Wextra",
                         "-Wno-unused-parameter", "-pthread"] + inc + ["-c", s, "-o", o])
    for src in CUDA:
        s = os.path.join(PKG, src)
        o = os.path.join(OBJ, os.path.basename(src) + ".o")
        objs.append(o)
        if force or not _newer(o, [s] + hdrs):
            jobs.append([_nvcc(), GENCODE, "-lineinfo", "-O3", "-std=c++17",
                         "-Xcompiler", "-fPIC", "-Xptxas", "-v"] + inc + ["-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            sys.stdout.write(o)
    lib = os.path.join(LIB, "libmicsa.so")
    if force or jobs or not os.path.exists(lib):
        _run([_nvcc(), GENCODE, "-shared", "-o", lib] + objs + ["-lpthread"] + _quadmath())
    drv_src = os.path.join(PKG, "host", "micsa_driver.c")
    drv = os.path.join(BIN, "micsa_run")
    if force or not _newer(drv, [drv_src, lib] + hdrs):
        _run(["gcc", "-O2", "-std=gnu11", "-ffp-contract=off", "-Wall", "-pthread"] + inc +
             [drv_src, "-o", drv, "-L" + LIB, "-lmicsa", "-Wl,-rpath,$ORIGIN/../lib", "-lm"])
    return lib


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
