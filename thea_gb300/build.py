"""Build recipe of the native library: every ``csrc/*.cu`` compiled for sm_103a by nvcc in parallel, linked into
``thea_gb300/_lib/libthea_gpu.so`` with the CUDA runtime linked statically.

All translation units use ``--fmad=false`` so that FP32 expressions round exactly as the reference's CPU code does
(no fused multiply-add), with IEEE division and square root (nvcc's defaults).
"""

import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libthea_gpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code too is compiled without floating-point contraction (aarch64 hosts would otherwise fuse multiply-adds)
NVCC_FLAGS = ["-O3", "-std=c++17", "--fmad=false", "-lineinfo",
              "-Xcompiler", "-fPIC,-fvisibility=hidden,-ffp-contract=off", "-Xptxas", "-v"]


def nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build thea_gb300")
    return cand


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False):
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".hpp", ".h"))]
    headers.append(os.path.join(os.path.dirname(HERE), "include", "thea_gpu.h"))
    objs = []
    jobs = []
    for src in sources():
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src[:-3] + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            cmd = [nvcc()] + ARCH + NVCC_FLAGS + ["-c", s, "-o", o]
            jobs.append((src, cmd))

    def run(job):
        src, cmd = job
        r = subprocess.run(cmd, capture_output=True, text=True)
        with open(os.path.join(BUILD, src[:-3] + ".log"), "w") as f:
            f.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed on %s:\n%s" % (src, r.stderr[-4000:]))
        return src

    with concurrent.futures.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for src in ex.map(run, jobs):
            if verbose:
                print("compiled", src, file=sys.stderr)
    if force or jobs or _stale(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", LIB] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stderr[-4000:])
        if verbose:
            print("linked", LIB, file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)
