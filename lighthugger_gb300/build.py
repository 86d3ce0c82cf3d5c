"""Build of the native library: lighthugger_gb300/_lib/liblh.so.

CUDA sources are compiled for sm_103a only, with --fmad=false (every float
operation rounds on its own, which is what makes culling, visibility and
depth bit exact) and IEEE division / square root.  Host C++ (scene
generator) is compiled with g++ without FMA contraction either.  Objects are
built in parallel; no cmake.  LH_NVCC_EXTRA adds nvcc flags, e.g.
"-DLH_BWD_MIN_BLOCKS=1" for another launch shape of the resolve adjoint
(objects are not rebuilt when only the flags change: pass force=True).
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "liblh.so")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")

CU_SOURCES = ["cull.cu", "raster.cu", "resolve.cu", "persistent.cu", "adjoint.cu", "display.cu", "capi.cu", "noalloc.cu", "waits.cu", "probe.cu"]
CPP_SOURCES = ["scene.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
              "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
              "-I", CSRC] + os.environ.get("LH_NVCC_EXTRA", "").split()
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-I", os.path.join(ROOT, "include"),
             "-I", os.path.join(CUDA_HOME, "include")]


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    inc = os.path.join(ROOT, "include", "lh")
    hs += [os.path.join(inc, f) for f in os.listdir(inc)]
    return hs


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(args):
    src, obj, kind, extra = args
    if kind == "cu":
        cmd = [NVCC] + ARCH + NVCC_FLAGS + extra + ["-c", src, "-o", obj]
    else:
        cmd = ["g++"] + CXX_FLAGS + extra + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stderr


def build(force=False, verbose=False, ptxas_verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    headers = _headers()
    jobs = []
    objs = []
    for s in CU_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s + ".o")
        objs.append(obj)
        extra = ["-Xptxas", "-v"] if ptxas_verbose else []
        if force or ptxas_verbose or _stale(obj, [src] + headers):
            jobs.append((src, obj, "cu", extra))
    for s in CPP_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append((src, obj, "cpp", []))
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for msg in ex.map(_compile, jobs):
                if verbose and msg:
                    print(msg)
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        cmd = [NVCC] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s" % (r.stdout, r.stderr))
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, ptxas_verbose="--ptxas" in sys.argv))
