"""Build of the GB300 library: every .cu with nvcc for sm_103a, every .cpp with g++,
linked into libnnpp_gb300.so next to this file.  Translation units compile in parallel;
objects go to _build/ (not committed)."""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(HERE, "..", "include")
OBJDIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libnnpp_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
                     "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
                     "-I", CSRC, "-I", INCLUDE]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I", CSRC, "-I", INCLUDE]


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _sources():
    srcs = []
    for f in sorted(os.listdir(CSRC)):
        if f.endswith(".cu") or f.endswith(".cpp"):
            srcs.append(os.path.join(CSRC, f))
    return srcs


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(INCLUDE, "nnpp_gb300.h"))
    return hs


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, verbose):
    obj = os.path.join(OBJDIR, os.path.basename(src) + ".o")
    deps = [src] + _headers()
    if not _stale(obj, deps):
        return obj
    if src.endswith(".cu"):
        cmd = [_nvcc()] + NVCC_FLAGS + ["-c", src, "-o", obj]
    else:
        cmd = ["g++"] + CXX_FLAGS + ["-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s\n%s" % (src, r.stdout, r.stderr))
    if verbose and r.stderr.strip():
        print(r.stderr, flush=True)
    return obj


def build(verbose=False, force=False):
    os.makedirs(OBJDIR, exist_ok=True)
    if force:
        for f in os.listdir(OBJDIR):
            os.remove(os.path.join(OBJDIR, f))
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if _stale(LIB, objs):
        cmd = [_nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-Xcompiler", "-fPIC", "-lcublas"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed\n%s\n%s" % (r.stdout, r.stderr))
    _build_driver(verbose)
    return LIB


DRIVER_SRC = os.path.join(HERE, "driver", "nnpp_run.cpp")
DRIVER = os.path.join(HERE, "nnpp_run")


def _build_driver(verbose):
    """The C++ job-file driver, linked against the library (rpath $ORIGIN)."""
    if not _stale(DRIVER, [DRIVER_SRC, LIB, os.path.join(INCLUDE, "nnpp_gb300.h")]):
        return DRIVER
    cmd = ["g++"] + CXX_FLAGS + [DRIVER_SRC, "-o", DRIVER, "-L", HERE, "-lnnpp_gb300", "-pthread",
                                 "-Wl,-rpath,$ORIGIN"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("driver build failed\n%s\n%s" % (r.stdout, r.stderr))
    return DRIVER


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
