"""Build recipe of the oracle (test infrastructure).

Compiles
  oracle/nnpp_oracle.cpp  -> oracle/liboracle.so        (always; g++ with OpenMP)
  oracle/ref_shim.cpp     -> oracle/_ref/libnnpp_ref.so (only where the reference's
                             sources are present: the checkout named by the environment
                             variable NNPP_REFERENCE_ROOT, else a checkout named
                             "reference" beside this repository)
The reference shim is compiled from the reference's own headers where they lie; nothing of
the reference is copied into this repository.  Both libraries are checkers for the tests,
never part of the product.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REFERENCE_ROOT = os.environ.get(
    "NNPP_REFERENCE_ROOT", os.path.normpath(os.path.join(HERE, "..", "..", "reference")))

# -ffp-contract=off: the reference is built without FMA contraction on x86-64 (-msse2,
# CMakeLists.txt:51-54); keeping products and sums separate makes the restatement give the
# same roundings on aarch64 hosts, where GCC would otherwise fuse them.
CXXFLAGS = ["-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-std=c++17"]


def _newer(target, sources):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


# The seeded workload generator (host C++, no CUDA) is compiled into the oracle library as
# well, so that the CPU-baseline and reference arms of the benchmark build their inputs
# without loading the product library.
PKG_CSRC = os.path.join(HERE, "..", "nnpp-mg-implant-corrosion-3d_gb300", "csrc")
SYNTH_SRCS = [os.path.join(PKG_CSRC, "synth.cpp"), os.path.join(PKG_CSRC, "errors.cpp")]


def _native_flag():
    """The host's own instruction set: -march=native where GCC accepts it (x86-64), else
    -mcpu=native (aarch64); None when neither compiles."""
    for flag in ("-march=native", "-mcpu=native"):
        r = subprocess.run(["g++", flag, "-x", "c++", "-fsyntax-only", "-"], input="int main(){}",
                           capture_output=True, text=True)
        if r.returncode == 0:
            return flag
    return None


def build_oracle(force=False, verbose=False, native=False):
    """liboracle.so (portable flags), or with native=True liboracle_native.so, the same
    sources for the host's own instruction set (the timed CPU baseline; -ffp-contract=off
    keeps every rounding, so both give the same bits).  Returns None for a native build the
    compiler does not support."""
    extra = []
    if native:
        flag = _native_flag()
        if flag is None:
            return None
        extra = [flag]
    out = os.path.join(HERE, "liboracle_native.so" if native else "liboracle.so")
    srcs = [os.path.join(HERE, "nnpp_oracle.cpp"),
            os.path.join(HERE, "..", "include", "nnpp_gb300.h"),
            os.path.abspath(__file__)] + SYNTH_SRCS
    if force or not _newer(out, srcs):
        cmd = ["g++"] + CXXFLAGS + extra + ["-I", os.path.join(HERE, "..", "include"), "-I", PKG_CSRC,
                                            srcs[0]] + SYNTH_SRCS + ["-o", out]
        if verbose:
            print(" ".join(cmd))
        subprocess.run(cmd, check=True)
    return out


def build_reference_shim(force=False, verbose=False):
    """Returns the path of the shim, or None when the reference is not present."""
    helpers = os.path.join(REFERENCE_ROOT, "src", "helpers")
    eigen = os.path.join(REFERENCE_ROOT, "eigen")
    kdtree = os.path.join(REFERENCE_ROOT, "libraries", "libkdtree++")
    if not (os.path.isdir(helpers) and os.path.isdir(eigen)):
        return None
    outdir = os.path.join(HERE, "_ref")
    os.makedirs(outdir, exist_ok=True)
    out = os.path.join(outdir, "libnnpp_ref.so")
    src = os.path.join(HERE, "ref_shim.cpp")
    deps = [src, os.path.join(helpers, "grid.h"), os.path.join(helpers, "utils.h"),
            os.path.join(helpers, "kd_tree_interface.h"), os.path.abspath(__file__)]
    if force or not _newer(out, deps):
        cmd = ["g++"] + CXXFLAGS + ["-w", "-I", helpers, "-I", eigen, "-I", kdtree, src, "-o", out]
        if verbose:
            print(" ".join(cmd))
        subprocess.run(cmd, check=True)
    return out


if __name__ == "__main__":
    force = "--force" in sys.argv
    print(build_oracle(force, True))
    print(build_oracle(force, True, native=True))
    print(build_reference_shim(force, True))
