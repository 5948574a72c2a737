"""Builds the reference baseline binary oracle/_ref/ptw_ref_walk.

TEST INFRASTRUCTURE.  Compiles the reference's own sources where they lie
(src/core/pagerank.cpp with the headers it includes from include/,
src/core/ and third_party/) against the project-written shims in
oracle/ref/shim for the libraries absent from this image (glog, libnuma,
the args flag parser; immintrin on aarch64), with ref_walk.cpp as main.
Nothing is copied out of the reference tree.  Flags follow the reference's
CMakeLists.txt:39-58 (-O3, OpenMP, PROFILE_LEVEL=PROFILE_BRIEF) minus the
host-specific -march=native / -mclflushopt, so the binary builds on x86_64
and aarch64 alike.

The reference tree is named by --ref or by the environment variable
PTW_REFERENCE_DIR; without either nothing is built (an existing binary is
still returned).

Usage: python oracle/ref/build_ref.py --ref /path/to/reference [--force]
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(os.path.dirname(HERE), "_ref")
BIN = os.path.join(OUT_DIR, "ptw_ref_walk")
REF_ENV = "PTW_REFERENCE_DIR"


def reference_dir(ref=None):
    """The reference tree: the argument, else $PTW_REFERENCE_DIR, else None."""
    return ref or os.environ.get(REF_ENV) or None


def build(ref=None, force=False):
    """Returns the binary path, or None when no reference tree is named."""
    ref = reference_dir(ref)
    if not ref or not os.path.isdir(os.path.join(ref, "src", "core")):
        return BIN if os.path.exists(BIN) else None
    srcs = [os.path.join(HERE, "ref_walk.cpp")]
    shim = os.path.join(HERE, "shim")
    deps = srcs + [os.path.join(shim, f) for f in ("numa.h", "numaif.h", "args.hxx", "immintrin.h")]
    if (not force and os.path.exists(BIN)
            and all(os.path.getmtime(d) <= os.path.getmtime(BIN) for d in deps)):
        return BIN
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = BIN + ".tmp%d" % os.getpid()
    cmd = ["g++", "-O3", "-std=c++14", "-fopenmp", "-w",
           "-DPROFILE_LEVEL=PROFILE_BRIEF",
           "-I", shim,
           "-I", os.path.join(ref, "include"),
           "-I", os.path.join(ref, "src", "core"),
           "-I", os.path.join(ref, "third_party"),
           *srcs, "-o", tmp]
    subprocess.check_call(cmd)
    os.replace(tmp, BIN)
    return BIN


if __name__ == "__main__":
    ref = None
    if "--ref" in sys.argv:
        ref = sys.argv[sys.argv.index("--ref") + 1]
    print(build(ref, force="--force" in sys.argv))
