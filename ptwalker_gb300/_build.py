"""Compiles libptw.so in-tree for sm_103a (GB300) with nvcc.

Translation units are compiled in parallel, then linked with a static CUDA
runtime so the library does not depend on which libcudart the host process
(e.g. PyTorch) loaded.  Output: ptwalker_gb300/_lib/libptw.so.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
SO = os.path.join(OUT, "libptw.so")
SOURCES = ["graph.cu", "walk.cu", "capi.cu", "noalloc.cu", "batch.cu", "exact.cu", "serve.cu", "mlp.cu", "probe.cu", "node2vec.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O2",
              "--expt-relaxed-constexpr"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(HERE, "..", "include", "ptw.h"))
    files.append(os.path.join(HERE, "cli", "ptw_cli.cpp"))
    files.append(os.path.abspath(__file__))
    return files


def up_to_date():
    if not os.path.exists(SO):
        return False
    t = os.path.getmtime(SO)
    if not all(os.path.lexists(os.path.join(OUT, "bin", a)) for a in APPS):
        return False
    return all(os.path.getmtime(f) <= t for f in _deps())


def build(force=False, verbose=False, extra_flags=()):
    if not force and up_to_date():
        return SO
    _compile_and_link(OUT, SO, extra_flags, verbose)
    build_cli()
    return SO


# The checked build (-DPTW_CHECKED): every kernel index the engine derives
# from data is checked against its bound; a failure is recorded on the
# device, the access is redirected in bounds, and the entry point returns
# PTW_ECUDA naming the failing sites.  Loaded instead of the normal library
# when PTW_CHECKED=1 is set in the environment.
CHECKED_OUT = os.path.join(OUT, "checked")
CHECKED_SO = os.path.join(CHECKED_OUT, "libptw.so")


def build_checked(force=False, verbose=False):
    if (not force and os.path.exists(CHECKED_SO)
            and all(os.path.getmtime(f) <= os.path.getmtime(CHECKED_SO) for f in _deps())):
        return CHECKED_SO
    _compile_and_link(CHECKED_OUT, CHECKED_SO, ["-DPTW_CHECKED"], verbose)
    return CHECKED_SO


def _compile_and_link(out_dir, so, extra_flags, verbose):
    os.makedirs(os.path.join(out_dir, "obj"), exist_ok=True)
    nvcc = _nvcc()

    def compile_one(src):
        obj = os.path.join(out_dir, "obj", src.replace(".cu", ".o"))
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, *extra_flags, "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = so + ".tmp%d" % os.getpid()
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-Xcompiler", "-fPIC"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, so)


CLI_SRC = os.path.join(HERE, "cli", "ptw_cli.cpp")
BIN_DIR = os.path.join(OUT, "bin")
APPS = ("pagerank", "ppr", "PPR", "rwr", "RWR", "deepwalk", "node2vec")


def build_cli():
    """C++ command-line apps linked against libptw.so (rpath to _lib)."""
    os.makedirs(BIN_DIR, exist_ok=True)
    exe = os.path.join(BIN_DIR, "ptw_cli")
    tmp = exe + ".tmp%d" % os.getpid()
    cmd = ["g++", "-O2", "-std=c++17", CLI_SRC, "-o", tmp, "-L", OUT, "-lptw",
           "-Wl,-rpath,$ORIGIN/.."]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("CLI build failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, exe)
    for app in APPS:
        link = os.path.join(BIN_DIR, app)
        if os.path.lexists(link):
            os.unlink(link)
        os.symlink("ptw_cli", link)
    return exe


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True,
                extra_flags=["-Xptxas", "-v"] if "--ptxas-v" in sys.argv else []))
