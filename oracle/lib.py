"""Build and load ``oracle.c`` (test infrastructure, see ``oracle/__init__``)."""
import ctypes
import os
import subprocess

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "oracle.c")
_SRCS = [_SRC, os.path.join(_HERE, "partitioned.c")]
_OUT_DIR = os.path.join(_HERE, "_build")
_SO = os.path.join(_OUT_DIR, "liboracle.so")
_lib = None


def build_lib(force=False):
    """Compile oracle.c with gcc + OpenMP; returns the .so path."""
    os.makedirs(_OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(_SO)
            and all(os.path.getmtime(_SO) >= os.path.getmtime(f) for f in _SRCS)):
        return _SO
    tmp = _SO + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-std=c11", *_SRCS, "-o", tmp]
    subprocess.check_call(cmd)
    os.replace(tmp, _SO)
    return _SO


def load_lib():
    global _lib
    if _lib is not None:
        return _lib
    lib = ctypes.CDLL(build_lib())
    u32p = ctypes.POINTER(ctypes.c_uint32)
    u64p = ctypes.POINTER(ctypes.c_uint64)
    i32p = ctypes.POINTER(ctypes.c_int32)
    lib.ora_philox4x32_10.argtypes = [u32p, u32p, u32p]
    lib.ora_philox4x32_10.restype = None
    lib.ora_rmat_edges.argtypes = [ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint64,
                                   ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                   ctypes.c_uint64, u32p, u32p]
    lib.ora_rmat_edges.restype = None
    lib.ora_replay_walks.argtypes = [u64p, u32p, ctypes.c_uint32, ctypes.c_uint64,
                                     ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64,
                                     ctypes.c_int, u32p, ctypes.c_uint32, ctypes.c_uint32,
                                     u32p, u32p, u32p, ctypes.c_int]
    lib.ora_replay_walks.restype = ctypes.c_uint64
    lib.ora_replay_paths.argtypes = [u64p, u32p, ctypes.c_uint32, ctypes.c_uint64,
                                     ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint64,
                                     ctypes.c_int, u32p, ctypes.c_uint32, i32p, ctypes.c_int]
    lib.ora_replay_paths.restype = None
    lib.ora_replay_node2vec.argtypes = [u64p, u32p, ctypes.c_uint32, ctypes.c_uint64,
                                        ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint64,
                                        ctypes.c_double, ctypes.c_double, ctypes.c_int, u32p,
                                        ctypes.c_uint32, ctypes.c_int, i32p, ctypes.c_int]
    lib.ora_replay_node2vec.restype = ctypes.c_uint64
    lib.ora_n2v_fold.argtypes = [ctypes.c_double, ctypes.c_double, u64p]
    lib.ora_n2v_fold.restype = ctypes.c_int
    lib.ora_csr_simple_symmetric.argtypes = [u64p, u32p, ctypes.c_uint32]
    lib.ora_csr_simple_symmetric.restype = ctypes.c_int
    lib.ora_n2v_thresholds.argtypes = [ctypes.c_double, ctypes.c_double, u64p]
    lib.ora_n2v_thresholds.restype = None
    lib.ora_rmat_clean_csr.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                       ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64,
                                       ctypes.c_int, ctypes.POINTER(ctypes.c_uint32),
                                       ctypes.POINTER(ctypes.c_uint64),
                                       ctypes.POINTER(u64p), ctypes.POINTER(u32p)]
    lib.ora_rmat_clean_csr.restype = ctypes.c_int
    lib.ora_partitioned_walks.argtypes = [u64p, u32p, ctypes.c_uint32, u32p, ctypes.c_uint64, ctypes.c_uint64,
                                          ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int, u32p, ctypes.c_uint32,
                                          ctypes.c_uint32, ctypes.c_uint64, u32p, ctypes.c_int, u64p]
    lib.ora_partitioned_walks.restype = ctypes.c_uint64
    lib.ora_degree_relabel.argtypes = [u64p, u32p, ctypes.c_uint32, u32p, u64p, u32p, ctypes.c_int]
    lib.ora_degree_relabel.restype = ctypes.c_int
    lib.ora_free.argtypes = [ctypes.c_void_p]
    lib.ora_free.restype = None
    _lib = lib
    return lib
