"""ctypes binding of libptw.so (declarations mirror include/ptw.h)."""
import ctypes
import os

from . import _build

PTW_OK = 0
PTW_EINVAL = -1
PTW_ENOMEM = -2
PTW_ECUDA = -3
PTW_ETIMEOUT = -4
PTW_EIO = -5
PTW_EFULL = -6
PTW_EBUSY = -7

PTW_FMT_BINARY = 0
PTW_FMT_TEXT = 1

PTW_START_PER_VERTEX = 0
PTW_START_UNIFORM = 1
PTW_START_SOURCES = 2

_ERRNAMES = {PTW_EINVAL: "PTW_EINVAL", PTW_ENOMEM: "PTW_ENOMEM", PTW_ECUDA: "PTW_ECUDA",
             PTW_ETIMEOUT: "PTW_ETIMEOUT", PTW_EIO: "PTW_EIO", PTW_EFULL: "PTW_EFULL",
             PTW_EBUSY: "PTW_EBUSY"}


class GraphInfo(ctypes.Structure):
    _fields_ = [("n_vertices", ctypes.c_uint32), ("id_bound", ctypes.c_uint32),
                ("n_edges", ctypes.c_uint64), ("max_degree", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32), ("device_bytes", ctypes.c_uint64)]


class WalkCfg(ctypes.Structure):
    _fields_ = [("n_walkers", ctypes.c_uint64), ("sp", ctypes.c_double),
                ("seed", ctypes.c_uint64), ("start_mode", ctypes.c_int32),
                ("max_moves", ctypes.c_uint32), ("h_sources", ctypes.POINTER(ctypes.c_uint32)),
                ("n_sources", ctypes.c_uint32), ("reserved", ctypes.c_uint32),
                ("first_walker", ctypes.c_uint64)]


class WalkStats(ctypes.Structure):
    _fields_ = [("walkers", ctypes.c_uint64), ("moves", ctypes.c_uint64),
                ("visits", ctypes.c_uint64), ("kernel_ms", ctypes.c_float),
                ("total_ms", ctypes.c_float)]


class Node2vecStats(ctypes.Structure):
    _fields_ = [("walkers", ctypes.c_uint64), ("moves", ctypes.c_uint64),
                ("trials", ctypes.c_uint64), ("checks", ctypes.c_uint64), ("probes", ctypes.c_uint64),
                ("kernel_ms", ctypes.c_float), ("total_ms", ctypes.c_float)]


class Query(ctypes.Structure):
    _fields_ = [("source", ctypes.c_uint32), ("query_id", ctypes.c_uint32), ("budget", ctypes.c_uint64)]


class BatchCfg(ctypes.Structure):
    _fields_ = [("sp", ctypes.c_double), ("seed", ctypes.c_uint64), ("app", ctypes.c_int32),
                ("max_moves", ctypes.c_uint32), ("table_bytes", ctypes.c_uint64),
                ("table_factor", ctypes.c_double), ("top_k", ctypes.c_uint32), ("flags", ctypes.c_uint32)]


PTW_BATCH_DEVICE_RESULTS = 1


class BatchPhases(ctypes.Structure):
    _fields_ = [("call_ms", ctypes.c_double), ("plan_ms", ctypes.c_double), ("device_ms", ctypes.c_double),
                ("upload_ms", ctypes.c_double), ("walk_ms", ctypes.c_double), ("count_ms", ctypes.c_double),
                ("place_ms", ctypes.c_double), ("copy_ms", ctypes.c_double), ("copy_tail_ms", ctypes.c_double),
                ("host_pages_ms", ctypes.c_double), ("copy_bytes", ctypes.c_uint64), ("waves", ctypes.c_uint32),
                ("reruns", ctypes.c_uint32)]


class BatchTune(ctypes.Structure):
    _fields_ = [("desc_walkers", ctypes.c_uint32), ("blocks_per_sm", ctypes.c_uint32),
                ("group_bytes", ctypes.c_uint64), ("dense_ratio", ctypes.c_uint32),
                ("ext_columns", ctypes.c_int32)]


class ServeStats(ctypes.Structure):
    _fields_ = [("ticks", ctypes.c_uint64), ("moves", ctypes.c_uint64), ("walkers", ctypes.c_uint64),
                ("completed", ctypes.c_uint64), ("entries", ctypes.c_uint64), ("retries", ctypes.c_uint64),
                ("pinned_bytes", ctypes.c_uint64), ("active", ctypes.c_uint32), ("pending", ctypes.c_uint32),
                ("step_ms", ctypes.c_double), ("device_ms", ctypes.c_double), ("collect_ms", ctypes.c_double)]


PTW_APP_VISITS = 0
PTW_APP_ENDPOINT = 1


class ServeCfg(ctypes.Structure):
    _fields_ = [("sp", ctypes.c_double), ("seed", ctypes.c_uint64), ("app", ctypes.c_int32),
                ("max_moves", ctypes.c_uint32), ("table_bytes", ctypes.c_uint64),
                ("tick_walkers", ctypes.c_uint64), ("max_active", ctypes.c_uint32),
                ("use_graph", ctypes.c_uint32), ("table_factor", ctypes.c_double),
                ("top_k", ctypes.c_uint32), ("staging_mb", ctypes.c_uint32)]


class ServeResult(ctypes.Structure):
    _fields_ = [("query_id", ctypes.c_uint32), ("source", ctypes.c_uint32), ("budget", ctypes.c_uint64),
                ("n_entries", ctypes.c_uint64), ("submit_s", ctypes.c_double),
                ("admit_s", ctypes.c_double), ("done_s", ctypes.c_double)]


class Tune(ctypes.Structure):
    _fields_ = [("block", ctypes.c_int32), ("ilp", ctypes.c_int32), ("chunk", ctypes.c_int32),
                ("hot_k", ctypes.c_int32), ("blocks_per_sm", ctypes.c_int32),
                ("min_blocks", ctypes.c_int32), ("paths_ilp", ctypes.c_int32),
                ("cache_hints", ctypes.c_int32), ("paths_named", ctypes.c_int32),
                ("ext_columns", ctypes.c_int32), ("gather_slots", ctypes.c_int32),
                ("warp_agg", ctypes.c_int32)]


# Every symbol include/ptw.h declares: (name, restype, argtypes).
_vp = ctypes.c_void_p
_u32p = ctypes.POINTER(ctypes.c_uint32)
_u64p = ctypes.POINTER(ctypes.c_uint64)
_i32p = ctypes.POINTER(ctypes.c_int32)
_f32p = ctypes.POINTER(ctypes.c_float)
_G = ctypes.c_void_p
_GP = ctypes.POINTER(ctypes.c_void_p)
SIGNATURES = [
    ("ptw_last_error", ctypes.c_char_p, []),
    ("ptw_version", ctypes.c_char_p, []),
    ("ptw_trim_memory", ctypes.c_int, []),
    ("ptw_graph_load", ctypes.c_int, [ctypes.c_char_p, ctypes.c_int32, ctypes.c_int32, _GP]),
    ("ptw_graph_from_edges", ctypes.c_int, [_u32p, _u32p, ctypes.c_uint64, ctypes.c_int32, _GP]),
    ("ptw_graph_from_csr", ctypes.c_int, [_u64p, _u32p, ctypes.c_uint32, _u32p, _GP]),
    ("ptw_graph_rmat", ctypes.c_int, [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_double,
                                      ctypes.c_double, ctypes.c_double, ctypes.c_uint64,
                                      ctypes.c_int32, _GP]),
    ("ptw_graph_get_info", ctypes.c_int, [_G, ctypes.POINTER(GraphInfo)]),
    ("ptw_graph_export_csr", ctypes.c_int, [_G, _u32p, _u64p, _u32p]),
    ("ptw_graph_export_edges", ctypes.c_int, [_G, _u32p, _u32p]),
    ("ptw_graph_save", ctypes.c_int, [_G, ctypes.c_char_p, ctypes.c_int32]),
    ("ptw_graph_free", None, [_G]),
    ("ptw_graph_set_tune", ctypes.c_int, [_G, ctypes.POINTER(Tune)]),
    ("ptw_graph_get_tune", ctypes.c_int, [_G, ctypes.POINTER(Tune)]),
    ("ptw_pagerank", ctypes.c_int, [_G, ctypes.POINTER(WalkCfg), _vp, ctypes.POINTER(WalkStats)]),
    ("ptw_pagerank_dev", ctypes.c_int, [_G, ctypes.POINTER(WalkCfg), _vp, ctypes.POINTER(WalkStats)]),
    ("ptw_pagerank_submit", ctypes.c_int, [_G, ctypes.POINTER(WalkCfg), _vp, ctypes.POINTER(ctypes.c_uint64)]),
    ("ptw_pagerank_wait", ctypes.c_int, [_G, ctypes.c_uint64, ctypes.POINTER(WalkStats)]),
    ("ptw_rwr", ctypes.c_int, [_G, ctypes.POINTER(WalkCfg), _vp, ctypes.POINTER(WalkStats)]),
    ("ptw_rwr_dev", ctypes.c_int, [_G, ctypes.POINTER(WalkCfg), _vp, ctypes.POINTER(WalkStats)]),
    ("ptw_deepwalk", ctypes.c_int, [_G, ctypes.POINTER(WalkCfg), ctypes.c_uint32, _vp,
                                    ctypes.POINTER(WalkStats)]),
    ("ptw_deepwalk_dev", ctypes.c_int, [_G, ctypes.POINTER(WalkCfg), ctypes.c_uint32, _vp,
                                        ctypes.POINTER(WalkStats)]),
    ("ptw_node2vec", ctypes.c_int, [_G, ctypes.POINTER(WalkCfg), ctypes.c_uint32, ctypes.c_double,
                                    ctypes.c_double, _vp, ctypes.POINTER(Node2vecStats)]),
    ("ptw_node2vec_dev", ctypes.c_int, [_G, ctypes.POINTER(WalkCfg), ctypes.c_uint32, ctypes.c_double,
                                        ctypes.c_double, _vp, ctypes.POINTER(Node2vecStats)]),
    ("ptw_graph_sync", ctypes.c_int, [_G]),
    ("ptw_graph_set_stream", ctypes.c_int, [_G, _vp]),
    ("ptw_autotune", ctypes.c_int, [_G, ctypes.c_double, ctypes.c_uint64, ctypes.POINTER(Tune)]),
    ("ptw_probe_gather", ctypes.c_int, [ctypes.c_uint64, ctypes.c_uint32, ctypes.POINTER(ctypes.c_double)]),
    ("ptw_pagerank_noalloc", ctypes.c_int, [_G, ctypes.POINTER(WalkCfg), _vp, _vp]),
    ("ptw_ppr_batch", ctypes.c_int, [_G, ctypes.POINTER(Query), ctypes.c_uint32,
                                     ctypes.POINTER(BatchCfg), _GP]),
    ("ptw_ppr_batch_resumable", ctypes.c_int, [_G, ctypes.POINTER(Query), ctypes.c_uint32,
                                               ctypes.POINTER(BatchCfg), ctypes.c_char_p, ctypes.c_uint32, _GP]),
    ("ptw_batch_info", ctypes.c_int, [_G, ctypes.POINTER(ctypes.c_uint32), _u64p,
                                      ctypes.POINTER(WalkStats)]),
    ("ptw_batch_export", ctypes.c_int, [_G, _u64p, _u32p, _u32p]),
    ("ptw_batch_view", ctypes.c_int, [_G, ctypes.POINTER(_u64p), ctypes.POINTER(_u32p),
                                      ctypes.POINTER(_u32p)]),
    ("ptw_batch_free", None, [_G]),
    ("ptw_batch_view_device", ctypes.c_int, [_G, ctypes.POINTER(_u64p), ctypes.POINTER(_u32p),
                                             ctypes.POINTER(_u32p)]),
    ("ptw_batch_get_phases", ctypes.c_int, [_G, ctypes.POINTER(BatchPhases)]),
    ("ptw_graph_set_batch_tune", ctypes.c_int, [_G, ctypes.POINTER(BatchTune)]),
    ("ptw_graph_get_batch_tune", ctypes.c_int, [_G, ctypes.POINTER(BatchTune)]),
    ("ptw_autotune_batch", ctypes.c_int, [_G, ctypes.POINTER(Query), ctypes.c_uint32, ctypes.POINTER(BatchCfg),
                                          ctypes.POINTER(BatchTune), ctypes.POINTER(ctypes.c_double)]),
    ("ptw_batch_l1", ctypes.c_int, [_G, _G, ctypes.c_double, ctypes.c_int32, ctypes.c_double,
                                    ctypes.POINTER(ctypes.c_double)]),
    ("ptw_batch_l1_many", ctypes.c_int, [_G, ctypes.POINTER(ctypes.c_void_p), ctypes.c_uint32, ctypes.c_double,
                                         ctypes.c_int32, ctypes.c_double, ctypes.POINTER(ctypes.c_double)]),
    ("ptw_batch_l1_pair", ctypes.c_int, [_G, _G, _G, ctypes.POINTER(ctypes.c_double)]),
    ("ptw_serve_open", ctypes.c_int, [_G, ctypes.POINTER(ServeCfg), _GP]),
    ("ptw_serve_submit", ctypes.c_int, [_G, ctypes.POINTER(Query)]),
    ("ptw_serve_step", ctypes.c_int, [_G, _u32p, _u32p, _u32p]),
    ("ptw_serve_poll", ctypes.c_int, [_G, ctypes.POINTER(ServeResult)]),
    ("ptw_serve_take", ctypes.c_int, [_G, _u32p, _u32p]),
    ("ptw_serve_view", ctypes.c_int, [_G, ctypes.POINTER(_u32p), ctypes.POINTER(_u32p)]),
    ("ptw_serve_get_stats", ctypes.c_int, [_G, ctypes.POINTER(ServeStats)]),
    ("ptw_serve_clock", ctypes.c_double, [_G]),
    ("ptw_serve_close", None, [_G]),
    ("ptw_serve_save", ctypes.c_int, [_G, ctypes.c_char_p]),
    ("ptw_serve_restore", ctypes.c_int, [_G, ctypes.c_char_p, _GP]),
    ("ptw_graph_chung_lu", ctypes.c_int, [ctypes.c_uint32, ctypes.c_double, ctypes.c_double,
                                          ctypes.c_uint64, _GP]),
    ("ptw_source_features", ctypes.c_int, [_G, _u32p, ctypes.c_uint32, _f32p]),
    ("ptw_mlp_create", ctypes.c_int, [ctypes.c_uint64, _GP]),
    ("ptw_mlp_set_params", ctypes.c_int, [_G, _f32p, _f32p]),
    ("ptw_mlp_get_params", ctypes.c_int, [_G, _f32p, _f32p]),
    ("ptw_mlp_forward", ctypes.c_int, [_G, _f32p, ctypes.c_uint32, _f32p]),
    ("ptw_mlp_grad", ctypes.c_int, [_G, _f32p, _f32p, ctypes.c_uint32, ctypes.POINTER(ctypes.c_double),
                                    _f32p]),
    ("ptw_mlp_train", ctypes.c_int, [_G, _f32p, _f32p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                     ctypes.c_float, ctypes.c_uint64, _f32p]),
    ("ptw_mlp_free", None, [_G]),
]

PTW_MLP_IN = 8
PTW_MLP_HIDDEN = 64
PTW_MLP_NPARAMS = 4801
PTW_MLP_NNORM = 18

PTW_NOALLOC_MAX_VERTICES = 1 << 22

_lib = None


def checked():
    """True when PTW_CHECKED=1 selects the index-checked build of the library."""
    return os.environ.get("PTW_CHECKED", "") == "1"


def lib_path():
    return _build.CHECKED_SO if checked() else _build.SO


def load(build_if_missing=True):
    """Loads libptw.so (the index-checked build when PTW_CHECKED=1); builds
    it first when it is missing or stale."""
    global _lib
    if _lib is not None:
        return _lib
    if checked():
        if build_if_missing:
            _build.build_checked()
    elif build_if_missing and not _build.up_to_date():
        _build.build()
    path = lib_path()
    if not os.path.exists(path):
        raise ImportError("%s is not built; run ptwalker_gb300._build.build()" % path)
    lib = ctypes.CDLL(path)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class PTWError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (_ERRNAMES.get(code, "PTW_ERR"), code, msg))
        self.code = code


def check(rc):
    if rc != PTW_OK:
        msg = load().ptw_last_error().decode("utf-8", "replace")
        raise PTWError(rc, msg)
    return rc
