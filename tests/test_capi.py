"""CPU checks of the C ABI: libptw.so builds for sm_103a, loads, and exports
every entry point include/ptw.h declares; the Python binding covers exactly
that set.  No compute calls (no GPU here)."""
import ctypes
import os
import re

import numpy as np
import pytest

from ptwalker_gb300 import _build, _capi
from ptwalker_gb300 import api

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    text = open(os.path.join(ROOT, "include", "ptw.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ptw_[a-z0-9_]+)\s*\(", text)))


def test_library_builds_and_exports_header_symbols():
    so = _build.build()
    lib = ctypes.CDLL(so)
    names = header_functions()
    assert len(names) >= 18
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_matches_header():
    bound = sorted(n for n, _, _ in _capi.SIGNATURES)
    assert bound == header_functions()


def test_struct_layouts(tmp_path):
    """ctypes structs match the C compiler's layout of include/ptw.h."""
    structs = {"ptw_graph_info": _capi.GraphInfo, "ptw_walk_cfg": _capi.WalkCfg,
               "ptw_walk_stats": _capi.WalkStats, "ptw_tune": _capi.Tune,
               "ptw_query": _capi.Query, "ptw_batch_cfg": _capi.BatchCfg,
               "ptw_serve_cfg": _capi.ServeCfg, "ptw_serve_result": _capi.ServeResult,
               "ptw_node2vec_stats": _capi.Node2vecStats,
               "ptw_serve_stats": _capi.ServeStats, "ptw_batch_phases": _capi.BatchPhases,
               "ptw_batch_tune": _capi.BatchTune}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "ptw.h"', "int main(void){"]
    for cname, py in structs.items():
        lines.append('printf("%%zu\\n", sizeof(%s));' % cname)
        for fname, _ in py._fields_:
            lines.append('printf("%%zu\\n", offsetof(%s, %s));' % (cname, fname))
    lines.append("return 0;}")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    import subprocess
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    got = [int(x) for x in subprocess.check_output([str(exe)]).split()]
    want = []
    for py in structs.values():
        want.append(ctypes.sizeof(py))
        want.extend(getattr(py, f).offset for f, _ in py._fields_)
    assert got == want


def test_version_and_errors_without_gpu():
    lib = _capi.load()
    assert b"sm_103a" in lib.ptw_version()
    # argument checks run before any device call
    rc = lib.ptw_graph_from_edges(None, None, 0, 0, ctypes.byref(ctypes.c_void_p()))
    assert rc == _capi.PTW_EINVAL
    assert b"empty" in lib.ptw_last_error()
    row = (ctypes.c_uint64 * 3)(0, 2, 1)
    col = (ctypes.c_uint32 * 2)(1, 0)
    rc = lib.ptw_graph_from_csr(row, col, 2, None, ctypes.byref(ctypes.c_void_p()))
    assert rc == _capi.PTW_EINVAL and b"decreases at row 1" in lib.ptw_last_error()
    rc = lib.ptw_graph_from_csr(None, col, 0, None, ctypes.byref(ctypes.c_void_p()))
    assert rc == _capi.PTW_EINVAL
    out = ctypes.c_double()
    assert lib.ptw_probe_gather(1 << 30, 3, ctypes.byref(out)) == _capi.PTW_EINVAL
    assert lib.ptw_probe_gather(16 << 30, 8, ctypes.byref(out)) == _capi.PTW_EINVAL
    rc = lib.ptw_graph_load(b"/nonexistent/file", _capi.PTW_FMT_TEXT, 0, ctypes.byref(ctypes.c_void_p()))
    assert rc == _capi.PTW_EIO
    rc = lib.ptw_graph_load(b"x", 7, 0, ctypes.byref(ctypes.c_void_p()))
    assert rc == _capi.PTW_EINVAL
    rc = lib.ptw_graph_rmat(0, 16, 0.57, 0.19, 0.19, 1, 1, ctypes.byref(ctypes.c_void_p()))
    assert rc == _capi.PTW_EINVAL
    rc = lib.ptw_graph_rmat(10, 16, 0.6, 0.3, 0.3, 1, 1, ctypes.byref(ctypes.c_void_p()))
    assert rc == _capi.PTW_EINVAL
    cfg = _capi.WalkCfg()
    rc = lib.ptw_pagerank(None, ctypes.byref(cfg), None, None)
    assert rc == _capi.PTW_EINVAL
    err = _capi.PTWError(rc, "x")
    assert "PTW_EINVAL" in str(err)


def test_malformed_text_edge_list_is_an_io_error(tmp_path):
    lib = _capi.load()
    p = tmp_path / "bad.txt"
    p.write_text("# comment\n0 1\n1 x\n")
    rc = lib.ptw_graph_load(str(p).encode(), _capi.PTW_FMT_TEXT, 0, ctypes.byref(ctypes.c_void_p()))
    assert rc == _capi.PTW_EIO
    assert b"line 3" in lib.ptw_last_error()
    p.write_bytes(b"\x00" * 12)
    rc = lib.ptw_graph_load(str(p).encode(), _capi.PTW_FMT_BINARY, 0, ctypes.byref(ctypes.c_void_p()))
    assert rc == _capi.PTW_EIO


def test_cli_rejects_bad_flags_without_a_gpu(tmp_path):
    import subprocess
    _build.build()
    for app in ("pagerank", "PPR", "RWR", "deepwalk"):
        r = subprocess.run([os.path.join(_build.BIN_DIR, app), "--help"], capture_output=True, text=True)
        assert r.returncode == 0 and r.stdout.startswith("usage:")
    exe = os.path.join(_build.BIN_DIR, "pagerank")
    r = subprocess.run([exe, "-f", "text", "-g", "x", "-w", "5", "--sp", "0.1", "--bogus", "1"],
                       capture_output=True, text=True)
    assert r.returncode == 1 and "unknown flag --bogus" in r.stderr
    r = subprocess.run([exe, "-f", "text", "-g", "x", "-w", "5"], capture_output=True, text=True)
    assert r.returncode == 1 and "--sp is required" in r.stderr
    r = subprocess.run([exe, "-f", "text", "-g", "x", "-w", "5", "-e", "2", "--sp", "0.1"],
                       capture_output=True, text=True)
    assert r.returncode == 1 and "exactly one of -w and -e" in r.stderr
    bad = tmp_path / "bad.txt"
    bad.write_text("0 1\nfoo\n")
    r = subprocess.run([exe, "-f", "text", "-g", str(bad), "-w", "5", "--sp", "0.1"],
                       capture_output=True, text=True)
    assert r.returncode == 2 and "malformed edge at line 2" in r.stderr


def test_cfg_builder():
    cfg, keep = api._cfg(10, 0.15, -1, "sources", [3, 4], 0, first_walker=7 << 32)
    assert cfg.seed == 0xFFFFFFFFFFFFFFFF
    assert cfg.start_mode == _capi.PTW_START_SOURCES and cfg.n_sources == 2
    assert list(keep) == [3, 4] and cfg.first_walker == 7 << 32
    with pytest.raises(ValueError):
        api._cfg(10, 0.15, 0, "uniform", [1], 0)
    with pytest.raises(KeyError):
        api._cfg(10, 0.15, 0, "nope", None, 0)
    t = api.Tune(block=128, ilp=4, chunk=64, hot_k=1024)
    assert api.Tune.from_c(t.to_c()).as_dict() == t.as_dict()
    with pytest.raises(ValueError):
        api._host_ptr(np.zeros(4, dtype=np.uint32)[::2])


def test_integration_examples_compile(tmp_path):
    """The C++ binding and serving examples of INTEGRATION.md compile against
    include/ptw.h as written."""
    import subprocess
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    blocks = re.findall(r"```cpp\n(.*?)```", text, re.S)
    binding = [b for b in blocks if "ptw_walk.hpp" in b]
    serving = [b for b in blocks if "ptw_serve_cfg cfg{}" in b]
    assert binding and serving
    src = binding[0] + """
static void consume(uint64_t, const uint32_t *, const uint32_t *, uint64_t) {}
int main() {
    PtwGraph G("graph.txt", false);
    std::vector<uint32_t> c = ptw_walk_counts(G, 10, 0.15, 1, {});
    uint32_t source_name = 1, query_id = 2;
""" + serving[0] + """
    return 0;
}
"""
    f = tmp_path / "example.cpp"
    f.write_text(src)
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I", os.path.join(ROOT, "include"), str(f)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_walks_that_cannot_end_are_rejected_without_gpu():
    """A stop probability below 2^-32 (0 included) gives a stop threshold of 0:
    without max_moves such a walk would never end on a graph whose vertices
    all have out-edges.  Every entry point rejects it before touching a
    graph or the device; with max_moves it passes that check (and then
    fails on the null graph).  Nothing is launched."""
    lib = _capi.load()
    tiny = 2.0 ** -33
    for sp, max_moves, ok in ((0.0, 0, False), (tiny, 0, False), (tiny, 3, True), (0.0, 3, True),
                              (-0.1, 5, False), (1.5, 0, False)):
        cfg = _capi.WalkCfg()
        cfg.n_walkers, cfg.sp, cfg.max_moves = 10, sp, max_moves
        for fn in (lambda: lib.ptw_pagerank(None, ctypes.byref(cfg), None, None),
                   lambda: lib.ptw_pagerank_dev(None, ctypes.byref(cfg), None, None),
                   lambda: lib.ptw_rwr(None, ctypes.byref(cfg), None, None),
                   lambda: lib.ptw_pagerank_noalloc(None, ctypes.byref(cfg), None, None)):
            assert fn() == _capi.PTW_EINVAL
            err = lib.ptw_last_error()
            assert (b"null" in err) == ok, (sp, max_moves, err)
        bc = _capi.BatchCfg()
        bc.sp, bc.max_moves = sp, max_moves
        assert lib.ptw_ppr_batch(None, None, 0, ctypes.byref(bc), None) == _capi.PTW_EINVAL
        assert (b"null" in lib.ptw_last_error()) == ok
        sc = _capi.ServeCfg()
        sc.sp, sc.max_moves = sp, max_moves
        assert lib.ptw_serve_open(None, ctypes.byref(sc), None) == _capi.PTW_EINVAL
        assert (b"null" in lib.ptw_last_error()) == ok
    assert lib.ptw_autotune(None, tiny, 0, None) == _capi.PTW_EINVAL


def test_cli_node2vec_flags_checked_before_any_gpu_work():
    """node2vec takes the reference's -p / -q (include/option.hpp:447-469):
    missing values are usage errors, found before the graph is loaded."""
    import subprocess
    from ptwalker_gb300 import _build
    exe = os.path.join(_build.BIN_DIR, "node2vec")
    for argv, msg in ((["-f", "text", "-g", "x.txt", "-w", "10", "-l", "5"], "-p and -q"),
                      (["-f", "text", "-g", "x.txt", "-w", "10", "-p", "2", "-q", "0.5"], "-l is required"),
                      (["-f", "text", "-g", "x.txt", "-w", "10", "-l", "5", "-p", "0", "-q", "1"], "-p and -q")):
        r = subprocess.run([exe] + argv, capture_output=True, text=True)
        assert r.returncode == 1 and msg in r.stderr, r.stderr


def test_cli_batch_flags_checked_before_any_gpu_work(tmp_path):
    """ppr --sources / --budget / --model / --tune usage errors are found
    before the graph is loaded."""
    import subprocess
    from ptwalker_gb300 import _build
    exe = os.path.join(_build.BIN_DIR, "ppr")
    base = ["-f", "text", "-g", "x.txt", "-w", "10", "--sp", "0.2"]
    for argv, msg in ((base, "--source or --sources"),
                      (base + ["--sources", "1,2", "--budget", "magic"], "--budget must be"),
                      (base + ["--sources", "1,2", "--budget", "learned"], "--model"),
                      (base + ["--sources", ",,"], "no valid vertex names")):
        r = subprocess.run([exe] + argv, capture_output=True, text=True)
        assert r.returncode == 1 and msg in r.stderr, r.stderr
    r = subprocess.run([os.path.join(_build.BIN_DIR, "pagerank"), "-f", "text", "-g", "x.txt", "-w", "10",
                        "--sp", "0.2", "--sources", "1"], capture_output=True, text=True)
    assert r.returncode == 1 and "--sources is for ppr" in r.stderr
