// C ABI of libptw: argument checking, host<->device staging and the
// edge-list loader.  See include/ptw.h for the reference interface each entry
// point replaces.
#include <cuda_runtime.h>
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <mutex>
#include <vector>

#include "ptw_internal.cuh"

namespace ptw {

static thread_local std::string g_last_error;

int fail(int code, const std::string &msg)
{
    g_last_error = msg;
    return code;
}

int host_exception()
{
    try {
        throw;
    } catch (const std::bad_alloc &) {
        return fail(PTW_ENOMEM, "host allocation failed");
    } catch (const std::exception &e) {
        return fail(PTW_EINVAL, std::string("host error: ") + e.what());
    } catch (...) {
        return fail(PTW_EINVAL, "unknown host error");
    }
}

int check_stop(double sp, uint32_t max_moves)
{
    if (!(sp >= 0.0 && sp <= 1.0)) return fail(PTW_EINVAL, "sp must be in [0, 1]");
    if (stop_threshold(sp) == 0 && max_moves == 0)
        return fail(PTW_EINVAL, "sp below 2^-32 (sp = 0 included) needs max_moves > 0: walks would never end");
    return PTW_OK;
}

int cuda_fail(cudaError_t e, const char *what)
{
    const int code = (e == cudaErrorMemoryAllocation) ? PTW_ENOMEM : PTW_ECUDA;
    cudaGetLastError();  // clear a sticky-free error so later calls can run
    return fail(code, std::string(what) + ": " + cudaGetErrorString(e));
}

namespace {
std::mutex g_pool_mu;
cudaMemPool_t g_pools[64] = {};
}  // namespace

cudaError_t pooled_alloc_async(void **p, size_t bytes, cudaStream_t st)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaMallocAsync(p, bytes, st);
    cudaMemPool_t pool;
    {
        std::lock_guard<std::mutex> lk(g_pool_mu);
        if (!g_pools[dev]) {
            cudaMemPoolProps props{};
            props.allocType = cudaMemAllocationTypePinned;
            props.location.type = cudaMemLocationTypeDevice;
            props.location.id = dev;
            size_t free_b = 0, total_b = 0;
            e = cudaMemGetInfo(&free_b, &total_b);
            if (e != cudaSuccess) return e;
            cudaMemPool_t np = nullptr;
            e = cudaMemPoolCreate(&np, &props);
            if (e != cudaSuccess) return e;
            // Memory freed to the pool stays mapped up to this much across
            // synchronisations: a batch of thousands of queries allocates and
            // frees tens of GB of count tables per call, and handing them back
            // to the CUDA driver at every synchronisation costs about 1.5 ms per GB
            // to unmap and as much again to map on the next call.
            uint64_t keep = std::max<uint64_t>(1ull << 30, (uint64_t)total_b / 4);
            e = cudaMemPoolSetAttribute(np, cudaMemPoolAttrReleaseThreshold, &keep);
            if (e != cudaSuccess) {
                cudaMemPoolDestroy(np);
                return e;
            }
            g_pools[dev] = np;
        }
        pool = g_pools[dev];
    }
    return cudaMallocFromPoolAsync(p, bytes, pool, st);
}

void trim_pools()
{
    std::lock_guard<std::mutex> lk(g_pool_mu);
    for (cudaMemPool_t p : g_pools)
        if (p) cudaMemPoolTrimTo(p, 0);
}

cudaError_t device_malloc_bytes(void **p, size_t bytes)
{
    cudaError_t e = cudaMalloc(p, bytes);
    if (e == cudaErrorMemoryAllocation) {
        // the pool may hold freed memory: wait for pending frees, hand it back, retry once
        cudaGetLastError();
        cudaDeviceSynchronize();
        trim_pools();
        e = cudaMalloc(p, bytes);
    }
    return e;
}

namespace {

// ---- edge-list parsing (include/io.hpp:39-90) -------------------------------

struct ParseChunk {
    std::vector<uint32_t> src, dst;
    uint64_t bad_line = 0;  // 1-based line number inside the chunk, 0 = ok
    uint64_t lines = 0;
};

inline bool is_space(char c) { return c == ' ' || c == '\t' || c == '\r'; }

// Parses [b, e) that starts at a line start.  Comment lines start with '#'.
// Blank lines are skipped; any other line must start with two unsigned
// decimal integers that fit in 32 bits.
void parse_range(const char *b, const char *e, ParseChunk *out)
{
    const char *p = b;
    while (p < e) {
        ++out->lines;
        const char *le = (const char *)memchr(p, '\n', (size_t)(e - p));
        if (!le) le = e;
        const char *q = p;
        while (q < le && is_space(*q)) ++q;
        if (q < le && *p != '#') {
            uint64_t v[2];
            bool ok = true;
            for (int k = 0; k < 2 && ok; ++k) {
                while (q < le && is_space(*q)) ++q;
                if (q >= le || *q < '0' || *q > '9') { ok = false; break; }
                uint64_t x = 0;
                while (q < le && *q >= '0' && *q <= '9') {
                    x = x * 10 + (uint64_t)(*q - '0');
                    if (x > 0xFFFFFFFFull) { ok = false; break; }
                    ++q;
                }
                v[k] = x;
            }
            if (!ok) {
                if (!out->bad_line) out->bad_line = out->lines;
                return;
            }
            out->src.push_back((uint32_t)v[0]);
            out->dst.push_back((uint32_t)v[1]);
        }
        p = le + 1;
    }
}

int read_edges(const char *path, int fmt, std::vector<uint32_t> &src, std::vector<uint32_t> &dst)
{
    const int fd = open(path, O_RDONLY);
    if (fd < 0) return fail(PTW_EIO, std::string("cannot open ") + path);
    struct stat stt;
    if (fstat(fd, &stt) != 0) {
        close(fd);
        return fail(PTW_EIO, std::string("cannot stat ") + path);
    }
    const size_t size = (size_t)stt.st_size;
    if (size == 0) {
        close(fd);
        return fail(PTW_EIO, std::string("empty edge file ") + path);
    }
    void *map = mmap(nullptr, size, PROT_READ, MAP_PRIVATE, fd, 0);
    close(fd);
    if (map == MAP_FAILED) return fail(PTW_EIO, std::string("cannot map ") + path);
    const char *data = (const char *)map;
    int rc = PTW_OK;
    if (fmt == PTW_FMT_BINARY) {
        if (size % 8 != 0) {
            rc = fail(PTW_EIO, "binary edge file size is not a multiple of 8 bytes");
        } else {
            const uint64_t m = size / 8;
            src.resize(m);
            dst.resize(m);
            const uint32_t *w = (const uint32_t *)data;
            for (uint64_t i = 0; i < m; ++i) {
                src[i] = w[2 * i];
                dst[i] = w[2 * i + 1];
            }
        }
    } else {
        unsigned nt = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
        if (size < (1u << 20)) nt = 1;
        std::vector<size_t> cut(nt + 1, size);
        cut[0] = 0;
        for (unsigned t = 1; t < nt; ++t) {
            size_t c = size * t / nt;
            while (c < size && data[c - 1] != '\n') ++c;
            cut[t] = std::max(c, cut[t - 1]);
        }
        std::vector<ParseChunk> parts(nt);
        try {
            parallel_for_threads(nt, [&](unsigned t) { parse_range(data + cut[t], data + cut[t + 1], &parts[t]); });
        } catch (...) {
            munmap(map, size);
            throw;
        }
        uint64_t line0 = 0, total = 0;
        for (unsigned t = 0; t < nt && rc == PTW_OK; ++t) {
            if (parts[t].bad_line) {
                rc = fail(PTW_EIO, std::string("malformed edge at line ") +
                                       std::to_string(line0 + parts[t].bad_line) + " of " + path);
            }
            line0 += parts[t].lines;
            total += parts[t].src.size();
        }
        if (rc == PTW_OK) {
            src.reserve(total);
            dst.reserve(total);
            for (auto &pc : parts) {
                src.insert(src.end(), pc.src.begin(), pc.src.end());
                dst.insert(dst.end(), pc.dst.begin(), pc.dst.end());
            }
        }
    }
    munmap(map, size);
    return rc;
}

int upload_and_build(const uint32_t *h_src, const uint32_t *h_dst, uint64_t m, bool undirected,
                     ptw_graph **out)
{
    if (!out) return fail(PTW_EINVAL, "null output handle");
    *out = nullptr;
    if (m == 0) return fail(PTW_EINVAL, "edge list is empty");
    if (!h_src || !h_dst) return fail(PTW_EINVAL, "null edge arrays");
    ptw_graph *g = new (std::nothrow) ptw_graph();
    if (!g) return fail(PTW_ENOMEM, "host allocation failed");
    int rc = graph_init_handle(g);
    uint32_t *d_src = nullptr, *d_dst = nullptr;
    if (rc == PTW_OK) {
        cudaError_t e = cudaMallocAsync(&d_src, m * 4, g->stream);
        if (e == cudaSuccess) e = cudaMallocAsync(&d_dst, m * 4, g->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(d_src, h_src, m * 4, cudaMemcpyHostToDevice, g->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(d_dst, h_dst, m * 4, cudaMemcpyHostToDevice, g->stream);
        if (e != cudaSuccess) {
            rc = cuda_fail(e, "edge upload");
            if (d_src) cudaFreeAsync(d_src, g->stream);
            if (d_dst) cudaFreeAsync(d_dst, g->stream);
        } else {
            rc = build_graph_from_device_edges(g, d_src, d_dst, m, undirected, false, false);
        }
    }
    if (rc != PTW_OK) {
        graph_release(g);
        delete g;
        return rc;
    }
    *out = g;
    return PTW_OK;
}

int check_cfg(const ptw_graph *g, const ptw_walk_cfg *cfg, bool needs_sp)
{
    if (!cfg) return fail(PTW_EINVAL, "null walk configuration");
    if (needs_sp) {  // checked before the graph, so it needs no device
        const int rc = check_stop(cfg->sp, cfg->max_moves);
        if (rc) return rc;
    }
    if (!g) return fail(PTW_EINVAL, "null graph");
    if (cfg->start_mode < PTW_START_PER_VERTEX || cfg->start_mode > PTW_START_SOURCES)
        return fail(PTW_EINVAL, "unknown start_mode");
    if (cfg->start_mode == PTW_START_SOURCES && (cfg->n_sources == 0 || !cfg->h_sources))
        return fail(PTW_EINVAL, "PTW_START_SOURCES needs at least one source");
    if (cfg->n_walkers > ~0ull - cfg->first_walker) return fail(PTW_EINVAL, "walker ids overflow 64 bits");
    return PTW_OK;
}

// Maps source names to internal ids and uploads them to the scratch table.
int upload_sources(ptw_graph *g, const ptw_walk_cfg *cfg)
{
    if (cfg->start_mode != PTW_START_SOURCES) return PTW_OK;
    const uint32_t n = g->dg.n;
    std::vector<uint32_t> ids(cfg->n_sources);
    for (uint32_t i = 0; i < cfg->n_sources; ++i) {
        const uint32_t nm = cfg->h_sources[i];
        const uint32_t *p = std::lower_bound(g->h_names, g->h_names + n, nm);
        if (p == g->h_names + n || *p != nm)
            return fail(PTW_EINVAL, "source " + std::to_string(nm) + " is not a vertex of the graph");
        ids[i] = g->h_idx2int[p - g->h_names];
    }
    if (g->sc.sources_cap < cfg->n_sources) {
        cudaFree(g->sc.sources);
        g->sc.sources = nullptr;
        g->sc.sources_cap = 0;
        PTW_CUDA(device_malloc(&g->sc.sources, (uint64_t)cfg->n_sources * 4));
        g->sc.sources_cap = cfg->n_sources;
    }
    PTW_CUDA(cudaMemcpyAsync(g->sc.sources, ids.data(), (uint64_t)cfg->n_sources * 4,
                             cudaMemcpyHostToDevice, g->stream));
    // ids must outlive the copy
    PTW_CUDA(cudaStreamSynchronize(g->stream));
    return PTW_OK;
}

int stage_bytes(ptw_graph *g, size_t bytes, void **out)
{
    if (g->sc.out_stage_bytes < bytes) {
        cudaFree(g->sc.out_stage);
        g->sc.out_stage = nullptr;
        g->sc.out_stage_bytes = 0;
        PTW_CUDA(device_malloc(&g->sc.out_stage, std::max<size_t>(bytes, 256)));
        g->sc.out_stage_bytes = std::max<size_t>(bytes, 256);
    }
    *out = g->sc.out_stage;
    return PTW_OK;
}

WalkLaunch make_launch(const ptw_walk_cfg *cfg)
{
    WalkLaunch wl;
    wl.w_begin = cfg->first_walker;
    wl.w_end = wl.w_begin + cfg->n_walkers;
    wl.thr = stop_threshold(cfg->sp);
    wl.seed = cfg->seed;
    wl.start_mode = cfg->start_mode;
    wl.n_sources = cfg->start_mode == PTW_START_SOURCES ? cfg->n_sources : 0;
    wl.max_moves = cfg->max_moves;
    return wl;
}

int finish_stats(ptw_graph *g, ptw_walk_stats *stats, uint64_t walkers, bool count_app)
{
    if (!stats) return PTW_OK;
    unsigned long long moves = 0;
    PTW_CUDA(cudaMemcpyAsync(&moves, g->sc.ctrl + 1, sizeof(moves), cudaMemcpyDeviceToHost, g->stream));
    PTW_CUDA(cudaStreamSynchronize(g->stream));
    stats->walkers = walkers;
    stats->moves = moves;
    stats->visits = count_app ? walkers + moves : 0;
    float ms = 0;
    PTW_CUDA(cudaEventElapsedTime(&ms, g->ev[0], g->ev[1]));
    stats->kernel_ms = ms;
    PTW_CUDA(cudaEventElapsedTime(&ms, g->ev[3], g->ev[2]));
    stats->total_ms = ms;
    return PTW_OK;
}

// Runs the count walk into g->sc.counts and scatters the result by name
// into d_by_name.  Events: ev0 before, ev1 after the kernel.
int run_count(ptw_graph *g, const ptw_walk_cfg *cfg, uint32_t *d_by_name)
{
    int rc = upload_sources(g, cfg);
    if (rc) return rc;
    // on extended columns the walk counts by name into d_by_name itself;
    // otherwise by internal id into the scratch, scattered by name after
    const bool by_name = cfg->n_walkers && count_walk_by_name(g, g->tune);
    PTW_CUDA(cudaEventRecord(g->ev[3], g->stream));
    if (by_name) PTW_CUDA(cudaMemsetAsync(d_by_name, 0, (uint64_t)g->dg.id_bound * 4, g->stream));
    else PTW_CUDA(cudaMemsetAsync(g->sc.counts, 0, (uint64_t)g->dg.n * 4, g->stream));
    PTW_CUDA(cudaEventRecord(g->ev[0], g->stream));
    if (cfg->n_walkers) {
        WalkLaunch wl = make_launch(cfg);
        if (by_name) wl.by_name = d_by_name;
        rc = launch_walk(g, wl, g->tune);
        if (rc) return rc;
    } else {
        PTW_CUDA(cudaMemsetAsync(g->sc.ctrl, 0, 2 * sizeof(unsigned long long), g->stream));
    }
    PTW_CUDA(cudaEventRecord(g->ev[1], g->stream));
    return by_name ? PTW_OK : launch_counts_by_name(g, d_by_name);
}

int run_endpoint(ptw_graph *g, const ptw_walk_cfg *cfg, uint32_t *d_pairs)
{
    int rc = upload_sources(g, cfg);
    if (rc) return rc;
    PTW_CUDA(cudaEventRecord(g->ev[3], g->stream));
    PTW_CUDA(cudaEventRecord(g->ev[0], g->stream));
    if (cfg->n_walkers) {
        WalkLaunch wl = make_launch(cfg);
        wl.endpoint = true;
        wl.pairs = d_pairs;
        rc = launch_walk(g, wl, g->tune);
        if (rc) return rc;
    } else {
        PTW_CUDA(cudaMemsetAsync(g->sc.ctrl, 0, 2 * sizeof(unsigned long long), g->stream));
    }
    PTW_CUDA(cudaEventRecord(g->ev[1], g->stream));
    return PTW_OK;
}

int run_paths(ptw_graph *g, const ptw_walk_cfg *cfg, uint32_t L, int32_t *d_paths)
{
    int rc = upload_sources(g, cfg);
    if (rc) return rc;
    PTW_CUDA(cudaEventRecord(g->ev[3], g->stream));
    PTW_CUDA(cudaMemsetAsync(g->sc.ctrl, 0, 2 * sizeof(unsigned long long), g->stream));
    PTW_CUDA(cudaEventRecord(g->ev[0], g->stream));
    if (cfg->n_walkers && L) {
        const uint64_t w0 = cfg->first_walker;
        rc = launch_paths(g, w0, w0 + cfg->n_walkers, L, cfg->seed, cfg->start_mode,
                          cfg->start_mode == PTW_START_SOURCES ? cfg->n_sources : 0, d_paths);
        if (rc) return rc;
    }
    PTW_CUDA(cudaEventRecord(g->ev[1], g->stream));
    return PTW_OK;
}

// Path walks delivered to host memory: the walkers run in chunks (at most 8,
// at least 2^20 walkers each) into the device staging, every chunk's paths
// copied to h_paths on the copy stream while the next chunks walk.  All
// chunk launches are issued before the copies, so a copy into pageable
// memory (which holds the calling thread) does not hold back the walks.
// Draws depend on walker ids only, so the paths equal one launch's.
// launch_chunk(w_begin, w_end, d_paths) issues one chunk on the graph's
// stream.  Events: ev0 before the first chunk, ev1 after the last, ev2
// after the last copy (on the graph's stream).
template <class F>
int paths_to_host(ptw_graph *g, const ptw_walk_cfg *cfg, uint32_t L, int32_t *h_paths, int32_t *stage,
                  F launch_chunk)
{
    const uint64_t W = cfg->n_walkers, w0 = cfg->first_walker;
    PTW_CUDA(cudaEventRecord(g->ev[0], g->stream));
    if (W == 0 || L == 0) {
        PTW_CUDA(cudaEventRecord(g->ev[1], g->stream));
        PTW_CUDA(cudaEventRecord(g->ev[2], g->stream));
        return PTW_OK;
    }
    if (!g->copy_stream) PTW_CUDA(cudaStreamCreateWithFlags(&g->copy_stream, cudaStreamNonBlocking));
    const uint64_t per = std::max<uint64_t>(1ull << 20, (W + 7) / 8);
    const uint64_t nc = (W + per - 1) / per;
    std::vector<cudaEvent_t> ev(nc, nullptr);
    struct Events {
        std::vector<cudaEvent_t> &e;
        ~Events()
        {
            for (cudaEvent_t x : e)
                if (x) cudaEventDestroy(x);
        }
    } guard{ev};
    for (uint64_t c = 0; c < nc; ++c) {
        PTW_CUDA(cudaEventCreateWithFlags(&ev[c], cudaEventDisableTiming));
        const uint64_t off = c * per, n = std::min(per, W - off);
        const int rc = launch_chunk(w0 + off, w0 + off + n, stage + off * L);
        if (rc) return rc;
        PTW_CUDA(cudaEventRecord(ev[c], g->stream));
    }
    PTW_CUDA(cudaEventRecord(g->ev[1], g->stream));
    for (uint64_t c = 0; c < nc; ++c) {
        const uint64_t off = c * per, n = std::min(per, W - off);
        PTW_CUDA(cudaStreamWaitEvent(g->copy_stream, ev[c], 0));
        PTW_CUDA(cudaMemcpyAsync(h_paths + off * L, stage + off * L, n * (uint64_t)L * 4, cudaMemcpyDeviceToHost,
                                 g->copy_stream));
    }
    PTW_CUDA(cudaEventRecord(ev[nc - 1], g->copy_stream));
    PTW_CUDA(cudaStreamWaitEvent(g->stream, ev[nc - 1], 0));
    PTW_CUDA(cudaEventRecord(g->ev[2], g->stream));
    PTW_CUDA(cudaStreamSynchronize(g->stream));
    return PTW_OK;
}

// Acceptance thresholds of the node2vec rejection draw: class weights
// {1/p (return), 1 (neighbour of the previous vertex), 1/q (other)} over
// their maximum M, as 32-bit fractions (2^32 = always accept).
int n2v_thresholds(double p, double q, uint64_t thr[3])
{
    if (!(p > 0.0 && q > 0.0 && p < 1e300 && q < 1e300))
        return fail(PTW_EINVAL, "node2vec p and q must be positive and finite");
    const double w[3] = {1.0 / p, 1.0, 1.0 / q};
    const double m = std::max(w[0], std::max(w[1], w[2]));
    const double lo = std::min(w[0], std::min(w[1], w[2]));
    if (m > 1024.0 * lo)
        return fail(PTW_EINVAL, "node2vec needs max(1/p, 1, 1/q) <= 1024 * min(1/p, 1, 1/q)");
    for (int c = 0; c < 3; ++c) thr[c] = w[c] >= m ? 1ull << 32 : (uint64_t)(w[c] / m * 4294967296.0);
    return PTW_OK;
}

int run_node2vec(ptw_graph *g, const ptw_walk_cfg *cfg, uint32_t L, double p, double q, const uint64_t thr[3],
                 int32_t *d_paths)
{
    int rc = upload_sources(g, cfg);
    if (rc) return rc;
    PTW_CUDA(cudaEventRecord(g->ev[3], g->stream));
    PTW_CUDA(cudaMemsetAsync(g->sc.ctrl, 0, 5 * sizeof(unsigned long long), g->stream));
    if (cfg->n_walkers && L && !(ensure_ext_columns(g) && ensure_edge_filter(g)))
        return fail(PTW_ENOMEM, "node2vec needs the extended column copy (16 bytes per CSR entry) and "
                                "the edge filter (2 bytes per CSR entry), which do not fit in device memory");
    PTW_CUDA(cudaEventRecord(g->ev[0], g->stream));
    if (cfg->n_walkers && L) {
        const uint64_t w0 = cfg->first_walker;
        rc = launch_node2vec(g, w0, w0 + cfg->n_walkers, L, cfg->seed, cfg->start_mode,
                             cfg->start_mode == PTW_START_SOURCES ? cfg->n_sources : 0, p, q, thr, d_paths);
        if (rc) return rc;
    }
    PTW_CUDA(cudaEventRecord(g->ev[1], g->stream));
    return PTW_OK;
}

int node2vec_stats(ptw_graph *g, const ptw_walk_cfg *cfg, ptw_node2vec_stats *stats)
{
    unsigned long long c[4];
    PTW_CUDA(cudaMemcpyAsync(c, g->sc.ctrl + 1, sizeof(c), cudaMemcpyDeviceToHost, g->stream));
    PTW_CUDA(cudaStreamSynchronize(g->stream));
    stats->walkers = cfg->n_walkers;
    stats->moves = c[0];
    stats->trials = c[1];
    stats->checks = c[2];
    stats->probes = c[3];
    float ms = 0;
    PTW_CUDA(cudaEventElapsedTime(&ms, g->ev[0], g->ev[1]));
    stats->kernel_ms = ms;
    PTW_CUDA(cudaEventElapsedTime(&ms, g->ev[3], g->ev[2]));
    stats->total_ms = ms;
    return PTW_OK;
}

}  // namespace
}  // namespace ptw

namespace ptw {
int check_word_status(ptw_graph *g)
{
#ifdef PTW_CHECKED
    unsigned long long w = 0;
    PTW_CUDA(cudaMemcpyAsync(&w, g->sc.ctrl + 7, sizeof(w), cudaMemcpyDeviceToHost, g->stream));
    PTW_CUDA(cudaStreamSynchronize(g->stream));
    if (w) {
        PTW_CUDA(cudaMemsetAsync(g->sc.ctrl + 7, 0, sizeof(w), g->stream));
        PTW_CUDA(cudaStreamSynchronize(g->stream));
        char msg[96];
        std::snprintf(msg, sizeof msg, "index check failed: site mask 0x%llx", w);
        return fail(PTW_ECUDA, msg);
    }
#else
    (void)g;
#endif
    return PTW_OK;
}
}  // namespace ptw

using namespace ptw;

extern "C" const char *ptw_last_error(void) { return g_last_error.c_str(); }

extern "C" int ptw_trim_memory(void)
try {
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return cuda_fail(e, "synchronise before trimming");
    trim_pools();
    return PTW_OK;
} catch (...) {
    return host_exception();
}

extern "C" const char *ptw_version(void) { return "ptwalker_gb300 0.1 (sm_103a)"; }

extern "C" int ptw_graph_load(const char *path, int32_t fmt, int32_t as_undirected, ptw_graph **out)
try {
    NvtxRange nvtx("ptw_graph_load");
    if (!path || !out) return fail(PTW_EINVAL, "null argument");
    if (fmt != PTW_FMT_BINARY && fmt != PTW_FMT_TEXT) return fail(PTW_EINVAL, "unknown graph format");
    std::vector<uint32_t> src, dst;
    int rc = read_edges(path, fmt, src, dst);
    if (rc) return rc;
    return upload_and_build(src.data(), dst.data(), src.size(), as_undirected != 0, out);
} catch (...) {
    return host_exception();
}

namespace ptw {
namespace {

// Decimal digits of x at p; returns the end.
inline char *put_u32(char *p, uint32_t x)
{
    char tmp[10];
    int k = 0;
    do {
        tmp[k++] = (char)('0' + x % 10);
        x /= 10;
    } while (x);
    while (k) *p++ = tmp[--k];
    return p;
}

}  // namespace
}  // namespace ptw

extern "C" int ptw_graph_save(const ptw_graph *g, const char *path, int32_t fmt)
try {
    NvtxRange nvtx("ptw_graph_save");
    if (!g || !path) return fail(PTW_EINVAL, "null argument");
    if (fmt != PTW_FMT_BINARY && fmt != PTW_FMT_TEXT) return fail(PTW_EINVAL, "unknown graph format");
    const uint64_t m = g->dg.m;
    std::vector<uint32_t> src(m), dst(m);
    int rc = ptw_graph_export_edges(g, src.data(), dst.data());
    if (rc) return rc;
    FILE *f = std::fopen(path, "wb");
    if (!f) return fail(PTW_EIO, std::string("cannot create ") + path);
    // Rounds of nt chunks: formatted in parallel, written in order.
    const unsigned nt = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    const uint64_t chunk = 1u << 22;
    std::vector<std::string> buf(nt);
    bool ok = true;
    for (uint64_t r0 = 0; r0 < m && ok; r0 += chunk * nt) {
        try {
            parallel_for_threads(nt, [&](unsigned t) {
                const uint64_t lo = std::min(m, r0 + t * chunk), hi = std::min(m, lo + chunk);
                std::string &b = buf[t];
                if (fmt == PTW_FMT_BINARY) {
                    b.resize((hi - lo) * 8);
                    uint32_t *w = reinterpret_cast<uint32_t *>(&b[0]);
                    for (uint64_t e = lo; e < hi; ++e) {
                        w[2 * (e - lo)] = src[e];
                        w[2 * (e - lo) + 1] = dst[e];
                    }
                } else {
                    b.resize((hi - lo) * 22);  // two 10-digit numbers, a space, a newline
                    char *p = &b[0];
                    for (uint64_t e = lo; e < hi; ++e) {
                        p = put_u32(p, src[e]);
                        *p++ = ' ';
                        p = put_u32(p, dst[e]);
                        *p++ = '\n';
                    }
                    b.resize(p - &b[0]);
                }
            });
        } catch (...) {
            std::fclose(f);
            throw;
        }
        for (unsigned t = 0; t < nt && ok; ++t)
            if (!buf[t].empty() && std::fwrite(buf[t].data(), 1, buf[t].size(), f) != buf[t].size()) ok = false;
    }
    if (std::fclose(f) != 0) ok = false;
    if (!ok) return fail(PTW_EIO, std::string("write failed: ") + path);
    return PTW_OK;
} catch (...) {
    return host_exception();
}

extern "C" int ptw_graph_from_edges(const uint32_t *h_src, const uint32_t *h_dst, uint64_t m,
                                    int32_t as_undirected, ptw_graph **out)
try {
    NvtxRange nvtx("ptw_graph_from_edges");
    return upload_and_build(h_src, h_dst, m, as_undirected != 0, out);
} catch (...) {
    return host_exception();
}

extern "C" int ptw_graph_from_csr(const uint64_t *h_row_ptr, const uint32_t *h_col, uint32_t n,
                                  const uint32_t *h_names, ptw_graph **out)
try {
    NvtxRange nvtx("ptw_graph_from_csr");
    if (!out) return fail(PTW_EINVAL, "null output handle");
    *out = nullptr;
    if (!h_row_ptr || n == 0) return fail(PTW_EINVAL, "CSR needs n >= 1 rows and a row_ptr array");
    if (h_row_ptr[0] != 0) return fail(PTW_EINVAL, "CSR row_ptr[0] must be 0");
    for (uint32_t i = 0; i < n; ++i)
        if (h_row_ptr[i + 1] < h_row_ptr[i])
            return fail(PTW_EINVAL, "CSR row_ptr decreases at row " + std::to_string(i));
    const uint64_t m = h_row_ptr[n];
    if (m == 0) return fail(PTW_EINVAL, "edge list is empty");
    if (!h_col) return fail(PTW_EINVAL, "null CSR column array");
    if (m >= (1ull << 32)) return fail(PTW_EINVAL, "graphs with 2^32 or more CSR entries are not supported");
    ptw_graph *g = new (std::nothrow) ptw_graph();
    if (!g) return fail(PTW_ENOMEM, "host allocation failed");
    int rc = graph_init_handle(g);
    uint32_t *d_src = nullptr, *d_dst = nullptr;
    if (rc == PTW_OK) rc = csr_to_device_edges(h_row_ptr, h_col, h_names, n, &d_src, &d_dst, g->stream);
    if (rc == PTW_OK) rc = build_graph_from_device_edges(g, d_src, d_dst, m, false, false, false);
    if (rc != PTW_OK) {
        graph_release(g);
        delete g;
        return rc;
    }
    *out = g;
    return PTW_OK;
} catch (...) {
    return host_exception();
}

extern "C" int ptw_graph_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c,
                              uint64_t seed, int32_t clean, ptw_graph **out)
try {
    NvtxRange nvtx("ptw_graph_rmat");
    if (!out) return fail(PTW_EINVAL, "null output handle");
    *out = nullptr;
    if (scale < 1 || scale > 31) return fail(PTW_EINVAL, "scale must be in [1, 31]");
    if (edge_factor < 1) return fail(PTW_EINVAL, "edge_factor must be >= 1");
    if (!(a >= 0 && b >= 0 && c >= 0 && a + b + c <= 1.0))
        return fail(PTW_EINVAL, "R-MAT probabilities must be >= 0 with a + b + c <= 1");
    const uint64_t m = (uint64_t)edge_factor << scale;
    if (m >= (1ull << 32)) return fail(PTW_EINVAL, "2^scale * edge_factor must be < 2^32");
    auto thr = [](double p) -> uint32_t {
        const double x = p * 4294967296.0;
        return x >= 4294967295.0 ? 0xFFFFFFFFu : (uint32_t)x;
    };
    ptw_graph *g = new (std::nothrow) ptw_graph();
    if (!g) return fail(PTW_ENOMEM, "host allocation failed");
    int rc = graph_init_handle(g);
    uint32_t *d_src = nullptr, *d_dst = nullptr;
    if (rc == PTW_OK) {
        cudaError_t e = cudaMallocAsync(&d_src, m * 4, g->stream);
        if (e == cudaSuccess) e = cudaMallocAsync(&d_dst, m * 4, g->stream);
        if (e != cudaSuccess) {
            rc = cuda_fail(e, "R-MAT edge buffers");
            if (d_src) cudaFreeAsync(d_src, g->stream);
        } else {
            rc = rmat_generate_device(scale, m, thr(a), thr(a + b), thr(a + b + c), seed, d_src, d_dst,
                                      g->stream);
            if (rc == PTW_OK)
                rc = build_graph_from_device_edges(g, d_src, d_dst, m, clean != 0, clean != 0, clean != 0);
        }
    }
    if (rc != PTW_OK) {
        graph_release(g);
        delete g;
        return rc;
    }
    *out = g;
    return PTW_OK;
} catch (...) {
    return host_exception();
}

extern "C" int ptw_graph_chung_lu(uint32_t n, double gamma, double mean_degree, uint64_t seed, ptw_graph **out)
try {
    NvtxRange nvtx("ptw_graph_chung_lu");
    if (!out) return fail(PTW_EINVAL, "null output handle");
    *out = nullptr;
    if (n < 2) return fail(PTW_EINVAL, "n must be >= 2");
    if (!(gamma > 1.0)) return fail(PTW_EINVAL, "gamma must be > 1");
    if (!(mean_degree > 0.0)) return fail(PTW_EINVAL, "mean_degree must be > 0");
    const double md = std::ceil((double)n * mean_degree / 2.0);
    if (md >= 2147483648.0) return fail(PTW_EINVAL, "n * mean_degree / 2 must be < 2^31");
    const uint64_t m = (uint64_t)md;
    ptw_graph *g = new (std::nothrow) ptw_graph();
    if (!g) return fail(PTW_ENOMEM, "host allocation failed");
    int rc = graph_init_handle(g);
    uint32_t *d_src = nullptr, *d_dst = nullptr;
    if (rc == PTW_OK) {
        cudaError_t e = cudaMallocAsync(&d_src, m * 4, g->stream);
        if (e == cudaSuccess) e = cudaMallocAsync(&d_dst, m * 4, g->stream);
        if (e != cudaSuccess) {
            rc = cuda_fail(e, "Chung-Lu edge buffers");
            if (d_src) cudaFreeAsync(d_src, g->stream);
        } else {
            rc = chung_lu_generate_device(n, gamma, m, seed, d_src, d_dst, g->stream);
            if (rc == PTW_OK) rc = build_graph_from_device_edges(g, d_src, d_dst, m, true, true, true);
        }
    }
    if (rc != PTW_OK) {
        graph_release(g);
        delete g;
        return rc;
    }
    *out = g;
    return PTW_OK;
} catch (...) {
    return host_exception();
}

extern "C" void ptw_graph_free(ptw_graph *g)
try {
    if (!g) return;
    cudaSetDevice(g->device);
    graph_release(g);
    delete g;
} catch (...) {
    host_exception();
}

extern "C" int ptw_graph_set_tune(ptw_graph *g, const ptw_tune *t)
try {
    if (!g || !t) return fail(PTW_EINVAL, "null argument");
    int rc = check_tune(*t);
    if (rc) return rc;
    g->tune = *t;
    drop_unused_columns(g);
    return PTW_OK;
} catch (...) {
    return host_exception();
}

extern "C" int ptw_graph_get_tune(const ptw_graph *g, ptw_tune *t)
try {
    if (!g || !t) return fail(PTW_EINVAL, "null argument");
    *t = g->tune;
    return PTW_OK;
} catch (...) {
    return host_exception();
}

extern "C" int ptw_pagerank_dev(ptw_graph *g, const ptw_walk_cfg *cfg, uint32_t *d_counts,
                                ptw_walk_stats *stats)
try {
    NvtxRange nvtx("ptw_pagerank_dev");
    int rc = check_cfg(g, cfg, true);
    if (rc) return rc;
    if (!d_counts) return fail(PTW_EINVAL, "null counts buffer");
    PTW_CUDA(cudaSetDevice(g->device));
    rc = run_count(g, cfg, d_counts);
    if (rc) return rc;
    PTW_CUDA(cudaEventRecord(g->ev[2], g->stream));
    if ((rc = check_word_status(g))) return rc;
    return finish_stats(g, stats, cfg->n_walkers, true);
} catch (...) {
    return host_exception();
}

extern "C" int ptw_pagerank(ptw_graph *g, const ptw_walk_cfg *cfg, uint32_t *h_counts,
                            ptw_walk_stats *stats)
try {
    NvtxRange nvtx("ptw_pagerank");
    int rc = check_cfg(g, cfg, true);
    if (rc) return rc;
    if (!h_counts) return fail(PTW_EINVAL, "null counts buffer");
    PTW_CUDA(cudaSetDevice(g->device));
    if (!g->sc.by_name) PTW_CUDA(device_malloc(&g->sc.by_name, (uint64_t)g->dg.id_bound * 4));
    rc = run_count(g, cfg, g->sc.by_name);
    if (rc) return rc;
    PTW_CUDA(cudaMemcpyAsync(h_counts, g->sc.by_name, (uint64_t)g->dg.id_bound * 4,
                             cudaMemcpyDeviceToHost, g->stream));
    PTW_CUDA(cudaEventRecord(g->ev[2], g->stream));
    PTW_CUDA(cudaStreamSynchronize(g->stream));
    if ((rc = check_word_status(g))) return rc;
    return finish_stats(g, stats, cfg->n_walkers, true);
} catch (...) {
    return host_exception();
}

// Pipelined count walk: the walk of one call overlaps the copy of the
// previous call's counts (copies run on a second stream).  Two calls may be
// in flight; each has its own device by-name buffer.
extern "C" int ptw_pagerank_submit(ptw_graph *g, const ptw_walk_cfg *cfg, uint32_t *h_counts, uint64_t *ticket)
try {
    NvtxRange nvtx("ptw_pagerank_submit");
    int rc = check_cfg(g, cfg, true);
    if (rc) return rc;
    if (!h_counts || !ticket) return fail(PTW_EINVAL, "null counts buffer or ticket");
    PTW_CUDA(cudaSetDevice(g->device));
    AsyncSlot *a = nullptr;
    for (AsyncSlot &x : g->async)
        if (x.ticket == 0 && (!a || x.by_name)) a = &x;  // prefer a slot already set up
    if (!a) return fail(PTW_EBUSY, "two pipelined walks in flight: wait for one first");
    if (!a->by_name) {
        if (!g->copy_stream) PTW_CUDA(cudaStreamCreateWithFlags(&g->copy_stream, cudaStreamNonBlocking));
        PTW_CUDA(device_malloc(&a->by_name, std::max<uint64_t>((uint64_t)g->dg.id_bound * 4, 4)));
        PTW_CUDA(cudaHostAlloc(&a->h_moves, sizeof(unsigned long long), cudaHostAllocDefault));
        PTW_CUDA(cudaEventCreate(&a->ev_start));
        PTW_CUDA(cudaEventCreate(&a->ev_walk));
        PTW_CUDA(cudaEventCreate(&a->ev_copy));
    } else {
        // the slot's previous copy (two calls back) must be done reading by_name
        PTW_CUDA(cudaStreamWaitEvent(g->stream, a->ev_copy, 0));
    }
    PTW_CUDA(cudaEventRecord(a->ev_start, g->stream));
    rc = run_count(g, cfg, a->by_name);
    if (rc) return rc;
    PTW_CUDA(cudaMemcpyAsync(a->h_moves, g->sc.ctrl + 1, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                             g->stream));
    PTW_CUDA(cudaEventRecord(a->ev_walk, g->stream));
    PTW_CUDA(cudaStreamWaitEvent(g->copy_stream, a->ev_walk, 0));
    PTW_CUDA(cudaMemcpyAsync(h_counts, a->by_name, (uint64_t)g->dg.id_bound * 4, cudaMemcpyDeviceToHost,
                             g->copy_stream));
    PTW_CUDA(cudaEventRecord(a->ev_copy, g->copy_stream));
    a->walkers = cfg->n_walkers;
    a->ticket = g->next_ticket++;
    *ticket = a->ticket;
    return PTW_OK;
} catch (...) {
    return host_exception();
}

extern "C" int ptw_pagerank_wait(ptw_graph *g, uint64_t ticket, ptw_walk_stats *stats)
try {
    NvtxRange nvtx("ptw_pagerank_wait");
    if (!g) return fail(PTW_EINVAL, "null graph");
    AsyncSlot *a = nullptr;
    for (AsyncSlot &x : g->async)
        if (ticket != 0 && x.ticket == ticket) a = &x;
    if (!a) return fail(PTW_EINVAL, "no pipelined walk in flight with ticket " + std::to_string(ticket));
    PTW_CUDA(cudaSetDevice(g->device));
    a->ticket = 0;  // the slot is free again whatever happens below
    PTW_CUDA(cudaEventSynchronize(a->ev_copy));
    if (const int rc = check_word_status(g)) return rc;
    if (stats) {
        stats->walkers = a->walkers;
        stats->moves = *a->h_moves;
        stats->visits = a->walkers + *a->h_moves;
        float ms = 0;
        PTW_CUDA(cudaEventElapsedTime(&ms, a->ev_start, a->ev_walk));
        stats->kernel_ms = ms;
        PTW_CUDA(cudaEventElapsedTime(&ms, a->ev_start, a->ev_copy));
        stats->total_ms = ms;
    }
    return PTW_OK;
} catch (...) {
    return host_exception();
}

extern "C" int ptw_rwr_dev(ptw_graph *g, const ptw_walk_cfg *cfg, uint32_t *d_pairs,
                           ptw_walk_stats *stats)
try {
    NvtxRange nvtx("ptw_rwr_dev");
    int rc = check_cfg(g, cfg, true);
    if (rc) return rc;
    if (!d_pairs && cfg->n_walkers) return fail(PTW_EINVAL, "null pairs buffer");
    if ((uintptr_t)d_pairs % 8) return fail(PTW_EINVAL, "pairs buffer must be 8-byte aligned");
    PTW_CUDA(cudaSetDevice(g->device));
    rc = run_endpoint(g, cfg, d_pairs);
    if (rc) return rc;
    PTW_CUDA(cudaEventRecord(g->ev[2], g->stream));
    if ((rc = check_word_status(g))) return rc;
    return finish_stats(g, stats, cfg->n_walkers, false);
} catch (...) {
    return host_exception();
}

extern "C" int ptw_rwr(ptw_graph *g, const ptw_walk_cfg *cfg, uint32_t *h_pairs, ptw_walk_stats *stats)
try {
    NvtxRange nvtx("ptw_rwr");
    int rc = check_cfg(g, cfg, true);
    if (rc) return rc;
    if (!h_pairs && cfg->n_walkers) return fail(PTW_EINVAL, "null pairs buffer");
    PTW_CUDA(cudaSetDevice(g->device));
    void *stage = nullptr;
    rc = stage_bytes(g, cfg->n_walkers * 8, &stage);
    if (rc) return rc;
    rc = run_endpoint(g, cfg, (uint32_t *)stage);
    if (rc) return rc;
    if (cfg->n_walkers)
        PTW_CUDA(cudaMemcpyAsync(h_pairs, stage, cfg->n_walkers * 8, cudaMemcpyDeviceToHost, g->stream));
    PTW_CUDA(cudaEventRecord(g->ev[2], g->stream));
    PTW_CUDA(cudaStreamSynchronize(g->stream));
    if ((rc = check_word_status(g))) return rc;
    return finish_stats(g, stats, cfg->n_walkers, false);
} catch (...) {
    return host_exception();
}

extern "C" int ptw_deepwalk_dev(ptw_graph *g, const ptw_walk_cfg *cfg, uint32_t L, int32_t *d_paths,
                                ptw_walk_stats *stats)
try {
    NvtxRange nvtx("ptw_deepwalk_dev");
    int rc = check_cfg(g, cfg, false);
    if (rc) return rc;
    if (!d_paths && cfg->n_walkers && L) return fail(PTW_EINVAL, "null paths buffer");
    if (g->dg.id_bound > 0x80000000u) return fail(PTW_EINVAL, "names above 2^31-1 do not fit int32 paths");
    PTW_CUDA(cudaSetDevice(g->device));
    rc = run_paths(g, cfg, L, d_paths);
    if (rc) return rc;
    PTW_CUDA(cudaEventRecord(g->ev[2], g->stream));
    if ((rc = check_word_status(g))) return rc;
    if (stats) {
        PTW_CUDA(cudaStreamSynchronize(g->stream));
        stats->walkers = cfg->n_walkers;
        stats->moves = L ? cfg->n_walkers * (uint64_t)(L - 1) : 0;  // dead ends excluded below
        stats->visits = 0;
        float ms = 0;
        PTW_CUDA(cudaEventElapsedTime(&ms, g->ev[0], g->ev[1]));
        stats->kernel_ms = ms;
        PTW_CUDA(cudaEventElapsedTime(&ms, g->ev[3], g->ev[2]));
        stats->total_ms = ms;
    }
    return PTW_OK;
} catch (...) {
    return host_exception();
}

extern "C" int ptw_deepwalk(ptw_graph *g, const ptw_walk_cfg *cfg, uint32_t L, int32_t *h_paths,
                            ptw_walk_stats *stats)
try {
    NvtxRange nvtx("ptw_deepwalk");
    int rc = check_cfg(g, cfg, false);
    if (rc) return rc;
    if (!h_paths && cfg->n_walkers && L) return fail(PTW_EINVAL, "null paths buffer");
    if (g->dg.id_bound > 0x80000000u) return fail(PTW_EINVAL, "names above 2^31-1 do not fit int32 paths");
    PTW_CUDA(cudaSetDevice(g->device));
    const uint64_t bytes = cfg->n_walkers * (uint64_t)L * 4;
    void *stage = nullptr;
    rc = stage_bytes(g, bytes, &stage);
    if (rc) return rc;
    rc = upload_sources(g, cfg);
    if (rc) return rc;
    PTW_CUDA(cudaEventRecord(g->ev[3], g->stream));
    PTW_CUDA(cudaMemsetAsync(g->sc.ctrl, 0, 2 * sizeof(unsigned long long), g->stream));
    const uint32_t ns = cfg->start_mode == PTW_START_SOURCES ? cfg->n_sources : 0;
    rc = paths_to_host(g, cfg, L, h_paths, (int32_t *)stage, [&](uint64_t b, uint64_t e, int32_t *d) {
        return launch_paths(g, b, e, L, cfg->seed, cfg->start_mode, ns, d);
    });
    if (rc) return rc;
    if ((rc = check_word_status(g))) return rc;
    if (stats) {
        stats->walkers = cfg->n_walkers;
        stats->moves = L ? cfg->n_walkers * (uint64_t)(L - 1) : 0;
        stats->visits = 0;
        float ms = 0;
        PTW_CUDA(cudaEventElapsedTime(&ms, g->ev[0], g->ev[1]));
        stats->kernel_ms = ms;
        PTW_CUDA(cudaEventElapsedTime(&ms, g->ev[3], g->ev[2]));
        stats->total_ms = ms;
    }
    return PTW_OK;
} catch (...) {
    return host_exception();
}

extern "C" int ptw_node2vec_dev(ptw_graph *g, const ptw_walk_cfg *cfg, uint32_t L, double p, double q,
                                int32_t *d_paths, ptw_node2vec_stats *stats)
try {
    NvtxRange nvtx("ptw_node2vec_dev");
    uint64_t thr[3];
    int rc = n2v_thresholds(p, q, thr);
    if (rc) return rc;
    rc = check_cfg(g, cfg, false);
    if (rc) return rc;
    if (!d_paths && cfg->n_walkers && L) return fail(PTW_EINVAL, "null paths buffer");
    if (g->dg.id_bound > 0x80000000u) return fail(PTW_EINVAL, "names above 2^31-1 do not fit int32 paths");
    PTW_CUDA(cudaSetDevice(g->device));
    rc = run_node2vec(g, cfg, L, p, q, thr, d_paths);
    if (rc) return rc;
    PTW_CUDA(cudaEventRecord(g->ev[2], g->stream));
    if ((rc = check_word_status(g))) return rc;
    return stats ? node2vec_stats(g, cfg, stats) : PTW_OK;
} catch (...) {
    return host_exception();
}

extern "C" int ptw_node2vec(ptw_graph *g, const ptw_walk_cfg *cfg, uint32_t L, double p, double q,
                            int32_t *h_paths, ptw_node2vec_stats *stats)
try {
    NvtxRange nvtx("ptw_node2vec");
    uint64_t thr[3];
    int rc = n2v_thresholds(p, q, thr);
    if (rc) return rc;
    rc = check_cfg(g, cfg, false);
    if (rc) return rc;
    if (!h_paths && cfg->n_walkers && L) return fail(PTW_EINVAL, "null paths buffer");
    if (g->dg.id_bound > 0x80000000u) return fail(PTW_EINVAL, "names above 2^31-1 do not fit int32 paths");
    PTW_CUDA(cudaSetDevice(g->device));
    const uint64_t bytes = cfg->n_walkers * (uint64_t)L * 4;
    void *stage = nullptr;
    rc = stage_bytes(g, bytes, &stage);
    if (rc) return rc;
    rc = upload_sources(g, cfg);
    if (rc) return rc;
    PTW_CUDA(cudaEventRecord(g->ev[3], g->stream));
    PTW_CUDA(cudaMemsetAsync(g->sc.ctrl, 0, 5 * sizeof(unsigned long long), g->stream));
    if (cfg->n_walkers && L && !(ensure_ext_columns(g) && ensure_edge_filter(g)))
        return fail(PTW_ENOMEM, "node2vec needs the extended column copy (16 bytes per CSR entry) and "
                                "the edge filter (2 bytes per CSR entry), which do not fit in device memory");
    const uint32_t ns = cfg->start_mode == PTW_START_SOURCES ? cfg->n_sources : 0;
    rc = paths_to_host(g, cfg, L, h_paths, (int32_t *)stage, [&](uint64_t b, uint64_t e, int32_t *d) -> int {
        // each chunk draws walker ids from a fresh cursor; the counters add up
        PTW_CUDA(cudaMemsetAsync(g->sc.ctrl, 0, sizeof(unsigned long long), g->stream));
        return launch_node2vec(g, b, e, L, cfg->seed, cfg->start_mode, ns, p, q, thr, d);
    });
    if (rc) return rc;
    if ((rc = check_word_status(g))) return rc;
    return stats ? node2vec_stats(g, cfg, stats) : PTW_OK;
} catch (...) {
    return host_exception();
}

extern "C" int ptw_autotune(ptw_graph *g, double sp, uint64_t n_walkers, ptw_tune *best)
try {
    NvtxRange nvtx("ptw_autotune");
    if (!g) return fail(PTW_EINVAL, "null graph");
    if (!(sp > 0.0 && sp <= 1.0) || stop_threshold(sp) == 0)
        return fail(PTW_EINVAL, "sp must be in [2^-32, 1]");
    PTW_CUDA(cudaSetDevice(g->device));
    ptw_walk_cfg cfg{};
    cfg.n_walkers = n_walkers ? n_walkers : g->dg.n;
    cfg.sp = sp;
    cfg.seed = 0x5eedull;
    cfg.start_mode = PTW_START_PER_VERTEX;
    const ptw_tune saved = g->tune;
    ptw_tune bt = saved;
    const int blocks[] = {256, 512, 768, 1024};
    const int ilps[] = {2, 4};
    const int chunks[] = {64, 256};
    const int hots[] = {0, 8192};
    const int minbs[] = {0, 2};
    const int hintss[] = {0, 1};
    const int exts[] = {0, 1};
    WalkLaunch wl = make_launch(&cfg);
    // Median time per launch of `reps` timings after one warm-up (the warm-up
    // also builds a column copy the candidate asks for); each timing runs
    // three walks back to back, as a caller's loop of walks does, so the
    // launch tails and gaps count the way they do there.  A walk is timed
    // with what a call does after it: counts by name straight from the walk
    // on extended columns, a scatter by name otherwise.  A negative time
    // marks a candidate that does not launch.
    if (!g->sc.by_name) PTW_CUDA(device_malloc(&g->sc.by_name, std::max<uint64_t>((uint64_t)g->dg.id_bound * 4, 4)));
    auto time_walk = [&](const ptw_tune &t, int reps, float *med) -> int {
        std::vector<float> ms(reps);
        const bool by_name = count_walk_by_name(g, t);
        WalkLaunch twl = wl;
        if (by_name) twl.by_name = g->sc.by_name;
        for (int rep = -1; rep < reps; ++rep) {
            PTW_CUDA(cudaEventRecord(g->ev[0], g->stream));
            for (int l = 0; l < 3; ++l) {
                if (by_name) PTW_CUDA(cudaMemsetAsync(g->sc.by_name, 0, (uint64_t)g->dg.id_bound * 4, g->stream));
                else PTW_CUDA(cudaMemsetAsync(g->sc.counts, 0, (uint64_t)g->dg.n * 4, g->stream));
                if (launch_walk(g, twl, t) != PTW_OK) {
                    *med = -1.f;
                    return PTW_OK;
                }
                if (!by_name && launch_counts_by_name(g, g->sc.by_name) != PTW_OK) {
                    *med = -1.f;
                    return PTW_OK;
                }
            }
            PTW_CUDA(cudaEventRecord(g->ev[1], g->stream));
            PTW_CUDA(cudaEventSynchronize(g->ev[1]));
            float x = 0;
            PTW_CUDA(cudaEventElapsedTime(&x, g->ev[0], g->ev[1]));
            if (rep >= 0) ms[rep] = x / 3.f;
        }
        std::sort(ms.begin(), ms.end());
        *med = reps % 2 ? ms[reps / 2] : 0.5f * (ms[reps / 2 - 1] + ms[reps / 2]);
        return PTW_OK;
    };
    // Stage 1: every candidate, median of 3.  The candidates differ by a few
    // percent, about the launch-to-launch noise, so stage 2 re-times the six
    // fastest in three interleaved rounds of 5 and keeps the lowest median.
    std::vector<std::pair<float, ptw_tune>> cand;
    for (int ex : exts)
    for (int hn : hintss)
    for (int mb : minbs)
    for (int hk : hots)
        for (int bl : blocks)
            for (int il : ilps)
                for (int ch : chunks) {
                    ptw_tune t{};
                    t.block = bl;
                    t.ilp = il;
                    t.chunk = ch;
                    t.hot_k = hk;
                    t.blocks_per_sm = 0;
                    t.min_blocks = mb;
                    t.cache_hints = hn;
                    t.paths_ilp = 2;
                    t.ext_columns = ex;  // walks only; the paths sweep sets bit 1
                    float med = 0;
                    int rc = time_walk(t, 3, &med);
                    if (rc) return rc;
                    if (med > 0) cand.push_back({med, t});
                }
    // walkers in shared memory: slots per thread x block x hot counters
    for (int gs : {8, 16})
        for (int bl : {128, 256})
            for (int hk : {0, 8192})
                for (int hn : {0, 1})
                    for (int ch : {64, 256}) {
                        ptw_tune t{};
                        t.block = bl;
                        t.ilp = 2;
                        t.chunk = ch;
                        t.hot_k = hk;
                        t.cache_hints = hn;
                        t.paths_ilp = 2;
                        t.gather_slots = gs;
                        float med = 0;
                        int rc = time_walk(t, 3, &med);
                        if (rc) return rc;
                        if (med > 0) cand.push_back({med, t});
                    }
    if (cand.empty()) return fail(PTW_EINVAL, "no walk configuration launches on this device");
    std::sort(cand.begin(), cand.end(), [](const auto &x, const auto &y) { return x.first < y.first; });
    // warp-aggregated visits for the three fastest register-resident candidates
    {
        std::vector<ptw_tune> agg;
        for (const auto &c : cand)
            if (agg.size() < 3 && c.second.min_blocks == 0 && c.second.gather_slots == 0) agg.push_back(c.second);
        for (ptw_tune t : agg) {
            t.warp_agg = 1;
            float med = 0;
            int rc = time_walk(t, 3, &med);
            if (rc) return rc;
            if (med > 0) cand.push_back({med, t});
        }
        std::sort(cand.begin(), cand.end(), [](const auto &x, const auto &y) { return x.first < y.first; });
    }
    cand.resize(std::min<size_t>(cand.size(), 6));
    std::vector<float> sum(cand.size(), 0.f);
    for (int round = 0; round < 3; ++round)
        for (size_t c = 0; c < cand.size(); ++c) {
            float med = 0;
            int rc = time_walk(cand[c].second, 5, &med);
            if (rc) return rc;
            sum[c] += med;
        }
    bt = cand[std::min_element(sum.begin(), sum.end()) - sum.begin()].second;
    // DeepWalk: groups per warp x column layout (extended / name-paired /
    // plain), timed on a short fixed-length walk each.
    {
        const uint64_t W = std::min<uint64_t>(g->dg.n, 1u << 20);
        const uint32_t L = 16;
        void *buf = nullptr;
        int rc = stage_bytes(g, W * L * 4, &buf);
        if (rc) return rc;
        float best_ms = 1e30f;
        const int walk_ext = bt.ext_columns & 1;
        bt.paths_ilp = 2;
        bt.paths_named = saved.paths_named;
        for (int cfg_i = 0; cfg_i < 9; ++cfg_i) {
            const int G = cfg_i % 3 == 0 ? 1 : cfg_i % 3 == 1 ? 2 : 4;
            const int layout = cfg_i / 3;  // 0 extended, 1 name-paired, 2 plain
            const int named = layout == 1 ? 1 : 0;
            const int ext = walk_ext | (layout == 0 ? 2 : 0);
            g->tune = bt;
            g->tune.paths_ilp = G;
            g->tune.paths_named = named;
            g->tune.ext_columns = ext;
            float tot = 0;
            for (int rep = 0; rep < 3; ++rep) {
                PTW_CUDA(cudaEventRecord(g->ev[0], g->stream));
                rc = launch_paths(g, 0, W, L, 0x5eedull + rep, PTW_START_PER_VERTEX, 0, (int32_t *)buf);
                if (rc) return rc;
                PTW_CUDA(cudaEventRecord(g->ev[1], g->stream));
                PTW_CUDA(cudaEventSynchronize(g->ev[1]));
                float ms = 0;
                PTW_CUDA(cudaEventElapsedTime(&ms, g->ev[0], g->ev[1]));
                if (rep) tot += ms;
            }
            if (tot < best_ms) {
                best_ms = tot;
                bt.paths_ilp = G;
                bt.paths_named = named;
                bt.ext_columns = ext;
            }
        }
    }
    g->tune = bt;
    drop_unused_columns(g);
    if (best) *best = bt;
    return PTW_OK;
} catch (...) {
    return host_exception();
}
