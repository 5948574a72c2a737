// Internal declarations shared by the libptw translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <exception>
#include <functional>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/ptw.h"
#include <nvtx3/nvToolsExt.h>

// Philox counter words that separate the purposes of a draw.
#define PTW_TAG_WALK 0x57414C4Bu  // "WALK": one draw per move
#define PTW_TAG_START 0x53545254u // "STRT": start-vertex draw
#define PTW_TAG_RMAT 0x524D4154u  // "RMAT": synthetic edge generation
#define PTW_TAG_CHUNGLU 0x43484C55u // "CHLU": Chung-Lu endpoints
#define PTW_TAG_N2V 0x4E320000u     // "N2" + trial pair index: node2vec candidate draws

namespace ptw {

// Names a host-side span for profilers (NVTX ranges; nothing is recorded
// unless a profiler is attached).
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

// Records msg as the calling thread's last error and returns code.
int fail(int code, const std::string &msg);
int cuda_fail(cudaError_t e, const char *what);
// Inside a catch block at the C ABI: records the host exception being
// handled and returns its status (PTW_ENOMEM for an allocation failure).
// No C++ exception crosses the ABI.
int host_exception();

// Runs fn(t) for t in [0, n) on n host threads.  An exception thrown on any
// of them (or while starting them) is rethrown here after every started
// thread has joined.
template <class F>
void parallel_for_threads(unsigned n, F fn)
{
    std::vector<std::thread> th;
    std::exception_ptr err;
    std::mutex mu;
    auto keep = [&] {
        std::lock_guard<std::mutex> lk(mu);
        if (!err) err = std::current_exception();
    };
    try {
        th.reserve(n);
        for (unsigned t = 0; t < n; ++t)
            th.emplace_back([&, t] {
                try {
                    fn(t);
                } catch (...) {
                    keep();
                }
            });
    } catch (...) {
        keep();
    }
    for (std::thread &x : th) x.join();
    if (err) std::rethrow_exception(err);
}

// Stop threshold of the termination draw: a walker stops after a move iff
// the draw's 32-bit word u satisfies u < floor(sp * 2^32); sp = 1 stops
// after every move.
inline uint64_t stop_threshold(double sp)
{
    if (sp >= 1.0) return 1ull << 32;
    return (uint64_t)(sp * 4294967296.0);
}

// Validates a stop probability and move cap: sp in [0, 1], and a walk that
// can end.  A threshold of 0 (sp below 2^-32, sp = 0 included) never stops
// a walker, so without max_moves a walk on a graph whose vertices all have
// out-edges would never return.
int check_stop(double sp, uint32_t max_moves);

#define PTW_CUDA(call)                                   \
    do {                                                 \
        cudaError_t _e = (call);                         \
        if (_e != cudaSuccess) return ptw::cuda_fail(_e, #call); \
    } while (0)

// Philox4x32-10 (Salmon et al., SC'11): ten rounds of the 4x32 S-box,
// multipliers 0xD2511F53 / 0xCD9E8D57, Weyl key increments 0x9E3779B9 /
// 0xBB67AE85.  ctr = (x, y, z, w), key = (k0, k1).
__device__ __forceinline__ uint4 philox(uint4 c, uint32_t k0, uint32_t k1)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint32_t hi0 = __umulhi(0xD2511F53u, c.x);
        const uint32_t lo0 = 0xD2511F53u * c.x;
        const uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z);
        const uint32_t lo1 = 0xCD9E8D57u * c.z;
        c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}

// Start vertex (internal id) of walker wid: PTW_START_PER_VERTEX takes the
// (wid mod n)-th vertex by name; PTW_START_UNIFORM draws a vertex with
// Philox(ctr = (wid_lo, wid_hi, 0, "STRT")); PTW_START_SOURCES draws from the
// source list the same way (one source needs no draw).
__device__ __forceinline__ uint32_t walker_start(int start_mode, const uint32_t *start_map,
                                                 const uint32_t *sources, uint32_t n, uint32_t n_sources,
                                                 uint32_t key0, uint32_t key1, uint64_t wid)
{
    if (start_mode == PTW_START_PER_VERTEX) {
        const uint32_t idx = wid < n ? (uint32_t)wid : (uint32_t)(wid % n);
        return start_map[idx];
    }
    if (start_mode == PTW_START_SOURCES && n_sources == 1) return sources[0];
    const uint4 r = philox(make_uint4((uint32_t)wid, (uint32_t)(wid >> 32), 0u, PTW_TAG_START), key0, key1);
    if (start_mode == PTW_START_UNIFORM) return start_map[__umulhi(r.x, n)];
    return sources[__umulhi(r.x, n_sources)];
}

// The same start as walker_start, as a canonical index (name rank): the
// index into vertex tables kept in name order (vtx_ext).  Consecutive
// walkers of PTW_START_PER_VERTEX then read consecutive records, and the
// per-vertex and uniform modes need no index-to-id lookup.
__device__ __forceinline__ uint32_t walker_start_index(int start_mode, const uint32_t *int2idx,
                                                       const uint32_t *sources, uint32_t n, uint32_t n_sources,
                                                       uint32_t key0, uint32_t key1, uint64_t wid)
{
    if (start_mode == PTW_START_PER_VERTEX) return wid < n ? (uint32_t)wid : (uint32_t)(wid % n);
    if (start_mode == PTW_START_SOURCES && n_sources == 1) return int2idx[sources[0]];
    const uint4 r = philox(make_uint4((uint32_t)wid, (uint32_t)(wid >> 32), 0u, PTW_TAG_START), key0, key1);
    if (start_mode == PTW_START_UNIFORM) return __umulhi(r.x, n);
    return int2idx[sources[__umulhi(r.x, n_sources)]];
}

// Index checks of the checked build (nvcc -DPTW_CHECKED; libptw built by
// ptwalker_gb300._build.build_checked): an index at or above its bound sets
// bit `site` of the graph's check word (scratch ctrl[7]) and is replaced by
// 0, so the access stays in bounds and the entry point reports the failure
// (check_word_status).  The normal build compiles the index unchanged.
// Sites: see kCheck* below.
enum : int {
    kCheckRecord = 0,   // row record / vertex record of a vertex id (< n)
    kCheckColumn = 1,   // CSR entry (< m)
    kCheckCounter = 2,  // per-vertex counter or name (< n)
    kCheckStart = 3,    // start map / source list entry
    kCheckTable = 4,    // count-table slot of a batched query
    kCheckQuery = 5,    // query-table entry or work descriptor
    kCheckPath = 6,     // path position (< walkers * L)
    kCheckFilter = 7,   // edge-filter block
};
#ifdef PTW_CHECKED
__device__ __forceinline__ uint64_t checked_index(uint64_t i, uint64_t n, unsigned long long *word, int site)
{
    if (i < n) return i;
    atomicOr(word, 1ull << site);
    return 0;
}
#define PTW_IDX(i, n, word, site) ptw::checked_index((i), (n), (word), (site))
#else
#define PTW_IDX(i, n, word, site) (i)
#endif

// L2 eviction-priority policies (PTX createpolicy) for the gathers:
// kind 0 = normal, 1 = evict_last (keep: row records, visit counters),
// 2 = evict_first (stream: the column array).
__device__ __forceinline__ uint64_t l2_policy(int kind)
{
    uint64_t p;
    if (kind == 1) asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    else if (kind == 2) asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    else asm("createpolicy.fractional.L2::evict_normal.b64 %0, 1.0;" : "=l"(p));
    return p;
}

__device__ __forceinline__ uint2 ld_hint_u2(const uint2 *p, uint64_t pol)
{
    uint2 r;
    asm("ld.global.nc.L2::cache_hint.v2.u32 {%0, %1}, [%2], %3;" : "=r"(r.x), "=r"(r.y) : "l"(p), "l"(pol));
    return r;
}

__device__ __forceinline__ uint4 ld_hint_u4(const uint4 *p, uint64_t pol)
{
    uint4 r;
    asm("ld.global.nc.L1::no_allocate.L2::cache_hint.v4.u32 {%0, %1, %2, %3}, [%4], %5;"
        : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
        : "l"(p), "l"(pol));
    return r;
}

// Asynchronous 16-byte global -> shared copy (cp.async, L1 bypassed) with an
// L2 eviction-priority policy; completes at the next cp_async_wait_all.
__device__ __forceinline__ void cp_async16(void *smem_dst, const void *gmem_src, uint64_t pol)
{
    const uint32_t d = (uint32_t)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.cg.shared.global.L2::cache_hint [%0], [%1], 16, %2;" ::"r"(d), "l"(gmem_src), "l"(pol)
                 : "memory");
}

__device__ __forceinline__ void cp_async_wait_all()
{
    asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

// Streaming 16-byte load: read-only path, no L1 allocation.
__device__ __forceinline__ uint4 ld_stream_u4(const uint4 *p)
{
    uint4 r;
    asm("ld.global.nc.L1::no_allocate.v4.u32 {%0, %1, %2, %3}, [%4];"
                 : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
                 : "l"(p));
    return r;
}

__device__ __forceinline__ uint32_t ld_hint_u32(const uint32_t *p, uint64_t pol)
{
    uint32_t r;
    asm("ld.global.nc.L1::no_allocate.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(r) : "l"(p), "l"(pol));
    return r;
}

__device__ __forceinline__ void red_add_hint(uint32_t *p, uint32_t v, uint64_t pol)
{
    asm volatile("red.global.add.L2::cache_hint.u32 [%0], %1, %2;" ::"l"(p), "r"(v), "l"(pol) : "memory");
}

// Device-resident graph.  Internal vertex ids are ranks by descending
// degree (ties by ascending name), so the hottest rows, counters and column
// blocks sit at the low end of every array and stay in L2.
struct DeviceGraph {
    uint32_t n = 0;
    uint64_t m = 0;
    uint32_t id_bound = 0;
    uint32_t max_degree = 0;
    uint2 *adj = nullptr;        // [n] {first column, degree} by internal id
    uint32_t *col = nullptr;     // [m] neighbour internal ids; row order = name order
    uint32_t *int2name = nullptr; // [n]
    uint32_t *idx2int = nullptr;  // [n] canonical index (name rank) -> internal
    uint32_t *int2idx = nullptr;  // [n] internal -> canonical index
    uint32_t *names = nullptr;    // [n] canonical index -> name (ascending)
    uint2 *col_named = nullptr;   // [m] {neighbour internal id, its name}; built on first path walk
    uint4 *col_ext = nullptr;     // [m] {neighbour id, its first column, its degree, its name};
                                  // built on the first walk with tune.ext_columns
    uint4 *vtx_ext = nullptr;     // [n] {id, first column, degree, name} by canonical index, built with col_ext
    uint32_t *edge_filter = nullptr; // blocked Bloom filter of the directed edges (u, v): blocks of
                                     // 8 words; built on the first node2vec walk
    uint64_t filter_blocks = 0;      // a power of two
    int simple_symmetric = -1;       // 1: no row repeats a neighbour and every edge has its
                                     // reverse; 0: not; -1: not checked yet (first node2vec walk)
};

// Scratch owned by a graph handle and reused by every call.
struct Scratch {
    uint32_t *counts = nullptr;           // [n] visit counts by internal id
    unsigned long long *ctrl = nullptr;   // [8]: walker cursor, moves, error flags
    uint32_t *sources = nullptr;          // source internal ids
    uint32_t sources_cap = 0;
    uint32_t *by_name = nullptr;          // [id_bound] staging for host-output calls
    void *out_stage = nullptr;            // device staging for host-output calls
    size_t out_stage_bytes = 0;
};

// One in-flight call of the pipelined count walk (ptw_pagerank_submit):
// its counts by name on the device, its moves in page-locked host memory,
// and events for the start, the end of the walk (moves copied) and the end
// of the copy to the caller's buffer.
struct AsyncSlot {
    uint32_t *by_name = nullptr;            // [id_bound]
    unsigned long long *h_moves = nullptr;  // page-locked
    cudaEvent_t ev_start = nullptr, ev_walk = nullptr, ev_copy = nullptr;
    uint64_t ticket = 0;                    // 0 = free
    uint64_t walkers = 0;
};

}  // namespace ptw

struct ptw_graph {
    ptw::DeviceGraph dg;
    ptw::Scratch sc;
    uint32_t *h_names = nullptr;   // [n] ascending, for host-side name lookups
    uint32_t *h_idx2int = nullptr; // [n] canonical index -> internal id
    cudaStream_t stream = nullptr;     // stream all work is issued on
    cudaStream_t own_stream = nullptr; // created with the handle
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    int device = 0;
    int num_sms = 0;
    ptw_tune tune{};
    ptw_batch_tune btune{};  // zero fields: defaults (see ptw_batch_tune)
    uint64_t device_bytes = 0;
    int ext_users = 0;  // open servers reading the extended columns (kept while > 0)
    ptw::AsyncSlot async[2];             // pipelined count walks in flight
    cudaStream_t copy_stream = nullptr;  // their copies to the host
    uint64_t next_ticket = 1;
};

namespace ptw {

// Builds a canonical + degree-sorted device graph from device edge arrays
// (consumes them).  Implemented in graph.cu.
int build_graph_from_device_edges(ptw_graph *g, uint32_t *d_src, uint32_t *d_dst, uint64_t m,
                                  bool as_undirected, bool clean, bool compact_names);
// Expands a validated host CSR (row_ptr[n+1], col[row_ptr[n]], optional
// names[n]) into device (src, dst) name arrays allocated on st; rejects a
// column index >= n and repeated names.  Implemented in graph.cu.
int csr_to_device_edges(const uint64_t *h_row_ptr, const uint32_t *h_col, const uint32_t *h_names,
                        uint32_t n, uint32_t **d_src, uint32_t **d_dst, cudaStream_t st);
int rmat_generate_device(uint32_t scale, uint64_t m, uint32_t ta, uint32_t tab, uint32_t tabc,
                         uint64_t seed, uint32_t *d_src, uint32_t *d_dst, cudaStream_t st);
int chung_lu_generate_device(uint32_t n, double gamma, uint64_t m, uint64_t seed, uint32_t *d_src,
                             uint32_t *d_dst, cudaStream_t st);
int graph_init_handle(ptw_graph *g);
void graph_release(ptw_graph *g);

// Walk launchers (walk.cu).
struct WalkLaunch {
    uint64_t w_begin = 0, w_end = 0;
    uint64_t thr = 0;
    uint64_t seed = 0;
    int start_mode = 0;
    uint32_t n_sources = 0;
    uint32_t max_moves = 0;
    bool endpoint = false;     // RWR endpoint app instead of counting
    uint32_t *pairs = nullptr; // endpoint output by walker (names)
    uint32_t *by_name = nullptr; // count walks: count straight into this by-name array (extended
                                 // columns; see count_walk_by_name), else into the graph's scratch
};
// True when the count walk under tune t reads the extended columns (built
// here if needed) and can count by name directly.
bool count_walk_by_name(ptw_graph *g, const ptw_tune &t);
int launch_walk(ptw_graph *g, const WalkLaunch &wl, const ptw_tune &t);
int launch_paths(ptw_graph *g, uint64_t w_begin, uint64_t w_end, uint32_t L, uint64_t seed,
                 int start_mode, uint32_t n_sources, int32_t *paths);
// Second-order (node2vec) paths (node2vec.cu): thr = acceptance thresholds
// {return, neighbour of the previous vertex, other} for the envelope
// max(1/p, 1, 1/q) (p and q pick the folded form on simple symmetric
// graphs); needs the extended column copy (PTW_ENOMEM when it does not fit).  Moves, candidate draws and
// row probes accumulate in ctrl[1..3].
int launch_node2vec(ptw_graph *g, uint64_t w_begin, uint64_t w_end, uint32_t L, uint64_t seed,
                    int start_mode, uint32_t n_sources, double p, double q, const uint64_t thr[3],
                    int32_t *paths);
// DeepWalk paths through the same per-lane loop (node2vec.cu); needs the
// extended column copy, which the caller has built.  Clears ctrl[0..1]
// (walker cursor, moves) first.
int launch_lane_deepwalk(ptw_graph *g, uint64_t w_begin, uint64_t w_end, uint32_t L, uint64_t seed,
                         int start_mode, uint32_t n_sources, int32_t *paths);
// Stream-ordered device allocation from a per-device pool that keeps up to
// a quarter of the device memory cached across synchronisations (the default
// pool hands memory back at each one), for count tables and the short-lived
// buffers of every result compaction.  Freed with cudaFreeAsync.
cudaError_t pooled_alloc_async(void **p, size_t bytes, cudaStream_t st);
// Hands the pools' cached memory back to the CUDA driver.
void trim_pools();
// cudaMalloc that, when the device is out of memory, trims the pools and
// retries once.
cudaError_t device_malloc_bytes(void **p, size_t bytes);
template <class T>
inline cudaError_t device_malloc(T **p, size_t bytes)
{
    return device_malloc_bytes(reinterpret_cast<void **>(p), bytes);
}

int launch_counts_by_name(ptw_graph *g, uint32_t *d_out);
int check_tune(const ptw_tune &t);
// Frees the column copies the graph's tune no longer reads.
void drop_unused_columns(ptw_graph *g);
// Checked build: waits for the graph's stream and fails with PTW_ECUDA
// naming the sites whose index checks tripped (clearing the word); the
// normal build returns PTW_OK at once.
int check_word_status(ptw_graph *g);

// Builds the edge filter of node2vec's neighbour test and checks whether
// the graph is simple and symmetric, on first use; false, without an error,
// when the filter does not fit in device memory.  Needs the extended columns.
bool ensure_edge_filter(ptw_graph *g);

// Builds the extended column copy (and the per-vertex records) on first use;
// false, without an error, when they do not fit in device memory.
bool ensure_ext_columns(ptw_graph *g);

// The query table a batch was run with (batch.cu).
const ptw_query *batch_queries(const ptw_batch *b);
uint32_t batch_top_k(const ptw_batch *b);
bool batch_device(const ptw_batch *b);  // results are device-resident

// (name, count) lists of nt tables in host memory: table i owns entries
// [seg[i], seg[i+1]), sorted by name.  Without a sink the lists land in the
// owned arrays names / counts; with one, sink(n) returns 2n words of caller
// memory (names in the first n, counts in the next n; nullptr = no memory).
// h_names / h_counts point at wherever they landed.  top_k > 0 keeps the
// top_k largest counts of every table instead, ordered by count descending
// and then by name (seg then delimits the kept entries).
// Host result array (new[]); page-locked with CUDA when host_pin took it,
// unregistered by the deleter before it is freed.
struct HostArrayDelete {
    void operator()(uint32_t *p) const;
};
using HostArray = std::unique_ptr<uint32_t[], HostArrayDelete>;
// Registers [p, p + bytes) of a HostArray with CUDA (page-locked), within a
// process-wide limit of a quarter of the host memory; false when refused.
bool host_pin(uint32_t *p, uint64_t bytes);

// CUDA-event intervals of the phases of a batch call on the device
// timeline (several spans of one phase add up), plus host-side waits.
struct PhaseTimer {
    enum { kUpload, kWalk, kCount, kPlace, kCopy, kPhases };
    struct Span {
        int phase;
        cudaEvent_t a, b;
    };
    std::vector<Span> spans;
    double host_pages_ms = 0, plan_ms = 0;
    uint64_t copy_bytes = 0;
    int last_place = -1, last_copy = -1;  // span indices
    // Opens a span of `phase` by recording an event on s; returns its index
    // (-1 when no event could be created: the span is then not timed).
    int begin(int phase, cudaStream_t s);
    void end(int span, cudaStream_t s);
    // Milliseconds per phase (after the recorded work has completed).
    void sums(double out[kPhases], double *copy_tail_ms) const;
    PhaseTimer() = default;
    PhaseTimer(const PhaseTimer &) = delete;
    PhaseTimer &operator=(const PhaseTimer &) = delete;
    ~PhaseTimer();
};

// Device memory from the library's pool, freed on a stream when dropped.
struct PoolArray {
    uint32_t *p = nullptr;
    cudaStream_t st = nullptr;
    PoolArray() = default;
    PoolArray(const PoolArray &) = delete;
    PoolArray &operator=(const PoolArray &) = delete;
    PoolArray(PoolArray &&o) noexcept : p(o.p), st(o.st) { o.p = nullptr; }
    PoolArray &operator=(PoolArray &&o) noexcept
    {
        if (this != &o) {
            reset();
            p = o.p;
            st = o.st;
            o.p = nullptr;
        }
        return *this;
    }
    cudaError_t alloc(uint64_t count, cudaStream_t s)
    {
        reset();
        st = s;
        void *q = nullptr;
        const cudaError_t e = pooled_alloc_async(&q, std::max<uint64_t>(count, 1) * 4, s);
        p = (uint32_t *)q;
        return e;
    }
    void reset()
    {
        if (p) cudaFreeAsync(p, st);
        p = nullptr;
    }
    ~PoolArray() { reset(); }
};

struct Compacted {
    uint32_t top_k = 0;
    // Device-resident results: the lists stay in d_names / d_counts (no host
    // buffers, no copy).
    bool device = false;
    PoolArray d_names, d_counts;
    PhaseTimer *ph = nullptr;  // phase spans of the call (may be null)
    uint64_t n = 0;
    std::vector<uint64_t> seg;
    HostArray names, counts;
    std::function<uint32_t *(uint64_t)> sink;
    uint32_t *h_names = nullptr, *h_counts = nullptr;
    // Optional host buffers of pre_cap entries, allocated before the walk
    // and faulted in on host threads while it runs (pre_join waits for
    // that); adopted when the lists fit, the unused tail handed back.
    HostArray pre_names, pre_counts;
    uint64_t pre_cap = 0;
    bool pre_pinned = false;   // pre_* are page-locked (known after pre_join)
    std::function<void()> pre_join;
    // Capacity of names / counts in entries, how many leading entries are
    // faulted in, and whether they are page-locked (a freed batch hands
    // them to the host cache).
    uint64_t cap = 0, touched = 0;
    bool pinned = false;
};
// Compacts nt count tables into *out (batch.cu).  Table i starts at slot
// h_base[i] of d_slots, an even slot (16-byte aligned; callers use 128-byte
// lines); a hash table (h_dense[i] == 0, or h_dense NULL) has h_cap[i]
// 64-bit slots, a dense table h_cap[i] = n 32-bit counters indexed by
// canonical vertex index.  The table's allocation must extend to the end of
// the 16-byte word holding its last entry (read, then masked).
int compact_tables(ptw_graph *g, unsigned long long *d_slots, const unsigned long long *h_base,
                   const uint32_t *h_cap, const uint8_t *h_dense, uint32_t nt, Compacted *out);
// The count table of a query: an open-addressing hash table sized from its
// budget, or, when the dense array of n 32-bit counters (which cannot fill)
// takes at most dense_ratio times its bytes, that array.  slots = 64-bit
// slots it occupies.
struct TableSize {
    uint64_t slots;
    bool dense;
};
TableSize count_table(double sp, uint32_t max_moves, int32_t app, double factor, uint64_t budget, uint32_t n,
                      uint32_t dense_ratio);
TableSize dense_table(uint32_t n);
// Splits [j0[i], j0[i] + count[i]) of every query entry i into walker
// descriptors {entry, first rank, count}, ordered round-robin within groups
// of consecutive entries whose tables add up to about group_bytes (0 = one
// group), group after group (batch.cu).
void interleave_descriptors(const std::vector<uint64_t> &j0, const std::vector<uint64_t> &count,
                            const std::vector<uint64_t> &table_bytes, uint64_t group_bytes,
                            std::vector<uint3> &desc);
// The same into a new buffer with descriptors of at most desc_walkers ranks,
// groups filled on up to `threads` host threads when there are many
// descriptors; returns the number of descriptors.
uint64_t interleave_descriptors(const std::vector<uint64_t> &j0, const std::vector<uint64_t> &count,
                                const std::vector<uint64_t> &table_bytes, uint64_t group_bytes,
                                std::unique_ptr<uint3[]> &desc, unsigned threads, uint32_t desc_walkers);
// Count-table bytes per descriptor group: about 3x the 129 MB L2.
constexpr uint64_t kGroupBytes = 384ull << 20;

}  // namespace ptw
