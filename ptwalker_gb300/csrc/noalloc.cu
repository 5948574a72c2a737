// ptw_pagerank_noalloc: the count walk of ptw_pagerank_dev without any
// device allocation.
//
// Who needs it: code that must not call cudaMalloc at the moment it runs --
// for example a host that has handed all device memory to its own pool
// allocator and forbids outside allocations, or a caller issuing work from a
// context where an allocation (and the device synchronisation cudaMalloc may
// imply) is not allowed.  Such a caller brings the graph (loaded earlier) and
// its own output buffer; the per-vertex counters and the walker cursor this
// walk needs beyond those live in one fixed array compiled into the library.
//
// The array, g_noalloc, is a file-scope __device__ variable: every GPU that
// loads the library holds it (about 16 MiB) until the process exits.  Host
// code cannot use its name as a device address, so set-up asks the runtime
// for the address once per device (cudaGetSymbolAddress, with that device
// current) and passes that pointer to the kernels.  The first call on a
// device performs this set-up, so make that first call before any stream
// capture begins.
//
// Every call reuses the same array and leaves its contents behind: each call
// clears the counters and the cursor before its walk.  Two calls whose work
// overlaps on the GPU (different streams, or different host threads) race on
// the array and give wrong counts; serialise them.
//
// A call issued on a stream other than the graph's is ordered against the
// graph's stream both ways through two events created at set-up: the walk
// waits for work already queued there, and work queued there later (and the
// synchronisation in ptw_graph_free) waits for the walk.
//
// The cached address belongs to the device's context: after cudaDeviceReset
// every graph is gone and this entry point must not be called again in that
// process.
#include <cstddef>
#include <mutex>

#include "ptw_internal.cuh"

namespace ptw {
namespace {

struct NoAllocScratch {
    unsigned long long ctrl[8];  // [0] walker cursor, [1] moves
    uint32_t counts[PTW_NOALLOC_MAX_VERTICES];
};

static __device__ __align__(256) NoAllocScratch g_noalloc;

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;

// Per-device set-up: the array's device address and the two ordering events.
struct NoAllocDevice {
    NoAllocScratch *addr = nullptr;
    cudaEvent_t ev_in = nullptr, ev_out = nullptr;
};
NoAllocDevice g_dev[kMaxDevices];

// Set-up on first use, with `device` current.
int device_setup(int device, NoAllocDevice **out)
{
    if (device < 0 || device >= kMaxDevices) return fail(PTW_EINVAL, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    NoAllocDevice &d = g_dev[device];
    if (!d.addr) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc)");
        cudaEvent_t a = nullptr, b = nullptr;
        e = cudaEventCreateWithFlags(&a, cudaEventDisableTiming);
        if (e != cudaSuccess) return cuda_fail(e, "cudaEventCreateWithFlags");
        e = cudaEventCreateWithFlags(&b, cudaEventDisableTiming);
        if (e != cudaSuccess) {
            cudaEventDestroy(a);
            return cuda_fail(e, "cudaEventCreateWithFlags");
        }
        d.ev_in = a;
        d.ev_out = b;
        d.addr = (NoAllocScratch *)p;
    }
    *out = &d;
    return PTW_OK;
}

struct NoAllocArgs {
    const uint2 *__restrict__ adj;
    const uint32_t *__restrict__ col;
    const uint32_t *__restrict__ start_map;
    NoAllocScratch *scratch;
    uint64_t w_begin, n_walk, thr;
    uint32_t n, key0, key1, max_moves;
    int start_mode;
};

constexpr uint32_t kNoAllocChunk = 256;  // walker ids a warp takes from the cursor at a time

__device__ __forceinline__ uint64_t min_u64(uint64_t x, uint64_t y) { return x < y ? x : y; }

// One walker per lane.  A lane whose walk ended takes the next id of its
// warp's private range at once (warp ballot, ranks by popcount); the warp
// takes a new range of kNoAllocChunk ids from the shared cursor when its
// range runs dry.  Same draws and the same visit semantics as the main
// count walk, so the counts do not depend on which lane walks which id.
__global__ void k_walk_noalloc(const NoAllocArgs a)
{
    constexpr unsigned kAll = 0xffffffffu;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t lt_mask = (1u << lane) - 1u;
    NoAllocScratch *s = a.scratch;
    bool act = false, exhausted = false;
    uint64_t wid = 0, next = 0, end = 0;  // warp-uniform range [next, end)
    uint32_t v = 0, step = 0;
    unsigned long long moves = 0;
    for (;;) {
        const unsigned need = __ballot_sync(kAll, !act);
        if (need != 0 && !exhausted) {
            const uint32_t n_need = __popc(need);
            const uint32_t rank = __popc(need & lt_mask);
            const uint32_t took = (uint32_t)min_u64(n_need, end - next);
            uint64_t my = ~0ull;
            if (!act && rank < took) my = next + rank;
            next += took;
            if (took < n_need) {
                unsigned long long base = 0;
                if (lane == 0) base = atomicAdd(&s->ctrl[0], (unsigned long long)kNoAllocChunk);
                base = __shfl_sync(kAll, base, 0);
                if (base >= a.n_walk) {
                    exhausted = true;
                    next = end = a.n_walk;
                } else {
                    next = base;
                    end = min_u64(base + kNoAllocChunk, a.n_walk);
                    const uint32_t take2 = (uint32_t)min_u64(n_need - took, end - next);
                    if (!act && rank >= took && rank - took < take2) my = next + (rank - took);
                    next += take2;
                }
            }
            if (my != ~0ull) {
                wid = a.w_begin + my;
                if (a.start_mode == PTW_START_PER_VERTEX) {
                    v = a.start_map[wid < a.n ? (uint32_t)wid : (uint32_t)(wid % a.n)];
                } else {
                    const uint4 r = philox(make_uint4((uint32_t)wid, (uint32_t)(wid >> 32), 0u, PTW_TAG_START),
                                           a.key0, a.key1);
                    v = a.start_map[__umulhi(r.x, a.n)];
                }
                step = 0;
                act = true;
                atomicAdd(&s->counts[v], 1u);
            }
        }
        if (!__any_sync(kAll, act)) break;  // every lane idle after a refill: no ids left
        if (act) {
            const uint2 rec = __ldg(&a.adj[v]);
            if (rec.y == 0) {
                act = false;
            } else {
                const uint4 r = philox(make_uint4((uint32_t)wid, (uint32_t)(wid >> 32), step, PTW_TAG_WALK),
                                       a.key0, a.key1);
                v = __ldg(&a.col[rec.x + __umulhi(r.x, rec.y)]);
                ++step;
                ++moves;
                atomicAdd(&s->counts[v], 1u);
                if ((uint64_t)r.y < a.thr || (a.max_moves && step >= a.max_moves)) act = false;
            }
        }
    }
    for (int o = 16; o; o >>= 1) moves += __shfl_xor_sync(kAll, moves, o);
    if (lane == 0 && moves) atomicAdd(&s->ctrl[1], moves);
}

__global__ void k_scatter_noalloc(const NoAllocScratch *s, const uint32_t *int2name, uint32_t n,
                                  uint32_t *out)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[int2name[i]] = s->counts[i];
}

}  // namespace
}  // namespace ptw

using namespace ptw;

extern "C" int ptw_pagerank_noalloc(const ptw_graph *g, const ptw_walk_cfg *cfg, uint32_t *d_counts,
                                    void *cuda_stream)
try {
    NvtxRange nvtx("ptw_pagerank_noalloc");
    if (!cfg) return fail(PTW_EINVAL, "null argument");
    if (const int rc0 = check_stop(cfg->sp, cfg->max_moves)) return rc0;
    if (!g || !d_counts) return fail(PTW_EINVAL, "null argument");
    if (g->dg.n > PTW_NOALLOC_MAX_VERTICES)
        return fail(PTW_EINVAL, "graph has " + std::to_string(g->dg.n) +
                                    " vertices; ptw_pagerank_noalloc holds counters for at most " +
                                    std::to_string(PTW_NOALLOC_MAX_VERTICES));
    if (cfg->start_mode != PTW_START_PER_VERTEX && cfg->start_mode != PTW_START_UNIFORM)
        return fail(PTW_EINVAL, "ptw_pagerank_noalloc supports per-vertex and uniform starts only");
    if (cfg->n_walkers > ~0ull - cfg->first_walker) return fail(PTW_EINVAL, "walker ids overflow 64 bits");
    PTW_CUDA(cudaSetDevice(g->device));
    NoAllocDevice *dv = nullptr;
    int rc = device_setup(g->device, &dv);
    if (rc) return rc;
    NoAllocScratch *s = dv->addr;
    cudaStream_t st = cuda_stream ? (cudaStream_t)cuda_stream : g->stream;
    const bool other_stream = st != g->stream;
    if (other_stream) {  // after the work already queued on the graph's stream
        PTW_CUDA(cudaEventRecord(dv->ev_in, g->stream));
        PTW_CUDA(cudaStreamWaitEvent(st, dv->ev_in, 0));
    }
    const uint32_t n = g->dg.n;
    // Clear what must start at zero: the control words and n counters.
    PTW_CUDA(cudaMemsetAsync(s, 0, offsetof(NoAllocScratch, counts) + (size_t)n * 4, st));
    if (cfg->n_walkers) {
        NoAllocArgs a;
        a.adj = g->dg.adj;
        a.col = g->dg.col;
        a.start_map = g->dg.idx2int;
        a.scratch = s;
        a.w_begin = cfg->first_walker;
        a.n_walk = cfg->n_walkers;
        a.thr = stop_threshold(cfg->sp);
        a.n = n;
        a.key0 = (uint32_t)cfg->seed;
        a.key1 = (uint32_t)(cfg->seed >> 32);
        a.max_moves = cfg->max_moves;
        a.start_mode = cfg->start_mode;
        int per_sm = 0;
        PTW_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_walk_noalloc, 256, 0));
        const uint64_t ranges = (cfg->n_walkers + kNoAllocChunk - 1) / kNoAllocChunk;
        uint64_t grid = (uint64_t)g->num_sms * (per_sm > 0 ? per_sm : 1);
        grid = grid < (ranges + 7) / 8 ? grid : (ranges + 7) / 8;  // no more warps than id ranges
        k_walk_noalloc<<<(unsigned)(grid ? grid : 1), 256, 0, st>>>(a);
        PTW_CUDA(cudaGetLastError());
    }
    if (g->dg.id_bound != n) PTW_CUDA(cudaMemsetAsync(d_counts, 0, (uint64_t)g->dg.id_bound * 4, st));
    const unsigned sgrid = (unsigned)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
    k_scatter_noalloc<<<sgrid ? sgrid : 1, 256, 0, st>>>(s, g->dg.int2name, n, d_counts);
    PTW_CUDA(cudaGetLastError());
    if (other_stream) {  // later work on the graph's stream (and ptw_graph_free) waits for the walk
        PTW_CUDA(cudaEventRecord(dv->ev_out, st));
        PTW_CUDA(cudaStreamWaitEvent(g->stream, dv->ev_out, 0));
    }
    return PTW_OK;
} catch (...) {
    return host_exception();
}
