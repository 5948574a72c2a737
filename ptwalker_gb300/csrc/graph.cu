// Device graph construction: canonical CSR + degree-sorted relabelling.
//
// Replaces the reference loader's CSR build and NUMA/cache partitioner
// (src/core/graph.hpp:277-785).  The reference compacts names in first
// appearance order, splits hubs (degree >= --db) from low-degree vertices,
// runs a max-cut split and L2-sized chunks and relabels randomly; all of that
// exists to keep CPU partitions cache-resident.  On one GB300 the whole CSR
// sits in HBM, so the only relabelling kept is by descending degree: the rows,
// counters and column blocks of hub vertices land at the low end of every
// array, where the 129 MB L2 keeps them.
//
// Pipeline (all on the graph's stream):
//   edges -> packed u64 keys (src<<b | dst) -> [drop self-loops] -> radix
//   sort -> [unique] -> names = sorted unique endpoints -> index space ->
//   degrees -> stable sort by degree (desc) -> internal CSR.
#include <cub/cub.cuh>

#include <algorithm>
#include <cstring>
#include <vector>

#include "ptw_internal.cuh"

namespace ptw {
namespace {

constexpr int kThreads = 256;

inline unsigned grid_for(uint64_t n, int threads = kThreads)
{
    uint64_t b = (n + threads - 1) / threads;
    return (unsigned)std::min<uint64_t>(std::max<uint64_t>(b, 1), 1u << 20);
}

__global__ void k_max2(const uint32_t *a, const uint32_t *b, uint64_t m, unsigned *out)
{
    unsigned mx = 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m;
         i += (uint64_t)gridDim.x * blockDim.x)
        mx = max(mx, max(a[i], b[i]));
    for (int o = 16; o; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, mx);
}

__global__ void k_make_keys(const uint32_t *src, const uint32_t *dst, uint64_t m, int bits,
                            bool both, bool drop_loops, unsigned long long *keys,
                            unsigned long long *n_out)
{
    // Warp-uniform trip count: blockDim is a multiple of 32, so every lane of
    // a warp runs the same iterations and the full-mask scan below is legal.
    const unsigned lane = threadIdx.x & 31;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i0 = blockIdx.x * (uint64_t)blockDim.x + (threadIdx.x & ~31u); i0 < m; i0 += stride) {
        const uint64_t i = i0 + lane;
        const bool valid = i < m;
        const uint64_t u = valid ? src[i] : 0, v = valid ? dst[i] : 0;
        const bool keep = valid && !(drop_loops && u == v);
        const unsigned nk = keep ? (both ? 2u : 1u) : 0u;
        // Warp-aggregated slot reservation keeps the output dense.
        unsigned incl = nk;
        for (int o = 1; o < 32; o <<= 1) {
            unsigned t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= (unsigned)o) incl += t;
        }
        const unsigned total = __shfl_sync(0xffffffffu, incl, 31);
        unsigned long long base = 0;
        if (lane == 31 && total) base = atomicAdd(n_out, (unsigned long long)total);
        base = __shfl_sync(0xffffffffu, base, 31);
        const uint64_t pos = base + incl - nk;
        if (nk >= 1) keys[pos] = (u << bits) | v;
        if (nk == 2) keys[pos + 1] = (v << bits) | u;
    }
}

__global__ void k_split_keys(const unsigned long long *keys, uint64_t m, int bits, uint32_t *s,
                             uint32_t *d)
{
    const unsigned long long mask = (1ull << bits) - 1;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m;
         i += (uint64_t)gridDim.x * blockDim.x) {
        s[i] = (uint32_t)(keys[i] >> bits);
        d[i] = (uint32_t)(keys[i] & mask);
    }
}

__device__ __forceinline__ uint32_t lower_bound_u32(const uint32_t *a, uint32_t n, uint32_t x)
{
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        uint32_t mid = lo + ((hi - lo) >> 1);
        if (a[mid] < x) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Names -> canonical indices, in place.
__global__ void k_to_index(uint32_t *x, uint64_t m, const uint32_t *names, uint32_t n)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m;
         i += (uint64_t)gridDim.x * blockDim.x)
        x[i] = lower_bound_u32(names, n, x[i]);
}

// Row bounds from the sorted source indices, without atomics (a hub of
// degree d would otherwise serialise d atomics on one counter): the first
// entry of a run of v records first[v], the last records end[v].
__global__ void k_row_bounds(const uint32_t *si, uint64_t m, uint32_t *first, uint32_t *end)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t v = si[i];
        if (i == 0 || si[i - 1] != v) first[v] = (uint32_t)i;
        if (i + 1 == m || si[i + 1] != v) end[v] = (uint32_t)(i + 1);
    }
}

// deg[v] = end[v] - first[v] in place (both 0 for a vertex without out-edges).
__global__ void k_degree_from_bounds(uint32_t *end_deg, const uint32_t *first, uint32_t n)
{
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n; v += (uint64_t)gridDim.x * blockDim.x)
        end_deg[v] -= first[v];
}

__global__ void k_iota(uint32_t *x, uint32_t n)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        x[i] = i;
}

// order[i] = canonical index of internal vertex i.
__global__ void k_relabel(const uint32_t *order, const uint32_t *deg_idx, const uint32_t *names,
                          uint32_t n, uint32_t *idx2int, uint32_t *int_deg, uint32_t *int2name)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t idx = order[i];
        idx2int[idx] = i;
        int_deg[i] = deg_idx[idx];
        int2name[i] = names[idx];
    }
}

__global__ void k_adj(const uint32_t *int_deg, const uint32_t *int_off, uint32_t n, uint2 *adj)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        adj[i] = make_uint2(int_off[i], int_deg[i]);
}

// Scatter canonical edges into internal rows.  Edge e belongs to canonical
// row si[e]; its rank inside the row is e - row_ptr[si[e]].
__global__ void k_fill_col(const uint32_t *si, const uint32_t *di, const uint32_t *row_ptr,
                           uint64_t m, const uint32_t *idx2int, const uint2 *adj, uint32_t *col)
{
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < m;
         e += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t s = si[e];
        const uint32_t r = (uint32_t)(e - row_ptr[s]);
        col[adj[idx2int[s]].x + r] = idx2int[di[e]];
    }
}

// Canonical export: one warp per internal row.
__global__ void k_export(const uint2 *adj, const uint32_t *col, const uint32_t *int2idx,
                         const uint32_t *canon_off, uint32_t n, uint32_t *out_col)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t warps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t i = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; i < n; i += warps) {
        const uint2 a = adj[i];
        const uint32_t base = canon_off[int2idx[i]];
        for (uint32_t r = lane; r < a.y; r += 32) out_col[base + r] = int2idx[col[a.x + r]];
    }
}

__global__ void k_deg_by_index(const uint2 *adj, const uint32_t *idx2int, uint32_t n, uint32_t *deg)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        deg[i] = adj[idx2int[i]].y;
}

__global__ void k_rmat(uint32_t scale, uint64_t m, uint32_t ta, uint32_t tab, uint32_t tabc,
                       uint32_t k0, uint32_t k1, uint32_t *src, uint32_t *dst)
{
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < m;
         e += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t u = 0, v = 0;
        uint4 w = make_uint4(0, 0, 0, 0);
        for (uint32_t l = 0; l < scale; ++l) {
            if ((l & 3u) == 0)
                w = philox(make_uint4((uint32_t)e, (uint32_t)(e >> 32), l >> 2, PTW_TAG_RMAT), k0, k1);
            const uint32_t x = (l & 3u) == 0 ? w.x : (l & 3u) == 1 ? w.y : (l & 3u) == 2 ? w.z : w.w;
            const uint32_t rb = x >= tab;
            const uint32_t cb = (x >= ta && x < tab) || x >= tabc;
            u = (u << 1) | rb;
            v = (v << 1) | cb;
        }
        src[e] = u;
        dst[e] = v;
    }
}

// Chung-Lu: vertex i has weight (i + 1)^(-expo), expo = 1 / (gamma - 1);
// both endpoints of an edge are drawn proportionally to weight by inverse
// CDF (binary search over the inclusive prefix sums).
__global__ void k_cl_weights(uint32_t n, double expo, double *w)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        w[i] = pow((double)i + 1.0, -expo);
}

__device__ __forceinline__ uint32_t cdf_pick(const double *cdf, uint32_t n, double x)
{
    uint32_t lo = 0, hi = n - 1;  // first i with cdf[i] > x
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (cdf[mid] > x) hi = mid;
        else lo = mid + 1;
    }
    return lo;
}

__global__ void k_cl_edges(uint64_t m, const double *cdf, uint32_t n, uint32_t k0, uint32_t k1, uint32_t *src,
                           uint32_t *dst)
{
    const double total = cdf[n - 1];
    const double inv53 = 1.0 / 9007199254740992.0;  // 2^-53
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < m;
         e += (uint64_t)gridDim.x * blockDim.x) {
        const uint4 r = philox(make_uint4((uint32_t)e, (uint32_t)(e >> 32), 0u, PTW_TAG_CHUNGLU), k0, k1);
        const double u1 = (double)(((uint64_t)(r.x >> 5) << 26) | (r.y >> 6)) * inv53;
        const double u2 = (double)(((uint64_t)(r.z >> 5) << 26) | (r.w >> 6)) * inv53;
        src[e] = cdf_pick(cdf, n, u1 * total);
        dst[e] = cdf_pick(cdf, n, u2 * total);
    }
}

// CSR -> (src, dst) names, one thread per entry.  The row of entry e is the
// largest r with row_ptr[r] <= e (row_ptr is validated non-decreasing with
// row_ptr[0] = 0 and row_ptr[n] = m on the host, so the search invariant
// row_ptr[lo] <= e < row_ptr[hi] holds from lo = 0, hi = n).  A column index
// >= n raises *bad and writes name 0 so the arrays stay defined.
__global__ void k_csr_to_edges(const uint64_t *row_ptr, const uint32_t *col, const uint32_t *names,
                               uint32_t n, uint64_t m, uint32_t *src, uint32_t *dst, unsigned *bad)
{
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < m;
         e += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t lo = 0, hi = n;
        while (hi - lo > 1) {
            const uint32_t mid = lo + (hi - lo) / 2;
            if (row_ptr[mid] <= e) lo = mid;
            else hi = mid;
        }
        const uint32_t c = col[e];
        if (c >= n) {
            atomicOr(bad, 1u);
            src[e] = dst[e] = 0;
            continue;
        }
        src[e] = names ? names[lo] : lo;
        dst[e] = names ? names[c] : c;
    }
}

// Raises *bad when two neighbours of a sorted array are equal.
__global__ void k_adjacent_equal(const uint32_t *x, uint32_t n, unsigned *bad)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i + 1 < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        if (x[i] == x[i + 1]) atomicOr(bad, 2u);
}

// Frees every pointer on scope exit (stream-ordered).
struct AsyncBufs {
    cudaStream_t st;
    std::vector<void *> ptrs;
    explicit AsyncBufs(cudaStream_t s) : st(s) {}
    template <typename T> cudaError_t alloc(T **p, uint64_t count)
    {
        void *q = nullptr;
        cudaError_t e = cudaMallocAsync(&q, std::max<uint64_t>(count, 1) * sizeof(T), st);
        if (e == cudaSuccess) ptrs.push_back(q);
        *p = (T *)q;
        return e;
    }
    void release(void *p)
    {
        for (auto &q : ptrs)
            if (q == p) {
                cudaFreeAsync(q, st);
                q = nullptr;
            }
    }
    ~AsyncBufs()
    {
        for (void *q : ptrs)
            if (q) cudaFreeAsync(q, st);
    }
};

template <typename F> cudaError_t cub_call(F f, cudaStream_t st)
{
    size_t bytes = 0;
    cudaError_t e = f(nullptr, bytes);
    if (e != cudaSuccess) return e;
    void *tmp = nullptr;
    e = cudaMallocAsync(&tmp, std::max<size_t>(bytes, 16), st);
    if (e != cudaSuccess) return e;
    e = f(tmp, bytes);
    cudaFreeAsync(tmp, st);
    return e;
}

int bits_for(uint64_t bound)
{
    int b = 1;
    while (b < 32 && (1ull << b) < bound) ++b;
    return b;
}

}  // namespace

int graph_init_handle(ptw_graph *g)
{
    PTW_CUDA(cudaGetDevice(&g->device));
    PTW_CUDA(cudaDeviceGetAttribute(&g->num_sms, cudaDevAttrMultiProcessorCount, g->device));
    PTW_CUDA(cudaStreamCreateWithFlags(&g->own_stream, cudaStreamNonBlocking));
    g->stream = g->own_stream;
    for (auto &e : g->ev) PTW_CUDA(cudaEventCreate(&e));
    g->tune.block = 256;
    g->tune.ilp = 2;
    g->tune.chunk = 256;
    g->tune.hot_k = 0;
    g->tune.blocks_per_sm = 0;
    g->tune.min_blocks = 0;
    g->tune.paths_ilp = 2;
    g->tune.cache_hints = 1;
    g->tune.paths_named = 1;
    return PTW_OK;
}

void graph_release(ptw_graph *g)
{
    if (!g) return;
    if (g->stream) cudaStreamSynchronize(g->stream);
    cudaFree(g->dg.adj);
    cudaFree(g->dg.col);
    cudaFree(g->dg.int2name);
    cudaFree(g->dg.idx2int);
    cudaFree(g->dg.int2idx);
    cudaFree(g->dg.names);
    cudaFree(g->dg.col_named);
    cudaFree(g->dg.col_ext);
    cudaFree(g->dg.vtx_ext);
    cudaFree(g->dg.edge_filter);
    cudaFree(g->sc.counts);
    cudaFree(g->sc.ctrl);
    cudaFree(g->sc.sources);
    cudaFree(g->sc.by_name);
    cudaFree(g->sc.out_stage);
    for (auto &e : g->ev)
        if (e) cudaEventDestroy(e);
    if (g->copy_stream) cudaStreamSynchronize(g->copy_stream);
    for (ptw::AsyncSlot &a : g->async) {
        cudaFree(a.by_name);
        cudaFreeHost(a.h_moves);
        for (cudaEvent_t e : {a.ev_start, a.ev_walk, a.ev_copy})
            if (e) cudaEventDestroy(e);
    }
    if (g->copy_stream) cudaStreamDestroy(g->copy_stream);
    if (g->own_stream) cudaStreamSynchronize(g->own_stream);
    if (g->own_stream) cudaStreamDestroy(g->own_stream);
    delete[] g->h_names;
    delete[] g->h_idx2int;
}

int rmat_generate_device(uint32_t scale, uint64_t m, uint32_t ta, uint32_t tab, uint32_t tabc,
                         uint64_t seed, uint32_t *d_src, uint32_t *d_dst, cudaStream_t st)
{
    k_rmat<<<grid_for(m), kThreads, 0, st>>>(scale, m, ta, tab, tabc, (uint32_t)seed,
                                             (uint32_t)(seed >> 32), d_src, d_dst);
    PTW_CUDA(cudaGetLastError());
    return PTW_OK;
}

int chung_lu_generate_device(uint32_t n, double gamma, uint64_t m, uint64_t seed, uint32_t *d_src,
                             uint32_t *d_dst, cudaStream_t st)
{
    AsyncBufs tmp(st);
    double *w = nullptr, *cdf = nullptr;
    PTW_CUDA(tmp.alloc(&w, n));
    PTW_CUDA(tmp.alloc(&cdf, n));
    k_cl_weights<<<grid_for(n), kThreads, 0, st>>>(n, 1.0 / (gamma - 1.0), w);
    PTW_CUDA(cub_call([&](void *t, size_t &b) {
        return cub::DeviceScan::InclusiveSum(t, b, w, cdf, (int64_t)n, st);
    }, st));
    k_cl_edges<<<grid_for(m), kThreads, 0, st>>>(m, cdf, n, (uint32_t)seed, (uint32_t)(seed >> 32), d_src, d_dst);
    PTW_CUDA(cudaGetLastError());
    PTW_CUDA(cudaStreamSynchronize(st));
    return PTW_OK;
}

int csr_to_device_edges(const uint64_t *h_row_ptr, const uint32_t *h_col, const uint32_t *h_names,
                        uint32_t n, uint32_t **d_src, uint32_t **d_dst, cudaStream_t st)
{
    *d_src = *d_dst = nullptr;
    const uint64_t m = h_row_ptr[n];
    AsyncBufs tmp(st);
    uint64_t *row = nullptr;
    uint32_t *col = nullptr, *names = nullptr, *src = nullptr, *dst = nullptr;
    unsigned *bad = nullptr;
    PTW_CUDA(tmp.alloc(&row, (uint64_t)n + 1));
    PTW_CUDA(tmp.alloc(&col, m));
    PTW_CUDA(tmp.alloc(&bad, 1));
    PTW_CUDA(cudaMemsetAsync(bad, 0, sizeof(unsigned), st));
    PTW_CUDA(cudaMemcpyAsync(row, h_row_ptr, ((uint64_t)n + 1) * 8, cudaMemcpyHostToDevice, st));
    PTW_CUDA(cudaMemcpyAsync(col, h_col, m * 4, cudaMemcpyHostToDevice, st));
    if (h_names) {
        uint32_t *sorted = nullptr;
        PTW_CUDA(tmp.alloc(&names, n));
        PTW_CUDA(tmp.alloc(&sorted, n));
        PTW_CUDA(cudaMemcpyAsync(names, h_names, (uint64_t)n * 4, cudaMemcpyHostToDevice, st));
        PTW_CUDA(cub_call([&](void *t, size_t &b) {
            return cub::DeviceRadixSort::SortKeys(t, b, names, sorted, (int64_t)n, 0, 32, st);
        }, st));
        k_adjacent_equal<<<grid_for(n), kThreads, 0, st>>>(sorted, n, bad);
        tmp.release(sorted);
    }
    // The edge arrays are handed to the caller, so they are not in tmp.
    PTW_CUDA(cudaMallocAsync(&src, std::max<uint64_t>(m, 1) * 4, st));
    cudaError_t e = cudaMallocAsync(&dst, std::max<uint64_t>(m, 1) * 4, st);
    if (e != cudaSuccess) {
        cudaFreeAsync(src, st);
        return cuda_fail(e, "CSR edge buffers");
    }
    k_csr_to_edges<<<grid_for(m), kThreads, 0, st>>>(row, col, names, n, m, src, dst, bad);
    unsigned h_bad = 0;
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h_bad, bad, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess || h_bad) {
        cudaFreeAsync(src, st);
        cudaFreeAsync(dst, st);
        if (e != cudaSuccess) return cuda_fail(e, "CSR expansion");
        return fail(PTW_EINVAL, (h_bad & 1) ? "CSR column index >= n" : "CSR vertex names are not distinct");
    }
    *d_src = src;
    *d_dst = dst;
    return PTW_OK;
}

int build_graph_from_device_edges(ptw_graph *g, uint32_t *d_src, uint32_t *d_dst, uint64_t m,
                                  bool as_undirected, bool clean, bool compact_names)
{
    cudaStream_t st = g->stream;
    AsyncBufs tmp(st);
    if (m == 0) return fail(PTW_EINVAL, "edge list is empty");

    // Name range -> key packing width.
    unsigned *d_max = nullptr;
    PTW_CUDA(tmp.alloc(&d_max, 1));
    PTW_CUDA(cudaMemsetAsync(d_max, 0, sizeof(unsigned), st));
    k_max2<<<grid_for(m), kThreads, 0, st>>>(d_src, d_dst, m, d_max);
    unsigned h_max = 0;
    PTW_CUDA(cudaMemcpyAsync(&h_max, d_max, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    PTW_CUDA(cudaStreamSynchronize(st));
    const uint64_t id_bound = (uint64_t)h_max + 1;
    const int bits = bits_for(id_bound);

    // Packed keys, optionally symmetrised / without self-loops.
    const uint64_t cap = as_undirected ? 2 * m : m;
    unsigned long long *keys = nullptr, *keys_alt = nullptr, *d_cnt = nullptr;
    PTW_CUDA(tmp.alloc(&keys, cap));
    PTW_CUDA(tmp.alloc(&d_cnt, 2));
    PTW_CUDA(cudaMemsetAsync(d_cnt, 0, 2 * sizeof(unsigned long long), st));
    k_make_keys<<<grid_for(m), kThreads, 0, st>>>(d_src, d_dst, m, bits, as_undirected, clean, keys,
                                                  d_cnt);
    PTW_CUDA(cudaGetLastError());
    unsigned long long h_cnt = 0;
    PTW_CUDA(cudaMemcpyAsync(&h_cnt, d_cnt, sizeof(h_cnt), cudaMemcpyDeviceToHost, st));
    PTW_CUDA(cudaStreamSynchronize(st));
    cudaFreeAsync(d_src, st);
    cudaFreeAsync(d_dst, st);
    uint64_t mm = h_cnt;
    if (mm == 0) return fail(PTW_EINVAL, "graph has no edges after clean-up");
    if (mm >= (1ull << 32)) return fail(PTW_EINVAL, "graphs with 2^32 or more CSR entries are not supported");

    PTW_CUDA(tmp.alloc(&keys_alt, mm));
    {
        cub::DoubleBuffer<unsigned long long> db(keys, keys_alt);
        PTW_CUDA(cub_call([&](void *t, size_t &b) {
            return cub::DeviceRadixSort::SortKeys(t, b, db, (int64_t)mm, 0, 2 * bits, st);
        }, st));
        if (db.Current() != keys) std::swap(keys, keys_alt);
    }
    if (clean) {
        PTW_CUDA(cub_call([&](void *t, size_t &b) {
            return cub::DeviceSelect::Unique(t, b, keys, keys_alt, d_cnt + 1, (int64_t)mm, st);
        }, st));
        PTW_CUDA(cudaMemcpyAsync(&h_cnt, d_cnt + 1, sizeof(h_cnt), cudaMemcpyDeviceToHost, st));
        PTW_CUDA(cudaStreamSynchronize(st));
        std::swap(keys, keys_alt);
        mm = h_cnt;
    }
    tmp.release(keys_alt);

    // Split into (src, dst) names, then the sorted unique name set.
    uint32_t *si = nullptr, *di = nullptr, *nm = nullptr, *nm_alt = nullptr;
    PTW_CUDA(tmp.alloc(&si, mm));
    PTW_CUDA(tmp.alloc(&di, mm));
    k_split_keys<<<grid_for(mm), kThreads, 0, st>>>(keys, mm, bits, si, di);
    tmp.release(keys);
    PTW_CUDA(tmp.alloc(&nm, 2 * mm));
    PTW_CUDA(tmp.alloc(&nm_alt, 2 * mm));
    PTW_CUDA(cudaMemcpyAsync(nm, si, mm * 4, cudaMemcpyDeviceToDevice, st));
    PTW_CUDA(cudaMemcpyAsync(nm + mm, di, mm * 4, cudaMemcpyDeviceToDevice, st));
    {
        cub::DoubleBuffer<uint32_t> db(nm, nm_alt);
        PTW_CUDA(cub_call([&](void *t, size_t &b) {
            return cub::DeviceRadixSort::SortKeys(t, b, db, (int64_t)(2 * mm), 0, bits, st);
        }, st));
        if (db.Current() != nm) std::swap(nm, nm_alt);
    }
    PTW_CUDA(cub_call([&](void *t, size_t &b) {
        return cub::DeviceSelect::Unique(t, b, nm, nm_alt, d_cnt + 1, (int64_t)(2 * mm), st);
    }, st));
    PTW_CUDA(cudaMemcpyAsync(&h_cnt, d_cnt + 1, sizeof(h_cnt), cudaMemcpyDeviceToHost, st));
    PTW_CUDA(cudaStreamSynchronize(st));
    const uint32_t n = (uint32_t)h_cnt;
    uint32_t *names = nm_alt;  // [n] ascending
    tmp.release(nm);

    k_to_index<<<grid_for(mm), kThreads, 0, st>>>(si, mm, names, n);
    k_to_index<<<grid_for(mm), kThreads, 0, st>>>(di, mm, names, n);
    if (compact_names) k_iota<<<grid_for(n), kThreads, 0, st>>>(names, n);
    PTW_CUDA(cudaGetLastError());

    // Degrees and canonical row offsets (u32: mm < 2^32).
    uint32_t *deg = nullptr, *row_ptr = nullptr;
    PTW_CUDA(tmp.alloc(&deg, n + 1));
    PTW_CUDA(tmp.alloc(&row_ptr, n + 1));
    PTW_CUDA(cudaMemsetAsync(deg, 0, (n + 1) * 4ull, st));
    {
        uint32_t *first = nullptr;
        PTW_CUDA(tmp.alloc(&first, n));
        PTW_CUDA(cudaMemsetAsync(first, 0, n * 4ull, st));
        k_row_bounds<<<grid_for(mm), kThreads, 0, st>>>(si, mm, first, deg);
        k_degree_from_bounds<<<grid_for(n), kThreads, 0, st>>>(deg, first, n);
        tmp.release(first);
    }
    PTW_CUDA(cub_call([&](void *t, size_t &b) {
        return cub::DeviceScan::ExclusiveSum(t, b, deg, row_ptr, (int64_t)n + 1, st);
    }, st));

    // Internal order: stable sort of canonical indices by descending degree.
    uint32_t *deg_keys = nullptr, *deg_keys_out = nullptr, *iota = nullptr, *order = nullptr;
    PTW_CUDA(tmp.alloc(&deg_keys_out, n));
    PTW_CUDA(tmp.alloc(&iota, n));
    PTW_CUDA(tmp.alloc(&order, n));
    deg_keys = deg;
    k_iota<<<grid_for(n), kThreads, 0, st>>>(iota, n);
    PTW_CUDA(cub_call([&](void *t, size_t &b) {
        return cub::DeviceRadixSort::SortPairsDescending(t, b, deg_keys, deg_keys_out, iota, order,
                                                         (int64_t)n, 0, 32, st);
    }, st));
    uint32_t h_maxdeg = 0;
    PTW_CUDA(cudaMemcpyAsync(&h_maxdeg, deg_keys_out, 4, cudaMemcpyDeviceToHost, st));

    DeviceGraph &dg = g->dg;
    dg.n = n;
    dg.m = mm;
    dg.id_bound = compact_names ? n : (uint32_t)id_bound;
    PTW_CUDA(device_malloc(&dg.adj, (uint64_t)n * sizeof(uint2)));
    PTW_CUDA(device_malloc(&dg.col, mm * 4));
    PTW_CUDA(device_malloc(&dg.int2name, (uint64_t)n * 4));
    PTW_CUDA(device_malloc(&dg.idx2int, (uint64_t)n * 4));
    PTW_CUDA(device_malloc(&dg.int2idx, (uint64_t)n * 4));
    PTW_CUDA(cudaMemcpyAsync(dg.int2idx, order, (uint64_t)n * 4, cudaMemcpyDeviceToDevice, st));
    PTW_CUDA(device_malloc(&dg.names, (uint64_t)n * 4));
    PTW_CUDA(cudaMemcpyAsync(dg.names, names, (uint64_t)n * 4, cudaMemcpyDeviceToDevice, st));
    uint32_t *int_deg = iota;  // reuse
    k_relabel<<<grid_for(n), kThreads, 0, st>>>(order, deg, names, n, dg.idx2int, int_deg,
                                                dg.int2name);
    uint32_t *int_off = deg_keys_out;  // reuse
    PTW_CUDA(cub_call([&](void *t, size_t &b) {
        return cub::DeviceScan::ExclusiveSum(t, b, int_deg, int_off, (int64_t)n, st);
    }, st));
    k_adj<<<grid_for(n), kThreads, 0, st>>>(int_deg, int_off, n, dg.adj);
    k_fill_col<<<grid_for(mm), kThreads, 0, st>>>(si, di, row_ptr, mm, dg.idx2int, dg.adj, dg.col);
    PTW_CUDA(cudaGetLastError());

    // Host copy of the ascending names for source lookups.
    g->h_names = new (std::nothrow) uint32_t[n];
    if (!g->h_names) return fail(PTW_ENOMEM, "host allocation of the name table failed");
    PTW_CUDA(cudaMemcpyAsync(g->h_names, names, (uint64_t)n * 4, cudaMemcpyDeviceToHost, st));
    g->h_idx2int = new (std::nothrow) uint32_t[n];
    if (!g->h_idx2int) return fail(PTW_ENOMEM, "host allocation of the index table failed");
    PTW_CUDA(cudaMemcpyAsync(g->h_idx2int, dg.idx2int, (uint64_t)n * 4, cudaMemcpyDeviceToHost, st));

    // Scratch reused by every walk.
    PTW_CUDA(device_malloc(&g->sc.counts, (uint64_t)n * 4));
    PTW_CUDA(device_malloc(&g->sc.ctrl, 8 * sizeof(unsigned long long)));
    PTW_CUDA(cudaMemsetAsync(g->sc.ctrl, 0, 8 * sizeof(unsigned long long), st));  // [7]: index checks
    PTW_CUDA(cudaStreamSynchronize(st));
    dg.max_degree = h_maxdeg;
    // symmetrised, self-loops dropped and duplicates removed: simple and
    // symmetric by construction (node2vec then skips its check)
    dg.simple_symmetric = as_undirected && clean ? 1 : -1;
    g->device_bytes = (uint64_t)n * (8 + 4 * 4 + 4) + mm * 4 + 64;
    return PTW_OK;
}

}  // namespace ptw

using namespace ptw;

extern "C" int ptw_graph_get_info(const ptw_graph *g, ptw_graph_info *info)
try {
    if (!g || !info) return fail(PTW_EINVAL, "null argument");
    info->n_vertices = g->dg.n;
    info->id_bound = g->dg.id_bound;
    info->n_edges = g->dg.m;
    info->max_degree = g->dg.max_degree;
    info->reserved = 0;
    info->device_bytes = g->device_bytes;
    return PTW_OK;
} catch (...) {
    return host_exception();
}

extern "C" int ptw_graph_export_csr(const ptw_graph *g, uint32_t *h_names, uint64_t *h_row_ptr,
                                    uint32_t *h_col)
try {
    if (!g) return fail(PTW_EINVAL, "null graph");
    const DeviceGraph &dg = g->dg;
    cudaStream_t st = g->stream;
    PTW_CUDA(cudaSetDevice(g->device));
    AsyncBufs tmp(st);
    uint32_t *deg = nullptr, *off = nullptr;
    PTW_CUDA(tmp.alloc(&deg, dg.n + 1));
    PTW_CUDA(tmp.alloc(&off, dg.n + 1));
    PTW_CUDA(cudaMemsetAsync(deg + dg.n, 0, 4, st));
    k_deg_by_index<<<grid_for(dg.n), kThreads, 0, st>>>(dg.adj, dg.idx2int, dg.n, deg);
    PTW_CUDA(cub_call([&](void *t, size_t &b) {
        return cub::DeviceScan::ExclusiveSum(t, b, deg, off, (int64_t)dg.n + 1, st);
    }, st));
    if (h_row_ptr) {
        std::vector<uint32_t> tmp_off(dg.n + 1);
        PTW_CUDA(cudaMemcpyAsync(tmp_off.data(), off, (dg.n + 1) * 4ull, cudaMemcpyDeviceToHost, st));
        PTW_CUDA(cudaStreamSynchronize(st));
        for (uint64_t i = 0; i <= dg.n; ++i) h_row_ptr[i] = tmp_off[i];
    }
    if (h_col) {
        uint32_t *c = nullptr;
        PTW_CUDA(tmp.alloc(&c, dg.m));
        k_export<<<grid_for((uint64_t)dg.n * 32), kThreads, 0, st>>>(dg.adj, dg.col, dg.int2idx, off,
                                                                    dg.n, c);
        PTW_CUDA(cudaGetLastError());
        PTW_CUDA(cudaMemcpyAsync(h_col, c, dg.m * 4, cudaMemcpyDeviceToHost, st));
    }
    if (h_names) std::memcpy(h_names, g->h_names, (uint64_t)dg.n * 4);
    PTW_CUDA(cudaStreamSynchronize(st));
    return PTW_OK;
} catch (...) {
    return host_exception();
}

extern "C" int ptw_graph_export_edges(const ptw_graph *g, uint32_t *h_src, uint32_t *h_dst)
try {
    if (!g || !h_src || !h_dst) return fail(PTW_EINVAL, "null argument");
    const DeviceGraph &dg = g->dg;
    std::vector<uint64_t> rp(dg.n + 1);
    int rc = ptw_graph_export_csr(g, nullptr, rp.data(), h_dst);
    if (rc) return rc;
    for (uint32_t i = 0; i < dg.n; ++i)
        for (uint64_t e = rp[i]; e < rp[i + 1]; ++e) h_src[e] = g->h_names[i];
    for (uint64_t e = 0; e < dg.m; ++e) h_dst[e] = g->h_names[h_dst[e]];
    return PTW_OK;
} catch (...) {
    return host_exception();
}

extern "C" int ptw_graph_sync(ptw_graph *g)
try {
    if (!g) return fail(PTW_EINVAL, "null graph");
    PTW_CUDA(cudaStreamSynchronize(g->stream));
    return PTW_OK;
} catch (...) {
    return host_exception();
}

extern "C" int ptw_graph_set_stream(ptw_graph *g, void *cuda_stream)
try {
    if (!g) return fail(PTW_EINVAL, "null graph");
    cudaStream_t s = cuda_stream ? (cudaStream_t)cuda_stream : g->own_stream;
    if (s != g->stream) {
        // Work already queued on the old stream completes before the switch.
        PTW_CUDA(cudaStreamSynchronize(g->stream));
    }
    g->stream = s;
    return PTW_OK;
} catch (...) {
    return host_exception();
}
