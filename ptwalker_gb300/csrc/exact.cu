// FP64 expected-count oracle on the device (K8 power iteration, K7 L1).
//
// For a source s and stop probability sp, with P = D^-1 A over out-edges,
//   pi_s = sp * sum_{k>=0} (1-sp)^k e_s^T P^k        (textbook PPR)
//   visits:   E[c | s] = pi_s / (sp (1-sp)) - sp/(1-sp) e_s
//   endpoint: E[end | s] = (pi_s - sp e_s) / (1-sp)
// which restates the walk semantics of src/core/solver.hpp:242-263 /
// :284-306 with the geometric length of src/core/pagerank.cpp:41-68.
// 32 sources are iterated together, one per lane: term_{k+1}[v] =
// (1-sp) * sum_{u -> v} term_k[u] / deg(u), a pull over the transposed CSR,
// so every sum is taken in a fixed order (deterministic FP64).  The iterate
// is stored divided by the out-degree of its vertex, so a pull adds rows
// without a per-edge multiply.  Iteration stops when sp * (mass of the new
// term) < tol for every source; the L1 error of the truncated series is then
// at most about 2 tol.
//
// L1 terms are summed on the device: result entries (names) map to
// internal ids through a dense name -> id table, and each query's terms are
// reduced over its entries.  Several batches over the same sources share
// one power iteration (ptw_batch_l1_many); two batches over the same
// sources are compared with each other through a dense per-query scratch
// row (ptw_batch_l1_pair).
#include <cub/cub.cuh>

#include <algorithm>
#include <vector>

#include "ptw_internal.cuh"

namespace ptw {
namespace {

constexpr int K = 32;

__global__ void k_transpose_keys(const uint2 *adj, const uint32_t *col, uint32_t n, unsigned long long *keys)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t warps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t u = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; u < n; u += warps) {
        const uint2 a = adj[u];
        for (uint32_t r = lane; r < a.y; r += 32)
            keys[a.x + r] = ((unsigned long long)col[a.x + r] << 32) | (uint32_t)u;
    }
}

__global__ void k_split_t(const unsigned long long *keys, uint64_t m, uint32_t *tcol, uint32_t *tdeg)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m; i += (uint64_t)gridDim.x * blockDim.x) {
        tcol[i] = (uint32_t)keys[i];
        atomicAdd(&tdeg[keys[i] >> 32], 1u);
    }
}

__global__ void k_inv_deg(const uint2 *adj, uint32_t n, double *inv)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        inv[i] = adj[i].y ? 1.0 / (double)adj[i].y : 0.0;
}

// x holds term_k[u][q] / deg(u).  term_{k+1}[v][q] = f * sum_{u in in(v)} x[u][q];
// xn[v][q] = term_{k+1}[v][q] / deg(v);  acc[v][q] += sp * term_{k+1}[v][q];
// mass[q] += sum_v term_{k+1}[v][q]  (block-reduced).
//
// Work is cut into segments of at most kSegEdges in-edges, one warp per
// segment, so a hub's in-list (millions of edges on a power-law graph) is
// spread over many warps instead of holding one warp for the whole
// iteration.  A vertex with one segment is finished by its warp; the
// segments of a vertex with several write partial sums, which k_pull_heavy
// adds in segment order (a fixed order: the sum is deterministic).
constexpr uint32_t kSegEdges = 2048;
constexpr uint32_t kNoPart = 0xFFFFFFFFu;

__device__ __forceinline__ double segment_sum(const uint32_t *tcol, const double *x, uint32_t e0, uint32_t e1,
                                              uint32_t lane)
{
    // four independent partial sums keep four row loads and adds in flight
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    uint32_t e = e0;
    for (; e + 4 <= e1; e += 4) {
        const uint32_t u0 = tcol[e], u1 = tcol[e + 1], u2 = tcol[e + 2], u3 = tcol[e + 3];
        s0 += x[(uint64_t)u0 * K + lane];
        s1 += x[(uint64_t)u1 * K + lane];
        s2 += x[(uint64_t)u2 * K + lane];
        s3 += x[(uint64_t)u3 * K + lane];
    }
    for (; e < e1; ++e) s0 += x[(uint64_t)tcol[e] * K + lane];
    return (s0 + s1) + (s2 + s3);
}

// Adds each lane's `local` over the block into mass[lane] (8 warps per block).
__device__ __forceinline__ void mass_flush(double local, double *mass)
{
    __shared__ double part[8][K];
    const uint32_t lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    part[wib][lane] = local;
    __syncthreads();
    if (wib == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += part[w][lane];
        atomicAdd(&mass[lane], t);
    }
}

// seg_v[s], [seg_e0[s], seg_e1[s]) = the vertex and in-edge range of segment
// s; seg_part[s] = its partial-sum slot, or kNoPart for a vertex's only segment.
__global__ void k_pull(const uint32_t *seg_v, const uint32_t *seg_e0, const uint32_t *seg_e1,
                       const uint32_t *seg_part, uint64_t nseg, const uint32_t *tcol, const double *inv,
                       const double *x, double *xn, double *acc, double *partial, double f, double sp,
                       double *mass)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t warps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    double local = 0.0;
    for (uint64_t sg = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; sg < nseg; sg += warps) {
        const double s = segment_sum(tcol, x, seg_e0[sg], seg_e1[sg], lane);
        const uint32_t p = seg_part[sg];
        if (p != kNoPart) {
            partial[(uint64_t)p * K + lane] = s;
            continue;
        }
        const uint64_t v = seg_v[sg];
        const double t = s * f;
        xn[v * K + lane] = t * inv[v];
        acc[v * K + lane] += sp * t;
        local += t;
    }
    mass_flush(local, mass);
}

// Vertices with several segments: heavy_v[h], partial slots
// [heavy_p0[h], heavy_p0[h + 1]) added in order.
__global__ void k_pull_heavy(const uint32_t *heavy_v, const uint32_t *heavy_p0, uint32_t nheavy, const double *inv,
                             const double *partial, double *xn, double *acc, double f, double sp, double *mass)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    double local = 0.0;
    for (uint32_t h = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; h < nheavy; h += warps) {
        double s = 0.0;
        for (uint32_t p = heavy_p0[h]; p < heavy_p0[h + 1]; ++p) s += partial[(uint64_t)p * K + lane];
        const uint64_t v = heavy_v[h];
        const double t = s * f;
        xn[v * K + lane] = t * inv[v];
        acc[v * K + lane] += sp * t;
        local += t;
    }
    mass_flush(local, mass);
}

// column sums of acc
__global__ void k_colsum(const double *acc, uint32_t n, double *sum)
{
    __shared__ double part[8][K];
    const uint32_t lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const uint64_t warps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    double local = 0.0;
    for (uint64_t v = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; v < n; v += warps)
        local += acc[v * K + lane];
    part[wib][lane] = local;
    __syncthreads();
    if (wib == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += part[w][lane];
        atomicAdd(&sum[lane], t);
    }
}

// map[name] = internal id of every vertex (the rest of [0, id_bound) is
// left as set by the caller).
__global__ void k_name_map(const uint32_t *names, const uint32_t *idx2int, uint32_t n, uint32_t *map)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        map[names[i]] = idx2int[i];
}

// C[k] = sum of the counts of query k's entries [off[k], off[k+1]) (grid y = k).
__global__ void k_count_sum(const unsigned long long *off, const uint32_t *cnt, unsigned long long *C)
{
    const uint32_t k = blockIdx.y;
    unsigned long long s = 0;
    for (uint64_t i = off[k] + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < off[k + 1];
         i += (uint64_t)gridDim.x * blockDim.x)
        s += cnt[i];
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0 && s) atomicAdd(&C[k], s);
}

// For query k of a group (column k of acc, source src[k]): over its entries,
// terms[2k] += e_v / E[k] and terms[2k+1] += |c_v / C[k] - e_v / E[k]|, with
// e from acc (= pi) per the app.
__global__ void k_l1_terms(const double *acc, const uint32_t *src, const unsigned long long *off,
                           const uint32_t *names, const uint32_t *cnt, const uint32_t *map,
                           const unsigned long long *C, const double *E, double a_mul, double a_sub, double *terms)
{
    const uint32_t k = blockIdx.y;
    const double Ck = (double)C[k], Ek = E[k];
    double s1 = 0.0, s2 = 0.0;
    if (Ck > 0.0)
        for (uint64_t i = off[k] + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < off[k + 1];
             i += (uint64_t)gridDim.x * blockDim.x) {
            const uint32_t v = map[names[i]];
            const double e = (acc[(uint64_t)v * K + k] * a_mul - (v == src[k] ? a_sub : 0.0)) / Ek;
            s1 += e;
            s2 += fabs((double)cnt[i] / Ck - e);
        }
    for (int o = 16; o; o >>= 1) {
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
        s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&terms[2 * k], s1);
        atomicAdd(&terms[2 * k + 1], s2);
    }
}

// Pair L1, reference side: D[k * n + id] = c / C[k] for query k's entries.
__global__ void k_pair_scatter(const unsigned long long *off, const uint32_t *names, const uint32_t *cnt,
                               const uint32_t *map, const unsigned long long *C, uint32_t n, double *D)
{
    const uint32_t k = blockIdx.y;
    const double Ck = (double)C[k];
    if (Ck == 0.0) return;
    for (uint64_t i = off[k] + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < off[k + 1];
         i += (uint64_t)gridDim.x * blockDim.x)
        D[(uint64_t)k * n + map[names[i]]] = (double)cnt[i] / Ck;
}

// Pair L1, other side: terms[2k] += |c / C[k] - D|, terms[2k+1] += D over
// query k's entries (D = the reference's share at the same vertex, 0 where
// it has none).  L1 = terms[2k] + (1 - terms[2k+1]): the reference's mass
// outside this query's entries adds its full share.
__global__ void k_pair_gather(const unsigned long long *off, const uint32_t *names, const uint32_t *cnt,
                              const uint32_t *map, const unsigned long long *C, uint32_t n, const double *D,
                              double *terms)
{
    const uint32_t k = blockIdx.y;
    const double Ck = (double)C[k];
    double s1 = 0.0, s2 = 0.0;
    if (Ck > 0.0)
        for (uint64_t i = off[k] + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < off[k + 1];
             i += (uint64_t)gridDim.x * blockDim.x) {
            const double d = D[(uint64_t)k * n + map[names[i]]];
            s1 += fabs((double)cnt[i] / Ck - d);
            s2 += d;
        }
    for (int o = 16; o; o >>= 1) {
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
        s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&terms[2 * k], s1);
        atomicAdd(&terms[2 * k + 1], s2);
    }
}

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

struct Free {
    cudaStream_t st;
    std::vector<void *> p;
    ~Free()
    {
        for (void *q : p) cudaFreeAsync(q, st);
    }
};

// Entries of queries [q0, q1) of a batch, on the device: the batch's own
// arrays when its results are device-resident, else its host arrays copied
// into the scratch arrays (each at least the segment's length).
struct Entries {
    const uint32_t *names = nullptr, *cnt = nullptr;
    std::vector<unsigned long long> rel;  // [q1 - q0 + 1] offsets into names / cnt
};

int batch_entries(const ptw_batch *b, uint32_t q0, uint32_t q1, cudaStream_t st, uint32_t *scratch_names,
                  uint32_t *scratch_cnt, Entries &e)
{
    const uint64_t *off = nullptr;
    const uint32_t *hn = nullptr, *hc = nullptr;
    int rc = ptw_batch_view(b, &off, &hn, &hc);
    if (rc) return rc;
    const uint64_t a = off[q0], z = off[q1];
    e.rel.resize(q1 - q0 + 1);
    for (uint32_t i = q0; i <= q1; ++i) e.rel[i - q0] = off[i] - a;
    if (batch_device(b)) {
        const uint64_t *doff = nullptr;
        const uint32_t *dn = nullptr, *dc = nullptr;
        rc = ptw_batch_view_device(b, &doff, &dn, &dc);
        if (rc) return rc;
        e.names = dn ? dn + a : nullptr;
        e.cnt = dc ? dc + a : nullptr;
        return PTW_OK;
    }
    if (z > a) {
        PTW_CUDA(cudaMemcpyAsync(scratch_names, hn + a, (z - a) * 4, cudaMemcpyHostToDevice, st));
        PTW_CUDA(cudaMemcpyAsync(scratch_cnt, hc + a, (z - a) * 4, cudaMemcpyHostToDevice, st));
    }
    e.names = scratch_names;
    e.cnt = scratch_cnt;
    return PTW_OK;
}

// Largest entry count of any group of `group` consecutive queries, over the
// host-resident batches (0 when all are device-resident).
uint64_t host_group_entries(const ptw_batch *const *bs, uint32_t nb, uint32_t nq, uint32_t group)
{
    uint64_t mx = 0;
    for (uint32_t j = 0; j < nb; ++j) {
        if (batch_device(bs[j])) continue;
        const uint64_t *off = nullptr;
        if (ptw_batch_view(bs[j], &off, nullptr, nullptr) != PTW_OK) continue;
        for (uint32_t q0 = 0; q0 < nq; q0 += group)
            mx = std::max<uint64_t>(mx, off[std::min(nq, q0 + group)] - off[q0]);
    }
    return mx;
}

// Batches scored together must hold the same queries (sources and count)
// and full result lists.
int check_same_queries(const ptw_batch *const *bs, uint32_t nb, uint32_t *nq_out)
{
    uint32_t nq0 = 0;
    for (uint32_t j = 0; j < nb; ++j) {
        if (!bs[j]) return fail(PTW_EINVAL, "null batch");
        if (batch_top_k(bs[j])) return fail(PTW_EINVAL, "the L1 error needs full results (batch run with top_k > 0)");
        uint32_t nq = 0;
        int rc = ptw_batch_info(bs[j], &nq, nullptr, nullptr);
        if (rc) return rc;
        if (j == 0) nq0 = nq;
        if (nq != nq0) return fail(PTW_EINVAL, "batches hold different numbers of queries");
        const ptw_query *a = batch_queries(bs[0]), *b = batch_queries(bs[j]);
        for (uint32_t i = 0; i < nq; ++i)
            if (a[i].source != b[i].source) return fail(PTW_EINVAL, "batches hold different query sources");
    }
    *nq_out = nq0;
    return PTW_OK;
}

// Dense name -> internal id table over [0, id_bound) on st.
int name_map(ptw_graph *g, cudaStream_t st, uint32_t *map)
{
    PTW_CUDA(cudaMemsetAsync(map, 0xFF, (uint64_t)g->dg.id_bound * 4, st));
    const unsigned gm = (unsigned)std::min<uint64_t>((g->dg.n + 255) / 256, (uint64_t)g->num_sms * 32);
    k_name_map<<<std::max(gm, 1u), 256, 0, st>>>(g->dg.names, g->dg.idx2int, g->dg.n, map);
    PTW_CUDA(cudaGetLastError());
    return PTW_OK;
}

// Blocks per query for kernels that stride over a query's entries.
unsigned entry_blocks(const std::vector<unsigned long long> &rel, unsigned num_sms)
{
    uint64_t mx = 1;
    for (size_t i = 0; i + 1 < rel.size(); ++i) mx = std::max<uint64_t>(mx, rel[i + 1] - rel[i]);
    return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((mx + 255) / 256, (uint64_t)num_sms * 4));
}

}  // namespace
}  // namespace ptw

using namespace ptw;

extern "C" int ptw_batch_l1_many(ptw_graph *g, const ptw_batch *const *bs, uint32_t nb, double sp, int32_t app,
                                 double tol, double *h_l1)
try {
    NvtxRange nvtx("ptw_batch_l1_many");
    if (!g || !bs || !h_l1 || nb == 0) return fail(PTW_EINVAL, "null argument");
    if (!(sp > 0.0 && sp < 1.0)) return fail(PTW_EINVAL, "sp must be in (0, 1)");
    if (app != PTW_APP_VISITS && app != PTW_APP_ENDPOINT) return fail(PTW_EINVAL, "unknown app");
    if (!(tol > 0.0)) return fail(PTW_EINVAL, "tol must be > 0");
    uint32_t nq = 0;
    int rc = check_same_queries(bs, nb, &nq);
    if (rc) return rc;
    PTW_CUDA(cudaSetDevice(g->device));
    const ptw_query *qs = batch_queries(bs[0]);
    const uint32_t n = g->dg.n;
    const uint64_t m = g->dg.m;
    cudaStream_t st = g->stream;
    Free fr{st, {}};
    auto dalloc = [&](void **p, uint64_t bytes) -> cudaError_t {
        cudaError_t e = cudaMallocAsync(p, std::max<uint64_t>(bytes, 16), st);
        if (e == cudaSuccess) fr.p.push_back(*p);
        return e;
    };
    // transposed CSR
    unsigned long long *keys, *keys2;
    uint32_t *tcol, *tdeg, *toff, *map;
    double *inv;
    PTW_CUDA(dalloc((void **)&keys, m * 8));
    PTW_CUDA(dalloc((void **)&keys2, m * 8));
    PTW_CUDA(dalloc((void **)&tcol, m * 4));
    PTW_CUDA(dalloc((void **)&tdeg, (n + 1ull) * 4));
    PTW_CUDA(dalloc((void **)&toff, (n + 1ull) * 4));
    PTW_CUDA(dalloc((void **)&inv, n * 8ull));
    PTW_CUDA(dalloc((void **)&map, (uint64_t)g->dg.id_bound * 4));
    const unsigned grid = (unsigned)std::min<uint64_t>(((uint64_t)n * 32 + 255) / 256, (uint64_t)g->num_sms * 64);
    k_transpose_keys<<<std::max(grid, 1u), 256, 0, st>>>(g->dg.adj, g->dg.col, n, keys);
    {
        cub::DoubleBuffer<unsigned long long> db(keys, keys2);
        PTW_CUDA(cub_call([&](void *t, size_t &bb) {
            return cub::DeviceRadixSort::SortKeys(t, bb, db, (int64_t)m, 0, 64, st);
        }, st));
        if (db.Current() != keys) std::swap(keys, keys2);
    }
    PTW_CUDA(cudaMemsetAsync(tdeg, 0, (n + 1ull) * 4, st));
    k_split_t<<<std::max(grid, 1u), 256, 0, st>>>(keys, m, tcol, tdeg);
    PTW_CUDA(cub_call([&](void *t, size_t &bb) {
        return cub::DeviceScan::ExclusiveSum(t, bb, tdeg, toff, (int64_t)n + 1, st);
    }, st));
    k_inv_deg<<<std::max(grid, 1u), 256, 0, st>>>(g->dg.adj, n, inv);
    PTW_CUDA(cudaGetLastError());
    rc = name_map(g, st, map);
    if (rc) return rc;
    // pull segments: every vertex's in-edges in pieces of at most kSegEdges
    std::vector<uint32_t> h_toff(n + 1ull);
    PTW_CUDA(cudaMemcpyAsync(h_toff.data(), toff, (n + 1ull) * 4, cudaMemcpyDeviceToHost, st));
    PTW_CUDA(cudaStreamSynchronize(st));
    std::vector<uint32_t> sv, se0, se1, spart, hv, hp0;
    uint32_t np = 0;  // partial-sum slots handed out
    sv.reserve(n + m / kSegEdges + 1);
    se0.reserve(sv.capacity());
    se1.reserve(sv.capacity());
    spart.reserve(sv.capacity());
    for (uint32_t v = 0; v < n; ++v) {
        const uint32_t a = h_toff[v], z = h_toff[v + 1];
        if (z - a <= kSegEdges) {
            sv.push_back(v);
            se0.push_back(a);
            se1.push_back(z);
            spart.push_back(kNoPart);
            continue;
        }
        hv.push_back(v);
        hp0.push_back(np);
        for (uint64_t e = a; e < z; e += kSegEdges) {
            sv.push_back(v);
            se0.push_back((uint32_t)e);
            se1.push_back((uint32_t)std::min<uint64_t>(z, e + kSegEdges));
            spart.push_back(np++);
        }
    }
    hp0.push_back(np);  // [nheavy + 1]
    const uint64_t nseg = sv.size();
    const uint32_t nheavy = (uint32_t)hv.size();
    uint32_t *d_sv, *d_se0, *d_se1, *d_spart, *d_hv, *d_hp0;
    double *partial;
    PTW_CUDA(dalloc((void **)&d_sv, nseg * 4));
    PTW_CUDA(dalloc((void **)&d_se0, nseg * 4));
    PTW_CUDA(dalloc((void **)&d_se1, nseg * 4));
    PTW_CUDA(dalloc((void **)&d_spart, nseg * 4));
    PTW_CUDA(dalloc((void **)&d_hv, (nheavy + 1ull) * 4));
    PTW_CUDA(dalloc((void **)&d_hp0, (nheavy + 1ull) * 4));
    PTW_CUDA(dalloc((void **)&partial, std::max<uint64_t>(np, 1) * K * 8));
    PTW_CUDA(cudaMemcpyAsync(d_sv, sv.data(), nseg * 4, cudaMemcpyHostToDevice, st));
    PTW_CUDA(cudaMemcpyAsync(d_se0, se0.data(), nseg * 4, cudaMemcpyHostToDevice, st));
    PTW_CUDA(cudaMemcpyAsync(d_se1, se1.data(), nseg * 4, cudaMemcpyHostToDevice, st));
    PTW_CUDA(cudaMemcpyAsync(d_spart, spart.data(), nseg * 4, cudaMemcpyHostToDevice, st));
    PTW_CUDA(cudaMemcpyAsync(d_hp0, hp0.data(), (nheavy + 1ull) * 4, cudaMemcpyHostToDevice, st));
    if (nheavy) PTW_CUDA(cudaMemcpyAsync(d_hv, hv.data(), nheavy * 4ull, cudaMemcpyHostToDevice, st));
    const unsigned pgrid = (unsigned)std::min<uint64_t>((nseg * 32 + 255) / 256, (uint64_t)g->num_sms * 64);
    const unsigned hgrid = (unsigned)std::min<uint64_t>((nheavy * 32ull + 255) / 256, (uint64_t)g->num_sms * 8);
    double *x, *y, *acc, *mass, *csum, *terms, *d_E;
    uint32_t *d_src, *s_names = nullptr, *s_cnt = nullptr;
    unsigned long long *d_off, *d_C;
    PTW_CUDA(dalloc((void **)&x, (uint64_t)n * K * 8));
    PTW_CUDA(dalloc((void **)&y, (uint64_t)n * K * 8));
    PTW_CUDA(dalloc((void **)&acc, (uint64_t)n * K * 8));
    PTW_CUDA(dalloc((void **)&mass, K * 8));
    PTW_CUDA(dalloc((void **)&csum, K * 8));
    PTW_CUDA(dalloc((void **)&terms, 2 * K * 8));
    PTW_CUDA(dalloc((void **)&d_E, K * 8));
    PTW_CUDA(dalloc((void **)&d_src, K * 4));
    PTW_CUDA(dalloc((void **)&d_off, (K + 1) * 8));
    PTW_CUDA(dalloc((void **)&d_C, K * 8));
    const uint64_t scratch = host_group_entries(bs, nb, nq, K);
    if (scratch) {
        PTW_CUDA(dalloc((void **)&s_names, scratch * 4));
        PTW_CUDA(dalloc((void **)&s_cnt, scratch * 4));
    }
    const double a_mul = app == PTW_APP_VISITS ? 1.0 / (sp * (1.0 - sp)) : 1.0 / (1.0 - sp);
    const double a_sub = sp / (1.0 - sp);
    for (uint32_t q0 = 0; q0 < nq; q0 += K) {
        const uint32_t nk = std::min<uint32_t>(K, nq - q0);
        std::vector<uint32_t> src(nk);
        std::vector<double> x0(nk);
        for (uint32_t k = 0; k < nk; ++k) {
            const uint32_t *p = std::lower_bound(g->h_names, g->h_names + n, qs[q0 + k].source);
            if (p == g->h_names + n || *p != qs[q0 + k].source) return fail(PTW_EINVAL, "query source not in graph");
            src[k] = g->h_idx2int[p - g->h_names];
        }
        // x = e_s / deg(s), acc = sp e_s in column k of each source
        for (uint32_t k = 0; k < nk; ++k) {
            uint2 rec;
            PTW_CUDA(cudaMemcpyAsync(&rec, g->dg.adj + src[k], 8, cudaMemcpyDeviceToHost, st));
            PTW_CUDA(cudaStreamSynchronize(st));
            x0[k] = rec.y ? 1.0 / (double)rec.y : 0.0;
        }
        PTW_CUDA(cudaMemsetAsync(x, 0, (uint64_t)n * K * 8, st));
        PTW_CUDA(cudaMemsetAsync(acc, 0, (uint64_t)n * K * 8, st));
        for (uint32_t k = 0; k < nk; ++k) {
            PTW_CUDA(cudaMemcpyAsync(x + (uint64_t)src[k] * K + k, &x0[k], 8, cudaMemcpyHostToDevice, st));
            PTW_CUDA(cudaMemcpyAsync(acc + (uint64_t)src[k] * K + k, &sp, 8, cudaMemcpyHostToDevice, st));
        }
        PTW_CUDA(cudaStreamSynchronize(st));  // x0 is read before it goes out of scope
        for (int it = 0; it < 100000; ++it) {
            PTW_CUDA(cudaMemsetAsync(mass, 0, K * 8, st));
            k_pull<<<std::max(pgrid, 1u), 256, 0, st>>>(d_sv, d_se0, d_se1, d_spart, nseg, tcol, inv, x, y, acc,
                                                        partial, 1.0 - sp, sp, mass);
            if (nheavy)
                k_pull_heavy<<<std::max(hgrid, 1u), 256, 0, st>>>(d_hv, d_hp0, nheavy, inv, partial, y, acc, 1.0 - sp,
                                                                  sp, mass);
            PTW_CUDA(cudaGetLastError());
            std::swap(x, y);
            double hm[K];
            PTW_CUDA(cudaMemcpyAsync(hm, mass, K * 8, cudaMemcpyDeviceToHost, st));
            PTW_CUDA(cudaStreamSynchronize(st));
            double mx = 0.0;
            for (uint32_t k = 0; k < nk; ++k) mx = std::max(mx, sp * hm[k]);
            if (mx < tol) break;
        }
        PTW_CUDA(cudaMemsetAsync(csum, 0, K * 8, st));
        k_colsum<<<std::max(grid, 1u), 256, 0, st>>>(acc, n, csum);
        double hs[K], hE[K];
        PTW_CUDA(cudaMemcpyAsync(hs, csum, K * 8, cudaMemcpyDeviceToHost, st));
        PTW_CUDA(cudaStreamSynchronize(st));
        for (uint32_t k = 0; k < nk; ++k) hE[k] = hs[k] * a_mul - a_sub;
        PTW_CUDA(cudaMemcpyAsync(d_E, hE, nk * 8, cudaMemcpyHostToDevice, st));
        PTW_CUDA(cudaMemcpyAsync(d_src, src.data(), nk * 4, cudaMemcpyHostToDevice, st));
        for (uint32_t j = 0; j < nb; ++j) {
            Entries e;
            rc = batch_entries(bs[j], q0, q0 + nk, st, s_names, s_cnt, e);
            if (rc) return rc;
            PTW_CUDA(cudaMemcpyAsync(d_off, e.rel.data(), (nk + 1) * 8ull, cudaMemcpyHostToDevice, st));
            PTW_CUDA(cudaMemsetAsync(d_C, 0, K * 8, st));
            PTW_CUDA(cudaMemsetAsync(terms, 0, 2 * K * 8, st));
            if (e.rel[nk] > 0) {
                const dim3 gg(entry_blocks(e.rel, g->num_sms), nk);
                k_count_sum<<<gg, 256, 0, st>>>(d_off, e.cnt, d_C);
                k_l1_terms<<<gg, 256, 0, st>>>(acc, d_src, d_off, e.names, e.cnt, map, d_C, d_E, a_mul, a_sub,
                                               terms);
                PTW_CUDA(cudaGetLastError());
            }
            double ht[2 * K];
            unsigned long long hC[K];
            PTW_CUDA(cudaMemcpyAsync(ht, terms, 2 * K * 8, cudaMemcpyDeviceToHost, st));
            PTW_CUDA(cudaMemcpyAsync(hC, d_C, K * 8, cudaMemcpyDeviceToHost, st));
            PTW_CUDA(cudaStreamSynchronize(st));  // also keeps e.rel alive until its upload ran
            for (uint32_t k = 0; k < nk; ++k)
                h_l1[(uint64_t)j * nq + q0 + k] = hC[k] == 0 ? 2.0 : 1.0 - ht[2 * k] + ht[2 * k + 1];
        }
    }
    return PTW_OK;
} catch (...) {
    return host_exception();
}

extern "C" int ptw_batch_l1(ptw_graph *g, const ptw_batch *b, double sp, int32_t app, double tol, double *h_l1)
{
    return ptw_batch_l1_many(g, &b, 1, sp, app, tol, h_l1);
}

extern "C" int ptw_batch_l1_pair(ptw_graph *g, const ptw_batch *a, const ptw_batch *ref, double *h_l1)
try {
    NvtxRange nvtx("ptw_batch_l1_pair");
    if (!g || !a || !ref || !h_l1) return fail(PTW_EINVAL, "null argument");
    const ptw_batch *bs[2] = {a, ref};
    uint32_t nq = 0;
    int rc = check_same_queries(bs, 2, &nq);
    if (rc) return rc;
    PTW_CUDA(cudaSetDevice(g->device));
    const uint32_t n = g->dg.n;
    cudaStream_t st = g->stream;
    Free fr{st, {}};
    auto dalloc = [&](void **p, uint64_t bytes) -> cudaError_t {
        cudaError_t e = cudaMallocAsync(p, std::max<uint64_t>(bytes, 16), st);
        if (e == cudaSuccess) fr.p.push_back(*p);
        return e;
    };
    // queries per pass: a dense row of n doubles each, at most 2 GB in all
    const uint32_t Q =
        (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(64, (2ull << 30) / (8ull * std::max(n, 1u))));
    uint32_t *map, *s_names[2] = {nullptr, nullptr}, *s_cnt[2] = {nullptr, nullptr};
    double *D, *terms;
    unsigned long long *d_off[2], *d_C[2];
    PTW_CUDA(dalloc((void **)&map, (uint64_t)g->dg.id_bound * 4));
    PTW_CUDA(dalloc((void **)&D, (uint64_t)Q * n * 8));
    PTW_CUDA(dalloc((void **)&terms, 2ull * Q * 8));
    for (int s = 0; s < 2; ++s) {
        PTW_CUDA(dalloc((void **)&d_off[s], (Q + 1ull) * 8));
        PTW_CUDA(dalloc((void **)&d_C[s], Q * 8ull));
        const uint64_t scratch = host_group_entries(&bs[s], 1, nq, Q);
        if (scratch) {
            PTW_CUDA(dalloc((void **)&s_names[s], scratch * 4));
            PTW_CUDA(dalloc((void **)&s_cnt[s], scratch * 4));
        }
    }
    rc = name_map(g, st, map);
    if (rc) return rc;
    for (uint32_t q0 = 0; q0 < nq; q0 += Q) {
        const uint32_t nk = std::min<uint32_t>(Q, nq - q0);
        Entries e[2];
        for (int s = 0; s < 2; ++s) {
            rc = batch_entries(bs[s], q0, q0 + nk, st, s_names[s], s_cnt[s], e[s]);
            if (rc) return rc;
            PTW_CUDA(cudaMemcpyAsync(d_off[s], e[s].rel.data(), (nk + 1) * 8ull, cudaMemcpyHostToDevice, st));
            PTW_CUDA(cudaMemsetAsync(d_C[s], 0, Q * 8ull, st));
            if (e[s].rel[nk] > 0)
                k_count_sum<<<dim3(entry_blocks(e[s].rel, g->num_sms), nk), 256, 0, st>>>(d_off[s], e[s].cnt,
                                                                                        d_C[s]);
        }
        PTW_CUDA(cudaMemsetAsync(D, 0, (uint64_t)nk * n * 8, st));
        PTW_CUDA(cudaMemsetAsync(terms, 0, 2ull * Q * 8, st));
        if (e[1].rel[nk] > 0)
            k_pair_scatter<<<dim3(entry_blocks(e[1].rel, g->num_sms), nk), 256, 0, st>>>(
                d_off[1], e[1].names, e[1].cnt, map, d_C[1], n, D);
        if (e[0].rel[nk] > 0)
            k_pair_gather<<<dim3(entry_blocks(e[0].rel, g->num_sms), nk), 256, 0, st>>>(
                d_off[0], e[0].names, e[0].cnt, map, d_C[0], n, D, terms);
        PTW_CUDA(cudaGetLastError());
        std::vector<double> ht(2ull * Q);
        std::vector<unsigned long long> hCa(Q), hCr(Q);
        PTW_CUDA(cudaMemcpyAsync(ht.data(), terms, 2ull * Q * 8, cudaMemcpyDeviceToHost, st));
        PTW_CUDA(cudaMemcpyAsync(hCa.data(), d_C[0], Q * 8ull, cudaMemcpyDeviceToHost, st));
        PTW_CUDA(cudaMemcpyAsync(hCr.data(), d_C[1], Q * 8ull, cudaMemcpyDeviceToHost, st));
        PTW_CUDA(cudaStreamSynchronize(st));
        for (uint32_t k = 0; k < nk; ++k) {
            if (hCa[k] == 0 && hCr[k] == 0) h_l1[q0 + k] = 0.0;
            else if (hCa[k] == 0 || hCr[k] == 0) h_l1[q0 + k] = 1.0;
            else h_l1[q0 + k] = ht[2 * k] + (1.0 - ht[2 * k + 1]);
        }
    }
    return PTW_OK;
} catch (...) {
    return host_exception();
}
