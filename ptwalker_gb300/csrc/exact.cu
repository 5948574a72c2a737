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
// so every sum is taken in a fixed order (deterministic FP64).  Iteration
// stops when sp * (mass of the new term) < tol for every source.
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

// y[v][q] = f * sum_{u in in(v)} x[u][q] * inv[u];  acc[v][q] += sp * y[v][q];
// mass[q] += sum_v y[v][q]  (block-reduced).
__global__ void k_pull(const uint32_t *toff, const uint32_t *tcol, const double *inv, uint32_t n,
                       const double *x, double *y, double *acc, double f, double sp, double *mass)
{
    __shared__ double part[8][K];
    const uint32_t lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const uint64_t warps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    double local = 0.0;
    for (uint64_t v = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; v < n; v += warps) {
        double s = 0.0;
        for (uint32_t e = toff[v]; e < toff[v + 1]; ++e) {
            const uint32_t u = tcol[e];
            s += x[(uint64_t)u * K + lane] * inv[u];
        }
        s *= f;
        y[v * K + lane] = s;
        acc[v * K + lane] += sp * s;
        local += s;
    }
    part[wib][lane] = local;
    __syncthreads();
    if (wib == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += part[w][lane];
        atomicAdd(&mass[lane], t);
    }
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

// For one query (column q, source src): sums over its sparse entries of
// e_v / E and |c_v / C - e_v / E|, with e from acc (= pi) per the app.
__global__ void k_l1_terms(const double *acc, uint32_t q, uint32_t src, const uint32_t *ids, const uint32_t *cnt,
                           uint64_t ne, double C, double E, double a_mul, double a_sub, double *out)
{
    double s1 = 0.0, s2 = 0.0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < ne; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t v = ids[i];
        const double e = (acc[(uint64_t)v * K + q] * a_mul - (v == src ? a_sub : 0.0)) / E;
        s1 += e;
        s2 += fabs((double)cnt[i] / C - e);
    }
    for (int o = 16; o; o >>= 1) {
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
        s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&out[0], s1);
        atomicAdd(&out[1], s2);
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

}  // namespace
}  // namespace ptw

using namespace ptw;

extern "C" int ptw_batch_l1(ptw_graph *g, const ptw_batch *b, double sp, int32_t app, double tol, double *h_l1)
try {
    NvtxRange nvtx("ptw_batch_l1");
    if (!g || !b || !h_l1) return fail(PTW_EINVAL, "null argument");
    if (!(sp > 0.0 && sp < 1.0)) return fail(PTW_EINVAL, "sp must be in (0, 1)");
    if (app != PTW_APP_VISITS && app != PTW_APP_ENDPOINT) return fail(PTW_EINVAL, "unknown app");
    if (!(tol > 0.0)) return fail(PTW_EINVAL, "tol must be > 0");
    if (batch_top_k(b)) return fail(PTW_EINVAL, "the L1 error needs full results (batch run with top_k > 0)");
    PTW_CUDA(cudaSetDevice(g->device));
    uint32_t nq = 0;
    uint64_t ne = 0;
    int rc = ptw_batch_info(b, &nq, &ne, nullptr);
    if (rc) return rc;
    std::vector<uint64_t> off(nq + 1);
    std::vector<uint32_t> names(ne), cnts(ne);
    rc = ptw_batch_export(b, off.data(), names.data(), cnts.data());
    if (rc) return rc;
    const ptw_query *qs = batch_queries(b);
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
    uint32_t *tcol, *tdeg, *toff;
    double *inv;
    PTW_CUDA(dalloc((void **)&keys, m * 8));
    PTW_CUDA(dalloc((void **)&keys2, m * 8));
    PTW_CUDA(dalloc((void **)&tcol, m * 4));
    PTW_CUDA(dalloc((void **)&tdeg, (n + 1ull) * 4));
    PTW_CUDA(dalloc((void **)&toff, (n + 1ull) * 4));
    PTW_CUDA(dalloc((void **)&inv, n * 8ull));
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
    double *x, *y, *acc, *mass, *csum, *terms;
    uint32_t *d_ids, *d_cnt;
    PTW_CUDA(dalloc((void **)&x, (uint64_t)n * K * 8));
    PTW_CUDA(dalloc((void **)&y, (uint64_t)n * K * 8));
    PTW_CUDA(dalloc((void **)&acc, (uint64_t)n * K * 8));
    PTW_CUDA(dalloc((void **)&mass, K * 8));
    PTW_CUDA(dalloc((void **)&csum, K * 8));
    PTW_CUDA(dalloc((void **)&terms, 16));
    uint64_t max_ent = 1;
    for (uint32_t i = 0; i < nq; ++i) max_ent = std::max<uint64_t>(max_ent, off[i + 1] - off[i]);
    PTW_CUDA(dalloc((void **)&d_ids, max_ent * 4));
    PTW_CUDA(dalloc((void **)&d_cnt, max_ent * 4));
    const double a_mul = app == PTW_APP_VISITS ? 1.0 / (sp * (1.0 - sp)) : 1.0 / (1.0 - sp);
    const double a_sub = app == PTW_APP_VISITS ? sp / (1.0 - sp) : sp / (1.0 - sp);
    std::vector<uint32_t> ids(max_ent);
    for (uint32_t q0 = 0; q0 < nq; q0 += K) {
        const uint32_t nb = std::min<uint32_t>(K, nq - q0);
        std::vector<uint32_t> src(nb);
        for (uint32_t k = 0; k < nb; ++k) {
            const uint32_t *p = std::lower_bound(g->h_names, g->h_names + n, qs[q0 + k].source);
            if (p == g->h_names + n || *p != qs[q0 + k].source) return fail(PTW_EINVAL, "query source not in graph");
            src[k] = g->h_idx2int[p - g->h_names];
        }
        PTW_CUDA(cudaMemsetAsync(x, 0, (uint64_t)n * K * 8, st));
        PTW_CUDA(cudaMemsetAsync(acc, 0, (uint64_t)n * K * 8, st));
        std::vector<double> one(1, 1.0), spv(1, sp);
        for (uint32_t k = 0; k < nb; ++k) {
            PTW_CUDA(cudaMemcpyAsync(x + (uint64_t)src[k] * K + k, one.data(), 8, cudaMemcpyHostToDevice, st));
            PTW_CUDA(cudaMemcpyAsync(acc + (uint64_t)src[k] * K + k, spv.data(), 8, cudaMemcpyHostToDevice, st));
        }
        for (int it = 0; it < 100000; ++it) {
            PTW_CUDA(cudaMemsetAsync(mass, 0, K * 8, st));
            k_pull<<<std::max(grid, 1u), 256, 0, st>>>(toff, tcol, inv, n, x, y, acc, 1.0 - sp, sp, mass);
            PTW_CUDA(cudaGetLastError());
            std::swap(x, y);
            double hm[K];
            PTW_CUDA(cudaMemcpyAsync(hm, mass, K * 8, cudaMemcpyDeviceToHost, st));
            PTW_CUDA(cudaStreamSynchronize(st));
            double mx = 0.0;
            for (uint32_t k = 0; k < nb; ++k) mx = std::max(mx, sp * hm[k]);
            if (mx < tol) break;
        }
        PTW_CUDA(cudaMemsetAsync(csum, 0, K * 8, st));
        k_colsum<<<std::max(grid, 1u), 256, 0, st>>>(acc, n, csum);
        double hs[K];
        PTW_CUDA(cudaMemcpyAsync(hs, csum, K * 8, cudaMemcpyDeviceToHost, st));
        PTW_CUDA(cudaStreamSynchronize(st));
        for (uint32_t k = 0; k < nb; ++k) {
            const uint32_t qi = q0 + k;
            const uint64_t e0 = off[qi], e1 = off[qi + 1];
            const double E = hs[k] * a_mul - a_sub;
            double C = 0.0;
            for (uint64_t e = e0; e < e1; ++e) {
                const uint32_t *p = std::lower_bound(g->h_names, g->h_names + n, names[e]);
                ids[e - e0] = g->h_idx2int[p - g->h_names];
                C += cnts[e];
            }
            if (e1 == e0 || C == 0.0) {
                h_l1[qi] = 2.0;
                continue;
            }
            PTW_CUDA(cudaMemcpyAsync(d_ids, ids.data(), (e1 - e0) * 4, cudaMemcpyHostToDevice, st));
            PTW_CUDA(cudaMemcpyAsync(d_cnt, cnts.data() + e0, (e1 - e0) * 4, cudaMemcpyHostToDevice, st));
            PTW_CUDA(cudaMemsetAsync(terms, 0, 16, st));
            const unsigned g2 = (unsigned)std::min<uint64_t>((e1 - e0 + 255) / 256, 1024);
            k_l1_terms<<<std::max(g2, 1u), 256, 0, st>>>(acc, k, src[k], d_ids, d_cnt, e1 - e0, C, E, a_mul, a_sub,
                                                         terms);
            double ht[2];
            PTW_CUDA(cudaMemcpyAsync(ht, terms, 16, cudaMemcpyDeviceToHost, st));
            PTW_CUDA(cudaStreamSynchronize(st));
            h_l1[qi] = 1.0 - ht[0] + ht[1];
        }
    }
    return PTW_OK;
} catch (...) {
    return host_exception();
}
