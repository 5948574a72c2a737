// Batched single-source PPR / RWR (K4).
//
// The reference answers one source per process (src/core/ppr.cpp:121-138,
// source hard-coded to internal id 0; RWR.cpp:109-128 records (start, end)
// pairs).  Here thousands of queries run in one persistent launch per wave:
//
//   device query table   q_off[q]  first global walker index of query q
//                         q_src[q]  source (internal id), q_qid[q] its query id
//                         q_tab[q], q_mask[q]  its count table (slot offset, size-1)
//   global walker index g -> query q = last q with q_off[q] <= g (binary search),
//   walker id (q_qid[q] << 32) + (g - q_off[q]): every draw depends on the
//   query id and the walker's rank in its query only, so a query's counts are
//   the same alone or in any batch and wave.
//
// Per-query counts are kept sparse in open-addressing tables of 64-bit slots
// (vertex internal id + 1 in the high half, count in the low half), sized
// from the query's budget; a query that finds no free slot within the probe
// limit raises its flag and the host runs it again with a table of 2n slots,
// which cannot fill.  Waves take queries in order while their tables fit the
// table budget (admission by device memory).  After a wave the tables are
// compacted into (name, count) lists sorted by name and copied to the host.
#include <cub/cub.cuh>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "batch_kernels.cuh"

struct ptw_batch {
    uint32_t nq = 0;
    std::vector<ptw_query> queries;
    std::vector<uint64_t> offsets;  // [nq + 1]
    std::vector<uint32_t> names, counts;
    ptw_walk_stats stats{};
};

namespace ptw {
namespace {

constexpr uint64_t kMaxBudget = 1ull << 28;

struct DevBuf {
    cudaStream_t st;
    std::vector<void *> ptrs;
    explicit DevBuf(cudaStream_t s) : st(s) {}
    template <typename T> cudaError_t alloc(T **p, uint64_t count)
    {
        void *q = nullptr;
        cudaError_t e = cudaMallocAsync(&q, std::max<uint64_t>(count, 1) * sizeof(T), st);
        if (e == cudaSuccess) ptrs.push_back(q);
        *p = (T *)q;
        return e;
    }
    ~DevBuf()
    {
        for (void *q : ptrs) cudaFreeAsync(q, st);
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

struct WaveQuery {
    uint32_t index;  // position in the caller's array
    uint32_t src;    // internal id
    uint32_t qid;
    uint64_t budget;
    uint64_t cap;    // table slots (power of two)
};

// Runs one wave; stores each query's sorted entries in per-query host lists.
int run_wave(ptw_graph *g, const std::vector<WaveQuery> &wq, const ptw_batch_cfg *cfg, uint64_t thr,
             std::vector<std::vector<uint32_t>> &names, std::vector<std::vector<uint32_t>> &cnts,
             std::vector<uint32_t> &overflow, uint64_t *moves_out)
{
    cudaStream_t st = g->stream;
    const uint32_t nq = (uint32_t)wq.size();
    std::vector<unsigned long long> h_off(nq + 1), h_tab(nq + 1);
    std::vector<uint32_t> h_src(nq), h_qid(nq), h_mask(nq), h_cap(nq);
    for (uint32_t i = 0; i < nq; ++i) {
        h_off[i + 1] = h_off[i] + wq[i].budget;
        h_tab[i + 1] = h_tab[i] + wq[i].cap;
        h_src[i] = wq[i].src;
        h_qid[i] = wq[i].qid;
        h_mask[i] = (uint32_t)(wq[i].cap - 1);
        h_cap[i] = (uint32_t)wq[i].cap;
    }
    const uint64_t total = h_off[nq], n_slots = h_tab[nq];
    DevBuf db(st);
    unsigned long long *d_off, *d_tab, *d_slots, *d_ctrl;
    uint32_t *d_src, *d_qid, *d_mask, *d_flag;
    PTW_CUDA(db.alloc(&d_off, nq + 1));
    PTW_CUDA(db.alloc(&d_tab, nq + 1));
    PTW_CUDA(db.alloc(&d_src, nq));
    PTW_CUDA(db.alloc(&d_qid, nq));
    PTW_CUDA(db.alloc(&d_mask, nq));
    PTW_CUDA(db.alloc(&d_flag, nq));
    PTW_CUDA(db.alloc(&d_ctrl, 2));
    PTW_CUDA(db.alloc(&d_slots, n_slots));
    PTW_CUDA(cudaMemcpyAsync(d_off, h_off.data(), (nq + 1) * 8ull, cudaMemcpyHostToDevice, st));
    PTW_CUDA(cudaMemcpyAsync(d_tab, h_tab.data(), (nq + 1) * 8ull, cudaMemcpyHostToDevice, st));
    PTW_CUDA(cudaMemcpyAsync(d_src, h_src.data(), nq * 4ull, cudaMemcpyHostToDevice, st));
    PTW_CUDA(cudaMemcpyAsync(d_qid, h_qid.data(), nq * 4ull, cudaMemcpyHostToDevice, st));
    PTW_CUDA(cudaMemcpyAsync(d_mask, h_mask.data(), nq * 4ull, cudaMemcpyHostToDevice, st));
    PTW_CUDA(cudaMemsetAsync(d_flag, 0, nq * 4ull, st));
    PTW_CUDA(cudaMemsetAsync(d_ctrl, 0, 16, st));
    PTW_CUDA(cudaMemsetAsync(d_slots, 0, n_slots * 8, st));

    BatchArgs a;
    a.adj = g->dg.adj;
    a.col = g->dg.col;
    a.q_off = d_off;
    a.q_j0 = nullptr;
    a.q_src = d_src;
    a.q_qid = d_qid;
    a.q_tab = d_tab;
    a.q_mask = d_mask;
    a.q_flag = d_flag;
    a.slots = d_slots;
    a.ctrl = d_ctrl;
    a.total = total;
    a.thr = thr;
    a.nq = nq;
    a.key0 = (uint32_t)cfg->seed;
    a.key1 = (uint32_t)(cfg->seed >> 32);
    a.max_moves = cfg->max_moves;
    a.chunk = 256;
    a.app = cfg->app;
    int per_sm = 0;
    PTW_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch, 256, 0));
    uint64_t grid = (uint64_t)g->num_sms * std::max(per_sm, 1);
    grid = std::min<uint64_t>(grid, std::max<uint64_t>(1, (total + a.chunk * 8 - 1) / (a.chunk * 8)));
    k_batch<<<(unsigned)grid, 256, 0, st>>>(a);
    PTW_CUDA(cudaGetLastError());
    std::vector<uint32_t> h_flag(nq);
    unsigned long long h_moves = 0;
    PTW_CUDA(cudaMemcpyAsync(h_flag.data(), d_flag, nq * 4ull, cudaMemcpyDeviceToHost, st));
    PTW_CUDA(cudaMemcpyAsync(&h_moves, d_ctrl + 1, 8, cudaMemcpyDeviceToHost, st));
    std::vector<std::vector<uint32_t> *> out_n(nq), out_c(nq);
    for (uint32_t i = 0; i < nq; ++i) {
        out_n[i] = &names[wq[i].index];
        out_c[i] = &cnts[wq[i].index];
    }
    int rc = compact_tables(g, d_slots, h_tab.data(), h_cap.data(), nq, out_n.data(), out_c.data());
    if (rc) return rc;
    *moves_out += h_moves;
    for (uint32_t i = 0; i < nq; ++i)
        if (h_flag[i]) {
            overflow.push_back(wq[i].index);
            names[wq[i].index].clear();
            cnts[wq[i].index].clear();
        }
    return PTW_OK;
}

uint64_t next_pow2(uint64_t x)
{
    uint64_t p = 1;
    while (p < x) p <<= 1;
    return p;
}

}  // namespace

const ptw_query *batch_queries(const ptw_batch *b) { return b->queries.data(); }

int compact_tables(ptw_graph *g, unsigned long long *d_slots, const unsigned long long *h_base,
                   const uint32_t *h_cap, uint32_t nt, std::vector<uint32_t> **names,
                   std::vector<uint32_t> **counts)
{
    if (nt == 0) return PTW_OK;
    cudaStream_t st = g->stream;
    DevBuf db(st);
    unsigned long long *d_base, *d_cnt, *d_seg, *d_fill;
    uint32_t *d_cap;
    PTW_CUDA(db.alloc(&d_base, nt));
    PTW_CUDA(db.alloc(&d_cap, nt));
    PTW_CUDA(db.alloc(&d_cnt, nt));
    PTW_CUDA(db.alloc(&d_seg, nt + 1));
    PTW_CUDA(db.alloc(&d_fill, nt));
    PTW_CUDA(cudaMemcpyAsync(d_base, h_base, nt * 8ull, cudaMemcpyHostToDevice, st));
    PTW_CUDA(cudaMemcpyAsync(d_cap, h_cap, nt * 4ull, cudaMemcpyHostToDevice, st));
    PTW_CUDA(cudaMemsetAsync(d_cnt, 0, nt * 8ull, st));
    PTW_CUDA(cudaMemsetAsync(d_fill, 0, nt * 8ull, st));
    PTW_CUDA(cudaMemsetAsync(d_seg, 0, 8, st));
    uint32_t max_cap = 0;
    for (uint32_t i = 0; i < nt; ++i) max_cap = std::max(max_cap, h_cap[i]);
    const unsigned gx = (unsigned)std::min<uint64_t>(256, (max_cap + 2047) / 2048);
    for (uint32_t t0 = 0; t0 < nt; t0 += 65535) {
        const uint32_t ny = std::min<uint32_t>(65535, nt - t0);
        k_tabs_count<<<dim3(std::max(gx, 1u), ny), 256, 0, st>>>(d_slots, d_base + t0, d_cap + t0, d_cnt + t0);
    }
    PTW_CUDA(cudaGetLastError());
    PTW_CUDA(cub_call([&](void *t, size_t &b) {
        return cub::DeviceScan::InclusiveSum(t, b, d_cnt, d_seg + 1, (int64_t)nt, st);
    }, st));
    std::vector<unsigned long long> h_seg(nt + 1);
    PTW_CUDA(cudaMemcpyAsync(h_seg.data(), d_seg, (nt + 1) * 8ull, cudaMemcpyDeviceToHost, st));
    PTW_CUDA(cudaStreamSynchronize(st));
    const uint64_t n_ent = h_seg[nt];
    std::vector<uint32_t> h_name(n_ent), h_cnt(n_ent);
    if (n_ent) {
        uint32_t *e_name, *e_cnt, *s_name, *s_cnt;
        PTW_CUDA(db.alloc(&e_name, n_ent));
        PTW_CUDA(db.alloc(&e_cnt, n_ent));
        PTW_CUDA(db.alloc(&s_name, n_ent));
        PTW_CUDA(db.alloc(&s_cnt, n_ent));
        for (uint32_t t0 = 0; t0 < nt; t0 += 65535) {
            const uint32_t ny = std::min<uint32_t>(65535, nt - t0);
            k_tabs_emit<<<dim3(std::max(gx, 1u), ny), 256, 0, st>>>(d_slots, d_base + t0, d_cap + t0, d_seg + t0,
                                                                   d_fill + t0, g->dg.int2name, e_name, e_cnt);
        }
        PTW_CUDA(cudaGetLastError());
        PTW_CUDA(cub_call([&](void *t, size_t &b) {
            return cub::DeviceSegmentedSort::SortPairs(t, b, e_name, s_name, e_cnt, s_cnt, (int64_t)n_ent,
                                                      (int64_t)nt, d_seg, d_seg + 1, st);
        }, st));
        PTW_CUDA(cudaMemcpyAsync(h_name.data(), s_name, n_ent * 4, cudaMemcpyDeviceToHost, st));
        PTW_CUDA(cudaMemcpyAsync(h_cnt.data(), s_cnt, n_ent * 4, cudaMemcpyDeviceToHost, st));
        PTW_CUDA(cudaStreamSynchronize(st));
    }
    for (uint32_t i = 0; i < nt; ++i) {
        names[i]->assign(h_name.begin() + h_seg[i], h_name.begin() + h_seg[i + 1]);
        counts[i]->assign(h_cnt.begin() + h_seg[i], h_cnt.begin() + h_seg[i + 1]);
    }
    return PTW_OK;
}

uint64_t table_slots(double sp, uint32_t max_moves, int32_t app, double factor, uint64_t budget, uint32_t n)
{
    const double len = max_moves ? std::min(1.0 / std::max(sp, 1e-12), (double)max_moves)
                                 : 1.0 / std::max(sp, 1e-12);
    const double per_walker = app == PTW_APP_VISITS ? len + 1.0 : 1.0;
    const double f = factor > 0 ? factor : 2.0;
    const double expect = std::ceil(f * per_walker * (double)budget) + 64.0;
    const uint64_t full_cap = next_pow2(2ull * n);
    return std::min(full_cap, std::max<uint64_t>(256, next_pow2((uint64_t)std::min(expect, 4e18))));
}

uint64_t full_table_slots(uint32_t n) { return next_pow2(2ull * n); }

}  // namespace ptw

using namespace ptw;

extern "C" int ptw_ppr_batch(ptw_graph *g, const ptw_query *h_queries, uint32_t nq, const ptw_batch_cfg *cfg,
                             ptw_batch **out)
{
    if (!g || !cfg || !out) return fail(PTW_EINVAL, "null argument");
    *out = nullptr;
    if (nq && !h_queries) return fail(PTW_EINVAL, "null query table");
    if (!(cfg->sp >= 0.0 && cfg->sp <= 1.0)) return fail(PTW_EINVAL, "sp must be in [0, 1]");
    if (cfg->sp == 0.0 && cfg->max_moves == 0)
        return fail(PTW_EINVAL, "sp = 0 needs max_moves > 0 (walks would never end)");
    if (cfg->app != PTW_APP_VISITS && cfg->app != PTW_APP_ENDPOINT) return fail(PTW_EINVAL, "unknown app");
    PTW_CUDA(cudaSetDevice(g->device));
    const uint32_t n = g->dg.n;
    std::vector<WaveQuery> all(nq);
    for (uint32_t i = 0; i < nq; ++i) {
        const ptw_query &q = h_queries[i];
        if (q.budget < 1 || q.budget > kMaxBudget)
            return fail(PTW_EINVAL, "query " + std::to_string(i) + ": budget must be in [1, 2^28]");
        const uint32_t *p = std::lower_bound(g->h_names, g->h_names + n, q.source);
        if (p == g->h_names + n || *p != q.source)
            return fail(PTW_EINVAL, "query " + std::to_string(i) + ": source " + std::to_string(q.source) +
                                        " is not a vertex of the graph");
        all[i].index = i;
        all[i].src = g->h_idx2int[p - g->h_names];
        all[i].qid = q.query_id;
        all[i].budget = q.budget;
        all[i].cap = table_slots(cfg->sp, cfg->max_moves, cfg->app, cfg->table_factor, q.budget, n);
    }
    uint64_t budget_bytes = cfg->table_bytes;
    if (budget_bytes == 0) {
        size_t fr = 0, tot = 0;
        PTW_CUDA(cudaMemGetInfo(&fr, &tot));
        budget_bytes = fr / 4;
    }
    ptw_batch *b = new (std::nothrow) ptw_batch();
    if (!b) return fail(PTW_ENOMEM, "host allocation failed");
    b->nq = nq;
    b->queries.assign(h_queries, h_queries + nq);
    std::vector<std::vector<uint32_t>> names(nq), cnts(nq);
    std::vector<uint32_t> overflow;
    const uint64_t thr = cfg->sp >= 1.0 ? (1ull << 32) : (uint64_t)(cfg->sp * 4294967296.0);
    uint64_t moves = 0;
    PTW_CUDA(cudaEventRecord(g->ev[3], g->stream));
    int rc = PTW_OK;
    // Waves in query order, admitted while their tables fit the budget.
    for (uint32_t i = 0; i < nq && rc == PTW_OK;) {
        std::vector<WaveQuery> wave;
        uint64_t bytes = 0;
        while (i < nq && (wave.empty() || bytes + all[i].cap * 8 <= budget_bytes) && wave.size() < (1u << 20)) {
            bytes += all[i].cap * 8;
            wave.push_back(all[i++]);
        }
        rc = run_wave(g, wave, cfg, thr, names, cnts, overflow, &moves);
    }
    // Queries whose table filled run again with 2n slots (they cannot fill).
    std::vector<uint32_t> again;
    again.swap(overflow);
    for (size_t k = 0; k < again.size() && rc == PTW_OK; ++k) {
        WaveQuery w = all[again[k]];
        w.cap = full_table_slots(n);
        uint64_t m2 = 0;
        rc = run_wave(g, {w}, cfg, thr, names, cnts, overflow, &m2);
        if (rc == PTW_OK && !overflow.empty()) rc = fail(PTW_EFULL, "count table overflow at 2n slots");
    }
    if (rc != PTW_OK) {
        delete b;
        return rc;
    }
    PTW_CUDA(cudaEventRecord(g->ev[2], g->stream));
    PTW_CUDA(cudaEventSynchronize(g->ev[2]));
    b->offsets.assign(nq + 1, 0);
    for (uint32_t i = 0; i < nq; ++i) b->offsets[i + 1] = b->offsets[i] + names[i].size();
    b->names.reserve(b->offsets[nq]);
    b->counts.reserve(b->offsets[nq]);
    uint64_t walkers = 0;
    for (uint32_t i = 0; i < nq; ++i) {
        b->names.insert(b->names.end(), names[i].begin(), names[i].end());
        b->counts.insert(b->counts.end(), cnts[i].begin(), cnts[i].end());
        walkers += all[i].budget;
    }
    b->stats.walkers = walkers;
    b->stats.moves = moves;
    b->stats.visits = cfg->app == PTW_APP_VISITS ? walkers + moves : walkers;
    float ms = 0;
    PTW_CUDA(cudaEventElapsedTime(&ms, g->ev[3], g->ev[2]));
    b->stats.total_ms = ms;
    b->stats.kernel_ms = ms;
    *out = b;
    return PTW_OK;
}

extern "C" int ptw_batch_info(const ptw_batch *b, uint32_t *nq, uint64_t *entries, ptw_walk_stats *stats)
{
    if (!b) return fail(PTW_EINVAL, "null batch");
    if (nq) *nq = b->nq;
    if (entries) *entries = b->offsets.empty() ? 0 : b->offsets.back();
    if (stats) *stats = b->stats;
    return PTW_OK;
}

extern "C" int ptw_batch_export(const ptw_batch *b, uint64_t *h_offsets, uint32_t *h_names, uint32_t *h_counts)
{
    if (!b) return fail(PTW_EINVAL, "null batch");
    if (h_offsets) std::memcpy(h_offsets, b->offsets.data(), b->offsets.size() * 8);
    if (h_names && !b->names.empty()) std::memcpy(h_names, b->names.data(), b->names.size() * 4);
    if (h_counts && !b->counts.empty()) std::memcpy(h_counts, b->counts.data(), b->counts.size() * 4);
    return PTW_OK;
}

extern "C" void ptw_batch_free(ptw_batch *b) { delete b; }
