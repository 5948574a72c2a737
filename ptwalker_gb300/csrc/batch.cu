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
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "batch_kernels.cuh"

struct ptw_batch {
    uint32_t nq = 0;
    std::vector<ptw_query> queries;
    std::vector<uint64_t> offsets;  // [nq + 1]
    std::unique_ptr<uint32_t[]> names, counts;
    ptw_walk_stats stats{};
    uint32_t top_k = 0;  // results hold each query's top_k largest counts only
};

namespace ptw {
namespace {
// Result of one wave: its queries (caller indices, in wave order), their
// compacted entries, and which of them overflowed (entries to be replaced).
struct WaveResult {
    std::vector<uint32_t> idx;
    Compacted c;
    std::vector<char> overflow;
};
}  // namespace
}  // namespace ptw

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
        cudaError_t e = pooled_alloc_async(&q, std::max<uint64_t>(count, 1) * sizeof(T), st);
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
    e = pooled_alloc_async(&tmp, std::max<size_t>(bytes, 16), st);
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

}  // namespace

// Splits [j0, j0 + count) of every entry into descriptors of at most
// kDescWalkers ranks, ordered round-robin over the entries.
void interleave_descriptors(const std::vector<uint64_t> &j0, const std::vector<uint64_t> &count,
                            std::vector<uint3> &desc)
{
    desc.clear();
    std::vector<uint32_t> live;
    for (uint32_t i = 0; i < count.size(); ++i)
        if (count[i]) live.push_back(i);
    for (uint64_t r = 0; !live.empty(); ++r) {
        size_t keep = 0;
        for (uint32_t i : live) {
            const uint64_t off = r * kDescWalkers;
            const uint64_t c = std::min<uint64_t>(kDescWalkers, count[i] - off);
            desc.push_back(make_uint3(i, (uint32_t)(j0[i] + off), (uint32_t)c));
            if (off + c < count[i]) live[keep++] = i;
        }
        live.resize(keep);
    }
}

namespace {

// Runs one wave; stores each query's sorted entries in per-query host lists.
int run_wave(ptw_graph *g, const std::vector<WaveQuery> &wq, const ptw_batch_cfg *cfg, uint64_t thr,
             std::vector<WaveResult> &waves, std::vector<uint32_t> &overflow, uint64_t *moves_out,
             float *walk_ms)
{
    cudaStream_t st = g->stream;
    const uint32_t nq = (uint32_t)wq.size();
    std::vector<unsigned long long> h_tab(nq + 1);
    std::vector<uint32_t> h_src(nq), h_qid(nq), h_mask(nq), h_cap(nq);
    std::vector<uint64_t> j0(nq, 0), cnt(nq);
    for (uint32_t i = 0; i < nq; ++i) {
        h_tab[i + 1] = h_tab[i] + wq[i].cap;
        h_src[i] = wq[i].src;
        h_qid[i] = wq[i].qid;
        h_mask[i] = (uint32_t)(wq[i].cap - 1);
        h_cap[i] = (uint32_t)wq[i].cap;
        cnt[i] = wq[i].budget;
    }
    std::vector<uint3> h_desc;
    interleave_descriptors(j0, cnt, h_desc);
    const uint64_t n_slots = h_tab[nq], nd = h_desc.size();
    DevBuf db(st);
    unsigned long long *d_tab, *d_slots, *d_ctrl;
    uint32_t *d_src, *d_qid, *d_mask, *d_flag;
    uint3 *d_desc;
    PTW_CUDA(db.alloc(&d_tab, nq + 1));
    PTW_CUDA(db.alloc(&d_src, nq));
    PTW_CUDA(db.alloc(&d_qid, nq));
    PTW_CUDA(db.alloc(&d_mask, nq));
    PTW_CUDA(db.alloc(&d_flag, nq));
    PTW_CUDA(db.alloc(&d_ctrl, 2));
    PTW_CUDA(db.alloc(&d_desc, nd));
    PTW_CUDA(db.alloc(&d_slots, n_slots));
    PTW_CUDA(cudaMemcpyAsync(d_tab, h_tab.data(), (nq + 1) * 8ull, cudaMemcpyHostToDevice, st));
    PTW_CUDA(cudaMemcpyAsync(d_src, h_src.data(), nq * 4ull, cudaMemcpyHostToDevice, st));
    PTW_CUDA(cudaMemcpyAsync(d_qid, h_qid.data(), nq * 4ull, cudaMemcpyHostToDevice, st));
    PTW_CUDA(cudaMemcpyAsync(d_mask, h_mask.data(), nq * 4ull, cudaMemcpyHostToDevice, st));
    PTW_CUDA(cudaMemcpyAsync(d_desc, h_desc.data(), nd * sizeof(uint3), cudaMemcpyHostToDevice, st));
    PTW_CUDA(cudaMemsetAsync(d_flag, 0, nq * 4ull, st));
    PTW_CUDA(cudaMemsetAsync(d_ctrl, 0, 16, st));
    PTW_CUDA(cudaMemsetAsync(d_slots, 0, n_slots * 8, st));

    BatchArgs a;
    a.adj = g->dg.adj;
    a.col = g->dg.col;
    a.desc = d_desc;
    a.q_src = d_src;
    a.q_qid = d_qid;
    a.q_tab = d_tab;
    a.q_mask = d_mask;
    a.q_flag = d_flag;
    a.slots = d_slots;
    a.ctrl = d_ctrl;
    a.ndesc = (uint32_t)nd;
    a.thr = thr;
    a.key0 = (uint32_t)cfg->seed;
    a.key1 = (uint32_t)(cfg->seed >> 32);
    a.max_moves = cfg->max_moves;
    a.app = cfg->app;
    if (nd >= (1ull << 32)) return fail(PTW_EINVAL, "wave too large");
    int per_sm = 0;
    PTW_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch, 256, 0));
    uint64_t grid = (uint64_t)g->num_sms * std::max(per_sm, 1);
    grid = std::min<uint64_t>(grid, std::max<uint64_t>(1, (nd + 7) / 8));
    PTW_CUDA(cudaEventRecord(g->ev[0], st));
    k_batch<<<(unsigned)grid, 256, 0, st>>>(a);
    PTW_CUDA(cudaEventRecord(g->ev[1], st));
    PTW_CUDA(cudaGetLastError());
    std::vector<uint32_t> h_flag(nq);
    unsigned long long h_moves = 0;
    PTW_CUDA(cudaMemcpyAsync(h_flag.data(), d_flag, nq * 4ull, cudaMemcpyDeviceToHost, st));
    PTW_CUDA(cudaMemcpyAsync(&h_moves, d_ctrl + 1, 8, cudaMemcpyDeviceToHost, st));
    WaveResult wr;
    wr.c.top_k = cfg->top_k;
    int rc = compact_tables(g, d_slots, h_tab.data(), h_cap.data(), nq, &wr.c);
    if (rc) return rc;
    float ms = 0;
    PTW_CUDA(cudaEventElapsedTime(&ms, g->ev[0], g->ev[1]));
    *walk_ms += ms;
    *moves_out += h_moves;
    if (std::getenv("PTW_TIMING"))
        std::fprintf(stderr, "[ptw] wave of %u queries, %llu descriptors, %llu slots: walk kernel %.1f ms\n", nq,
                     (unsigned long long)nd, (unsigned long long)n_slots, ms);
    wr.idx.resize(nq);
    wr.overflow.assign(nq, 0);
    for (uint32_t i = 0; i < nq; ++i) {
        wr.idx[i] = wq[i].index;
        if (h_flag[i]) {
            overflow.push_back(wq[i].index);
            wr.overflow[i] = 1;
        }
    }
    waves.push_back(std::move(wr));
    return PTW_OK;
}

// Concatenates the waves' entries in caller query order.  One wave holding
// every query in order (the common case) is adopted without a copy.
int assemble(ptw_batch *b, std::vector<WaveResult> &waves)
{
    const uint32_t nq = b->nq;
    std::vector<const WaveResult *> src_w(nq, nullptr);
    std::vector<uint32_t> src_i(nq, 0);
    for (const WaveResult &w : waves)
        for (uint32_t k = 0; k < w.idx.size(); ++k)
            if (!w.overflow[k]) {
                src_w[w.idx[k]] = &w;
                src_i[w.idx[k]] = k;
            }
    b->offsets.assign(nq + 1, 0);
    for (uint32_t i = 0; i < nq; ++i) {
        const WaveResult *w = src_w[i];
        const uint64_t len = w ? w->c.seg[src_i[i] + 1] - w->c.seg[src_i[i]] : 0;
        b->offsets[i + 1] = b->offsets[i] + len;
    }
    const uint64_t total = b->offsets[nq];
    bool adopt = waves.size() == 1 && waves[0].idx.size() == nq;
    if (adopt)
        for (uint32_t k = 0; k < nq; ++k) adopt = adopt && waves[0].idx[k] == k && !waves[0].overflow[k];
    if (adopt) {
        b->names = std::move(waves[0].c.names);
        b->counts = std::move(waves[0].c.counts);
        return PTW_OK;
    }
    if (!total) return PTW_OK;
    b->names.reset(new (std::nothrow) uint32_t[total]);
    b->counts.reset(new (std::nothrow) uint32_t[total]);
    if (!b->names || !b->counts) return fail(PTW_ENOMEM, "host allocation of batch results failed");
    for (uint32_t i = 0; i < nq; ++i) {
        const WaveResult *w = src_w[i];
        if (!w) continue;
        const uint64_t a = w->c.seg[src_i[i]], len = b->offsets[i + 1] - b->offsets[i];
        std::memcpy(b->names.get() + b->offsets[i], w->c.names.get() + a, len * 4);
        std::memcpy(b->counts.get() + b->offsets[i], w->c.counts.get() + a, len * 4);
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
uint32_t batch_top_k(const ptw_batch *b) { return b->top_k; }

int compact_tables(ptw_graph *g, unsigned long long *d_slots, const unsigned long long *h_base,
                   const uint32_t *h_cap, uint32_t nt, Compacted *out)
{
    out->n = 0;
    out->seg.assign(nt + 1, 0);
    out->names.reset();
    out->counts.reset();
    out->h_names = out->h_counts = nullptr;
    if (nt == 0) return PTW_OK;
    cudaStream_t st = g->stream;
    const bool timing = std::getenv("PTW_TIMING") != nullptr;
    auto clk = [] { return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count(); };
    const double t0 = timing ? (cudaStreamSynchronize(st), clk()) : 0.0;
    double t1 = 0, t2 = 0;
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
    PTW_CUDA(cudaMemcpyAsync(out->seg.data(), d_seg, (nt + 1) * 8ull, cudaMemcpyDeviceToHost, st));
    PTW_CUDA(cudaStreamSynchronize(st));
    const uint64_t n_ent = out->seg[nt];
    // top-k: every table keeps its min(k, entries) largest counts
    const uint32_t k = out->top_k;
    std::vector<uint64_t> kseg;
    uint64_t n_out = n_ent;
    if (k && n_ent) {
        kseg.assign(nt + 1, 0);
        for (uint32_t i = 0; i < nt; ++i)
            kseg[i + 1] = kseg[i] + std::min<uint64_t>(k, out->seg[i + 1] - out->seg[i]);
        n_out = kseg[nt];
    }
    out->n = n_out;
    if (n_ent) {
        if (out->sink) {
            uint32_t *base = out->sink(n_out);
            if (!base) return fail(PTW_ENOMEM, "host staging of results failed");
            out->h_names = base;
            out->h_counts = base + n_out;
        } else {
            out->names.reset(new (std::nothrow) uint32_t[n_out]);  // no value-initialisation
            out->counts.reset(new (std::nothrow) uint32_t[n_out]);
            if (!out->names || !out->counts) return fail(PTW_ENOMEM, "host allocation of batch results failed");
            out->h_names = out->names.get();
            out->h_counts = out->counts.get();
        }
        int name_bits = 1, q_bits = 1;
        while (name_bits < 32 && (1ull << name_bits) < g->dg.id_bound) ++name_bits;
        while ((1ull << q_bits) < nt) ++q_bits;
        unsigned long long *e_key, *s_key;
        uint32_t *e_cnt, *s_cnt, *s_name;
        PTW_CUDA(db.alloc(&e_key, n_ent));
        PTW_CUDA(db.alloc(&s_key, n_ent));
        PTW_CUDA(db.alloc(&e_cnt, n_ent));
        PTW_CUDA(db.alloc(&s_cnt, n_ent));
        // top-k with (table, ~count, name) in 64 bits: one sort, keys only
        const bool packed = k && q_bits + 32 + name_bits <= 64;
        for (uint32_t t0 = 0; t0 < nt; t0 += 65535) {
            const uint32_t ny = std::min<uint32_t>(65535, nt - t0);
            k_tabs_emit<<<dim3(std::max(gx, 1u), ny), 256, 0, st>>>(d_slots, d_base + t0, d_cap + t0, d_seg + t0,
                                                                   d_fill + t0, g->dg.int2name, t0, name_bits,
                                                                   packed, e_key, e_cnt);
        }
        PTW_CUDA(cudaGetLastError());
        const unsigned kg = (unsigned)std::min<uint64_t>((n_ent + 255) / 256, (uint64_t)g->num_sms * 32);
        uint32_t *o_name = nullptr, *o_cnt = nullptr;
        if (packed) {
            PTW_CUDA(cub_call([&](void *t, size_t &b) {
                return cub::DeviceRadixSort::SortKeys(t, b, e_key, s_key, (int64_t)n_ent, 0,
                                                      q_bits + 32 + name_bits, st);
            }, st));
        } else {
            // one radix sort over (table, name): tables stay in their segments
            PTW_CUDA(cub_call([&](void *t, size_t &b) {
                return cub::DeviceRadixSort::SortPairs(t, b, e_key, s_key, e_cnt, s_cnt, (int64_t)n_ent, 0,
                                                       name_bits + q_bits, st);
            }, st));
        }
        if (packed) {
            unsigned long long *d_kseg;
            PTW_CUDA(db.alloc(&d_kseg, nt + 1));
            PTW_CUDA(db.alloc(&o_name, n_out));
            PTW_CUDA(db.alloc(&o_cnt, n_out));
            PTW_CUDA(cudaMemcpyAsync(d_kseg, kseg.data(), (nt + 1) * 8ull, cudaMemcpyHostToDevice, st));
            k_topk_copy_packed<<<std::max(kg, 1u), 256, 0, st>>>(s_key, n_ent, name_bits, d_seg, d_kseg, k, o_name,
                                                                 o_cnt);
            PTW_CUDA(cudaGetLastError());
            out->seg = kseg;
        } else if (k) {
            // re-key by (table, count descending) with the name as value; the
            // radix sort is stable, so equal counts stay in name order
            k_count_keys<<<std::max(kg, 1u), 256, 0, st>>>(s_key, s_cnt, n_ent, name_bits, e_key, e_cnt);
            PTW_CUDA(cudaGetLastError());
            PTW_CUDA(cub_call([&](void *t, size_t &b) {
                return cub::DeviceRadixSort::SortPairs(t, b, e_key, s_key, e_cnt, s_cnt, (int64_t)n_ent, 0,
                                                       32 + q_bits, st);
            }, st));
            unsigned long long *d_kseg;
            PTW_CUDA(db.alloc(&d_kseg, nt + 1));
            PTW_CUDA(db.alloc(&o_name, n_out));
            PTW_CUDA(db.alloc(&o_cnt, n_out));
            PTW_CUDA(cudaMemcpyAsync(d_kseg, kseg.data(), (nt + 1) * 8ull, cudaMemcpyHostToDevice, st));
            k_topk_copy<<<std::max(kg, 1u), 256, 0, st>>>(s_key, s_cnt, n_ent, d_seg, d_kseg, k, o_name, o_cnt);
            PTW_CUDA(cudaGetLastError());
            out->seg = kseg;
        } else {
            s_name = (uint32_t *)e_key;  // reuse the unsorted-key buffer
            k_key_names<<<std::max(kg, 1u), 256, 0, st>>>(s_key, n_ent, (1ull << name_bits) - 1, s_name);
            PTW_CUDA(cudaGetLastError());
            o_name = s_name;
            o_cnt = s_cnt;
        }
        if (timing) {
            PTW_CUDA(cudaStreamSynchronize(st));
            t1 = clk();
        }
        PTW_CUDA(cudaMemcpyAsync(out->h_names, o_name, n_out * 4, cudaMemcpyDeviceToHost, st));
        PTW_CUDA(cudaMemcpyAsync(out->h_counts, o_cnt, n_out * 4, cudaMemcpyDeviceToHost, st));
        PTW_CUDA(cudaStreamSynchronize(st));
        if (timing) t2 = clk();
    }
    if (timing)
        std::fprintf(stderr, "[ptw] compact %u tables, %llu entries: device %.1f ms, d2h %.1f ms\n", nt,
                     (unsigned long long)n_ent, 1e3 * (t1 - t0), 1e3 * (t2 - t1));
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
    std::vector<WaveResult> waves;
    std::vector<uint32_t> overflow;
    const uint64_t thr = cfg->sp >= 1.0 ? (1ull << 32) : (uint64_t)(cfg->sp * 4294967296.0);
    uint64_t moves = 0;
    float walk_ms = 0;
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
        rc = run_wave(g, wave, cfg, thr, waves, overflow, &moves, &walk_ms);
    }
    // Queries whose table filled run again with 2n slots (they cannot fill).
    std::vector<uint32_t> again;
    again.swap(overflow);
    for (size_t k = 0; k < again.size() && rc == PTW_OK; ++k) {
        WaveQuery w = all[again[k]];
        w.cap = full_table_slots(n);
        uint64_t m2 = 0;
        rc = run_wave(g, {w}, cfg, thr, waves, overflow, &m2, &walk_ms);
        if (rc == PTW_OK && !overflow.empty()) rc = fail(PTW_EFULL, "count table overflow at 2n slots");
    }
    if (rc == PTW_OK) rc = assemble(b, waves);
    if (rc != PTW_OK) {
        delete b;
        return rc;
    }
    PTW_CUDA(cudaEventRecord(g->ev[2], g->stream));
    PTW_CUDA(cudaEventSynchronize(g->ev[2]));
    uint64_t walkers = 0;
    for (uint32_t i = 0; i < nq; ++i) walkers += all[i].budget;
    b->top_k = cfg->top_k;
    b->stats.walkers = walkers;
    b->stats.moves = moves;
    b->stats.visits = cfg->app == PTW_APP_VISITS ? walkers + moves : walkers;
    float ms = 0;
    PTW_CUDA(cudaEventElapsedTime(&ms, g->ev[3], g->ev[2]));
    b->stats.total_ms = ms;
    b->stats.kernel_ms = walk_ms;  // walker kernels only; total_ms includes compaction and copies
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
    const uint64_t n = b->offsets.empty() ? 0 : b->offsets.back();
    if (h_offsets) std::memcpy(h_offsets, b->offsets.data(), b->offsets.size() * 8);
    if (h_names && n) std::memcpy(h_names, b->names.get(), n * 4);
    if (h_counts && n) std::memcpy(h_counts, b->counts.get(), n * 4);
    return PTW_OK;
}

extern "C" int ptw_batch_view(const ptw_batch *b, const uint64_t **offsets, const uint32_t **names,
                              const uint32_t **counts)
{
    if (!b) return fail(PTW_EINVAL, "null batch");
    if (offsets) *offsets = b->offsets.data();
    if (names) *names = b->names.get();
    if (counts) *counts = b->counts.get();
    return PTW_OK;
}

extern "C" void ptw_batch_free(ptw_batch *b) { delete b; }
