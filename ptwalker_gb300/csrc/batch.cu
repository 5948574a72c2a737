// Batched single-source PPR / RWR (K4) and the device FP64 oracle (K7/K8).
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

#include "ptw_internal.cuh"

struct ptw_batch {
    uint32_t nq = 0;
    std::vector<ptw_query> queries;
    std::vector<uint64_t> offsets;  // [nq + 1]
    std::vector<uint32_t> names, counts;
    ptw_walk_stats stats{};
};

namespace ptw {
namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr uint32_t kProbeLimit = 256;
constexpr uint64_t kMaxBudget = 1ull << 28;

__device__ __forceinline__ uint32_t mix32(uint32_t x)
{
    // MurmurHash3 32-bit finaliser (Appleby, public domain)
    x ^= x >> 16;
    x *= 0x85ebca6bu;
    x ^= x >> 13;
    x *= 0xc2b2ae35u;
    x ^= x >> 16;
    return x;
}

// Adds inc to the count of key in the table at slots[0 .. mask].
__device__ __forceinline__ void tab_add(unsigned long long *slots, uint32_t mask, uint32_t key, uint32_t inc,
                                        uint32_t *flag)
{
    const unsigned long long tag = (unsigned long long)(key + 1) << 32;
    uint32_t h = mix32(key) & mask;
    for (uint32_t probe = 0; probe < kProbeLimit && probe <= mask; ++probe) {
        unsigned long long *s = slots + h;
        unsigned long long cur = *(volatile unsigned long long *)s;
        if ((cur & 0xFFFFFFFF00000000ull) == tag) {
            atomicAdd(s, (unsigned long long)inc);
            return;
        }
        if (cur == 0) {
            const unsigned long long prev = atomicCAS(s, 0ull, tag | inc);
            if (prev == 0) return;
            if ((prev & 0xFFFFFFFF00000000ull) == tag) {
                atomicAdd(s, (unsigned long long)inc);
                return;
            }
        }
        h = (h + 1) & mask;
    }
    atomicOr(flag, 1u);
}

struct BatchArgs {
    const uint2 *__restrict__ adj;
    const uint32_t *__restrict__ col;
    const unsigned long long *__restrict__ q_off;  // [nq + 1]
    const uint32_t *__restrict__ q_src;
    const uint32_t *__restrict__ q_qid;
    const unsigned long long *__restrict__ q_tab;
    const uint32_t *__restrict__ q_mask;
    uint32_t *q_flag;
    unsigned long long *slots;
    unsigned long long *ctrl;  // [0] cursor, [1] moves
    uint64_t total;
    uint64_t thr;
    uint32_t nq, key0, key1, max_moves, chunk;
    int app;
};

__device__ __forceinline__ uint32_t find_query(const unsigned long long *q_off, uint32_t nq, uint64_t g)
{
    uint32_t lo = 0, hi = nq;  // q_off[lo] <= g < q_off[hi]
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (q_off[mid] <= g) lo = mid;
        else hi = mid;
    }
    return lo;
}

constexpr int kBatchIlp = 2;

__global__ void __launch_bounds__(256) k_batch(const BatchArgs a)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t lt_mask = (1u << lane) - 1u;
    uint32_t q[kBatchIlp], v[kBatchIlp], step[kBatchIlp], j[kBatchIlp], qid[kBatchIlp], mask[kBatchIlp];
    unsigned long long *tab[kBatchIlp];
    bool act[kBatchIlp];
#pragma unroll
    for (int k = 0; k < kBatchIlp; ++k) {
        act[k] = false;
        q[k] = v[k] = step[k] = j[k] = qid[k] = mask[k] = 0;
        tab[k] = nullptr;
    }
    uint64_t next = 0, end = 0;
    bool exhausted = false;
    unsigned long long moves = 0;
    for (;;) {
#pragma unroll
        for (int k = 0; k < kBatchIlp; ++k) {
            const unsigned need = __ballot_sync(kFull, !act[k]);
            if (need == 0 || exhausted) continue;
            const uint32_t n_need = __popc(need);
            const uint32_t rank = __popc(need & lt_mask);
            uint64_t my = ~0ull;
            const uint64_t avail = end - next;
            const uint32_t took = (uint32_t)(n_need < avail ? n_need : avail);
            if (!act[k] && rank < took) my = next + rank;
            next += took;
            if (took < n_need) {
                unsigned long long base = 0;
                if (lane == 0) base = atomicAdd(&a.ctrl[0], (unsigned long long)a.chunk);
                base = __shfl_sync(kFull, base, 0);
                if (base >= a.total) {
                    exhausted = true;
                    next = end = a.total;
                } else {
                    next = base;
                    end = base + a.chunk < a.total ? base + a.chunk : a.total;
                    const uint64_t rem = end - next;
                    const uint32_t take2 = (uint32_t)((n_need - took) < rem ? (n_need - took) : rem);
                    if (!act[k] && rank >= took && rank - took < take2) my = next + (rank - took);
                    next += take2;
                }
            }
            const bool got = my != ~0ull;
            if (got) {
                const uint32_t qq = find_query(a.q_off, a.nq, my);
                q[k] = qq;
                j[k] = (uint32_t)(my - a.q_off[qq]);
                qid[k] = a.q_qid[qq];
                v[k] = a.q_src[qq];
                tab[k] = a.slots + a.q_tab[qq];
                mask[k] = a.q_mask[qq];
                step[k] = 0;
                act[k] = true;
            }
            if (a.app == PTW_APP_VISITS) {
                // Start visits: one table update per (warp, query) group.
                const unsigned gm = __ballot_sync(kFull, got);
                if (got) {
                    const unsigned grp = __match_any_sync(gm, q[k]);
                    if ((grp & lt_mask) == 0) tab_add(tab[k], mask[k], v[k], __popc(grp), &a.q_flag[q[k]]);
                }
            }
        }
        bool any = false;
#pragma unroll
        for (int k = 0; k < kBatchIlp; ++k) any |= act[k];
        if (!__any_sync(kFull, any)) break;

        uint2 rec[kBatchIlp];
#pragma unroll
        for (int k = 0; k < kBatchIlp; ++k)
            if (act[k]) rec[k] = __ldg(&a.adj[v[k]]);
        uint4 r[kBatchIlp];
#pragma unroll
        for (int k = 0; k < kBatchIlp; ++k)
            if (act[k]) r[k] = philox(make_uint4(j[k], qid[k], step[k], PTW_TAG_WALK), a.key0, a.key1);
        uint32_t nb[kBatchIlp];
#pragma unroll
        for (int k = 0; k < kBatchIlp; ++k)
            if (act[k] && rec[k].y != 0) nb[k] = __ldg(&a.col[rec[k].x + __umulhi(r[k].x, rec[k].y)]);
#pragma unroll
        for (int k = 0; k < kBatchIlp; ++k) {
            if (!act[k]) continue;
            bool done;
            if (rec[k].y == 0) {
                done = true;
            } else {
                v[k] = nb[k];
                ++step[k];
                ++moves;
                if (a.app == PTW_APP_VISITS) tab_add(tab[k], mask[k], v[k], 1u, &a.q_flag[q[k]]);
                done = (uint64_t)r[k].y < a.thr || (a.max_moves && step[k] >= a.max_moves);
            }
            if (done) {
                if (a.app == PTW_APP_ENDPOINT) tab_add(tab[k], mask[k], v[k], 1u, &a.q_flag[q[k]]);
                act[k] = false;
            }
        }
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) moves += __shfl_xor_sync(kFull, moves, o);
    if (lane == 0 && moves) atomicAdd(&a.ctrl[1], moves);
}

// Slot s of the wave belongs to the query q with q_tab[q] <= s < q_tab[q+1].
__device__ __forceinline__ uint32_t slot_query(const unsigned long long *q_tab, uint32_t nq, uint64_t s)
{
    uint32_t lo = 0, hi = nq;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (q_tab[mid] <= s) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Per-query number of occupied slots (warp-aggregated per query).
__global__ void k_tab_count(const unsigned long long *slots, uint64_t n_slots,
                            const unsigned long long *q_tab, uint32_t nq, unsigned long long *cnt)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t s0 = blockIdx.x * (uint64_t)blockDim.x + (threadIdx.x & ~31u); s0 < n_slots; s0 += stride) {
        const uint64_t s = s0 + lane;
        const bool occ = s < n_slots && slots[s] != 0;
        const unsigned om = __ballot_sync(kFull, occ);
        if (occ) {
            const uint32_t qq = slot_query(q_tab, nq, s);
            const unsigned grp = __match_any_sync(om, qq);
            if ((grp & ((1u << lane) - 1u)) == 0) atomicAdd(&cnt[qq], (unsigned long long)__popc(grp));
        }
    }
}

// Writes each occupied slot as (name, count) into its query's segment.
__global__ void k_tab_emit(const unsigned long long *slots, uint64_t n_slots, const unsigned long long *q_tab,
                           uint32_t nq, const unsigned long long *seg_off, unsigned long long *fill,
                           const uint32_t *int2name, uint32_t *out_name, uint32_t *out_cnt)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t s0 = blockIdx.x * (uint64_t)blockDim.x + (threadIdx.x & ~31u); s0 < n_slots; s0 += stride) {
        const uint64_t s = s0 + lane;
        const unsigned long long w = s < n_slots ? slots[s] : 0ull;
        const bool occ = w != 0;
        const unsigned om = __ballot_sync(kFull, occ);
        if (occ) {
            const uint32_t qq = slot_query(q_tab, nq, s);
            const unsigned grp = __match_any_sync(om, qq);
            const int leader = __ffs(grp) - 1;
            unsigned long long base = 0;
            if (lane == (uint32_t)leader) base = atomicAdd(&fill[qq], (unsigned long long)__popc(grp));
            base = __shfl_sync(grp, base, leader);
            const uint64_t pos = seg_off[qq] + base + __popc(grp & ((1u << lane) - 1u));
            out_name[pos] = int2name[(uint32_t)(w >> 32) - 1];
            out_cnt[pos] = (uint32_t)(w & 0xFFFFFFFFull);
        }
    }
}

uint64_t next_pow2(uint64_t x)
{
    uint64_t p = 1;
    while (p < x) p <<= 1;
    return p;
}

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

// Runs one wave; appends each query's sorted entries to per-query host lists.
int run_wave(ptw_graph *g, const std::vector<WaveQuery> &wq, const ptw_batch_cfg *cfg, uint64_t thr,
             std::vector<std::vector<uint32_t>> &names, std::vector<std::vector<uint32_t>> &cnts,
             std::vector<uint32_t> &overflow, uint64_t *moves_out)
{
    cudaStream_t st = g->stream;
    const uint32_t nq = (uint32_t)wq.size();
    std::vector<unsigned long long> h_off(nq + 1), h_tab(nq + 1);
    std::vector<uint32_t> h_src(nq), h_qid(nq), h_mask(nq);
    for (uint32_t i = 0; i < nq; ++i) {
        h_off[i + 1] = h_off[i] + wq[i].budget;
        h_tab[i + 1] = h_tab[i] + wq[i].cap;
        h_src[i] = wq[i].src;
        h_qid[i] = wq[i].qid;
        h_mask[i] = (uint32_t)(wq[i].cap - 1);
    }
    const uint64_t total = h_off[nq], n_slots = h_tab[nq];
    DevBuf db(st);
    unsigned long long *d_off, *d_tab, *d_slots, *d_ctrl, *d_cnt, *d_seg, *d_fill;
    uint32_t *d_src, *d_qid, *d_mask, *d_flag;
    PTW_CUDA(db.alloc(&d_off, nq + 1));
    PTW_CUDA(db.alloc(&d_tab, nq + 1));
    PTW_CUDA(db.alloc(&d_src, nq));
    PTW_CUDA(db.alloc(&d_qid, nq));
    PTW_CUDA(db.alloc(&d_mask, nq));
    PTW_CUDA(db.alloc(&d_flag, nq));
    PTW_CUDA(db.alloc(&d_ctrl, 2));
    PTW_CUDA(db.alloc(&d_cnt, nq));
    PTW_CUDA(db.alloc(&d_seg, nq + 1));
    PTW_CUDA(db.alloc(&d_fill, nq));
    PTW_CUDA(db.alloc(&d_slots, n_slots));
    PTW_CUDA(cudaMemcpyAsync(d_off, h_off.data(), (nq + 1) * 8ull, cudaMemcpyHostToDevice, st));
    PTW_CUDA(cudaMemcpyAsync(d_tab, h_tab.data(), (nq + 1) * 8ull, cudaMemcpyHostToDevice, st));
    PTW_CUDA(cudaMemcpyAsync(d_src, h_src.data(), nq * 4ull, cudaMemcpyHostToDevice, st));
    PTW_CUDA(cudaMemcpyAsync(d_qid, h_qid.data(), nq * 4ull, cudaMemcpyHostToDevice, st));
    PTW_CUDA(cudaMemcpyAsync(d_mask, h_mask.data(), nq * 4ull, cudaMemcpyHostToDevice, st));
    PTW_CUDA(cudaMemsetAsync(d_flag, 0, nq * 4ull, st));
    PTW_CUDA(cudaMemsetAsync(d_ctrl, 0, 16, st));
    PTW_CUDA(cudaMemsetAsync(d_cnt, 0, nq * 8ull, st));
    PTW_CUDA(cudaMemsetAsync(d_fill, 0, nq * 8ull, st));
    PTW_CUDA(cudaMemsetAsync(d_slots, 0, n_slots * 8, st));

    BatchArgs a;
    a.adj = g->dg.adj;
    a.col = g->dg.col;
    a.q_off = d_off;
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

    const unsigned sgrid = (unsigned)std::min<uint64_t>((n_slots + 255) / 256, (uint64_t)g->num_sms * 32);
    k_tab_count<<<std::max(sgrid, 1u), 256, 0, st>>>(d_slots, n_slots, d_tab, nq, d_cnt);
    PTW_CUDA(cudaMemsetAsync(d_seg, 0, 8, st));
    PTW_CUDA(cub_call([&](void *t, size_t &b) {
        return cub::DeviceScan::InclusiveSum(t, b, d_cnt, d_seg + 1, (int64_t)nq, st);
    }, st));
    std::vector<unsigned long long> h_seg(nq + 1);
    std::vector<uint32_t> h_flag(nq);
    unsigned long long h_moves = 0;
    PTW_CUDA(cudaMemcpyAsync(h_seg.data(), d_seg, (nq + 1) * 8ull, cudaMemcpyDeviceToHost, st));
    PTW_CUDA(cudaMemcpyAsync(h_flag.data(), d_flag, nq * 4ull, cudaMemcpyDeviceToHost, st));
    PTW_CUDA(cudaMemcpyAsync(&h_moves, d_ctrl + 1, 8, cudaMemcpyDeviceToHost, st));
    PTW_CUDA(cudaStreamSynchronize(st));
    *moves_out += h_moves;
    const uint64_t n_ent = h_seg[nq];
    uint32_t *e_name, *e_cnt, *s_name, *s_cnt;
    PTW_CUDA(db.alloc(&e_name, n_ent));
    PTW_CUDA(db.alloc(&e_cnt, n_ent));
    PTW_CUDA(db.alloc(&s_name, n_ent));
    PTW_CUDA(db.alloc(&s_cnt, n_ent));
    if (n_ent) {
        k_tab_emit<<<std::max(sgrid, 1u), 256, 0, st>>>(d_slots, n_slots, d_tab, nq, d_seg, d_fill,
                                                        g->dg.int2name, e_name, e_cnt);
        PTW_CUDA(cudaGetLastError());
        PTW_CUDA(cub_call([&](void *t, size_t &b) {
            return cub::DeviceSegmentedSort::SortPairs(t, b, e_name, s_name, e_cnt, s_cnt, (int64_t)n_ent,
                                                      (int64_t)nq, d_seg, d_seg + 1, st);
        }, st));
    }
    std::vector<uint32_t> h_name(n_ent), h_cnt(n_ent);
    if (n_ent) {
        PTW_CUDA(cudaMemcpyAsync(h_name.data(), s_name, n_ent * 4, cudaMemcpyDeviceToHost, st));
        PTW_CUDA(cudaMemcpyAsync(h_cnt.data(), s_cnt, n_ent * 4, cudaMemcpyDeviceToHost, st));
    }
    PTW_CUDA(cudaStreamSynchronize(st));
    for (uint32_t i = 0; i < nq; ++i) {
        const uint32_t qi = wq[i].index;
        if (h_flag[i]) {
            overflow.push_back(qi);
            continue;
        }
        names[qi].assign(h_name.begin() + h_seg[i], h_name.begin() + h_seg[i + 1]);
        cnts[qi].assign(h_cnt.begin() + h_seg[i], h_cnt.begin() + h_seg[i + 1]);
    }
    return PTW_OK;
}

}  // namespace

const ptw_query *batch_queries(const ptw_batch *b) { return b->queries.data(); }

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
    // Queries -> internal sources and table sizes.
    std::vector<WaveQuery> all(nq);
    const double len = cfg->max_moves ? std::min(1.0 / std::max(cfg->sp, 1e-12), (double)cfg->max_moves)
                                      : 1.0 / std::max(cfg->sp, 1e-12);
    const double per_walker = cfg->app == PTW_APP_VISITS ? len + 1.0 : 1.0;
    const uint64_t full_cap = next_pow2(2ull * n);
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
        const double factor = cfg->table_factor > 0 ? cfg->table_factor : 2.0;
        const double expect = std::ceil(factor * per_walker * (double)q.budget) + 64.0;
        all[i].cap = std::min(full_cap, std::max<uint64_t>(256, next_pow2((uint64_t)expect)));
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
        while (i < nq && (wave.empty() || bytes + all[i].cap * 8 <= budget_bytes) &&
               wave.size() < (1u << 20)) {
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
        w.cap = full_cap;
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
