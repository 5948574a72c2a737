// Kernels shared by the batched PPR/RWR executor (batch.cu) and the serving
// runtime (serve.cu).  See batch.cu for the query-table layout.
#pragma once

#include "ptw_internal.cuh"

namespace ptw {
namespace {

constexpr unsigned kBFull = 0xffffffffu;
constexpr uint32_t kProbeLimit = 256;

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

// Adds inc to the count of key in the table slots[0 .. mask]; 64-bit slots
// hold (key + 1) << 32 | count.  Sets *flag when no slot is free within the
// probe limit (the caller re-runs that query with a larger table).
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

// Work of one launch: descriptor d runs walker ranks desc[d].y ..
// desc[d].y + desc[d].z - 1 of query entry q = desc[d].x, whose walker ids
// are (q_qid[q] << 32) + rank, source q_src[q], count table at slots +
// q_tab[q] (q_mask[q] + 1 slots).  Descriptors are ordered round-robin over
// the queries (the host builds them so), and a warp takes one descriptor at
// a time, so the walkers in flight belong to many queries at once and no
// single query's hot slots serialise the whole GPU.
struct BatchArgs {
    const uint2 *__restrict__ adj;
    const uint32_t *__restrict__ col;
    const uint3 *__restrict__ desc;  // [ndesc] {entry, first rank, count}
    const uint32_t *__restrict__ q_src;
    const uint32_t *__restrict__ q_qid;
    const unsigned long long *__restrict__ q_tab;
    const uint32_t *__restrict__ q_mask;
    uint32_t *q_flag;
    unsigned long long *slots;
    unsigned long long *ctrl;  // [0] descriptor cursor, [1] moves
    uint32_t ndesc;
    uint64_t thr;
    uint32_t key0, key1, max_moves;
    int app;
};

// Walker ranks per descriptor (host side splits queries into chunks of it).
constexpr uint32_t kDescWalkers = 256;

constexpr int kBatchIlp = 2;

// Counts one visit of key v in query entry q's table, aggregated over the
// lanes of the warp that visit the same (query, vertex) now.
__device__ __forceinline__ void visit_agg(unsigned mask_active, bool on, uint32_t q, uint32_t v,
                                          unsigned long long *tab, uint32_t tmask, uint32_t *flag, uint32_t lane)
{
    const unsigned m = __ballot_sync(mask_active, on);
    if (!on) return;
    const unsigned long long key = ((unsigned long long)q << 32) | v;
    const unsigned grp = __match_any_sync(m, key);
    if ((grp & ((1u << lane) - 1u)) == 0) tab_add(tab, tmask, v, __popc(grp), flag);
}

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
    // Warp-uniform current descriptor: entry dq, ranks [dnext, dend).
    uint32_t dq = 0, dnext = 0, dend = 0;
    bool exhausted = false;
    unsigned long long moves = 0;
    for (;;) {
#pragma unroll
        for (int k = 0; k < kBatchIlp; ++k) {
            const unsigned need = __ballot_sync(kBFull, !act[k]);
            bool got = false;
            if (need != 0 && !exhausted) {
                uint32_t n_need = __popc(need);
                uint32_t rank = __popc(need & lt_mask);
                uint32_t done_before = 0;  // lanes served from earlier descriptors
                // Serve the needing lanes from the current descriptor, then
                // from newly taken ones, until all are served or work ends.
                while (n_need > done_before) {
                    const uint32_t avail = dend - dnext;
                    const uint32_t take = n_need - done_before < avail ? n_need - done_before : avail;
                    if (!act[k] && rank >= done_before && rank < done_before + take) {
                        q[k] = dq;
                        j[k] = dnext + (rank - done_before);
                        got = true;
                    }
                    dnext += take;
                    done_before += take;
                    if (done_before == n_need) break;
                    unsigned long long d = 0;
                    if (lane == 0) d = atomicAdd(&a.ctrl[0], 1ull);
                    d = __shfl_sync(kBFull, d, 0);
                    if (d >= a.ndesc) {
                        exhausted = true;
                        break;
                    }
                    const uint3 ds = a.desc[d];
                    dq = ds.x;
                    dnext = ds.y;
                    dend = ds.y + ds.z;
                }
            }
            if (got) {
                qid[k] = a.q_qid[q[k]];
                v[k] = a.q_src[q[k]];
                tab[k] = a.slots + a.q_tab[q[k]];
                mask[k] = a.q_mask[q[k]];
                step[k] = 0;
                act[k] = true;
            }
            if (a.app == PTW_APP_VISITS) {
                // Start visits: one table update per (warp, query) group.
                visit_agg(kBFull, got, q[k], v[k], tab[k], mask[k], &a.q_flag[q[k]], lane);
            }
        }
        bool any = false;
#pragma unroll
        for (int k = 0; k < kBatchIlp; ++k) any |= act[k];
        if (!__any_sync(kBFull, any)) break;

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
            // every lane runs the aggregation calls (warp-collective)
            const bool moved = act[k] && rec[k].y != 0;
            if (moved) {
                v[k] = nb[k];
                ++step[k];
                ++moves;
            }
            if (a.app == PTW_APP_VISITS) visit_agg(kBFull, moved, q[k], v[k], tab[k], mask[k], &a.q_flag[q[k]], lane);
            const bool done = act[k] && (!moved || (uint64_t)r[k].y < a.thr || (a.max_moves && step[k] >= a.max_moves));
            if (a.app == PTW_APP_ENDPOINT) visit_agg(kBFull, done, q[k], v[k], tab[k], mask[k], &a.q_flag[q[k]], lane);
            if (done) act[k] = false;
        }
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) moves += __shfl_xor_sync(kBFull, moves, o);
    if (lane == 0 && moves) atomicAdd(&a.ctrl[1], moves);
}

// ---- compaction of count tables into (name, count) lists ------------------

// Table i occupies slots[t_base[i] .. t_base[i] + t_cap[i]).  blockIdx.y = i.
__global__ void k_tabs_count(const unsigned long long *slots, const unsigned long long *t_base,
                             const uint32_t *t_cap, unsigned long long *cnt)
{
    const uint32_t i = blockIdx.y;
    const unsigned long long *s = slots + t_base[i];
    const uint32_t cap = t_cap[i];
    uint32_t c = 0;
    for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x < cap; x += gridDim.x * blockDim.x) c += s[x] != 0;
    for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(kBFull, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(&cnt[i], (unsigned long long)c);
}

// Writes each occupied slot of table i (= t_index0 + blockIdx.y) into the
// table's segment as key (i << name_bits | name) and count, so one radix
// sort of the keys orders every table's entries by name in place.
__global__ void k_tabs_emit(const unsigned long long *slots, const unsigned long long *t_base,
                            const uint32_t *t_cap, const unsigned long long *seg_off, unsigned long long *fill,
                            const uint32_t *int2name, uint32_t t_index0, int name_bits,
                            unsigned long long *out_key, uint32_t *out_cnt)
{
    const uint32_t i = blockIdx.y;
    const unsigned long long *s = slots + t_base[i];
    const uint32_t cap = t_cap[i];
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t x0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); x0 < cap; x0 += stride) {
        const uint32_t x = x0 + lane;
        const unsigned long long w = x < cap ? s[x] : 0ull;
        const unsigned om = __ballot_sync(kBFull, w != 0);
        if (!om) continue;
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(&fill[i], (unsigned long long)__popc(om));
        base = __shfl_sync(kBFull, base, 0);
        if (w) {
            const uint64_t pos = seg_off[i] + base + __popc(om & ((1u << lane) - 1u));
            out_key[pos] = ((unsigned long long)(t_index0 + i) << name_bits) | int2name[(uint32_t)(w >> 32) - 1];
            out_cnt[pos] = (uint32_t)(w & 0xFFFFFFFFull);
        }
    }
}

__global__ void k_key_names(const unsigned long long *key, uint64_t n, unsigned long long mask, uint32_t *name)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        name[i] = (uint32_t)(key[i] & mask);
}

}  // namespace
}  // namespace ptw
