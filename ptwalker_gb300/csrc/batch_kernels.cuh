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

// Query table of one launch: entry q runs walkers q_j0[q] .. q_j0[q] +
// (q_off[q+1] - q_off[q]) - 1 of query q_qid[q] from source q_src[q], counting
// into the table at slots + q_tab[q] (q_mask[q] + 1 slots).
struct BatchArgs {
    const uint2 *__restrict__ adj;
    const uint32_t *__restrict__ col;
    const unsigned long long *__restrict__ q_off;  // [nq + 1]
    const unsigned long long *__restrict__ q_j0;   // [nq] or null (= 0)
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

__device__ __forceinline__ uint32_t find_entry(const unsigned long long *off, uint32_t nq, uint64_t g)
{
    uint32_t lo = 0, hi = nq;  // off[lo] <= g < off[hi]
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (off[mid] <= g) lo = mid;
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
            const unsigned need = __ballot_sync(kBFull, !act[k]);
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
                base = __shfl_sync(kBFull, base, 0);
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
                const uint32_t qq = find_entry(a.q_off, a.nq, my);
                q[k] = qq;
                j[k] = (uint32_t)(my - a.q_off[qq] + (a.q_j0 ? a.q_j0[qq] : 0ull));
                qid[k] = a.q_qid[qq];
                v[k] = a.q_src[qq];
                tab[k] = a.slots + a.q_tab[qq];
                mask[k] = a.q_mask[qq];
                step[k] = 0;
                act[k] = true;
            }
            if (a.app == PTW_APP_VISITS) {
                // Start visits: one table update per (warp, query) group.
                const unsigned gm = __ballot_sync(kBFull, got);
                if (got) {
                    const unsigned grp = __match_any_sync(gm, q[k]);
                    if ((grp & lt_mask) == 0) tab_add(tab[k], mask[k], v[k], __popc(grp), &a.q_flag[q[k]]);
                }
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

__global__ void k_tabs_emit(const unsigned long long *slots, const unsigned long long *t_base,
                            const uint32_t *t_cap, const unsigned long long *seg_off, unsigned long long *fill,
                            const uint32_t *int2name, uint32_t *out_name, uint32_t *out_cnt)
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
            out_name[pos] = int2name[(uint32_t)(w >> 32) - 1];
            out_cnt[pos] = (uint32_t)(w & 0xFFFFFFFFull);
        }
    }
}

}  // namespace
}  // namespace ptw
