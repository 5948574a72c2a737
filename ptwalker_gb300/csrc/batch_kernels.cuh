// Kernels shared by the batched PPR/RWR executor (batch.cu) and the serving
// runtime (serve.cu).  See batch.cu for the query-table layout.
#pragma once

#include "ptw_internal.cuh"

namespace ptw {
namespace {

constexpr unsigned kBFull = 0xffffffffu;
constexpr uint32_t kProbeLimit = 256;
// q_mask value of a query whose counts are a dense array of n 32-bit
// counters indexed by canonical vertex index (instead of a hash table).
constexpr uint32_t kDenseMask = 0xFFFFFFFFu;

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

// Adds inc to the count of internal vertex v: in a dense array (mask ==
// kDenseMask) one fire-and-forget reduction at its canonical index, else a
// hash-table insert.
__device__ __forceinline__ void count_add(unsigned long long *tab, uint32_t mask, uint32_t v, uint32_t inc,
                                          uint32_t *flag, const uint32_t *__restrict__ int2idx)
{
    if (mask == kDenseMask) atomicAdd(reinterpret_cast<uint32_t *>(tab) + __ldg(&int2idx[v]), inc);
    else tab_add(tab, mask, v, inc, flag);
}

// Work of one launch: descriptor d runs walker ranks desc[d].y ..
// desc[d].y + desc[d].z - 1 of query entry q = desc[d].x, whose walker ids
// are (q_qid[q] << 32) + rank, source q_src[q], count table at slots +
// q_tab[q] (q_mask[q] + 1 slots, or a dense array when q_mask[q] ==
// kDenseMask).  Descriptors are ordered round-robin over
// the queries (the host builds them so), and a warp takes one descriptor at
// a time, so the walkers in flight belong to many queries at once and no
// single query's hot slots serialise the whole GPU.
struct BatchArgs {
    const uint2 *__restrict__ adj;
    const uint32_t *__restrict__ col;
    const uint4 *__restrict__ col_ext;     // EXT: {id, first column, degree, name} per entry
    const uint32_t *__restrict__ int2idx;  // internal id -> canonical index (dense tables)
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
                                          unsigned long long *tab, uint32_t tmask, uint32_t *flag, uint32_t lane,
                                          const uint32_t *__restrict__ int2idx)
{
    const unsigned m = __ballot_sync(mask_active, on);
    if (!on) return;
    const unsigned long long key = ((unsigned long long)q << 32) | v;
    const unsigned grp = __match_any_sync(m, key);
    if ((grp & ((1u << lane) - 1u)) == 0) count_add(tab, tmask, v, __popc(grp), flag, int2idx);
}

// EXT: moves read the extended column copy and keep the row record of the
// current vertex in registers (one gather per move instead of two).
template <bool EXT>
__global__ void __launch_bounds__(256) k_batch(const BatchArgs a)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t lt_mask = (1u << lane) - 1u;
    uint32_t q[kBatchIlp], v[kBatchIlp], step[kBatchIlp], j[kBatchIlp], qid[kBatchIlp], mask[kBatchIlp];
    unsigned long long *tab[kBatchIlp];
    bool act[kBatchIlp], have[kBatchIlp];
    uint2 rec[kBatchIlp];
#pragma unroll
    for (int k = 0; k < kBatchIlp; ++k) {
        act[k] = have[k] = false;
        q[k] = v[k] = step[k] = j[k] = qid[k] = mask[k] = 0;
        tab[k] = nullptr;
        rec[k] = make_uint2(0u, 0u);
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
                have[k] = false;
            }
            if (a.app == PTW_APP_VISITS) {
                // Start visits: one table update per (warp, query) group.
                visit_agg(kBFull, got, q[k], v[k], tab[k], mask[k], &a.q_flag[q[k]], lane, a.int2idx);
            }
        }
        bool any = false;
#pragma unroll
        for (int k = 0; k < kBatchIlp; ++k) any |= act[k];
        if (!__any_sync(kBFull, any)) break;

#pragma unroll
        for (int k = 0; k < kBatchIlp; ++k)
            if (act[k] && !(EXT && have[k])) rec[k] = __ldg(&a.adj[v[k]]);
        uint4 r[kBatchIlp];
#pragma unroll
        for (int k = 0; k < kBatchIlp; ++k)
            if (act[k]) r[k] = philox(make_uint4(j[k], qid[k], step[k], PTW_TAG_WALK), a.key0, a.key1);
        uint32_t nb[kBatchIlp];
        uint2 nrec[kBatchIlp];
#pragma unroll
        for (int k = 0; k < kBatchIlp; ++k) {
            if (act[k] && rec[k].y != 0) {
                const uint32_t e = rec[k].x + __umulhi(r[k].x, rec[k].y);
                if (EXT) {
                    const uint4 x = __ldg(&a.col_ext[e]);
                    nb[k] = x.x;
                    nrec[k] = make_uint2(x.y, x.z);
                } else {
                    nb[k] = __ldg(&a.col[e]);
                }
            }
        }
#pragma unroll
        for (int k = 0; k < kBatchIlp; ++k) {
            // every lane runs the aggregation calls (warp-collective)
            const bool moved = act[k] && rec[k].y != 0;
            if (moved) {
                v[k] = nb[k];
                if (EXT) {
                    rec[k] = nrec[k];
                    have[k] = true;
                }
                ++step[k];
                ++moves;
            }
            if (a.app == PTW_APP_VISITS)
                visit_agg(kBFull, moved, q[k], v[k], tab[k], mask[k], &a.q_flag[q[k]], lane, a.int2idx);
            const bool done = act[k] && (!moved || (uint64_t)r[k].y < a.thr || (a.max_moves && step[k] >= a.max_moves));
            if (a.app == PTW_APP_ENDPOINT)
                visit_agg(kBFull, done, q[k], v[k], tab[k], mask[k], &a.q_flag[q[k]], lane, a.int2idx);
            if (done) act[k] = false;
        }
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) moves += __shfl_xor_sync(kBFull, moves, o);
    if (lane == 0 && moves) atomicAdd(&a.ctrl[1], moves);
}

// ---- compaction of count tables into (name, count) lists ------------------

// Monotone bin of a count: exact below 256, then 16 bins per octave.
constexpr uint32_t kCountBins = 640;
__device__ __forceinline__ uint32_t count_bin(uint32_t c)
{
    if (c < 256) return c;
    const uint32_t e = 31 - __clz(c);  // 8 .. 31
    return 256 + (e - 8) * 16 + ((c >> (e - 4)) & 15u);
}

// An occupied entry (hash slot with a key, or a nonzero dense counter) whose
// count falls in bin thr or above.
__device__ __forceinline__ bool kept(unsigned long long w, uint32_t thr)
{
    return w != 0 && (thr == 0 || count_bin((uint32_t)(w & 0xFFFFFFFFull)) >= thr);
}

// Entry x of table i: a 64-bit hash slot, or a 32-bit dense counter.
__device__ __forceinline__ unsigned long long table_word(const unsigned long long *s, bool dense, uint64_t x)
{
    return dense ? (unsigned long long)reinterpret_cast<const uint32_t *>(s)[x] : s[x];
}

// Compaction work is cut into chunks of kChunk entries of one table:
// chunk c covers entries [ch[c].y, min(ch[c].y + kChunk, t_cap[t])) of table
// t = ch[c].x, so every block gets the same amount of table to read whatever
// the spread of table sizes.  Table t starts at slots + t_base[t] and has
// t_cap[t] entries: 64-bit hash slots, or 32-bit counters when t_dense[t].
constexpr uint32_t kChunk = 8192;

// Occupied entries per table: one atomic per chunk.
__global__ void __launch_bounds__(256) k_tabs_count(const unsigned long long *slots, const unsigned long long *t_base,
                                                    const uint32_t *t_cap, const uint8_t *t_dense, const uint2 *ch,
                                                    unsigned long long *cnt)
{
    __shared__ uint32_t warp_n[8];
    const uint2 c = ch[blockIdx.x];
    const uint32_t t = c.x;
    const unsigned long long *s = slots + t_base[t];
    const bool dense = t_dense[t] != 0;
    const uint64_t lo = c.y, hi = lo + kChunk < t_cap[t] ? lo + kChunk : t_cap[t];
    uint32_t k = 0;
    for (uint64_t x = lo + threadIdx.x; x < hi; x += 256) k += table_word(s, dense, x) != 0;
    for (int o = 16; o; o >>= 1) k += __shfl_xor_sync(kBFull, k, o);
    if ((threadIdx.x & 31) == 0) warp_n[threadIdx.x >> 5] = k;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t tot = 0;
        for (int w = 0; w < 8; ++w) tot += warp_n[w];
        if (tot) atomicAdd(&cnt[t], (unsigned long long)tot);
    }
}

// Writes each occupied entry of the chunk's table t into the table's
// segment as key (t << name_bits | name) and count, so one radix sort of the
// keys orders every table's entries by name in place.  The block counts its
// chunk's entries, reserves that many positions with a single atomic on the
// table's fill cursor, then writes them (warp offsets through shared
// memory).  Dense tables (entry x = canonical index x, name idx_names[x])
// are emitted the same way.  With t_thr, only entries whose count bin
// (count_bin) is at least t_thr[t] are emitted; with by_count the key is
// (t, ~count, name), which orders each table by count descending, then name
// (the caller checks that it fits 64 bits).  Launch with 256 threads.
__global__ void __launch_bounds__(256) k_tabs_emit(const unsigned long long *slots, const unsigned long long *t_base,
                            const uint32_t *t_cap, const uint8_t *t_dense, const uint2 *ch,
                            const unsigned long long *seg_off, unsigned long long *fill,
                            const uint32_t *int2name, const uint32_t *idx_names, int name_bits,
                            bool by_count, const uint32_t *t_thr, unsigned long long *out_key, uint32_t *out_cnt)
{
    __shared__ uint32_t warp_n[8];
    __shared__ unsigned long long base_s;
    const uint2 chunk = ch[blockIdx.x];
    const uint32_t i = chunk.x;
    const bool dense = t_dense[i] != 0;
    const unsigned long long *s = slots + t_base[i];
    const uint32_t thr = t_thr ? t_thr[i] : 0u;  // keep entries whose count bin >= thr
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint64_t lo = chunk.y, hi = lo + kChunk < t_cap[i] ? lo + kChunk : t_cap[i];
    // pass 1: occupied slots of the chunk
    uint32_t c = 0;
    for (uint64_t x = lo + threadIdx.x; x < hi; x += 256) c += kept(table_word(s, dense, x), thr);
    for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(kBFull, c, o);
    if (lane == 0) warp_n[warp] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int w = 0; w < 8; ++w) t += warp_n[w];
        base_s = t ? atomicAdd(&fill[i], (unsigned long long)t) : 0ull;
    }
    __syncthreads();
    unsigned long long pos0 = seg_off[i] + base_s;
    const unsigned long long tagged = (unsigned long long)i << (by_count ? 32 + name_bits : name_bits);
    // pass 2: tiles of 256 slots in order
    for (uint64_t x0 = lo; x0 < hi; x0 += 256) {
        const uint64_t x = x0 + threadIdx.x;
        unsigned long long w = x < hi ? table_word(s, dense, x) : 0ull;
        if (!kept(w, thr)) w = 0;
        const unsigned om = __ballot_sync(kBFull, w != 0);
        __syncthreads();  // previous tile's readers of warp_n are done
        if (lane == 0) warp_n[warp] = __popc(om);
        __syncthreads();
        uint32_t before = 0, total = 0;
        for (int k = 0; k < 8; ++k) {
            const uint32_t v = warp_n[k];
            before += k < (int)warp ? v : 0u;
            total += v;
        }
        if (w) {
            const unsigned long long p = pos0 + before + __popc(om & ((1u << lane) - 1u));
            const uint32_t cnt = (uint32_t)(w & 0xFFFFFFFFull);
            const unsigned long long inv = by_count ? (unsigned long long)(0xFFFFFFFFu - cnt) << name_bits : 0ull;
            const uint32_t name = dense ? idx_names[x] : int2name[(uint32_t)(w >> 32) - 1];
            out_key[p] = tagged | inv | name;
            out_cnt[p] = cnt;
        }
        pos0 += total;
    }
}

// Top-k selection, histogram: counts of the occupied entries of every table
// with more than k of them, by count_bin, into hist[t * kCountBins + bin].
__global__ void __launch_bounds__(256) k_tabs_hist(const unsigned long long *slots, const unsigned long long *t_base,
                                                   const uint32_t *t_cap, const uint8_t *t_dense, const uint2 *ch,
                                                   const unsigned long long *cnt, uint32_t k, uint32_t *hist)
{
    __shared__ uint32_t h[kCountBins];
    const uint2 c = ch[blockIdx.x];
    const uint32_t i = c.x;
    if (cnt[i] <= k) return;  // every entry is kept
    for (uint32_t b = threadIdx.x; b < kCountBins; b += blockDim.x) h[b] = 0;
    __syncthreads();
    const unsigned long long *s = slots + t_base[i];
    const bool dense = t_dense[i] != 0;
    const uint64_t lo = c.y, hi = lo + kChunk < t_cap[i] ? lo + kChunk : t_cap[i];
    for (uint64_t x = lo + threadIdx.x; x < hi; x += blockDim.x) {
        const unsigned long long w = table_word(s, dense, x);
        if (w) atomicAdd(&h[count_bin((uint32_t)(w & 0xFFFFFFFFull))], 1u);
    }
    __syncthreads();
    for (uint32_t b = threadIdx.x; b < kCountBins; b += blockDim.x)
        if (h[b]) atomicAdd(&hist[(uint64_t)i * kCountBins + b], h[b]);
}

// Top-k selection, threshold: the lowest bin thr[i] such that the entries in
// bins >= thr[i] number at least k (0 = keep every entry when there are at
// most k); sel[i] = how many entries that keeps.  One warp per table.
__global__ void k_tabs_thresh(const unsigned long long *cnt, const uint32_t *hist, uint32_t nt, uint32_t k,
                              uint32_t *thr, unsigned long long *sel)
{
    const uint32_t i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (i >= nt || (threadIdx.x & 31) != 0) return;
    if (cnt[i] <= k) {
        thr[i] = 0;
        sel[i] = cnt[i];
        return;
    }
    const uint32_t *h = hist + (uint64_t)i * kCountBins;
    unsigned long long acc = 0;
    uint32_t b = kCountBins;
    while (b > 0 && acc < k) acc += h[--b];
    thr[i] = b > 0 ? b : 1;  // bin 0 is the empty count and never occupied
    sel[i] = acc;
}

// Sorted hash entries j (keys table << name_bits | name, counts) go to
// position seg[t] + (j - hseg[t]) of their table t's output segment.
__global__ void k_place_hash(const unsigned long long *key, const uint32_t *cnt, uint64_t n, int name_bits,
                             const unsigned long long *seg, const unsigned long long *hseg, uint32_t *out_name,
                             uint32_t *out_cnt)
{
    const unsigned long long nmask = (1ull << name_bits) - 1;
    for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < n; j += (uint64_t)gridDim.x * blockDim.x) {
        const unsigned long long k = key[j];
        const uint32_t t = (uint32_t)(k >> name_bits);
        const uint64_t p = seg[t] + (j - hseg[t]);
        out_name[p] = (uint32_t)(k & nmask);
        out_cnt[p] = cnt[j];
    }
}

// Dense tables in name order without a sort.  Work is cut into warp chunks
// of kWarpChunk counters: warp w of the grid takes chunk c = w % chunks of
// dense table dl[w / chunks] (chunks per table = ceil(n / kWarpChunk)).
constexpr uint32_t kWarpChunk = 256;
constexpr uint32_t kWarpSteps = kWarpChunk / 32;

// Pass 1: nonzero counters per warp chunk -> cc[w], the chunk's loads
// issued together.  (Four chunks per warp measured slower: 224 against
// 147 us on 512 queries at R-MAT scale 20, registers limiting residency.)
constexpr uint32_t kCountChunks = 1;
__global__ void __launch_bounds__(256) k_dense_chunks(const unsigned long long *slots,
                                                      const unsigned long long *t_base, const uint32_t *dl,
                                                      uint32_t n, uint32_t chunks, uint64_t nw,
                                                      unsigned long long *cc)
{
    const uint64_t w0 = ((blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5) * kCountChunks;
    if (w0 >= nw) return;  // whole warp leaves together
    const uint32_t lane = threadIdx.x & 31;
    uint32_t v[kCountChunks][kWarpSteps];
#pragma unroll
    for (uint32_t q = 0; q < kCountChunks; ++q) {
        const uint64_t w = w0 + q;
        const uint32_t *c = w < nw ? reinterpret_cast<const uint32_t *>(slots + t_base[dl[w / chunks]]) : nullptr;
        const uint64_t lo = (w % chunks) * (uint64_t)kWarpChunk;
        const uint64_t hi = lo + kWarpChunk < n ? lo + kWarpChunk : n;
#pragma unroll
        for (uint32_t j = 0; j < kWarpSteps; ++j) {
            const uint64_t x = lo + j * 32 + lane;
            v[q][j] = (c && x < hi) ? c[x] : 0u;
        }
    }
#pragma unroll
    for (uint32_t q = 0; q < kCountChunks; ++q) {
        uint32_t k = 0;
#pragma unroll
        for (uint32_t j = 0; j < kWarpSteps; ++j) k += v[q][j] != 0;
        for (int o = 16; o; o >>= 1) k += __shfl_xor_sync(kBFull, k, o);
        if (lane == 0 && w0 + q < nw) cc[w0 + q] = k;
    }
}

// Pass 2: each warp writes its chunk's nonzero counters in index (= name)
// order at seg[t] + cpos[w] - cpos[table's first chunk] + rank, where cpos is
// the exclusive scan of pass 1; ranks within the chunk come from ballots, so
// no block-wide synchronisation is needed.
__global__ void __launch_bounds__(256) k_dense_place(const unsigned long long *slots,
                                                     const unsigned long long *t_base, const uint32_t *dl,
                                                     uint32_t n, uint32_t chunks, uint64_t nw,
                                                     const unsigned long long *cpos, const unsigned long long *seg,
                                                     const uint32_t *idx_names, uint32_t *out_name, uint32_t *out_cnt)
{
    const uint64_t w = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    if (w >= nw) return;  // whole warp leaves together
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t y = w / chunks;
    const uint32_t t = dl[y];
    const uint32_t *c = reinterpret_cast<const uint32_t *>(slots + t_base[t]);
    const uint64_t lo = (w % chunks) * (uint64_t)kWarpChunk;
    const uint64_t hi = lo + kWarpChunk < n ? lo + kWarpChunk : n;
    unsigned long long pos = seg[t] + cpos[w] - cpos[y * chunks];
    uint32_t v[kWarpSteps];  // the chunk's counters, loaded before any write
#pragma unroll
    for (uint32_t j = 0; j < kWarpSteps; ++j) {
        const uint64_t x = lo + j * 32 + lane;
        v[j] = x < hi ? c[x] : 0u;
    }
#pragma unroll
    for (uint32_t j = 0; j < kWarpSteps; ++j) {
        const unsigned om = __ballot_sync(kBFull, v[j] != 0);
        if (v[j]) {
            const uint64_t x = lo + j * 32 + lane;
            const unsigned long long p = pos + __popc(om & ((1u << lane) - 1u));
            out_name[p] = idx_names[x];
            out_cnt[p] = v[j];
        }
        pos += __popc(om);
    }
}

__global__ void k_key_names(const unsigned long long *key, uint64_t n, unsigned long long mask, uint32_t *name)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        name[i] = (uint32_t)(key[i] & mask);
}

// Top-k, step 1: key (table << 32 | ~count) with the name as value, from the
// (table << name_bits | name) keys and counts of the name-ordered lists.
__global__ void k_count_keys(const unsigned long long *key, const uint32_t *cnt, uint64_t n, int name_bits,
                             unsigned long long *ckey, uint32_t *name)
{
    const unsigned long long mask = (1ull << name_bits) - 1;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const unsigned long long k = key[i];
        ckey[i] = ((k >> name_bits) << 32) | (unsigned long long)(0xFFFFFFFFu - cnt[i]);
        name[i] = (uint32_t)(k & mask);
    }
}

// Top-k, step 2: entry i of the count-ordered lists is rank i - seg[t] of its
// table t; ranks below k go to position kseg[t] + rank of the output.
__global__ void k_topk_copy(const unsigned long long *ckey, const uint32_t *name, uint64_t n,
                            const unsigned long long *seg, const unsigned long long *kseg, uint32_t k,
                            uint32_t *out_name, uint32_t *out_cnt)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const unsigned long long c = ckey[i];
        const uint32_t t = (uint32_t)(c >> 32);
        const uint64_t r = i - seg[t];
        if (r < k) {
            const uint64_t p = kseg[t] + r;
            out_name[p] = name[i];
            out_cnt[p] = 0xFFFFFFFFu - (uint32_t)(c & 0xFFFFFFFFull);
        }
    }
}

// Top-k from (table, ~count, name) keys sorted in one pass: entry i is rank
// i - seg[t] of its table t; ranks below k go to kseg[t] + rank.
__global__ void k_topk_copy_packed(const unsigned long long *key, uint64_t n, int name_bits,
                                   const unsigned long long *seg, const unsigned long long *kseg, uint32_t k,
                                   uint32_t *out_name, uint32_t *out_cnt)
{
    const unsigned long long nmask = (1ull << name_bits) - 1;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const unsigned long long c = key[i];
        const uint32_t t = (uint32_t)(c >> (32 + name_bits));
        const uint64_t r = i - seg[t];
        if (r < k) {
            const uint64_t p = kseg[t] + r;
            out_name[p] = (uint32_t)(c & nmask);
            out_cnt[p] = 0xFFFFFFFFu - (uint32_t)((c >> name_bits) & 0xFFFFFFFFull);
        }
    }
}

}  // namespace
}  // namespace ptw
