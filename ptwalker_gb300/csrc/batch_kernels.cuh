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
// kDenseMask) one fire-and-forget reduction at v's canonical index idx,
// else a hash-table insert of v.
__device__ __forceinline__ void count_add(unsigned long long *tab, uint32_t mask, uint32_t v, uint32_t idx,
                                          uint32_t inc, uint32_t *flag, uint32_t n, unsigned long long *check)
{
    if (mask == kDenseMask) atomicAdd(reinterpret_cast<uint32_t *>(tab) + PTW_IDX(idx, n, check, kCheckTable), inc);
    else tab_add(tab, mask, v, inc, flag);
    (void)n;
    (void)check;
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
    uint32_t ext_idx;  // 1: names are 0..n-1, so an extended column's name is the canonical index
    const uint3 *__restrict__ desc;  // [ndesc] {entry, first rank, count}
    const uint32_t *__restrict__ q_src;
    const uint32_t *__restrict__ q_qid;
    const unsigned long long *__restrict__ q_tab;
    const uint32_t *__restrict__ q_mask;
    uint32_t *q_flag;
    unsigned long long *slots;
    unsigned long long *ctrl;  // [0] descriptor cursor, [1] moves
    unsigned long long *check; // index-check word (checked build)
    uint64_t n_slots;          // slots of all tables (index checks)
    uint64_t m;                // CSR entries (index checks)
    uint32_t n, nq;            // vertices, query entries (index checks)
    uint32_t ndesc;
    uint64_t thr;
    uint32_t key0, key1, max_moves;
    int app;
};

// Walker ranks per descriptor (host side splits queries into chunks of it).
constexpr uint32_t kDescWalkers = 256;

constexpr int kBatchIlp = 2;

// Counts one visit of key v (canonical index idx, used by dense tables) in
// query entry q's table, aggregated over the lanes of the warp that visit
// the same (query, vertex) now.
__device__ __forceinline__ void visit_agg(unsigned mask_active, bool on, uint32_t q, uint32_t v, uint32_t idx,
                                          unsigned long long *tab, uint32_t tmask, uint32_t *flag, uint32_t lane,
                                          const BatchArgs &a)
{
    const unsigned m = __ballot_sync(mask_active, on);
    if (!on) return;
    const unsigned long long key = ((unsigned long long)q << 32) | v;
    const unsigned grp = __match_any_sync(m, key);
    if ((grp & ((1u << lane) - 1u)) == 0) count_add(tab, tmask, v, idx, __popc(grp), flag, a.n, a.check);
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
                q[k] = (uint32_t)PTW_IDX(q[k], a.nq, a.check, kCheckQuery);
                qid[k] = a.q_qid[q[k]];
                v[k] = a.q_src[q[k]];
                tab[k] = a.slots + a.q_tab[q[k]];
                mask[k] = a.q_mask[q[k]];
#ifdef PTW_CHECKED
                {
                    const uint64_t tslots = mask[k] == kDenseMask ? ((uint64_t)a.n + 1) / 2 : (uint64_t)mask[k] + 1;
                    if (a.q_tab[q[k]] + tslots > a.n_slots) {  // table outside the slots: count into slot 0
                        atomicOr(a.check, 1ull << kCheckTable);
                        tab[k] = a.slots;
                        mask[k] = 0;
                    }
                }
#endif
                step[k] = 0;
                act[k] = true;
                have[k] = false;
            }
            if (a.app == PTW_APP_VISITS) {
                // Start visits: one table update per (warp, query) group.
                const uint32_t sidx =
                    got && mask[k] == kDenseMask ? __ldg(&a.int2idx[PTW_IDX(v[k], a.n, a.check, kCheckCounter)]) : 0u;
                visit_agg(kBFull, got, q[k], v[k], sidx, tab[k], mask[k], &a.q_flag[q[k]], lane, a);
            }
        }
        bool any = false;
#pragma unroll
        for (int k = 0; k < kBatchIlp; ++k) any |= act[k];
        if (!__any_sync(kBFull, any)) break;

#pragma unroll
        for (int k = 0; k < kBatchIlp; ++k)
            if (act[k] && !(EXT && have[k])) rec[k] = __ldg(&a.adj[PTW_IDX(v[k], a.n, a.check, kCheckRecord)]);
        uint4 r[kBatchIlp];
#pragma unroll
        for (int k = 0; k < kBatchIlp; ++k)
            if (act[k]) r[k] = philox(make_uint4(j[k], qid[k], step[k], PTW_TAG_WALK), a.key0, a.key1);
        uint32_t nb[kBatchIlp], nidx[kBatchIlp];
        uint2 nrec[kBatchIlp];
#pragma unroll
        for (int k = 0; k < kBatchIlp; ++k) {
            nidx[k] = 0;
            if (act[k] && rec[k].y != 0) {
                const uint32_t e = rec[k].x + __umulhi(r[k].x, rec[k].y);
                if (EXT) {
                    const uint4 x = __ldg(&a.col_ext[PTW_IDX(e, a.m, a.check, kCheckColumn)]);
                    nb[k] = x.x;
                    nrec[k] = make_uint2(x.y, x.z);
                    nidx[k] = x.w;  // the neighbour's name: its canonical index when a.ext_idx
                } else {
                    nb[k] = __ldg(&a.col[PTW_IDX(e, a.m, a.check, kCheckColumn)]);
                }
            }
        }
        // Canonical indices of the new vertices for dense tables, every
        // slot's load issued before any table update waits on one (with
        // a.ext_idx the gathered column entry already holds it).
#pragma unroll
        for (int k = 0; k < kBatchIlp; ++k)
            if (act[k] && rec[k].y != 0 && mask[k] == kDenseMask && !(EXT && a.ext_idx))
                nidx[k] = __ldg(&a.int2idx[PTW_IDX(nb[k], a.n, a.check, kCheckCounter)]);
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
                visit_agg(kBFull, moved, q[k], v[k], nidx[k], tab[k], mask[k], &a.q_flag[q[k]], lane, a);
            const bool done = act[k] && (!moved || (uint64_t)r[k].y < a.thr || (a.max_moves && step[k] >= a.max_moves));
            if (a.app == PTW_APP_ENDPOINT) {
                // a walker stuck at its start (no out-edge) ends where it began
                const uint32_t eidx =
                    moved ? nidx[k]
                          : done && mask[k] == kDenseMask ? __ldg(&a.int2idx[PTW_IDX(v[k], a.n, a.check, kCheckCounter)])
                                                          : 0u;
                visit_agg(kBFull, done, q[k], v[k], eidx, tab[k], mask[k], &a.q_flag[q[k]], lane, a);
            }
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

// Compaction reads the count tables in block chunks of 16 KB of one table
// (4,096 dense counters or 2,048 hash slots): one 256-thread block per
// chunk, 2 KB per warp, four 16-byte loads per lane issued together, so
// that with four or more blocks per SM enough bytes are in flight to stream
// the tables at HBM rate (the placement pass also keeps every kept entry's
// name in registers, which bounds the chunk).  Table t starts at slots +
// t_base[t] on a 16-byte boundary (128 bytes in practice) and has t_len[t]
// entries (32-bit counters when t_dense[t], else 64-bit hash slots holding
// (key + 1) << 32 | count); its chunks are tch[t] .. tch[t + 1] - 1 of the
// grid.  A lane's last 16-byte word may reach past the table's last entry
// (still inside its allocation); those entries are masked.
constexpr uint32_t kChunkBytes = 16384;
constexpr uint32_t kLaneVecs = kChunkBytes / 16 / 256;  // 16-byte words per lane

// The block's table (the last table whose first chunk is at or below the
// block index; tables without chunks are skipped over) and chunk.
struct Chunk {
    uint32_t t;
    bool dense;
    uint64_t first;       // table entry of the chunk's first entry
    uint32_t n;           // entries in the chunk
    const uint4 *p;       // the chunk's first 16-byte word
};

__device__ __forceinline__ uint32_t chunk_table(const unsigned long long *tch, uint32_t nt, unsigned long long b)
{
    uint32_t lo = 0, hi = nt;  // tch[lo] <= b < tch[hi]
    while (hi - lo > 1) {
        const uint32_t mid = lo + (hi - lo) / 2;
        if (tch[mid] <= b) lo = mid;
        else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ Chunk chunk_of(uint32_t t, unsigned long long b, const unsigned long long *slots,
                                          const unsigned long long *t_base, const uint32_t *t_len,
                                          const uint8_t *t_dense, const unsigned long long *tch)
{
    Chunk c;
    c.t = t;
    c.dense = t_dense[c.t] != 0;
    const uint32_t per = c.dense ? kChunkBytes / 4 : kChunkBytes / 8;
    c.first = (uint64_t)(b - tch[c.t]) * per;
    const uint64_t left = t_len[c.t] - c.first;
    c.n = (uint32_t)(left < per ? left : per);
    c.p = reinterpret_cast<const uint4 *>(slots + t_base[c.t]) + (c.dense ? c.first / 4 : c.first / 2);
    return c;
}

// The block's chunk: thread 0 looks the table up, the block synchronises.
__device__ __forceinline__ Chunk block_chunk(const unsigned long long *slots, const unsigned long long *t_base,
                                             const uint32_t *t_len, const uint8_t *t_dense,
                                             const unsigned long long *tch, uint32_t nt, uint32_t *s_t)
{
    if (threadIdx.x == 0) *s_t = chunk_table(tch, nt, blockIdx.x);
    __syncthreads();
    return chunk_of(*s_t, blockIdx.x, slots, t_base, t_len, t_dense, tch);
}

// Chunk b for one warp, without a block-wide synchronisation.
__device__ __forceinline__ Chunk warp_chunk(unsigned long long b, const unsigned long long *slots,
                                            const unsigned long long *t_base, const uint32_t *t_len,
                                            const uint8_t *t_dense, const unsigned long long *tch, uint32_t nt)
{
    uint32_t t = 0;
    if ((threadIdx.x & 31) == 0) t = chunk_table(tch, nt, b);
    t = __shfl_sync(kBFull, t, 0);
    return chunk_of(t, b, slots, t_base, t_len, t_dense, tch);
}

// Word j of the lane: chunk word w = warp * 32 * kLaneVecs + j * 32 + lane
// (coalesced per j), entries w * EPV .. w * EPV + EPV - 1 of the chunk.
template <int EPV>
__device__ __forceinline__ void load_chunk(const Chunk &c, uint4 (&v)[kLaneVecs])
{
    const uint32_t w0 = (threadIdx.x >> 5) * (32 * kLaneVecs) + (threadIdx.x & 31);
    const uint32_t words = (c.n + EPV - 1) / EPV;
#pragma unroll
    for (uint32_t j = 0; j < kLaneVecs; ++j) {
        const uint32_t w = w0 + 32 * j;
        v[j] = w < words ? ld_stream_u4(c.p + w) : make_uint4(0u, 0u, 0u, 0u);
    }
}

// Entry e of word j: its count and, for a hash slot, key + 1 (0 = empty).
template <int EPV>
__device__ __forceinline__ void word_entry(const uint4 &x, int e, uint32_t &count, uint32_t &tag)
{
    if (EPV == 4) {
        count = e == 0 ? x.x : e == 1 ? x.y : e == 2 ? x.z : x.w;
        tag = count;
    } else {
        count = e == 0 ? x.x : x.z;
        tag = e == 0 ? x.y : x.w;
    }
}

// Pass 1: occupied entries per warp piece of a chunk (cc[b * 8 + warp], and
// hc for hash tables only; the pieces in this order are the tables' entries
// in order) and per table (cnt); with HIST also each table's histogram of
// count_bin over its occupied entries (hist[t * kCountBins + bin]), for
// top-k selection.
template <int EPV, bool HIST>
__device__ __forceinline__ uint32_t count_chunk(const Chunk &c, uint32_t *h)
{
    uint4 v[kLaneVecs];
    load_chunk<EPV>(c, v);
    const uint32_t w0 = (threadIdx.x >> 5) * (32 * kLaneVecs) + (threadIdx.x & 31);
    uint32_t k = 0;
#pragma unroll
    for (uint32_t j = 0; j < kLaneVecs; ++j)
#pragma unroll
        for (int e = 0; e < EPV; ++e) {
            uint32_t cnt, tag;
            word_entry<EPV>(v[j], e, cnt, tag);
            if (tag != 0 && (w0 + 32 * j) * EPV + e < c.n) {
                ++k;
                if (HIST) atomicAdd(&h[count_bin(cnt)], 1u);
            }
        }
    return k;
}

template <bool HIST>
__global__ void __launch_bounds__(256) k_tabs_count(const unsigned long long *slots, const unsigned long long *t_base,
                                                    const uint32_t *t_len, const uint8_t *t_dense,
                                                    const unsigned long long *tch, uint32_t nt,
                                                    unsigned long long *cnt, unsigned long long *cc,
                                                    unsigned long long *hc, uint32_t *hist)
{
    __shared__ uint32_t s_t;
    __shared__ uint32_t warp_n[8];
    __shared__ uint32_t h[HIST ? kCountBins : 1];
    if (HIST)
        for (uint32_t b = threadIdx.x; b < kCountBins; b += 256) h[b] = 0;
    const Chunk c = block_chunk(slots, t_base, t_len, t_dense, tch, nt, &s_t);  // synchronises
    uint32_t k = c.dense ? count_chunk<4, HIST>(c, h) : count_chunk<2, HIST>(c, h);
    for (int o = 16; o; o >>= 1) k += __shfl_xor_sync(kBFull, k, o);
    if ((threadIdx.x & 31) == 0) {
        const uint64_t wi = (uint64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
        warp_n[threadIdx.x >> 5] = k;
        cc[wi] = k;
        hc[wi] = c.dense ? 0u : k;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t tot = 0;
        for (int w = 0; w < 8; ++w) tot += warp_n[w];
        if (tot) atomicAdd(&cnt[c.t], (unsigned long long)tot);
    }
    if (HIST)
        for (uint32_t b = threadIdx.x; b < kCountBins; b += 256)
            if (h[b]) atomicAdd(&hist[(uint64_t)c.t * kCountBins + b], h[b]);
}

// Pass 2: writes the chunk's kept entries in entry order.
//  Full lists (TOPK false): a dense chunk's (name, count) pairs go straight
//  to the output at pos[b] (name order = index order); a hash chunk's names
//  and counts go to the sort input at hpos[b], which keeps each hash table's
//  entries in one range (sorted by name within it afterwards).
//  Top-k (TOPK true): entries whose count bin is at least thr[t] go to the
//  sort input as (t, ~count, name) keys (by_count) or (t << name_bits |
//  name) keys with counts, at sseg[t] + a block reservation on fill[t].
// pos and hpos are exclusive scans of pass 1's cc and hc over the warp
// pieces in table order, so pos[b * 8 + warp] is also the output position of
// a dense piece.  Warps work on their own: ranks come from a warp scan of
// per-word counts packed one byte per word, top-k reserves per warp, and
// each warp stages its kept entries (name, count) in rank order in its part
// of shared memory, so the stores to global memory are whole coalesced rows
// and the kernel has no block-wide synchronisation.
constexpr uint32_t kWarpStage = 32 * kLaneVecs * 4;

template <int EPV, bool TOPK>
__device__ __forceinline__ void place_chunk(const Chunk &c, uint32_t thr, uint32_t *s_nm, uint32_t *s_ct,
                                            unsigned long long *__restrict__ fill, unsigned long long base,
                                            const uint32_t *__restrict__ int2name,
                                            const uint32_t *__restrict__ idx_names, int name_bits, bool by_count,
                                            uint32_t *__restrict__ out_name, uint32_t *__restrict__ out_cnt,
                                            unsigned long long *__restrict__ key_out, uint32_t *__restrict__ cnt_out)
{
    uint4 v[kLaneVecs];
    load_chunk<EPV>(c, v);
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t w0 = warp * (32 * kLaneVecs) + lane;
    // A dense piece's names are contiguous and do not depend on its
    // counters: they are loaded together with them (16 bytes per whole word).
    uint4 nv[kLaneVecs];
#pragma unroll
    for (uint32_t j = 0; j < kLaneVecs; ++j) {
        const uint32_t x = (w0 + 32 * j) * EPV;
        nv[j] = EPV == 4 && x + 4 <= c.n
                    ? ld_stream_u4(reinterpret_cast<const uint4 *>(idx_names + c.first + x))
                    : make_uint4(0u, 0u, 0u, 0u);
    }
    uint32_t km = 0;  // kept entries, bit j * EPV + e
    unsigned long long packed = 0;
#pragma unroll
    for (uint32_t j = 0; j < kLaneVecs; ++j) {
        uint32_t n_j = 0;
#pragma unroll
        for (int e = 0; e < EPV; ++e) {
            uint32_t cnt, tag;
            word_entry<EPV>(v[j], e, cnt, tag);
            const bool keep = tag != 0 && (w0 + 32 * j) * EPV + e < c.n && (!TOPK || count_bin(cnt) >= thr);
            km |= (uint32_t)keep << (j * EPV + e);
            n_j += keep;
        }
        packed |= (unsigned long long)n_j << (8 * j);
    }
    // Names of the kept entries, all loads issued before any is used (they
    // land while the ranks are scanned): for a dense piece from the names
    // loaded above (scalar loads for the table's last, partial word), for a
    // hash slot int2name[key].
    uint32_t nm[kLaneVecs][EPV];
#pragma unroll
    for (uint32_t j = 0; j < kLaneVecs; ++j) {
        const uint32_t wm = (km >> (j * EPV)) & ((1u << EPV) - 1u);
        const uint64_t x0 = c.first + (uint64_t)(w0 + 32 * j) * EPV;
        if (EPV == 4) {
            if ((w0 + 32 * j) * EPV + 4 <= c.n) {
                nm[j][0] = nv[j].x;
                nm[j][1] = nv[j].y;
                nm[j][2 % EPV] = nv[j].z;
                nm[j][3 % EPV] = nv[j].w;
            } else {
#pragma unroll
                for (int e = 0; e < EPV; ++e) nm[j][e] = (wm >> e) & 1u ? idx_names[x0 + e] : 0u;
            }
        } else {
#pragma unroll
            for (int e = 0; e < EPV; ++e) {
                uint32_t cnt, tag;
                word_entry<EPV>(v[j], e, cnt, tag);
                nm[j][e] = (wm >> e) & 1u ? int2name[tag - 1] : 0u;
            }
        }
    }
    // per-word inclusive scan over the lanes; a byte never exceeds 32 * EPV
    unsigned long long inc = packed;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long y = __shfl_up_sync(kBFull, inc, o);
        if (lane >= (uint32_t)o) inc += y;
    }
    const unsigned long long tot = __shfl_sync(kBFull, inc, 31);
    const unsigned long long exc = inc - packed;
    uint32_t wsum = 0;
#pragma unroll
    for (uint32_t j = 0; j < kLaneVecs; ++j) wsum += (uint32_t)(tot >> (8 * j)) & 0xFFu;
    if (TOPK) {
        unsigned long long r0 = 0;
        if (lane == 0 && wsum) r0 = atomicAdd(&fill[c.t], (unsigned long long)wsum);
        base += __shfl_sync(kBFull, r0, 0);
    }
    // stage in warp-local rank order, then write whole rows
    uint32_t *wn = s_nm, *wc = s_ct;  // this warp's part of shared memory
    uint32_t jb = 0;
#pragma unroll
    for (uint32_t j = 0; j < kLaneVecs; ++j) {
        uint32_t r = jb + ((uint32_t)(exc >> (8 * j)) & 0xFFu);
#pragma unroll
        for (int e = 0; e < EPV; ++e) {
            if (!((km >> (j * EPV + e)) & 1u)) continue;
            uint32_t cnt, tag;
            word_entry<EPV>(v[j], e, cnt, tag);
            wn[r] = nm[j][e];
            wc[r] = cnt;
            ++r;
        }
        jb += (uint32_t)(tot >> (8 * j)) & 0xFFu;
    }
    __syncwarp();
    const unsigned long long p = base;
    const unsigned long long tagged = (unsigned long long)c.t << (by_count ? 32 + name_bits : name_bits);
    for (uint32_t i = lane; i < wsum; i += 32) {
        const uint32_t name = wn[i], cnt = wc[i];
        if (TOPK) {
            const unsigned long long inv = by_count ? (unsigned long long)(0xFFFFFFFFu - cnt) << name_bits : 0ull;
            key_out[p + i] = tagged | inv | name;
        } else {
            out_name[p + i] = name;
        }
        (TOPK ? cnt_out : out_cnt)[p + i] = cnt;
    }
}

// Block i of a launch works on chunk chunk0 + i (a launch may cover the
// chunks of a range of tables).
template <bool TOPK>
__global__ void __launch_bounds__(256, 4) k_tabs_place(const unsigned long long *slots, const unsigned long long *t_base,
                                                       const uint32_t *t_len, const uint8_t *t_dense,
                                                       const unsigned long long *tch, uint32_t nt,
                                                       unsigned long long chunk0,
                                                       const unsigned long long *pos, const unsigned long long *hpos,
                                                       const uint32_t *t_thr, const unsigned long long *sseg,
                                                       unsigned long long *fill, const uint32_t *int2name,
                                                       const uint32_t *idx_names, int name_bits, bool by_count,
                                                       uint32_t *out_name, uint32_t *out_cnt, uint32_t *h_name,
                                                       uint32_t *h_cnt, unsigned long long *key_out,
                                                       uint32_t *cnt_out)
{
    __shared__ uint32_t s_nm[8 * kWarpStage], s_ct[8 * kWarpStage];
    const uint32_t warp = threadIdx.x >> 5;
    const unsigned long long b = chunk0 + blockIdx.x;
    const Chunk c = warp_chunk(b, slots, t_base, t_len, t_dense, tch, nt);
    const uint32_t thr = TOPK ? t_thr[c.t] : 0u;
    if (TOPK && sseg[c.t + 1] == sseg[c.t]) return;  // nothing kept in this table (warp-uniform)
    const uint64_t wi = b * 8 + warp;
    const unsigned long long base = TOPK ? sseg[c.t] : c.dense ? pos[wi] : hpos[wi];
    uint32_t *wn = s_nm + warp * kWarpStage, *wc = s_ct + warp * kWarpStage;
    if (c.dense)
        place_chunk<4, TOPK>(c, thr, wn, wc, fill, base, int2name, idx_names, name_bits, by_count, out_name,
                             out_cnt, key_out, cnt_out);
    else
        place_chunk<2, TOPK>(c, thr, wn, wc, fill, base, int2name, idx_names, name_bits, by_count, h_name, h_cnt,
                             key_out, cnt_out);
}

// Top-k selection, threshold: the lowest bin thr[i] such that the entries in
// bins >= thr[i] number at least k (0 = keep every entry when there are at
// most k); sel[i] = how many entries that keeps.  One warp per table: lane l
// sums the strip of 20 bins l-th from the top, a scan over the lanes finds
// the strip where the running count from the top reaches k, and that lane
// walks its strip down to the bin.
constexpr uint32_t kThreshStrip = kCountBins / 32;
static_assert(kCountBins % 32 == 0, "bins split into 32 strips");

__global__ void k_tabs_thresh(const unsigned long long *cnt, const uint32_t *hist, uint32_t nt, uint32_t k,
                              uint32_t *thr, unsigned long long *sel)
{
    const uint32_t i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const uint32_t lane = threadIdx.x & 31;
    if (i >= nt) return;  // whole warp leaves together
    if (cnt[i] <= k) {
        if (lane == 0) {
            thr[i] = 0;
            sel[i] = cnt[i];
        }
        return;
    }
    const uint32_t *h = hist + (uint64_t)i * kCountBins;
    const uint32_t top = kCountBins - kThreshStrip * lane;  // strip [top - kThreshStrip, top)
    unsigned long long strip = 0;
    for (uint32_t b = top - kThreshStrip; b < top; ++b) strip += h[b];
    unsigned long long inc = strip;  // entries in strips 0 .. lane (from the top)
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long y = __shfl_up_sync(kBFull, inc, o);
        if (lane >= (uint32_t)o) inc += y;
    }
    // cnt[i] > k entries in all bins, so some lane's running count reaches k
    // (lane 31, the bottom strip, otherwise: it ends at bin 1 with them all)
    const unsigned reach = __ballot_sync(kBFull, inc >= k);
    const uint32_t first = reach ? __ffs(reach) - 1 : 31u;
    if (lane == first) {
        unsigned long long acc = inc - strip;
        uint32_t b = top;
        while (b > top - kThreshStrip && acc < k) acc += h[--b];
        thr[i] = b > 0 ? b : 1;  // bin 0 is the empty count and never occupied
        sel[i] = acc;
    }
}

// Hash entries j in [j0, j1), sorted by name within their table t's range
// [hseg[t], hseg[t + 1]), go to position seg[t] + (j - hseg[t]) of the
// output.
__global__ void k_place_hash(const uint32_t *name, const uint32_t *cnt, uint64_t j0, uint64_t j1,
                             const unsigned long long *hseg, uint32_t nt, const unsigned long long *seg,
                             uint32_t *out_name, uint32_t *out_cnt)
{
    for (uint64_t j = j0 + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < j1;
         j += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t lo = 0, hi = nt;  // hseg[lo] <= j < hseg[hi]
        while (hi - lo > 1) {
            const uint32_t mid = lo + (hi - lo) / 2;
            if (hseg[mid] <= j) lo = mid;
            else hi = mid;
        }
        const uint64_t p = seg[lo] + (j - hseg[lo]);
        out_name[p] = name[j];
        out_cnt[p] = cnt[j];
    }
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
