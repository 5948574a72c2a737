// Second-order (node2vec) walks for sm_103a.
//
// The reference parses -p / -q (include/option.hpp:447-469), builds a
// neighbour query for them (src/core/graph.hpp:787-820: a Bloom filter over
// the edges, then a binary search in the sorted row) and marks its solver
// for node2vec (src/core/node2vec.cpp:8-24, src/core/solver.hpp:156-159);
// its test states the law (src/test/debug/test_node2vec.cpp with
// third_party/knightking/test_node2vec.hpp:47-80): from v, reached from t,
// the next vertex x is drawn over v's row with weight 1/p if x == t, 1 if x
// is an out-neighbour of t, 1/q otherwise; the first move is uniform.
//
// k_lane_paths draws by rejection over v's row.  Trial k of move s takes two
// words of Philox(ctr = (wid_lo, wid_hi, s, "N2" + k/2)) -- (x, y) for even
// k, (z, w) for odd k --, reads the candidate's extended column entry
// {id, first column, degree, name} (one 16-byte gather: the candidate's own
// row record comes with it) and accepts iff the second word is below the
// threshold of the candidate's class.  Most trials are decided without the
// neighbour query: a return to t is known from the id, a word below both
// the neighbour and the other threshold accepts and a word above both
// rejects.  Only the words between them ask whether the candidate x is an
// out-neighbour of t, the way the reference's has_neighbor does
// (src/core/graph.hpp:811-820): a Bloom filter over the edges first, then a
// binary search of t's row for x's name (rows are in ascending name order)
// only when the filter does not rule the edge out.  The filter is blocked:
// one 32-byte block per edge key, one bit in each of its 8 words, so a test
// is one sector read; at 16 bits per edge (15.5 edges per block at R-MAT
// scale 24) a non-edge passes with probability E[(1 - (31/32)^k)^8] over
// Poisson block loads k, about 0.1%.
// On a graph whose edges all have their reverse, the search takes the
// shorter of the two rows (x in t's row, or t in x's row).
//
// Outlier folding (KnightKing, Yang et al., SOSP'19) for a small p: when
// the return weight 1/p is the only largest weight and the graph is simple
// and symmetric (t then appears exactly once in v's row), the envelope is
// M' = max(1, 1/q) and the return edge's excess sits in an appendix of
// a = (1/p - M') / M' slots beside the row.  In fixed point (2^20 units per
// slot, a_fx = floor(a * 2^20)) the trial's first word places the point
// pos = floor(cu * (degree * 2^20 + a_fx) / 2^32): pos >= degree * 2^20 goes
// back to t with no read at all, else the candidate is entry pos >> 20,
// accepted against thresholds relative to M'.  On R-MAT scale 24, p = 0.25,
// q = 4 takes 13.1 candidate draws per move without folding and 3.3 with it.
//
// Trial 65535 is accepted whatever its word, so every move ends; the host
// keeps max(w) / min(w) <= 1024, which puts that cap below 1e-27 per move.
//
// Each walker's path is staged in a shared-memory row and written out in
// segments of up to 32 positions.
#include <algorithm>

#include "ptw_internal.cuh"

namespace ptw {
namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kLaneWarps = 4;                // warps per block
constexpr uint32_t kN2vMaxTrials = 65536u;  // trials per move before the last is taken

// MurmurHash3 64-bit finaliser (Appleby, public domain).
__host__ __device__ __forceinline__ uint64_t fmix64(uint64_t k)
{
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdull;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ull;
    k ^= k >> 33;
    return k;
}

// Filter block of the directed edge (u, v) (internal ids) and the bit of
// each of its 8 words.
struct FilterKey {
    uint64_t block;
    uint64_t bits;  // 5 bits per word
};

__device__ __forceinline__ FilterKey filter_key(uint32_t u, uint32_t v, uint64_t blocks)
{
    const uint64_t key = ((uint64_t)u << 32) | v;
    return FilterKey{fmix64(key) & (blocks - 1), fmix64(key + 0x9E3779B97F4A7C15ull)};
}

// One warp per vertex: sets the bits of every out-edge.
__global__ void k_build_edge_filter(const uint2 *__restrict__ adj, const uint32_t *__restrict__ col, uint32_t n,
                                    uint64_t blocks, uint32_t *__restrict__ filter)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
    for (uint64_t u = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; u < n; u += warps) {
        const uint2 r = adj[u];
        for (uint32_t i = lane; i < r.y; i += 32) {
            const FilterKey fk = filter_key((uint32_t)u, col[(uint64_t)r.x + i], blocks);
            uint32_t *blk = filter + fk.block * 8;
#pragma unroll
            for (int j = 0; j < 8; ++j) atomicOr(&blk[j], 1u << ((fk.bits >> (5 * j)) & 31));
        }
    }
}

// Arguments of k_lane_paths (DeepWalk and node2vec).
struct LaneArgs {
    const uint4 *__restrict__ vtx_ext;    // {id, first column, degree, name} by canonical index
    const uint4 *__restrict__ col_ext;    // {id, first column, degree, name} per CSR entry
    const uint32_t *__restrict__ filter;  // edge filter, filter_blocks blocks of 8 words
    uint64_t filter_blocks;
    const uint32_t *__restrict__ int2idx;  // internal -> canonical index
    const uint32_t *__restrict__ sources;
    int32_t *__restrict__ paths;
    unsigned long long *__restrict__ ctrl;  // [0] walker cursor, [1] moves, [2] candidate draws, [3] neighbour tests, [4] row probes
    uint64_t w_begin, n_walk;
    uint64_t m;                           // CSR entries (index checks)
    uint64_t thr_ret, thr_nb, thr_out;    // acceptance thresholds (2^32 = always)
    uint64_t fold_fx;                     // appendix width a_fx (folding on when fold != 0)
    uint32_t fold;
    uint32_t sym;                         // every edge has its reverse: search the shorter row
    uint32_t tag;                         // draw tag: "N2" + trial pair, or "WALK"
    uint32_t n, L;
    uint32_t key0, key1;
    uint32_t n_sources;
    int start_mode;
    int hints;
};

// Walker slot states.
enum : uint32_t { kIdle = 0, kDraw = 1, kFilter = 2, kSearch = 3 };

// ILP walker slots per lane, each an independent state machine: every pass
// of the loop issues one read per active slot -- a candidate's column entry
// (kDraw), an edge-filter block (kFilter) or one entry of the previous
// vertex's row (kSearch) -- and then consumes it, so a slot that rejects or
// searches does not hold back the other lanes of its warp.  A slot whose
// walk ends takes the next walker id from a warp-private range refilled
// from one global cursor (ctrl[0]).  Each slot stages C path positions of
// its walker in a shared-memory row and writes them out as one contiguous
// segment of the walker's path row.  First-order DeepWalk
// (src/core/deepwalk.cpp:25-28) runs through the same loop with every
// threshold at 2^32 and draw tag "WALK": each move then accepts its first
// candidate, the neighbour mulhi(x, degree) of
// Philox(ctr = (wid_lo, wid_hi, s, "WALK")), the draw of the other walk
// kernels.
template <int ILP>
__global__ void __launch_bounds__(kLaneWarps * 32) k_lane_paths(const LaneArgs a)
{
    constexpr uint32_t C = 32;
    __shared__ int32_t stage[kLaneWarps][ILP][32][C + 1];
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t wib = threadIdx.x >> 5;
    const uint32_t lt_mask = (1u << lane) - 1u;
    const uint64_t pol_keep = l2_policy(a.hints ? 1 : 0);
    const uint64_t pol_stream = l2_policy(a.hints ? 2 : 0);
    const uint64_t thr_lo = a.thr_nb < a.thr_out ? a.thr_nb : a.thr_out;
    const uint64_t thr_hi = a.thr_nb < a.thr_out ? a.thr_out : a.thr_nb;
    const uint32_t chunk = 32 * ILP;
    unsigned long long moves = 0, trials = 0, checks = 0, probes = 0;

    uint64_t wid[ILP], fbits[ILP];
    uint32_t st[ILP], v[ILP], t[ILP], p[ILP], c0[ILP], k[ILP], au[ILP], lo[ILP], hi[ILP], mid[ILP];
    uint32_t vname[ILP], tname[ILP], skey[ILP], soff[ILP];  // names of v and t; the searched row and key
    bool appx[ILP];                                         // the draw fell in the appendix (back to t)
    uint2 rec[ILP], trec[ILP];  // {first column, degree} of v and of t
    uint4 r[ILP], cx[ILP];      // draw words; candidate {id, first column, degree, name}
#pragma unroll
    for (int s = 0; s < ILP; ++s) {
        st[s] = kIdle;
        wid[s] = fbits[s] = 0;
        v[s] = t[s] = p[s] = c0[s] = k[s] = au[s] = lo[s] = hi[s] = mid[s] = 0;
        vname[s] = tname[s] = skey[s] = soff[s] = 0;
        appx[s] = false;
        rec[s] = trec[s] = make_uint2(0u, 0u);
        r[s] = cx[s] = make_uint4(0u, 0u, 0u, 0u);
    }
    uint64_t next = 0, end = 0;  // warp-uniform walker range [next, end) relative to w_begin
    bool exhausted = false;

    // Writes positions [c0, p) of slot s from its stage row: 16-byte stores
    // from the first 16-byte boundary of the path row on, single words
    // around them.
    auto flush = [&](int s) {
        int32_t *dst = a.paths + PTW_IDX((wid[s] - a.w_begin) * (uint64_t)a.L, a.n_walk * (uint64_t)a.L, &a.ctrl[7],
                                         kCheckPath);
        const int32_t *row = stage[wib][s][lane];
        uint32_t i = c0[s];
        for (; i < p[s] && (reinterpret_cast<uintptr_t>(dst + i) & 15); ++i) dst[i] = row[i - c0[s]];
        for (; i + 4 <= p[s]; i += 4) {
            const uint32_t o = i - c0[s];
            *reinterpret_cast<int4 *>(dst + i) = make_int4(row[o], row[o + 1], row[o + 2], row[o + 3]);
        }
        for (; i < p[s]; ++i) dst[i] = row[i - c0[s]];
        c0[s] = p[s];
    };
    // The walker of slot s stands at a vertex without out-edges: the rest
    // of its path is -1.
    auto finish_dead = [&](int s) {
        int32_t *dst = a.paths + (wid[s] - a.w_begin) * (uint64_t)a.L;
        for (uint32_t i = p[s]; i < a.L; ++i) dst[i] = -1;
        st[s] = kIdle;
    };

    for (;;) {
        // ---- refill idle slots ---------------------------------------------
#pragma unroll
        for (int s = 0; s < ILP; ++s) {
            const unsigned need = __ballot_sync(kFull, st[s] == kIdle);
            if (need == 0 || exhausted) continue;
            const uint32_t n_need = __popc(need);
            const uint32_t rank = __popc(need & lt_mask);
            uint64_t my = ~0ull;
            const uint32_t took = (uint32_t)(end - next < n_need ? end - next : n_need);
            if (st[s] == kIdle && rank < took) my = next + rank;
            next += took;
            if (took < n_need) {
                unsigned long long base = 0;
                if (lane == 0) base = atomicAdd(&a.ctrl[0], (unsigned long long)chunk);
                base = __shfl_sync(kFull, base, 0);
                if (base >= a.n_walk) {
                    exhausted = true;
                    next = end = a.n_walk;
                } else {
                    next = base;
                    end = base + chunk < a.n_walk ? base + chunk : a.n_walk;
                    const uint32_t rest = n_need - took;
                    const uint32_t take2 = (uint32_t)(end - next < rest ? end - next : rest);
                    if (st[s] == kIdle && rank >= took && rank - took < take2) my = next + (rank - took);
                    next += take2;
                }
            }
            if (my != ~0ull) {
                wid[s] = a.w_begin + my;
                const uint32_t si = walker_start_index(a.start_mode, a.int2idx, a.sources, a.n, a.n_sources,
                                                       a.key0, a.key1, wid[s]);
                // {id, first column, degree, name}
                const uint4 vx = ld_hint_u4(&a.vtx_ext[PTW_IDX(si, a.n, &a.ctrl[7], kCheckRecord)], pol_keep);
                v[s] = vx.x;
                rec[s] = make_uint2(vx.y, vx.z);
                vname[s] = vx.w;
                stage[wib][s][lane][0] = (int32_t)vx.w;
                p[s] = 1;
                c0[s] = 0;
                k[s] = 0;
                st[s] = kDraw;
                if (a.L == 1 || rec[s].y == 0) {
                    flush(s);
                    finish_dead(s);
                }
            }
        }
        bool any = false;
#pragma unroll
        for (int s = 0; s < ILP; ++s) any |= st[s] != kIdle;
        // walkers that end at their start (L = 1, no out-edge) leave every
        // slot idle while ids remain: refill again
        if (!__any_sync(kFull, any)) {
            if (exhausted) break;
            continue;
        }

        // ---- one read per active slot --------------------------------------
        uint4 x[ILP], x2[ILP];
#pragma unroll
        for (int s = 0; s < ILP; ++s) {
            if (st[s] == kDraw) {
                if ((k[s] & 1) == 0)
                    r[s] = philox(make_uint4((uint32_t)wid[s], (uint32_t)(wid[s] >> 32), p[s] - 1,
                                             a.tag + (k[s] >> 1)),
                                  a.key0, a.key1);
                const uint32_t cu = (k[s] & 1) ? r[s].z : r[s].x;
                au[s] = (k[s] & 1) ? r[s].w : r[s].y;
                uint32_t idx;
                appx[s] = false;
                if (a.fold && p[s] > 1) {
                    const uint64_t deg_fx = (uint64_t)rec[s].y << 20;
                    const uint64_t tf = deg_fx + a.fold_fx;
                    const uint64_t pos = (uint64_t)cu * (tf >> 32) + (((uint64_t)cu * (tf & 0xFFFFFFFFull)) >> 32);
                    appx[s] = pos >= deg_fx;
                    idx = (uint32_t)(pos >> 20);
                } else {
                    idx = __umulhi(cu, rec[s].y);
                }
                if (appx[s]) x[s] = make_uint4(t[s], trec[s].x, trec[s].y, tname[s]);
                else
                    x[s] = ld_hint_u4(&a.col_ext[PTW_IDX((uint64_t)rec[s].x + idx, a.m, &a.ctrl[7], kCheckColumn)],
                                      pol_stream);
            } else if (st[s] == kFilter) {
                const FilterKey fk = filter_key(t[s], cx[s].x, a.filter_blocks);
                fbits[s] = fk.bits;
                const uint4 *blk = reinterpret_cast<const uint4 *>(
                    a.filter + PTW_IDX(fk.block, a.filter_blocks, &a.ctrl[7], kCheckFilter) * 8);
                x[s] = ld_hint_u4(blk, pol_stream);
                x2[s] = ld_hint_u4(blk + 1, pol_stream);
            } else if (st[s] == kSearch) {
                mid[s] = lo[s] + ((hi[s] - lo[s]) >> 1);
                x[s] = ld_hint_u4(&a.col_ext[PTW_IDX((uint64_t)soff[s] + mid[s], a.m, &a.ctrl[7], kCheckColumn)],
                                  pol_stream);
            }
        }

        // ---- consume ------------------------------------------------------
#pragma unroll
        for (int s = 0; s < ILP; ++s) {
            if (st[s] == kIdle) continue;
            int verdict = -1;  // -1 undecided, 0 reject, 1 accept
            if (st[s] == kDraw) {
                cx[s] = x[s];
                ++trials;
                if (appx[s] || p[s] == 1 || k[s] + 1 == kN2vMaxTrials) verdict = 1;
                else if (cx[s].x == t[s]) verdict = (uint64_t)au[s] < a.thr_ret;
                else if ((uint64_t)au[s] < thr_lo) verdict = 1;
                else if ((uint64_t)au[s] >= thr_hi) verdict = 0;
                else st[s] = kFilter;
            } else if (st[s] == kFilter) {
                ++checks;
                const uint32_t w[8] = {x[s].x, x[s].y, x[s].z, x[s].w, x2[s].x, x2[s].y, x2[s].z, x2[s].w};
                bool pass = true;
#pragma unroll
                for (int j = 0; j < 8; ++j) pass &= (w[j] >> ((fbits[s] >> (5 * j)) & 31)) & 1u;
                if (!pass) {
                    verdict = (uint64_t)au[s] < a.thr_out;
                } else {
                    // search the shorter row: x in t's, or (every edge having
                    // its reverse) t in x's
                    lo[s] = 0;
                    if (a.sym && cx[s].z < trec[s].y) {
                        soff[s] = cx[s].y;
                        hi[s] = cx[s].z;
                        skey[s] = tname[s];
                    } else {
                        soff[s] = trec[s].x;
                        hi[s] = trec[s].y;
                        skey[s] = cx[s].w;
                    }
                    // an empty row holds nothing (both rows hold at least
                    // the edge through v, so this does not happen)
                    if (hi[s] == 0) verdict = (uint64_t)au[s] < a.thr_out;
                    else st[s] = kSearch;
                }
            } else {
                ++probes;
                if (x[s].w == skey[s]) {
                    verdict = (uint64_t)au[s] < a.thr_nb;
                } else {
                    if (x[s].w < skey[s]) lo[s] = mid[s] + 1;
                    else hi[s] = mid[s];
                    if (lo[s] >= hi[s]) verdict = (uint64_t)au[s] < a.thr_out;
                }
            }
            if (verdict == 0) {
                ++k[s];
                st[s] = kDraw;
            } else if (verdict == 1) {
                t[s] = v[s];
                trec[s] = rec[s];
                tname[s] = vname[s];
                vname[s] = cx[s].w;
                v[s] = cx[s].x;
                rec[s] = make_uint2(cx[s].y, cx[s].z);
                stage[wib][s][lane][p[s] - c0[s]] = (int32_t)cx[s].w;
                ++p[s];
                ++moves;
                k[s] = 0;
                st[s] = kDraw;
                if (p[s] == a.L || p[s] - c0[s] == C || rec[s].y == 0) flush(s);
                if (p[s] == a.L) st[s] = kIdle;
                else if (rec[s].y == 0) finish_dead(s);
            }
        }
    }

#pragma unroll
    for (int o = 16; o; o >>= 1) {
        moves += __shfl_xor_sync(kFull, moves, o);
        trials += __shfl_xor_sync(kFull, trials, o);
        checks += __shfl_xor_sync(kFull, checks, o);
        probes += __shfl_xor_sync(kFull, probes, o);
    }
    if (lane == 0) {
        if (moves) atomicAdd(&a.ctrl[1], moves);
        if (trials) atomicAdd(&a.ctrl[2], trials);
        if (checks) atomicAdd(&a.ctrl[3], checks);
        if (probes) atomicAdd(&a.ctrl[4], probes);
    }
}

// One warp per vertex u: sets *bad when u's row repeats a neighbour or an
// edge (u, v) has no reverse (binary search of v's row for u's name).
__global__ void k_check_simple_symmetric(const uint2 *__restrict__ adj, const uint4 *__restrict__ col_ext,
                                         const uint32_t *__restrict__ int2name, uint32_t n,
                                         unsigned int *__restrict__ bad)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
    for (uint64_t u = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; u < n; u += warps) {
        const uint2 r = adj[u];
        const uint32_t nu = int2name[u];
        for (uint32_t i = lane; i < r.y; i += 32) {
            const uint64_t e = (uint64_t)r.x + i;
            const uint4 c = col_ext[e];
            bool fail = i > 0 && col_ext[e - 1].x == c.x;
            uint32_t lo = 0, hi = c.z;
            while (lo < hi) {
                const uint32_t mid = lo + ((hi - lo) >> 1);
                if (col_ext[(uint64_t)c.y + mid].w < nu) lo = mid + 1;
                else hi = mid;
            }
            fail |= !(lo < c.z && col_ext[(uint64_t)c.y + lo].w == nu);
            if (fail) atomicOr(bad, 1u);
        }
    }
}

}  // namespace

bool ensure_edge_filter(ptw_graph *g)
{
    if (g->dg.edge_filter) return true;
    const DeviceGraph &dg = g->dg;
    // 16 bits per edge, rounded up to a power of two of 32-byte blocks
    uint64_t blocks = 1;
    while (blocks * 16 < dg.m) blocks <<= 1;
    uint32_t *f = nullptr;
    if (device_malloc(&f, blocks * 32) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (cudaMemsetAsync(f, 0, blocks * 32, g->stream) != cudaSuccess) {
        cudaFree(f);
        return false;
    }
    const unsigned grid = (unsigned)std::min<uint64_t>((dg.n + 7) / 8, (uint64_t)g->num_sms * 64);
    k_build_edge_filter<<<std::max(grid, 1u), 256, 0, g->stream>>>(dg.adj, dg.col, dg.n, blocks, f);
    if (cudaGetLastError() != cudaSuccess) {
        cudaFree(f);
        return false;
    }
    g->dg.edge_filter = f;
    g->dg.filter_blocks = blocks;
    g->device_bytes += blocks * 32;
    if (g->dg.simple_symmetric < 0 && g->dg.col_ext) {
        unsigned int *d_bad = nullptr;
        unsigned int h_bad = 1;
        if (device_malloc(&d_bad, sizeof(unsigned int)) == cudaSuccess) {
            if (cudaMemsetAsync(d_bad, 0, sizeof(unsigned int), g->stream) == cudaSuccess) {
                k_check_simple_symmetric<<<std::max(grid, 1u), 256, 0, g->stream>>>(dg.adj, g->dg.col_ext, dg.int2name,
                                                                                    dg.n, d_bad);
                if (cudaGetLastError() == cudaSuccess &&
                    cudaMemcpyAsync(&h_bad, d_bad, sizeof(h_bad), cudaMemcpyDeviceToHost, g->stream) == cudaSuccess &&
                    cudaStreamSynchronize(g->stream) == cudaSuccess)
                    g->dg.simple_symmetric = h_bad ? 0 : 1;
            }
            cudaFree(d_bad);
        }
        cudaGetLastError();
        if (g->dg.simple_symmetric < 0) g->dg.simple_symmetric = 0;  // unknown: fold nothing
    }
    return true;
}

namespace {

// Launches k_lane_paths<ILP>, ILP = 1, 2 or 4.
int launch_lane_paths(ptw_graph *g, LaneArgs &a, int ilp)
{
    const void *fn = ilp == 1 ? (const void *)k_lane_paths<1>
                              : ilp == 4 ? (const void *)k_lane_paths<4> : (const void *)k_lane_paths<2>;
    int per_sm = 0;
    PTW_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kLaneWarps * 32, 0));
    per_sm = std::max(per_sm, 1);
    const uint64_t per_block = (uint64_t)kLaneWarps * 32 * ilp;  // walker slots per block
    uint64_t grid = std::min<uint64_t>((uint64_t)g->num_sms * per_sm, (a.n_walk + per_block - 1) / per_block);
    grid = std::max<uint64_t>(grid, 1);
    void *args[] = {&a};
    PTW_CUDA(cudaLaunchKernel(fn, dim3((unsigned)grid), dim3(kLaneWarps * 32), args, 0, g->stream));
    return PTW_OK;
}

LaneArgs lane_args(ptw_graph *g, uint64_t w_begin, uint64_t w_end, uint32_t L, uint64_t seed, int start_mode,
                  uint32_t n_sources, int32_t *paths)
{
    const DeviceGraph &dg = g->dg;
    LaneArgs a{};
    a.vtx_ext = dg.vtx_ext;
    a.col_ext = dg.col_ext;
    a.filter = dg.edge_filter;
    a.filter_blocks = dg.filter_blocks;
    a.int2idx = dg.int2idx;
    a.sources = g->sc.sources;
    a.paths = paths;
    a.ctrl = g->sc.ctrl;
    a.w_begin = w_begin;
    a.n_walk = w_end - w_begin;
    a.m = dg.m;
    a.n = dg.n;
    a.L = L;
    a.key0 = (uint32_t)seed;
    a.key1 = (uint32_t)(seed >> 32);
    a.n_sources = n_sources;
    a.start_mode = start_mode;
    a.hints = g->tune.cache_hints;
    return a;
}

}  // namespace

int launch_node2vec(ptw_graph *g, uint64_t w_begin, uint64_t w_end, uint32_t L, uint64_t seed,
                    int start_mode, uint32_t n_sources, double p, double q, const uint64_t thr[3], int32_t *paths)
{
    if (!ensure_ext_columns(g) || !ensure_edge_filter(g))
        return fail(PTW_ENOMEM, "node2vec needs the extended column copy (16 bytes per CSR entry) and "
                                "the edge filter (2 bytes per CSR entry), which do not fit in device memory");
    LaneArgs a = lane_args(g, w_begin, w_end, L, seed, start_mode, n_sources, paths);
    a.thr_ret = thr[0];
    a.thr_nb = thr[1];
    a.thr_out = thr[2];
    a.sym = g->dg.simple_symmetric == 1 ? 1u : 0u;
    if (a.sym) {
        // outlier folding when 1/p is the only largest weight: envelope
        // M' = max(1, 1/q), thresholds against M', appendix a_fx
        const double w[3] = {1.0 / p, 1.0, 1.0 / q};
        const double m = std::max(w[1], w[2]);
        if (w[0] > m) {
            a.fold = 1;
            a.thr_ret = 1ull << 32;
            a.thr_nb = w[1] >= m ? 1ull << 32 : (uint64_t)(w[1] / m * 4294967296.0);
            a.thr_out = w[2] >= m ? 1ull << 32 : (uint64_t)(w[2] / m * 4294967296.0);
            a.fold_fx = (uint64_t)((w[0] - m) / m * 1048576.0);
        }
    }
    a.tag = PTW_TAG_N2V;
    // One slot per lane: with rejections the slots of a lane wait on each
    // other's reads (R-MAT scale 24, p = 2, q = 0.5: 24.9 / 22.8 / 12.8 G
    // moves/s with 1 / 2 / 4 slots).
    return launch_lane_paths(g, a, 1);
}

int launch_lane_deepwalk(ptw_graph *g, uint64_t w_begin, uint64_t w_end, uint32_t L, uint64_t seed,
                         int start_mode, uint32_t n_sources, int32_t *paths)
{
    PTW_CUDA(cudaMemsetAsync(g->sc.ctrl, 0, 2 * sizeof(unsigned long long), g->stream));
    LaneArgs a = lane_args(g, w_begin, w_end, L, seed, start_mode, n_sources, paths);
    a.thr_ret = a.thr_nb = a.thr_out = 1ull << 32;  // every first candidate accepted
    a.tag = PTW_TAG_WALK;
    return launch_lane_paths(g, a, g->tune.paths_ilp == 1 || g->tune.paths_ilp == 4 ? g->tune.paths_ilp : 2);
}

}  // namespace ptw
