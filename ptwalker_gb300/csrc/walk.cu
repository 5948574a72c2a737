// Walker-update kernels for sm_103a.
//
// K1/K2 k_walk: persistent walker pool.  Replaces the reference's per-thread
// walker containers, partition sweeps and migrations
// (src/core/solver.hpp:194-498, :850-1028) and the direct sampler
// (src/core/sampler.hpp:214-217).  Each lane holds ILP walkers.  A lane whose
// walker ended is refilled from a warp-private range of walker ids: the warp
// ballots the empty lanes, ranks them with a popcount prefix and takes ids
// from its range, drawing a new range of `chunk` ids from one global cursor
// when it runs dry.  Every draw is a pure function of (seed, walker id, step),
// so scheduling never changes a result.
//
// Per move (count apps, pagerank.cpp:86-89 / ppr.cpp:114-117):
//   {off, deg} = adj[v]                      one 8-byte random load
//   u = Philox4x32-10(key=seed, ctr=(wid_lo, wid_hi, step, "WALK"))
//   v = col[off + mulhi(u.x, deg)]           one 4-byte random load
//   counts[v] += 1                           one fire-and-forget reduction
//   stop iff u.y < floor(sp * 2^32)
// With the extended column copy (EXT) the column entry also carries the
// neighbour's {off, deg} (and name), so a move is one dependent 16-byte
// gather: the walker keeps {off, deg} of its vertex in registers and loads a
// row record only at its start vertex.
//
// K3 k_paths: DeepWalk (src/core/deepwalk.cpp:25-28) on the plain or
// name-paired columns.  One walker per lane, all walks the same length, so a
// warp stays converged.  Each warp stages the next 32 path positions of its
// 32 walkers in shared memory and writes them out row by row, so every store
// instruction writes 32 consecutive int32 of one path row.  On the extended
// columns DeepWalk runs in the per-lane loop of node2vec.cu.
#include <algorithm>

#include "ptw_internal.cuh"

namespace ptw {
namespace {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ uint64_t umin64(uint64_t x, uint64_t y) { return x < y ? x : y; }

struct WalkArgs {
    const uint2 *__restrict__ adj;
    const uint32_t *__restrict__ col;
    const uint4 *__restrict__ col_ext;       // EXT: {id, first column, degree, name} per entry
    const uint4 *__restrict__ vtx_ext;       // {id, first column, degree, name} by canonical index
    const uint32_t *__restrict__ start_map;  // canonical index -> internal
    const uint32_t *__restrict__ int2idx;    // internal -> canonical index
    const uint32_t *__restrict__ sources;    // internal ids
    const uint32_t *__restrict__ int2name;
    uint32_t *__restrict__ counts;
    uint32_t *__restrict__ pairs;            // endpoint app: [2 * walkers] names
    unsigned long long *__restrict__ ctrl;   // [0] cursor, [1] moves
    uint64_t w_begin;
    uint64_t n_walk;
    uint64_t thr;
    uint64_t m;  // CSR entries (index checks)
    uint32_t n;
    uint32_t key0, key1;
    uint32_t n_sources;
    uint32_t max_moves;
    uint32_t chunk;
    uint32_t hot_k;
    int start_mode;
    int hints;  // L2 eviction priorities on (see l2_policy)
    int by_name;  // EXT count walks: counts[] is indexed by vertex name (the caller's output)
};

__device__ __forceinline__ uint32_t start_vertex(const WalkArgs &a, uint64_t wid)
{
    return walker_start(a.start_mode, a.start_map, a.sources, a.n, a.n_sources, a.key0, a.key1, wid);
}

__device__ __forceinline__ uint32_t start_index(const WalkArgs &a, uint64_t wid)
{
    return walker_start_index(a.start_mode, a.int2idx, a.sources, a.n, a.n_sources, a.key0, a.key1, wid);
}

// Counts a visit of internal vertex v (name nm): ids below hot_k in shared
// memory, the others in counts[] by internal id, or by name when by_name.
template <bool HOT>
__device__ __forceinline__ void count_visit(const WalkArgs &a, uint32_t *s_hot, uint32_t v, uint32_t nm,
                                            uint64_t pol)
{
    if (HOT && v < a.hot_k) atomicAdd(&s_hot[v], 1u);
    else if (a.by_name) red_add_hint(&a.counts[nm], 1u, pol);
    else red_add_hint(&a.counts[PTW_IDX(v, a.n, &a.ctrl[7], kCheckCounter)], 1u, pol);
}

// Warp-aggregated visit (all 32 lanes call it): lanes with `on` set count
// vertex v; lanes counting the same non-hot vertex merge into one reduction
// of the group's size by its lowest lane.
template <bool HOT>
__device__ __forceinline__ void count_visit_agg(const WalkArgs &a, uint32_t *s_hot, uint32_t v, bool on,
                                                uint32_t lt_mask, uint64_t pol)
{
    const bool hot = HOT && v < a.hot_k;
    const unsigned m = __ballot_sync(kFull, on && !hot);
    if (!on) return;
    if (hot) {
        atomicAdd(&s_hot[v], 1u);
        return;
    }
    const unsigned grp = __match_any_sync(m, v);
    if ((grp & lt_mask) == 0)
        red_add_hint(&a.counts[PTW_IDX(v, a.n, &a.ctrl[7], kCheckCounter)], (uint32_t)__popc(grp), pol);
}

template <bool ENDPOINT, int ILP, bool HOT, bool EXT, bool AGG = false>
__device__ __forceinline__ void walk_body(const WalkArgs &a, uint32_t *s_hot)
{
    if (HOT) {
        for (uint32_t i = threadIdx.x; i < a.hot_k; i += blockDim.x) s_hot[i] = 0;
        __syncthreads();
    }
    const uint64_t pol_keep = l2_policy(a.hints ? 1 : 0);   // row records, counters
    const uint64_t pol_stream = l2_policy(a.hints ? 2 : 0); // column array
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t lt_mask = (1u << lane) - 1u;

    uint64_t wid[ILP];
    uint32_t v[ILP], step[ILP], s0[ILP];
    bool act[ILP], have[ILP];
    uint2 rec[ILP];  // {first column, degree} of v (kept across moves with EXT)
#pragma unroll
    for (int k = 0; k < ILP; ++k) {
        act[k] = have[k] = false;
        wid[k] = 0;
        v[k] = step[k] = s0[k] = 0;
        rec[k] = make_uint2(0u, 0u);
    }
    // Warp-uniform walker-id range [next, end) relative to w_begin.
    uint64_t next = 0, end = 0;
    bool exhausted = false;
    unsigned long long moves = 0;

    for (;;) {
        // ---- refill empty slots ------------------------------------------
#pragma unroll
        for (int k = 0; k < ILP; ++k) {
            const unsigned need = __ballot_sync(kFull, !act[k]);
            if (need == 0 || exhausted) continue;
            const uint32_t n_need = __popc(need);
            const uint32_t rank = __popc(need & lt_mask);
            uint64_t my = ~0ull;
            const uint64_t avail = end - next;
            const uint32_t took = (uint32_t)umin64(n_need, avail);
            if (!act[k] && rank < took) my = next + rank;
            next += took;
            if (took < n_need) {
                unsigned long long base = 0;
                if (lane == 0) base = atomicAdd(&a.ctrl[0], (unsigned long long)a.chunk);
                base = __shfl_sync(kFull, base, 0);
                if (base >= a.n_walk) {
                    exhausted = true;
                    next = end = a.n_walk;
                } else {
                    next = base;
                    end = umin64(base + a.chunk, a.n_walk);
                    const uint32_t take2 = (uint32_t)umin64(n_need - took, end - next);
                    if (!act[k] && rank >= took && rank - took < take2) my = next + (rank - took);
                    next += take2;
                }
            }
            if (my != ~0ull) {
                wid[k] = a.w_begin + my;
                // EXT count walks by name hold the start's canonical index
                // until its record is loaded
                v[k] = EXT && a.by_name ? start_index(a, wid[k]) : start_vertex(a, wid[k]);
                s0[k] = v[k];
                step[k] = 0;
                act[k] = true;
                have[k] = false;
                if (!ENDPOINT && !(EXT && a.by_name)) count_visit<HOT>(a, s_hot, v[k], 0u, pol_keep);
            }
        }
        bool any = false;
#pragma unroll
        for (int k = 0; k < ILP; ++k) any |= act[k];
        if (!__any_sync(kFull, any)) break;

        // ---- one move for every active slot --------------------------------
#pragma unroll
        for (int k = 0; k < ILP; ++k) {
            if (!act[k] || (EXT && have[k])) continue;
            if (EXT && a.by_name) {
                // a walker's first move: its start record, with the start's name
                // for its start visit
                const uint4 vx = ld_hint_u4(&a.vtx_ext[PTW_IDX(v[k], a.n, &a.ctrl[7], kCheckRecord)], pol_keep);
                v[k] = vx.x;
                rec[k] = make_uint2(vx.y, vx.z);
                if (!ENDPOINT) count_visit<HOT>(a, s_hot, v[k], vx.w, pol_keep);
            } else {
                rec[k] = ld_hint_u2(&a.adj[PTW_IDX(v[k], a.n, &a.ctrl[7], kCheckRecord)], pol_keep);
            }
        }
        uint4 r[ILP];
#pragma unroll
        for (int k = 0; k < ILP; ++k)
            if (act[k])
                r[k] = philox(make_uint4((uint32_t)wid[k], (uint32_t)(wid[k] >> 32), step[k], PTW_TAG_WALK),
                              a.key0, a.key1);
        uint32_t nb[ILP], nnm[ILP];
        uint2 nrec[ILP];
#pragma unroll
        for (int k = 0; k < ILP; ++k) {
            nnm[k] = 0;
            if (act[k] && rec[k].y != 0) {
                const uint32_t e = rec[k].x + __umulhi(r[k].x, rec[k].y);
                if (EXT) {
                    const uint4 x = ld_hint_u4(&a.col_ext[PTW_IDX(e, a.m, &a.ctrl[7], kCheckColumn)], pol_stream);
                    nb[k] = x.x;
                    nrec[k] = make_uint2(x.y, x.z);
                    nnm[k] = x.w;
                } else {
                    nb[k] = ld_hint_u32(&a.col[PTW_IDX(e, a.m, &a.ctrl[7], kCheckColumn)], pol_stream);
                }
            }
        }
#pragma unroll
        for (int k = 0; k < ILP; ++k) {
            bool counted = false;  // AGG: this lane moved and counts v[k] below
            if (act[k]) {
                bool done;
                if (rec[k].y == 0) {
                    done = true;  // no out-edge: the walk ends here
                } else {
                    v[k] = nb[k];
                    if (EXT) {
                        rec[k] = nrec[k];
                        have[k] = true;
                    }
                    ++step[k];
                    ++moves;
                    if (!ENDPOINT) {
                        if (AGG) counted = true;
                        else count_visit<HOT>(a, s_hot, v[k], nnm[k], pol_keep);
                    }
                    done = (uint64_t)r[k].y < a.thr || (a.max_moves && step[k] >= a.max_moves);
                }
                if (done) {
                    if (ENDPOINT) {
                        const uint64_t j = wid[k] - a.w_begin;
                        *reinterpret_cast<uint2 *>(&a.pairs[2 * j]) =
                            make_uint2(a.int2name[s0[k]], a.int2name[v[k]]);
                    }
                    act[k] = false;
                }
            }
            if (AGG && !ENDPOINT) count_visit_agg<HOT>(a, s_hot, v[k], counted, lt_mask, pol_keep);
        }
    }

    // ---- flush ------------------------------------------------------------
#pragma unroll
    for (int o = 16; o; o >>= 1) moves += __shfl_xor_sync(kFull, moves, o);
    if (lane == 0 && moves) atomicAdd(&a.ctrl[1], moves);
    if (HOT) {
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < a.hot_k; i += blockDim.x)
            if (s_hot[i]) atomicAdd(&a.counts[a.by_name ? a.int2name[i] : i], s_hot[i]);
    }
}

// Register budget chosen by the compiler (ILP=4: 72 registers, one
// 512-thread block per SM).
template <bool ENDPOINT, int ILP, bool HOT, bool EXT>
__global__ void k_walk(const WalkArgs a)
{
    extern __shared__ uint32_t s_hot[];
    walk_body<ENDPOINT, ILP, HOT, EXT>(a, s_hot);
}

// Count walks with warp-aggregated visits (tune.warp_agg).
template <int ILP, bool HOT, bool EXT>
__global__ void k_walk_agg(const WalkArgs a)
{
    extern __shared__ uint32_t s_hot[];
    walk_body<false, ILP, HOT, EXT, true>(a, s_hot);
}

// Register caps so that two blocks fit on an SM, for more walkers in flight:
// two 512-thread blocks (64 registers), two 768-thread blocks (42
// registers; ILP 2 holds 3072 walkers per SM) or two 1024-thread blocks
// (32 registers; 4096 walkers per SM at ILP 2, with a few spills).
template <bool ENDPOINT, int ILP, bool HOT, bool EXT>
__global__ void __launch_bounds__(512, 2) k_walk_b2(const WalkArgs a)
{
    extern __shared__ uint32_t s_hot[];
    walk_body<ENDPOINT, ILP, HOT, EXT>(a, s_hot);
}

template <bool ENDPOINT, int ILP, bool HOT, bool EXT>
__global__ void __launch_bounds__(768, 2) k_walk_b2_768(const WalkArgs a)
{
    extern __shared__ uint32_t s_hot[];
    walk_body<ENDPOINT, ILP, HOT, EXT>(a, s_hot);
}

template <bool ENDPOINT, int ILP, bool HOT, bool EXT>
__global__ void __launch_bounds__(1024, 2) k_walk_b2_1024(const WalkArgs a)
{
    extern __shared__ uint32_t s_hot[];
    walk_body<ENDPOINT, ILP, HOT, EXT>(a, s_hot);
}

// K1/K2 with walkers in shared memory.  Each thread owns S walker slots;
// a slot holds the walker's id, step, start name, flags and a 16-byte
// landing buffer with the record {id, first column, degree, name} of the
// vertex it stands on.  One round: refill empty slots (warp ballot, as in
// walk_body) and start their record gathers; for every other walker draw the
// move and start the gather of the chosen column entry; wait for all of the
// thread's gathers; count the landed vertices and apply the stop decisions.
// The gathers are cp.async copies into shared memory, so a thread has S of
// them in flight without holding S destination registers: with 4096
// walkers per SM in flight the random-gather rate of the GPU is reached,
// where register-resident walkers stop at about 2048.  Draws and semantics
// are those of walk_body, so results are identical.
constexpr uint32_t kSlotActive = 1, kSlotStart = 2, kSlotMoved = 4, kSlotStop = 8;

template <bool ENDPOINT, bool HOT, int S>
__global__ void __launch_bounds__(256) k_walk_async(const WalkArgs a)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const uint32_t T = blockDim.x;
    const uint32_t tid = threadIdx.x;
    uint4 *land = reinterpret_cast<uint4 *>(smem);                              // [S*T]
    unsigned long long *wid = reinterpret_cast<unsigned long long *>(land + S * T); // [S*T]
    uint32_t *step = reinterpret_cast<uint32_t *>(wid + S * T);                  // [S*T]
    uint32_t *s0n = step + S * T;                                                // [S*T] start name
    uint32_t *flag = s0n + S * T;                                                // [S*T]
    uint32_t *s_hot = flag + S * T;                                              // [hot_k]
    if (HOT) {
        for (uint32_t i = tid; i < a.hot_k; i += T) s_hot[i] = 0;
    }
#pragma unroll
    for (int k = 0; k < S; ++k) flag[k * T + tid] = 0;
    __syncthreads();
    const uint64_t pol_keep = l2_policy(a.hints ? 1 : 0);
    const uint64_t pol_stream = l2_policy(a.hints ? 2 : 0);
    const uint32_t lane = tid & 31;
    const uint32_t lt_mask = (1u << lane) - 1u;
    uint64_t next = 0, end = 0;
    bool exhausted = false;
    unsigned long long moves = 0;

    for (;;) {
        // ---- refill empty slots; start their record gathers --------------
#pragma unroll 1
        for (int k = 0; k < S; ++k) {
            const uint32_t i = k * T + tid;
            const bool empty = (flag[i] & kSlotActive) == 0;
            const unsigned need = __ballot_sync(kFull, empty);
            if (need == 0 || exhausted) continue;
            const uint32_t n_need = __popc(need);
            const uint32_t rank = __popc(need & lt_mask);
            uint64_t my = ~0ull;
            const uint64_t avail = end - next;
            const uint32_t took = (uint32_t)umin64(n_need, avail);
            if (empty && rank < took) my = next + rank;
            next += took;
            if (took < n_need) {
                unsigned long long base = 0;
                if (lane == 0) base = atomicAdd(&a.ctrl[0], (unsigned long long)a.chunk);
                base = __shfl_sync(kFull, base, 0);
                if (base >= a.n_walk) {
                    exhausted = true;
                    next = end = a.n_walk;
                } else {
                    next = base;
                    end = umin64(base + a.chunk, a.n_walk);
                    const uint32_t take2 = (uint32_t)umin64(n_need - took, end - next);
                    if (empty && rank >= took && rank - took < take2) my = next + (rank - took);
                    next += take2;
                }
            }
            if (my != ~0ull) {
                const uint64_t w = a.w_begin + my;
                wid[i] = w;
                step[i] = 0;
                flag[i] = kSlotActive | kSlotStart;
                cp_async16(&land[i], &a.vtx_ext[PTW_IDX(start_index(a, w), a.n, &a.ctrl[7], kCheckRecord)], pol_keep);
            }
        }
        bool any = false;
#pragma unroll 1
        for (int k = 0; k < S; ++k) any |= (flag[k * T + tid] & kSlotActive) != 0;
        if (!__any_sync(kFull, any)) break;

        // ---- draw and start one move for every walker standing on a record
#pragma unroll 1
        for (int k = 0; k < S; ++k) {
            const uint32_t i = k * T + tid;
            const uint32_t f = flag[i];
            if ((f & kSlotActive) == 0 || (f & kSlotStart)) continue;
            const uint4 x = land[i];  // {v, first column, degree, name}
            if (x.z == 0) {           // no out-edge: the walk ends here
                if (ENDPOINT) {
                    const uint64_t j = wid[i] - a.w_begin;
                    *reinterpret_cast<uint2 *>(&a.pairs[2 * j]) = make_uint2(s0n[i], x.w);
                }
                flag[i] = 0;
                continue;
            }
            const uint64_t w = wid[i];
            const uint32_t st = step[i];
            const uint4 r = philox(make_uint4((uint32_t)w, (uint32_t)(w >> 32), st, PTW_TAG_WALK), a.key0, a.key1);
            const bool stop = (uint64_t)r.y < a.thr || (a.max_moves && st + 1 >= a.max_moves);
            flag[i] = kSlotActive | kSlotMoved | (stop ? kSlotStop : 0u);
            cp_async16(&land[i], &a.col_ext[PTW_IDX((uint64_t)x.y + __umulhi(r.x, x.z), a.m, &a.ctrl[7], kCheckColumn)],
                       pol_stream);
        }
        cp_async_wait_all();

        // ---- count the landed vertices, apply the stop decisions -----------
#pragma unroll 1
        for (int k = 0; k < S; ++k) {
            const uint32_t i = k * T + tid;
            const uint32_t f = flag[i];
            if ((f & kSlotActive) == 0) continue;
            const uint4 x = land[i];
            if (f & kSlotStart) {
                s0n[i] = x.w;
                if (!ENDPOINT) count_visit<HOT>(a, s_hot, x.x, 0u, pol_keep);
                flag[i] = kSlotActive;
            } else if (f & kSlotMoved) {
                step[i] += 1;
                ++moves;
                if (!ENDPOINT) count_visit<HOT>(a, s_hot, x.x, 0u, pol_keep);
                if (f & kSlotStop) {
                    if (ENDPOINT) {
                        const uint64_t j = wid[i] - a.w_begin;
                        *reinterpret_cast<uint2 *>(&a.pairs[2 * j]) = make_uint2(s0n[i], x.w);
                    }
                    flag[i] = 0;
                } else {
                    flag[i] = kSlotActive;
                }
            }
        }
    }

#pragma unroll
    for (int o = 16; o; o >>= 1) moves += __shfl_xor_sync(kFull, moves, o);
    if (lane == 0 && moves) atomicAdd(&a.ctrl[1], moves);
    if (HOT) {
        __syncthreads();
        for (uint32_t i = tid; i < a.hot_k; i += T)
            if (s_hot[i]) atomicAdd(&a.counts[i], s_hot[i]);
    }
}

// Dynamic shared memory of k_walk_async: 36 bytes per slot + hot counters.
inline size_t async_smem(int slots, int block, uint32_t hot_k)
{
    return (size_t)slots * block * 36 + (size_t)hot_k * 4;
}

struct PathArgs {
    const uint2 *__restrict__ adj;
    const uint32_t *__restrict__ col;
    const uint2 *__restrict__ col_named;  // {internal id, name} per column entry
    const uint32_t *__restrict__ start_map;
    const uint32_t *__restrict__ sources;
    const uint32_t *__restrict__ int2name;
    int32_t *__restrict__ paths;
    unsigned long long *check;  // index-check word (checked build)
    uint64_t w_begin, n_walk;
    uint64_t m;  // CSR entries (index checks)
    uint32_t n, L;
    uint32_t key0, key1;
    uint32_t n_sources;
    int start_mode;
    int hints;
};

constexpr int kPathWarps = 4;  // warps per block

// G groups of 32 consecutive walkers per warp (one walker of each group per
// lane), stepped together so a lane has G gathers in flight.  MODE 0 reads
// the row record, the column entry and the neighbour's name (three random
// reads per move); MODE 1 reads {internal id, name} pairs from col_named (two:
// row record, pair).  With the extended columns (one read per move) DeepWalk
// runs in the per-lane loop of node2vec.cu instead.
template <int G, int MODE>
__global__ void __launch_bounds__(kPathWarps * 32) k_paths(const PathArgs a)
{
    // C path positions are staged per walker before a flush; rows are padded
    // to C+1 words so the per-lane column writes do not conflict on banks.
    constexpr uint32_t C = G == 1 ? 32 : 16;
    __shared__ int32_t stage[kPathWarps][G][32][C + 1];
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t wib = threadIdx.x >> 5;
    const uint64_t n_groups = (a.n_walk + 31) / 32;
    const uint64_t warps = (uint64_t)gridDim.x * kPathWarps;

    WalkArgs sa;  // start-vertex helper view
    sa.start_map = a.start_map;
    sa.sources = a.sources;
    sa.n = a.n;
    sa.key0 = a.key0;
    sa.key1 = a.key1;
    sa.n_sources = a.n_sources;
    sa.start_mode = a.start_mode;
    const uint64_t pol_keep = l2_policy(a.hints ? 1 : 0);   // row records, names
    const uint64_t pol_stream = l2_policy(a.hints ? 2 : 0); // column array

    for (uint64_t g0 = (blockIdx.x * (uint64_t)kPathWarps + wib) * G; g0 < n_groups; g0 += warps * G) {
        uint64_t wid[G];
        uint32_t v[G], rows[G];
        bool dead[G];
        uint2 rec[G];
#pragma unroll
        for (int g = 0; g < G; ++g) {
            const uint64_t grp = g0 + g;
            const uint64_t j = grp * 32 + lane;  // walker offset
            const bool valid = j < a.n_walk;
            wid[g] = a.w_begin + j;
            rows[g] = grp < n_groups ? (uint32_t)umin64(32, a.n_walk - grp * 32) : 0;
            v[g] = valid ? start_vertex(sa, wid[g]) : 0;
            dead[g] = !valid;
            stage[wib][g][lane][0] = valid ? (int32_t)a.int2name[v[g]] : -1;
        }
        uint32_t c0 = 0;  // path position of stage column 0
        for (uint32_t p = 1; p <= a.L; ++p) {
            if (p == a.L || p % C == 0) {
                // flush columns [c0, p) of every group's rows; consecutive
                // lanes write consecutive positions of one path row
                __syncwarp();
                const uint32_t cols = p - c0;
#pragma unroll
                for (int g = 0; g < G; ++g)
                    for (uint32_t idx = lane; idx < rows[g] * cols; idx += 32) {
                        const uint32_t rr = idx / cols, cc = idx - rr * cols;
                        a.paths[((g0 + g) * 32 + rr) * (uint64_t)a.L + c0 + cc] = stage[wib][g][rr][cc];
                    }
                __syncwarp();
                c0 = p;
                if (p == a.L) break;
            }
#pragma unroll
            for (int g = 0; g < G; ++g)
                if (!dead[g]) rec[g] = ld_hint_u2(&a.adj[PTW_IDX(v[g], a.n, a.check, kCheckRecord)], pol_keep);
            uint4 r[G];
#pragma unroll
            for (int g = 0; g < G; ++g)
                if (!dead[g])
                    r[g] = philox(make_uint4((uint32_t)wid[g], (uint32_t)(wid[g] >> 32), p - 1, PTW_TAG_WALK),
                                  a.key0, a.key1);
            uint32_t nm[G];
#pragma unroll
            for (int g = 0; g < G; ++g) {
                if (!dead[g]) {
                    if (rec[g].y == 0) {
                        dead[g] = true;
                    } else if (MODE == 1) {
                        const uint2 cn = ld_hint_u2(
                            &a.col_named[PTW_IDX((uint64_t)rec[g].x + __umulhi(r[g].x, rec[g].y), a.m, a.check,
                                                 kCheckColumn)],
                            pol_stream);
                        v[g] = cn.x;
                        nm[g] = cn.y;
                    } else {
                        v[g] = ld_hint_u32(&a.col[PTW_IDX((uint64_t)rec[g].x + __umulhi(r[g].x, rec[g].y), a.m, a.check,
                                                          kCheckColumn)],
                                           pol_stream);
                    }
                }
            }
#pragma unroll
            for (int g = 0; g < G; ++g) {
                int32_t out = -1;
                if (!dead[g])
                    out = MODE != 0 ? (int32_t)nm[g]
                                    : (int32_t)ld_hint_u32(&a.int2name[PTW_IDX(v[g], a.n, a.check, kCheckCounter)],
                                                           pol_keep);
                stage[wib][g][lane][p - c0] = out;
            }
        }
    }
}

__global__ void k_name_columns(const uint32_t *col, const uint32_t *int2name, uint64_t m, uint2 *col_named)
{
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < m; e += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t c = col[e];
        col_named[e] = make_uint2(c, int2name[c]);
    }
}

// {neighbour id, its first column, its degree, its name} for every entry.
__global__ void k_ext_columns(const uint32_t *col, const uint2 *adj, const uint32_t *int2name, uint64_t m,
                              uint4 *col_ext)
{
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < m; e += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t c = col[e];
        const uint2 r = adj[c];
        col_ext[e] = make_uint4(c, r.x, r.y, int2name[c]);
    }
}

// The vertex records in canonical order (by name rank).
__global__ void k_vertex_ext(const uint2 *adj, const uint32_t *int2name, const uint32_t *idx2int, uint32_t n,
                             uint4 *vtx_ext)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t v = idx2int[i];
        const uint2 r = adj[v];
        vtx_ext[i] = make_uint4(v, r.x, r.y, int2name[v]);
    }
}

__global__ void k_counts_by_name(const uint32_t *counts, const uint32_t *int2name, uint32_t n,
                                 uint32_t *out)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[int2name[i]] = counts[i];
}

// cap: 0 = no register cap, 512 / 768 / 1024 = two blocks of that size per SM.
template <bool E, int ILP, bool H, bool X> void *walk_fn(int cap)
{
    switch (cap) {
    case 512: return (void *)k_walk_b2<E, ILP, H, X>;
    case 768: return (void *)k_walk_b2_768<E, ILP, H, X>;
    case 1024: return (void *)k_walk_b2_1024<E, ILP, H, X>;
    default: return (void *)k_walk<E, ILP, H, X>;
    }
}

template <bool E, bool H, bool X> void *walk_fn_ilp(int ilp, int cap)
{
    switch (ilp) {
    case 1: return walk_fn<E, 1, H, X>(cap);
    case 4: return walk_fn<E, 4, H, X>(cap);
    default: return walk_fn<E, 2, H, X>(cap);
    }
}

template <bool X> void *pick_walk_x(bool endpoint, int ilp, bool hot, int cap)
{
    if (endpoint) return walk_fn_ilp<true, false, X>(ilp, cap);
    if (hot) return walk_fn_ilp<false, true, X>(ilp, cap);
    return walk_fn_ilp<false, false, X>(ilp, cap);
}

void *pick_walk_async(bool endpoint, bool hot, int slots)
{
    if (slots == 16) {
        if (endpoint) return (void *)k_walk_async<true, false, 16>;
        return hot ? (void *)k_walk_async<false, true, 16> : (void *)k_walk_async<false, false, 16>;
    }
    if (endpoint) return (void *)k_walk_async<true, false, 8>;
    return hot ? (void *)k_walk_async<false, true, 8> : (void *)k_walk_async<false, false, 8>;
}

template <bool H, bool X> void *agg_fn(int ilp)
{
    switch (ilp) {
    case 1: return (void *)k_walk_agg<1, H, X>;
    case 4: return (void *)k_walk_agg<4, H, X>;
    default: return (void *)k_walk_agg<2, H, X>;
    }
}

void *pick_walk_agg(int ilp, bool hot, bool ext)
{
    if (ext) return hot ? agg_fn<true, true>(ilp) : agg_fn<false, true>(ilp);
    return hot ? agg_fn<true, false>(ilp) : agg_fn<false, false>(ilp);
}

// min_blocks 2 picks the register cap by block size (checked by check_tune).
void *pick_walk(bool endpoint, int ilp, bool hot, int min_blocks, int block, bool ext)
{
    const int cap = min_blocks != 2 ? 0 : block <= 512 ? 512 : block <= 768 ? 768 : 1024;
    return ext ? pick_walk_x<true>(endpoint, ilp, hot, cap) : pick_walk_x<false>(endpoint, ilp, hot, cap);
}

}  // namespace

// Builds the extended column copy on first use; false (and no error) when
// it does not fit in device memory, so the caller walks without it.
bool count_walk_by_name(ptw_graph *g, const ptw_tune &t)
{
    return !t.gather_slots && !t.warp_agg && (t.ext_columns & 1) && ensure_ext_columns(g);
}

bool ensure_ext_columns(ptw_graph *g)
{
    if (g->dg.col_ext) return true;
    const DeviceGraph &dg = g->dg;
    uint4 *cx = nullptr;
    if (device_malloc(&cx, std::max<uint64_t>(dg.m, 1) * sizeof(uint4)) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    const unsigned grid = (unsigned)std::min<uint64_t>((dg.m + 255) / 256, (uint64_t)g->num_sms * 64);
    k_ext_columns<<<std::max(grid, 1u), 256, 0, g->stream>>>(dg.col, dg.adj, dg.int2name, dg.m, cx);
    if (cudaGetLastError() != cudaSuccess) {
        cudaFree(cx);
        return false;
    }
    uint4 *vx = nullptr;
    if (device_malloc(&vx, std::max<uint32_t>(dg.n, 1) * sizeof(uint4)) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(cx);
        return false;
    }
    const unsigned vgrid = (unsigned)std::min<uint64_t>((dg.n + 255) / 256, (uint64_t)g->num_sms * 64);
    k_vertex_ext<<<std::max(vgrid, 1u), 256, 0, g->stream>>>(dg.adj, dg.int2name, dg.idx2int, dg.n, vx);
    if (cudaGetLastError() != cudaSuccess) {
        cudaFree(cx);
        cudaFree(vx);
        return false;
    }
    g->dg.col_ext = cx;
    g->dg.vtx_ext = vx;
    g->device_bytes += dg.m * sizeof(uint4) + (uint64_t)dg.n * sizeof(uint4);
    return true;
}

void drop_unused_columns(ptw_graph *g)
{
    DeviceGraph &dg = g->dg;
    if (dg.col_ext && !g->tune.ext_columns && !g->tune.gather_slots && g->ext_users == 0) {
        cudaStreamSynchronize(g->stream);
        cudaFree(dg.col_ext);
        cudaFree(dg.vtx_ext);
        dg.col_ext = nullptr;
        dg.vtx_ext = nullptr;
        g->device_bytes -= dg.m * sizeof(uint4) + (uint64_t)dg.n * sizeof(uint4);
    }
    if (dg.col_named && ((g->tune.ext_columns & 2) || !g->tune.paths_named)) {
        cudaStreamSynchronize(g->stream);
        cudaFree(dg.col_named);
        dg.col_named = nullptr;
        g->device_bytes -= dg.m * sizeof(uint2);
    }
}

int check_tune(const ptw_tune &t)
{
    if (t.block < 32 || t.block > 1024 || t.block % 32)
        return fail(PTW_EINVAL, "tune.block must be a multiple of 32 in [32, 1024]");
    if (t.ilp != 1 && t.ilp != 2 && t.ilp != 4) return fail(PTW_EINVAL, "tune.ilp must be 1, 2 or 4");
    if (t.chunk < 1 || t.chunk > (1 << 20)) return fail(PTW_EINVAL, "tune.chunk must be in [1, 2^20]");
    if (t.hot_k < 0 || t.hot_k > 48 * 1024)
        return fail(PTW_EINVAL, "tune.hot_k must be in [0, 49152]");
    if (t.blocks_per_sm < 0 || t.blocks_per_sm > 64) return fail(PTW_EINVAL, "tune.blocks_per_sm out of range");
    if (t.min_blocks != 0 && t.min_blocks != 1 && t.min_blocks != 2)
        return fail(PTW_EINVAL, "tune.min_blocks must be 0, 1 or 2");
    if (t.min_blocks == 2 && t.block > 512 && t.block != 768 && t.block != 1024)
        return fail(PTW_EINVAL, "tune.min_blocks = 2 needs tune.block <= 512, 768 or 1024");
    if (t.paths_ilp != 0 && t.paths_ilp != 1 && t.paths_ilp != 2 && t.paths_ilp != 4)
        return fail(PTW_EINVAL, "tune.paths_ilp must be 1, 2 or 4 (0 = default)");
    if (t.cache_hints != 0 && t.cache_hints != 1) return fail(PTW_EINVAL, "tune.cache_hints must be 0 or 1");
    if (t.paths_named != 0 && t.paths_named != 1) return fail(PTW_EINVAL, "tune.paths_named must be 0 or 1");
    if (t.ext_columns < 0 || t.ext_columns > 3) return fail(PTW_EINVAL, "tune.ext_columns must be in [0, 3]");
    if (t.gather_slots != 0 && t.gather_slots != 8 && t.gather_slots != 16)
        return fail(PTW_EINVAL, "tune.gather_slots must be 0, 8 or 16");
    if (t.gather_slots && t.block > 256) return fail(PTW_EINVAL, "tune.gather_slots needs tune.block <= 256");
    if (t.warp_agg != 0 && t.warp_agg != 1) return fail(PTW_EINVAL, "tune.warp_agg must be 0 or 1");
    if (t.warp_agg && (t.min_blocks == 2 || t.gather_slots))
        return fail(PTW_EINVAL, "tune.warp_agg needs min_blocks 0 and gather_slots 0");
    return PTW_OK;
}

int launch_walk(ptw_graph *g, const WalkLaunch &wl, const ptw_tune &t)
{
    int rc = check_tune(t);
    if (rc) return rc;
    const DeviceGraph &dg = g->dg;
    WalkArgs a;
    a.adj = dg.adj;
    a.col = dg.col;
    a.start_map = dg.idx2int;
    a.int2idx = dg.int2idx;
    a.sources = g->sc.sources;
    a.int2name = dg.int2name;
    a.counts = g->sc.counts;
    a.pairs = wl.pairs;
    a.ctrl = g->sc.ctrl;
    a.w_begin = wl.w_begin;
    a.n_walk = wl.w_end - wl.w_begin;
    a.thr = wl.thr;
    a.m = dg.m;
    a.n = dg.n;
    a.key0 = (uint32_t)wl.seed;
    a.key1 = (uint32_t)(wl.seed >> 32);
    a.n_sources = wl.n_sources;
    a.max_moves = wl.max_moves;
    a.chunk = (uint32_t)t.chunk;
    const bool hot = !wl.endpoint && t.hot_k > 0;
    a.hot_k = hot ? std::min<uint32_t>((uint32_t)t.hot_k, dg.n) : 0;
    a.start_mode = wl.start_mode;
    a.hints = t.cache_hints;

    const bool slots = t.gather_slots != 0 && ensure_ext_columns(g);
    const bool ext = !slots && (t.ext_columns & 1) && ensure_ext_columns(g);
    a.col_ext = g->dg.col_ext;
    a.vtx_ext = g->dg.vtx_ext;
    // extended columns carry each neighbour's name: count straight into the
    // caller's by-name array (no scatter after the walk)
    a.by_name = 0;
    if (wl.by_name) {
        if (!(ext && !t.warp_agg && !wl.endpoint)) return fail(PTW_EINVAL, "counting by name needs the plain walk on extended columns");
        a.by_name = 1;
        a.counts = wl.by_name;
    }
    void *fn = slots ? pick_walk_async(wl.endpoint, hot, t.gather_slots)
               : (t.warp_agg && !wl.endpoint) ? pick_walk_agg(t.ilp, hot, ext)
                                              : pick_walk(wl.endpoint, t.ilp, hot, t.min_blocks, t.block, ext);
    const size_t smem = slots ? async_smem(t.gather_slots, t.block, a.hot_k) : hot ? (size_t)a.hot_k * 4 : 0;
    if (smem > 227 * 1024) return fail(PTW_EINVAL, "tune.gather_slots x tune.block x hot_k need too much shared memory");
    if (smem > 48 * 1024)
        PTW_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    PTW_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, t.block, smem));
    if (per_sm < 1) return fail(PTW_EINVAL, "walk kernel does not fit on an SM with this tune");
    if (t.blocks_per_sm > 0) per_sm = std::min(per_sm, (int)t.blocks_per_sm);
    uint64_t grid = (uint64_t)g->num_sms * per_sm;
    // No more warps than walker ranges to hand out.
    const uint64_t warps_needed = (a.n_walk + (uint64_t)a.chunk - 1) / a.chunk;
    const uint64_t max_blocks = std::max<uint64_t>(1, (warps_needed + t.block / 32 - 1) / (t.block / 32));
    grid = std::min(grid, max_blocks);

    PTW_CUDA(cudaMemsetAsync(g->sc.ctrl, 0, 2 * sizeof(unsigned long long), g->stream));
    void *args[] = {&a};
    PTW_CUDA(cudaLaunchKernel(fn, dim3((unsigned)grid), dim3(t.block), args, smem, g->stream));
    return PTW_OK;
}

int launch_paths(ptw_graph *g, uint64_t w_begin, uint64_t w_end, uint32_t L, uint64_t seed,
                 int start_mode, uint32_t n_sources, int32_t *paths)
{
    const DeviceGraph &dg = g->dg;
    PathArgs a;
    a.adj = dg.adj;
    a.col = dg.col;
    a.start_map = dg.idx2int;
    a.sources = g->sc.sources;
    a.int2name = dg.int2name;
    a.paths = paths;
    a.check = g->sc.ctrl + 7;
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
    // Extended columns (16 bytes per CSR entry) take precedence; then
    // name-paired columns, built once on the first path walk (8 bytes per
    // CSR entry); without either the kernel looks names up per move.
    const bool ext = (g->tune.ext_columns & 2) && ensure_ext_columns(g);
    bool named = !ext && g->tune.paths_named != 0;
    if (named && !g->dg.col_named) {
        uint2 *cn = nullptr;
        if (device_malloc(&cn, std::max<uint64_t>(dg.m, 1) * sizeof(uint2)) == cudaSuccess) {
            const unsigned grid = (unsigned)std::min<uint64_t>((dg.m + 255) / 256, (uint64_t)g->num_sms * 64);
            k_name_columns<<<std::max(grid, 1u), 256, 0, g->stream>>>(dg.col, dg.int2name, dg.m, cn);
            PTW_CUDA(cudaGetLastError());
            g->dg.col_named = cn;
            g->device_bytes += dg.m * sizeof(uint2);
        } else {
            cudaGetLastError();  // no room: walk with per-move name lookups
            named = false;
        }
    }
    a.col_named = g->dg.col_named;
    // With extended columns the walkers run in the per-lane loop of
    // node2vec.cu, each slot refilled as its walk ends (no warp lockstep).
    if (ext) return launch_lane_deepwalk(g, w_begin, w_end, L, seed, start_mode, n_sources, paths);
    const int G = g->tune.paths_ilp == 1 || g->tune.paths_ilp == 4 ? g->tune.paths_ilp : 2;
    const void *fn;
    if (named)
        fn = G == 1 ? (const void *)k_paths<1, 1> : G == 4 ? (const void *)k_paths<4, 1> : (const void *)k_paths<2, 1>;
    else
        fn = G == 1 ? (const void *)k_paths<1, 0> : G == 4 ? (const void *)k_paths<4, 0> : (const void *)k_paths<2, 0>;
    int per_sm = 0;
    PTW_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kPathWarps * 32, 0));
    per_sm = std::max(per_sm, 1);
    const uint64_t groups = (a.n_walk + 31) / 32;
    const uint64_t per_block = (uint64_t)kPathWarps * G;
    uint64_t grid = std::min<uint64_t>((uint64_t)g->num_sms * per_sm, (groups + per_block - 1) / per_block);
    grid = std::max<uint64_t>(grid, 1);
    void *args[] = {&a};
    PTW_CUDA(cudaLaunchKernel(fn, dim3((unsigned)grid), dim3(kPathWarps * 32), args, 0, g->stream));
    return PTW_OK;
}

int launch_counts_by_name(ptw_graph *g, uint32_t *d_out)
{
    const DeviceGraph &dg = g->dg;
    if (dg.id_bound != dg.n)
        PTW_CUDA(cudaMemsetAsync(d_out, 0, (uint64_t)dg.id_bound * 4, g->stream));
    const unsigned grid = (unsigned)std::min<uint64_t>((dg.n + 255) / 256, (uint64_t)g->num_sms * 16);
    k_counts_by_name<<<std::max(grid, 1u), 256, 0, g->stream>>>(g->sc.counts, dg.int2name, dg.n, d_out);
    PTW_CUDA(cudaGetLastError());
    return PTW_OK;
}

}  // namespace ptw
