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
// k_node2vec draws by rejection over v's row.  Trial k of move s takes two
// words of Philox(ctr = (wid_lo, wid_hi, s, "N2" + k/2)) -- (x, y) for even
// k, (z, w) for odd k --, reads the candidate's extended column entry
// {id, first column, degree, name} (one 16-byte gather: the candidate's own
// row record comes with it) and accepts iff the second word is below the
// threshold of the candidate's class.  Most trials are decided without the
// neighbour query: a return to t is known from the id, a word below both
// the neighbour and the other threshold accepts and a word above both
// rejects.  Only the words between them search t's row for the candidate's
// name (rows are in ascending name order), all groups of a lane searching in
// step so their probes are in flight together.  Trial 65535 is accepted
// whatever its word, so every move ends; the host keeps max(w) / min(w) <=
// 1024, which puts that cap below 1e-27 per move.
//
// Paths are staged in shared memory and written row by row as in k_paths.
#include <algorithm>

#include "ptw_internal.cuh"

namespace ptw {
namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kN2vWarps = 4;                // warps per block
constexpr uint32_t kN2vMaxTrials = 65536u;  // trials per move before the last is taken

struct N2vArgs {
    const uint2 *__restrict__ adj;
    const uint4 *__restrict__ col_ext;    // {id, first column, degree, name} per CSR entry
    const uint32_t *__restrict__ start_map;
    const uint32_t *__restrict__ sources;
    const uint32_t *__restrict__ int2name;
    int32_t *__restrict__ paths;
    unsigned long long *__restrict__ ctrl;  // [1] moves, [2] candidate draws, [3] row probes
    uint64_t w_begin, n_walk;
    uint64_t thr_ret, thr_nb, thr_out;    // acceptance thresholds (2^32 = always)
    uint32_t n, L;
    uint32_t key0, key1;
    uint32_t n_sources;
    int start_mode;
    int hints;
};

// Name of CSR entry e, read from its extended column entry.
__device__ __forceinline__ uint32_t entry_name(const uint4 *col_ext, uint64_t e, uint64_t pol)
{
    return ld_hint_u32(reinterpret_cast<const uint32_t *>(col_ext) + 4 * e + 3, pol);
}

// G groups of 32 consecutive walkers per warp, one walker of each group per
// lane.
template <int G>
__global__ void __launch_bounds__(kN2vWarps * 32) k_node2vec(const N2vArgs a)
{
    constexpr uint32_t C = G == 1 ? 32 : 16;
    __shared__ int32_t stage[kN2vWarps][G][32][C + 1];
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t wib = threadIdx.x >> 5;
    const uint64_t n_groups = (a.n_walk + 31) / 32;
    const uint64_t warps = (uint64_t)gridDim.x * kN2vWarps;
    const uint64_t pol_keep = l2_policy(a.hints ? 1 : 0);
    const uint64_t pol_stream = l2_policy(a.hints ? 2 : 0);
    const uint64_t thr_lo = a.thr_nb < a.thr_out ? a.thr_nb : a.thr_out;
    const uint64_t thr_hi = a.thr_nb < a.thr_out ? a.thr_out : a.thr_nb;
    unsigned long long moves = 0, trials = 0, probes = 0;

    for (uint64_t g0 = (blockIdx.x * (uint64_t)kN2vWarps + wib) * G; g0 < n_groups; g0 += warps * G) {
        uint64_t wid[G];
        uint32_t v[G], t[G], rows[G];
        uint2 rec[G], trec[G];  // {first column, degree} of v and of t
        bool dead[G];
#pragma unroll
        for (int g = 0; g < G; ++g) {
            const uint64_t grp = g0 + g;
            const uint64_t j = grp * 32 + lane;
            const bool valid = j < a.n_walk;
            wid[g] = a.w_begin + j;
            rows[g] = grp < n_groups ? (uint32_t)(a.n_walk - grp * 32 < 32 ? a.n_walk - grp * 32 : 32) : 0;
            v[g] = valid ? walker_start(a.start_mode, a.start_map, a.sources, a.n, a.n_sources, a.key0, a.key1,
                                        wid[g])
                         : 0;
            dead[g] = !valid;
            rec[g] = valid ? ld_hint_u2(&a.adj[v[g]], pol_keep) : make_uint2(0u, 0u);
            t[g] = 0;
            trec[g] = make_uint2(0u, 0u);
            stage[wib][g][lane][0] = valid ? (int32_t)a.int2name[v[g]] : -1;
        }
        uint32_t c0 = 0;
        for (uint32_t p = 1; p <= a.L; ++p) {
            if (p == a.L || p % C == 0) {
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
            // move p-1: trials until one is accepted
            bool pend[G];
            uint32_t k[G], nm[G], au[G];
            uint4 r[G], cx[G];
            bool any = false;
#pragma unroll
            for (int g = 0; g < G; ++g) {
                if (!dead[g] && rec[g].y == 0) dead[g] = true;
                pend[g] = !dead[g];
                any |= pend[g];
                k[g] = 0;
                nm[g] = 0;
            }
            while (any) {
#pragma unroll
                for (int g = 0; g < G; ++g) {
                    if (!pend[g]) continue;
                    if ((k[g] & 1) == 0)
                        r[g] = philox(make_uint4((uint32_t)wid[g], (uint32_t)(wid[g] >> 32), p - 1,
                                                 PTW_TAG_N2V + (k[g] >> 1)),
                                      a.key0, a.key1);
                    const uint32_t cu = (k[g] & 1) ? r[g].z : r[g].x;
                    au[g] = (k[g] & 1) ? r[g].w : r[g].y;
                    cx[g] = ld_hint_u4(&a.col_ext[rec[g].x + __umulhi(cu, rec[g].y)], pol_stream);
                    ++trials;
                }
                bool acc[G], chk[G];
                uint32_t lo[G], hi[G];
                bool searching = false;
#pragma unroll
                for (int g = 0; g < G; ++g) {
                    acc[g] = false;
                    chk[g] = false;
                    if (!pend[g]) continue;
                    if (p == 1 || k[g] + 1 == kN2vMaxTrials) acc[g] = true;
                    else if (cx[g].x == t[g]) acc[g] = (uint64_t)au[g] < a.thr_ret;
                    else if ((uint64_t)au[g] < thr_lo) acc[g] = true;
                    else if ((uint64_t)au[g] >= thr_hi) acc[g] = false;
                    else chk[g] = true;
                    lo[g] = 0;
                    hi[g] = chk[g] ? trec[g].y : 0;
                    searching |= chk[g];
                }
                // is the candidate an out-neighbour of t?  Binary search of
                // t's row by name, every searching group one probe per round.
                bool found[G];
#pragma unroll
                for (int g = 0; g < G; ++g) found[g] = false;
                while (searching) {
                    searching = false;
#pragma unroll
                    for (int g = 0; g < G; ++g) {
                        if (!chk[g] || found[g] || lo[g] >= hi[g]) continue;
                        const uint32_t mid = lo[g] + ((hi[g] - lo[g]) >> 1);
                        const uint32_t nmid = entry_name(a.col_ext, (uint64_t)trec[g].x + mid, pol_stream);
                        ++probes;
                        if (nmid == cx[g].w) found[g] = true;
                        else if (nmid < cx[g].w) lo[g] = mid + 1;
                        else hi[g] = mid;
                        searching |= !found[g] && lo[g] < hi[g];
                    }
                }
                any = false;
#pragma unroll
                for (int g = 0; g < G; ++g) {
                    if (!pend[g]) continue;
                    if (chk[g]) acc[g] = (uint64_t)au[g] < (found[g] ? a.thr_nb : a.thr_out);
                    if (acc[g]) {
                        pend[g] = false;
                        t[g] = v[g];
                        trec[g] = rec[g];
                        v[g] = cx[g].x;
                        rec[g] = make_uint2(cx[g].y, cx[g].z);
                        nm[g] = cx[g].w;
                        ++moves;
                    } else {
                        ++k[g];
                        any = true;
                    }
                }
            }
#pragma unroll
            for (int g = 0; g < G; ++g) stage[wib][g][lane][p - c0] = dead[g] ? -1 : (int32_t)nm[g];
        }
    }

#pragma unroll
    for (int o = 16; o; o >>= 1) {
        moves += __shfl_xor_sync(kFull, moves, o);
        trials += __shfl_xor_sync(kFull, trials, o);
        probes += __shfl_xor_sync(kFull, probes, o);
    }
    if (lane == 0) {
        if (moves) atomicAdd(&a.ctrl[1], moves);
        if (trials) atomicAdd(&a.ctrl[2], trials);
        if (probes) atomicAdd(&a.ctrl[3], probes);
    }
}

}  // namespace

int launch_node2vec(ptw_graph *g, uint64_t w_begin, uint64_t w_end, uint32_t L, uint64_t seed,
                    int start_mode, uint32_t n_sources, const uint64_t thr[3], int32_t *paths)
{
    if (!ensure_ext_columns(g))
        return fail(PTW_ENOMEM, "node2vec needs the extended column copy (16 bytes per CSR entry), "
                                "which does not fit in device memory");
    const DeviceGraph &dg = g->dg;
    N2vArgs a;
    a.adj = dg.adj;
    a.col_ext = dg.col_ext;
    a.start_map = dg.idx2int;
    a.sources = g->sc.sources;
    a.int2name = dg.int2name;
    a.paths = paths;
    a.ctrl = g->sc.ctrl;
    a.w_begin = w_begin;
    a.n_walk = w_end - w_begin;
    a.thr_ret = thr[0];
    a.thr_nb = thr[1];
    a.thr_out = thr[2];
    a.n = dg.n;
    a.L = L;
    a.key0 = (uint32_t)seed;
    a.key1 = (uint32_t)(seed >> 32);
    a.n_sources = n_sources;
    a.start_mode = start_mode;
    a.hints = g->tune.cache_hints;
    const int G = g->tune.paths_ilp == 1 || g->tune.paths_ilp == 4 ? g->tune.paths_ilp : 2;
    const void *fn = G == 1 ? (const void *)k_node2vec<1> : G == 4 ? (const void *)k_node2vec<4>
                                                                    : (const void *)k_node2vec<2>;
    int per_sm = 0;
    PTW_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kN2vWarps * 32, 0));
    per_sm = std::max(per_sm, 1);
    const uint64_t groups = (a.n_walk + 31) / 32;
    const uint64_t per_block = (uint64_t)kN2vWarps * G;
    uint64_t grid = std::min<uint64_t>((uint64_t)g->num_sms * per_sm, (groups + per_block - 1) / per_block);
    grid = std::max<uint64_t>(grid, 1);
    void *args[] = {&a};
    PTW_CUDA(cudaLaunchKernel(fn, dim3((unsigned)grid), dim3(kN2vWarps * 32), args, 0, g->stream));
    return PTW_OK;
}

}  // namespace ptw
