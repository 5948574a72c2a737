/*
 * CPU oracle for the walker-update path.  TEST INFRASTRUCTURE ONLY: the
 * tests, the smoke check and the CPU-baseline leg of bench.py load this file
 * as a checker; the GPU product never links or calls it.
 *
 * What it restates (reference paths are relative to the PTWalker project):
 *
 *  - Walker update, count-before-move apps (pagerank / PPR):
 *      src/core/solver.hpp:242-263  (update; if sid>0 {sample; sid--} else finish)
 *      src/core/pagerank.cpp:86-89  (update = rooted_value[vid]++)
 *    Every position of a walker is counted, the start included, so a walker
 *    that makes L moves contributes L+1 visits.
 *  - Walk length: src/core/pagerank.cpp:41-68 draws L = 1 + k with
 *    P(k) = (1-sp)^k sp from a 128-entry CDF.  Here the same law is produced
 *    step by step: after every move the walker stops with probability sp.
 *  - Move-then-update app (RWR endpoint): src/core/solver.hpp:284-306 and
 *    src/core/RWR.cpp:76-105 -- the walker records (start, vertex after its
 *    last move).
 *  - Fixed-length walks (DeepWalk): src/core/deepwalk.cpp:25-28 makes L-1
 *    moves, so a path holds L vertices.
 *  - Neighbour choice: src/core/sampler.hpp:214-217 (uniform over the CSR row,
 *    multi-edges counted with multiplicity).
 *  - Second-order (node2vec) walks: the law of the reference's node2vec test
 *    (see ora_replay_node2vec below).
 *
 * The reference draws from an unseeded xorshift* (include/random.hpp:144-177),
 * so its trajectories cannot be reproduced.  This oracle and the GPU engine
 * instead share one counter-based stream, Philox4x32-10 (Salmon, Moraes, Dror,
 * Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC'11), keyed by the
 * seed and indexed by (walker id, step, purpose):
 *
 *    key = (seed_lo, seed_hi)
 *    start draw  : ctr = (wid_lo, wid_hi, 0,    PTW_TAG_START)
 *    move `step` : ctr = (wid_lo, wid_hi, step, PTW_TAG_WALK)
 *                  out.x -> neighbour index  = mulhi32(out.x, degree)
 *                  out.y -> stop after move  iff out.y < thr, thr = floor(sp * 2^32)
 *    R-MAT edge e, levels 4j..4j+3 : ctr = (e_lo, e_hi, j, PTW_TAG_RMAT)
 *    node2vec trials 2k, 2k+1 of move `step` : ctr = (wid_lo, wid_hi, step, PTW_TAG_N2V + k)
 *
 * All graph arguments are in canonical index space: vertex i is the i-th
 * smallest vertex name, and each CSR row lists neighbour indices in ascending
 * order with multi-edges adjacent.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define PTW_TAG_WALK  0x57414C4Bu /* "WALK" */
#define PTW_TAG_START 0x53545254u /* "STRT" */
#define PTW_TAG_RMAT  0x524D4154u /* "RMAT" */

enum { ORA_START_PER_VERTEX = 0, ORA_START_UNIFORM = 1, ORA_START_SOURCES = 2 };

/* Philox4x32-10 as specified in the SC'11 paper: ten rounds of the 4x32
 * S-box with multipliers 0xD2511F53 / 0xCD9E8D57 and Weyl key increments
 * 0x9E3779B9 / 0xBB67AE85. */
void ora_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t x0 = ctr[0], x1 = ctr[1], x2 = ctr[2], x3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; r++) {
        uint64_t p0 = (uint64_t)0xD2511F53u * x0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * x2;
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ x1 ^ k0;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ x3 ^ k1;
        x1 = (uint32_t)p1;
        x3 = (uint32_t)p0;
        x0 = n0;
        x2 = n2;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = x0; out[1] = x1; out[2] = x2; out[3] = x3;
}

static inline uint32_t mulhi32(uint32_t a, uint32_t b)
{
    return (uint32_t)(((uint64_t)a * b) >> 32);
}

static inline void draw(uint64_t seed, uint64_t wid, uint32_t word2, uint32_t tag, uint32_t out[4])
{
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint32_t ctr[4] = {(uint32_t)wid, (uint32_t)(wid >> 32), word2, tag};
    ora_philox4x32_10(ctr, key, out);
}

/* Raw R-MAT edge generator (no symmetrisation or clean-up).  Edge e picks one
 * of four quadrants per level from a 32-bit draw u: u < ta -> (0,0),
 * u < tab -> (0,1), u < tabc -> (1,0), else (1,1); level 0 sets the top bit. */
void ora_rmat_edges(uint32_t scale, uint64_t e_begin, uint64_t e_end,
                    uint32_t ta, uint32_t tab, uint32_t tabc, uint64_t seed,
                    uint32_t *src, uint32_t *dst)
{
#pragma omp parallel for schedule(static)
    for (int64_t e = (int64_t)e_begin; e < (int64_t)e_end; e++) {
        uint32_t u = 0, v = 0, w[4];
        for (uint32_t l = 0; l < scale; l++) {
            if ((l & 3u) == 0) draw(seed, (uint64_t)e, l >> 2, PTW_TAG_RMAT, w);
            uint32_t x = w[l & 3u];
            uint32_t rb = x >= tab;                       /* quadrants (1,0),(1,1) */
            uint32_t cb = (x >= ta && x < tab) || x >= tabc; /* quadrants (0,1),(1,1) */
            u = (u << 1) | rb;
            v = (v << 1) | cb;
        }
        src[e - e_begin] = u;
        dst[e - e_begin] = v;
    }
}

/* ---- R-MAT clean-up straight to a canonical CSR ------------------------
 * Symmetrise, drop self-loops and duplicates, drop isolated vertices and
 * rename the rest 0..n-1 in ascending order -- the same graph the numpy
 * path in graph.py builds, at a speed that makes scale 24 practical.  Keys
 * (u << bits | v) are sorted with a parallel LSD radix sort. */

static void radix_sort_u64(uint64_t *a, uint64_t *tmp, uint64_t n, int key_bits, int nt)
{
    const int R = 11, B = 1 << R;
    uint64_t *hist = (uint64_t *)calloc((size_t)nt * B, sizeof(uint64_t));
    for (int shift = 0; shift < key_bits; shift += R) {
        memset(hist, 0, (size_t)nt * B * sizeof(uint64_t));
#pragma omp parallel num_threads(nt)
        {
            int t = 0;
#ifdef _OPENMP
            t = omp_get_thread_num();
#endif
            uint64_t lo = n * (uint64_t)t / nt, hi = n * (uint64_t)(t + 1) / nt;
            uint64_t *h = hist + (size_t)t * B;
            for (uint64_t i = lo; i < hi; i++) h[(a[i] >> shift) & (B - 1)]++;
#pragma omp barrier
#pragma omp single
            {
                uint64_t sum = 0;
                for (int d = 0; d < B; d++)
                    for (int tt = 0; tt < nt; tt++) {
                        uint64_t c = hist[(size_t)tt * B + d];
                        hist[(size_t)tt * B + d] = sum;
                        sum += c;
                    }
            }
            for (uint64_t i = lo; i < hi; i++) tmp[h[(a[i] >> shift) & (B - 1)]++] = a[i];
        }
        uint64_t *s = a; a = tmp; tmp = s;
    }
    /* an odd number of passes leaves the result in the scratch buffer */
    if (((key_bits + R - 1) / R) & 1) memcpy(tmp, a, n * sizeof(uint64_t));
    free(hist);
}

int ora_rmat_clean_csr(uint32_t scale, uint32_t edge_factor, uint32_t ta, uint32_t tab,
                       uint32_t tabc, uint64_t seed, int n_threads, uint32_t *n_out,
                       uint64_t *m_out, uint64_t **row_ptr_out, uint32_t **col_out)
{
    const uint64_t m = (uint64_t)edge_factor << scale;
    const int bits = (int)scale;
    const uint64_t V = 1ull << scale;
    const uint64_t SENT = ~0ull;
    if (n_threads < 1) n_threads = 1;
    uint64_t *keys = (uint64_t *)malloc(2 * m * sizeof(uint64_t));
    uint64_t *tmp = (uint64_t *)malloc(2 * m * sizeof(uint64_t));
    if (!keys || !tmp) { free(keys); free(tmp); return -2; }
#pragma omp parallel for schedule(static) num_threads(n_threads)
    for (int64_t e = 0; e < (int64_t)m; e++) {
        uint32_t u = 0, v = 0, w[4];
        for (uint32_t l = 0; l < scale; l++) {
            if ((l & 3u) == 0) draw(seed, (uint64_t)e, l >> 2, PTW_TAG_RMAT, w);
            uint32_t x = w[l & 3u];
            u = (u << 1) | (uint32_t)(x >= tab);
            v = (v << 1) | (uint32_t)((x >= ta && x < tab) || x >= tabc);
        }
        if (u == v) {
            keys[2 * e] = keys[2 * e + 1] = SENT;
        } else {
            keys[2 * e] = ((uint64_t)u << bits) | v;
            keys[2 * e + 1] = ((uint64_t)v << bits) | u;
        }
    }
    /* sentinels sort last when the full 64-bit width is not sorted: map
     * them to the largest 2*bits-bit value + 1 range by clearing high bits
     * after sorting on 2*bits+1 bits. */
    const uint64_t mask = (2 * bits + 1 >= 64) ? ~0ull : ((1ull << (2 * bits + 1)) - 1);
#pragma omp parallel for schedule(static) num_threads(n_threads)
    for (int64_t i = 0; i < (int64_t)(2 * m); i++)
        if (keys[i] == SENT) keys[i] = mask;
    radix_sort_u64(keys, tmp, 2 * m, 2 * bits + 1, n_threads);
    free(tmp);
    /* unique, dropping sentinels */
    uint64_t mm = 0;
    for (uint64_t i = 0; i < 2 * m; i++) {
        if (keys[i] == mask) break;
        if (mm == 0 || keys[i] != keys[mm - 1]) keys[mm++] = keys[i];
    }
    /* present vertices (symmetric: every endpoint is a source) */
    uint32_t *rank = (uint32_t *)calloc(V + 1, sizeof(uint32_t));
    if (!rank) { free(keys); return -2; }
    for (uint64_t i = 0; i < mm; i++) rank[keys[i] >> bits] = 1;
    uint32_t n = 0;
    for (uint64_t x = 0; x < V; x++) {
        uint32_t p = rank[x];
        rank[x] = n;
        n += p;
    }
    uint64_t *row_ptr = (uint64_t *)calloc((size_t)n + 1, sizeof(uint64_t));
    uint32_t *col = (uint32_t *)malloc((mm ? mm : 1) * sizeof(uint32_t));
    if (!row_ptr || !col) { free(keys); free(rank); free(row_ptr); free(col); return -2; }
    const uint64_t lowmask = (1ull << bits) - 1;
#pragma omp parallel for schedule(static) num_threads(n_threads)
    for (int64_t i = 0; i < (int64_t)mm; i++) col[i] = rank[keys[i] & lowmask];
    for (uint64_t i = 0; i < mm; i++) row_ptr[rank[keys[i] >> bits] + 1]++;
    for (uint32_t i = 0; i < n; i++) row_ptr[i + 1] += row_ptr[i];
    free(keys);
    free(rank);
    *n_out = n;
    *m_out = mm;
    *row_ptr_out = row_ptr;
    *col_out = col;
    return 0;
}

void ora_free(void *p) { free(p); }

static inline uint32_t start_index(uint64_t wid, uint32_t n, int start_mode,
                                   const uint32_t *sources, uint32_t n_sources, uint64_t seed)
{
    uint32_t w[4];
    switch (start_mode) {
    case ORA_START_PER_VERTEX:
        return (uint32_t)(wid % n);
    case ORA_START_UNIFORM:
        draw(seed, wid, 0, PTW_TAG_START, w);
        return mulhi32(w[0], n);
    default:
        if (n_sources == 1) return sources[0];
        draw(seed, wid, 0, PTW_TAG_START, w);
        return sources[mulhi32(w[0], n_sources)];
    }
}

/*
 * Replays walkers wid in [w_begin, w_end) and returns the total number of
 * moves.  Walker semantics: count the start; then repeat { if the vertex has
 * no out-edge, stop; move to a uniform neighbour; count it; stop if the
 * termination draw hits or max_moves (if non-zero) is reached }.
 * counts[n] accumulates visits (may be NULL); pairs[2*(w-w_begin)] receives
 * (start, end) indices (may be NULL); moves_out[w-w_begin] the move count
 * (may be NULL).  n_threads > 1 runs the walkers with OpenMP.
 */
uint64_t ora_replay_walks(const uint64_t *row_ptr, const uint32_t *col, uint32_t n,
                          uint64_t w_begin, uint64_t w_end, uint64_t thr, uint64_t seed,
                          int start_mode, const uint32_t *sources, uint32_t n_sources,
                          uint32_t max_moves, uint32_t *counts, uint32_t *pairs,
                          uint32_t *moves_out, int n_threads)
{
    uint64_t total = 0;
#ifdef _OPENMP
    if (n_threads < 1) n_threads = 1;
#pragma omp parallel for schedule(dynamic, 4096) reduction(+ : total) num_threads(n_threads)
#endif
    for (int64_t wi = (int64_t)w_begin; wi < (int64_t)w_end; wi++) {
        uint64_t wid = (uint64_t)wi;
        uint32_t v = start_index(wid, n, start_mode, sources, n_sources, seed);
        uint32_t s0 = v;
        if (counts) {
#pragma omp atomic
            counts[v]++;
        }
        uint32_t step = 0;
        for (;;) {
            uint64_t b = row_ptr[v], deg = row_ptr[v + 1] - b;
            if (deg == 0) break;
            uint32_t w[4];
            draw(seed, wid, step, PTW_TAG_WALK, w);
            v = col[b + mulhi32(w[0], (uint32_t)deg)];
            step++;
            if (counts) {
#pragma omp atomic
                counts[v]++;
            }
            if ((uint64_t)w[1] < thr) break;
            if (max_moves && step >= max_moves) break;
        }
        if (pairs) {
            pairs[2 * (wid - w_begin)] = s0;
            pairs[2 * (wid - w_begin) + 1] = v;
        }
        if (moves_out) moves_out[wid - w_begin] = step;
        total += step;
    }
    return total;
}

/*
 * Fixed-length walks: walker wid writes L vertex indices to
 * paths[(wid-w_begin)*L ...]: the start, then L-1 moves.  A walker that
 * reaches a vertex without out-edges writes -1 for every remaining position.
 */
void ora_replay_paths(const uint64_t *row_ptr, const uint32_t *col, uint32_t n,
                      uint64_t w_begin, uint64_t w_end, uint32_t L, uint64_t seed,
                      int start_mode, const uint32_t *sources, uint32_t n_sources,
                      int32_t *paths, int n_threads)
{
#ifdef _OPENMP
    if (n_threads < 1) n_threads = 1;
#pragma omp parallel for schedule(dynamic, 1024) num_threads(n_threads)
#endif
    for (int64_t wi = (int64_t)w_begin; wi < (int64_t)w_end; wi++) {
        uint64_t wid = (uint64_t)wi;
        int32_t *row = paths + (wid - w_begin) * (uint64_t)L;
        uint32_t v = start_index(wid, n, start_mode, sources, n_sources, seed);
        if (L == 0) continue;
        row[0] = (int32_t)v;
        int dead = 0;
        for (uint32_t step = 0; step + 1 < L; step++) {
            if (!dead) {
                uint64_t b = row_ptr[v], deg = row_ptr[v + 1] - b;
                if (deg == 0) {
                    dead = 1;
                } else {
                    uint32_t w[4];
                    draw(seed, wid, step, PTW_TAG_WALK, w);
                    v = col[b + mulhi32(w[0], (uint32_t)deg)];
                }
            }
            row[step + 1] = dead ? -1 : (int32_t)v;
        }
    }
}

/*
 * Second-order (node2vec) walks.  The reference parses -p / -q
 * (include/option.hpp:447-469), prepares its neighbour query for them
 * (src/core/graph.hpp:787-820: Bloom filter, then binary search in the
 * sorted row) and calls FMobSolver::set_node2vec (src/core/node2vec.cpp:8-24,
 * src/core/solver.hpp:156-159), whose second-order step is commented out; its
 * test (src/test/debug/test_node2vec.cpp, with the transition matrix of
 * third_party/knightking/test_node2vec.hpp:47-80) states the law this replay
 * follows, the node2vec law of Grover and Leskovec (KDD'16): from vertex v,
 * reached from t, the next vertex x is drawn over the CSR row of v (multi-edges
 * with multiplicity) with weight 1/p if x == t, 1 if x is an out-neighbour of
 * t, 1/q otherwise.  The first move (no t yet) is uniform.
 *
 * Drawing is rejection sampling over the row (the method of KnightKing, Yang
 * et al., SOSP'19): trial k of move `step` takes two 32-bit words of
 *    draw(seed, wid, step, PTW_TAG_N2V + k/2): words (0, 1) for even k,
 *    (2, 3) for odd k;
 * the first word picks the candidate x = row[mulhi32(word, degree)], the
 * second accepts it iff word < thr[class(x)], with
 *    thr[c] = w_c >= M ? 2^32 : floor(w_c / M * 2^32),   M = max(1/p, 1, 1/q).
 * The first move accepts trial 0.  Trial ORA_N2V_MAX_TRIALS - 1 is accepted
 * whatever its draw, so a move always ends; callers keep max(w)/min(w) <=
 * 1024, which makes reaching it less likely than 1e-27 per move.
 * Paths are written as in ora_replay_paths; the return value is the number of
 * trials (candidate draws) made.  simple_symmetric (ora_csr_simple_symmetric
 * of the graph) enables the outlier folding below for a small p.
 */
#define PTW_TAG_N2V 0x4E320000u /* "N2" + trial pair index */
#define ORA_N2V_MAX_TRIALS 65536u

void ora_n2v_thresholds(double p, double q, uint64_t thr[3])
{
    double w[3] = {1.0 / p, 1.0, 1.0 / q}; /* return, neighbour of t, other */
    double m = w[0] > w[1] ? w[0] : w[1];
    if (w[2] > m) m = w[2];
    for (int c = 0; c < 3; c++)
        thr[c] = w[c] >= m ? (uint64_t)1 << 32 : (uint64_t)(w[c] / m * 4294967296.0);
}

/*
 * Outlier folding (KnightKing, Yang et al., SOSP'19) for a small p: when the
 * return weight 1/p is the only largest weight, the envelope of the
 * rejection draw is M' = max(1, 1/q) instead, and the return edge's excess
 * (1/p - M') sits in an appendix beside the row.  On a graph whose rows hold
 * no repeated neighbour and whose edges all have their reverse (a simple
 * symmetric graph), t appears exactly once in the row of v, so the appendix
 * has width a = (1/p - M') / M' slots.  In fixed point with 2^20 units per
 * slot (a_fx = floor(a * 2^20)), trial words (cu, au) place the point
 * pos = floor(cu * (deg * 2^20 + a_fx) / 2^32); pos >= deg * 2^20 returns to
 * t at once, else the candidate is row[pos >> 20], accepted iff
 * au < thr'[class], thr' the thresholds against M'.  thr[0..2] are thr',
 * thr[3] = a_fx; ora_n2v_fold returns 0 (and leaves thr alone) when the
 * return weight is not the only largest one.
 */
int ora_n2v_fold(double p, double q, uint64_t thr[4])
{
    double w[3] = {1.0 / p, 1.0, 1.0 / q};
    double m = w[1] > w[2] ? w[1] : w[2];
    if (!(w[0] > m)) return 0;
    thr[0] = (uint64_t)1 << 32;
    for (int c = 1; c < 3; c++)
        thr[c] = w[c] >= m ? (uint64_t)1 << 32 : (uint64_t)(w[c] / m * 4294967296.0);
    thr[3] = (uint64_t)((w[0] - m) / m * 1048576.0);
    return 1;
}

/* 1 iff no row holds a repeated neighbour and every edge (u, v) has its
 * reverse (v, u). */
int ora_csr_simple_symmetric(const uint64_t *row_ptr, const uint32_t *col, uint32_t n)
{
    int ok = 1;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 4096) reduction(& : ok)
#endif
    for (int64_t ui = 0; ui < (int64_t)n; ui++) {
        uint32_t u = (uint32_t)ui;
        for (uint64_t e = row_ptr[u]; e < row_ptr[u + 1]; e++) {
            if (e > row_ptr[u] && col[e] == col[e - 1]) ok = 0;
            uint32_t v = col[e];
            uint64_t lo = row_ptr[v], hi = row_ptr[v + 1];
            while (lo < hi) {
                uint64_t mid = lo + (hi - lo) / 2;
                if (col[mid] < u) lo = mid + 1;
                else hi = mid;
            }
            if (!(lo < row_ptr[v + 1] && col[lo] == u)) ok = 0;
        }
    }
    return ok;
}

static int row_has(const uint64_t *row_ptr, const uint32_t *col, uint32_t t, uint32_t x)
{
    uint64_t lo = row_ptr[t], hi = row_ptr[t + 1];
    while (lo < hi) {
        uint64_t mid = lo + (hi - lo) / 2;
        if (col[mid] < x) lo = mid + 1;
        else hi = mid;
    }
    return lo < row_ptr[t + 1] && col[lo] == x;
}

uint64_t ora_replay_node2vec(const uint64_t *row_ptr, const uint32_t *col, uint32_t n,
                             uint64_t w_begin, uint64_t w_end, uint32_t L, uint64_t seed,
                             double p, double q, int start_mode, const uint32_t *sources,
                             uint32_t n_sources, int simple_symmetric, int32_t *paths, int n_threads)
{
    uint64_t thr[4] = {0, 0, 0, 0};
    ora_n2v_thresholds(p, q, thr);
    const int fold = simple_symmetric && ora_n2v_fold(p, q, thr);
    uint64_t trials_total = 0;
#ifdef _OPENMP
    if (n_threads < 1) n_threads = 1;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : trials_total) num_threads(n_threads)
#endif
    for (int64_t wi = (int64_t)w_begin; wi < (int64_t)w_end; wi++) {
        uint64_t wid = (uint64_t)wi;
        int32_t *row = paths + (wid - w_begin) * (uint64_t)L;
        uint32_t v = start_index(wid, n, start_mode, sources, n_sources, seed);
        if (L == 0) continue;
        row[0] = (int32_t)v;
        uint32_t t = 0;
        int dead = 0;
        for (uint32_t step = 0; step + 1 < L; step++) {
            if (!dead) {
                uint64_t b = row_ptr[v], deg = row_ptr[v + 1] - b;
                if (deg == 0) {
                    dead = 1;
                } else {
                    uint32_t w[4], x = 0;
                    for (uint32_t k = 0;; k++) {
                        if ((k & 1) == 0) draw(seed, wid, step, PTW_TAG_N2V + (k >> 1), w);
                        uint32_t cu = w[(k & 1) * 2], au = w[(k & 1) * 2 + 1];
                        trials_total++;
                        if (fold && step > 0) {
                            uint64_t tf = (deg << 20) + thr[3];
                            uint64_t pos = (uint64_t)cu * (tf >> 32) + (((uint64_t)cu * (tf & 0xFFFFFFFFu)) >> 32);
                            if (pos >= (deg << 20)) { /* the appendix: back to t */
                                x = t;
                                break;
                            }
                            x = col[b + (pos >> 20)];
                        } else {
                            x = col[b + mulhi32(cu, (uint32_t)deg)];
                        }
                        if (step == 0 || k + 1 == ORA_N2V_MAX_TRIALS) break;
                        int c = x == t ? 0 : row_has(row_ptr, col, t, x) ? 1 : 2;
                        if ((uint64_t)au < thr[c]) break;
                    }
                    t = v;
                    v = x;
                }
            }
            row[step + 1] = dead ? -1 : (int32_t)v;
        }
    }
    return trials_total;
}
