/*
 * Partitioned walker sweeps: the reference's solver design restated as the
 * timed CPU baseline.  TEST / MEASUREMENT INFRASTRUCTURE ONLY (the bench's
 * CPU-baseline leg and reference arm time it; the tests check it); the GPU
 * product never links or calls it.
 *
 * The reference (paths relative to the PTWalker project) splits the
 * vertices into partitions sized to the CPU caches
 * (src/core/graph.hpp:159-169, :385-485), keeps unfinished walkers in
 * per-(thread, partition) pools (src/core/solver.hpp:568-671) and sweeps: a
 * thread takes a partition, advances every walker in its pools until the
 * walker finishes or moves into another partition
 * (src/core/solver.hpp:222-309), and hands the movers to the pools of their
 * new partitions (src/core/solver.hpp:359-479).  A partition's counters are
 * touched only by the thread sweeping it, so counting needs no atomics, and
 * its rows and counters stay in that core's caches while it is swept.
 *
 * Here: the vertices are relabelled by descending degree (as the reference
 * does when it loads a graph, src/core/graph.hpp:515-628), so the hubs that
 * most walkers stand on share partitions; partitions are ranges of
 * consecutive ids cut so that a partition's row offsets, counters and column
 * entries take about part_bytes (a hub whose row alone is larger gets a
 * partition of its own, as the reference's hub partitions do,
 * src/core/graph.hpp:159-169); walkers are 16-byte records kept in pools per
 * (thread, partition), as in the reference.  The draws are the oracle's
 * Philox stream (oracle.c), and every position is counted once when the
 * walker is processed there, so the counts and the move total equal
 * ora_replay_walks's bit for bit.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define PTW_TAG_WALK 0x57414C4Bu  /* "WALK" */
#define PTW_TAG_START 0x53545254u /* "STRT" */

typedef struct {
    uint64_t wid;
    uint32_t v;
    uint32_t st; /* moves made << 1 | 1 when the last move's draw stops the walk */
} walker_t;

/* a growable walker pool */
typedef struct {
    walker_t *w;
    size_t n, cap;
} pool_t;

static inline uint32_t mulhi(uint32_t a, uint32_t b) { return (uint32_t)(((uint64_t)a * b) >> 32); }

/* Philox4x32-10 (Salmon et al., SC'11), the same function as
 * ora_philox4x32_10 in oracle.c, inlined here because the baseline is timed. */
static inline void draw(uint64_t seed, uint64_t wid, uint32_t word2, uint32_t tag, uint32_t out[4])
{
    uint32_t x0 = (uint32_t)wid, x1 = (uint32_t)(wid >> 32), x2 = word2, x3 = tag;
    uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    for (int r = 0; r < 10; ++r) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * x0, p1 = (uint64_t)0xCD9E8D57u * x2;
        const uint32_t y0 = (uint32_t)(p1 >> 32) ^ x1 ^ k0, y1 = (uint32_t)p1;
        const uint32_t y2 = (uint32_t)(p0 >> 32) ^ x3 ^ k1, y3 = (uint32_t)p0;
        x0 = y0;
        x1 = y1;
        x2 = y2;
        x3 = y3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = x0;
    out[1] = x1;
    out[2] = x2;
    out[3] = x3;
}

/* appends x; returns 0 when host memory runs out */
static inline int push(pool_t *l, walker_t x)
{
    if (l->n == l->cap) {
        const size_t c = l->cap ? 2 * l->cap : 64;
        walker_t *p = (walker_t *)realloc(l->w, c * sizeof *p);
        if (!p) return 0;
        l->w = p;
        l->cap = c;
    }
    l->w[l->n++] = x;
    return 1;
}

static inline uint32_t start_index(uint64_t wid, uint32_t n, int start_mode, const uint32_t *sources,
                                   uint32_t n_sources, uint64_t seed)
{
    uint32_t w[4];
    if (start_mode == 0) return (uint32_t)(wid % n);
    if (start_mode == 1) {
        draw(seed, wid, 0, PTW_TAG_START, w);
        return mulhi(w[0], n);
    }
    if (n_sources == 1) return sources[0];
    draw(seed, wid, 0, PTW_TAG_START, w);
    return sources[mulhi(w[0], n_sources)];
}

/* the partition holding id v: the last p with bounds[p] <= v */
static inline uint32_t part_of(const uint32_t *bounds, uint32_t P, uint32_t v)
{
    uint32_t lo = 0, hi = P; /* bounds[lo] <= v < bounds[hi] */
    while (hi - lo > 1) {
        const uint32_t mid = lo + (hi - lo) / 2;
        if (bounds[mid] <= v) lo = mid;
        else hi = mid;
    }
    return lo;
}

static inline int thread_id(void)
{
#ifdef _OPENMP
    return omp_get_thread_num();
#else
    return 0;
#endif
}

/*
 * Count walks of walkers [w_begin, w_end) (semantics of ora_replay_walks).
 * The graph may be relabelled: perm (NULL = none) maps a canonical vertex
 * index to its id in row_ptr / col, whose rows keep the canonical order of
 * their neighbours (so neighbour rank r is the same neighbour); start
 * indices are mapped through it, sources are given relabelled.  counts[n]
 * (by relabelled id) is overwritten.  info[3] (may be NULL): partitions,
 * sweeps, walkers moved between partitions.  Returns the total number of
 * moves, or UINT64_MAX when host memory runs out.
 *
 * Pools: cur[t * P + p] holds the walkers thread t handed to partition p in
 * the previous sweep.  A sweep takes partitions dynamically; the thread that
 * takes p advances the walkers of every thread's pool for p and appends each
 * walker that crosses into partition q to its own pool nxt[self * P + q].
 */
uint64_t ora_partitioned_walks(const uint64_t *row_ptr, const uint32_t *col, uint32_t n, const uint32_t *perm,
                               uint64_t w_begin, uint64_t w_end, uint64_t thr, uint64_t seed, int start_mode,
                               const uint32_t *sources, uint32_t n_sources, uint32_t max_moves,
                               uint64_t part_bytes, uint32_t *counts, int n_threads, uint64_t *info)
{
    const int T = n_threads < 1 ? 1 : n_threads;
    const uint64_t W = w_end - w_begin;
    memset(counts, 0, (size_t)n * sizeof *counts);
    if (info) info[0] = info[1] = info[2] = 0;
    if (n == 0 || W == 0) return 0;
    /* partitions: consecutive ids while the bytes (12 per vertex, 4 per
     * column entry) stay within part_bytes; bounds[p] = first id of p */
    const uint64_t budget = part_bytes ? part_bytes : 1;
    uint32_t *bounds = (uint32_t *)malloc(((size_t)n + 1) * sizeof *bounds);
    uint32_t P = 0;
    if (bounds) {
        uint64_t bytes = 0;
        for (uint32_t v = 0; v < n; ++v) {
            const uint64_t b = 12 + 4 * (row_ptr[v + 1] - row_ptr[v]);
            if (v == 0 || bytes + b > budget) {
                bounds[P++] = v;
                bytes = 0;
            }
            bytes += b;
        }
        bounds[P] = n;
    }
    const size_t NP = (size_t)T * P;
    pool_t *cur = (pool_t *)calloc(NP ? NP : 1, sizeof *cur);
    pool_t *nxt = (pool_t *)calloc(NP ? NP : 1, sizeof *nxt);
    uint64_t *moves = (uint64_t *)calloc((size_t)T * 8, sizeof *moves); /* one cache line per thread */
    uint64_t total = UINT64_MAX, sweeps = 0, migrations = 0;
    int ok = bounds && cur && nxt && moves;

    if (ok) {
        /* each thread places a static slice of the walkers at their starts */
#pragma omp parallel num_threads(T) reduction(& : ok)
        {
            const int t = thread_id();
            pool_t *mine = cur + (size_t)t * P;
#pragma omp for schedule(static)
            for (int64_t i = 0; i < (int64_t)W; ++i) {
                const uint64_t wid = w_begin + (uint64_t)i;
                uint32_t v = start_index(wid, n, start_mode, sources, n_sources, seed);
                if (perm && start_mode != 2) v = perm[v];
                const walker_t x = {wid, v, 0u};
                ok &= push(&mine[part_of(bounds, P, v)], x);
            }
        }
    }
    size_t active = ok ? (size_t)W : 0;
    while (ok && active) {
        ++sweeps;
#pragma omp parallel num_threads(T) reduction(& : ok)
        {
            const int self = thread_id();
            pool_t *out = nxt + (size_t)self * P;
            uint64_t mv = 0;
#pragma omp for schedule(dynamic, 1)
            for (int64_t p = 0; p < (int64_t)P; ++p) {
                const uint32_t lo = bounds[p], span = bounds[p + 1] - bounds[p];
                for (int t = 0; t < T; ++t) {
                    pool_t *in = &cur[(size_t)t * P + p];
                    for (size_t i = 0; i < in->n; ++i) {
                        const walker_t x = in->w[i];
                        uint32_t v = x.v, step = x.st >> 1;
                        int stop = (int)(x.st & 1);
                        counts[v]++; /* arrival: the start, or a move from another partition */
                        while (!stop) {
                            const uint64_t b = row_ptr[v], deg = row_ptr[v + 1] - b;
                            if (deg == 0) break;
                            uint32_t r[4];
                            draw(seed, x.wid, step, PTW_TAG_WALK, r);
                            v = col[b + mulhi(r[0], (uint32_t)deg)];
                            ++step;
                            ++mv;
                            stop = (uint64_t)r[1] < thr || (max_moves && step >= max_moves);
                            if (v - lo >= span) { /* into another partition's pool */
                                const walker_t y = {x.wid, v, (step << 1) | (uint32_t)stop};
                                ok &= push(&out[part_of(bounds, P, v)], y);
                                break;
                            }
                            counts[v]++;
                        }
                    }
                    in->n = 0;
                }
            }
            moves[(size_t)self * 8] += mv;
        }
        active = 0;
        for (size_t i = 0; i < NP; ++i) active += nxt[i].n;
        migrations += active;
        pool_t *sw = cur;
        cur = nxt;
        nxt = sw;
    }
    if (ok) {
        total = 0;
        for (int t = 0; t < T; ++t) total += moves[(size_t)t * 8];
    }
    if (info) {
        info[0] = P;
        info[1] = sweeps;
        info[2] = migrations;
    }
    free(bounds);
    for (size_t i = 0; cur && i < NP; ++i) free(cur[i].w);
    for (size_t i = 0; nxt && i < NP; ++i) free(nxt[i].w);
    free(cur);
    free(nxt);
    free(moves);
    return total;
}

/*
 * The graph relabelled by descending degree, ties by index (graph-load work
 * of the partitioned walks): perm[canonical index] = new id; row_ptr_out
 * [n + 1] and col_out [m] hold the relabelled CSR, each row keeping the
 * canonical order of its neighbours.  Returns 0, or -1 when host memory runs
 * out.
 */
int ora_degree_relabel(const uint64_t *row_ptr, const uint32_t *col, uint32_t n, uint32_t *perm,
                       uint64_t *row_ptr_out, uint32_t *col_out, int n_threads)
{
    const int T = n_threads < 1 ? 1 : n_threads;
    uint64_t maxdeg = 0;
    for (uint32_t v = 0; v < n; ++v) {
        const uint64_t d = row_ptr[v + 1] - row_ptr[v];
        if (d > maxdeg) maxdeg = d;
    }
    /* counting sort by degree, descending; stable, so ties stay in index order */
    uint64_t *first = (uint64_t *)calloc(maxdeg + 2, sizeof *first);
    uint32_t *order = (uint32_t *)malloc(((size_t)n + 1) * sizeof *order);
    if (!first || !order) {
        free(first);
        free(order);
        return -1;
    }
    for (uint32_t v = 0; v < n; ++v) first[maxdeg - (row_ptr[v + 1] - row_ptr[v]) + 1]++;
    for (uint64_t d = 1; d <= maxdeg + 1; ++d) first[d] += first[d - 1];
    for (uint32_t v = 0; v < n; ++v) {
        const uint64_t slot = first[maxdeg - (row_ptr[v + 1] - row_ptr[v])]++;
        order[slot] = v;
        perm[v] = (uint32_t)slot;
    }
    row_ptr_out[0] = 0;
    for (uint32_t j = 0; j < n; ++j) row_ptr_out[j + 1] = row_ptr_out[j] + (row_ptr[order[j] + 1] - row_ptr[order[j]]);
#pragma omp parallel for schedule(dynamic, 4096) num_threads(T)
    for (int64_t j = 0; j < (int64_t)n; ++j) {
        const uint32_t v = order[j];
        const uint64_t a = row_ptr[v], len = row_ptr[v + 1] - a, o = row_ptr_out[j];
        for (uint64_t e = 0; e < len; ++e) col_out[o + e] = perm[col[a + e]];
    }
    free(first);
    free(order);
    return 0;
}
