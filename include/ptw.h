/*
 * ptw.h -- C ABI of the GB300 random-walk engine (libptw.so).
 *
 * The reference (PTWalker, a FlashMob fork) has no C ABI: its "plugin API" is
 * the compile-time app template passed to
 *     walk(FMobSolver*, uint64_t walker_num, int walk_len, uint64_t mem_quota,
 *          Alg& myapp, uint16_t walker_size)          src/core/solver.hpp:1049-1074
 * with the graph from
 *     Graph::load(path, GraphFormat, as_undirected, degree_boundary)
 *                                                      src/core/graph.hpp:277
 * and the apps pagerank (src/core/pagerank.cpp:10-90), PPR
 * (src/core/ppr.cpp:10-118), RWR (src/core/RWR.cpp:15-106) and DeepWalk
 * (src/core/deepwalk.cpp:10-41).  Each entry point below replaces one of
 * those pieces; the citation is on the declaration.
 *
 * Conventions
 *   - Status codes: PTW_OK (0) or a negative PTW_E* value; the message of the
 *     last failure on the calling thread is returned by ptw_last_error().
 *     No entry point aborts the process (the reference CHECK-aborts).
 *   - Vertex names are the u32 ids of the edge list.  Outputs indexed "by
 *     name" have id_bound = (largest name + 1) entries; names that do not
 *     occur in the graph read 0.
 *   - A ptw_graph owns its device memory and one CUDA stream.  A handle must
 *     not be used from two host threads at once.
 *   - Pointers named h_* are host memory; pointers named d_* are device
 *     memory on the graph's device.  Any host buffer works; pinned buffers
 *     copy faster.
 */
#ifndef PTW_H
#define PTW_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PTW_OK 0
#define PTW_EINVAL (-1)   /* invalid argument */
#define PTW_ENOMEM (-2)   /* device or host allocation refused */
#define PTW_ECUDA (-3)    /* CUDA runtime error */
#define PTW_ETIMEOUT (-4) /* a bounded device-side wait gave up */
#define PTW_EIO (-5)      /* file could not be read or parsed */
#define PTW_EFULL (-6)    /* a device table has no free capacity */
#define PTW_EBUSY (-7)    /* too many pipelined calls in flight */

#define PTW_FMT_BINARY 0  /* raw Edge{u32 src; u32 dst}[]   include/io.hpp:39-53 */
#define PTW_FMT_TEXT 1    /* "%u %u" lines, '#' comments    include/io.hpp:76-90 */

#define PTW_START_PER_VERTEX 0 /* walker w starts at the (w mod n)-th vertex by ascending name */
#define PTW_START_UNIFORM 1    /* uniform over vertices, with replacement (pagerank.cpp:70-80) */
#define PTW_START_SOURCES 2    /* uniform over a source list; one source = PPR (ppr.cpp:91-108) */

typedef struct ptw_graph ptw_graph;

typedef struct ptw_graph_info {
    uint32_t n_vertices;   /* distinct names in the edge list */
    uint32_t id_bound;     /* largest name + 1 */
    uint64_t n_edges;      /* CSR entries (directed edges after as_undirected) */
    uint32_t max_degree;
    uint32_t reserved;
    uint64_t device_bytes; /* resident device memory held by the graph */
} ptw_graph_info;

/* Walk configuration: the flag set -w / --sp / -l of the reference
 * (include/option.hpp:227-302) plus a seed and a start mode. */
typedef struct ptw_walk_cfg {
    uint64_t n_walkers;        /* -w */
    double sp;                 /* --sp: stop probability after each move, 0 < sp <= 1 */
    uint64_t seed;
    int32_t start_mode;        /* PTW_START_* */
    uint32_t max_moves;        /* 0 = unbounded (geometric length only) */
    const uint32_t *h_sources; /* names, for PTW_START_SOURCES */
    uint32_t n_sources;
    uint32_t reserved;
    uint64_t first_walker;     /* global id of the first walker: walkers are
                                  first_walker .. first_walker + n_walkers - 1.
                                  Every draw depends on the global id only, so
                                  a run split into shards equals the whole run;
                                  PPR query q uses first_walker = q << 32. */
} ptw_walk_cfg;

typedef struct ptw_walk_stats {
    uint64_t walkers;  /* walkers run */
    uint64_t moves;    /* edge traversals (walker steps) */
    uint64_t visits;   /* counted positions = walkers + moves for count apps */
    float kernel_ms;   /* device time of the walk kernel */
    float total_ms;    /* device time of the whole call, copies included */
} ptw_walk_stats;

/* Launch parameters of the walk kernels (chosen by ptw_autotune). */
typedef struct ptw_tune {
    int32_t block;         /* threads per block (multiple of 32) */
    int32_t ilp;           /* walkers held per thread: 1, 2 or 4 */
    int32_t chunk;         /* walker ids taken per warp refill */
    int32_t hot_k;         /* vertex ids < hot_k counted in shared memory (0 = off) */
    int32_t blocks_per_sm; /* 0 = as many as fit */
    int32_t min_blocks;    /* 2 = cap registers so two blocks fit per SM (block <= 512, 768 or
                              1024: 64, 42 or 32 registers); 0 = no cap */
    int32_t paths_ilp;     /* DeepWalk: groups of 32 walkers per warp, 1, 2 or 4 */
    int32_t cache_hints;   /* 1 = L2 evict_last for row records and counters, evict_first
                              for the column array; 0 = default L2 policy */
    int32_t paths_named;   /* DeepWalk: 1 = keep a {neighbour, name} column copy (8 bytes per
                              CSR entry, built on the first path walk) so a move needs no
                              separate name lookup; 0 = look names up per move */
    int32_t ext_columns;   /* bit 0: count / endpoint walks, bit 1: DeepWalk paths read a
                              {neighbour, its first column, its degree, its name} column copy
                              (16 bytes per CSR entry, built on first use), so a move is one
                              16-byte gather with no row-record load; 0 = off.  Falls back to
                              off when the copy does not fit. */
    int32_t gather_slots;  /* count / endpoint walks: 0 = walkers in registers (ilp per thread);
                              8 or 16 = walkers in shared memory, this many per thread, each
                              move an asynchronous 16-byte gather (cp.async) into shared memory,
                              so a thread keeps that many gathers in flight without registers.
                              Uses the extended column copy and a 16-byte record per vertex. */
    int32_t warp_agg;      /* count walks: 1 = lanes of a warp that visit the same vertex in the
                              same move merge their visits (__match_any_sync) into one reduction;
                              0 = one reduction per visit.  Needs min_blocks 0, gather_slots 0 */
} ptw_tune;

const char *ptw_last_error(void);
const char *ptw_version(void);

/* Device memory that batched queries and serving free goes back to a pool
 * that keeps up to a quarter of the device memory mapped between calls, so
 * the next call reuses it instead of mapping tens of GB again.  This hands
 * that cached memory back to the CUDA driver (after waiting for the device).  An
 * engine allocation that finds the device full trims and retries by itself;
 * call this before allocating elsewhere in the process when memory is short.
 * The reference's MemoryPool likewise holds every allocation until the pool
 * itself is freed (include/memory.hpp:174-205). */
int ptw_trim_memory(void);

/* ---- graph ------------------------------------------------------------ */

/* Replaces Graph::load (src/core/graph.hpp:277-785) with read_text_graph /
 * read_binary_graph (include/io.hpp:39-90).  Builds a degree-sorted device
 * CSR in place of the NUMA/cache partitioner. */
int ptw_graph_load(const char *path, int32_t fmt, int32_t as_undirected, ptw_graph **out);

/* Same as ptw_graph_load from in-memory edge arrays (graph.hpp:284-318). */
int ptw_graph_from_edges(const uint32_t *h_src, const uint32_t *h_dst, uint64_t m,
                         int32_t as_undirected, ptw_graph **out);

/* Same from a CSR, the inverse of ptw_graph_export_csr: row i of the n rows
 * is vertex h_names[i] (vertex i when h_names is NULL) and lists its out-
 * neighbours as row indices h_col[h_row_ptr[i] .. h_row_ptr[i+1]).  Replaces
 * the CSR half of Graph::load (graph.hpp:715-769).  Duplicates and
 * self-loops are kept; a row with no entries whose vertex is no one's
 * neighbour is not a vertex of the graph, as in an edge list.  PTW_EINVAL
 * for row_ptr[0] != 0, a decreasing row_ptr, a column index >= n, repeated
 * names or no entries. */
int ptw_graph_from_csr(const uint64_t *h_row_ptr /*[n+1]*/, const uint32_t *h_col /*[row_ptr[n]]*/,
                       uint32_t n, const uint32_t *h_names /*[n] or NULL*/, ptw_graph **out);

/* Synthetic R-MAT graph built on the device (no reference counterpart; the
 * reference reads files only).  2^scale * edge_factor raw edges with
 * quadrant probabilities a, b, c, 1-a-b-c; clean != 0 symmetrises, drops
 * self-loops, duplicates and isolated vertices and renames vertices 0..n-1. */
int ptw_graph_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c,
                   uint64_t seed, int32_t clean, ptw_graph **out);

int ptw_graph_get_info(const ptw_graph *g, ptw_graph_info *info);

/* Canonical CSR: vertex i = i-th smallest name, rows list neighbour
 * indices ascending.  Any output pointer may be NULL. */
int ptw_graph_export_csr(const ptw_graph *g, uint32_t *h_names /*[n]*/,
                         uint64_t *h_row_ptr /*[n+1]*/, uint32_t *h_col /*[m]*/);

/* Sorted edge list by (src, dst) name: the text/binary writer input
 * (include/io.hpp:55-74, :92-105). */
int ptw_graph_export_edges(const ptw_graph *g, uint32_t *h_src, uint32_t *h_dst);

/* Writes the graph's directed edges, sorted by (src, dst) name, in the
 * reference's text ("%u %u" per line) or binary (Edge{u32, u32}) format:
 * write_text_graph / write_binary_graph (include/io.hpp:55-74, :92-105),
 * formatted on all host threads.  PTW_EIO when the file cannot be written. */
int ptw_graph_save(const ptw_graph *g, const char *path, int32_t fmt);

void ptw_graph_free(ptw_graph *g);

int ptw_graph_set_tune(ptw_graph *g, const ptw_tune *t);
int ptw_graph_get_tune(const ptw_graph *g, ptw_tune *t);

/* ---- walks ------------------------------------------------------------ */

/* Visit counting: pagerank (src/core/pagerank.cpp:86-89) and single-source
 * PPR (src/core/ppr.cpp:114-117) driven by the solver loop
 * (src/core/solver.hpp:242-263).  Counts every position, start included,
 * into h_counts[id_bound] by name. */
int ptw_pagerank(ptw_graph *g, const ptw_walk_cfg *cfg, uint32_t *h_counts,
                 ptw_walk_stats *stats);

/* Pipelined form of ptw_pagerank for a caller that runs many walks: submit
 * launches the walk and the copy of its counts into h_counts[id_bound] and
 * returns at once with a ticket; wait blocks until that call's counts are
 * in h_counts and fills stats (kernel_ms = walk and scatter by name,
 * total_ms = until the copy ended).  The copy of one call runs on a second
 * stream while the next call walks.  Two calls may be in flight per graph
 * (a third submit returns PTW_EBUSY); h_counts must stay valid until the
 * wait and should be page-locked (cudaHostAlloc) for the copy to overlap.
 * Results equal ptw_pagerank's with the same configuration. */
int ptw_pagerank_submit(ptw_graph *g, const ptw_walk_cfg *cfg, uint32_t *h_counts, uint64_t *ticket);
int ptw_pagerank_wait(ptw_graph *g, uint64_t ticket, ptw_walk_stats *stats);

/* Device variant: d_counts[id_bound] receives the counts by name.  Runs on
 * the graph's stream and does not synchronise unless stats != NULL. */
int ptw_pagerank_dev(ptw_graph *g, const ptw_walk_cfg *cfg, uint32_t *d_counts,
                     ptw_walk_stats *stats);

/* RWR endpoint app (src/core/RWR.cpp:76-105, type=1 loop at
 * src/core/solver.hpp:284-306): h_pairs[2*w] = start name, h_pairs[2*w+1] =
 * name after the last move, for w in [0, n_walkers). */
int ptw_rwr(ptw_graph *g, const ptw_walk_cfg *cfg, uint32_t *h_pairs, ptw_walk_stats *stats);
int ptw_rwr_dev(ptw_graph *g, const ptw_walk_cfg *cfg, uint32_t *d_pairs, ptw_walk_stats *stats);

/* DeepWalk (src/core/deepwalk.cpp:25-37): n_walkers walks of L vertices
 * (L-1 moves), written as names into h_paths[n_walkers * L] (row-major,
 * int32).  A walk that reaches a vertex without out-edges is padded with -1.
 * cfg->sp and cfg->max_moves are ignored.  The host variant walks in chunks
 * whose copies into h_paths overlap the next chunks' walks (page-locked
 * h_paths copy fastest). */
int ptw_deepwalk(ptw_graph *g, const ptw_walk_cfg *cfg, uint32_t L, int32_t *h_paths,
                 ptw_walk_stats *stats);
int ptw_deepwalk_dev(ptw_graph *g, const ptw_walk_cfg *cfg, uint32_t L, int32_t *d_paths,
                     ptw_walk_stats *stats);

/* Second-order (node2vec) walks.  The reference parses -p / -q
 * (include/option.hpp:447-469) and prepares a neighbour query for them
 * (src/core/graph.hpp:787-820) in src/core/node2vec.cpp:8-24; its test
 * (src/test/debug/test_node2vec.cpp, third_party/knightking/test_node2vec.hpp:47-80)
 * states the law: from v, reached from t, the next vertex x is drawn over
 * v's out-edges with weight 1/p if x == t, 1 if x is an out-neighbour of t,
 * 1/q otherwise; the first move is uniform.  n_walkers walks of L vertices
 * (L-1 moves), written as names into h_paths[n_walkers * L] (row-major,
 * int32), padded with -1 after a vertex without out-edges, as ptw_deepwalk.
 * p and q must be positive and finite with max(1/p, 1, 1/q) / min(1/p, 1, 1/q)
 * <= 1024 (PTW_EINVAL otherwise).  Needs the extended column copy (16 bytes
 * per CSR entry) and an edge filter (a blocked Bloom filter, about 2 bytes
 * per CSR entry), both built on first use (PTW_ENOMEM when they do not fit).
 * cfg->sp and cfg->max_moves are ignored. */
typedef struct ptw_node2vec_stats {
    uint64_t walkers;
    uint64_t moves;    /* edge traversals */
    uint64_t trials;   /* candidate draws (>= moves; rejected candidates included) */
    uint64_t checks;   /* neighbour tests (edge-filter reads) */
    uint64_t probes;   /* reads of the previous vertex's row by the tests the filter passed */
    float kernel_ms;   /* device time of the walk kernel */
    float total_ms;    /* device time of the whole call, copies included */
} ptw_node2vec_stats;
int ptw_node2vec(ptw_graph *g, const ptw_walk_cfg *cfg, uint32_t L, double p, double q,
                 int32_t *h_paths, ptw_node2vec_stats *stats);
/* Device variant: d_paths[n_walkers * L] on the graph's device; runs on the
 * graph's stream and does not synchronise unless stats != NULL. */
int ptw_node2vec_dev(ptw_graph *g, const ptw_walk_cfg *cfg, uint32_t L, double p, double q,
                     int32_t *d_paths, ptw_node2vec_stats *stats);

/* Synchronise the graph's stream. */
int ptw_graph_sync(ptw_graph *g);

/* Run the graph's work on a caller-owned cudaStream_t from now on (NULL
 * returns to the graph's own stream), so callers can order and time it with
 * their own events.  No reference counterpart (the reference is CPU-only). */
int ptw_graph_set_stream(ptw_graph *g, void *cuda_stream);

/* ---- batched PPR / RWR ------------------------------------------------- */

/* One single-source query.  Its walkers have ids (query_id << 32) + j,
 * j < budget, so its result is the same alone or in any batch. */
typedef struct ptw_query {
    uint32_t source;   /* vertex name */
    uint32_t query_id;
    uint64_t budget;   /* walkers, 1 .. 2^28 */
} ptw_query;

#define PTW_APP_VISITS 0   /* count every position (PPR: src/core/ppr.cpp:114-117) */
#define PTW_APP_ENDPOINT 1 /* count the vertex after the last move (RWR: src/core/RWR.cpp:99-105) */

typedef struct ptw_batch_cfg {
    double sp;            /* stop probability after each move */
    uint64_t seed;
    int32_t app;          /* PTW_APP_* */
    uint32_t max_moves;   /* 0 = unbounded */
    uint64_t table_bytes; /* device memory for the count tables of one wave; 0 = 1/4 of free */
    double table_factor;  /* hash-table slots per expected counted position; 0 = 2.  A query
                             whose hash table would take at least 4n bytes counts into a
                             dense array of n 32-bit counters instead; a query
                             whose hash table fills is run again with a dense array, so results
                             never depend on it */
    uint32_t top_k;       /* 0 = every visited vertex, by name; k > 0 = each query's k largest
                             counts, by count descending then name (selected on the device) */
    uint32_t flags;       /* PTW_BATCH_* bits */
} ptw_batch_cfg;

/* The result lists stay in device memory for a GPU consumer (no copy to the
 * host): read them with ptw_batch_view_device; ptw_batch_export copies them
 * to the host on demand. */
#define PTW_BATCH_DEVICE_RESULTS 1u

typedef struct ptw_batch ptw_batch; /* the sparse results of one batch (host memory) */

/* Launch parameters of the batched walker kernel (ptw_ppr_batch only; the
 * serving loop keeps the defaults).  Zero fields take the defaults. */
typedef struct ptw_batch_tune {
    uint32_t desc_walkers;  /* walker ranks per work descriptor, 32 .. 65536; 0 = 256 */
    uint32_t blocks_per_sm; /* walker-kernel blocks (256 threads) per SM; 0 = as many as fit */
    uint64_t group_bytes;   /* descriptors interleave over groups of consecutive queries whose
                               count tables add up to about this many bytes, group after group;
                               0 = 384 MiB; UINT64_MAX = all queries in one group */
    uint32_t dense_ratio;   /* a query counts into a dense array of n counters when that takes
                               at most this many times its hash table's bytes; 0 = 1 */
    int32_t ext_columns;    /* 1 = walk the extended column copy, 2 = the plain columns,
                               0 = as bit 0 of the graph's walk tune */
} ptw_batch_tune;
int ptw_graph_set_batch_tune(ptw_graph *g, const ptw_batch_tune *t);
int ptw_graph_get_batch_tune(const ptw_graph *g, ptw_batch_tune *t);

/* Runs nq queries: the reference runs one source per process
 * (src/core/ppr.cpp:121-138 hard-codes internal id 0); here a device query
 * table feeds one persistent walker launch per wave of queries, waves sized
 * so their per-query hash tables fit table_bytes.  Results are kept sparse:
 * (vertex name, count) pairs per query, sorted by name. */
int ptw_ppr_batch(ptw_graph *g, const ptw_query *h_queries, uint32_t nq, const ptw_batch_cfg *cfg,
                  ptw_batch **out);
/* The same batch, resumable (no counterpart in the reference; its walks
 * restart from scratch).  Each completed wave's lists are appended to the
 * file at checkpoint_path (created when absent) before the next wave runs;
 * a call finds the waves already in the file and runs only the queries
 * without results.  At most max_waves waves run per call (0 = no limit):
 * while queries remain, the call returns PTW_OK with *out = NULL, and a
 * later call (or a new process) continues.  Draws depend on (seed, query
 * id, walker rank) only, so the final results equal one uninterrupted
 * ptw_ppr_batch call bit for bit.  The file is tied to the graph, the
 * configuration and the query table: another batch's file is PTW_EINVAL.
 * Host results only (no PTW_BATCH_DEVICE_RESULTS).  The caller deletes
 * the file when done. */
int ptw_ppr_batch_resumable(ptw_graph *g, const ptw_query *h_queries, uint32_t nq, const ptw_batch_cfg *cfg,
                            const char *checkpoint_path, uint32_t max_waves, ptw_batch **out);
/* Number of queries, total (name, count) entries, and walk statistics. */
int ptw_batch_info(const ptw_batch *b, uint32_t *nq, uint64_t *entries, ptw_walk_stats *stats);
/* h_offsets[nq + 1]: query i owns entries [h_offsets[i], h_offsets[i+1]).
 * Any pointer may be NULL. */
int ptw_batch_export(const ptw_batch *b, uint64_t *h_offsets, uint32_t *h_names, uint32_t *h_counts);
/* The same arrays without a copy: pointers into the batch's own host memory,
 * valid until ptw_batch_free. */
int ptw_batch_view(const ptw_batch *b, const uint64_t **offsets, const uint32_t **names,
                   const uint32_t **counts);
/* Device pointers of a batch run with PTW_BATCH_DEVICE_RESULTS: d_offsets
 * [nq + 1] (uint64), d_names / d_counts [entries], valid until
 * ptw_batch_free.  PTW_EINVAL for a batch whose results are on the host.
 * (ptw_batch_view of such a batch returns the host offsets and NULL lists.) */
int ptw_batch_view_device(const ptw_batch *b, const uint64_t **d_offsets, const uint32_t **d_names,
                          const uint32_t **d_counts);

/* Where the time of a batch call went.  Device phases are CUDA-event
 * intervals on the call's streams, summed over waves; host phases are wall
 * clock.  No counterpart in the reference. */
typedef struct ptw_batch_phases {
    double call_ms;        /* host: the whole ptw_ppr_batch call */
    double plan_ms;        /* host: query table and walker descriptors */
    double device_ms;      /* device: first upload to the last result copy */
    double upload_ms;      /* device: query table and descriptor uploads, count-table clear */
    double walk_ms;        /* device: the walker kernel */
    double count_ms;       /* device: compaction pass 1 (entries per chunk and table) and its scans */
    double place_ms;       /* device: compaction pass 2, hash-table sorts and placement (or top-k) */
    double copy_ms;        /* device: result copies to the host, summed over copies */
    double copy_tail_ms;   /* device: end of the last compaction kernel to the end of the last copy */
    double host_pages_ms;  /* host: waiting for result pages to be faulted in / page-locked */
    uint64_t copy_bytes;   /* bytes copied device -> host */
    uint32_t waves;        /* walker launches (waves, plus reruns of overflowed queries) */
    uint32_t reruns;       /* queries rerun with a dense array after their hash table filled */
} ptw_batch_phases;
int ptw_batch_get_phases(const ptw_batch *b, ptw_batch_phases *out);

/* Frees a batch and its result arrays.  Large host result arrays are
 * allocated for each batch and faulted in and page-locked while the device
 * walks (within a quarter of the host memory for all of them), so their
 * copies from the device run at link speed; freeing them takes a few ms
 * per GB.  Device-resident results go back to the library's memory pool at
 * once: finish (synchronise) every read of them first. */
void ptw_batch_free(ptw_batch *b);

/* FP64 oracle on the device: for each source name, the exact expected count
 * vector of the app (visits: pi_s / (sp (1-sp)) - sp/(1-sp) e_s; endpoint:
 * (pi_s - sp e_s) / (1-sp)) by power iteration until the added mass is below
 * tol, and the L1 distance between it and the normalised sparse counts of
 * query i of batch b (both normalised to sum 1).  h_l1[nq].  PTW_EINVAL for
 * a batch run with top_k > 0 (its lists are truncated). */
int ptw_batch_l1(ptw_graph *g, const ptw_batch *b, double sp, int32_t app, double tol, double *h_l1);
/* The same for nb batches over the same query sources (e.g. one query table
 * run with two budget rules), sharing one power iteration per 32 sources:
 * h_l1[j * nq + i] for query i of batch bs[j].  The truncated series is
 * within about 2 tol of the exact expectation in L1.  No counterpart in the
 * reference. */
int ptw_batch_l1_many(ptw_graph *g, const ptw_batch *const *bs, uint32_t nb, double sp, int32_t app, double tol,
                      double *h_l1);
/* L1 distance between the normalised counts of query i of batch a and of
 * batch ref (same query sources), h_l1[nq]: e.g. a low-budget estimate
 * against a high-budget one of the same query ids.  No counterpart in the
 * reference. */
int ptw_batch_l1_pair(ptw_graph *g, const ptw_batch *a, const ptw_batch *ref, double *h_l1);

/* ---- serving loop with continuous batching ----------------------------- */

/* No counterpart in the reference (one query per process).  Queries are
 * submitted as they arrive; each ptw_serve_step admits waiting queries while
 * their count tables fit the device table arena (admission by device
 * memory) and free query slots remain, then runs one tick: every active
 * query gets a share of tick_walkers walkers, all in one launch, so queries
 * that arrived while others were running share the GPU with them.  A query
 * completes when all its walkers have run; its sparse result is then
 * compacted and kept on the host until taken.  The tick's copy-in, walk
 * kernel and copy-out are one CUDA graph, replayed with new parameters. */
typedef struct ptw_server ptw_server;

typedef struct ptw_serve_cfg {
    double sp;
    uint64_t seed;
    int32_t app;            /* PTW_APP_* */
    uint32_t max_moves;
    uint64_t table_bytes;   /* device arena for count tables; 0 = 1/4 of free memory */
    uint64_t tick_walkers;  /* walkers started per tick over all active queries; 0 = 2^23 */
    uint32_t max_active;    /* query slots; 0 = 4096 */
    uint32_t use_graph;     /* 1 = replay the tick as a CUDA graph */
    double table_factor;    /* as in ptw_batch_cfg */
    uint32_t top_k;         /* as in ptw_batch_cfg */
    uint32_t staging_mb;    /* page-locked host staging for results, reserved at open, in MiB;
                               0 = 32.  It grows (doubling) when a tick's results need more:
                               a server that returns full vectors (top_k = 0) should reserve
                               what its largest ticks need (hundreds of MB) to keep the growth
                               out of its first ticks */
} ptw_serve_cfg;

typedef struct ptw_serve_result {
    uint32_t query_id;
    uint32_t source;
    uint64_t budget;
    uint64_t n_entries;     /* (name, count) pairs */
    double submit_s;        /* host clock (s since open) at submission */
    double admit_s;         /* ... when its table was allocated */
    double done_s;          /* ... when its result reached the host */
} ptw_serve_result;

int ptw_serve_open(ptw_graph *g, const ptw_serve_cfg *cfg, ptw_server **out);
/* Queues one query (validated now: unknown source or bad budget = PTW_EINVAL). */
int ptw_serve_submit(ptw_server *s, const ptw_query *q);
/* Admits, runs one tick, collects completed queries; *n_active and
 * *n_pending (may be NULL) report the state after the tick. */
int ptw_serve_step(ptw_server *s, uint32_t *n_done, uint32_t *n_active, uint32_t *n_pending);
/* Oldest completed, not yet taken result: 1 and *r filled, or 0 if none. */
int ptw_serve_poll(ptw_server *s, ptw_serve_result *r);
/* Copies the polled result's entries (n_entries each) and drops it; NULL
 * outputs drop it without copying. */
int ptw_serve_take(ptw_server *s, uint32_t *h_names, uint32_t *h_counts);
/* Zero-copy view of the polled result's entries: pinned host memory the
 * device wrote them to, valid until that result is taken or the server is
 * closed. */
int ptw_serve_view(const ptw_server *s, const uint32_t **names, const uint32_t **counts);

typedef struct ptw_serve_stats {
    uint64_t ticks;         /* steps that ran a tick */
    uint64_t moves;         /* walker moves run */
    uint64_t walkers;       /* walkers run */
    uint64_t completed;     /* queries completed */
    uint64_t entries;       /* (name, count) entries produced */
    uint64_t retries;       /* queries re-run with a table that cannot fill */
    uint64_t pinned_bytes;  /* pinned host staging held for results */
    uint32_t active;        /* queries holding a table now */
    uint32_t pending;       /* queries waiting for admission now */
    double step_ms;         /* host wall time inside ptw_serve_step */
    double device_ms;       /* device time of the ticks: plan copy-in, walk, flag copy-out */
    double collect_ms;      /* compaction and copy-out of completed queries */
} ptw_serve_stats;
/* Counters since ptw_serve_open. */
int ptw_serve_get_stats(const ptw_server *s, ptw_serve_stats *out);
/* Seconds since ptw_serve_open on the server's clock. */
double ptw_serve_clock(const ptw_server *s);
void ptw_serve_close(ptw_server *s);
/* Saves a server's state between steps (no counterpart in the reference,
 * which has no server): its configuration, clock and statistics, the
 * pending queries, the active queries with the walker ranks run so far and
 * their count tables, and the finished results not yet taken.  Written to
 * path.tmp, then renamed over path. */
int ptw_serve_save(const ptw_server *s, const char *path);
/* Opens a server on graph g (the graph the state was saved from, else
 * PTW_EINVAL) in the saved state; the clock continues from the saved one.
 * Draws depend on (seed, query id, walker rank) only, so every query
 * finishes with the same counts as on the server that was saved.
 * PTW_ENOMEM when the table arena here cannot hold the saved active
 * queries (a smaller table_bytes or less free device memory). */
int ptw_serve_restore(ptw_graph *g, const char *path, ptw_server **out);

/* Synthetic Chung-Lu power-law graph built on the device: n vertices with
 * expected degrees proportional to (i + 1)^(-1/(gamma-1)), mean degree
 * mean_degree; symmetrised, self-loops, duplicates and isolated vertices
 * removed, names 0..n'-1.  No reference counterpart. */
int ptw_graph_chung_lu(uint32_t n, double gamma, double mean_degree, uint64_t seed, ptw_graph **out);

/* ---- learned walker budgets --------------------------------------------- */

/* No counterpart in the reference, which gives every query the same walker
 * count.  Eight cheap features per source (K5), one warp per source:
 *   0 log(1+deg)        1 mean log(1+deg(u))   2 max log(1+deg(u))
 *   3 min log(1+deg(u)) 4 log(1+sum deg(u))    5 std log(1+deg(u))
 *   6 fraction of neighbours of degree 1      7 log(1+sum deg(u)/deg)
 * over the out-neighbours u of the source.  h_feat[ns * 8]. */
int ptw_source_features(ptw_graph *g, const uint32_t *h_sources, uint32_t ns, float *h_feat);

/* FP32 MLP 8 -> 64 -> 64 -> 1 (ReLU) trained with MSE and Adam on the GPU by
 * hand-written forward / backward / update kernels (K6).  Inputs are
 * standardised with mean / std taken from the training data; so is the
 * target.  Parameter order: W1[8][64], b1[64], W2[64][64], b2[64], w3[64], b3.
 * h_norm: mu[8], sigma[8], target mu, target sigma. */
#define PTW_MLP_IN 8
#define PTW_MLP_HIDDEN 64
#define PTW_MLP_NPARAMS 4801
#define PTW_MLP_NNORM 18
typedef struct ptw_mlp ptw_mlp;
int ptw_mlp_create(uint64_t seed, ptw_mlp **out);
int ptw_mlp_set_params(ptw_mlp *m, const float *h_params, const float *h_norm);
int ptw_mlp_get_params(const ptw_mlp *m, float *h_params, float *h_norm);
/* h_y[B]: de-standardised predictions. */
int ptw_mlp_forward(ptw_mlp *m, const float *h_x, uint32_t B, float *h_y);
/* Loss on standardised targets and its gradient (h_grad may be NULL). */
int ptw_mlp_grad(ptw_mlp *m, const float *h_x, const float *h_t, uint32_t B, double *h_loss, float *h_grad);
/* Sets the standardisation from (h_x, h_t), then runs `epochs` passes of
 * mini-batch Adam; h_loss_curve[epochs] (may be NULL) gets the mean loss. */
int ptw_mlp_train(ptw_mlp *m, const float *h_x, const float *h_t, uint32_t N, uint32_t batch, uint32_t epochs,
                  float lr, uint64_t seed, float *h_loss_curve);
void ptw_mlp_free(ptw_mlp *m);

/* Count walk that allocates no device memory.  No counterpart in the
 * reference.  For callers that cannot call cudaMalloc when they run (a host
 * whose pool allocator owns all device memory, or a context where an
 * allocation or its implied synchronisation is not allowed).  Same results
 * as ptw_pagerank_dev: counts by name into the caller's d_counts[id_bound],
 * issued on cuda_stream (NULL = the graph's stream), asynchronous.  On
 * another stream the walk waits for work already queued on the graph's
 * stream, and the graph's stream (so ptw_graph_free too) waits for the walk.
 * Limits: graphs of at most PTW_NOALLOC_MAX_VERTICES vertices (PTW_EINVAL
 * beyond), per-vertex or uniform starts only.  The per-vertex counters and
 * the walker cursor live in one fixed device array inside the library
 * (about 16 MiB on every GPU that loads it, held until exit).  The first call
 * on a device looks up that array's address and creates two ordering
 * events: make it before any stream capture, and do not call this again
 * after cudaDeviceReset in the same process.  All calls share the array:
 * calls that overlap on the GPU race and must be serialised. */
#define PTW_NOALLOC_MAX_VERTICES (1u << 22)
int ptw_pagerank_noalloc(const ptw_graph *g, const ptw_walk_cfg *cfg, uint32_t *d_counts,
                         void *cuda_stream);

/* Autotuner of the batched kernel (the idea of the reference's per-setting
 * step-cost cache, src/core/mini_bmk.hpp:62-117): runs the caller's batch
 * (q, nq, cfg; results kept on the device and discarded) under candidate
 * ptw_batch_tune values and times the device phases from the first upload
 * to the end of compaction.  Descriptor size x group bytes first, then
 * blocks per SM x dense ratio x column layout around the best, then the
 * three fastest again in interleaved rounds.  Stores the fastest in the
 * graph and returns it; *best_ms (may be NULL) gets its median time. */
int ptw_autotune_batch(ptw_graph *g, const ptw_query *q, uint32_t nq, const ptw_batch_cfg *cfg,
                       ptw_batch_tune *best, double *best_ms);

/* Autotuner (the idea of the sampler micro-benchmark cache,
 * src/core/mini_bmk.hpp:62-117): times the count walk over candidate
 * launch parameters on this graph and device, stores the fastest in the
 * graph and returns it. n_walkers = 0 means one walker per vertex. */
int ptw_autotune(ptw_graph *g, double sp, uint64_t n_walkers, ptw_tune *best);

/* Measurement only: random 4-byte gathers per second that the current GPU
 * serves from an array of array_bytes (filled with hashed values), each of
 * `chains` (1, 2, 4 or 8) independent chains per thread loading at an index
 * hashed from its previous value.  Above L2 size this is the ceiling of a
 * walk move's dependent gather, which a streaming copy peak overstates. */
int ptw_probe_gather(uint64_t array_bytes, uint32_t chains, double *loads_per_s);

#ifdef __cplusplus
}
#endif

#endif /* PTW_H */
