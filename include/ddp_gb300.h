/*
 * ddp_gb300 — GA* and dynamic A* on int32 CSR graphs, GB300 (sm_103a).
 *
 * C-ABI boundary.  Plain pointers and sizes, opaque handles, integer status
 * codes; no C++ or torch types cross it.  Each entry point names the
 * reference interface (lkoshale/DDP, LIB/include and the standalone
 * programs) that it replaces.
 *
 * Conventions shared by every entry point:
 *   - Graphs are directed, node ids 0..n-1, arc weights uint32 (the
 *     reference's `unsigned int` weights), costs int32 with DDP_INF
 *     (= INT_MAX) for "unreachable", as the reference's Cx array.
 *   - A cost is f(t) = g(t) + h(t), the value the reference reports as
 *     Cx[target] (LIB/include/a_star.h:239-245, GA_star/A_star_cpu.cpp:191).
 *     With the heuristics built here h(t) = 0, so the cost is the path weight.
 *   - Offsets may be given in the reference's layout (n entries, the last
 *     row ends at e) or with a sentinel (n+1 entries); both are accepted.
 *   - Host arrays passed in are copied before the call returns; the caller
 *     keeps ownership.  Handles own their device memory.
 *   - Calls on one handle are serialised by the handle; different handles
 *     may be used from different threads.
 *   - On failure a call returns a non-zero DDP_ERR_* code and
 *     ddp_last_error() describes it (per calling thread).  Nothing calls
 *     exit(): the reference's gpuErrchk -> exit(code)
 *     (LIB/include/utils.cuh:10-18) becomes a returned status.
 */
#ifndef DDP_GB300_H
#define DDP_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DDP_INF 2147483647

enum ddp_status {
    DDP_OK = 0,
    DDP_ERR_INVALID = 1,        /* bad argument (range, size, null)            */
    DDP_ERR_CUDA = 2,           /* CUDA runtime error                          */
    DDP_ERR_IO = 3,             /* file missing / malformed                    */
    DDP_ERR_OOM = 4,            /* device or host allocation failed            */
    DDP_ERR_QUEUE_OVERFLOW = 5, /* a search queue outgrew its capacity         */
    DDP_ERR_TIMEOUT = 6,        /* a bounded device-side wait gave up          */
    DDP_ERR_NO_DEVICE = 7       /* no usable CUDA device                       */
};

/* Heuristic kinds for ddp_heuristic_build. */
enum ddp_heuristic_kind {
    DDP_H_ZERO = 0,      /* h = 0 (Dijkstra order)                              */
    DDP_H_BFS_HOPS = 1,  /* reverse-BFS hop count to the target x min arc
                            weight (GA_star/bfs_hx.cu on the reverse graph of
                            DA_star/genOpCSR.cpp); unreachable -> pruned      */
    DDP_H_MANHATTAN = 2, /* |dx| + |dy| on node coordinates x min arc weight   */
    DDP_H_USER = 3,      /* caller-supplied array (a_star.h:34 set_huiristics) */
    DDP_H_EUCLID = 5,    /* floor(rho * floor(|xy(v) - xy(t)|)), rho a 16.16
                            fixed-point lower bound of w / length over the arcs
                            (ddp_graph_set_euclid); integer arithmetic only    */
    DDP_H_BFS_CAPPED = 4, /* DDP_H_BFS_HOPS with the BFS stopped after the level
                            where it has reached max(4096, n/32) nodes; nodes
                            not reached get (last level + 1) x min weight,
                            which stays admissible and consistent            */
    DDP_H_LANDMARK = 6,  /* ALT: max over landmarks L of d(L,t) - d(L,v) and
                            d(v,L) - d(t,L) (triangle inequality: admissible;
                            consistent while the table is unscaled); needs
                            ddp_landmarks_build.  No
                            reference counterpart (the reference only has
                            bfs_hx.cu hop counts, which carry little on random
                            graphs)                                           */
    DDP_H_BIDIR = 7,     /* batch and serving only: no heuristic; a forward
                            search from s and a reverse search from t meet
                            in the middle (bidirectional Dijkstra).  No
                            table, so it stays valid under updates.  No
                            reference counterpart                             */
    DDP_H_BIDIR_EUCLID = 8,    /* DDP_H_BIDIR steered by average Euclidean
                                  potentials (bidirectional A*): coordinates
                                  and ddp_graph_set_euclid's scale          */
    DDP_H_BIDIR_MANHATTAN = 9  /* DDP_H_BIDIR steered by average Manhattan
                                  potentials (x min weight): grids whose arcs
                                  join 4-neighbours                          */
};

typedef struct ddp_graph ddp_graph;         /* device-resident CSR + reverse CSR */
typedef struct ddp_heuristic ddp_heuristic; /* device-resident h for one target  */
typedef struct ddp_query ddp_query;         /* result of one single-query solve  */
typedef struct ddp_batch ddp_batch;         /* multi-query engine (slots)        */

/* Search options (all fields 0 = automatic). */
typedef struct ddp_opts {
    int32_t K;         /* nodes expanded per iteration (the reference's K queues);
                          0 = the whole current bucket                          */
    int32_t delta;     /* bucket width on f; 0 = chosen from the arc weights    */
    int32_t block;     /* threads per CTA                                        */
    int32_t grid;      /* CTAs (single query) or concurrent slots (batch)        */
    int64_t queue_cap; /* entries per search queue                               */
    void *stream;      /* cudaStream_t; NULL = the handle's own stream           */
    int32_t group;     /* batch: CTAs working on one query (1 = one CTA)          */
    int32_t flags;     /* DDP_OPT_* bits                                          */
} ddp_opts;

/* ddp_opts.flags */
#define DDP_OPT_SYNC 1    /* one-CTA slots use the phase-synchronous engine      */
#define DDP_OPT_ONE_CTA 2 /* ddp_solve: one CTA with the asynchronous engine      */
#define DDP_OPT_HASH 4    /* DDP_H_BIDIR batches: each slot keeps its closed set in
                             a hash table sized to the touched nodes, not n     */

/* ---- library ----------------------------------------------------------- */
const char *ddp_last_error(void);
int ddp_version(void);
/* Number of CUDA devices visible (0 on a machine without a GPU). */
int ddp_device_count(void);

/* ---- graph: LIB/include/graph.h:13-43 (Graph<T>), graph.cuh:12-89
 *      (GPU_Graph<T>::__gpu_alloc H2D copy) ----------------------------- */
/* n nodes, e arcs; offsets has n (reference layout) or n+1 entries
 * (offsets_len); cols[e] with col < 0 = absent arc; weights[e]. */
int ddp_graph_from_csr(int32_t n, int64_t e, const int32_t *offsets, int32_t offsets_len,
                       const int32_t *cols, const uint32_t *weights, ddp_graph **out);
/* Reads the reference's graph.txt format ("N E", E cols, N offsets,
 * E weights; Graph<T>::read_graph, graph.h:93-118) and uploads it. */
int ddp_graph_load_text(const char *path, ddp_graph **out);
/* Node coordinates (x,y interleaved, 2n int32) for the Manhattan heuristic. */
int ddp_graph_set_coords(ddp_graph *g, const int32_t *xy);
/* 16.16 fixed-point scale of the Euclidean heuristic: rho_fp / 65536 must not
 * exceed w / length for any arc (length measured in coordinate units). */
int ddp_graph_set_euclid(ddp_graph *g, uint32_t rho_fp);
int ddp_graph_info(const ddp_graph *g, int32_t *n, int64_t *e, uint32_t *wmin, uint32_t *wmax);
/* Copies the current forward CSR back (offsets n+1, cols/weights e). */
int ddp_graph_read_csr(const ddp_graph *g, int32_t *offsets, int32_t *cols, uint32_t *weights);
int ddp_graph_free(ddp_graph *g);

/* ---- heuristic: GA_star/bfs_hx.cu (program), LIB a_star.h:34
 *      set_huiristics(U*) ------------------------------------------------ */
/* Landmark table for DDP_H_LANDMARK: `count` (4, 8, ..., 64) landmarks picked
 * farthest-first from a seeded start, with distances to and from every
 * node from 2 x count exhaustive searches on the device, stored as 16-bit
 * entries (count x 4 bytes per node): exact while every distance is below
 * 65535, else floor(d / s) with the smallest such scale s, the bound then
 * losing at most s - 1 per landmark term.  out_ids (nullable) receives the landmarks.  Updates to the graph
 * (ddp_dyn_update, ddp_serve_update) make the table stale: landmark
 * heuristics then fail with DDP_ERR_INVALID until it is rebuilt.  No
 * reference counterpart. */
int ddp_landmarks_build(ddp_graph *g, int32_t count, uint64_t seed, int32_t *out_ids);

/* ddp_landmarks_build with the entry width chosen: bits = 16 (as above) or
 * 8 (count = 8, 16, ..., 128; count x 2 bytes per node; exact while every
 * distance is below 255, else floor(d / s) with the smallest such s).
 * Halving the row halves the bytes each heuristic evaluation reads, for a
 * bound that is up to s - 1 weaker per term.  No reference counterpart. */
int ddp_landmarks_build_bits(ddp_graph *g, int32_t count, int32_t bits, uint64_t seed, int32_t *out_ids);

/* Builds h for `target` on the device.  user_h (DDP_H_USER only) holds n
 * values; negative values mean "target unreachable from here".  out_h
 * (optional, n values) receives h, -1 for nodes that cannot reach target. */
int ddp_heuristic_build(ddp_graph *g, int32_t target, int32_t kind, const int32_t *user_h,
                        int32_t *out_h, ddp_heuristic **out);
int ddp_heuristic_free(ddp_heuristic *h);

/* ---- single query GA*: LIB a_star.cu:109-303 (GPU_A_Star::get_path) ----- */
/* h may be NULL (h = 0).  The result handle holds the cost and the path. */
int ddp_solve(ddp_graph *g, const ddp_heuristic *h, int32_t source, int32_t target,
              const ddp_opts *opts, ddp_query **out);
/* Cost of a finished query (DDP_INF when the target is unreachable). */
int ddp_query_cost(const ddp_query *q, int32_t *cost);
/* Path source..target (a_star.cu:281-301).  *len = full length (0 when
 * unreachable); at most cap ids are written. */
int ddp_path_read(const ddp_query *q, int32_t *buf, int32_t cap, int32_t *len);
/* Device counters of a query, DDP_STATS values: [0] nodes expanded,
 * [1] arcs scanned, [2] successful relaxations, [3] search phases,
 * [4] nodes reached by the heuristic BFS, [5] reverse arcs it scanned
 * (4 and 5 are filled when the heuristic BFS runs inside a batch),
 * [6] open-list entries re-read by bucket splits, [7] distinct nodes
 * reached. */
#define DDP_STATS 8
int ddp_query_stats(const ddp_query *q, int64_t *stats);
int ddp_query_free(ddp_query *q);

/* ---- batched multi-query engine (no reference counterpart: the
 *      reference solves one (s,t) per process, GA_v2.cu:301-305) --------- */
/* hkind: DDP_H_ZERO, DDP_H_BFS_HOPS / DDP_H_BFS_CAPPED (per target, built
 * inside the batch kernel), DDP_H_MANHATTAN, DDP_H_EUCLID (coordinates),
 * DDP_H_LANDMARK (ddp_landmarks_build first) or DDP_H_BIDIR,
 * DDP_H_BIDIR_EUCLID, DDP_H_BIDIR_MANHATTAN (one-CTA slots, 32 bytes per
 * node of slot state).  opts: group = CTAs per slot
 * (1 = the asynchronous one-CTA engine), block, K, delta, grid = slot cap;
 * ddp_batch_tune picks them.  A query whose search outgrew
 * its slot's queues reports cost -1 from ddp_batch_solve_device;
 * ddp_batch_solve re-runs such queries on the single-query engine. */
int ddp_batch_create(ddp_graph *g, int32_t hkind, const ddp_opts *opts, ddp_batch **out);
/* Solves n queries from host arrays; out_cost[n]; out_path_len[n] optional. */
int ddp_batch_solve(ddp_batch *b, int32_t n, const int32_t *sources, const int32_t *targets,
                    int32_t *out_cost, int32_t *out_path_len);
/* Same with device pointers and no host synchronisation (stream-ordered on
 * the batch's stream); d_cost / d_path_len are device arrays of n
 * (d_path_len may be NULL).  Repeated calls replay a CUDA graph of the
 * launch while its arguments are unchanged; any change (other arrays, a
 * rebuilt landmark table, a re-laid-out dynamic graph) captures it again.
 * Fails with DDP_ERR_INVALID when the landmark table is stale.  Paths of
 * such a solve are read back from the caller's d_sources / d_targets: keep
 * them unchanged until ddp_batch_path is done. */
int ddp_batch_solve_device(ddp_batch *b, int32_t n, const int32_t *d_sources,
                           const int32_t *d_targets, int32_t *d_cost, int32_t *d_path_len);
/* Waits for the batch stream. */
int ddp_batch_sync(ddp_batch *b);
/* Path of query i of the last solve (source..target). */
int ddp_batch_path(ddp_batch *b, int32_t i, int32_t *buf, int32_t cap, int32_t *len);
/* Per-query device counters of the last solve: stats[DDP_STATS*i + k] as
 * in ddp_query_stats; start/end (optional) = device timestamps in ns. */
int ddp_batch_stats(ddp_batch *b, int64_t *stats, int64_t *t_start_ns, int64_t *t_end_ns);
/* Engine shape: concurrent query slots, queue capacity per slot, threads
 * per CTA. */
int ddp_batch_info(const ddp_batch *b, int32_t *slots, int64_t *queue_cap, int32_t *block);
/* CTAs per query slot of the batch engine. */
int ddp_batch_group(const ddp_batch *b, int32_t *group);
/* Kernel launches of the last solve (for accounting). */
int ddp_batch_launches(const ddp_batch *b, int32_t *launches);
int ddp_batch_free(ddp_batch *b);

/* Autotuner: times the batch engine on the n sample queries for a grid of
 * slot shapes (group x block), then bucket widths around the automatic one,
 * then K (multi-CTA slots), and returns the fastest options in *best (other
 * fields copied from base, which may be NULL).  Every configuration must
 * return the same costs, else DDP_ERR_CUDA.  best_qps / trials (nullable)
 * receive the winner's queries/s and the number of timed configurations.
 * The reference fixes K by hand per run; no counterpart. */
int ddp_batch_tune(ddp_graph *g, int32_t hkind, int32_t n, const int32_t *sources, const int32_t *targets,
                   const ddp_opts *base, ddp_opts *best, double *best_qps, int32_t *trials);

/* ---- dynamic A*: DA_star/DA_dyn_cpu.cu (program), LIB d_a_star.cuh:9-86
 *      (GPU_D_A_Star, declared there but not compiling) ------------------- */
typedef struct ddp_dyn ddp_dyn;
/* Runs the initial A* from source to target on g (hkind DDP_H_ZERO or
 * DDP_H_BFS_HOPS) and keeps the search resident.  The graph switches to a
 * layout with growable rows; it stays usable by every other call and
 * ddp_graph_read_csr returns its current arcs.  One dynamic search per graph
 * at a time.  opts.grid = CTAs of the initial search (0 = half the SMs);
 * opts.group = CTAs of each update batch's repair and resumed search
 * (0 = the initial search's grid; 1 = one CTA, block barriers; more = a
 * cooperative grid of that many). */
int ddp_dyn_create(ddp_graph *g, int32_t source, int32_t target, int32_t hkind,
                   const ddp_opts *opts, ddp_dyn **out);
/* Applies one update batch (DA_dyn_cpu.cu:1295-1326 Updates.txt lines):
 * flag 1 = insert u->v with weight w (appended to row u), flag 0 = delete the
 * first live u->v arc of the pre-batch graph, flag 2 = set the weight of
 * that arc to w (no reference counterpart; a delete plus an insert gives the
 * same arc set).  Deletes and weight changes run first, in batch order, each
 * on the graph as the earlier ones left it; inserts follow.  A batch of up
 * to 4,096 updates is applied on the device (one upload); larger batches,
 * and batches whose rows no longer fit the arrays' reserve, are applied on
 * the host copy of the graph, which is laid out again as needed.  Repairs
 * the search incrementally and returns the new cost (DDP_INF when the target
 * became unreachable). */
int ddp_dyn_update(ddp_dyn *d, int32_t n, const int32_t *flag, const int32_t *u, const int32_t *v,
                   const uint32_t *w, int32_t *out_cost);
int ddp_dyn_cost(const ddp_dyn *d, int32_t *cost);
int ddp_dyn_path(ddp_dyn *d, int32_t *buf, int32_t cap, int32_t *len);
/* Counters of the last create/update: cost, path length, status, search
 * phases, invalidated nodes, re-seeded nodes, relaxed arc heads, lowered hop
 * counts, expanded nodes, scanned arcs (10 values). */
int ddp_dyn_stats(const ddp_dyn *d, int64_t *stats);
/* CTAs of the initial search and of each update batch's repair and resumed
 * search (opts.grid and opts.group as resolved against the device). */
int ddp_dyn_grid(const ddp_dyn *d, int32_t *search_ctas, int32_t *update_ctas);
int ddp_dyn_free(ddp_dyn *d);

/* Up to k successive source -> target paths by last-arc deletion
 * (k-short/DA_dyn_cpu.cu:1297-1340): path i is the shortest path after the
 * last arcs of paths 0..i-1 were deleted, found by the dynamic search.
 * costs[i] (DDP_INF once no path is left); the paths are concatenated in
 * path_buf, path i at [path_offsets[i], path_offsets[i+1]); *found = paths
 * found.  The deletions stay in the graph, as in the reference, unless
 * restore != 0 (the arcs are re-inserted, at the ends of their rows).
 * DDP_ERR_INVALID when path_cap is too small (path_offsets[k] is then the
 * size needed; costs are filled). */
int ddp_kpaths(ddp_graph *g, int32_t source, int32_t target, int32_t hkind, int32_t k, int32_t restore,
               int32_t *costs, int32_t *path_buf, int64_t path_cap, int64_t *path_offsets, int32_t *found);

/* ---- serving: continuous batching with interleaved updates (no reference
 *      counterpart: the reference answers one (s,t) per process) --------- */
typedef struct ddp_server ddp_server;
/* Slots (one CTA each, fixed queue/state footprint; as many as fit in half of
 * free device memory) serve requests published in a ring of max_requests
 * entries in pinned host memory mapped into the device.  The graph is kept
 * in `versions` (2..64) device copies so that updates never stop searches
 * in flight; the graph switches to the dynamic layout.  hkind: ZERO,
 * BFS_HOPS, BFS_CAPPED, MANHATTAN, EUCLID, or LANDMARK (a fixed graph:
 * ddp_serve_update then fails with DDP_ERR_INVALID). */
int ddp_serve_create(ddp_graph *g, int32_t hkind, const ddp_opts *opts, int64_t max_requests,
                     int32_t versions, ddp_server **out);
/* Publishes n requests; *first_id = id of the first.  Non-blocking. */
int ddp_serve_submit(ddp_server *s, int32_t n, const int32_t *sources, const int32_t *targets,
                     int64_t *first_id);
/* Collects up to max finished requests: id, cost (DDP_INF = unreachable),
 * host-observed latency (submit to this poll) and graph version.  Any array
 * may be NULL.  Non-blocking except for rare re-runs of oversized searches. */
int ddp_serve_poll(ddp_server *s, int32_t max, int64_t *ids, int32_t *costs, int64_t *latency_ns,
                   int32_t *versions, int32_t *nout);
/* Applies an update batch (ddp_dyn_update flags): the master graph changes
 * and is published as the next version once its ring buffer is free;
 * searches already running keep the version they started on. */
int ddp_serve_update(ddp_server *s, int32_t n, const int32_t *flag, const int32_t *u, const int32_t *v,
                     const uint32_t *w);
/* Records each request's s..t path (at most path_cap node ids per request,
 * in host memory: max_requests x path_cap x 4 bytes).  Call before the
 * first submit. */
int ddp_serve_record_paths(ddp_server *s, int32_t path_cap);
/* Path of a polled request (over the graph version it ran on): copies up to
 * cap ids, *len = the length (0 when t is unreachable).  DDP_ERR_INVALID
 * when paths are not recorded, the request was not polled yet, or its path
 * is longer than path_cap (*len then holds the length). */
int ddp_serve_path(ddp_server *s, int64_t id, int32_t *buf, int32_t cap, int32_t *len);
/* submitted, completed, slots, kernel launches, graph version, re-runs */
int ddp_serve_stats(const ddp_server *s, int64_t *stats6);
int ddp_serve_free(ddp_server *s);

/* ---- reverse-BFS hop counts without device allocation ------------------
 * No counterpart in the reference.  For callers that cannot let a library
 * call cudaMalloc (for example a service that gives all device memory to its
 * own pool at start-up, or one that must not fail on a late allocation while
 * serving): every input and output is a device array the caller owns, and
 * the scratch this kernel needs lives in a fixed array inside the library
 * (about 8 MiB, held on every GPU that loads the library until exit).
 *   d_rev_offsets: n+1 int32, reverse CSR offsets (row v = arcs into v)
 *   d_rev_sources: int32 sources of those arcs (negative = absent arc)
 *   d_hops: n int32 out, hops from v to target, -1 when v cannot reach
 *           the target
 * n is limited to DDP_NOALLOC_MAX_NODES; larger graphs are rejected with
 * DDP_ERR_INVALID.  The first call on a device looks up the scratch address
 * (make it before any stream capture).  The call is synchronous on `stream`
 * (NULL = default stream).  All calls share the one scratch array: calls that
 * overlap on the GPU race, so serialise them. */
#define DDP_NOALLOC_MAX_NODES 1048576
int ddp_bfs_hops_noalloc(int32_t n, const int32_t *d_rev_offsets, const int32_t *d_rev_sources,
                         int32_t target, int32_t *d_hops, void *stream);

/* ---- host-side text I/O in the reference's formats --------------------- */
/* graph.txt (graph.h:93-118); *off gets n+1 entries.  Free with ddp_free. */
int ddp_io_read_graph_text(const char *path, int32_t *n, int64_t *e, int32_t **off,
                           int32_t **col, uint32_t **w);
/* Writes the reference layout (n offsets, no sentinel).  off has n+1. */
int ddp_io_write_graph_text(const char *path, int32_t n, int64_t e, const int32_t *off,
                            const int32_t *col, const uint32_t *w);
/* Hx.txt: n whitespace-separated ints (bfs_hx.cu:158-172). */
/* Binary graph file ("DDPG", version 1, n and e as int64, off[n+1], col[e],
 * w[e], little-endian): loads without parsing.  No reference counterpart. */
int ddp_io_write_graph_bin(const char *path, int32_t n, int64_t e, const int32_t *off, const int32_t *col,
                           const uint32_t *w);
int ddp_io_read_graph_bin(const char *path, int32_t *n, int64_t *e, int32_t **off, int32_t **col, uint32_t **w);
int ddp_io_read_ints_text(const char *path, int64_t max, int32_t *out, int64_t *count);
int ddp_io_write_ints_text(const char *path, int64_t n, const int32_t *vals);
/* Updates.txt (DA_dyn_cpu.cu:1295-1326): batches of "count" then count
 * lines "flag u v w".  Arrays are allocated; free with ddp_free. */
int ddp_io_read_updates_text(const char *path, int32_t *nbatches, int32_t **counts,
                             int32_t **flag, int32_t **u, int32_t **v, uint32_t **w);
int ddp_io_write_updates_text(const char *path, int32_t nbatches, const int32_t *counts,
                              const int32_t *flag, const int32_t *u, const int32_t *v,
                              const uint32_t *w);
void ddp_free(void *p);

/* ---- seeded generators (GA_star/GenerateCSR.cpp + randomGraph.py,
 *      maze/create_maze.cpp, DA_star/genDynamicGraph.cpp) --------------- */
int ddp_gen_random_chain(int32_t n, int64_t e_total, uint32_t wmin, uint32_t wmax, uint64_t seed,
                         int32_t *off, int32_t *col, uint32_t *w, int32_t *perm_out);
int ddp_gen_maze(int32_t rows, int32_t cols, uint32_t wall_permille, uint64_t seed,
                 int32_t *cell_node, int32_t *n_nodes, int64_t *n_arcs, int32_t *off, int32_t *col,
                 uint32_t *w, int32_t *xy);
int ddp_gen_updates(int32_t n, int64_t e, const int32_t *off, const int32_t *col, const uint32_t *w,
                    const int32_t *protect_next, int32_t nbatches, int32_t per_batch,
                    int32_t inserts_per_batch, uint32_t wmin, uint32_t wmax, uint64_t seed,
                    int32_t *flag, int32_t *uu, int32_t *vv, uint32_t *ww);
/* Maze with every cell a node (node = row * cols + col; a wall cell has no
 * arcs), as maze/create_maze.cpp:64-113 builds it; off has rows*cols+1
 * entries, col/w at most 4 per cell. */
int ddp_gen_grid_from_walls(int32_t rows, int32_t cols, const uint8_t *wall, int32_t *off, int32_t *col,
                            uint32_t *w, int64_t *n_arcs);
/* Obstacle-move update batches (maze/create_maze.cpp:137-251): per batch,
 * `moves` walls open and `moves` open cells (not in `protect`, nullable)
 * close; unit arcs inserted both ways between each opened cell and its open
 * neighbours, arcs deleted both ways around each closed cell; every batch
 * is consistent with ddp_dyn_update's semantics.  `wall` is updated in
 * place; counts[b] = lines of batch b; lines in flag/u/v/w (capacity cap,
 * at most 16 x moves per batch); -3 when cap is too small. */
int ddp_gen_maze_moves(int32_t rows, int32_t cols, uint8_t *wall, const uint8_t *protect, int32_t nbatches,
                       int32_t moves, uint64_t seed, int32_t *counts, int32_t *flag, int32_t *u, int32_t *v,
                       uint32_t *w, int64_t cap, int64_t *total);
/* Points uniform on [0, side)^2 (xy, 2n int32), each joined both ways to its
 * k nearest neighbours, w = max(1, round(wscale * length / spacing)) with
 * spacing = side / sqrt(n).  off has n+1 entries; col/w hold at most 2kn arcs. */
int ddp_gen_geometric(int32_t n, int32_t k, int32_t side, uint32_t wscale, uint64_t seed, int32_t threads,
                      int32_t *xy, int32_t *off, int32_t *col, uint32_t *w, int64_t *n_arcs);
int ddp_gen_pairs(int32_t n, const int32_t *off, const int32_t *col, int32_t npairs, int32_t hop_lo,
                  int32_t hop_hi, int32_t bfs_cap_level, uint64_t seed, int32_t threads, int32_t *S,
                  int32_t *T, int32_t *want_hops);

#ifdef __cplusplus
}
#endif

#endif /* DDP_GB300_H */
