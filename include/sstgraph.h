/*
 * sstgraph.h -- C ABI of the GB300 dynamic-graph library (libsstgraph_gb300.so).
 *
 * One handle = one graph resident in one GPU's HBM: per-vertex sorted uint32
 * neighbour sets kept as packed memory arrays, updated by batches and
 * traversed by device kernels.  The reference's graph type on this path is
 * SSTGraph::SparseMatrixV<true> (binary CSR, el_t = uint32_t), a header-only
 * C++ template with no ABI; each entry point below names the reference
 * member or call site it stands in for (paths inside the reference project).
 *
 * Conventions
 *  - Every call returns an sst_status (0 = SST_OK, negative = error).  On
 *    error, sst_last_error_message() describes it.
 *  - `pairs` arrays are interleaved (row, col) uint32 pairs, n pairs long.
 *  - Pointer arguments are host memory unless SST_DEVICE_PTR is set in
 *    `flags`, in which case all array arguments of that call are device
 *    memory of the graph's GPU.  Calls on host memory return after the work
 *    and the copies are done; calls on device memory are ordered on the
 *    graph's stream (sst_set_stream) and may return before the GPU finishes.
 *  - The library never writes the caller's input arrays (the reference's
 *    insert_batch/remove_batch sort the caller's buffer in place,
 *    SparseMatrix.hpp:578,664; here the sort happens in device scratch).
 *  - There is no CPU fallback: without a usable GPU the calls return
 *    SST_EDEVICE.
 *  - One writer at a time per handle; calls on one handle are not
 *    thread-safe (the reference has no locks either, SparseMatrix.hpp).
 */
#ifndef SSTGRAPH_H
#define SSTGRAPH_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* symbols the shared library exports */
#if defined(__GNUC__)
#define SST_API __attribute__((visibility("default")))
#else
#define SST_API
#endif

typedef int32_t sst_status;
#define SST_OK 0
#define SST_EINVAL (-1)    /* bad argument (null handle, id out of range) */
#define SST_ENOMEM (-2)    /* device allocation failed */
#define SST_EBUDGET (-3)   /* the operation would exceed the HBM budget */
#define SST_ETIMEDOUT (-4) /* a bounded device wait ran out */
#define SST_EDEVICE (-5)   /* CUDA error or no usable device */
#define SST_ESTATE (-6)    /* call not valid in the handle's state */

#define SST_HOST_PTR 0u
#define SST_DEVICE_PTR 1u
/* accepted for source compatibility with the reference's semi_sorted
 * argument (SparseMatrix.hpp:167-168); the device always sorts */
#define SST_SEMI_SORTED 2u

typedef struct sst_graph sst_graph;

typedef struct sst_config {
  int device;                  /* CUDA device ordinal (default 0) */
  uint64_t hbm_budget_bytes;   /* 0 = no budget */
  uint64_t initial_slots;      /* slab slots to reserve up front (0 = auto) */
  float upper_root;            /* PMA root upper density (0 = default .85) */
  float lower_root;            /* PMA root lower density (0 = default .20) */
  float grow_fill;             /* density after a resize (0 = default .70) */
  uint32_t keep_self_loops;    /* 1 = insert (v, v) as well: rows are plain
                                  sets (the TinySet facade); 0 = skip them as
                                  SparseMatrix.hpp:570,602 does */
  uint32_t weighted;           /* 1 = every edge carries a uint32 value
                                  (SparseMatrixV<true, uint32_t>) */
} sst_config;

/* ---- lifetime ------------------------------------------------------- */
/* SparseMatrixV(el_t height, el_t width)  SparseMatrix.hpp:73-87
 * rows = height (CSR lines), cols = width; cfg may be NULL */
SST_API sst_status sst_graph_create(uint32_t height, uint32_t width,
                            const sst_config *cfg, sst_graph **out);
/* ~SparseMatrixV  SparseMatrix.hpp:141-146 */
SST_API sst_status sst_graph_destroy(sst_graph *g);
/* copy constructor SparseMatrixV(const SparseMatrixV&)  SparseMatrix.hpp:88-96
 * (deep copy on the device) */
SST_API sst_status sst_graph_clone(const sst_graph *g, sst_graph **out);
/* order the graph's work on a caller stream (a cudaStream_t); NULL = the
 * library's own stream */
SST_API sst_status sst_set_stream(sst_graph *g, void *stream);
SST_API sst_status sst_sync(sst_graph *g);
/* Launch mode of update batches (no reference counterpart).  1 (default):
 * the planning launches of a raw-pair, unweighted batch of up to 2^20 pairs
 * (key sort to plan readback) are captured once per batch size and graph
 * layout and replayed as one CUDA graph launch; 0: every kernel is launched
 * directly; 2: the launches a replay would run (same size classes, same
 * kernel forms) are launched directly, so a profiler can time each of them.
 * Results are the same in every mode. */
SST_API sst_status sst_set_plan_graphs(sst_graph *g, int enable);
SST_API const char *sst_last_error_message(void);
SST_API const char *sst_status_string(sst_status s);

/* ---- updates -------------------------------------------------------- */
/* insert_batch(tuple<el_t,el_t>*, uint64_t, bool)  SparseMatrix.hpp:556-643
 * set union per row; self-loops are skipped (:570,602); pairs with an id
 * out of range are skipped and reported through *n_invalid (may be NULL) */
SST_API sst_status sst_insert_batch(sst_graph *g, const uint32_t *pairs, uint64_t n,
                            uint32_t flags, uint64_t *n_invalid);
/* remove_batch  SparseMatrix.hpp:645-718; absent edges are no-ops */
SST_API sst_status sst_remove_batch(sst_graph *g, const uint32_t *pairs, uint64_t n,
                            uint32_t flags, uint64_t *n_invalid);
/* Batched form of insert_batch / remove_batch: nbatches batches, batch i
 * being pairs[offsets[i] .. offsets[i+1]) (offsets has nbatches+1 entries,
 * offsets[0] = 0) with ops[i] = 1 to insert, 0 to remove.  The graph ends as
 * if the batches ran one after another; they run as one pipeline pass (the
 * last operation on each edge decides). */
SST_API sst_status sst_update_batches(sst_graph *g, const uint32_t *pairs,
                                      const uint64_t *offsets,
                                      const uint8_t *ops, uint32_t nbatches,
                                      uint32_t flags, uint64_t *n_invalid);
/* Weighted graphs (sst_config.weighted = 1; SparseMatrixV<true, uint32_t>,
 * internal/test.hpp:699-846): insert_batch with one value per pair.  An edge
 * already present takes the new value, and of several equal pairs in one
 * batch the last value given wins (the reference's insert updates the value
 * of a present key, PMA.hpp:1137-1145).  Plain sst_insert_batch on a
 * weighted graph gives value 1.  The batched form, relabelling and building
 * from a CSR take unweighted graphs only (SST_ESTATE). */
SST_API sst_status sst_insert_batch_weighted(sst_graph *g, const uint32_t *pairs,
                                             const uint32_t *values, uint64_t n,
                                             uint32_t flags, uint64_t *n_invalid);
/* value(el_t, el_t)  SparseMatrix.hpp:727: values[i] of pair i (0 where
 * absent); found may be NULL */
SST_API sst_status sst_values_batch(sst_graph *g, const uint32_t *pairs, uint64_t n,
                                   uint32_t *values, uint8_t *found, uint32_t flags);
/* the whole weighted graph as a CSR with its values */
SST_API sst_status sst_to_csr_values(sst_graph *g, uint64_t *offsets, uint32_t *cols,
                                     uint32_t *values, uint32_t flags);
/* insert(el_t, el_t) / remove(el_t, el_t)  SparseMatrix.hpp:164-166 */
SST_API sst_status sst_insert(sst_graph *g, uint32_t row, uint32_t col);
SST_API sst_status sst_remove(sst_graph *g, uint32_t row, uint32_t col);
/* rebuild from a CSR whose rows are sorted and duplicate-free
 * (the reference loads files then inserts in batches, internal/test.hpp:427-450) */
SST_API sst_status sst_build_from_csr(sst_graph *g, const uint64_t *offsets,
                              const uint32_t *cols, uint32_t flags);

/* ---- graph files (the reference drivers' readers,
 *      internal/helpers.hpp:379-657) -------------------------------------
 * .mtx (Matrix Market coordinate, one-based, every entry symmetrised in file
 * order, values ignored, rows must equal cols) and PBBS .adj / .adj.shuf
 * (AdjacencyGraph / WeightedAdjacencyGraph, weights ignored).  Host only:
 * sst_read_graph_file returns the (row, col) pairs in *pairs (free with
 * sst_free); sst_load_graph_file builds a rows x rows graph from them with
 * one batch insert, as the reference's drivers do (internal/test.hpp:427-450). */
SST_API sst_status sst_read_graph_file(const char *path, uint32_t *rows,
                                       uint64_t *n_pairs, uint32_t **pairs);
SST_API void sst_free(void *p);
SST_API sst_status sst_load_graph_file(const char *path, const sst_config *cfg,
                                       sst_graph **out);

/* ---- queries -------------------------------------------------------- */
/* has(el_t, el_t)  SparseMatrix.hpp:162,721-727 ; out[i] = 0/1 */
SST_API sst_status sst_has_batch(sst_graph *g, const uint32_t *pairs, uint64_t n,
                         uint8_t *out, uint32_t flags);
SST_API sst_status sst_has(sst_graph *g, uint32_t row, uint32_t col, int *out);
/* num_nodes / get_rows / get_cols  SparseMatrix.hpp:56,150-161 */
SST_API sst_status sst_num_nodes(const sst_graph *g, uint64_t *out);
SST_API sst_status sst_get_rows(const sst_graph *g, uint32_t *out);
SST_API sst_status sst_get_cols(const sst_graph *g, uint32_t *out);
/* M()  SparseMatrix.hpp:518-525 */
SST_API sst_status sst_M(sst_graph *g, uint64_t *out);
/* getDegree  SparseMatrix.hpp:57-59 (all rows, or one) */
SST_API sst_status sst_degrees(sst_graph *g, uint32_t *out, uint32_t flags);
SST_API sst_status sst_get_degree(sst_graph *g, uint32_t v, uint32_t *out);
/* map_neighbors copy-out  SparseMatrix.hpp:218-253: the neighbours of v in
 * ascending order; writes min(deg, cap) ids, *deg = full degree */
SST_API sst_status sst_neighbors(sst_graph *g, uint32_t v, uint32_t *out,
                         uint64_t cap, uint64_t *deg);
/* map_range over all rows  SparseMatrix.hpp:255-315: the whole graph as a
 * CSR (offsets[rows+1], cols[M]) */
SST_API sst_status sst_to_csr(sst_graph *g, uint64_t *offsets, uint32_t *cols,
                      uint32_t flags);
/* common_neighbors(u, v, early_end)  SparseMatrix.hpp:61-71, per pair */
SST_API sst_status sst_common_neighbors_batch(sst_graph *g, const uint32_t *pairs,
                                      uint64_t n, int early_end,
                                      uint64_t *out, uint32_t flags);
/* touch_all_sum  SparseMatrix.hpp:436-454 */
SST_API sst_status sst_touch_all_sum(sst_graph *g, uint64_t *out);
/* get_memory_size  SparseMatrix.hpp:317,528-535: device bytes held (the
 * storage, plus the scratch the graph keeps between calls) */
SST_API sst_status sst_memory_size(sst_graph *g, uint64_t *out);
/* Frees the scratch a graph keeps between calls (no reference counterpart:
 * the reference allocates per call): update-batch scratch, staging, the
 * captured planning graphs, the leaf directory and the traversal buffers.
 * The next call that needs them allocates them again; tuning is kept.
 * Useful after a bulk load, whose large batches grow the scratch. */
SST_API sst_status sst_release_scratch(sst_graph *g);
/* degree_order_map()  SparseMatrix.hpp:737-752: map[v] = rank of v when the
 * vertices are ordered by (degree, id) descending */
SST_API sst_status sst_degree_order_map(sst_graph *g, uint32_t *map,
                                        uint32_t flags);
/* rewrite_graph(new_label_map)  SparseMatrix.hpp:754-766: a new graph (same
 * shape, same configuration) holding every edge (u, v) as (map[u], map[v]);
 * rows must equal columns */
SST_API sst_status sst_rewrite_graph(sst_graph *g, const uint32_t *map,
                                     uint32_t flags, sst_graph **out);
/* uniform samples of existing edges: edge of rank
 * floor(draw(seed, first+i) * M / 2^64) in (row, col) order */
SST_API sst_status sst_sample_edges(sst_graph *g, uint64_t seed, uint64_t first,
                            uint64_t count, uint32_t *pairs, uint32_t flags);

/* ---- traversal (EdgeMap/VertexMap algorithms; the algorithm library
 *      EdgeMapVertexMap is absent from the reference tree, so the entry
 *      points follow its call sites in internal/test.hpp:476-618) -------
 * The graph must be symmetric (every (u,v) stored with (v,u)), as the
 * reference drivers build it from symmetrised inputs: the pull (dense
 * frontier) steps and PageRank read a vertex's stored row as its in-edges.
 * On a directed graph the results are not defined.  Every traversal entry
 * point below (and the serving loop, and the snapshot's PageRank) needs as
 * many rows as columns and returns SST_EINVAL otherwise: column ids index
 * per-vertex arrays of `rows` entries. */
/* BFS(g, src)  test.hpp:486: parents (parent[src] = src, -1 unreached)
 * and/or depths (-1 unreached); either pointer may be NULL */
SST_API sst_status sst_bfs(sst_graph *g, uint32_t src, int32_t *parents,
                   int32_t *depths, uint32_t flags);
/* PR_S<double>(g, iters)  test.hpp:527 */
SST_API sst_status sst_pagerank(sst_graph *g, uint32_t iters, double damping,
                        double *out, uint32_t flags);
/* PageRank that allocates nothing during the call (no counterpart in the
 * reference).  For callers that cannot let a call allocate: a serving loop
 * under a fixed HBM budget, or a host program sharing the GPU whose other
 * streams would stall on the device-wide synchronisation of cudaMalloc /
 * cudaFree.  Matches sst_pagerank within 1e-9 relative (it sums FP64
 * values in warp order, not sst_pagerank's exact fixed-point sums); its
 * scratch is one fixed array inside the library, so graphs are limited to
 * 262,144 rows (larger ones, and graphs with more columns than rows, get
 * SST_EINVAL) and d_rank must be device memory.  The first call on a device
 * looks the array up (make it before capturing a stream); calls that overlap
 * on the GPU share the array and race. */
SST_API sst_status sst_pagerank_noalloc(sst_graph *g, uint32_t iters,
                                        double damping, double *d_rank);
/* CC(g)  test.hpp:571: label = smallest vertex id of the component */
SST_API sst_status sst_cc(sst_graph *g, uint32_t *labels, uint32_t flags);
/* BC(g, src)  test.hpp:547: single-source dependency scores */
SST_API sst_status sst_bc(sst_graph *g, uint32_t src, double *out, uint32_t flags);
/* TC(g)  test.hpp:606: triangles (each once); per_vertex may be NULL */
SST_API sst_status sst_tc(sst_graph *g, uint64_t *total, uint64_t *per_vertex,
                  uint32_t flags);
/* Multi-source forms (no reference counterpart; the batched traversal of
 * k <= 64 sources).  Output is k x rows, row i for srcs[i]:
 * sst_bfs_multi writes depths (-1 unreached), one traversal for all
 * sources; sst_bc_multi writes for each source exactly what sst_bc writes
 * (same arithmetic order), every launch covering all sources. */
SST_API sst_status sst_bfs_multi(sst_graph *g, const uint32_t *srcs, uint32_t k,
                                 int32_t *depths, uint32_t flags);
SST_API sst_status sst_bc_multi(sst_graph *g, const uint32_t *srcs, uint32_t k,
                                double *out, uint32_t flags);
/* Traversal tuning (no reference counterpart).  sst_autotune times the
 * knobs on this graph and keeps the fastest: PageRank over chunk_leaves
 * {8,16,32} x pr_lanes {4,8,16}, then pr_hot {0,2048,4096,8192,16384,24576}, then BFS
 * over bfs_alpha {5,10,20,40,80};
 * pr_ms / bfs_ms report the winners' times (3 PageRank iterations; one BFS).
 * The leaf itself stays 32 slots (one 128-byte line): it is the storage
 * format, not a launch parameter. */
typedef struct sst_tuning {
  uint32_t chunk_leaves; /* leaves per warp work item of the pull lists (1..32) */
  uint32_t pr_lanes;     /* lanes per one-leaf vertex in PageRank (4, 8, 16) */
  uint32_t bfs_alpha;    /* BFS pulls once (frontier + its edges) * alpha > m */
  float pr_ms, bfs_ms;
  uint32_t pr_hot;       /* PageRank: contributions of ids below this staged in
                            shared memory (0..24576; pays on degree-ordered
                            graphs, sst_degree_order_map) */
} sst_tuning;
SST_API sst_status sst_autotune(sst_graph *g, sst_tuning *out);
SST_API sst_status sst_get_tuning(sst_graph *g, sst_tuning *out);
SST_API sst_status sst_set_tuning(sst_graph *g, const sst_tuning *in);
/* BF(g, src)  test.hpp:611-634: shortest-path lengths over the edge values
 * of a weighted graph (push Bellman-Ford); unreachable = INT32_MAX, lengths
 * at or above 2^31-1 saturate there.  Directed: rows are out-edges. */
SST_API sst_status sst_bf(sst_graph *g, uint32_t src, int32_t *dist, uint32_t flags);
/* TouchAll(g)  test.hpp:476 */
SST_API sst_status sst_touch_all(sst_graph *g, uint64_t *out);

/* per-vertex triangle counts of listed vertices: out[i] = triangles that
 * contain vertices[i] (the serving loop's per-vertex TC query) */
SST_API sst_status sst_tc_vertices(sst_graph *g, const uint32_t *vertices,
                                   uint64_t k, uint64_t *out, uint32_t flags);

/* ---- byte-width snapshot: the device form of TinySetV_small's rows
 *      (TinySet_small.hpp:204-293,852-881).  Each row keeps the low B bytes
 *      of its ids (B = 4, 3, 2, 1 by the row's length, with the reference's
 *      thresholds), bucketed by the high part; read-only, built from a
 *      graph's current contents, independent of it afterwards. ---------- */
typedef struct sst_compact sst_compact;
/* get_thresholds(max_el)  TinySet_small.hpp:227-263: rows with fewer than
 * t[0] ids keep 4-byte keys, fewer than t[1] 3-byte, fewer than t[2]
 * 2-byte, the rest 1-byte (host only, no device needed) */
SST_API sst_status sst_compact_widths(uint64_t max_el, uint32_t thresholds[3]);
/* snapshot of g (unweighted graphs; weighted ones get SST_ESTATE) */
SST_API sst_status sst_compact_create(sst_graph *g, sst_compact **out);
SST_API sst_status sst_compact_destroy(sst_compact *c);
/* storage_bytes: the rows and their index; device_bytes: everything the
 * snapshot holds (with PageRank work lists and buffers); rows_per_width[i]:
 * rows stored with (i + 1)-byte keys.  Any pointer may be NULL. */
SST_API sst_status sst_compact_info(sst_compact *c, uint64_t *storage_bytes,
                                    uint64_t *device_bytes, uint64_t *edges,
                                    uint64_t rows_per_width[4]);
/* the snapshot decoded as a CSR (offsets[rows+1], cols[M]) */
SST_API sst_status sst_compact_to_csr(sst_compact *c, uint64_t *offsets,
                                      uint32_t *cols, uint32_t flags);
/* has(row, col) per pair, out[i] = 0/1 */
SST_API sst_status sst_compact_has_batch(sst_compact *c, const uint32_t *pairs,
                                         uint64_t n, uint8_t *out, uint32_t flags);
/* PR_S<double>  test.hpp:527 on the snapshot: the same result, bit for bit,
 * as sst_pagerank on the graph it was taken from */
SST_API sst_status sst_compact_pagerank(sst_compact *c, uint32_t iters,
                                        double damping, double *out,
                                        uint32_t flags);
/* BFS(g, src)  test.hpp:486 on the snapshot: depths (-1 unreached), equal
 * to sst_bfs's on the graph it was taken from; the same push / pull switch */
SST_API sst_status sst_compact_bfs(sst_compact *c, uint32_t src, int32_t *depths,
                                   uint32_t flags);
/* CC(g)  test.hpp:571 on the snapshot: each label the component's smallest
 * vertex id, equal to sst_cc's */
SST_API sst_status sst_compact_cc(sst_compact *c, uint32_t *labels, uint32_t flags);
/* BC(g, src)  test.hpp:547 on the snapshot: single-source dependency scores,
 * within 1e-9 relative of sst_bc's (FP64 sums in another order); the rows
 * are decoded into temporary device memory */
SST_API sst_status sst_compact_bc(sst_compact *c, uint32_t src, double *out,
                                  uint32_t flags);
/* TC(g)  test.hpp:606 on the snapshot: triangles (each once), equal to
 * sst_tc's; per_vertex may be NULL (the snapshot's rows are decoded and
 * oriented into temporary device memory) */
SST_API sst_status sst_compact_tc(sst_compact *c, uint64_t *total, uint64_t *per_vertex,
                                  uint32_t flags);
/* the stream the snapshot's work runs on (NULL: its own), as sst_set_stream */
SST_API sst_status sst_compact_set_stream(sst_compact *c, void *stream);
SST_API sst_status sst_compact_sync(sst_compact *c);

/* ---- serving loop (no reference counterpart: the reference has no
 *      request loop; this keeps the graph on the device and serves a mixed
 *      stream) --------------------------------------------------------- */
typedef struct sst_server sst_server;
typedef struct sst_server_config {
  uint32_t query_slots;      /* concurrent queries, each on its own snapshot */
  uint64_t hbm_budget_bytes; /* live graph + slots must fit (0 = no budget) */
  uint32_t max_coalesce;     /* update requests fused per pass (0 = all) */
} sst_server_config;

#define SST_REQ_INSERT 1       /* pairs[n] inserted */
#define SST_REQ_REMOVE 2       /* pairs[n] removed */
#define SST_REQ_BFS 3          /* out: int32 depths[rows] from src */
#define SST_REQ_PAGERANK 4     /* out: double ranks[rows], iters, damping */
#define SST_REQ_TC_VERTICES 5  /* pairs = n vertex ids, out: uint64 [n] */

typedef struct sst_request {
  int32_t kind;
  const uint32_t *pairs; /* update pairs or query vertices (host; copied) */
  uint64_t n;
  uint32_t src;
  uint32_t iters;
  double damping;
  void *out; /* host output of a query (written before completion) */
} sst_request;

typedef struct sst_request_info {
  sst_status status;
  uint64_t epoch;  /* update requests applied before the query's snapshot,
                      or after the update's pass */
  double queue_ms, run_ms, total_ms;
} sst_request_info;

/* one writer applies all pending updates per pass as a batched pass; query
 * slots (as many as query_slots and the HBM budget allow) run queries on
 * snapshots refreshed between passes, overlapping the writer on the GPU */
SST_API sst_status sst_server_create(sst_graph *g, const sst_server_config *cfg,
                                     sst_server **out);
SST_API sst_status sst_server_slots(sst_server *s, uint32_t *slots);
SST_API sst_status sst_server_submit(sst_server *s, const sst_request *req,
                                     uint64_t *ticket);
/* waits for a request; returns its status and fills info */
SST_API sst_status sst_server_wait(sst_server *s, uint64_t ticket,
                                   uint32_t timeout_ms, sst_request_info *info);
SST_API sst_status sst_server_stats(sst_server *s, uint64_t *epoch,
                                    uint64_t *passes, uint64_t *update_edges);
/* finishes queued requests, then stops the threads and frees the slots */
SST_API sst_status sst_server_destroy(sst_server *s);

/* ---- generators (device; same streams as the CPU oracle) ------------ */
/* RMAT edges first..first+count-1 of stream `seed`, 2^scale vertices */
SST_API sst_status sst_gen_rmat(uint32_t scale, double a, double b, double c,
                        uint64_t seed, uint64_t first, uint64_t count,
                        uint32_t *pairs, uint32_t flags);
/* uniform pairs over n vertices */
SST_API sst_status sst_gen_er(uint32_t n, uint64_t seed, uint64_t first,
                      uint64_t count, uint32_t *pairs, uint32_t flags);
/* the reference update-benchmark stream rMat<uint32_t>(nn, hash64(0), a, b, c)
 * internal/rmat_util.h:82-131, internal/test.hpp:645-654 */
SST_API sst_status sst_gen_ref_rmat(uint32_t nn, double a, double b, double c,
                            uint64_t first, uint64_t count, uint32_t *pairs,
                            uint32_t flags);

/* ---- instrumentation -------------------------------------------------- */
/* kernel profiler (the reference times whole calls with gettimeofday,
 * internal/helpers.hpp:239-243): between start and collect every kernel
 * launch is bracketed by CUDA events on its stream; collect writes a JSON
 * object {"kernel": {"launches": L, "ms": T}, ...} into buf (NUL-terminated,
 * truncated to cap) and stops profiling.  kernel_filter (may be NULL)
 * limits the events to kernels whose name contains it. */
SST_API sst_status sst_profile_start(const char *kernel_filter);
SST_API sst_status sst_profile_collect(char *buf, uint64_t cap);
/* raw device layout for structural checks (no reference counterpart):
 * vertex table (base[rows], cap[rows], deg[rows]) and, when slots / lcnt are
 * non-NULL, the first *nslots slab slots and their leaf counts
 * (*nslots / 32 bytes).  *nslots returns the slab's used extent. */
SST_API sst_status sst_raw_state(sst_graph *g, uint64_t *base, uint32_t *cap,
                                 uint32_t *deg, uint32_t *slots, uint8_t *lcnt,
                                 uint64_t *nslots);
/* number of kernel launches this library issued since load */
SST_API uint64_t sst_kernel_launches(void);
/* Diagnostic (no reference counterpart): how many times a tile of the
 * single-pass scans (update batches, launched directly) polls a
 * predecessor's status before it stops waiting and reduces the
 * predecessors' inputs itself.  Default 8192; 0 makes every tile after the
 * first take that fallback.  Results are the same for every value; the
 * setting is process-wide and returns the previous value in *old (may be
 * NULL). */
SST_API sst_status sst_set_scan_lookback_polls(uint32_t polls, uint32_t *old);

#ifdef __cplusplus
}
#endif
#endif /* SSTGRAPH_H */
