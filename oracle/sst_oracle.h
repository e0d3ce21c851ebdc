/*
 * sst_oracle.h -- CPU restatement of SSTGraph's hot path, TEST INFRASTRUCTURE.
 *
 * This is the checker, not the product: only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg may load it.  The product path (the CUDA
 * library behind include/sstgraph.h) never calls into it.
 *
 * What it restates, and from where (paths inside the reference project):
 *  - graph storage semantics of SparseMatrixV<true> (binary CSR):
 *    set semantics per row, ascending map order, self-loops dropped on
 *    insert, absent removes are no-ops
 *      include/SSTGraph/SparseMatrix.hpp:556-718 (insert_batch/remove_batch)
 *      include/SSTGraph/PMA.hpp:1084-1183,1224-1363 (insert/remove)
 *      include/SSTGraph/TinySet_small.hpp:295-353 (ordered map)
 *  - common_neighbors(u, v, early_end)
 *      include/SSTGraph/SparseMatrix.hpp:61-71,
 *      include/SSTGraph/TinySet_small.hpp:357-407 (early-end merge)
 *  - touch_all_sum  include/SSTGraph/SparseMatrix.hpp:436-454
 *  - the reference batch stream rMat / hash32 / hash64
 *      include/SSTGraph/internal/rmat_util.h:29-131, internal/test.hpp:636-654
 *  - BFS / PR_S / CC / BC / TC: the algorithm library (EdgeMapVertexMap) is
 *    absent from the reference tree; the call sites fix the output contracts
 *    (internal/test.hpp:476-618).  The definitions used here are written out
 *    next to each function; their parity against the reference is UNPINNED
 *    (no golden outputs exist) and they are pinned instead against networkx
 *    and an independent numpy restatement in tests/.
 *
 * The storage part is pinned against the reference's own code compiled here
 * (oracle/_ref, see oracle/Makefile) through tests/golden/.
 */
#ifndef SST_ORACLE_H
#define SST_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sst_o_graph sst_o_graph;

/* ---- hashes and generators (bit-identical to the device generators) ---- */
uint64_t sst_o_mix64(uint64_t z);
uint64_t sst_o_draw(uint64_t seed, uint64_t i, uint64_t j);
uint64_t sst_o_ref_hash64(uint64_t u);
uint32_t sst_o_ref_hash32(uint32_t a);
/* RMAT edges first..first+count-1 of stream `seed`, 2^scale vertices,
 * quadrant probabilities a, b, c (d = rest), 32-bit fixed-point thresholds */
void sst_o_rmat(uint32_t scale, double a, double b, double c, uint64_t seed,
                uint64_t first, uint64_t count, uint32_t *pairs);
/* uniform random pairs (Erdos-Renyi G(n, m) with replacement) */
void sst_o_er(uint32_t n, uint64_t seed, uint64_t first, uint64_t count,
              uint32_t *pairs);
/* the reference's update-benchmark stream:
 * rMat<uint32_t>(nn, random_aspen().ith_rand(0), a, b, c)(i) */
void sst_o_ref_rmat_stream(uint32_t nn, double a, double b, double c,
                           uint64_t first, uint64_t count, uint32_t *pairs);

/* ---- graph ---- */
sst_o_graph *sst_o_new(uint32_t n);
/* height rows, column ids below width */
sst_o_graph *sst_o_new2(uint32_t height, uint32_t width);
void sst_o_free(sst_o_graph *g);
uint32_t sst_o_num_nodes(const sst_o_graph *g);
void sst_o_insert_batch(sst_o_graph *g, const uint32_t *pairs, uint64_t b);
void sst_o_remove_batch(sst_o_graph *g, const uint32_t *pairs, uint64_t b);
uint64_t sst_o_M(const sst_o_graph *g);
uint32_t sst_o_degree(const sst_o_graph *g, uint32_t v);
int sst_o_has(const sst_o_graph *g, uint32_t r, uint32_t c);
void sst_o_degrees(const sst_o_graph *g, uint32_t *out);
void sst_o_to_csr(const sst_o_graph *g, uint64_t *offsets, uint32_t *cols);
uint64_t sst_o_common_neighbors(const sst_o_graph *g, uint32_t a, uint32_t b,
                                int early_end);
uint64_t sst_o_touch_all_sum(const sst_o_graph *g);
/* edges of rank floor(draw(seed, first+i, 0) * M / 2^64) in (row, col)
 * order: uniform samples of existing edges */
void sst_o_sample_edges(const sst_o_graph *g, uint64_t seed, uint64_t first,
                        uint64_t count, uint32_t *pairs);

/* ---- algorithms ---- */
void sst_o_bfs(const sst_o_graph *g, uint32_t src, int32_t *depth);
void sst_o_pagerank(const sst_o_graph *g, uint32_t iters, double damping,
                    double *rank);
void sst_o_cc(const sst_o_graph *g, uint32_t *label);
void sst_o_bc(const sst_o_graph *g, uint32_t src, double *dep);
uint64_t sst_o_tc(const sst_o_graph *g, uint64_t *per_vertex);

#ifdef __cplusplus
}
#endif
#endif
