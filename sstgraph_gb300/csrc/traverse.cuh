// EdgeMap/VertexMap traversal over the device PMA: BFS, PageRank, CC, BC,
// TC and pairwise common-neighbour counts.  Output pointers are device
// memory of the graph's GPU.
#pragma once
#include "graph.cuh"

namespace sst {

sst_status bfs(sst_graph *g, uint32_t src, int32_t *d_parents,
               int32_t *d_depths);
sst_status pagerank(sst_graph *g, uint32_t iters, double damping,
                    double *d_rank);
sst_status cc(sst_graph *g, uint32_t *d_labels);
sst_status bc(sst_graph *g, uint32_t src, double *d_dep);
// k <= 64 sources (host array) in one traversal; d_depth is k x n
// (row per source, -1 unreached)
sst_status bfs_multi(sst_graph *g, const uint32_t *h_srcs, uint32_t k,
                     int32_t *d_depth);
// single-source BC of each of k <= 64 sources, all sources per launch;
// d_dep is k x n, row s equal to bc(g, srcs[s])
sst_status bc_multi(sst_graph *g, const uint32_t *h_srcs, uint32_t k,
                    double *d_dep);
sst_status tc(sst_graph *g, uint64_t *total, uint64_t *d_per_vertex);
// shortest-path lengths from src over edge values (weighted graphs);
// unreachable and lengths >= 2^31-1 read INT32_MAX
sst_status bellman_ford(sst_graph *g, uint32_t src, int32_t *d_out);
sst_status get_tuning(sst_graph *g, sst_tuning *out);
sst_status set_tuning(sst_graph *g, const sst_tuning *in);
sst_status autotune(sst_graph *g, sst_tuning *out);
sst_status tc_vertices(sst_graph *g, const uint32_t *d_vs, uint64_t k,
                       uint64_t *d_out);
sst_status graph_copy_into(sst_graph *dst, sst_graph *src);
sst_status common_neighbors_batch(sst_graph *g, const uint32_t *d_pairs,
                                  uint64_t n, bool early_end,
                                  uint64_t *d_out);

}  // namespace sst
