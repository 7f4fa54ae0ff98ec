/*
 * gst_gen.h — seeded synthetic instances for the GST solver (host only).
 *
 * Graphs and groups are produced with a project-written xoshiro256** stream
 * seeded through splitmix64, so a (generator, parameters, seed) triple gives
 * the same instance on every platform (no std:: distributions involved).
 * Graphs come back as undirected CSR (each edge in both rows, rows sorted by
 * neighbour ID, as graph_v_of_v_idealID keeps them); groups as a
 * (group_ptr, members) pair.
 */
#ifndef GST_GEN_H_
#define GST_GEN_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gst_host_graph gst_host_graph;
typedef struct gst_host_groups gst_host_groups;

/* Connected random graph with the structure of the reference's generator
 * (graph_hash_of_mixed_weighted_generate_random_connected_graph.h:43-107):
 * a random recursive spanning tree (vertex i joins a uniform earlier
 * vertex), then uniform extra edges until E undirected edges, no duplicates
 * or self loops; integer weights uniform in [wmin, wmax]. NULL on bad
 * parameters (E < V-1 or E > V(V-1)/2). No counterpart entry point in the
 * reference (its generator is seeded from time(0)). */
gst_host_graph *gst_gen_random_connected(int32_t V, int64_t E, int32_t wmin, int32_t wmax, uint64_t seed);

/* Barabasi-Albert preferential attachment: a clique on m+1 vertices, then
 * each new vertex attaches to m distinct earlier vertices chosen with
 * probability proportional to degree; weights uniform in [wmin, wmax]. */
gst_host_graph *gst_gen_barabasi_albert(int32_t V, int32_t m, int32_t wmin, int32_t wmax, uint64_t seed);

int32_t gst_host_graph_num_vertices(const gst_host_graph *g);
int64_t gst_host_graph_num_entries(const gst_host_graph *g);
/* Copies out row_ptr[V+1], col[nnz], w[nnz]. */
void gst_host_graph_copy(const gst_host_graph *g, int32_t *row_ptr, int32_t *col, int32_t *w);
void gst_host_graph_free(gst_host_graph *g);

/* k groups of `size` distinct vertices drawn uniformly
 * (graph_hash_of_mixed_weighted_generate_random_groups_of_vertices.h:5-52,
 * with size_min = size_max = size). */
gst_host_groups *gst_gen_groups_uniform(int32_t V, int32_t k, int32_t size, uint64_t seed);

/* k groups whose sizes follow Zipf(s) on {1,2,...} clipped to
 * [size_min, size_max]; members are distinct within a group and drawn with
 * probability proportional to degree in the CSR graph (row_ptr, col). */
gst_host_groups *gst_gen_groups_zipf_degree(const int32_t *row_ptr, const int32_t *col, int32_t V, int64_t nnz,
                                            int32_t k, double s, int32_t size_min, int32_t size_max,
                                            uint64_t seed);

int32_t gst_host_groups_k(const gst_host_groups *q);
int64_t gst_host_groups_num_members(const gst_host_groups *q);
/* Copies out group_ptr[k+1] and members[num_members]. */
void gst_host_groups_copy(const gst_host_groups *q, int32_t *group_ptr, int32_t *members);
void gst_host_groups_free(gst_host_groups *q);

#ifdef __cplusplus
}
#endif
#endif /* GST_GEN_H_ */
