/*
 * gst.h — C ABI of the GB300 exact group Steiner tree (GST) solver.
 *
 * One call solves one query exactly with the DPBF dynamic program: a graph
 * (integer-weighted, undirected, in CSR form) and k vertex groups go in; a
 * minimum-cost tree touching every group and its cost come out.
 *
 * The functions replace the reference's single-GPU entry point
 *   graph_hash_of_mixed_weighted DPBF_GPU(node **host_tree, node *host_tree_one_d,
 *       CSR_graph &graph, std::unordered_set<int> &cumpulsory_group_vertices,
 *       graph_v_of_v_idealID &group_graph, graph_v_of_v_idealID &input_graph,
 *       int *pointer1, int *real_cost, int *community, int *c_size,
 *       non_overlapped_group_sets s, double *rt)
 * declared at rucgraph/DPQ.cuh:57 and defined at src/DPQ.cu:501-768, and the
 * CSR upload of toCSR (rucgraph/graph_v_of_v_idealID/csr_graph.hpp:29-65).
 * Plain pointers and sizes only; every call returns a gst_status and never
 * exits the process (the reference prints and returns an empty tree, or
 * calls exit(), where these return GST_INFEASIBLE / GST_BAD_INPUT).
 *
 * Threading: calls on one gst_graph are serialised internally (the graph
 * owns one device workspace); distinct graphs may be used from distinct
 * threads. All device work runs on the device that was current when the
 * graph was uploaded, on a stream the graph owns; every call returns only
 * after its device work finished (synchronous, like DPBF_GPU).
 */
#ifndef GST_H_
#define GST_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum gst_status {
  GST_OK = 0,
  GST_INFEASIBLE = 1, /* no tree covers every group (reference: src/DPQ.cu:620-624) */
  GST_BAD_INPUT = 2,  /* malformed CSR, group list, k out of range, negative weight */
  GST_OOM = 3,        /* a device or host allocation failed */
  GST_TIMEOUT = 4,    /* a convergence loop hit gst_opts.max_rounds */
  GST_CUDA_ERROR = 5, /* a CUDA runtime call failed; see gst_last_error() */
  GST_OVERFLOW = 6,   /* a tree cost reached GST_COST_LIMIT (int32 headroom) */
  GST_INTERNAL = 7,   /* an internal consistency check failed */
  GST_TOO_LARGE = 8   /* input beyond the fixed capacity of gst_group_distances_noalloc */
} gst_status;

/* Largest number of groups per query (the state table is V x 2^k). */
#define GST_MAX_K 16
/* Every tree cost must stay below this; larger sums report GST_OVERFLOW. */
#define GST_COST_LIMIT 1073741823

typedef struct gst_graph gst_graph;
typedef struct gst_result gst_result;

/* Solve options. Zero-initialise, set struct_size = sizeof(gst_opts), then
 * change what you need; a NULL pointer means all defaults. */
typedef struct gst_opts {
  int32_t struct_size;
  /* Upper bound on the optimal cost known to the caller (the cost of any
   * feasible tree); states whose cost plus the one-label lower bound
   * exceeds it are pruned. <= 0: no bound. A bound below the true optimum
   * makes the solve return GST_INFEASIBLE. */
  int32_t upper_bound;
  /* Cap on growth rounds per DP wave; 0 = V + 1 (always enough). */
  int32_t max_rounds;
  /* 1 = drive the DP through a captured CUDA graph (one launch per query);
   * 0 = launch kernels from the host loop. Both give identical results. */
  int32_t use_graph;
  /* 1 = fill the per-kernel statistics returned by gst_result_stats. */
  int32_t collect_stats;
  /* A growth round runs dense (every vertex, every neighbour row, no
   * candidate marks) when the previous round changed more than
   * V >> dense_shift vertices; 0 = the default (1; 2 when the solve prunes
   * with upper_bound or refine_bound, or the value gst_autotune chose for
   * this k). A tuning knob only: results do not depend on it. */
  int32_t dense_shift;
  /* 1 = after every DP wave, lower the pruning bound to the cheapest
   * feasible subgraph seen so far: a state T(v,S) plus v's shortest paths
   * (wave-1 states) to the groups outside S, as PrunedDP++ updates its
   * best solution (graph_v_of_v_idealID_PrunedDPPlusPlus.h:668-711). Turns
   * pruning on from wave 2 even without an upper_bound. Exact either way. */
  int32_t refine_bound;
  /* gst_solve_batch: solve contexts run concurrently, each with its own
   * workspace and streams over the one resident graph; 0 = the tuned value
   * (gst_autotune), else 4. Capped at 8. */
  int32_t concurrency;
  /* gst_solve_batch: >= 2 = solve the batch in chunks of this many queries
   * with equal k, each chunk one launch of a CUDA graph that holds every
   * query's whole solve as a parallel branch (captured once per k and chunk
   * size, on the graph's own context and its lanes); 1 = the concurrent
   * solve contexts of `concurrency` instead; 0 = the tuned choice
   * (gst_autotune), else contexts. Capped at 8. Results never depend on it. */
  int32_t batch_graph;
  int32_t reserved[7];
} gst_opts;

/* ---------------------------------------------------------------- graph -- */

/* Copies a CSR graph to the current device and keeps it resident.
 * row_ptr[V+1] (row_ptr[0] = 0, non-decreasing, row_ptr[V] = nnz),
 * col[nnz] in [0,V), w[nnz] in [0, GST_COST_LIMIT). Undirected graphs list
 * each edge in both rows, as toCSR does; weights are the reference's int
 * truncation of its double weights (csr_graph.hpp:46). Parallel entries
 * are allowed (the lighter one wins).
 * Replaces toCSR's cudaMallocManaged + cudaMemcpy (csr_graph.hpp:55-61). */
gst_status gst_graph_upload(const int32_t *row_ptr, const int32_t *col, const int32_t *w, int32_t V,
                            int64_t nnz, gst_graph **out);

/* Frees the device copy and the workspace (csr_graph: caller frees,
 * rucgraph/test_gpu.h:281-283). NULL is ignored. */
void gst_graph_free(gst_graph *g);

int32_t gst_graph_num_vertices(const gst_graph *g);
int64_t gst_graph_num_entries(const gst_graph *g);

/* ---------------------------------------------------------------- solve -- */

/* Solves one query: group g (0 <= g < k) is members[group_ptr[g] ..
 * group_ptr[g+1]). Bit g of a group-set mask stands for group g (the
 * reference uses the iteration order of its unordered_set, DPQ.cu:22-34;
 * the optimal cost does not depend on the order).
 * On GST_OK, *out holds the optimal cost, the root vertex and the tree.
 * On GST_INFEASIBLE, *out holds an empty tree and cost -1.
 * Replaces DPBF_GPU (src/DPQ.cu:501-768). */
gst_status gst_solve(gst_graph *g, const int32_t *group_ptr, const int32_t *members, int32_t k,
                     const gst_opts *opts, gst_result **out);

/* Solves nq independent queries on one resident graph. Query q has ks[q]
 * groups; the groups of all queries are concatenated: query q owns groups
 * [b_q, b_q + ks[q]) with b_q = ks[0] + ... + ks[q-1], and group j is
 * members[group_ptr[j] .. group_ptr[j+1]). out[q] receives each query's
 * result (also for infeasible queries); the return value is the first
 * non-OK, non-INFEASIBLE status, else GST_OK. A query whose k is 0 or above
 * GST_MAX_K fails alone: its result has status GST_BAD_INPUT and the other
 * queries are solved on their own groups (b_q still counts its ks[q]); a
 * negative k rejects the whole batch (GST_BAD_INPUT, every out[q] NULL).
 * No counterpart in the reference (it runs one query per DPBF_GPU call). */
gst_status gst_solve_batch(gst_graph *g, int32_t nq, const int32_t *ks, const int32_t *group_ptr,
                           const int32_t *members, const gst_opts *opts, gst_result **out);

/* Tunes the graph for a sample of queries (laid out as for
 * gst_solve_batch): for every k present, the dense-round shift (1..4) that
 * solves its sample fastest; then the batch execution that solves the whole
 * sample fastest: concurrent solve contexts (1, 2, 4 or 8) or batch graphs
 * of 2, 4 or 8 queries. Later solves with dense_shift 0 and batches with
 * concurrency 0 and batch_graph 0 use the tuned values; *lanes_out receives
 * the tuned concurrency (or the batch graph size when that won). Results
 * never depend on tuning. No counterpart in the reference. */
gst_status gst_autotune(gst_graph *g, int32_t nq, const int32_t *ks, const int32_t *group_ptr,
                        const int32_t *members, const gst_opts *opts, int32_t *lanes_out);

/* What gst_autotune chose for a graph, as a plain record that a caller can
 * keep (for instance in a file keyed by the graph's size and the queries'
 * k) and hand to a later graph of the same shape instead of tuning again.
 * dense_shift[k]: the dense-round shift of k-group solves (0 = default,
 * else 1..4); concurrency: solve contexts of a batch (0 = default, else
 * 1..8); batch_graph: queries per batch graph (0 = contexts, else 2..8).
 * Results never depend on it. No counterpart in the reference. */
typedef struct gst_tuning {
  int32_t dense_shift[GST_MAX_K + 1];
  int32_t concurrency;
  int32_t batch_graph;
  int32_t reserved[6];
} gst_tuning;

/* Copies g's tuned values into *out. */
gst_status gst_get_tuning(const gst_graph *g, gst_tuning *out);

/* Sets g's tuned values from *t; GST_BAD_INPUT (g unchanged) when a value
 * is out of its range. */
gst_status gst_set_tuning(gst_graph *g, const gst_tuning *t);

/* ---------------------------------------------------------------- pool -- */

/* Replicas of one graph on several devices (query-level scaling: a query's
 * DP does not partition, independent queries do). gst_pool_solve_batch
 * hands chunks of queries to one host thread per replica (work stealing);
 * each replica runs them as gst_solve_batch does. A device may appear more
 * than once (two replicas on one GPU). No counterpart in the reference. */
typedef struct gst_pool gst_pool;
gst_status gst_pool_create(const int32_t *row_ptr, const int32_t *col, const int32_t *w, int32_t V, int64_t nnz,
                           const int32_t *devices, int32_t num_devices, gst_pool **out);
void gst_pool_free(gst_pool *p);
int32_t gst_pool_num_replicas(const gst_pool *p);
/* As gst_solve_batch; out[q] also records which replica solved query q
 * (gst_result_replica). */
gst_status gst_pool_solve_batch(gst_pool *p, int32_t nq, const int32_t *ks, const int32_t *group_ptr,
                                const int32_t *members, const gst_opts *opts, gst_result **out);

/* --------------------------------------------------------------- result -- */

void gst_result_free(gst_result *r);
/* Batch results: ms2[0] = the query's own solve (host wall time),
 * ms2[1] = its completion since the batch began. */
void gst_result_latency(const gst_result *r, double *ms2);
/* Pool results: index of the replica that solved the query (-1 otherwise). */
int32_t gst_result_replica(const gst_result *r);
gst_status gst_result_status(const gst_result *r);
/* Optimal cost (DPBF_GPU's *real_cost), -1 if infeasible. */
int32_t gst_result_cost(const gst_result *r);
/* Vertex whose full-mask state attains the cost (DPQ.cu:712-721). */
int32_t gst_result_root(const gst_result *r);
/* Distinct tree vertices / edges. Edges are (u, v, w) triples, u < v. */
int32_t gst_result_num_vertices(const gst_result *r);
int32_t gst_result_num_edges(const gst_result *r);
/* Copy out; buffers must hold num_vertices / 3*num_edges int32. */
void gst_result_vertices(const gst_result *r, int32_t *vertices);
void gst_result_edges(const gst_result *r, int32_t *edges);
/* DP states settled (DPBF_GPU's *pointer1 counter, DPQ.cu:675). */
int64_t gst_result_states(const gst_result *r);
/* CUDA kernels the solve launched (no counterpart in the reference). */
int64_t gst_result_launches(const gst_result *r);
/* Device milliseconds: [0] whole solve, [1] growth rounds (DPBF_GPU's *rt,
 * DPQ.cu:707-709), [2] merges, [3] argmin + backtrack. [1]-[3] are measured
 * by the host-launched driver and, with the CUDA-graph driver, when
 * collect_stats is set (a graph with per-wave event nodes); 0 otherwise. */
void gst_result_times(const gst_result *r, double *ms4);
/* Statistics (filled when opts.collect_stats): [0] growth rounds launched,
 * [1] vertices scanned, [2] CSR entries scanned, [3] neighbour rows
 * gathered, [4] state entries gathered, [5] states improved, [6] merge
 * splits evaluated, [7] algorithmic bytes of the growth kernel. */
void gst_result_stats(const gst_result *r, int64_t *stats8);

/* ------------------------------------------------- allocation-free call -- */

/* Largest graph gst_group_distances_noalloc accepts. */
#define GST_NOALLOC_MAX_VERTICES (1 << 20)

/* Distance from every vertex to the nearest of `sources` (one group), for
 * callers that cannot allocate device memory: code inside a host
 * application or serving stack that owns all device memory through its own
 * pool (cudaMalloc/cudaFree would bypass its accounting), latency-critical
 * paths that cannot take cudaMalloc's implicit device synchronisation, and
 * plugins loaded after such a process has fixed its memory budget. This
 * call allocates nothing: no cudaMalloc, cudaFree, stream, event or host
 * heap memory.
 *
 * All pointers are DEVICE pointers owned by the caller: the CSR graph
 * (row_ptr[V+1], col[nnz], w[nnz], same rules as gst_graph_upload; rows
 * outside [0, nnz] and out-of-range entries give GST_BAD_INPUT),
 * sources[num_sources] (vertex IDs), and the outputs dist[V] (GST_COST_LIMIT
 * where unreachable) and pred[V] (the CSR entry e of u's row with col[e] the
 * next vertex towards the sources and dist[u] = dist[col[e]] + w[e]; -1 for
 * sources and unreachable vertices). `stream` is a cudaStream_t (NULL: the
 * default stream). The call is synchronous: between batches of rounds it
 * copies a few control words to the host and waits on `stream`
 * (cudaStreamSynchronize), and it returns after all its work on that
 * stream is done.
 *
 * Limit: V <= GST_NOALLOC_MAX_VERTICES, else GST_TOO_LARGE and nothing runs.
 * The frontier scratch (3 MiB + 256 B) is a fixed array in the library's
 * device image, held on every GPU that loads the library until the process
 * exits. The first call on a device looks up that array's address (once per
 * device, with the device current); make that first call before capturing
 * any stream. Every call shares the array and leaves its contents behind;
 * each call clears what it uses first, but calls whose work overlaps on one
 * GPU (other streams, other host threads) race and corrupt each other.
 * Errors are returned as the status only (gst_last_error() is not set):
 * GST_BAD_INPUT for NULL pointers, V < 1 or a source / CSR entry out of
 * range, GST_OVERFLOW, GST_TIMEOUT, GST_CUDA_ERROR. A CUDA error still
 * pending from the caller's own earlier work makes the call return
 * GST_CUDA_ERROR before it launches anything, and the error is left
 * pending for the caller to read. With num_sources = 0 every vertex is
 * unreachable (dist GST_COST_LIMIT, pred -1).
 * No counterpart in the reference. */
gst_status gst_group_distances_noalloc(const int32_t *row_ptr, const int32_t *col, const int32_t *w, int32_t V,
                                       int64_t nnz, const int32_t *sources, int32_t num_sources, int32_t *dist,
                                       int32_t *pred, void *stream);

/* ---------------------------------------------------------------- misc -- */

/* Message of the last failing call on this thread ("" if none). */
const char *gst_last_error(void);
const char *gst_version(void);

#ifdef __cplusplus
}
#endif
#endif /* GST_H_ */
