/* Learned upper-bound proposal for the GB300 GST solver (libgst).
 *
 * No counterpart in the reference: an addition on top of the DPBF entry
 * point of gst.h. A small message-passing network scores the vertices of a
 * query; its top-scored vertex roots a feasible tree (a shortest path from
 * the root to the nearest member of every group, then an MST repair over
 * the tree's vertices with non-essential leaves removed). That tree's cost
 * is a proven upper bound: gst_solve_learned runs the exact DP pruned by it
 * (exact for any bound >= the optimum) and falls back to the unpruned DP
 * whenever no proposal can be made. The optimal cost never depends on the
 * network, only the time to reach it does.
 *
 * Network: 16 query features per vertex, h0 = relu(W0 x + b0), three
 * layers h_l = relu(Ws_l h_{l-1} + Wn_l mean_{N(v)} h_{l-1} + b_l) of width
 * 64, score = wo . h3 + bo. Parameters are one flat float vector:
 *   W0[64][16], b0[64], then per layer Ws[64][64], Wn[64][64], b[64],
 *   then wo[64], bo  (GST_SCORER_NUM_PARAMS floats).
 * Inference runs in bf16 with fp32 accumulation; training (one query per
 * step, listwise softmax loss against the vertices of a known optimal
 * tree, Adam) runs fp32 forward and backward kernels on the device.
 * Training requires a graph whose CSR lists both directions of every edge
 * (the backward pass of the mean aggregation walks rows as columns).
 */
#ifndef GST_LEARN_H
#define GST_LEARN_H

#include "gst.h"

#ifdef __cplusplus
extern "C" {
#endif

#define GST_SCORER_FEATURES 16
#define GST_SCORER_HIDDEN 64
#define GST_SCORER_LAYERS 3
#define GST_SCORER_NUM_PARAMS 25921

typedef struct gst_scorer gst_scorer;

/* Parameter count (GST_SCORER_NUM_PARAMS). */
int64_t gst_scorer_num_params(void);

/* Copies params (GST_SCORER_NUM_PARAMS floats) to the current device. */
gst_status gst_scorer_create(const float* params, gst_scorer** out);
void gst_scorer_free(gst_scorer* s);
/* Current parameters back to the host. */
gst_status gst_scorer_get_params(const gst_scorer* s, float* out);

/* Scores every vertex for a query (caller vertex IDs, V floats).
 * precision 0 = bf16 inference path, 1 = fp32 training forward path. */
gst_status gst_scorer_scores(gst_graph* g, gst_scorer* s, const int32_t* group_ptr, const int32_t* members, int32_t k,
                             int32_t precision, float* scores);

/* One training step on one query whose optimal tree has the n vertices
 * tree_vertices (caller IDs). Writes the loss; with grads non-null also
 * the gradient (GST_SCORER_NUM_PARAMS floats) before any update; with
 * apply != 0 takes an Adam step of learning rate lr. */
gst_status gst_scorer_train_step(gst_graph* g, gst_scorer* s, const int32_t* group_ptr, const int32_t* members,
                                 int32_t k, const int32_t* tree_vertices, int32_t n, float lr, int32_t apply,
                                 float* loss, float* grads);

/* The proposal alone: a feasible tree (gst_result: cost, vertices, edges)
 * rooted at the top-scored vertex, or, with s NULL, at the vertex chosen by
 * a fixed feature score (most groups within 1, then 2, then 3 hops, then
 * degree): the same pipeline without the network. */
gst_status gst_propose(gst_graph* g, gst_scorer* s, const int32_t* group_ptr, const int32_t* members, int32_t k,
                       gst_result** out);

/* The exact DP pruned by the proposal's cost (opts as for gst_solve; its
 * upper_bound is replaced by the proposal's cost). With s NULL the fixed
 * feature score roots the proposal. With opts->use_graph the proposal runs
 * on a serving lane of g (its own stream and scorer buffers, allocated on
 * first use and freed with g) while the captured DP runs: it starts once
 * the DP's wave 1 has grown, takes its paths from that wave, and its cost
 * reaches the running DP as a bound (waves that started without it prune
 * from the next round on); a proposal the DP outruns is given up. The host
 * loop proposes first and then solves. */
gst_status gst_solve_learned(gst_graph* g, gst_scorer* s, const int32_t* group_ptr, const int32_t* members, int32_t k,
                             const gst_opts* opts, gst_result** out);

/* Pruning bound as the last DP wave saw it (after the refinements of
 * gst_opts.refine_bound; 0 = the solve ran unpruned; a concurrent
 * proposal's cost when lower), the cost of the learned path's proposed
 * tree (0 = no proposal, the fallback ran) and the host wall time of the
 * proposal in ms. gst_solve_learned always refines. */
int32_t gst_result_upper_bound(const gst_result* r);
int32_t gst_result_proposal_cost(const gst_result* r);
/* 1 when the proposal ran beside the DP (gst_solve_learned with use_graph):
 * then times[0] spans both (the solve's stream records its end after the
 * proposal returned), else times[0] is the DP's alone. */
int32_t gst_result_proposal_concurrent(const gst_result* r);
/* gst_solve_learned: host wall time of the whole call in ms. */
double gst_result_wall_ms(const gst_result* r);
double gst_result_proposal_ms(const gst_result* r);

#ifdef __cplusplus
}
#endif

#endif /* GST_LEARN_H */
