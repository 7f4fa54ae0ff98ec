/*
 * gst_debug.h — diagnostics of the GST solver (not needed to solve).
 */
#ifndef GST_DEBUG_H_
#define GST_DEBUG_H_

#include <stdint.h>

#include "gst.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Copies the DP state table of the last gst_solve on g into
 * out[v * 2^k + S] (cost of the best tree rooted at v covering group set S;
 * GST_COST_LIMIT where none; entry S = 0 is set to GST_COST_LIMIT). k must
 * be the k of that solve. The reference keeps the same table in host memory
 * after DPBF_GPU returns (host_tree, src/DPQ.cu:711); libgst keeps it on the
 * device and copies it only on request. */
gst_status gst_graph_debug_table(gst_graph *g, int32_t k, int32_t *out);

typedef struct gst_scorer gst_scorer;

/* Test of the scorer layer's bounded waits: runs the first layer's
 * tensor-core GEMM on g's activation buffers (whatever they hold) with the
 * first tile of every CTA waiting for extra_bytes more than its TMA loads
 * deliver, so that the wait runs out (after about a second at most).
 * *flag_out receives the layer's error flag (1: a load wait ran out; 0:
 * none did) and the status is GST_INTERNAL when it is set; the flag is
 * cleared again and the graph stays usable. extra_bytes = 0 runs the GEMM
 * normally (flag 0, GST_OK). */
gst_status gst_debug_scorer_wait_timeout(gst_graph *g, const gst_scorer *sc, uint32_t extra_bytes,
                                         int32_t *flag_out);

#ifdef __cplusplus
}
#endif
#endif /* GST_DEBUG_H_ */
