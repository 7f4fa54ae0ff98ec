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

#ifdef __cplusplus
}
#endif
#endif /* GST_DEBUG_H_ */
