/*
 * gst_io.h — readers of the reference's dataset files (host only).
 *
 * The reference's experiment harness (rucgraph/test_gpu.h:115-121) loads a
 * dataset as three text files, parsed by
 * rucgraph/graph_hash_of_mixed_weighted_read_for_GSTP.h:
 *   <name>.in   read_input_graph (:157-204): first line "V E C", then
 *               "input_graph Vertex v nw c" and "input_graph Edge v1 v2 ec"
 *               lines (ec truncated to int, both directions stored, rows
 *               sorted by neighbour ID);
 *   <name>.g    read_Group (:243-274): "g<id>:m1 m2 ..." per group, group
 *               id-1 holding the members;
 *   <name>.gK   read_inquire (:275-302): one query per line, space-separated
 *               values whose last token is ignored; the harness turns value
 *               x into group index x - V (test_gpu.h:147-150).
 * and its fixture instances (simple_iterative_tests.text) by
 * graph_hash_of_mixed_weighted_read_for_GSTP (:9-72). These readers return
 * the same graph and groups in the forms gst_graph_upload / gst_solve take.
 * They differ from the reference only in failing with GST_BAD_INPUT (and a
 * message) where the reference would crash or getchar()/exit(1).
 */
#ifndef GST_IO_H_
#define GST_IO_H_

#include <stdint.h>

#include "gst.h"
#include "gst_gen.h"

#ifdef __cplusplus
extern "C" {
#endif

/* <name>.in -> CSR (gst_host_graph_copy). num_communities receives C from
 * the header line (may be NULL); the per-vertex community is not kept. */
gst_status gst_read_graph_file(const char *path, gst_host_graph **out, int32_t *num_communities);

/* <name>.g -> all groups of the dataset, group g = line id g+1, members
 * sorted (gst_host_groups_copy). Ids missing from the file are empty. */
gst_status gst_read_groups_file(const char *path, gst_host_groups **out);

/* <name>.gK -> the queries: "group" q of the result lists query q's group
 * indices (value - V, as the harness computes them). */
gst_status gst_read_queries_file(const char *path, int32_t V, gst_host_groups **out);

/* A GSTP instance (graph_hash_of_mixed_weighted_save_for_GSTP's text):
 * the input graph (vertex IDs 0..V-1, later Edge lines replace a pair's
 * weight) and the query's groups in increasing group-vertex ID order
 * (group_vertices lines), members from the group_graph edges. */
gst_status gst_read_gstp_instance(const char *path, gst_host_graph **graph, gst_host_groups **groups);

#ifdef __cplusplus
}
#endif
#endif /* GST_IO_H_ */
