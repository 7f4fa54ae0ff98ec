// Learned upper-bound proposal: a small message-passing vertex scorer whose
// top-scored vertex roots a feasible tree (shortest paths to each group,
// then an MST repair on the tree's vertices); that tree's cost is an upper
// bound that prunes the exact DP. An addition with no counterpart in the
// reference; the DP itself stays exact whatever the scorer says.
//
// Network (hidden width 64, three message-passing layers):
//   h0 = relu(W0 x + b0)                           x: 16 query features
//   h_l = relu(Ws_l h_{l-1} + Wn_l mean_{u in N(v)} h_{l-1}(u) + b_l)
//   score(v) = wo . h3(v) + bo
// Inference stores activations and weights in bf16 and accumulates in
// fp32 (tcgen05 GEMMs over 128-vertex tiles); training runs every kernel
// in fp32. Parameters are one flat fp32 vector laid out as below.
#pragma once
#include <cstdint>

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "dpbf.cuh"

namespace gst {

constexpr int kFeat = 16;
constexpr int kHid = 64;
constexpr int kMpLayers = 3;
constexpr int64_t kOffW0 = 0;                              // [kHid][kFeat]
constexpr int64_t kOffB0 = kOffW0 + kHid * kFeat;          // [kHid]
constexpr int64_t kLayerParams = 2 * kHid * kHid + kHid;   // Ws [kHid][kHid], Wn [kHid][kHid], b [kHid]
constexpr int64_t kOffL1 = kOffB0 + kHid;                  // layer l (1-based) at kOffL1 + (l-1)*kLayerParams
constexpr int64_t kOffWo = kOffL1 + kMpLayers * kLayerParams;  // [kHid]
constexpr int64_t kOffBo = kOffWo + kHid;                  // scalar
constexpr int64_t kNumParams = kOffBo + 1;

__host__ __device__ constexpr int64_t layer_off(int l) { return kOffL1 + (int64_t)(l - 1) * kLayerParams; }

// ------------------------------------------------------------- features --
// out[v] = in[v] | OR of in[u] over neighbours u (groups within one more
// hop). With member_nbrs non-null, also counts neighbours that belong to
// some group.
cudaError_t launch_reach(const GraphDev& g, const int32_t* hub_of, const uint32_t* in, uint32_t* out,
                         int32_t* member_nbrs, cudaStream_t s);
// x[v][0..15] from the group masks (see learn_kernels.cu for the list).
cudaError_t launch_features(const GraphDev& g, const uint32_t* m0, const uint32_t* r1, const uint32_t* r2,
                            const uint32_t* r3, const int32_t* member_nbrs, int32_t k, float* x, cudaStream_t s);

// ------------------------------------------------------------ inference --
// bf16 copies of the weights for inference: w0 fp32 is used as is; wcat
// holds, per layer, [kHid][2*kHid] bf16 rows [Ws[o][:] | Wn[o][:]].
cudaError_t launch_pack_bf16(const float* params, __nv_bfloat16* wcat, cudaStream_t s);
// h0 = relu(W0 x + b0) in bf16.
cudaError_t launch_infer_l0(int32_t V, const float* x, const float* params, __nv_bfloat16* h0, cudaStream_t s);
// Hub rows' neighbour sums for one layer, fp32, one 32-entry chunk per warp
// (hub_sum[nbig][kHid], zeroed by the caller).
cudaError_t launch_hub_sum_bf16(const GraphDev& g, const __nv_bfloat16* hin, float* hub_sum, cudaStream_t s);
// TMA descriptor of a bf16 activation buffer (V rows of kHid values, 128
// bytes each): 128-row boxes, 128-byte swizzle, rows past V read as zero.
cudaError_t make_act_map(const __nv_bfloat16* buf, int32_t V, CUtensorMap* out);
// One message-passing layer (l = 1..3): the neighbour mean into agg
// (V x kHid bf16 scratch), then the tcgen05 layer GEMM over [h | agg]
// (hin_map, agg_map: make_act_map of hin and agg). On the last layer, with
// scores non-null, writes scores instead of activations. *err (device) is
// set non-zero if a tensor-core or TMA wait of the layer ran out.
cudaError_t launch_infer_layer(const GraphDev& g, const int32_t* hub_of, const float* hub_sum,
                               const __nv_bfloat16* hin, const CUtensorMap& hin_map, __nv_bfloat16* agg,
                               const CUtensorMap& agg_map, const __nv_bfloat16* wcat_l, const float* params, int l,
                               __nv_bfloat16* hout, float* scores, int32_t* err, cudaStream_t s);
// The layer GEMM alone (launch_infer_layer runs it after the neighbour
// mean). extra_tx > 0 makes each CTA's first tile wait for more bytes than
// its loads deliver, so that the wait runs out and sets *err (the test of
// the bounded waits); 0 otherwise.
cudaError_t launch_layer_gemm(int32_t V, const CUtensorMap& hin_map, const CUtensorMap& agg_map,
                              const __nv_bfloat16* wcat_l, const float* params, int l, __nv_bfloat16* hout,
                              float* scores, int32_t* err, uint32_t extra_tx, cudaStream_t s);
// The proposal's root without a network: most groups within 1 hop, then 2,
// then 3, then degree (s = 1000 x3 + 100 x4 + 10 x5 + x1).
cudaError_t launch_feature_score(int32_t V, const float* x, float* s, cudaStream_t st);
// Top-scored vertices, in two passes: a histogram of the top 12 bits of
// the order-preserving score keys (hist[4096], zeroed by the caller), then
// the vertices whose key bin is >= bin_lo appended as (key, v) to out
// (*count counts them, at most cap are written).
constexpr int kScoreBins = 4096;
cudaError_t launch_score_hist(int32_t V, const float* scores, uint32_t* hist, cudaStream_t s);
cudaError_t launch_score_select(int32_t V, const float* scores, uint32_t bin_lo, uint2* out, int32_t* count,
                                int32_t cap, cudaStream_t s);
// argmax of scores (ties to the smaller ID) packed as an order-preserving
// key: *best = (key(score) << 32) | (0xffffffff - v).
cudaError_t launch_argmax(int32_t V, const float* scores, unsigned long long* best, cudaStream_t s);

// ------------------------------------------------------------- training --
// y = relu(x1 W1^T + x2 W2^T + b), W row-major [kHid][k]; x2 may be null.
cudaError_t launch_dense_fwd(int32_t V, const float* x1, int k1, const float* w1, const float* x2, const float* w2,
                             const float* b, float* y, cudaStream_t s);
// y = dz W (W [kHid][kHid]), i.e. the data gradient of a kHid->kHid layer.
cudaError_t launch_dense_bwd_data(int32_t V, const float* dz, const float* w, float* y, cudaStream_t s);
// dw[o][c] += sum_v dz[v][o] x[v][c] (c < k), db[o] += sum_v dz[v][o] (db may be null)
cudaError_t launch_dense_bwd_weight(int32_t V, const float* dz, const float* x, int k, float* dw, float* db,
                                    cudaStream_t s);
// out[v] = mean over neighbours of x (kHid channels, fp32)
cudaError_t launch_mean_agg(const GraphDev& g, const float* x, float* out, cudaStream_t s);
// dz_prev[u] = (h[u] > 0) * (add[u] + sum over neighbours v of t[v] / deg(v)):
// the transpose of mean aggregation (the CSR lists both directions of
// every edge), plus the self path, through the ReLU of h.
cudaError_t launch_agg_bwd(const GraphDev& g, const float* t, const float* add, const float* h, float* dz_prev,
                           cudaStream_t s);
// s[v] = wo . h[v] + bo
cudaError_t launch_score(int32_t V, const float* h, const float* params, float* s, cudaStream_t st);
// Listwise loss over all vertices: loss = -(1/n) sum_{v in T} log softmax(s)_v
// with T = {v : label[v]}, n = |T|. Writes ds (dloss/ds) and adds the loss
// to *loss. red: 2 floats of scratch.
cudaError_t launch_softmax_loss(int32_t V, const float* s, const uint8_t* label, int32_t n, float* ds, float* loss,
                                float* red, cudaStream_t st);
// Output layer: dwo += sum_v ds_v h[v], dbo += sum ds; dz[v][c] = (h>0) ds_v wo[c].
cudaError_t launch_out_bwd(int32_t V, const float* ds, const float* h, const float* params, float* grad, float* dz,
                           cudaStream_t s);
// label[ids[i]] = 1 for i < n (label zeroed by the caller)
cudaError_t launch_set_labels(const int32_t* ids, int32_t n, uint8_t* label, cudaStream_t s);

// ------------------------------------------------------------ proposal --
// For each group (one block each): the member closest to the root by the
// distances of a one-group solve rooted there (dist = its level-1 slice,
// row stride `stride`), then the walk along its parent records to the
// root, emitting (v, child, w) edges in internal IDs. Members are caller
// IDs (perm maps them). out_n[0] counts edges (capped at cap, stopped
// walks set out_n[1]); out_n[2] is set when some group cannot reach the
// root.
cudaError_t launch_ub_paths(const GraphDev& g, const int32_t* dist, const int32_t* par, int32_t stride,
                            const int32_t* group_ptr, const int32_t* members, const int32_t* perm, int32_t k,
                            int3* out_e, int32_t* out_n, int32_t cap, cudaStream_t s);

// The root's paths to the nearest member of every group over a solve's own
// wave 1 (cost / par: the table, level 1 at its start with row stride
// stride1; gmask: the query's group masks, internal IDs). Counters as for
// launch_ub_paths; a walk that meets an inconsistent record stops.
cudaError_t launch_root_paths(const GraphDev& g, const int32_t* cost, const int32_t* par, int32_t stride1,
                              const uint32_t* gmask, int32_t root, int32_t k, int3* out_e, int32_t* out_n, int32_t cap,
                              cudaStream_t s);

// Adam step over the flat parameter vector (bias-corrected, step t >= 1).
cudaError_t launch_adam(int64_t n, float* p, const float* g, float* m, float* v, float lr, int32_t t, cudaStream_t s);

}  // namespace gst
