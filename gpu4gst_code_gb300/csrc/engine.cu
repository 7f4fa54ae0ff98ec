// Host driver of the GB300 DPBF solver behind the C ABI of include/gst.h.
//
// One query runs as k DP waves (one per popcount level l of the group-set
// masks). Wave l: a merge pass fills every state (v,S), |S| = l, from the
// finished lower waves; then growth rounds relax all masks of the wave
// along graph edges until no state changes (a multi-source shortest-path
// fixpoint per mask). The last wave needs no growth: growth can only raise
// min_v T(v,full). The answer is argmin_v T(v,full); the tree is read back
// from the parent records on the device.
//
// Two drivers run the same kernels:
//   host loop    the host launches growth rounds in batches and polls the
//                round's change count between batches;
//   CUDA graph   (gst_opts.use_graph) the whole query is one captured graph,
//                each wave's growth a conditional while node whose body is
//                one round; the round's last block sets the condition, so a
//                query is one graph launch and one host synchronisation.
// Per-query scalars (bound, round cap, stats switch) live in device memory,
// so one instantiated graph per k serves every query.
//
// Compared with DPBF_GPU (src/DPQ.cu:501-768): no V x 2^k host table and no
// full-table host<->device copies (DPQ.cu:592,635,661,711), no host-side
// re-initialisation (DPQ.cu:638-659), no managed memory, and no host
// synchronisation after every launch (DPQ.cu:684-702).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <mutex>
#include <thread>
#include <atomic>
#include <new>
#include <string>
#include <unordered_set>
#include <utility>
#include <vector>

#include "dpbf.cuh"
#include "gst.h"
#include "gst_debug.h"
#include "gst_learn.h"
#include "learn.cuh"

using namespace gst;

// ----------------------------------------------------------------- errors --
namespace {
thread_local std::string g_last_error;

gst_status fail(gst_status s, const std::string& msg) {
  g_last_error = msg;
  return s;
}

#define GST_CUDA(call)                                                                           \
  do {                                                                                           \
    cudaError_t e_ = (call);                                                                     \
    if (e_ != cudaSuccess) {                                                                     \
      return fail(e_ == cudaErrorMemoryAllocation ? GST_OOM : GST_CUDA_ERROR,                    \
                  std::string(#call) + ": " + cudaGetErrorString(e_));                           \
    }                                                                                            \
  } while (0)

template <class T>
void dfree(T*& p) {
  if (p) cudaFree(p);
  p = nullptr;
}

int binom(int n, int r) {
  if (r < 0 || r > n) return 0;
  int64_t c = 1;
  for (int i = 1; i <= r; ++i) c = c * (n - r + i) / i;
  return (int)c;
}

constexpr int32_t kTreePrefix = 4096;   // tree entries read back with the counters
constexpr int kPollEvery = 8;           // host loop: rounds launched between polls
constexpr int kEvents = 3 * GST_MAX_K + 8;
// splits of every level for k = kMergeTabK: (3^k - 2^(k+1) + 1) / 2
constexpr int64_t kMaxMergeSplits = 28501;
constexpr int kProposeTop = 64;        // top-scored vertices offered to the proposal's repair
constexpr int kProposeRounds = 8;      // growth rounds of the proposal's root distances
constexpr int32_t kDefaultLanes = 4;   // concurrent solve contexts of a batch
constexpr int32_t kMaxLanes = 8;
}  // namespace

// ---------------------------------------------------------------- objects --
struct QueryGraph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  uint64_t gen = 0;  // workspace generation it was captured against
};

// One CUDA graph for a chunk of q queries with k groups each (gst_solve_batch
// with gst_opts.batch_graph): the whole solve of every query as parallel
// branches, one per solve context (the graph's own workspace and its lanes').
struct BatchGraph {
  int32_t k = 0, q = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<uint64_t> gens;         // workspace generation of every branch's context at capture
  std::vector<cudaEvent_t> fork, join;  // capture-time fork / join points of the branches
};

struct Workspace {
  uint64_t gen = 1;           // bumped whenever a captured buffer moves
  int32_t k_cap = 0;          // cost/par sized for this many groups
  int32_t* cost = nullptr;    // V * sum of row strides
  int32_t* par = nullptr;
  uint32_t* gmask = nullptr;  // V
  uint8_t* flags = nullptr;   // 6 * vpad: change flags x3, candidate flags x3
  Counters* ctr = nullptr;
  GrowCtl* ctl = nullptr;
  SolveParams* d_params = nullptr;
  long long* stats = nullptr;
  MaskInfo* minfo = nullptr;  // 2^GST_MAX_K
  int32_t* lmasks = nullptr;  // 2^GST_MAX_K
  int32_t* msplit_ptr = nullptr;  // merge split tables of every level (k <= kMergeTabK)
  int2* msplits = nullptr;
  std::vector<int32_t> h_msp_off, h_ms_off, h_ms_n;  // per level: offsets into the two, split count
  int32_t tables_k = 0;       // k the mask tables describe
  int32_t* d_group_ptr = nullptr;
  int32_t* d_members = nullptr;
  int64_t members_cap = 0;
  int2* qa = nullptr;
  int2* qb = nullptr;
  int32_t* out_v = nullptr;
  int3* out_e = nullptr;
  int32_t bt_cap = 0;
  unsigned long long* hub_min = nullptr;  // nbig x hub_stride scratch minima
  int32_t* hub_cnt = nullptr;             // nbig chunk counters
  int32_t hub_stride = 0;
  int32_t* capt = nullptr;  // V x the widest row stride: the current wave's pruning caps
  // tour-bound tables: path (k x 2^k x k), W2 (k x 2^k), then the current
  // level's compact tables (at most 4,410 words at k = 10), kTourMaxK sized
  int32_t* tour = nullptr;
  // pinned host mirrors
  Counters* h_ctr = nullptr;
  GrowCtl* h_ctl = nullptr;
  SolveParams* h_params = nullptr;
  long long* h_stats = nullptr;
  int32_t* h_out_v = nullptr;
  int3* h_out_e = nullptr;
  cudaEvent_t ev[kEvents] = {};
  // recorded by every query graph once wave 1 has grown (an external event
  // node): a proposal running beside the solve reads wave 1 after it
  cudaEvent_t ev_wave1 = nullptr;
  std::vector<int32_t> h_lvl_base, h_lvl_m, h_lvl_stride;
  QueryGraph qg[GST_MAX_K + 1];
  // the same graphs with the per-wave timing events as external event nodes
  // (solves with statistics on: their merge and growth times are read back)
  QueryGraph qg_timed[GST_MAX_K + 1];
};

// Buffers of the learned proposal (allocated on first use).
struct LearnWs {
  int32_t V = 0;
  // features + inference
  uint32_t* r1 = nullptr;
  uint32_t* r2 = nullptr;
  uint32_t* r3 = nullptr;
  int32_t* mnb = nullptr;
  float* x = nullptr;                 // V x kFeat
  __nv_bfloat16* hb[3] = {nullptr, nullptr, nullptr};  // V x kHid each: two activations, the neighbour mean
  CUtensorMap hb_map[3];              // their TMA descriptors (make_act_map)
  int32_t* infer_err = nullptr;       // set by the layer GEMM when one of its waits ran out
  float* hub_sum = nullptr;           // nbig x kHid
  float* scores = nullptr;            // V
  unsigned long long* best = nullptr;
  uint32_t* hist = nullptr;           // kScoreBins
  uint2* top = nullptr;               // (key, v) of the top-scored vertices
  int32_t top_cap = 0;
  int3* pe = nullptr;                 // proposal path edges
  int32_t* pn = nullptr;              // [count, stopped, unreachable]
  int32_t pe_cap = 0;
  // training (fp32)
  float* h[kMpLayers + 1] = {};       // h0..h3, V x kHid
  float* a[kMpLayers + 1] = {};       // a1..a3 (a[0] unused)
  float* dz = nullptr;
  float* dzp = nullptr;
  float* t = nullptr;
  float* u = nullptr;
  float* s = nullptr;                 // V
  float* ds = nullptr;                // V
  uint8_t* label = nullptr;           // V
  int32_t* ids = nullptr;             // tree vertices
  int32_t ids_cap = 0;
  float* red = nullptr;               // loss scratch (2) + loss (1)
  float* grad = nullptr;              // kNumParams
};

struct gst_graph {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t side = nullptr;  // captures conditional bodies
  // learned overlap (gst_solve_learned): the solve's parameters are on the
  // device; its graph has finished; the end of the lane's queued work
  cudaEvent_t ev_params = nullptr, ev_done = nullptr, ev_side = nullptr;
  cudaEvent_t ev_poll = nullptr;  // wait_or_stop's marker on this context's stream
  int32_t V = 0;
  int64_t nnz = 0;
  int32_t* d_row_ptr = nullptr;
  int2* d_adj = nullptr;
  int32_t* d_big = nullptr;
  int32_t nbig = 0;
  int32_t deg_big = kDegBigMin;  // hub threshold of this graph
  int32_t* d_order = nullptr;  // vertices of degree <= deg_big, by decreasing degree
  int2* d_hub_chunk = nullptr;  // (hub index, first CSR entry) per 32-entry chunk of a hub row
  int32_t* d_chunk_vtx = nullptr;  // the hub vertex of each chunk
  int64_t nchunks = 0;
  int4* d_hub_seg = nullptr;  // (hub vertex, hub index, first entry, segments of the hub) per kHubSeg-entry segment
  int64_t nsegs = 0;
  int32_t max_w = 0;  // largest edge weight
  // Internal vertex IDs: perm[caller ID] and its inverse (see gst_graph_upload)
  std::vector<int32_t> perm, inv;
  int32_t* d_perm = nullptr;
  int32_t* d_hub_of = nullptr;  // hub index of a vertex, -1 for the others
  std::vector<int32_t> h_row;   // host copy of the internal CSR (proposal repair)
  std::vector<int2> h_adj;
  std::vector<int32_t> h_slot;  // V-sized scratch of the repair (all zero between uses)
  std::mutex mu;
  Workspace ws;
  LearnWs lw;
  // Serving lanes: extra solve contexts sharing this graph's device arrays
  // (own workspace and streams), used by concurrent batches.
  bool owns_device = true;
  const gst_graph* parent = nullptr;
  std::vector<gst_graph*> lanes;
  // Tuning (gst_autotune): dense-round shift per k (0 = default) and the
  // batch concurrency (0 = default).
  int32_t tuned_shift[GST_MAX_K + 1] = {};
  int32_t tuned_lanes = 0;
  int32_t tuned_batch_graph = 0;  // queries per batch graph chosen by gst_autotune (0: lanes)
  std::vector<BatchGraph*> batch_graphs;
};

struct gst_result {
  gst_status status = GST_OK;
  int32_t cost = -1;
  int32_t root = -1;
  std::vector<int32_t> vertices;
  std::vector<int32_t> edges;  // (u, v, w) triples, u < v
  int64_t states = 0;
  int64_t launches = 0;  // kernels this solve launched
  double ms[4] = {0, 0, 0, 0};
  int64_t stats[kNumStats] = {};
  double lat_ms[2] = {0, 0};  // batch: own solve wall time, completion since the batch began
  int32_t replica = -1;       // pool: replica that solved the query
  int32_t ub = 0;             // pruning bound at the last wave (0 = none)
  int32_t proposal_cost = 0;  // cost of the learned path's proposed tree
  double propose_ms = 0;      // host wall time of the proposal
  int32_t proposal_concurrent = 0;  // the proposal ran beside the DP, on a serving lane
  double wall_ms = 0;         // learned solves: host wall time of the whole call
};

struct gst_scorer {
  int device = 0;
  float* params = nullptr;         // kNumParams fp32
  __nv_bfloat16* wcat = nullptr;   // kMpLayers x kHid x 2 kHid bf16
  float* m = nullptr;              // Adam moments
  float* v = nullptr;
  int32_t t = 0;                   // Adam steps taken
};

namespace {

GraphDev graph_dev(const gst_graph* g) {
  GraphDev d;
  d.V = g->V;
  d.row_ptr = g->d_row_ptr;
  d.adj = g->d_adj;
  d.big = g->d_big;
  d.deg_big = g->deg_big;
  d.nbig = g->nbig;
  d.order = g->d_order;
  d.nsmall = g->V - g->nbig;
  d.hub_chunk = g->d_hub_chunk;
  d.chunk_vtx = g->d_chunk_vtx;
  d.nchunks = g->nchunks;
  d.hub_seg = g->d_hub_seg;
  d.nsegs = g->nsegs;
  d.hub_min = g->ws.hub_min;
  d.hub_cnt = g->ws.hub_cnt;
  d.hub_stride = g->ws.hub_stride;
  return d;
}

void drop_graphs(Workspace& ws) {
  for (QueryGraph* set : {ws.qg, ws.qg_timed})
    for (int k = 0; k <= GST_MAX_K; ++k) {
      QueryGraph& q = set[k];
      if (q.exec) cudaGraphExecDestroy(q.exec);
      if (q.graph) cudaGraphDestroy(q.graph);
      q = QueryGraph{};
    }
}

void free_learn(LearnWs& lw) {
  dfree(lw.r1);
  dfree(lw.r2);
  dfree(lw.r3);
  dfree(lw.mnb);
  dfree(lw.x);
  dfree(lw.hb[0]);
  dfree(lw.hb[1]);
  dfree(lw.hb[2]);
  dfree(lw.hub_sum);
  dfree(lw.scores);
  dfree(lw.best);
  dfree(lw.hist);
  dfree(lw.top);
  dfree(lw.pe);
  dfree(lw.pn);
  dfree(lw.infer_err);
  for (auto& p : lw.h) dfree(p);
  for (auto& p : lw.a) dfree(p);
  dfree(lw.dz);
  dfree(lw.dzp);
  dfree(lw.t);
  dfree(lw.u);
  dfree(lw.s);
  dfree(lw.ds);
  dfree(lw.label);
  dfree(lw.ids);
  dfree(lw.red);
  dfree(lw.grad);
  lw = LearnWs{};
}

void free_workspace(Workspace& ws) {
  drop_graphs(ws);
  dfree(ws.cost);
  dfree(ws.par);
  dfree(ws.gmask);
  dfree(ws.flags);
  dfree(ws.ctr);
  dfree(ws.ctl);
  dfree(ws.d_params);
  dfree(ws.stats);
  dfree(ws.minfo);
  dfree(ws.lmasks);
  dfree(ws.msplit_ptr);
  dfree(ws.msplits);
  dfree(ws.d_group_ptr);
  dfree(ws.d_members);
  dfree(ws.qa);
  dfree(ws.qb);
  dfree(ws.out_v);
  dfree(ws.out_e);
  dfree(ws.hub_min);
  dfree(ws.hub_cnt);
  dfree(ws.capt);
  dfree(ws.tour);
  for (void* p : {(void*)ws.h_ctr, (void*)ws.h_ctl, (void*)ws.h_params, (void*)ws.h_stats, (void*)ws.h_out_v,
                  (void*)ws.h_out_e})
    if (p) cudaFreeHost(p);
  ws.h_ctr = nullptr;
  ws.h_ctl = nullptr;
  ws.h_params = nullptr;
  ws.h_stats = nullptr;
  ws.h_out_v = nullptr;
  ws.h_out_e = nullptr;
  for (auto& e : ws.ev)
    if (e) {
      cudaEventDestroy(e);
      e = nullptr;
    }
  if (ws.ev_wave1) cudaEventDestroy(ws.ev_wave1);
  ws.ev_wave1 = nullptr;
  ws.k_cap = 0;
  ws.tables_k = 0;
  ws.members_cap = 0;
  ws.bt_cap = 0;
}

// Stride of the flag arrays: V rounded up to 16 bytes, so word atomics on
// candidate bytes stay aligned in every array.
int64_t vpad_of(int64_t V) { return (V + 15) & ~int64_t(15); }

// Row strides of every level for k groups; returns their sum.
int64_t total_stride(int32_t k) {
  int64_t s = 0;
  for (int l = 1; l <= k; ++l) s += row_stride(binom(k, l));
  return s;
}

// Allocates everything a query with k groups and `nmembers` members needs.
gst_status ensure_workspace(gst_graph* g, int32_t k, int64_t nmembers) {
  Workspace& ws = g->ws;
  const int64_t V = g->V;
  if (!ws.gmask) {
    GST_CUDA(cudaMalloc(&ws.gmask, V * sizeof(uint32_t)));
    GST_CUDA(cudaMalloc(&ws.flags, 6 * (size_t)vpad_of(V)));
    GST_CUDA(cudaMalloc(&ws.ctr, sizeof(Counters)));
    GST_CUDA(cudaMalloc(&ws.ctl, sizeof(GrowCtl)));
    GST_CUDA(cudaMalloc(&ws.d_params, sizeof(SolveParams)));
    GST_CUDA(cudaMalloc(&ws.stats, kNumStats * sizeof(long long)));
    GST_CUDA(cudaMalloc(&ws.minfo, sizeof(MaskInfo) << GST_MAX_K));
    GST_CUDA(cudaMalloc(&ws.lmasks, sizeof(int32_t) << GST_MAX_K));
    GST_CUDA(cudaMalloc(&ws.msplit_ptr, ((size_t(1) << kMergeTabK) + kMergeTabK + 2) * sizeof(int32_t)));
    GST_CUDA(cudaMalloc(&ws.msplits, kMaxMergeSplits * sizeof(int2)));
    GST_CUDA(cudaMallocHost(&ws.h_ctr, sizeof(Counters)));
    GST_CUDA(cudaMallocHost(&ws.h_ctl, sizeof(GrowCtl)));
    GST_CUDA(cudaMallocHost(&ws.h_params, sizeof(SolveParams)));
    GST_CUDA(cudaMallocHost(&ws.h_stats, kNumStats * sizeof(long long)));
    GST_CUDA(cudaMallocHost(&ws.h_out_v, kTreePrefix * sizeof(int32_t)));
    GST_CUDA(cudaMallocHost(&ws.h_out_e, kTreePrefix * sizeof(int3)));
    for (auto& e : ws.ev) GST_CUDA(cudaEventCreate(&e));
    GST_CUDA(cudaEventCreateWithFlags(&ws.ev_wave1, cudaEventDisableTiming));
    // backtrack capacity: states of one optimal derivation
    ws.bt_cap = (int32_t)std::min<int64_t>(4 * V + 256, 1 << 24);
    GST_CUDA(cudaMalloc(&ws.qa, (size_t)ws.bt_cap * sizeof(int2)));
    GST_CUDA(cudaMalloc(&ws.qb, (size_t)ws.bt_cap * sizeof(int2)));
    GST_CUDA(cudaMalloc(&ws.out_v, (size_t)ws.bt_cap * sizeof(int32_t)));
    GST_CUDA(cudaMalloc(&ws.out_e, (size_t)ws.bt_cap * sizeof(int3)));
    GST_CUDA(cudaMalloc(&ws.tour, ((size_t)kTourMaxK * (1 << kTourMaxK) * (kTourMaxK + 1) + kTourCompactWords) *
                                      sizeof(int32_t)));
  }
  if (k > ws.k_cap) {
    dfree(ws.cost);
    dfree(ws.par);
    ws.k_cap = 0;
    ++ws.gen;
    const size_t entries = (size_t)V * (size_t)total_stride(k);
    GST_CUDA(cudaMalloc(&ws.cost, entries * sizeof(int32_t)));
    GST_CUDA(cudaMalloc(&ws.par, entries * sizeof(int32_t)));
    dfree(ws.hub_min);
    dfree(ws.hub_cnt);
    dfree(ws.capt);
    int32_t smax = 4;
    for (int l = 1; l <= k; ++l) smax = std::max(smax, row_stride(binom(k, l)));
    GST_CUDA(cudaMalloc(&ws.capt, (size_t)V * smax * sizeof(int32_t)));
    ws.hub_stride = smax;
    const size_t nh = std::max<size_t>(1, (size_t)g->nbig);
    GST_CUDA(cudaMalloc(&ws.hub_min, nh * (size_t)smax * sizeof(unsigned long long)));
    GST_CUDA(cudaMalloc(&ws.hub_cnt, nh * sizeof(int32_t)));
    ws.k_cap = k;
  }
  if (nmembers > ws.members_cap || !ws.d_group_ptr) {
    dfree(ws.d_group_ptr);
    dfree(ws.d_members);
    ws.members_cap = 0;
    ++ws.gen;
    const int64_t cap = std::max<int64_t>(2 * nmembers, 4096);
    GST_CUDA(cudaMalloc(&ws.d_group_ptr, (GST_MAX_K + 1) * sizeof(int32_t)));
    GST_CUDA(cudaMalloc(&ws.d_members, (size_t)cap * sizeof(int32_t)));
    ws.members_cap = cap;
  }
  return GST_OK;
}

// Mask order: by popcount, then by value. Uploads MaskInfo[mask] and the
// per-level mask lists for k.
gst_status ensure_tables(gst_graph* g, int32_t k) {
  Workspace& ws = g->ws;
  if (ws.tables_k == k) return GST_OK;
  const int W = 1 << k;
  std::vector<MaskInfo> info((size_t)W);
  std::vector<int32_t> lm((size_t)total_stride(k), 0);
  ws.h_lvl_base.assign((size_t)k + 2, 0);
  ws.h_lvl_m.assign((size_t)k + 2, 0);
  ws.h_lvl_stride.assign((size_t)k + 2, 0);
  int32_t base = 0;
  for (int l = 1; l <= k; ++l) {
    ws.h_lvl_base[l] = base;
    ws.h_lvl_m[l] = binom(k, l);
    ws.h_lvl_stride[l] = row_stride(ws.h_lvl_m[l]);
    int32_t rank = 0;
    for (int S = 1; S < W; ++S)
      if (__builtin_popcount((unsigned)S) == l) {
        info[(size_t)S] = MaskInfo{base, ws.h_lvl_stride[l], rank, l};
        lm[(size_t)(base + rank)] = S;
        ++rank;
      }
    base += ws.h_lvl_stride[l];
  }
  info[0] = MaskInfo{0, 0, 0, 0};
  // merge split tables (k <= kMergeTabK): per level, per mask in rank order,
  // every split S1 | S2 = S with S1 holding S's lowest group
  std::vector<int32_t> msp;
  std::vector<int2> ms;
  ws.h_msp_off.assign((size_t)k + 2, 0);
  ws.h_ms_off.assign((size_t)k + 2, 0);
  ws.h_ms_n.assign((size_t)k + 2, 0);
  if (k <= kMergeTabK) {
    for (int l = 1; l <= k; ++l) {
      ws.h_msp_off[l] = (int32_t)msp.size();
      ws.h_ms_off[l] = (int32_t)ms.size();
      for (int32_t rank = 0; rank < ws.h_lvl_m[l]; ++rank) {
        msp.push_back((int32_t)ms.size() - ws.h_ms_off[l]);
        const uint32_t S = (uint32_t)lm[(size_t)(ws.h_lvl_base[l] + rank)];
        if (l < 2) continue;
        const uint32_t low = S & (0u - S), rest = S ^ low;
        for (uint32_t sub = (rest - 1u) & rest;; sub = (sub - 1u) & rest) {
          const uint32_t s1 = sub | low, s2 = S ^ s1;
          const MaskInfo& i1 = info[s1];
          const MaskInfo& i2 = info[s2];
          ms.push_back(make_int2((i1.level << 24) | i1.rank, (i2.level << 24) | i2.rank));
          if (sub == 0u) break;
        }
      }
      msp.push_back((int32_t)ms.size() - ws.h_ms_off[l]);
      ws.h_ms_n[l] = (int32_t)ms.size() - ws.h_ms_off[l];
    }
    if (ms.size() > (size_t)kMaxMergeSplits) return fail(GST_INTERNAL, "merge split table overflow");
    GST_CUDA(cudaMemcpyAsync(ws.msplit_ptr, msp.data(), msp.size() * sizeof(int32_t), cudaMemcpyHostToDevice,
                             g->stream));
    if (!ms.empty())
      GST_CUDA(cudaMemcpyAsync(ws.msplits, ms.data(), ms.size() * sizeof(int2), cudaMemcpyHostToDevice, g->stream));
  }
  GST_CUDA(cudaMemcpyAsync(ws.minfo, info.data(), info.size() * sizeof(MaskInfo), cudaMemcpyHostToDevice,
                           g->stream));
  GST_CUDA(cudaMemcpyAsync(ws.lmasks, lm.data(), lm.size() * sizeof(int32_t), cudaMemcpyHostToDevice, g->stream));
  GST_CUDA(cudaStreamSynchronize(g->stream));  // host vectors go out of scope
  ws.tables_k = k;
  return GST_OK;
}

gst_status validate_groups(const gst_graph* g, const int32_t* group_ptr, const int32_t* members, int32_t k,
                           bool* empty_group) {
  if (!group_ptr || k < 1 || k > GST_MAX_K) return fail(GST_BAD_INPUT, "k must be in [1, GST_MAX_K]");
  if (group_ptr[0] != 0) return fail(GST_BAD_INPUT, "group_ptr[0] must be 0");
  *empty_group = false;
  for (int32_t i = 0; i < k; ++i) {
    if (group_ptr[i + 1] < group_ptr[i]) return fail(GST_BAD_INPUT, "group_ptr must be non-decreasing");
    if (group_ptr[i + 1] == group_ptr[i]) *empty_group = true;
  }
  if (group_ptr[k] > 0 && !members) return fail(GST_BAD_INPUT, "members is NULL");
  for (int32_t i = 0; i < group_ptr[k]; ++i)
    if (members[i] < 0 || members[i] >= g->V) return fail(GST_BAD_INPUT, "group member out of range");
  return GST_OK;
}

LevelArgs level_args(gst_graph* g, int32_t k, int32_t l) {
  Workspace& ws = g->ws;
  LevelArgs a{};
  a.level = l;
  a.m = ws.h_lvl_m[l];
  a.stride = ws.h_lvl_stride[l];
  a.k = k;
  a.base = (int64_t)ws.h_lvl_base[l] * g->V;
  a.stride1 = ws.h_lvl_stride[1];
  a.lmasks = ws.lmasks + ws.h_lvl_base[l];
  a.minfo = ws.minfo;
  a.cost = ws.cost;
  a.par = ws.par;
  a.gmask = ws.gmask;
  a.vpad = (int32_t)vpad_of(g->V);
  a.flags = ws.flags;
  a.cand = ws.flags + 3 * vpad_of(g->V);
  a.ctl = ws.ctl;
  a.ctr = ws.ctr;
  a.stats = ws.stats;
  a.params = ws.d_params;
  a.msplit_ptr = k <= kMergeTabK ? ws.msplit_ptr + ws.h_msp_off[l] : nullptr;
  a.msplits = k <= kMergeTabK ? ws.msplits + ws.h_ms_off[l] : nullptr;
  a.nsplits = k <= kMergeTabK ? ws.h_ms_n[l] : 0;
  a.use_cond = 0;
  a.capt = ws.capt;
  a.tour = (k <= kTourMaxK && l >= 2 && l < k) ? ws.tour : nullptr;  // the last merge has no groups left
  return a;
}

MergeLevels merge_levels(const gst_graph* g, int32_t k) {
  const Workspace& ws = g->ws;
  MergeLevels ml{};
  for (int l = 1; l <= std::min(k, kMergeTabK); ++l) {
    ml.off[l] = (int64_t)ws.h_lvl_base[l] * g->V;
    ml.stride[l] = ws.h_lvl_stride[l];
    ml.mbase[l] = ws.h_lvl_base[l];
  }
  ml.lmasks_all = ws.lmasks;
  return ml;
}

// Work before the waves: group masks and counters.
gst_status enqueue_prologue(gst_graph* g, int32_t k, cudaStream_t s, int64_t* launches) {
  Workspace& ws = g->ws;
  GST_CUDA(cudaMemsetAsync(ws.gmask, 0, (size_t)g->V * sizeof(uint32_t), s));
  GST_CUDA(cudaMemsetAsync(ws.ctr, 0, sizeof(Counters), s));
  GST_CUDA(cudaMemsetAsync(&ws.ctr->best, 0xff, sizeof(unsigned long long), s));
  GST_CUDA(cudaMemsetAsync(ws.stats, 0, kNumStats * sizeof(long long), s));
  if (g->nbig > 0) {  // hub scratch: minima "none", counters zero
    GST_CUDA(cudaMemsetAsync(ws.hub_min, 0xff, (size_t)g->nbig * ws.hub_stride * sizeof(unsigned long long), s));
    GST_CUDA(cudaMemsetAsync(ws.hub_cnt, 0, (size_t)g->nbig * sizeof(int32_t), s));
  }
  GST_CUDA(launch_group_masks(ws.d_group_ptr, ws.d_members, g->d_perm, k, ws.gmask, s));
  ++*launches;
  return GST_OK;
}

// Wave l's merge, preceded by the reset of its flags and loop control.
gst_status enqueue_merge(gst_graph* g, const LevelArgs& a, cudaStream_t s, int64_t* launches) {
  Workspace& ws = g->ws;
  GST_CUDA(cudaMemsetAsync(ws.flags, 0, 6 * (size_t)vpad_of(g->V), s));
  GST_CUDA(cudaMemsetAsync(ws.ctl, 0, sizeof(GrowCtl), s));
  if (a.tour) {  // the tour bound's tables for the bound as it stands now (no-op without one)
    GST_CUDA(launch_tour_table(a, ws.d_group_ptr, ws.d_members, g->d_perm, ws.tour, s));
    ++*launches;
  }
  GST_CUDA(launch_merge(graph_dev(g), a, merge_levels(g, a.k), s));
  ++*launches;
  if (a.level < a.k) {  // how round 0 of the wave starts
    GST_CUDA(launch_seed(graph_dev(g), a, g->num_sms, s));
    ++*launches;
  }
  return GST_OK;
}

// Argmin, backtrack and the read-back of counters and a tree prefix.
gst_status enqueue_epilogue(gst_graph* g, int32_t k, cudaStream_t s, int64_t* launches) {
  Workspace& ws = g->ws;
  const GraphDev gd = graph_dev(g);
  const int32_t* full_slice = ws.cost + (int64_t)ws.h_lvl_base[k] * g->V;
  GST_CUDA(launch_argmin(gd, full_slice, ws.h_lvl_stride[k], ws.ctr, s));
  GST_CUDA(launch_backtrack(gd, g->nnz, ws.par, ws.minfo, (1 << k) - 1, ws.ctr, ws.qa, ws.qb, ws.out_v, ws.out_e,
                            ws.bt_cap, s));
  *launches += 2;
  const size_t pre = (size_t)std::min(kTreePrefix, ws.bt_cap);
  GST_CUDA(cudaMemcpyAsync(ws.h_ctr, ws.ctr, sizeof(Counters), cudaMemcpyDeviceToHost, s));
  GST_CUDA(cudaMemcpyAsync(ws.h_params, ws.d_params, sizeof(SolveParams), cudaMemcpyDeviceToHost, s));
  GST_CUDA(cudaMemcpyAsync(ws.h_stats, ws.stats, kNumStats * sizeof(long long), cudaMemcpyDeviceToHost, s));
  GST_CUDA(cudaMemcpyAsync(ws.h_out_v, ws.out_v, pre * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  GST_CUDA(cudaMemcpyAsync(ws.h_out_e, ws.out_e, pre * sizeof(int3), cudaMemcpyDeviceToHost, s));
  return GST_OK;
}

// Adds a while node to the graph being captured on `s`; its body (one
// growth round) is captured on the side stream.
gst_status capture_growth_loop(gst_graph* g, LevelArgs a, cudaStream_t s) {
  cudaStreamCaptureStatus cs;
  cudaGraph_t cg = nullptr;
  const cudaGraphNode_t* deps = nullptr;
  size_t ndeps = 0;
  GST_CUDA(cudaStreamGetCaptureInfo(s, &cs, nullptr, &cg, &deps, nullptr, &ndeps));
  if (cs != cudaStreamCaptureStatusActive) return fail(GST_INTERNAL, "stream is not capturing");
  cudaGraphConditionalHandle h;
  GST_CUDA(cudaGraphConditionalHandleCreate(&h, cg, 1, cudaGraphCondAssignDefault));
  cudaGraphNodeParams p{};
  p.type = cudaGraphNodeTypeConditional;
  p.conditional.handle = h;
  p.conditional.type = cudaGraphCondTypeWhile;
  p.conditional.size = 1;
  cudaGraphNode_t node;
  GST_CUDA(cudaGraphAddNode(&node, cg, deps, nullptr, ndeps, &p));
  GST_CUDA(cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
  cudaGraph_t body = p.conditional.phGraph_out[0];
  a.cond = h;
  a.use_cond = 1;
  GST_CUDA(cudaStreamBeginCaptureToGraph(g->side, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
  int64_t body_launches = 0;
  const cudaError_t le = launch_grow_round(graph_dev(g), a, g->num_sms, g->side, &body_launches);
  cudaGraph_t done = nullptr;
  const cudaError_t ee = cudaStreamEndCapture(g->side, &done);
  GST_CUDA(le);
  GST_CUDA(ee);
  return GST_OK;
}

// Captures and instantiates the whole query for k (workspace generation
// gen). timed: the per-wave events become external event nodes, so the
// host reads each wave's merge and growth time after the launch (a few
// microseconds more per query; used for solves with statistics on).
gst_status build_query_graph(gst_graph* g, int32_t k, bool timed = false) {
  Workspace& ws = g->ws;
  QueryGraph& q = timed ? ws.qg_timed[k] : ws.qg[k];
  if (q.exec && q.gen == ws.gen) return GST_OK;
  if (q.exec) cudaGraphExecDestroy(q.exec);
  if (q.graph) cudaGraphDestroy(q.graph);
  q = QueryGraph{};
  cudaStream_t s = g->stream;
  int64_t launches = 0;
  auto record = [&](cudaEvent_t e) {
    return timed ? cudaEventRecordWithFlags(e, s, cudaEventRecordExternal) : cudaEventRecord(e, s);
  };
  GST_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
  gst_status st = enqueue_prologue(g, k, s, &launches);
  for (int32_t l = 1; st == GST_OK && l <= k; ++l) {
    const LevelArgs a = level_args(g, k, l);
    if (record(ws.ev[3 * l]) != cudaSuccess) st = fail(GST_CUDA_ERROR, "event record");
    if (st == GST_OK) st = enqueue_merge(g, a, s, &launches);
    if (st == GST_OK && record(ws.ev[3 * l + 1]) != cudaSuccess)
      st = fail(GST_CUDA_ERROR, "event record");
    if (st == GST_OK && l < k) st = capture_growth_loop(g, a, s);
    // refinement after the last grown wave would only tighten the final
    // merge's cap, and the final merge evaluates every split either way
    if (st == GST_OK && l < k - 1 && launch_ub_refine(graph_dev(g), a, g->num_sms, s) != cudaSuccess)
      st = fail(GST_CUDA_ERROR, "bound refinement launch");
    if (st == GST_OK && record(ws.ev[3 * l + 2]) != cudaSuccess)
      st = fail(GST_CUDA_ERROR, "event record");
    if (st == GST_OK && l == 1 && cudaEventRecordWithFlags(ws.ev_wave1, s, cudaEventRecordExternal) != cudaSuccess)
      st = fail(GST_CUDA_ERROR, "event record");
  }
  if (st == GST_OK && record(ws.ev[1]) != cudaSuccess) st = fail(GST_CUDA_ERROR, "event record");
  if (st == GST_OK) st = enqueue_epilogue(g, k, s, &launches);
  cudaGraph_t graph = nullptr;
  const cudaError_t ee = cudaStreamEndCapture(s, &graph);
  if (st != GST_OK) {
    if (graph) cudaGraphDestroy(graph);
    return st;
  }
  GST_CUDA(ee);
  cudaGraphExec_t exec = nullptr;
  const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
  if (ie != cudaSuccess) {
    cudaGraphDestroy(graph);
    return fail(GST_CUDA_ERROR, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(ie));
  }
  q.graph = graph;
  q.exec = exec;
  q.gen = ws.gen;
  return GST_OK;
}

float elapsed(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) {
    cudaGetLastError();  // a timing gap is not an error of the solve
    ms = 0.f;
  }
  return ms;
}

// Builds the host result from the device walk: distinct vertices, distinct
// edges (u < v), and a check that the edges cost exactly the DP optimum.
gst_status collect_tree(gst_graph* g, gst_result* r, int32_t cost, int32_t root) {
  Workspace& ws = g->ws;
  const Counters& c = *ws.h_ctr;
  if (c.bt_overflow) return fail(GST_INTERNAL, "tree walk failed (code " + std::to_string(c.bt_overflow) + ")");
  const int32_t nv = c.bt_nv, ne = c.bt_ne;
  std::vector<int32_t> hv((size_t)nv);
  std::vector<int3> he((size_t)ne);
  if (nv <= kTreePrefix && ne <= kTreePrefix) {
    std::copy(ws.h_out_v, ws.h_out_v + nv, hv.begin());
    std::copy(ws.h_out_e, ws.h_out_e + ne, he.begin());
  } else {
    if (nv) GST_CUDA(cudaMemcpyAsync(hv.data(), ws.out_v, (size_t)nv * 4, cudaMemcpyDeviceToHost, g->stream));
    if (ne)
      GST_CUDA(cudaMemcpyAsync(he.data(), ws.out_e, (size_t)ne * sizeof(int3), cudaMemcpyDeviceToHost, g->stream));
    GST_CUDA(cudaStreamSynchronize(g->stream));
  }
  // back to caller IDs (the walk checked every ID against V)
  for (auto& v : hv) v = g->inv[(size_t)v];
  for (auto& e : he) {
    e.x = g->inv[(size_t)e.x];
    e.y = g->inv[(size_t)e.y];
  }
  root = g->inv[(size_t)root];
  std::sort(hv.begin(), hv.end());
  hv.erase(std::unique(hv.begin(), hv.end()), hv.end());
  std::vector<std::pair<std::pair<int32_t, int32_t>, int32_t>> es;
  es.reserve(he.size());
  for (auto& e : he) es.push_back({{std::min(e.x, e.y), std::max(e.x, e.y)}, e.z});
  std::sort(es.begin(), es.end());
  // one entry per vertex pair (the lightest, should parallel entries exist)
  std::vector<std::pair<std::pair<int32_t, int32_t>, int32_t>> uniq;
  for (auto& e : es)
    if (uniq.empty() || uniq.back().first != e.first) uniq.push_back(e);
  int64_t sum = 0;
  for (auto& e : uniq) sum += e.second;
  if (sum != cost)
    return fail(GST_INTERNAL, "tree weight " + std::to_string(sum) + " != DP cost " + std::to_string(cost));
  // with zero-weight edges the union could hold a cycle: keep a BFS tree
  if (uniq.size() + 1 != hv.size()) {
    std::vector<std::pair<std::pair<int32_t, int32_t>, int32_t>> tree;
    std::unordered_set<int32_t> seen{root};
    bool grew = true;
    while (grew) {
      grew = false;
      for (auto& e : uniq) {
        bool a = seen.count(e.first.first), b = seen.count(e.first.second);
        if (a != b) {
          seen.insert(a ? e.first.second : e.first.first);
          tree.push_back(e);
          grew = true;
        }
      }
    }
    uniq.swap(tree);
  }
  r->vertices = std::move(hv);
  r->edges.clear();
  for (auto& e : uniq) {
    r->edges.push_back(e.first.first);
    r->edges.push_back(e.first.second);
    r->edges.push_back(e.second);
  }
  r->cost = cost;
  r->root = root;
  return GST_OK;
}

// Host-loop driver: launches growth rounds in batches, polling the change
// count of the last completed round between batches.
gst_status run_host_loop(gst_graph* g, int32_t k, int64_t* launches, bool* timeout) {
  Workspace& ws = g->ws;
  cudaStream_t s = g->stream;
  const GraphDev gd = graph_dev(g);
  // GST_TRACE=1 in the environment: poll and report every round (slow;
  // diagnostics of frontier sizes only)
  static const bool trace = std::getenv("GST_TRACE") != nullptr;
  const int batch = trace ? 1 : kPollEvery;
  const gst_status pst = enqueue_prologue(g, k, s, launches);
  if (pst != GST_OK) return pst;
  for (int32_t l = 1; l <= k; ++l) {
    const LevelArgs a = level_args(g, k, l);
    GST_CUDA(cudaEventRecord(ws.ev[3 * l], s));
    gst_status st = enqueue_merge(g, a, s, launches);
    if (st != GST_OK) return st;
    GST_CUDA(cudaEventRecord(ws.ev[3 * l + 1], s));
    if (l < k) {
      for (int64_t r = 0;; r += batch) {
        for (int i = 0; i < batch; ++i) {
          if (trace) GST_CUDA(cudaEventRecord(ws.ev[kEvents - 2], s));
          GST_CUDA(launch_grow_round(gd, a, g->num_sms, s, launches));
          if (trace) GST_CUDA(cudaEventRecord(ws.ev[kEvents - 1], s));
        }
        GST_CUDA(cudaMemcpyAsync(ws.h_ctl, ws.ctl, sizeof(GrowCtl), cudaMemcpyDeviceToHost, s));
        GST_CUDA(cudaStreamSynchronize(s));
        if (trace) {
          std::fprintf(stderr, "gst-trace wave %d round %d changed %d  %.3f ms", l, ws.h_ctl->round - 1,
                       ws.h_ctl->last_changed, elapsed(ws.ev[kEvents - 2], ws.ev[kEvents - 1]));
          if (ws.h_params->stats_on) {  // this round's share of the counters
            static long long prev[kNumStats];
            long long cur[kNumStats];
            GST_CUDA(cudaMemcpy(cur, ws.stats, sizeof(cur), cudaMemcpyDeviceToHost));
            if (ws.h_ctl->round == 1) std::fill(prev, prev + kNumStats, 0LL);
            std::fprintf(stderr, "  vertices %lld entries %lld rows %lld improved %lld", cur[kStatVertices] - prev[kStatVertices],
                         cur[kStatEntries] - prev[kStatEntries], cur[kStatRows] - prev[kStatRows],
                         cur[kStatImproved] - prev[kStatImproved]);
            std::copy(cur, cur + kNumStats, prev);
          }
          std::fprintf(stderr, "\n");
        }
        if (ws.h_ctl->timeout) {
          *timeout = true;
          return GST_OK;
        }
        if (ws.h_ctl->last_changed == 0) break;
      }
      if (l < k - 1) {  // not after the last grown wave (see build_query_graph)
        GST_CUDA(launch_ub_refine(gd, a, g->num_sms, s));
        ++*launches;
      }
    }
    GST_CUDA(cudaEventRecord(ws.ev[3 * l + 2], s));
  }
  GST_CUDA(cudaEventRecord(ws.ev[1], s));
  return enqueue_epilogue(g, k, s, launches);
}

// The per-query scalars of g's workspace (pinned host copy) for a solve of
// k groups under options o.
void fill_params(gst_graph* g, int32_t k, const gst_opts& o) {
  Workspace& ws = g->ws;
  ws.h_params->ub = o.upper_bound > 0 ? o.upper_bound : 0;
  ws.h_params->max_rounds = (int32_t)std::min<int64_t>(o.max_rounds > 0 ? o.max_rounds : (int64_t)g->V + 1, INT32_MAX);
  ws.h_params->stats_on = o.collect_stats ? 1 : 0;
  ws.h_params->k = k;
  ws.h_params->ovf_limit = kInf - std::max<int32_t>(g->max_w, 1);
  const gst_graph* tg = g->parent ? g->parent : g;
  const int32_t tuned = tg->tuned_shift[k];
  // default threshold: V/2 unpruned; V/4 when the solve prunes (fewer rows
  // change per round, so sparse rounds stay cheaper for longer)
  const bool pruned = o.refine_bound != 0 || o.upper_bound > 0;
  ws.h_params->dense_shift = o.dense_shift > 0 && o.dense_shift < 31 ? o.dense_shift
                             : tuned > 0                              ? tuned
                             : pruned                                 ? kDefaultDenseShiftPruned
                                                                      : kDefaultDenseShift;
  ws.h_params->refine = o.refine_bound ? 1 : 0;
  ws.h_params->late_bound = 0;
}

// The result of a finished captured solve, from the counters, statistics and
// tree prefix its epilogue copied to g's pinned host buffers.
gst_status finish_solve(gst_graph* g, int32_t k, gst_result* r) {
  Workspace& ws = g->ws;
  const Counters& c = *ws.h_ctr;
  r->ub = ws.h_params->ub;  // the bound as the last wave saw it (refined on the device)
  r->launches = 1 + k + (k - 1) + std::max(k - 2, 0) + (k <= kTourMaxK ? std::max(k - 2, 0) : 0) +
                (int64_t)c.grow_launches + 2;
  r->states = (int64_t)c.states;
  std::copy(ws.h_stats, ws.h_stats + kNumStats, r->stats);
  if (c.timeout) return fail(GST_TIMEOUT, "growth did not converge within max_rounds");
  if (c.overflow) return fail(GST_OVERFLOW, "a tree cost reached GST_COST_LIMIT");
  if (c.best == ~0ull) {
    r->status = GST_INFEASIBLE;
    r->cost = -1;
    return GST_INFEASIBLE;
  }
  return collect_tree(g, r, (int32_t)(c.best >> 32), (int32_t)(c.best & 0xffffffffull));
}

// Waits for the work queued so far on g->stream; with stop given, returns
// GST_TIMEOUT as soon as (*stop)() holds instead (the queued work still
// runs: the caller orders the context's next use after it).
gst_status wait_or_stop(gst_graph* g, const std::function<bool()>* stop) {
  if (!stop) {
    GST_CUDA(cudaStreamSynchronize(g->stream));
    return GST_OK;
  }
  if (!g->ev_poll) GST_CUDA(cudaEventCreateWithFlags(&g->ev_poll, cudaEventDisableTiming));
  GST_CUDA(cudaEventRecord(g->ev_poll, g->stream));
  for (;;) {
    const cudaError_t e = cudaEventQuery(g->ev_poll);
    if (e == cudaSuccess) return GST_OK;
    if (e != cudaErrorNotReady) GST_CUDA(e);
    if ((*stop)()) return fail(GST_TIMEOUT, "stopped: the solve it served finished first");
    std::this_thread::yield();
  }
}

// One query. Caller holds g->mu and has validated the groups. With a
// captured graph, `concurrent` (if given) runs on the host right after the
// graph's launch (g->ev_done is recorded behind it), before the wait for
// it; it may lower the bound in the device parameters
// (SolveParams::late_bound is set for it) once g->ev_params, recorded after
// their upload, has completed. With `stop`, the wait for the graph gives up
// once (*stop)() holds (wait_or_stop).
gst_status solve_one(gst_graph* g, const int32_t* group_ptr, const int32_t* members, int32_t k,
                     const gst_opts& o, gst_result* r, const std::function<void()>* concurrent = nullptr,
                     const std::function<bool()>* stop = nullptr) {
  Workspace& ws = g->ws;
  const int64_t nmembers = group_ptr[k];
  gst_status st = ensure_workspace(g, k, nmembers);
  if (st != GST_OK) return st;
  st = ensure_tables(g, k);
  if (st != GST_OK) return st;
  cudaStream_t s = g->stream;
  const bool use_graph = o.use_graph != 0;
  // a non-sticky error left by an unrelated earlier runtime call would
  // otherwise surface at this solve's first kernel-launch check
  cudaGetLastError();
  const bool timed = use_graph && o.collect_stats != 0;
  if (use_graph) {
    st = build_query_graph(g, k, timed);
    if (st != GST_OK) return st;
  }
  fill_params(g, k, o);
  if (concurrent && use_graph) ws.h_params->late_bound = 1;  // the concurrent work may lower the bound mid-solve

  GST_CUDA(cudaEventRecord(ws.ev[0], s));
  GST_CUDA(cudaMemcpyAsync(ws.d_params, ws.h_params, sizeof(SolveParams), cudaMemcpyHostToDevice, s));
  GST_CUDA(cudaMemcpyAsync(ws.d_group_ptr, group_ptr, (size_t)(k + 1) * 4, cudaMemcpyHostToDevice, s));
  if (nmembers)
    GST_CUDA(cudaMemcpyAsync(ws.d_members, members, (size_t)nmembers * 4, cudaMemcpyHostToDevice, s));
  if (concurrent) GST_CUDA(cudaEventRecord(g->ev_params, s));
  int64_t launches = 0;
  bool timeout = false;
  if (use_graph) {
    GST_CUDA(cudaGraphLaunch((timed ? ws.qg_timed[k] : ws.qg[k]).exec, s));
    if (concurrent) {  // host work (and its own stream) while the graph runs
      GST_CUDA(cudaEventRecord(g->ev_done, s));
      (*concurrent)();
    }
  } else {
    st = run_host_loop(g, k, &launches, &timeout);
    if (st != GST_OK) return st;
    if (timeout) {
      GST_CUDA(cudaStreamSynchronize(s));
      r->launches = launches;
      return fail(GST_TIMEOUT, "growth did not converge within max_rounds");
    }
  }
  GST_CUDA(cudaEventRecord(ws.ev[2], s));
  st = wait_or_stop(g, stop);
  if (st != GST_OK) return st;
  const Counters& c = *ws.h_ctr;
  // masks, k merges, a seed per grown wave, a refinement per grown wave but
  // the last, the tour tables (k <= kTourMaxK, waves 2..k-1), the growth
  // kernels (each launch counts itself on the device), argmin and backtrack
  if (use_graph)
    launches = 1 + k + (k - 1) + std::max(k - 2, 0) + (k <= kTourMaxK ? std::max(k - 2, 0) : 0) +
               (int64_t)c.grow_launches + 2;
  r->ub = ws.h_params->ub;  // the bound as the last wave saw it (refined on the device)
  r->launches = launches;
  r->states = (int64_t)c.states;
  std::copy(ws.h_stats, ws.h_stats + kNumStats, r->stats);
  r->ms[0] = elapsed(ws.ev[0], ws.ev[2]);
  double merge_ms = 0, grow_ms = 0;
  if (!use_graph || timed) {  // the per-wave events ran in this solve
    for (int32_t l = 1; l <= k; ++l) {
      merge_ms += elapsed(ws.ev[3 * l], ws.ev[3 * l + 1]);
      if (l < k) grow_ms += elapsed(ws.ev[3 * l + 1], ws.ev[3 * l + 2]);
    }
    r->ms[3] = elapsed(ws.ev[1], ws.ev[2]);
  }
  r->ms[1] = grow_ms;
  r->ms[2] = merge_ms;
  if (c.timeout) return fail(GST_TIMEOUT, "growth did not converge within max_rounds");
  if (c.overflow) return fail(GST_OVERFLOW, "a tree cost reached GST_COST_LIMIT");
  if (c.best == ~0ull) {
    r->status = GST_INFEASIBLE;
    r->cost = -1;
    return GST_INFEASIBLE;
  }
  const int32_t cost = (int32_t)(c.best >> 32);
  const int32_t root = (int32_t)(c.best & 0xffffffffull);
  return collect_tree(g, r, cost, root);
}

gst_opts resolve_opts(const gst_opts* opts) {
  gst_opts o;
  std::memset(&o, 0, sizeof(o));
  o.struct_size = sizeof(o);
  if (opts) {
    const size_t n = std::min<size_t>(sizeof(o), opts->struct_size > 0 ? (size_t)opts->struct_size : sizeof(o));
    std::memcpy(&o, opts, n);
  }
  return o;
}


// ------------------------------------------------------- learned proposal --
struct TreeEdge {
  int32_t u, v, w;  // u < v, internal IDs
  bool operator<(const TreeEdge& o) const { return u != o.u ? u < o.u : (v != o.v ? v < o.v : w < o.w); }
};

struct HostTree {
  bool ok = false;
  int64_t cost = 0;
  std::vector<int32_t> vertices;  // internal IDs, sorted
  std::vector<TreeEdge> edges;
};

// MST of the subgraph induced by `set` (internal IDs), kept to the
// component of `root`, then leaves removed while every group keeps a
// member in the tree. ok = the result covers all k groups.
HostTree mst_repair(gst_graph* g, std::vector<int32_t> set, int32_t root,
                    const std::unordered_map<int32_t, uint32_t>& gbits, int32_t k) {
  HostTree out;
  std::sort(set.begin(), set.end());
  set.erase(std::unique(set.begin(), set.end()), set.end());
  const size_t n = set.size();
  auto idx = [&](int32_t v) -> int64_t {
    auto it = std::lower_bound(set.begin(), set.end(), v);
    return (it != set.end() && *it == v) ? it - set.begin() : -1;
  };
  // slot + 1 of every set vertex in a V-sized scratch array (zero outside)
  std::vector<int32_t>& slot = g->h_slot;
  if (slot.size() != (size_t)g->V) slot.assign((size_t)g->V, 0);
  const gst_graph* hg = g->parent ? g->parent : g;  // lanes share their graph's host CSR
  for (size_t i = 0; i < n; ++i) slot[(size_t)set[i]] = (int32_t)i + 1;
  std::vector<std::pair<int32_t, std::pair<int32_t, int32_t>>> ind;  // (w, (i, j))
  for (size_t i = 0; i < n; ++i) {
    const int32_t v = set[i];
    for (int32_t e = hg->h_row[(size_t)v]; e < hg->h_row[(size_t)v + 1]; ++e) {
      const int2 x = hg->h_adj[(size_t)e];
      if (x.x <= v) continue;
      const int32_t j = slot[(size_t)x.x] - 1;
      if (j >= 0) ind.push_back({x.y, {(int32_t)i, j}});
    }
  }
  for (size_t i = 0; i < n; ++i) slot[(size_t)set[i]] = 0;
  std::sort(ind.begin(), ind.end());
  std::vector<int32_t> dsu(n);
  for (size_t i = 0; i < n; ++i) dsu[i] = (int32_t)i;
  auto find = [&](int32_t a) {
    while (dsu[(size_t)a] != a) {
      dsu[(size_t)a] = dsu[(size_t)dsu[(size_t)a]];
      a = dsu[(size_t)a];
    }
    return a;
  };
  std::vector<std::vector<std::pair<int32_t, int32_t>>> adj(n);  // (neighbour, w)
  for (auto& e : ind) {
    const int32_t a = find(e.second.first), b = find(e.second.second);
    if (a == b) continue;
    dsu[(size_t)a] = b;
    adj[(size_t)e.second.first].push_back({e.second.second, e.first});
    adj[(size_t)e.second.second].push_back({e.second.first, e.first});
  }
  if (n == 0) return out;
  int64_t ri = idx(root);
  if (ri < 0) ri = 0;  // the root was pruned by an earlier repair: any vertex's component
  const int32_t rc = find((int32_t)ri);
  std::vector<char> alive(n, 0);
  std::vector<uint32_t> bits(n, 0u);
  std::vector<int32_t> cover((size_t)k, 0), deg(n, 0);
  size_t left = 0;
  for (size_t i = 0; i < n; ++i) {
    if (find((int32_t)i) != rc) continue;
    alive[i] = 1;
    ++left;
    auto it = gbits.find(set[i]);
    bits[i] = it == gbits.end() ? 0u : it->second;
    for (int32_t gi = 0; gi < k; ++gi) cover[(size_t)gi] += (bits[i] >> gi) & 1u;
    deg[i] = (int32_t)adj[i].size();
  }
  for (int32_t gi = 0; gi < k; ++gi)
    if (cover[(size_t)gi] == 0) return out;  // the component misses a group
  std::vector<size_t> stack;
  for (size_t i = 0; i < n; ++i)
    if (alive[i] && deg[i] <= 1) stack.push_back(i);
  while (!stack.empty() && left > 1) {
    const size_t i = stack.back();
    stack.pop_back();
    if (!alive[i] || deg[i] > 1) continue;
    bool needed = false;
    for (int32_t gi = 0; gi < k; ++gi)
      if (((bits[i] >> gi) & 1u) && cover[(size_t)gi] <= 1) needed = true;
    if (needed) continue;
    alive[i] = 0;
    --left;
    for (int32_t gi = 0; gi < k; ++gi) cover[(size_t)gi] -= (bits[i] >> gi) & 1u;
    for (auto& nb : adj[i])
      if (alive[(size_t)nb.first] && --deg[(size_t)nb.first] <= 1) stack.push_back((size_t)nb.first);
  }
  for (size_t i = 0; i < n; ++i) {
    if (!alive[i]) continue;
    out.vertices.push_back(set[i]);
    for (auto& nb : adj[i])
      if ((size_t)nb.first > i && alive[(size_t)nb.first]) {
        out.cost += nb.second;
        out.edges.push_back({set[i], set[(size_t)nb.first], nb.second});
      }
  }
  out.ok = true;
  return out;
}

gst_status alloc_learn_infer(gst_graph* g) {
  LearnWs& lw = g->lw;
  const size_t V = (size_t)g->V;
  lw.V = g->V;
  GST_CUDA(cudaMalloc(&lw.r1, V * 4));
  GST_CUDA(cudaMalloc(&lw.r2, V * 4));
  GST_CUDA(cudaMalloc(&lw.r3, V * 4));
  GST_CUDA(cudaMalloc(&lw.mnb, V * 4));
  GST_CUDA(cudaMalloc(&lw.x, V * kFeat * sizeof(float)));
  GST_CUDA(cudaMalloc(&lw.hb[0], V * kHid * sizeof(__nv_bfloat16)));
  GST_CUDA(cudaMalloc(&lw.hb[1], V * kHid * sizeof(__nv_bfloat16)));
  GST_CUDA(cudaMalloc(&lw.hb[2], V * kHid * sizeof(__nv_bfloat16)));
  for (int i = 0; i < 3; ++i) GST_CUDA(make_act_map(lw.hb[i], g->V, &lw.hb_map[i]));
  GST_CUDA(cudaMalloc(&lw.hub_sum, std::max<size_t>(1, (size_t)g->nbig) * kHid * sizeof(float)));
  GST_CUDA(cudaMalloc(&lw.scores, V * sizeof(float)));
  GST_CUDA(cudaMalloc(&lw.best, sizeof(unsigned long long)));
  GST_CUDA(cudaMalloc(&lw.hist, kScoreBins * sizeof(uint32_t)));
  lw.top_cap = 1 << 16;
  GST_CUDA(cudaMalloc(&lw.top, (size_t)lw.top_cap * sizeof(uint2)));
  lw.pe_cap = (int32_t)std::min<int64_t>((int64_t)GST_MAX_K * (g->V + 1), 1 << 22);
  GST_CUDA(cudaMalloc(&lw.pe, (size_t)lw.pe_cap * sizeof(int3)));
  GST_CUDA(cudaMalloc(&lw.pn, 4 * sizeof(int32_t)));
  GST_CUDA(cudaMalloc(&lw.infer_err, sizeof(int32_t)));
  GST_CUDA(cudaMemset(lw.infer_err, 0, sizeof(int32_t)));
  return GST_OK;
}

// The inference workspace, allocated on first use; infer_err is the last
// allocation, so a workspace with it is complete (a failed allocation frees
// what it made).
gst_status ensure_learn_infer(gst_graph* g) {
  if (g->lw.infer_err) return GST_OK;
  const gst_status st = alloc_learn_infer(g);
  if (st != GST_OK) free_learn(g->lw);
  return st;
}

gst_status ensure_learn_train(gst_graph* g, int32_t nids) {
  LearnWs& lw = g->lw;
  const size_t V = (size_t)g->V;
  if (!lw.h[0]) {
    const size_t act = V * kHid * sizeof(float);
    for (auto& p : lw.h) GST_CUDA(cudaMalloc(&p, act));
    for (int l = 1; l <= kMpLayers; ++l) GST_CUDA(cudaMalloc(&lw.a[l], act));
    GST_CUDA(cudaMalloc(&lw.dz, act));
    GST_CUDA(cudaMalloc(&lw.dzp, act));
    GST_CUDA(cudaMalloc(&lw.t, act));
    GST_CUDA(cudaMalloc(&lw.u, act));
    GST_CUDA(cudaMalloc(&lw.s, V * sizeof(float)));
    GST_CUDA(cudaMalloc(&lw.ds, V * sizeof(float)));
    GST_CUDA(cudaMalloc(&lw.label, V));
    GST_CUDA(cudaMalloc(&lw.red, 4 * sizeof(float)));
    GST_CUDA(cudaMalloc(&lw.grad, kNumParams * sizeof(float)));
  }
  if (nids > lw.ids_cap) {
    dfree(lw.ids);
    lw.ids_cap = 0;
    GST_CUDA(cudaMalloc(&lw.ids, (size_t)std::max(nids, 1024) * sizeof(int32_t)));
    lw.ids_cap = std::max(nids, 1024);
  }
  return GST_OK;
}

// Group masks of a query into ws.gmask (internal IDs).
gst_status upload_groups(gst_graph* g, const int32_t* group_ptr, const int32_t* members, int32_t k) {
  Workspace& ws = g->ws;
  const int64_t nmembers = group_ptr[k];
  // the group masks and member lists; the table is only the proposal's
  // two-group distance solve's (a serving lane proposing beside a solve of
  // k groups holds no k-group table)
  gst_status st = ensure_workspace(g, 2, nmembers);
  if (st != GST_OK) return st;
  cudaStream_t s = g->stream;
  GST_CUDA(cudaMemcpyAsync(ws.d_group_ptr, group_ptr, (size_t)(k + 1) * 4, cudaMemcpyHostToDevice, s));
  if (nmembers)
    GST_CUDA(cudaMemcpyAsync(ws.d_members, members, (size_t)nmembers * 4, cudaMemcpyHostToDevice, s));
  GST_CUDA(cudaMemsetAsync(ws.gmask, 0, (size_t)g->V * sizeof(uint32_t), s));
  GST_CUDA(launch_group_masks(ws.d_group_ptr, ws.d_members, g->d_perm, k, ws.gmask, s));
  return GST_OK;
}

// Query features into lw.x (after upload_groups).
gst_status compute_features(gst_graph* g, int32_t k) {
  LearnWs& lw = g->lw;
  const GraphDev gd = graph_dev(g);
  cudaStream_t s = g->stream;
  GST_CUDA(launch_reach(gd, g->d_hub_of, g->ws.gmask, lw.r1, lw.mnb, s));
  GST_CUDA(launch_reach(gd, g->d_hub_of, lw.r1, lw.r2, nullptr, s));
  GST_CUDA(launch_reach(gd, g->d_hub_of, lw.r2, lw.r3, nullptr, s));
  GST_CUDA(launch_features(gd, g->ws.gmask, lw.r1, lw.r2, lw.r3, lw.mnb, k, lw.x, s));
  return GST_OK;
}

// bf16 inference: scores into lw.scores.
gst_status infer_scores(gst_graph* g, const gst_scorer* sc, const std::function<bool()>* stop = nullptr) {
  LearnWs& lw = g->lw;
  const GraphDev gd = graph_dev(g);
  cudaStream_t s = g->stream;
  GST_CUDA(launch_infer_l0(g->V, lw.x, sc->params, lw.hb[0], s));
  for (int l = 1; l <= kMpLayers; ++l) {
    const __nv_bfloat16* hin = lw.hb[(l - 1) & 1];
    if (g->nbig > 0) {
      GST_CUDA(cudaMemsetAsync(lw.hub_sum, 0, (size_t)g->nbig * kHid * sizeof(float), s));
      GST_CUDA(launch_hub_sum_bf16(gd, hin, lw.hub_sum, s));
    }
    const bool last = l == kMpLayers;
    GST_CUDA(launch_infer_layer(gd, g->d_hub_of, lw.hub_sum, hin, lw.hb_map[(l - 1) & 1], lw.hb[2], lw.hb_map[2],
                                sc->wcat + (size_t)(l - 1) * kHid * 2 * kHid, sc->params, l,
                                last ? nullptr : lw.hb[l & 1], last ? lw.scores : nullptr, lw.infer_err, s));
    if (stop && !last) {  // beside a solve: give up between layers once it finished
      const gst_status st = wait_or_stop(g, stop);
      if (st != GST_OK) return st;
    }
  }
  int32_t err = 0;
  GST_CUDA(cudaMemcpyAsync(&err, lw.infer_err, sizeof(err), cudaMemcpyDeviceToHost, s));
  const gst_status wst = wait_or_stop(g, stop);
  if (wst != GST_OK) return wst;
  if (err) {
    GST_CUDA(cudaMemsetAsync(lw.infer_err, 0, sizeof(int32_t), s));
    return fail(GST_INTERNAL, err == 1 ? "scorer layer: a TMA load did not complete" : "scorer layer: an MMA did not complete");
  }
  return GST_OK;
}

// fp32 forward: activations into lw.h / lw.a, scores into lw.s.
gst_status train_forward(gst_graph* g, const gst_scorer* sc) {
  LearnWs& lw = g->lw;
  const GraphDev gd = graph_dev(g);
  cudaStream_t s = g->stream;
  const int32_t V = g->V;
  const float* p = sc->params;
  GST_CUDA(launch_dense_fwd(V, lw.x, kFeat, p + kOffW0, nullptr, nullptr, p + kOffB0, lw.h[0], s));
  for (int l = 1; l <= kMpLayers; ++l) {
    const float* L = p + layer_off(l);
    GST_CUDA(launch_mean_agg(gd, lw.h[l - 1], lw.a[l], s));
    GST_CUDA(launch_dense_fwd(V, lw.h[l - 1], kHid, L, lw.a[l], L + kHid * kHid, L + 2 * kHid * kHid, lw.h[l], s));
  }
  GST_CUDA(launch_score(V, lw.h[kMpLayers], p, lw.s, s));
  return GST_OK;
}

// Gradient of the listwise loss into lw.grad (after train_forward and the labels).
gst_status train_backward(gst_graph* g, const gst_scorer* sc, int32_t n) {
  LearnWs& lw = g->lw;
  const GraphDev gd = graph_dev(g);
  cudaStream_t s = g->stream;
  const int32_t V = g->V;
  const float* p = sc->params;
  GST_CUDA(cudaMemsetAsync(lw.grad, 0, kNumParams * sizeof(float), s));
  GST_CUDA(cudaMemsetAsync(lw.red + 2, 0, sizeof(float), s));
  GST_CUDA(launch_softmax_loss(V, lw.s, lw.label, n, lw.ds, lw.red + 2, lw.red, s));
  GST_CUDA(launch_out_bwd(V, lw.ds, lw.h[kMpLayers], p, lw.grad, lw.dz, s));
  for (int l = kMpLayers; l >= 1; --l) {
    const float* L = p + layer_off(l);
    float* G = lw.grad + layer_off(l);
    GST_CUDA(launch_dense_bwd_weight(V, lw.dz, lw.h[l - 1], kHid, G, G + 2 * kHid * kHid, s));
    GST_CUDA(launch_dense_bwd_weight(V, lw.dz, lw.a[l], kHid, G + kHid * kHid, nullptr, s));
    GST_CUDA(launch_dense_bwd_data(V, lw.dz, L + kHid * kHid, lw.t, s));  // through Wn, then the aggregation
    GST_CUDA(launch_dense_bwd_data(V, lw.dz, L, lw.u, s));                // through Ws
    GST_CUDA(launch_agg_bwd(gd, lw.t, lw.u, lw.h[l - 1], lw.dzp, s));
    std::swap(lw.dz, lw.dzp);
  }
  GST_CUDA(launch_dense_bwd_weight(V, lw.dz, lw.x, kFeat, lw.grad + kOffW0, lw.grad + kOffB0, s));
  return GST_OK;
}

// A feasible tree of the query rooted at the top-scored vertex (or the
// fixed feature score with sc NULL), written into r (caller IDs). With
// stop, every wait gives up (GST_TIMEOUT) once (*stop)() holds: the
// proposal is no longer needed, and its queued work still runs. With dp,
// the captured solve of the same query running on dp's stream, the paths
// to the groups come from that solve's wave 1 (after its ev_wave1) instead
// of a two-group solve of the proposal's own.
gst_status propose_tree(gst_graph* g, const gst_scorer* sc, const int32_t* group_ptr, const int32_t* members,
                        int32_t k, const gst_opts& o, gst_result* r, const std::function<bool()>* stop = nullptr,
                        const gst_graph* dp = nullptr) {
  LearnWs& lw = g->lw;
  Workspace& ws = g->ws;
  cudaStream_t s = g->stream;
  // GST_TRACE=1: report the proposal's phases (host wall clock, synchronising)
  static const bool trace = std::getenv("GST_TRACE") != nullptr;
  auto tp = std::chrono::steady_clock::now();
  auto phase = [&](const char* name) {
    if (!trace) return;
    cudaStreamSynchronize(s);
    const auto now = std::chrono::steady_clock::now();
    std::fprintf(stderr, "gst-trace proposal %s %.3f ms\n", name,
                 std::chrono::duration<double, std::milli>(now - tp).count());
    tp = now;
  };
  gst_status st = ensure_learn_infer(g);
  if (st != GST_OK) return st;
  // beside a solve, the device work starts once the solve's wave 1 has
  // grown: its dense rounds are the solve's most bandwidth-bound part, and
  // the paths below read wave 1 anyway
  if (dp) GST_CUDA(cudaStreamWaitEvent(s, dp->ws.ev_wave1, 0));
  st = upload_groups(g, group_ptr, members, k);
  if (st != GST_OK) return st;
  st = compute_features(g, k);
  if (st != GST_OK) return st;
  phase("features");
  int64_t launches = 5;  // group masks, three reach passes, features
  if (sc) {
    st = infer_scores(g, sc, stop);
    if (st != GST_OK) return st;
    launches += 1 + kMpLayers * (g->nbig > 0 ? 3 : 2);
  } else {
    GST_CUDA(launch_feature_score(g->V, lw.x, lw.scores, s));
    launches += 1;
  }
  launches += 3;  // argmax, histogram, selection
  phase("scores");
  GST_CUDA(cudaMemsetAsync(lw.best, 0, sizeof(unsigned long long), s));
  GST_CUDA(launch_argmax(g->V, lw.scores, lw.best, s));
  GST_CUDA(cudaMemsetAsync(lw.hist, 0, kScoreBins * sizeof(uint32_t), s));
  GST_CUDA(launch_score_hist(g->V, lw.scores, lw.hist, s));
  unsigned long long best = 0;
  std::vector<uint32_t> hist(kScoreBins);
  GST_CUDA(cudaMemcpyAsync(&best, lw.best, sizeof(best), cudaMemcpyDeviceToHost, s));
  GST_CUDA(cudaMemcpyAsync(hist.data(), lw.hist, kScoreBins * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  st = wait_or_stop(g, stop);
  if (st != GST_OK) return st;
  if (best == 0) return fail(GST_INTERNAL, "no vertex scored");
  const int32_t root = (int32_t)(0xffffffffull - (best & 0xffffffffull));
  // the kProposeTop top-scored vertices: the lowest histogram bin that
  // holds them, then the vertices of that bin and above, sorted on the host
  uint32_t bin_lo = kScoreBins - 1;
  for (uint32_t acc = 0;; --bin_lo) {
    acc += hist[bin_lo];
    if (acc >= (uint32_t)kProposeTop || bin_lo == 0) break;
  }
  GST_CUDA(cudaMemsetAsync(lw.pn + 3, 0, sizeof(int32_t), s));
  GST_CUDA(launch_score_select(g->V, lw.scores, bin_lo, lw.top, lw.pn + 3, lw.top_cap, s));
  int32_t ntop = 0;
  GST_CUDA(cudaMemcpyAsync(&ntop, lw.pn + 3, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  st = wait_or_stop(g, stop);
  if (st != GST_OK) return st;
  ntop = std::min(ntop, lw.top_cap);
  std::vector<uint2> cand((size_t)ntop);
  if (ntop) {
    GST_CUDA(cudaMemcpyAsync(cand.data(), lw.top, cand.size() * sizeof(uint2), cudaMemcpyDeviceToHost, s));
    st = wait_or_stop(g, stop);
    if (st != GST_OK) return st;
  }
  std::sort(cand.begin(), cand.end(), [](const uint2& a, const uint2& b) { return a.x != b.x ? a.x > b.x : a.y < b.y; });
  std::vector<int32_t> top;
  for (size_t i = 0; i < cand.size() && (int)i < kProposeTop; ++i) top.push_back((int32_t)cand[i].y);
  phase("top");
  if (dp) {
    // the root's paths over the running solve's wave 1 (complete: the
    // stream waited for it above): exact distances from every vertex to
    // every group, grown before its later waves
    GST_CUDA(cudaMemsetAsync(lw.pn, 0, 4 * sizeof(int32_t), s));
    GST_CUDA(launch_root_paths(graph_dev(g), dp->ws.cost, dp->ws.par, dp->ws.h_lvl_stride[1], ws.gmask, root, k,
                               lw.pe, lw.pn, lw.pe_cap, s));
    launches += 1;
  } else {
    // distances to the root: a two-group solve whose groups are both {root}
    // grows wave 1 to the full shortest-path fixpoint from the root (a
    // one-group solve would stop after its only, last, wave's merge); the
    // row of wave 1 has stride 4 either way
    const int32_t gp1[3] = {0, 1, 2};
    const int32_t mem1[2] = {g->inv[(size_t)root], g->inv[(size_t)root]};
    // The growth is capped at kProposeRounds rounds: every finite distance
    // is the length of an actual path even before the fixpoint, so the tree
    // stays feasible; a group still out of reach drops the proposal.
    gst_opts o1 = o;
    o1.upper_bound = 0;
    o1.refine_bound = 0;
    o1.max_rounds = kProposeRounds;
    gst_result tmp;
    st = solve_one(g, gp1, mem1, 2, o1, &tmp, nullptr, stop);
    if (st == GST_TIMEOUT && stop && (*stop)()) return st;  // stopped, not out of rounds
    if (st == GST_TIMEOUT) {  // the capped rounds ran out: the distances so far are actual paths
      st = GST_OK;
      g_last_error.clear();
    }
    if (st != GST_OK) return st;
    launches += tmp.launches + 1;  // + the path walk
    phase("root distances");
    // nearest member of every group and its path to the root
    const int64_t nmembers = group_ptr[k];
    GST_CUDA(cudaMemcpyAsync(ws.d_group_ptr, group_ptr, (size_t)(k + 1) * 4, cudaMemcpyHostToDevice, s));
    if (nmembers)
      GST_CUDA(cudaMemcpyAsync(ws.d_members, members, (size_t)nmembers * 4, cudaMemcpyHostToDevice, s));
    GST_CUDA(cudaMemsetAsync(lw.pn, 0, 4 * sizeof(int32_t), s));
    GST_CUDA(launch_ub_paths(graph_dev(g), ws.cost, ws.par, ws.h_lvl_stride[1], ws.d_group_ptr, ws.d_members,
                             g->d_perm, k, lw.pe, lw.pn, lw.pe_cap, s));
  }
  int32_t pn[4];
  GST_CUDA(cudaMemcpyAsync(pn, lw.pn, sizeof(pn), cudaMemcpyDeviceToHost, s));
  st = wait_or_stop(g, stop);
  if (st != GST_OK) return st;
  if (pn[2]) return fail(GST_INFEASIBLE, "a group cannot reach the proposal's root");
  if (pn[1] || pn[0] > lw.pe_cap) return fail(GST_INTERNAL, "proposal path walk failed");
  std::vector<int3> pe((size_t)pn[0]);
  if (pn[0]) {
    GST_CUDA(cudaMemcpyAsync(pe.data(), lw.pe, pe.size() * sizeof(int3), cudaMemcpyDeviceToHost, s));
    GST_CUDA(cudaStreamSynchronize(s));
  }
  phase("paths");

  // union of the paths (a subtree of the shortest-path tree)
  std::vector<int32_t> tv{root};
  std::vector<TreeEdge> te;
  for (const int3& e : pe) {
    tv.push_back(e.x);
    tv.push_back(e.y);
    te.push_back({std::min(e.x, e.y), std::max(e.x, e.y), e.z});
  }
  std::sort(tv.begin(), tv.end());
  tv.erase(std::unique(tv.begin(), tv.end()), tv.end());
  std::sort(te.begin(), te.end());
  te.erase(std::unique(te.begin(), te.end(), [](const TreeEdge& a, const TreeEdge& b) { return a.u == b.u && a.v == b.v; }),
           te.end());
  HostTree pick;
  pick.vertices = tv;
  pick.edges = te;
  pick.cost = 0;
  for (auto& e : te) pick.cost += e.w;

  // repairs: an MST of the subgraph induced by a vertex set, restricted to
  // the root's component, with non-essential leaves removed; tried on the
  // path union, on the path union plus the top-scored vertices, and again
  // on each result's own vertices
  std::unordered_map<int32_t, uint32_t> gbits;
  for (int32_t gi = 0; gi < k; ++gi)
    for (int32_t i = group_ptr[gi]; i < group_ptr[gi + 1]; ++i) gbits[g->perm[(size_t)members[i]]] |= 1u << gi;
  std::vector<int32_t> with_top = tv;
  with_top.insert(with_top.end(), top.begin(), top.end());
  for (const std::vector<int32_t>* set : {&tv, &with_top}) {
    HostTree t = mst_repair(g, *set, root, gbits, k);
    for (int pass = 0; pass < 2 && t.ok; ++pass) {
      if (t.cost < pick.cost) pick = t;
      HostTree t2 = mst_repair(g, t.vertices, root, gbits, k);
      if (!t2.ok || t2.cost >= t.cost) break;
      t = std::move(t2);
    }
    if (t.ok && t.cost < pick.cost) pick = t;
  }
  phase("repair");
  r->vertices.clear();
  r->edges.clear();
  for (int32_t v : pick.vertices) r->vertices.push_back(g->inv[(size_t)v]);
  std::sort(r->vertices.begin(), r->vertices.end());
  for (auto& e : pick.edges) {
    const int32_t a = g->inv[(size_t)e.u], b = g->inv[(size_t)e.v];
    r->edges.push_back(std::min(a, b));
    r->edges.push_back(std::max(a, b));
    r->edges.push_back(e.w);
  }
  if (pick.cost >= GST_COST_LIMIT) return fail(GST_OVERFLOW, "proposal cost reached GST_COST_LIMIT");
  r->cost = (int32_t)pick.cost;
  r->root = g->inv[(size_t)root];
  r->launches = launches;
  r->status = GST_OK;
  return GST_OK;
}
// Serving lanes: n extra contexts that share g's device arrays.
gst_status ensure_lanes(gst_graph* g, int32_t n) {
  std::lock_guard<std::mutex> lock(g->mu);
  while ((int32_t)g->lanes.size() < n) {
    auto* l = new (std::nothrow) gst_graph;
    if (!l) return fail(GST_OOM, "host allocation failed");
    l->owns_device = false;
    l->parent = g;
    l->device = g->device;
    l->num_sms = g->num_sms;
    l->V = g->V;
    l->nnz = g->nnz;
    l->d_row_ptr = g->d_row_ptr;
    l->d_adj = g->d_adj;
    l->d_big = g->d_big;
    l->deg_big = g->deg_big;
    l->nbig = g->nbig;
    l->d_order = g->d_order;
    l->d_hub_chunk = g->d_hub_chunk;
    l->d_chunk_vtx = g->d_chunk_vtx;
    l->nchunks = g->nchunks;
    l->d_hub_seg = g->d_hub_seg;
    l->nsegs = g->nsegs;
    l->max_w = g->max_w;
    l->perm = g->perm;
    l->inv = g->inv;
    l->d_perm = g->d_perm;
    l->d_hub_of = g->d_hub_of;
    g->lanes.push_back(l);  // freed with g from here on
    cudaError_t e;
    if ((e = cudaStreamCreateWithFlags(&l->stream, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaStreamCreateWithFlags(&l->side, cudaStreamNonBlocking)) != cudaSuccess)
      return fail(GST_CUDA_ERROR, std::string("lane streams: ") + cudaGetErrorString(e));
  }
  return GST_OK;
}


// Captures every solve context's whole query for k groups (prologue, the
// waves with their growth while-loops, epilogue) as parallel branches of one
// graph: ctx[0] (the graph itself) on its stream, the others forked from it
// and joined back. The branches share nothing but the resident graph, so
// they run concurrently and each ends on its own; one launch and one host
// synchronisation serve the whole chunk.
gst_status build_batch_graph(gst_graph* g, int32_t k, const std::vector<gst_graph*>& ctx, BatchGraph* bg) {
  const size_t q = ctx.size();
  for (cudaEvent_t e : bg->fork) cudaEventDestroy(e);
  for (cudaEvent_t e : bg->join) cudaEventDestroy(e);
  bg->fork.assign(q, nullptr);
  bg->join.assign(q, nullptr);
  for (size_t i = 0; i < q; ++i) {
    GST_CUDA(cudaEventCreateWithFlags(&bg->fork[i], cudaEventDisableTiming));
    GST_CUDA(cudaEventCreateWithFlags(&bg->join[i], cudaEventDisableTiming));
  }
  cudaStream_t s = g->stream;
  GST_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
  gst_status st = GST_OK;
  auto cuda = [&](cudaError_t e, const char* what) {
    if (st == GST_OK && e != cudaSuccess) st = fail(GST_CUDA_ERROR, std::string(what) + ": " + cudaGetErrorString(e));
  };
  for (size_t i = 1; i < q; ++i) {
    cuda(cudaEventRecord(bg->fork[i], s), "batch fork");
    cuda(cudaStreamWaitEvent(ctx[i]->stream, bg->fork[i], 0), "batch fork wait");
  }
  for (size_t i = 0; i < q && st == GST_OK; ++i) {
    gst_graph* c = ctx[i];
    cudaStream_t cs = c->stream;
    int64_t launches = 0;
    st = enqueue_prologue(c, k, cs, &launches);
    for (int32_t l = 1; st == GST_OK && l <= k; ++l) {
      const LevelArgs a = level_args(c, k, l);
      st = enqueue_merge(c, a, cs, &launches);
      if (st == GST_OK && l < k) st = capture_growth_loop(c, a, cs);
      if (st == GST_OK && l < k - 1) cuda(launch_ub_refine(graph_dev(c), a, c->num_sms, cs), "bound refinement launch");
    }
    if (st == GST_OK) st = enqueue_epilogue(c, k, cs, &launches);
  }
  for (size_t i = 1; i < q; ++i) {
    cuda(cudaEventRecord(bg->join[i], ctx[i]->stream), "batch join");
    cuda(cudaStreamWaitEvent(s, bg->join[i], 0), "batch join wait");
  }
  cudaGraph_t graph = nullptr;
  const cudaError_t ee = cudaStreamEndCapture(s, &graph);
  if (st != GST_OK) {
    if (graph) cudaGraphDestroy(graph);
    return st;
  }
  GST_CUDA(ee);
  cudaGraphExec_t exec = nullptr;
  const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
  if (ie != cudaSuccess) {
    cudaGraphDestroy(graph);
    return fail(GST_CUDA_ERROR, std::string("cudaGraphInstantiate (batch): ") + cudaGetErrorString(ie));
  }
  if (bg->exec) cudaGraphExecDestroy(bg->exec);
  if (bg->graph) cudaGraphDestroy(bg->graph);
  bg->graph = graph;
  bg->exec = exec;
  bg->k = k;
  bg->q = (int32_t)q;
  bg->gens.clear();
  for (gst_graph* c : ctx) bg->gens.push_back(c->ws.gen);
  return GST_OK;
}

// Solves q queries of k groups each (query i on context ctx[i]) with one
// launch of the chunk's batch graph. The caller holds every context's
// mutex and has validated the groups; nmem_cap sizes every member buffer
// alike, so one capture serves later chunks. wall_ms: the chunk's host wall
// time; dev_ms: its device time.
gst_status solve_chunk(gst_graph* g, int32_t k, const std::vector<gst_graph*>& ctx,
                       const std::vector<const int32_t*>& gps, const std::vector<const int32_t*>& mems,
                       int64_t nmem_cap, const gst_opts& o, std::vector<gst_result*>& res, double* dev_ms) {
  const size_t q = ctx.size();
  for (gst_graph* c : ctx) {
    gst_status st = ensure_workspace(c, k, nmem_cap);
    if (st != GST_OK) return st;
    st = ensure_tables(c, k);
    if (st != GST_OK) return st;
  }
  BatchGraph* bg = nullptr;
  for (BatchGraph* b : g->batch_graphs)
    if (b->k == k && b->q == (int32_t)q) bg = b;
  bool fresh = bg && bg->exec && bg->gens.size() == q;
  for (size_t i = 0; fresh && i < q; ++i) fresh = bg->gens[i] == ctx[i]->ws.gen;
  if (!fresh) {
    if (!bg) {
      bg = new (std::nothrow) BatchGraph;
      if (!bg) return fail(GST_OOM, "host allocation failed");
      g->batch_graphs.push_back(bg);
    }
    const gst_status st = build_batch_graph(g, k, ctx, bg);
    if (st != GST_OK) return st;
  }
  cudaStream_t s = g->stream;
  for (size_t i = 0; i < q; ++i) {  // the queries' scalars and groups, ahead of the launch on the same stream
    Workspace& ws = ctx[i]->ws;
    fill_params(ctx[i], k, o);
    const int64_t nm = gps[i][k];
    GST_CUDA(cudaMemcpyAsync(ws.d_params, ws.h_params, sizeof(SolveParams), cudaMemcpyHostToDevice, s));
    GST_CUDA(cudaMemcpyAsync(ws.d_group_ptr, gps[i], (size_t)(k + 1) * 4, cudaMemcpyHostToDevice, s));
    if (nm) GST_CUDA(cudaMemcpyAsync(ws.d_members, mems[i], (size_t)nm * 4, cudaMemcpyHostToDevice, s));
  }
  Workspace& ws0 = g->ws;
  GST_CUDA(cudaEventRecord(ws0.ev[0], s));
  GST_CUDA(cudaGraphLaunch(bg->exec, s));
  GST_CUDA(cudaEventRecord(ws0.ev[2], s));
  GST_CUDA(cudaStreamSynchronize(s));
  *dev_ms = elapsed(ws0.ev[0], ws0.ev[2]);
  gst_status first = GST_OK;
  for (size_t i = 0; i < q; ++i) {
    g_last_error.clear();
    const gst_status st = finish_solve(ctx[i], k, res[i]);
    res[i]->status = st;
    res[i]->ms[0] = *dev_ms;  // the chunk's device time (its queries ran together)
    if (st != GST_OK && st != GST_INFEASIBLE && first == GST_OK) first = st;
  }
  return first;
}

// gst_solve_batch with batch graphs: the valid queries grouped by k, each
// group in chunks of up to q queries, every chunk one launch of its batch
// graph (solve_chunk) over the graph's context and q - 1 lanes.
gst_status solve_batch_graphs(gst_graph* g, int32_t nq, const int32_t* ks, const std::vector<std::vector<int32_t>>& gps,
                              const std::vector<const int32_t*>& mems, const std::vector<gst_status>& pre,
                              const gst_opts& o, int32_t q, gst_result** out) {
  gst_status st = ensure_lanes(g, q - 1);
  if (st != GST_OK) return st;
  std::vector<gst_graph*> ctx{g};
  for (int32_t i = 0; i + 1 < q; ++i) ctx.push_back(g->lanes[(size_t)i]);
  std::vector<std::unique_lock<std::mutex>> locks;
  for (gst_graph* c : ctx) locks.emplace_back(c->mu);
  int prev = -1;
  cudaGetDevice(&prev);
  if (prev != g->device) cudaSetDevice(g->device);
  cudaGetLastError();
  const auto t0 = std::chrono::steady_clock::now();
  gst_status first = GST_OK;
  std::string first_msg;
  auto note = [&](gst_status s2) {
    if (s2 != GST_OK && s2 != GST_INFEASIBLE && first == GST_OK) {
      first = s2;
      first_msg = g_last_error;
    }
  };
  std::vector<std::vector<int32_t>> by_k(GST_MAX_K + 1);
  for (int32_t i = 0; i < nq; ++i) {
    auto* r = new (std::nothrow) gst_result;
    if (!r) {
      note(fail(GST_OOM, "host allocation failed"));
      continue;
    }
    out[i] = r;
    if (pre[(size_t)i] != GST_OK) {
      r->status = pre[(size_t)i];
      note(fail(pre[(size_t)i], "k out of range in batch"));
      continue;
    }
    bool empty = false;
    g_last_error.clear();
    const gst_status v = validate_groups(g, gps[(size_t)i].data(), mems[(size_t)i], ks[i], &empty);
    if (v != GST_OK || empty) {
      r->status = v != GST_OK ? v : GST_INFEASIBLE;
      note(r->status);
      continue;
    }
    by_k[(size_t)ks[i]].push_back(i);
  }
  for (int32_t k = 1; k <= GST_MAX_K; ++k) {
    const auto& ids = by_k[(size_t)k];
    int64_t nmem = 0;
    for (int32_t i : ids) nmem = std::max<int64_t>(nmem, gps[(size_t)i][(size_t)k]);
    for (size_t c0 = 0; c0 < ids.size(); c0 += (size_t)q) {
      const size_t n = std::min(ids.size() - c0, (size_t)q);
      std::vector<gst_graph*> cc(ctx.begin(), ctx.begin() + (ptrdiff_t)n);
      std::vector<const int32_t*> cg, cm;
      std::vector<gst_result*> cr;
      for (size_t j = 0; j < n; ++j) {
        const int32_t i = ids[c0 + j];
        cg.push_back(gps[(size_t)i].data());
        cm.push_back(mems[(size_t)i]);
        cr.push_back(out[i]);
      }
      const auto ts = std::chrono::steady_clock::now();
      double dev_ms = 0;
      g_last_error.clear();
      const gst_status s2 = solve_chunk(g, k, cc, cg, cm, nmem, o, cr, &dev_ms);
      const auto te = std::chrono::steady_clock::now();
      for (gst_result* r : cr) {
        if (s2 != GST_OK && s2 != GST_INFEASIBLE && r->status == GST_OK && r->cost < 0) r->status = s2;
        r->lat_ms[0] = std::chrono::duration<double, std::milli>(te - ts).count();
        r->lat_ms[1] = std::chrono::duration<double, std::milli>(te - t0).count();
      }
      note(s2);
    }
  }
  if (prev >= 0 && prev != g->device) cudaSetDevice(prev);
  if (first != GST_OK) g_last_error = first_msg;
  return first;
}

}  // namespace

namespace gst {
void set_last_error(const std::string& msg) { g_last_error = msg; }
}  // namespace gst

// ------------------------------------------------------------------ C ABI --
extern "C" {

gst_status gst_graph_upload(const int32_t* row_ptr, const int32_t* col, const int32_t* w, int32_t V, int64_t nnz,
                            gst_graph** out) {
  g_last_error.clear();
  if (!out) return fail(GST_BAD_INPUT, "out is NULL");
  *out = nullptr;
  if (V < 1 || !row_ptr) return fail(GST_BAD_INPUT, "V must be >= 1 and row_ptr non-NULL");
  if (nnz < 0 || nnz >= INT32_MAX) return fail(GST_BAD_INPUT, "nnz must be in [0, 2^31-1)");
  if (nnz > 0 && (!col || !w)) return fail(GST_BAD_INPUT, "col / w is NULL");
  if (row_ptr[0] != 0 || row_ptr[V] != nnz) return fail(GST_BAD_INPUT, "row_ptr[0] must be 0 and row_ptr[V] nnz");
  for (int32_t v = 0; v < V; ++v)
    if (row_ptr[v + 1] < row_ptr[v]) return fail(GST_BAD_INPUT, "row_ptr must be non-decreasing");
  int32_t max_w = 0;
  for (int64_t e = 0; e < nnz; ++e) {
    if (col[e] < 0 || col[e] >= V) return fail(GST_BAD_INPUT, "col entry out of range");
    if (w[e] < 0 || w[e] >= GST_COST_LIMIT) return fail(GST_BAD_INPUT, "weights must be in [0, GST_COST_LIMIT)");
    max_w = std::max(max_w, w[e]);
  }
  auto* g = new (std::nothrow) gst_graph;
  if (!g) return fail(GST_OOM, "host allocation failed");
  g->V = V;
  g->nnz = nnz;
  g->max_w = max_w;
  // Relabelling. Sparse rounds give each warp a tile of kCandTile
  // consecutive IDs, and a lane works through its share of the tile's
  // candidates one vertex at a time, so a tile of high-degree vertices is a
  // long serial tail (generators and real graphs alike tend to give the
  // high-degree vertices neighbouring IDs). Vertices ranked by decreasing
  // degree are cut into runs of kDealRun consecutive ranks, and the runs are
  // dealt out over the tiles round-robin: a tile holds at most a run or two
  // of the heaviest vertices (about one per lane), while the rows of
  // similarly hot vertices stay side by side, sharing cache lines in the
  // dense rounds' neighbour gathers.
  constexpr int64_t kDealRun = 32;
  static_assert(kCandTile % kDealRun == 0, "tiles hold whole runs");
  const int32_t* rp = row_ptr;  // the caller's CSR
  std::vector<int32_t> bydeg((size_t)V);
  for (int32_t v = 0; v < V; ++v) bydeg[(size_t)v] = v;
  std::stable_sort(bydeg.begin(), bydeg.end(),
                   [&](int32_t a, int32_t b) { return rp[a + 1] - rp[a] > rp[b + 1] - rp[b]; });
  g->perm.resize((size_t)V);
  g->inv.resize((size_t)V);
  {
    const int64_t ntiles = ((int64_t)V + kCandTile - 1) / kCandTile;
    size_t r = 0;
    for (int64_t run = 0; run < kCandTile / kDealRun; ++run)
      for (int64_t t = 0; t < ntiles; ++t)
        for (int64_t i = 0; i < kDealRun; ++i) {
          const int64_t id = t * kCandTile + run * kDealRun + i;
          if (id >= V) continue;
          const int32_t old = bydeg[r++];
          g->perm[(size_t)old] = (int32_t)id;
          g->inv[(size_t)id] = old;
        }
  }
  // the CSR in internal IDs, each row's entries in the caller's order
  std::vector<int32_t> nrow((size_t)V + 1);
  std::vector<int2> adj((size_t)nnz);
  nrow[0] = 0;
  for (int32_t n = 0; n < V; ++n) {
    const int32_t o = g->inv[(size_t)n];
    int32_t pos = nrow[(size_t)n];
    for (int32_t e = rp[o]; e < rp[o + 1]; ++e) adj[(size_t)pos++] = make_int2(g->perm[(size_t)col[e]], w[e]);
    nrow[(size_t)n + 1] = pos;
  }
  row_ptr = nrow.data();
  // Growth order of the non-hub vertices: by decreasing degree within
  // windows of kOrderWindow consecutive IDs, so the 32 lanes of a warp walk
  // rows of similar length while a window's rows stay close in memory.
  std::vector<int32_t> big, order;
  g->deg_big = (int32_t)std::min<int64_t>(kDegBigMax, std::max<int64_t>(kDegBigMin, (4 * nnz + V - 1) / V));
  for (int32_t v = 0; v < V; ++v) (row_ptr[v + 1] - row_ptr[v] > g->deg_big ? big : order).push_back(v);
  constexpr size_t kOrderWindow = 1024;
  for (size_t w0 = 0; w0 < order.size(); w0 += kOrderWindow) {
    const size_t w1 = std::min(order.size(), w0 + kOrderWindow);
    std::stable_sort(order.begin() + (ptrdiff_t)w0, order.begin() + (ptrdiff_t)w1, [&](int32_t a, int32_t b) {
      return row_ptr[a + 1] - row_ptr[a] > row_ptr[b + 1] - row_ptr[b];
    });
  }
  g->nbig = (int32_t)big.size();
  std::vector<int32_t> hub_of((size_t)V, -1);
  for (int32_t h = 0; h < g->nbig; ++h) hub_of[(size_t)big[(size_t)h]] = h;
  std::vector<int2> chunks;
  std::vector<int32_t> chunk_vtx;
  for (int32_t h = 0; h < g->nbig; ++h)
    for (int32_t e = row_ptr[big[(size_t)h]]; e < row_ptr[big[(size_t)h] + 1]; e += 32) {
      chunks.push_back(make_int2(h, e));
      chunk_vtx.push_back(big[(size_t)h]);
    }
  g->nchunks = (int64_t)chunks.size();
  std::vector<int4> segs;
  for (int32_t h = 0; h < g->nbig; ++h) {
    const int32_t u = big[(size_t)h], b = row_ptr[u], e = row_ptr[u + 1];
    const int32_t n = (e - b + kHubSeg - 1) / kHubSeg;
    for (int32_t x = b; x < e; x += kHubSeg) segs.push_back(make_int4(u, h, x, n));
  }
  g->nsegs = (int64_t)segs.size();
  auto cleanup = [&](gst_status s) {
    gst_graph_free(g);
    return s;
  };
  cudaError_t e;
  if ((e = cudaGetDevice(&g->device)) != cudaSuccess ||
      (e = cudaDeviceGetAttribute(&g->num_sms, cudaDevAttrMultiProcessorCount, g->device)) != cudaSuccess ||
      (e = cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking)) != cudaSuccess ||
      (e = cudaStreamCreateWithFlags(&g->side, cudaStreamNonBlocking)) != cudaSuccess)
    return cleanup(fail(GST_CUDA_ERROR, std::string("device setup: ") + cudaGetErrorString(e)));
  auto up = [&](void** dst, const void* src, size_t bytes) -> cudaError_t {
    cudaError_t x = cudaMalloc(dst, bytes ? bytes : 4);
    if (x != cudaSuccess || !bytes) return x;
    return cudaMemcpyAsync(*dst, src, bytes, cudaMemcpyHostToDevice, g->stream);
  };
  if ((e = up((void**)&g->d_row_ptr, row_ptr, (size_t)(V + 1) * 4)) != cudaSuccess ||
      (e = up((void**)&g->d_perm, g->perm.data(), (size_t)V * 4)) != cudaSuccess ||
      (e = up((void**)&g->d_hub_of, hub_of.data(), (size_t)V * 4)) != cudaSuccess ||
      (e = up((void**)&g->d_adj, adj.data(), adj.size() * sizeof(int2))) != cudaSuccess ||
      (e = up((void**)&g->d_big, big.data(), big.size() * 4)) != cudaSuccess ||
      (e = up((void**)&g->d_order, order.data(), order.size() * 4)) != cudaSuccess ||
      (e = up((void**)&g->d_hub_chunk, chunks.data(), chunks.size() * sizeof(int2))) != cudaSuccess ||
      (e = up((void**)&g->d_chunk_vtx, chunk_vtx.data(), chunk_vtx.size() * sizeof(int32_t))) != cudaSuccess ||
      (e = up((void**)&g->d_hub_seg, segs.data(), segs.size() * sizeof(int4))) != cudaSuccess ||
      (e = cudaStreamSynchronize(g->stream)) != cudaSuccess)
    return cleanup(fail(e == cudaErrorMemoryAllocation ? GST_OOM : GST_CUDA_ERROR,
                        std::string("graph upload: ") + cudaGetErrorString(e)));
  g->h_row = std::move(nrow);
  g->h_adj = std::move(adj);
  *out = g;
  return GST_OK;
}

void gst_graph_free(gst_graph* g) {
  if (!g) return;
  for (gst_graph* l : g->lanes) gst_graph_free(l);
  g->lanes.clear();
  int prev = -1;
  cudaGetDevice(&prev);
  cudaSetDevice(g->device);
  if (g->stream) cudaStreamSynchronize(g->stream);
  for (BatchGraph* b : g->batch_graphs) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    for (cudaEvent_t e : b->fork) cudaEventDestroy(e);
    for (cudaEvent_t e : b->join) cudaEventDestroy(e);
    delete b;
  }
  g->batch_graphs.clear();
  free_workspace(g->ws);
  free_learn(g->lw);
  if (g->owns_device) {
    dfree(g->d_row_ptr);
    dfree(g->d_perm);
    dfree(g->d_hub_of);
    dfree(g->d_adj);
    dfree(g->d_big);
    dfree(g->d_order);
    dfree(g->d_hub_chunk);
    dfree(g->d_chunk_vtx);
    dfree(g->d_hub_seg);
  }
  if (g->stream) cudaStreamDestroy(g->stream);
  if (g->side) cudaStreamDestroy(g->side);
  for (cudaEvent_t e : {g->ev_params, g->ev_done, g->ev_side, g->ev_poll})
    if (e) cudaEventDestroy(e);
  if (prev >= 0) cudaSetDevice(prev);
  delete g;
}

int32_t gst_graph_num_vertices(const gst_graph* g) { return g ? g->V : 0; }
int64_t gst_graph_num_entries(const gst_graph* g) { return g ? g->nnz : 0; }

gst_status gst_solve(gst_graph* g, const int32_t* group_ptr, const int32_t* members, int32_t k,
                     const gst_opts* opts, gst_result** out) {
  g_last_error.clear();
  if (!out) return fail(GST_BAD_INPUT, "out is NULL");
  *out = nullptr;
  if (!g) return fail(GST_BAD_INPUT, "graph is NULL");
  bool empty_group = false;
  gst_status st = validate_groups(g, group_ptr, members, k, &empty_group);
  if (st != GST_OK) return st;
  auto* r = new (std::nothrow) gst_result;
  if (!r) return fail(GST_OOM, "host allocation failed");
  *out = r;
  if (empty_group) {  // a group without members can never be covered
    r->status = GST_INFEASIBLE;
    return GST_INFEASIBLE;
  }
  const gst_opts o = resolve_opts(opts);
  std::lock_guard<std::mutex> lock(g->mu);
  int prev = -1;
  cudaGetDevice(&prev);
  if (prev != g->device) cudaSetDevice(g->device);
  st = solve_one(g, group_ptr, members, k, o, r);
  if (prev >= 0 && prev != g->device) cudaSetDevice(prev);
  r->status = st;
  return st;
}

gst_status gst_solve_batch(gst_graph* g, int32_t nq, const int32_t* ks, const int32_t* group_ptr,
                           const int32_t* members, const gst_opts* opts, gst_result** out) {
  g_last_error.clear();
  if (!out || !g || nq < 0 || (nq > 0 && (!ks || !group_ptr))) return fail(GST_BAD_INPUT, "bad batch arguments");
  const gst_opts o = resolve_opts(opts);
  // Query q's groups start at ks[0] + ... + ks[q-1], counting queries whose
  // k is out of range too: such a query fails alone (GST_BAD_INPUT in its
  // result) and the later queries keep their own groups. A negative k
  // leaves the layout undefined, so it rejects the whole batch.
  for (int32_t q = 0; q < nq; ++q) {
    out[q] = nullptr;
    if (ks[q] < 0) return fail(GST_BAD_INPUT, "negative k in batch");
  }
  // per-query group arrays, rebased
  std::vector<std::vector<int32_t>> gps((size_t)nq);
  std::vector<const int32_t*> mems((size_t)nq, nullptr);
  std::vector<gst_status> pre((size_t)nq, GST_OK);
  int64_t gbase = 0;
  for (int32_t q = 0; q < nq; ++q) {
    const int64_t b = gbase;
    gbase += ks[q];
    if (ks[q] < 1 || ks[q] > GST_MAX_K) {
      pre[(size_t)q] = GST_BAD_INPUT;
      continue;
    }
    auto& gp = gps[(size_t)q];
    gp.resize((size_t)ks[q] + 1);
    for (int32_t i = 0; i <= ks[q]; ++i) gp[(size_t)i] = group_ptr[b + i] - group_ptr[b];
    mems[(size_t)q] = members ? members + group_ptr[b] : nullptr;
  }
  const int32_t bgq = o.batch_graph >= 2 ? o.batch_graph
                      : (o.batch_graph == 0 && o.concurrency <= 0) ? g->tuned_batch_graph
                                                                   : 0;
  if (bgq >= 2) return solve_batch_graphs(g, nq, ks, gps, mems, pre, o, std::min(bgq, kMaxLanes), out);
  const int32_t want = o.concurrency > 0 ? o.concurrency : (g->tuned_lanes > 0 ? g->tuned_lanes : kDefaultLanes);
  const int32_t nl = std::max(1, std::min({want, nq, kMaxLanes}));
  gst_status st = ensure_lanes(g, nl - 1);
  if (st != GST_OK) return st;
  std::vector<gst_graph*> ctx{g};
  for (int32_t i = 0; i + 1 < nl; ++i) ctx.push_back(g->lanes[(size_t)i]);
  std::atomic<int32_t> next{0};
  std::vector<std::string> errs((size_t)nq);
  const auto t0 = std::chrono::steady_clock::now();
  auto worker = [&](gst_graph* c) {
    cudaSetDevice(c->device);
    std::lock_guard<std::mutex> lock(c->mu);
    for (int32_t q; (q = next.fetch_add(1)) < nq;) {
      auto* r = new (std::nothrow) gst_result;
      if (!r) {
        errs[(size_t)q] = "host allocation failed";
        continue;
      }
      out[q] = r;
      if (pre[(size_t)q] != GST_OK) {  // this query alone fails; its result says so
        r->status = pre[(size_t)q];
        errs[(size_t)q] = "k out of range in batch";
        continue;
      }
      const auto ts = std::chrono::steady_clock::now();
      g_last_error.clear();
      bool empty = false;
      const int32_t k = ks[q];
      gst_status s2 = validate_groups(c, gps[(size_t)q].data(), mems[(size_t)q], k, &empty);
      if (s2 == GST_OK && empty) s2 = GST_INFEASIBLE;
      if (s2 == GST_OK) {
        cudaGetLastError();
        s2 = solve_one(c, gps[(size_t)q].data(), mems[(size_t)q], k, o, r);
      }
      r->status = s2;
      if (s2 != GST_OK && s2 != GST_INFEASIBLE) errs[(size_t)q] = g_last_error;
      const auto te = std::chrono::steady_clock::now();
      r->lat_ms[0] = std::chrono::duration<double, std::milli>(te - ts).count();
      r->lat_ms[1] = std::chrono::duration<double, std::milli>(te - t0).count();
    }
  };
  if (nl == 1) {
    worker(g);
  } else {
    std::vector<std::thread> th;
    for (gst_graph* c : ctx) th.emplace_back(worker, c);
    for (auto& t : th) t.join();
  }
  gst_status first = GST_OK;
  for (int32_t q = 0; q < nq; ++q) {
    const gst_status sq = out[q] ? out[q]->status : pre[(size_t)q] != GST_OK ? pre[(size_t)q] : GST_OOM;
    if (sq != GST_OK && sq != GST_INFEASIBLE && first == GST_OK) {
      first = sq;
      g_last_error = errs[(size_t)q];
    }
  }
  return first;
}

gst_status gst_autotune(gst_graph* g, int32_t nq, const int32_t* ks, const int32_t* group_ptr,
                        const int32_t* members, const gst_opts* opts, int32_t* lanes_out) {
  g_last_error.clear();
  if (!g || nq < 1 || !ks || !group_ptr) return fail(GST_BAD_INPUT, "bad autotune arguments");
  gst_opts o = resolve_opts(opts);
  // 1. dense-round shift per k: up to two sample queries of that k each
  std::vector<int64_t> offs((size_t)nq + 1, 0);
  for (int32_t q = 0; q < nq; ++q) {
    if (ks[q] < 1 || ks[q] > GST_MAX_K) return fail(GST_BAD_INPUT, "k out of range in autotune");
    offs[(size_t)q + 1] = offs[(size_t)q] + ks[q];
  }
  for (int32_t k = 1; k <= GST_MAX_K; ++k) {
    std::vector<int32_t> sample;
    for (int32_t q = 0; q < nq && sample.size() < 2; ++q)
      if (ks[q] == k) sample.push_back(q);
    if (sample.empty()) continue;
    double best_ms = 1e300;
    int32_t best_shift = kDefaultDenseShift;
    for (int32_t shift : {1, 2, 3, 4}) {
      double ms = 0;
      for (int rep = 0; rep < 2; ++rep)  // the first pass also captures the query graphs
        for (int32_t q : sample) {
          std::vector<int32_t> gp((size_t)k + 1);
          for (int32_t i = 0; i <= k; ++i) gp[(size_t)i] = group_ptr[offs[(size_t)q] + i] - group_ptr[offs[(size_t)q]];
          gst_opts oq = o;
          oq.dense_shift = shift;
          gst_result* r = nullptr;
          const gst_status sq = gst_solve(g, gp.data(), members ? members + group_ptr[offs[(size_t)q]] : nullptr, k, &oq, &r);
          if (sq != GST_OK && sq != GST_INFEASIBLE) {
            gst_result_free(r);
            return sq;
          }
          if (rep == 1) ms += r->ms[0];
          gst_result_free(r);
        }
      if (ms < best_ms) {
        best_ms = ms;
        best_shift = shift;
      }
    }
    g->tuned_shift[k] = best_shift;
  }
  // 2. batch execution: the sample as one batch per candidate (concurrent
  // contexts l = 1, 2, 4, 8, or batch graphs of l = -2, -4, -8 queries),
  // wall time
  std::vector<gst_result*> res((size_t)nq, nullptr);
  double best_s = 1e300;
  int32_t best_l = 1;
  for (int32_t l : {1, 2, 4, 8, -2, -4, -8}) {
    if (std::abs(l) > kMaxLanes) continue;
    gst_opts ob = o;
    ob.concurrency = l > 0 ? l : 1;
    ob.batch_graph = l > 0 ? 1 : -l;
    for (int rep = 0; rep < 2; ++rep) {
      const auto t0 = std::chrono::steady_clock::now();
      const gst_status sb = gst_solve_batch(g, nq, ks, group_ptr, members, &ob, res.data());
      const double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      for (auto*& r : res) {
        gst_result_free(r);
        r = nullptr;
      }
      if (sb != GST_OK && sb != GST_INFEASIBLE) return sb;
      if (rep == 1 && sec < best_s) {
        best_s = sec;
        best_l = l;
      }
    }
  }
  g->tuned_lanes = best_l > 0 ? best_l : 0;
  g->tuned_batch_graph = best_l < 0 ? -best_l : 0;
  if (lanes_out) *lanes_out = best_l > 0 ? best_l : -best_l;
  return GST_OK;
}

gst_status gst_get_tuning(const gst_graph* g, gst_tuning* out) {
  g_last_error.clear();
  if (!g || !out) return fail(GST_BAD_INPUT, "null graph or tuning record");
  *out = gst_tuning{};
  for (int k = 0; k <= GST_MAX_K; ++k) out->dense_shift[k] = g->tuned_shift[k];
  out->concurrency = g->tuned_lanes;
  out->batch_graph = g->tuned_batch_graph;
  return GST_OK;
}

gst_status gst_set_tuning(gst_graph* g, const gst_tuning* t) {
  g_last_error.clear();
  if (!g || !t) return fail(GST_BAD_INPUT, "null graph or tuning record");
  for (int k = 0; k <= GST_MAX_K; ++k)
    if (t->dense_shift[k] < 0 || t->dense_shift[k] > 4) return fail(GST_BAD_INPUT, "dense_shift out of range");
  if (t->concurrency < 0 || t->concurrency > kMaxLanes) return fail(GST_BAD_INPUT, "concurrency out of range");
  if (t->batch_graph != 0 && (t->batch_graph < 2 || t->batch_graph > kMaxLanes))
    return fail(GST_BAD_INPUT, "batch_graph out of range");
  for (int k = 0; k <= GST_MAX_K; ++k) g->tuned_shift[k] = t->dense_shift[k];
  g->tuned_lanes = t->concurrency;
  g->tuned_batch_graph = t->batch_graph;
  return GST_OK;
}

struct gst_pool {
  std::vector<gst_graph*> replicas;
};

gst_status gst_pool_create(const int32_t* row_ptr, const int32_t* col, const int32_t* w, int32_t V, int64_t nnz,
                           const int32_t* devices, int32_t num_devices, gst_pool** out) {
  g_last_error.clear();
  if (!out || !devices || num_devices < 1) return fail(GST_BAD_INPUT, "devices / out missing");
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess) return fail(GST_CUDA_ERROR, "cudaGetDeviceCount failed");
  for (int32_t i = 0; i < num_devices; ++i)
    if (devices[i] < 0 || devices[i] >= count) return fail(GST_BAD_INPUT, "device index out of range");
  auto* p = new (std::nothrow) gst_pool;
  if (!p) return fail(GST_OOM, "host allocation failed");
  int prev = -1;
  cudaGetDevice(&prev);
  for (int32_t i = 0; i < num_devices; ++i) {
    cudaSetDevice(devices[i]);
    gst_graph* g = nullptr;
    const gst_status st = gst_graph_upload(row_ptr, col, w, V, nnz, &g);
    if (st != GST_OK) {
      const std::string msg = g_last_error;
      gst_pool_free(p);
      if (prev >= 0) cudaSetDevice(prev);
      return fail(st, "replica " + std::to_string(i) + ": " + msg);
    }
    p->replicas.push_back(g);
  }
  if (prev >= 0) cudaSetDevice(prev);
  *out = p;
  return GST_OK;
}

void gst_pool_free(gst_pool* p) {
  if (!p) return;
  for (gst_graph* g : p->replicas) gst_graph_free(g);
  delete p;
}

int32_t gst_pool_num_replicas(const gst_pool* p) { return p ? (int32_t)p->replicas.size() : 0; }

gst_status gst_pool_solve_batch(gst_pool* p, int32_t nq, const int32_t* ks, const int32_t* group_ptr,
                                const int32_t* members, const gst_opts* opts, gst_result** out) {
  g_last_error.clear();
  if (!p || p->replicas.empty() || !out || nq < 0 || (nq > 0 && (!ks || !group_ptr)))
    return fail(GST_BAD_INPUT, "bad pool batch arguments");
  // where each query's groups start (as gst_solve_batch: a query whose k is
  // out of range fails alone, a negative k rejects the batch)
  std::vector<int64_t> gofs((size_t)nq + 1, 0);
  for (int32_t q = 0; q < nq; ++q) {
    out[q] = nullptr;
    if (ks[q] < 0) return fail(GST_BAD_INPUT, "negative k in batch");
    gofs[(size_t)q + 1] = gofs[(size_t)q] + ks[q];
  }
  const int32_t chunk = std::max(1, std::min(16, nq / (4 * (int32_t)p->replicas.size()) + 1));
  std::atomic<int32_t> next{0};
  std::vector<gst_status> sts(p->replicas.size(), GST_OK);
  std::vector<std::string> errs(p->replicas.size());
  auto worker = [&](size_t ri) {
    gst_graph* g = p->replicas[ri];
    cudaSetDevice(g->device);
    for (int32_t q0; (q0 = next.fetch_add(chunk)) < nq;) {
      const int32_t n = std::min(chunk, nq - q0);
      // the chunk's groups as their own batch (group_ptr rebased to its first group)
      const int64_t g0 = gofs[(size_t)q0], g1 = gofs[(size_t)q0 + n];
      std::vector<int32_t> gp((size_t)(g1 - g0 + 1));
      for (int64_t i = 0; i <= g1 - g0; ++i) gp[(size_t)i] = group_ptr[g0 + i] - group_ptr[g0];
      const gst_status st = gst_solve_batch(g, n, ks + q0, gp.data(), members ? members + group_ptr[g0] : nullptr,
                                            opts, out + q0);
      for (int32_t i = 0; i < n; ++i)
        if (out[q0 + i]) out[q0 + i]->replica = (int32_t)ri;
      if (st != GST_OK && st != GST_INFEASIBLE && sts[ri] == GST_OK) {
        sts[ri] = st;
        errs[ri] = g_last_error;
      }
    }
  };
  std::vector<std::thread> th;
  for (size_t ri = 0; ri < p->replicas.size(); ++ri) th.emplace_back(worker, ri);
  for (auto& t : th) t.join();
  for (size_t ri = 0; ri < sts.size(); ++ri)
    if (sts[ri] != GST_OK) {
      g_last_error = errs[ri];
      return sts[ri];
    }
  return GST_OK;
}

int32_t gst_result_replica(const gst_result* r) { return r ? r->replica : -1; }

void gst_result_latency(const gst_result* r, double* ms2) {
  if (r && ms2) std::copy(r->lat_ms, r->lat_ms + 2, ms2);
}

void gst_result_free(gst_result* r) { delete r; }
gst_status gst_result_status(const gst_result* r) { return r ? r->status : GST_BAD_INPUT; }
int32_t gst_result_cost(const gst_result* r) { return r ? r->cost : -1; }
int32_t gst_result_root(const gst_result* r) { return r ? r->root : -1; }
int32_t gst_result_num_vertices(const gst_result* r) { return r ? (int32_t)r->vertices.size() : 0; }
int32_t gst_result_num_edges(const gst_result* r) { return r ? (int32_t)(r->edges.size() / 3) : 0; }
void gst_result_vertices(const gst_result* r, int32_t* v) {
  if (r && v) std::copy(r->vertices.begin(), r->vertices.end(), v);
}
void gst_result_edges(const gst_result* r, int32_t* e) {
  if (r && e) std::copy(r->edges.begin(), r->edges.end(), e);
}
int64_t gst_result_states(const gst_result* r) { return r ? r->states : 0; }
int64_t gst_result_launches(const gst_result* r) { return r ? r->launches : 0; }
void gst_result_times(const gst_result* r, double* ms4) {
  if (r && ms4) std::copy(r->ms, r->ms + 4, ms4);
}
void gst_result_stats(const gst_result* r, int64_t* s8) {
  if (r && s8) std::copy(r->stats, r->stats + kNumStats, s8);
}

gst_status gst_graph_debug_table(gst_graph* g, int32_t k, int32_t* out) {
  g_last_error.clear();
  if (!g || !out || k < 1 || k > GST_MAX_K) return fail(GST_BAD_INPUT, "bad arguments");
  std::lock_guard<std::mutex> lock(g->mu);
  Workspace& ws = g->ws;
  if (ws.tables_k != k || ws.k_cap < k || !ws.cost) return fail(GST_BAD_INPUT, "no solve with this k on record");
  const int64_t V = g->V;
  const int64_t W = int64_t(1) << k;
  std::vector<int32_t> dev((size_t)(V * total_stride(k)));
  GST_CUDA(cudaMemcpy(dev.data(), ws.cost, dev.size() * sizeof(int32_t), cudaMemcpyDeviceToHost));
  for (int64_t v = 0; v < V; ++v) out[v * W] = kInf;
  for (int l = 1; l <= k; ++l) {
    const int64_t base = (int64_t)ws.h_lvl_base[l] * V;
    const int32_t s = ws.h_lvl_stride[l];
    int32_t rank = 0;
    for (int32_t S = 1; S < (int32_t)W; ++S) {
      if (__builtin_popcount((unsigned)S) != l) continue;
      for (int64_t v = 0; v < V; ++v) out[v * W + S] = dev[(size_t)(base + (int64_t)g->perm[(size_t)v] * s + rank)];
      ++rank;
    }
  }
  return GST_OK;
}

// ------------------------------------------------------ learned proposal --
int64_t gst_scorer_num_params(void) { return kNumParams; }

gst_status gst_scorer_create(const float* params, gst_scorer** out) {
  g_last_error.clear();
  if (!out || !params) return fail(GST_BAD_INPUT, "params / out is NULL");
  *out = nullptr;
  auto* sc = new (std::nothrow) gst_scorer;
  if (!sc) return fail(GST_OOM, "host allocation failed");
  auto bad = [&](cudaError_t e) {
    gst_scorer_free(sc);
    return fail(e == cudaErrorMemoryAllocation ? GST_OOM : GST_CUDA_ERROR,
                std::string("scorer setup: ") + cudaGetErrorString(e));
  };
  cudaError_t e;
  if ((e = cudaGetDevice(&sc->device)) != cudaSuccess) return bad(e);
  const size_t pb = kNumParams * sizeof(float);
  if ((e = cudaMalloc(&sc->params, pb)) != cudaSuccess || (e = cudaMalloc(&sc->m, pb)) != cudaSuccess ||
      (e = cudaMalloc(&sc->v, pb)) != cudaSuccess ||
      (e = cudaMalloc(&sc->wcat, (size_t)kMpLayers * kHid * 2 * kHid * sizeof(__nv_bfloat16))) != cudaSuccess ||
      (e = cudaMemcpy(sc->params, params, pb, cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemset(sc->m, 0, pb)) != cudaSuccess || (e = cudaMemset(sc->v, 0, pb)) != cudaSuccess ||
      (e = launch_pack_bf16(sc->params, sc->wcat, 0)) != cudaSuccess || (e = cudaDeviceSynchronize()) != cudaSuccess)
    return bad(e);
  *out = sc;
  return GST_OK;
}

void gst_scorer_free(gst_scorer* sc) {
  if (!sc) return;
  int prev = -1;
  cudaGetDevice(&prev);
  cudaSetDevice(sc->device);
  dfree(sc->params);
  dfree(sc->wcat);
  dfree(sc->m);
  dfree(sc->v);
  if (prev >= 0) cudaSetDevice(prev);
  delete sc;
}

gst_status gst_scorer_get_params(const gst_scorer* sc, float* out) {
  g_last_error.clear();
  if (!sc || !out) return fail(GST_BAD_INPUT, "bad arguments");
  GST_CUDA(cudaMemcpy(out, sc->params, kNumParams * sizeof(float), cudaMemcpyDeviceToHost));
  return GST_OK;
}

namespace {
// Common checks of the learned entry points; takes the graph's lock.
gst_status learn_enter(gst_graph* g, const int32_t* group_ptr, const int32_t* members, int32_t k) {
  g_last_error.clear();
  if (!g) return fail(GST_BAD_INPUT, "graph is NULL");
  bool empty = false;
  gst_status st = validate_groups(g, group_ptr, members, k, &empty);
  if (st != GST_OK) return st;
  if (empty) return fail(GST_INFEASIBLE, "a group has no members");
  return GST_OK;
}

struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    cudaGetDevice(&prev);
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};
}  // namespace

gst_status gst_scorer_scores(gst_graph* g, gst_scorer* sc, const int32_t* group_ptr, const int32_t* members, int32_t k,
                             int32_t precision, float* scores) {
  gst_status st = learn_enter(g, group_ptr, members, k);
  if (st != GST_OK) return st;
  if (!sc || !scores) return fail(GST_BAD_INPUT, "scorer / scores is NULL");
  std::lock_guard<std::mutex> lock(g->mu);
  DeviceGuard dg(g->device);
  cudaGetLastError();
  st = ensure_learn_infer(g);
  if (st == GST_OK && precision) st = ensure_learn_train(g, 0);
  if (st == GST_OK) st = upload_groups(g, group_ptr, members, k);
  if (st == GST_OK) st = compute_features(g, k);
  if (st != GST_OK) return st;
  const float* src = g->lw.scores;
  if (precision) {
    st = train_forward(g, sc);
    src = g->lw.s;
  } else {
    st = infer_scores(g, sc);
  }
  if (st != GST_OK) return st;
  std::vector<float> tmp((size_t)g->V);
  GST_CUDA(cudaMemcpyAsync(tmp.data(), src, tmp.size() * sizeof(float), cudaMemcpyDeviceToHost, g->stream));
  GST_CUDA(cudaStreamSynchronize(g->stream));
  for (int32_t v = 0; v < g->V; ++v) scores[v] = tmp[(size_t)g->perm[(size_t)v]];
  return GST_OK;
}

gst_status gst_scorer_train_step(gst_graph* g, gst_scorer* sc, const int32_t* group_ptr, const int32_t* members,
                                 int32_t k, const int32_t* tree_vertices, int32_t n, float lr, int32_t apply,
                                 float* loss, float* grads) {
  gst_status st = learn_enter(g, group_ptr, members, k);
  if (st != GST_OK) return st;
  if (!sc || !tree_vertices || n < 1) return fail(GST_BAD_INPUT, "scorer / tree vertices missing");
  std::vector<int32_t> ids;
  ids.reserve((size_t)n);
  for (int32_t i = 0; i < n; ++i) {
    if (tree_vertices[i] < 0 || tree_vertices[i] >= g->V) return fail(GST_BAD_INPUT, "tree vertex out of range");
    ids.push_back(g->perm[(size_t)tree_vertices[i]]);
  }
  std::sort(ids.begin(), ids.end());
  ids.erase(std::unique(ids.begin(), ids.end()), ids.end());
  std::lock_guard<std::mutex> lock(g->mu);
  DeviceGuard dg(g->device);
  cudaGetLastError();
  cudaStream_t s = g->stream;
  st = ensure_learn_infer(g);
  if (st == GST_OK) st = ensure_learn_train(g, (int32_t)ids.size());
  if (st == GST_OK) st = upload_groups(g, group_ptr, members, k);
  if (st == GST_OK) st = compute_features(g, k);
  if (st == GST_OK) st = train_forward(g, sc);
  if (st != GST_OK) return st;
  LearnWs& lw = g->lw;
  GST_CUDA(cudaMemsetAsync(lw.label, 0, (size_t)g->V, s));
  GST_CUDA(cudaMemcpyAsync(lw.ids, ids.data(), ids.size() * sizeof(int32_t), cudaMemcpyHostToDevice, s));
  GST_CUDA(launch_set_labels(lw.ids, (int32_t)ids.size(), lw.label, s));
  st = train_backward(g, sc, (int32_t)ids.size());
  if (st != GST_OK) return st;
  float l = 0.0f;
  GST_CUDA(cudaMemcpyAsync(&l, lw.red + 2, sizeof(float), cudaMemcpyDeviceToHost, s));
  if (grads) GST_CUDA(cudaMemcpyAsync(grads, lw.grad, kNumParams * sizeof(float), cudaMemcpyDeviceToHost, s));
  if (apply) {
    ++sc->t;
    GST_CUDA(launch_adam(kNumParams, sc->params, lw.grad, sc->m, sc->v, lr, sc->t, s));
    GST_CUDA(launch_pack_bf16(sc->params, sc->wcat, s));
  }
  GST_CUDA(cudaStreamSynchronize(s));
  if (loss) *loss = l;
  return GST_OK;
}

gst_status gst_debug_scorer_wait_timeout(gst_graph* g, const gst_scorer* sc, uint32_t extra_bytes, int32_t* flag_out) {
  g_last_error.clear();
  if (!g || !sc || !flag_out) return fail(GST_BAD_INPUT, "null argument");
  if (extra_bytes > (1u << 16)) return fail(GST_BAD_INPUT, "extra_bytes above 64 KiB");
  DeviceGuard dg(g->device);
  std::lock_guard<std::mutex> lock(g->mu);
  gst_status st = ensure_learn_infer(g);
  if (st != GST_OK) return st;
  LearnWs& lw = g->lw;
  cudaStream_t s = g->stream;
  GST_CUDA(launch_layer_gemm(g->V, lw.hb_map[0], lw.hb_map[2], sc->wcat, sc->params, 1, lw.hb[1], nullptr,
                             lw.infer_err, extra_bytes, s));
  int32_t flag = 0;
  GST_CUDA(cudaMemcpyAsync(&flag, lw.infer_err, sizeof(flag), cudaMemcpyDeviceToHost, s));
  GST_CUDA(cudaStreamSynchronize(s));
  GST_CUDA(cudaMemsetAsync(lw.infer_err, 0, sizeof(int32_t), s));
  GST_CUDA(cudaStreamSynchronize(s));
  *flag_out = flag;
  return flag ? fail(GST_INTERNAL, "scorer layer: a wait ran out") : GST_OK;
}

gst_status gst_propose(gst_graph* g, gst_scorer* sc, const int32_t* group_ptr, const int32_t* members, int32_t k,
                       gst_result** out) {
  if (!out) return fail(GST_BAD_INPUT, "out is NULL");
  *out = nullptr;
  gst_status st = learn_enter(g, group_ptr, members, k);
  if (st != GST_OK) return st;
  auto* r = new (std::nothrow) gst_result;
  if (!r) return fail(GST_OOM, "host allocation failed");
  *out = r;
  std::lock_guard<std::mutex> lock(g->mu);
  DeviceGuard dg(g->device);
  cudaGetLastError();
  const auto t0 = std::chrono::steady_clock::now();
  gst_opts o = resolve_opts(nullptr);
  o.use_graph = 1;
  st = propose_tree(g, sc, group_ptr, members, k, o, r);
  r->propose_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  r->status = st;
  return st;
}

gst_status gst_solve_learned(gst_graph* g, gst_scorer* sc, const int32_t* group_ptr, const int32_t* members, int32_t k,
                             const gst_opts* opts, gst_result** out) {
  if (!out) return fail(GST_BAD_INPUT, "out is NULL");
  *out = nullptr;
  g_last_error.clear();
  if (!g) return fail(GST_BAD_INPUT, "graph is NULL");
  bool empty = false;
  gst_status st = validate_groups(g, group_ptr, members, k, &empty);
  if (st != GST_OK) return st;
  auto* r = new (std::nothrow) gst_result;
  if (!r) return fail(GST_OOM, "host allocation failed");
  *out = r;
  if (empty) {
    r->status = GST_INFEASIBLE;
    return GST_INFEASIBLE;
  }
  gst_opts o = resolve_opts(opts);
  o.refine_bound = 1;
  o.upper_bound = 0;  // the proposal's cost is the bound
  // A captured solve runs the proposal on a serving lane while its graph
  // runs: the proposal takes its paths from the solve's own wave 1, its
  // cost reaches the running DP as a bound through launch_bound_min, and a
  // proposal that the DP outran is given up at its next wait. The host loop
  // proposes first (paths from a two-group solve) and solves under it.
  const bool overlap = o.use_graph != 0 && g->parent == nullptr;
  if (overlap) {
    st = ensure_lanes(g, 1);
    if (st != GST_OK) return st;
  }
  gst_graph* lane = overlap ? g->lanes[0] : nullptr;
  std::unique_lock<std::mutex> lock(g->mu);
  std::unique_lock<std::mutex> lane_lock;
  if (lane) lane_lock = std::unique_lock<std::mutex>(lane->mu);
  DeviceGuard dg(g->device);
  cudaGetLastError();
  const auto t0 = std::chrono::steady_clock::now();
  gst_result prop;
  gst_status pst = GST_INTERNAL;
  double pms = 0;
  if (overlap) {
    for (cudaEvent_t* e : {&g->ev_params, &g->ev_done, &g->ev_side})
      if (!*e) GST_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    bool finished = false;  // the DP's graph has completed (latched)
    const std::function<bool()> stop = [&]() {
      return finished = finished || cudaEventQuery(g->ev_done) == cudaSuccess;
    };
    bool bounded = false;
    const std::function<void()> propose = [&]() {
      pst = propose_tree(lane, sc, group_ptr, members, k, o, &prop, &stop, g);
      if (pst == GST_OK && prop.cost > 0 && !stop()) {
        // after the solve's parameters are on the device, so that their
        // upload does not overwrite the bound
        if (cudaStreamWaitEvent(lane->stream, g->ev_params, 0) != cudaSuccess ||
            launch_bound_min(g->ws.d_params, prop.cost, lane->stream) != cudaSuccess)
          pst = GST_INTERNAL;
        else
          bounded = true;
      }
      // the solve ends after the lane's queued work: the bound lands before
      // the next solve uploads its parameters, and a given-up proposal's
      // kernels finish before the lane is used again
      if (cudaEventRecord(g->ev_side, lane->stream) != cudaSuccess ||
          cudaStreamWaitEvent(g->stream, g->ev_side, 0) != cudaSuccess)
        pst = GST_INTERNAL;
      pms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    };
    st = solve_one(g, group_ptr, members, k, o, r, &propose);
    r->propose_ms = pms;
    r->proposal_concurrent = 1;
    if (bounded) r->proposal_cost = prop.cost;
    r->launches += prop.launches + (bounded ? 1 : 0);  // + the bound's
    // the bound the solve ended with: the proposal's may have landed after
    // the last wave copied the parameters back
    if (bounded && (r->ub <= 0 || prop.cost < r->ub)) r->ub = prop.cost;
    if (st != GST_INFEASIBLE || !bounded) {
      // a failed proposal only forgoes its bound: the DP decided alone
      if (st == GST_OK || st == GST_INFEASIBLE) g_last_error.clear();
      r->status = st;
      r->wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
      return st;
    }
    // an infeasible verdict under a proposal's bound: decided again unpruned
    // (a feasible proposal makes it impossible; kept as a guard)
  } else {
    pst = propose_tree(g, sc, group_ptr, members, k, o, &prop);
    pms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (pst == GST_OK && prop.cost > 0) {
      o.upper_bound = prop.cost;
      st = solve_one(g, group_ptr, members, k, o, r);
      if (st == GST_OK) {
        r->status = GST_OK;
        r->proposal_cost = prop.cost;
        r->propose_ms = pms;
        r->launches += prop.launches;
        r->wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        return GST_OK;
      }
      if (st != GST_INFEASIBLE) {
        r->status = st;
        return st;
      }
    }
  }
  // no usable proposal (or a zero-cost one): the unpruned DP decides
  g_last_error.clear();
  const int64_t plaunches = prop.launches;
  *r = gst_result{};
  o.upper_bound = 0;
  st = solve_one(g, group_ptr, members, k, o, r);
  r->status = st;
  r->propose_ms = pms;
  r->launches += plaunches;
  r->wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return st;
}

int32_t gst_result_upper_bound(const gst_result* r) { return r ? r->ub : 0; }
int32_t gst_result_proposal_cost(const gst_result* r) { return r ? r->proposal_cost : 0; }
double gst_result_proposal_ms(const gst_result* r) { return r ? r->propose_ms : 0.0; }
int32_t gst_result_proposal_concurrent(const gst_result* r) { return r ? r->proposal_concurrent : 0; }
double gst_result_wall_ms(const gst_result* r) { return r ? r->wall_ms : 0.0; }

const char* gst_last_error(void) { return g_last_error.c_str(); }
const char* gst_version(void) { return "gst-gb300 0.2 (sm_103a)"; }

}  // extern "C"
