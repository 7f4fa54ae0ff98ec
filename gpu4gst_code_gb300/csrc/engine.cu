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
// Compared with DPBF_GPU (src/DPQ.cu:501-768): no V x 2^k host table and no
// full-table host<->device copies (DPQ.cu:592,635,661,711), no host-side
// re-initialisation (DPQ.cu:638-659), no managed memory, and the growth
// loop polls the device only every few rounds instead of after every
// launch (DPQ.cu:684-702).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <unordered_set>
#include <utility>
#include <vector>

#include "dpbf.cuh"
#include "gst.h"
#include "gst_debug.h"

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
}  // namespace

// ---------------------------------------------------------------- objects --
struct Workspace {
  int32_t k_cap = 0;          // cost/par sized for this many groups
  int32_t* cost = nullptr;    // V * (2^k_cap - 1)
  int32_t* par = nullptr;
  uint32_t* gmask = nullptr;  // V
  uint8_t* flags = nullptr;   // 3 * V
  Counters* ctr = nullptr;
  long long* stats = nullptr;
  MaskInfo* minfo = nullptr;  // 2^GST_MAX_K
  int32_t* lmasks = nullptr;  // 2^GST_MAX_K
  int32_t tables_k = 0;       // k the mask tables describe
  int32_t* d_group_ptr = nullptr;
  int32_t* d_members = nullptr;
  int64_t members_cap = 0;
  int2* qa = nullptr;
  int2* qb = nullptr;
  int32_t* out_v = nullptr;
  int3* out_e = nullptr;
  int32_t bt_cap = 0;
  Counters* h_ctr = nullptr;  // pinned
  int32_t* h_changed = nullptr;
  cudaEvent_t ev[2 * GST_MAX_K + 4] = {};
  std::vector<int32_t> h_lvl_base, h_lvl_m;
};

struct gst_graph {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  int32_t V = 0;
  int64_t nnz = 0;
  int32_t* d_row_ptr = nullptr;
  int2* d_adj = nullptr;
  int32_t* d_big = nullptr;
  int32_t nbig = 0;
  std::vector<int32_t> h_row_ptr;
  std::mutex mu;
  Workspace ws;
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
};

namespace {

GraphDev graph_dev(const gst_graph* g) {
  GraphDev d;
  d.V = g->V;
  d.row_ptr = g->d_row_ptr;
  d.adj = g->d_adj;
  d.big = g->d_big;
  d.nbig = g->nbig;
  return d;
}

void free_workspace(Workspace& ws) {
  dfree(ws.cost);
  dfree(ws.par);
  dfree(ws.gmask);
  dfree(ws.flags);
  dfree(ws.ctr);
  dfree(ws.stats);
  dfree(ws.minfo);
  dfree(ws.lmasks);
  dfree(ws.d_group_ptr);
  dfree(ws.d_members);
  dfree(ws.qa);
  dfree(ws.qb);
  dfree(ws.out_v);
  dfree(ws.out_e);
  if (ws.h_ctr) cudaFreeHost(ws.h_ctr);
  if (ws.h_changed) cudaFreeHost(ws.h_changed);
  ws.h_ctr = nullptr;
  ws.h_changed = nullptr;
  for (auto& e : ws.ev)
    if (e) {
      cudaEventDestroy(e);
      e = nullptr;
    }
  ws.k_cap = 0;
  ws.tables_k = 0;
  ws.members_cap = 0;
  ws.bt_cap = 0;
}

// Allocates everything a query with k groups and `nmembers` members needs.
gst_status ensure_workspace(gst_graph* g, int32_t k, int64_t nmembers) {
  Workspace& ws = g->ws;
  const int64_t V = g->V;
  if (!ws.gmask) {
    GST_CUDA(cudaMalloc(&ws.gmask, V * sizeof(uint32_t)));
    GST_CUDA(cudaMalloc(&ws.flags, 3 * V));
    GST_CUDA(cudaMalloc(&ws.ctr, sizeof(Counters)));
    GST_CUDA(cudaMalloc(&ws.stats, kNumStats * sizeof(long long)));
    GST_CUDA(cudaMalloc(&ws.minfo, sizeof(MaskInfo) << GST_MAX_K));
    GST_CUDA(cudaMalloc(&ws.lmasks, sizeof(int32_t) << GST_MAX_K));
    GST_CUDA(cudaMallocHost(&ws.h_ctr, sizeof(Counters)));
    GST_CUDA(cudaMallocHost(&ws.h_changed, 4 * sizeof(int32_t)));
    for (auto& e : ws.ev) GST_CUDA(cudaEventCreate(&e));
    // backtrack capacity: states of one optimal derivation
    ws.bt_cap = (int32_t)std::min<int64_t>(4 * V + 256, 1 << 24);
    GST_CUDA(cudaMalloc(&ws.qa, (size_t)ws.bt_cap * sizeof(int2)));
    GST_CUDA(cudaMalloc(&ws.qb, (size_t)ws.bt_cap * sizeof(int2)));
    GST_CUDA(cudaMalloc(&ws.out_v, (size_t)ws.bt_cap * sizeof(int32_t)));
    GST_CUDA(cudaMalloc(&ws.out_e, (size_t)ws.bt_cap * sizeof(int3)));
  }
  if (k > ws.k_cap) {
    dfree(ws.cost);
    dfree(ws.par);
    ws.k_cap = 0;
    const size_t entries = (size_t)V * ((size_t(1) << k) - 1);
    GST_CUDA(cudaMalloc(&ws.cost, entries * sizeof(int32_t)));
    GST_CUDA(cudaMalloc(&ws.par, entries * sizeof(int32_t)));
    ws.k_cap = k;
  }
  if (nmembers > ws.members_cap || !ws.d_group_ptr) {
    dfree(ws.d_group_ptr);
    dfree(ws.d_members);
    ws.members_cap = 0;
    const int64_t cap = std::max<int64_t>(nmembers, 1024);
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
  std::vector<int32_t> lm;
  lm.reserve((size_t)W);
  ws.h_lvl_base.assign((size_t)k + 2, 0);
  ws.h_lvl_m.assign((size_t)k + 2, 0);
  int32_t base = 0;
  for (int l = 1; l <= k; ++l) {
    ws.h_lvl_base[l] = base;
    ws.h_lvl_m[l] = binom(k, l);
    int32_t rank = 0;
    for (int S = 1; S < W; ++S)
      if (__builtin_popcount((unsigned)S) == l) {
        info[(size_t)S] = MaskInfo{base, ws.h_lvl_m[l], rank++, l};
        lm.push_back(S);
      }
    base += ws.h_lvl_m[l];
  }
  info[0] = MaskInfo{0, 0, 0, 0};
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

// Builds the host result from the device walk: distinct vertices, distinct
// edges (u < v), and a check that the edges cost exactly the DP optimum.
gst_status collect_tree(gst_graph* g, gst_result* r, int32_t cost, int32_t root) {
  Workspace& ws = g->ws;
  const Counters& c = *ws.h_ctr;
  if (c.bt_overflow) return fail(GST_INTERNAL, "tree walk failed (code " + std::to_string(c.bt_overflow) + ")");
  const int32_t nv = c.bt_nv, ne = c.bt_ne;
  std::vector<int32_t> hv((size_t)nv);
  std::vector<int3> he((size_t)ne);
  if (nv) GST_CUDA(cudaMemcpyAsync(hv.data(), ws.out_v, (size_t)nv * 4, cudaMemcpyDeviceToHost, g->stream));
  if (ne) GST_CUDA(cudaMemcpyAsync(he.data(), ws.out_e, (size_t)ne * sizeof(int3), cudaMemcpyDeviceToHost, g->stream));
  GST_CUDA(cudaStreamSynchronize(g->stream));
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

float elapsed(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  return ms;
}

// One query. Caller holds g->mu and has validated the groups.
gst_status solve_one(gst_graph* g, const int32_t* group_ptr, const int32_t* members, int32_t k,
                     const gst_opts& o, gst_result* r) {
  Workspace& ws = g->ws;
  const int64_t nmembers = group_ptr[k];
  gst_status st = ensure_workspace(g, k, nmembers);
  if (st != GST_OK) return st;
  st = ensure_tables(g, k);
  if (st != GST_OK) return st;
  cudaStream_t s = g->stream;
  const int64_t V = g->V;
  const int32_t full = (1 << k) - 1;
  const GraphDev gd = graph_dev(g);
  const int64_t max_rounds = o.max_rounds > 0 ? o.max_rounds : V + 1;

  GST_CUDA(cudaEventRecord(ws.ev[0], s));
  GST_CUDA(cudaMemcpyAsync(ws.d_group_ptr, group_ptr, (size_t)(k + 1) * 4, cudaMemcpyHostToDevice, s));
  if (nmembers)
    GST_CUDA(cudaMemcpyAsync(ws.d_members, members, (size_t)nmembers * 4, cudaMemcpyHostToDevice, s));
  GST_CUDA(cudaMemsetAsync(ws.gmask, 0, V * sizeof(uint32_t), s));
  GST_CUDA(cudaMemsetAsync(ws.ctr, 0, sizeof(Counters), s));
  GST_CUDA(cudaMemsetAsync(&ws.ctr->best, 0xff, sizeof(unsigned long long), s));
  GST_CUDA(cudaMemsetAsync(ws.stats, 0, kNumStats * sizeof(long long), s));
  GST_CUDA(launch_group_masks(ws.d_group_ptr, ws.d_members, k, (int32_t)nmembers, ws.gmask, s));
  int64_t launches = nmembers > 0 ? 1 : 0;

  uint8_t* F[3] = {ws.flags, ws.flags + V, ws.flags + 2 * V};
  int32_t* C = ws.ctr->changed;
  double grow_ms = 0, merge_ms = 0;
  int ev_i = 1;
  bool timeout = false;
  for (int32_t l = 1; l <= k && !timeout; ++l) {
    LevelArgs a{};
    a.level = l;
    a.m = ws.h_lvl_m[l];
    a.k = k;
    a.base = (int64_t)ws.h_lvl_base[l] * V;
    a.lmasks = ws.lmasks + ws.h_lvl_base[l];
    a.minfo = ws.minfo;
    a.cost = ws.cost;
    a.par = ws.par;
    a.gmask = ws.gmask;
    a.ctr = ws.ctr;
    a.stats = o.collect_stats ? ws.stats : nullptr;
    a.ub = (l >= 2 && o.upper_bound > 0) ? o.upper_bound : 0;
    a.base1 = 0;
    // merge = "round -1": writes frontier F[2] and count C[2]
    GST_CUDA(cudaMemsetAsync(ws.flags, 0, 3 * V, s));
    GST_CUDA(cudaMemsetAsync(C, 0, 3 * sizeof(int32_t), s));
    a.next_flag = F[2];
    a.cur_changed = C + 2;
    cudaEvent_t e0 = ws.ev[ev_i++];
    cudaEvent_t e1 = ws.ev[ev_i++];
    GST_CUDA(cudaEventRecord(e0, s));
    GST_CUDA(launch_merge(gd, a, s));
    ++launches;
    GST_CUDA(cudaEventRecord(e1, s));
    if (l == k) {
      GST_CUDA(cudaEventSynchronize(e1));
      merge_ms += elapsed(e0, e1);
      break;
    }
    // growth rounds, polled every `batch` launches; converged rounds exit
    // on their first instruction
    int64_t r = 0;
    const int batch = 8;
    for (;;) {
      for (int i = 0; i < batch; ++i, ++r) {
        a.cur_flag = F[(r + 2) % 3];
        a.next_flag = F[r % 3];
        a.clear_flag = F[(r + 1) % 3];
        a.prev_changed = C + (r + 2) % 3;
        a.cur_changed = C + r % 3;
        a.zero_changed = C + (r + 1) % 3;
        GST_CUDA(launch_grow_round(gd, a, g->num_sms, s));
        ++launches;
      }
      GST_CUDA(cudaMemcpyAsync(ws.h_changed, C + (r - 1) % 3, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
      GST_CUDA(cudaStreamSynchronize(s));
      if (*ws.h_changed == 0) break;
      if (r >= max_rounds) {
        timeout = true;
        break;
      }
    }
    cudaEvent_t e2 = ws.ev[ev_i++];
    GST_CUDA(cudaEventRecord(e2, s));
    GST_CUDA(cudaEventSynchronize(e2));
    merge_ms += elapsed(e0, e1);
    grow_ms += elapsed(e1, e2);
    ev_i -= 3;  // reuse the three events for the next wave
  }
  if (timeout) return fail(GST_TIMEOUT, "growth did not converge within max_rounds");
  cudaEvent_t eb0 = ws.ev[ev_i], eb1 = ws.ev[ev_i + 1];
  GST_CUDA(cudaEventRecord(eb0, s));
  const int32_t* full_slice = ws.cost + (int64_t)ws.h_lvl_base[k] * V;
  GST_CUDA(launch_argmin(gd, full_slice, ws.ctr, s));
  GST_CUDA(launch_backtrack(gd, g->nnz, ws.par, ws.minfo, full, ws.ctr, ws.qa, ws.qb, ws.out_v, ws.out_e,
                            ws.bt_cap, s));
  launches += 2;
  r->launches = launches;
  GST_CUDA(cudaEventRecord(eb1, s));
  GST_CUDA(cudaMemcpyAsync(ws.h_ctr, ws.ctr, sizeof(Counters), cudaMemcpyDeviceToHost, s));
  if (o.collect_stats)
    GST_CUDA(cudaMemcpyAsync(r->stats, ws.stats, kNumStats * sizeof(long long), cudaMemcpyDeviceToHost, s));
  GST_CUDA(cudaStreamSynchronize(s));
  r->ms[0] = elapsed(ws.ev[0], eb1);
  r->ms[1] = grow_ms;
  r->ms[2] = merge_ms;
  r->ms[3] = elapsed(eb0, eb1);
  const Counters& c = *ws.h_ctr;
  r->states = (int64_t)c.states;
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

}  // namespace

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
  std::vector<int2> adj((size_t)nnz);
  for (int64_t e = 0; e < nnz; ++e) {
    if (col[e] < 0 || col[e] >= V) return fail(GST_BAD_INPUT, "col entry out of range");
    if (w[e] < 0 || w[e] >= GST_COST_LIMIT) return fail(GST_BAD_INPUT, "weights must be in [0, GST_COST_LIMIT)");
    adj[(size_t)e] = make_int2(col[e], w[e]);
  }
  auto* g = new (std::nothrow) gst_graph;
  if (!g) return fail(GST_OOM, "host allocation failed");
  g->V = V;
  g->nnz = nnz;
  g->h_row_ptr.assign(row_ptr, row_ptr + V + 1);
  std::vector<int32_t> big;
  for (int32_t v = 0; v < V; ++v)
    if (row_ptr[v + 1] - row_ptr[v] > kDegBig) big.push_back(v);
  g->nbig = (int32_t)big.size();
  auto cleanup = [&](gst_status s) {
    gst_graph_free(g);
    return s;
  };
  cudaError_t e;
  if ((e = cudaGetDevice(&g->device)) != cudaSuccess ||
      (e = cudaDeviceGetAttribute(&g->num_sms, cudaDevAttrMultiProcessorCount, g->device)) != cudaSuccess ||
      (e = cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking)) != cudaSuccess)
    return cleanup(fail(GST_CUDA_ERROR, std::string("device setup: ") + cudaGetErrorString(e)));
  auto up = [&](void** dst, const void* src, size_t bytes) -> cudaError_t {
    cudaError_t x = cudaMalloc(dst, bytes ? bytes : 4);
    if (x != cudaSuccess || !bytes) return x;
    return cudaMemcpyAsync(*dst, src, bytes, cudaMemcpyHostToDevice, g->stream);
  };
  if ((e = up((void**)&g->d_row_ptr, row_ptr, (size_t)(V + 1) * 4)) != cudaSuccess ||
      (e = up((void**)&g->d_adj, adj.data(), adj.size() * sizeof(int2))) != cudaSuccess ||
      (e = up((void**)&g->d_big, big.data(), big.size() * 4)) != cudaSuccess ||
      (e = cudaStreamSynchronize(g->stream)) != cudaSuccess)
    return cleanup(fail(e == cudaErrorMemoryAllocation ? GST_OOM : GST_CUDA_ERROR,
                        std::string("graph upload: ") + cudaGetErrorString(e)));
  *out = g;
  return GST_OK;
}

void gst_graph_free(gst_graph* g) {
  if (!g) return;
  int prev = -1;
  cudaGetDevice(&prev);
  cudaSetDevice(g->device);
  if (g->stream) cudaStreamSynchronize(g->stream);
  free_workspace(g->ws);
  dfree(g->d_row_ptr);
  dfree(g->d_adj);
  dfree(g->d_big);
  if (g->stream) cudaStreamDestroy(g->stream);
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
  gst_status first = GST_OK;
  int64_t gbase = 0;
  for (int32_t q = 0; q < nq; ++q) {
    out[q] = nullptr;
    if (ks[q] < 1 || ks[q] > GST_MAX_K) {
      if (first == GST_OK) first = fail(GST_BAD_INPUT, "k out of range in batch");
      continue;
    }
    std::vector<int32_t> gp((size_t)ks[q] + 1);
    for (int32_t i = 0; i <= ks[q]; ++i) gp[(size_t)i] = group_ptr[gbase + i] - group_ptr[gbase];
    const int32_t* mem = members ? members + group_ptr[gbase] : nullptr;
    gst_status st = gst_solve(g, gp.data(), mem, ks[q], opts, &out[q]);
    if (st != GST_OK && st != GST_INFEASIBLE && first == GST_OK) first = st;
    gbase += ks[q];
  }
  return first;
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
  std::vector<int32_t> dev((size_t)(V * (W - 1)));
  GST_CUDA(cudaMemcpy(dev.data(), ws.cost, dev.size() * sizeof(int32_t), cudaMemcpyDeviceToHost));
  for (int64_t v = 0; v < V; ++v) out[v * W] = kInf;
  for (int l = 1; l <= k; ++l) {
    const int64_t base = (int64_t)ws.h_lvl_base[l] * V;
    const int32_t m = ws.h_lvl_m[l];
    int32_t rank = 0;
    for (int32_t S = 1; S < (int32_t)W; ++S) {
      if (__builtin_popcount((unsigned)S) != l) continue;
      for (int64_t v = 0; v < V; ++v) out[v * W + S] = dev[(size_t)(base + v * m + rank)];
      ++rank;
    }
  }
  return GST_OK;
}

const char* gst_last_error(void) { return g_last_error.c_str(); }
const char* gst_version(void) { return "gst-gb300 0.1 (sm_103a)"; }

}  // extern "C"
