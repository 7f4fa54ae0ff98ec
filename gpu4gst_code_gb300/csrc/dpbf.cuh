// Internal declarations shared by the DPBF kernels (dpbf_kernels.cu) and the
// host driver behind the C ABI (engine.cu).
//
// State table layout in HBM ("level-major, vertex-major within a level"):
// the 2^k - 1 non-empty group-set masks are ordered by popcount (the DP
// wave, or level), then by value. Level l holds m_l = C(k,l) masks; its
// slice starts at entry base_l * V with base_l = sum_{l'<l} m_l', and the
// m_l entries of vertex v are contiguous at base_l*V + v*m_l + rank(S).
// Growth at level l therefore gathers one contiguous m_l-entry row per
// neighbour, and a merge reads the lower-level rows of its own vertex.
// cost[] holds int32 tree costs (GST_INF = no tree); par[] holds how the
// state was last improved:
//   par >= 0        grown over CSR entry par of this vertex (col = child),
//   par <  0        merged from S1 = -par and S ^ S1,
//   par == GST_LEAF the vertex itself (S inside its groups, cost 0).
#pragma once
#include <cstdint>

#include <cuda_runtime.h>

namespace gst {

constexpr int32_t kInf = 0x3FFFFFFF;  // == GST_COST_LIMIT; finite costs stay below
constexpr int32_t kLeaf = INT32_MIN;
constexpr int kDegBig = 64;        // rows longer than this go to a CTA of their own
constexpr int kGrowThreads = 256;  // block size of growth / merge kernels

// Per-mask position in the table (device copy built on the host for each k).
struct MaskInfo {
  int32_t base;   // base_l of the mask's level
  int32_t m;      // masks in that level
  int32_t rank;   // index within the level
  int32_t level;  // popcount
};

// Statistic slots (int64) accumulated by kernels when stats are on.
enum StatSlot {
  kStatRounds = 0,
  kStatVertices = 1,
  kStatEntries = 2,
  kStatRows = 3,
  kStatGathered = 4,
  kStatImproved = 5,
  kStatSplits = 6,
  kStatBytes = 7,
  kNumStats = 8
};

// Device-side counters of one solve (a small int32 block).
struct Counters {
  int32_t changed[3];  // rotating per-round change counts
  int32_t overflow;    // a candidate reached kInf
  int32_t bt_overflow; // backtrack ran out of capacity
  int32_t bt_nv, bt_ne, bt_states;
  unsigned long long best;  // (cost << 32) | root, argmin of the full mask
  unsigned long long states;  // states written by merges + growth
};

struct GraphDev {
  int32_t V;
  const int32_t* row_ptr;  // V+1
  const int2* adj;         // (col, w) per CSR entry
  const int32_t* big;      // vertices with degree > kDegBig
  int32_t nbig;
};

struct LevelArgs {
  int32_t level, m, k;
  int64_t base;                // base_l * V
  const int32_t* lmasks;       // masks of this level, by rank
  const MaskInfo* minfo;       // indexed by mask
  int32_t* cost;
  int32_t* par;
  const uint32_t* gmask;       // groups(v) bit mask
  const uint8_t* cur_flag;     // changed in the previous round
  uint8_t* next_flag;          // changed in this round
  uint8_t* clear_flag;         // cleared for the round after next
  const int32_t* prev_changed;
  int32_t* cur_changed;
  int32_t* zero_changed;
  Counters* ctr;
  long long* stats;            // nullptr when off
  // pruning (upper_bound > 0): drop a state when cost + LB(v, full^S) > ub,
  // LB = max over groups g outside S of cost(v,{g}) (level-1 slice).
  int32_t ub;
  int64_t base1;               // level-1 slice (== 0)
};

// Launchers (dpbf_kernels.cu). All asynchronous on `stream`.
cudaError_t launch_group_masks(const int32_t* group_ptr, const int32_t* members, int32_t k, int32_t nmembers,
                               uint32_t* gmask, cudaStream_t stream);
cudaError_t launch_merge(const GraphDev& g, const LevelArgs& a, cudaStream_t stream);
cudaError_t launch_grow_round(const GraphDev& g, const LevelArgs& a, int num_sms, cudaStream_t stream);
cudaError_t launch_argmin(const GraphDev& g, const int32_t* full_slice, Counters* ctr, cudaStream_t stream);
cudaError_t launch_backtrack(const GraphDev& g, int64_t nnz, const int32_t* par, const MaskInfo* minfo,
                             int32_t full, Counters* ctr, int2* qa, int2* qb, int32_t* out_v, int3* out_e,
                             int32_t cap, cudaStream_t stream);

}  // namespace gst
