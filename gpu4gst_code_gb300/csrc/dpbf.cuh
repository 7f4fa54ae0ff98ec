// Internal declarations shared by the DPBF kernels (dpbf_kernels.cu) and the
// host driver behind the C ABI (engine.cu).
//
// State table layout in HBM ("level-major, vertex-major within a level"):
// the 2^k - 1 non-empty group-set masks are ordered by popcount (the DP
// wave, or level), then by value. Level l holds m_l = C(k,l) masks in a row
// of stride s_l = m_l rounded up to a multiple of 4 (padding entries hold
// kInf), so every row starts on a 16-byte boundary and can be moved with
// int4 loads. Level l's slice starts at entry base_l * V with
// base_l = sum_{l'<l} s_l', and vertex v's row is at base_l*V + v*s_l.
// Growth at level l gathers one contiguous row per neighbour; a merge reads
// the lower-level rows of its own vertex.
// cost[] holds int32 tree costs (kInf = no tree); par[] holds how the state
// was last improved:
//   par >= 0      grown over CSR entry par of this vertex (col = child),
//   par <  0      merged from S1 = -par and S ^ S1,
//   par == kLeaf  the vertex itself (S inside its groups, cost 0).
#pragma once
#include <cstdint>

#include <cuda_runtime.h>

namespace gst {

constexpr int32_t kInf = 0x3FFFFFFF;  // == GST_COST_LIMIT; finite costs stay below
constexpr int32_t kLeaf = INT32_MIN;
// Rows longer than GraphDev::deg_big entries are hubs, relaxed in 32-entry
// chunks by any warp; deg_big = 4 x the average degree, clamped to
// [kDegBigMin, kDegBigMax] (parent codes of other rows fit a byte).
constexpr int kDegBigMin = 32;
constexpr int kDegBigMax = 64;
constexpr int kGrowThreads = 256;  // block size of growth / merge kernels
// Longest hub segment a warp relaxes in registers (hubs up to this degree
// are relaxed whole, with no scratch row).
constexpr int kHubSeg = 256;
constexpr int kMaxThreadMasks = 24;  // waves with stride <= this: a thread per vertex (sparse rounds)
// Dense rounds of waves with stride <= this run a team of stride/4 lanes per
// vertex, each lane holding four masks (k_grow_team).
constexpr int kMaxTeamStride = 32;
// Sparse rounds scan candidate flags in tiles of this many consecutive
// vertex IDs (one warp each). The graph is relabelled at upload so that
// every tile holds a mix of degrees (see gst_graph_upload).
constexpr int kCandTile = 256;
// Dense rounds when the previous round changed more than V >> this
// (sparse rounds with marking stay cheaper up to about half the graph).
constexpr int kDefaultDenseShift = 1;
constexpr int kDefaultDenseShiftPruned = 2;  // solves with a bound or bound refinement

__host__ __device__ constexpr int32_t row_stride(int32_t m) { return (m + 3) & ~3; }

// Per-mask position in the table (device copy built on the host for each k).
struct MaskInfo {
  int32_t base;    // base_l of the mask's level
  int32_t stride;  // row stride s_l of that level
  int32_t rank;    // index within the level
  int32_t level;   // popcount
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

// Per-query scalars read by the kernels from device memory, so one
// captured CUDA graph serves every query with the same k.
struct SolveParams {
  int32_t ub;          // upper bound for pruning (<= 0: none)
  int32_t max_rounds;  // growth rounds allowed per wave
  int32_t stats_on;    // accumulate StatSlot counters
  int32_t k;
  // Stored costs stay below kInf - (largest edge weight): then adding any
  // weight to a finite cost stays below kInf, so relaxations need no
  // overflow test. A cost that reaches the limit is reported (GST_OVERFLOW).
  int32_t ovf_limit;
  int32_t dense_shift;  // dense round when the previous one changed > V >> dense_shift
  int32_t refine;       // lower ub between waves from partial trees (k_ub_refine)
  // A bound may arrive while the solve runs (launch_bound_min from another
  // stream): every merge writes its wave's caps (kInf without a bound yet)
  // and the tour table is built without a bound, so that a wave whose merge
  // saw no bound can still prune by caps and tours once one arrives.
  int32_t late_bound;
};

// Growth-loop control of the current wave (reset before each wave).
// Round r uses change-count slot r%3 and reads slot (r+2)%3 (the previous
// round; the merge acts as round -1 and fills slot 2); the last block to
// finish a round publishes its total and advances `round`.
struct GrowCtl {
  int32_t round;
  uint32_t done;        // blocks finished in the current round
  int32_t changed[3];   // rotating per-round change counts
  int32_t dense[3];     // round ran dense (all vertices, no candidate marks)
  int32_t last_changed; // changes of the last completed round
  int32_t timeout;      // stopped by max_rounds with changes pending
  uint32_t work[3];     // rotating per-round work counters (vertex batches / candidate tiles taken)
};

// Device-side counters of one solve.
struct Counters {
  int32_t overflow;     // a candidate reached kInf
  int32_t bt_overflow;  // backtrack ran out of capacity / found a bad record
  int32_t bt_nv, bt_ne, bt_states;
  int32_t rounds_total; // growth rounds that did work, all waves
  int32_t timeout;
  int32_t grow_launches;      // growth-round kernels launched (each counts itself)
  int32_t pad;
  unsigned long long best;    // (cost << 32) | root, argmin of the full mask
  unsigned long long states;  // states written by merges + growth
};

struct GraphDev {
  int32_t V;
  const int32_t* row_ptr;  // V+1
  const int2* adj;         // (col, w) per CSR entry
  int32_t deg_big;         // hub threshold (see kDegBigMin)
  const int32_t* big;      // vertices with degree > deg_big
  int32_t nbig;
  const int32_t* order;    // the other vertices by decreasing degree
  int32_t nsmall;          // V - nbig
  const int2* hub_chunk;   // (hub index, first CSR entry) per 32-entry chunk
  const int32_t* chunk_vtx;  // the hub vertex of each chunk
  int64_t nchunks;
  // hub rows cut into segments of at most kHubSeg entries, relaxed by one
  // warp each: (hub vertex, hub index, first CSR entry, segments of that hub)
  const int4* hub_seg;
  int64_t nsegs;
  unsigned long long* hub_min;  // per hub: hub_stride packed (cost, entry) minima
  int32_t* hub_cnt;             // per hub: chunks finished this round
  int32_t hub_stride;
};

struct LevelArgs {
  int32_t level, m, stride, k;
  int64_t base;                // base_l * V
  int32_t stride1;             // row stride of wave 1 (pruning bound)
  const int32_t* lmasks;       // masks of this level, by rank
  const MaskInfo* minfo;       // indexed by mask
  int32_t* cost;
  int32_t* par;
  const uint32_t* gmask;       // groups(v) bit mask
  int32_t vpad;                // V rounded up to a multiple of 16: stride of the flag arrays
  uint8_t* flags;              // changed flags F[0..2] (vpad bytes each)
  uint8_t* cand;               // candidate flags C[0..2] (vpad bytes each, 16-byte aligned)
  GrowCtl* ctl;
  Counters* ctr;
  long long* stats;
  const SolveParams* params;
  // merge split table of this level (k <= kMergeTabK): for mask rank j,
  // splits [msplit_ptr[j], msplit_ptr[j+1]) of msplits, each
  // ((level1 << 24) | rank1, (level2 << 24) | rank2) with S1 holding S's
  // lowest group
  const int32_t* msplit_ptr;
  const int2* msplits;
  int32_t nsplits;
  cudaGraphConditionalHandle cond;  // while-loop handle when captured
  int32_t use_cond;
  // pruning caps of this level's states, written by the merge when a bound
  // exists (level >= 2): cap(v,S) = ub - LB(v, groups outside S), rows of
  // stride `stride`; growth keeps a state only if its cost is <= its cap
  int32_t* capt;
  // tour table of the PrunedDP++ tour bound (k <= kTourMaxK, 2 <= level < k;
  // null otherwise): path[(i << k | X) * k + j] = the cheapest order of
  // visiting the groups of X from group i to group j, over lower bounds of
  // the group-to-group distances, clamped at the bound; then W2 (k x 2^k);
  // then, at k x 2^k x (k + 1), the level's compact tables that the merges
  // copy to shared memory: for mask rank j, the W2 values of the n = k -
  // level groups outside S_j and the path values of their pairs i < i2
  const int32_t* tour;
};

// Groups up to which the merge adds PrunedDP++'s tour bounds to the one-label
// bound. k_tour_table keeps the k x 2^k x k path table in shared memory up
// to kTourSmemMaxK groups (162 KB at k = 9) and builds it in place in the
// tour buffer (global memory, 400 KB at k = 10) beyond.
constexpr int kTourMaxK = 10;
constexpr int kTourSmemMaxK = 9;
// Room for the largest level's compact tour tables (C(10,4) masks x (6 + 15)
// entries = 4,410 words at k = 10).
constexpr int kTourCompactWords = 8192;

// Words of the compact tour tables of level l at k groups: C(k, l) masks x
// (n + n (n - 1) / 2) entries, n = k - l groups outside each.
constexpr int64_t tour_compact_words(int k, int l) {
  int64_t c = 1;
  for (int i = 0; i < l; ++i) c = c * (k - i) / (i + 1);
  const int64_t n = k - l;
  return c * (n + n * (n - 1) / 2);
}
constexpr bool tour_compact_fits() {
  for (int k = 2; k <= kTourMaxK; ++k)
    for (int l = 2; l < k; ++l)
      if (tour_compact_words(k, l) > kTourCompactWords) return false;
  return true;
}
static_assert(tour_compact_fits(), "the compact tour tables of every level fit their room");

// Queries with at most kMergeTabK groups merge from per-level split tables
// (k_merge_staged: a thread per vertex; k_merge_team: a team of lanes per
// vertex for long lower-level rows); larger k use k_merge.
constexpr int kMergeTabK = 10;

// Where each level's rows live, for the split-table merges.
struct MergeLevels {
  int64_t off[kMergeTabK + 1];     // base_l * V
  int32_t stride[kMergeTabK + 1];  // row stride of level l
  int32_t mbase[kMergeTabK + 1];   // base_l: level l's masks start at lmasks_all[mbase[l]]
  const int32_t* lmasks_all;
};

// Launchers (dpbf_kernels.cu). All asynchronous on `stream`.
// members are caller IDs; perm maps them to internal IDs
cudaError_t launch_group_masks(const int32_t* group_ptr, const int32_t* members, const int32_t* perm, int32_t k,
                               uint32_t* gmask, cudaStream_t stream);
cudaError_t launch_merge(const GraphDev& g, const LevelArgs& a, const MergeLevels& ml, cudaStream_t stream);
// One growth round: a hub-relaxation kernel (when the graph has hubs) and
// the round kernel proper. Adds the kernels launched to *launches.
cudaError_t launch_grow_round(const GraphDev& g, const LevelArgs& a, int num_sms, cudaStream_t stream,
                              int64_t* launches);
cudaError_t launch_seed(const GraphDev& g, const LevelArgs& a, int num_sms, cudaStream_t stream);
// Before wave a.level's merge (a.tour non-null): the tour table for the
// current bound, from wave 1's distances of the query's members.
cudaError_t launch_tour_table(const LevelArgs& a, const int32_t* group_ptr, const int32_t* members,
                              const int32_t* perm, int32_t* tour, cudaStream_t stream);
// After wave a.level's growth: with params->refine set, lowers params->ub to
// the cheapest T(v,S) + sum of T(v,{g}) over the groups g outside S.
cudaError_t launch_ub_refine(const GraphDev& g, const LevelArgs& a, int num_sms, cudaStream_t stream);
// Lowers params->ub to cand (none yet: to cand) by a CAS loop on the device.
cudaError_t launch_bound_min(SolveParams* params, int32_t cand, cudaStream_t stream);
cudaError_t launch_argmin(const GraphDev& g, const int32_t* full_slice, int32_t stride, Counters* ctr,
                          cudaStream_t stream);
cudaError_t launch_backtrack(const GraphDev& g, int64_t nnz, const int32_t* par, const MaskInfo* minfo,
                             int32_t full, Counters* ctr, int2* qa, int2* qb, int32_t* out_v, int3* out_e,
                             int32_t cap, cudaStream_t stream);

}  // namespace gst
