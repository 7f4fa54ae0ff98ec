// DPBF kernels for sm_103a: group masks, merge, growth round, argmin and
// backtrack. Plain SIMT integer code: the DP is min-plus over int32 costs
// and is bound by memory traffic and latency (growth) and the INT32 pipe
// (merge); nothing here is a contraction, so no tensor-core path applies.
//
// What each kernel replaces in the reference (src/DPQ.cu):
//   k_group_masks   set_max_ID / get_max (:22-47) — groups(v) as a bit mask
//   k_merge         the merge half of Relax (:286-314) and the seeding of
//                   T(v,p)=0 for p inside groups(v) (:638-659), done as one
//                   pass per DP wave over every vertex's submask splits
//   k_grow_*        dis0_init (:404-433) and the grow half of Relax
//                   (:259-282): one label-correcting round, pull form
//   k_argmin        host min scan over T(v,full) (:712-721)
//   k_backtrack     host BFS over parent records (:729-758)
#include <algorithm>
#include <climits>
#include <cstdint>

#include "dpbf.cuh"

namespace gst {

namespace {

__device__ __forceinline__ long long warp_sum_ll(long long x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

// Sums N per-thread counters over the block; the totals land in thread 0.
// Every thread of the block must call it.
template <int N>
__device__ __forceinline__ void block_sum(long long (&v)[N]) {
  __shared__ long long part[kGrowThreads / 32][N];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < N; ++i) v[i] = warp_sum_ll(v[i]);
  if (lane == 0) {
#pragma unroll
    for (int i = 0; i < N; ++i) part[warp][i] = v[i];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
#pragma unroll
      for (int i = 0; i < N; ++i) v[i] += part[w][i];
    }
  }
}

__device__ __forceinline__ void add_stat(long long* stats, int slot, long long x) {
  if (x) atomicAdd(reinterpret_cast<unsigned long long*>(stats + slot), static_cast<unsigned long long>(x));
}

// Largest cost allowed for state (v,S) under the bound: ub - LB(v, full^S)
// with LB = max over groups g outside S of dist(v, g) (one-label bound,
// src/DPQ.cu:361-403, applied per remaining group set). Under a bound, wave
// 1 grows only light states (2 * cost <= ub, see below), so T(v,{g}) is the
// exact distance when it is light and otherwise only known to exceed ub/2:
// min(T(v,{g}), ub/2 + 1) is a valid lower bound in both cases.
// -1 = state dead. The merges for k <= 8 add the tour bound (k_merge_staged);
// every merge writes the caps of its wave to the cap table, which growth
// reads (cap_at).
__device__ __forceinline__ int32_t prune_cap(const LevelArgs& a, int32_t ub, int32_t v, uint32_t S) {
  const int32_t* d = a.cost + (int64_t)v * a.stride1;  // wave 1 slice starts at 0; rank({g}) = g
  const int32_t beyond = ub / 2 + 1;
  int32_t lb = 0;
#pragma unroll
  for (int gg = 0; gg < 16; ++gg)  // predicated, so the loads overlap
    if (gg < a.k && !((S >> gg) & 1u)) lb = max(lb, min(__ldg(d + gg), beyond));
  const int32_t cap = ub - lb;
  return cap < 0 ? -1 : cap;
}

// Under a bound ub >= OPT, a state of cost c is "light" when 2c <= ub. An
// optimal tree has a vertex r (its weighted centroid) where every subtree
// hanging off r costs at most OPT/2, so it is derived from light states by
// growth and by merges of light states, except for the merges at r itself,
// whose last step joins a state with its complement (the rule of PrunedDP++,
// rucgraph/graph_v_of_v_idealID_PrunedDPPlusPlus.h:795). Hence: only light
// states grow; merges below the last wave use light parts only; the last
// wave merges any parts. Heavy states are kept for that last merge.
__device__ __forceinline__ int32_t light_or_inf(int32_t c, int32_t ub) {
  return (ub > 0 && 2 * c > ub) ? kInf : c;  // 2 * kInf < 2^31: no wrap
}

}  // namespace

// ------------------------------------------------------------ group masks --
__global__ void k_group_masks(const int32_t* __restrict__ group_ptr, const int32_t* __restrict__ members,
                              const int32_t* __restrict__ perm, int32_t k, uint32_t* __restrict__ gmask) {
  const int32_t n = group_ptr[k];
  for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    int32_t g = 0;
    while (g + 1 < k && group_ptr[g + 1] <= i) ++g;
    atomicOr(gmask + perm[members[i]], 1u << g);
  }
}

// Growth under a bound (waves >= 2): the cap of state (v, mask rank j) that
// the wave's merge wrote (read-only during the wave).
__device__ __forceinline__ int32_t cap_at(const LevelArgs& a, int32_t v, int j) {
  return __ldg(a.capt + (int64_t)v * a.stride + j);
}

// PrunedDP++'s conditional tree merging (graph_v_of_v_idealID_PrunedDPPlusPlus.h:
// 915-921): below the last wave, a merged state costing more than 2/3 of the
// bound is dropped. Exact for ub >= OPT: at the optimal tree's weighted
// centroid r every branch costs at most OPT/2, and the branches split into
// two sides of at most 2/3 OPT each, each side built from light merges
// (parts of at most OPT/2); the last wave joins the two sides. So no merge
// below the last wave needs a result above 2/3 OPT, and heavier merged
// states neither grow nor serve as lower-wave parts (light rules). The
// leaf states (cost 0) are never dropped. floor(2 ub / 3) without overflow.
__device__ __forceinline__ int32_t merged_keep(const LevelArgs& a, int32_t ub) {
  if (ub <= 0 || a.level >= a.k) return INT_MAX;
  return (ub / 3) * 2 + ((ub % 3) * 2) / 3;
}

// ------------------------------------------------------------------ merge --
// One thread per (v, slot) of the level's rows: T(v,S) = 0 when S is inside
// groups(v), else the best split T(v,S1) + T(v,S^S1) over S1 holding the
// lowest bit of S (each unordered split once); padding slots get kInf.
// Writes every entry of the level slice, marks vertices with a finite entry
// as changed in "round -1" (flag array 2, count slot 2) and makes round 0 a
// full sweep.
__global__ void __launch_bounds__(kGrowThreads) k_merge(GraphDev g, LevelArgs a) {
  const int64_t total = (int64_t)g.V * a.stride;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int32_t ub = (a.level >= 2) ? a.params->ub : 0;
  const int32_t ub_light = a.params->ub;
  const int32_t ovf_limit = a.params->ovf_limit;
  const int32_t keep23 = merged_keep(a, ub);
  const bool late = a.params->late_bound != 0;
  uint8_t* flag2 = a.flags + 2 * (int64_t)a.vpad;
  long long acc[3] = {0, 0, 0};  // finite states, splits, overflow
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += stride) {
    const int32_t v = (int32_t)(idx / a.stride);
    const int32_t j = (int32_t)(idx - (int64_t)v * a.stride);
    int32_t best = kInf;
    int32_t code = kLeaf;
    int32_t cap = -1;  // padding slots: nothing fits
    if (j < a.m) {
      const uint32_t S = (uint32_t)__ldg(a.lmasks + j);
      if ((__ldg(a.gmask + v) & S) == S) best = 0;
      // under a bound, a state whose lower bound alone exceeds it is dead:
      // no split needs enumerating
      cap = (ub > 0 && a.level >= 2) ? prune_cap(a, ub, v, S) : kInf;
      if (cap < 0) best = kInf;
      if (a.level >= 2 && best != 0 && cap >= 0) {
        const uint32_t low = S & (0u - S), rest = S ^ low;
        for (uint32_t sub = (rest - 1u) & rest;; sub = (sub - 1u) & rest) {
          const uint32_t s1 = sub | low, s2 = S ^ s1;
          const MaskInfo i1 = a.minfo[s1], i2 = a.minfo[s2];
          int32_t c1 = a.cost[(int64_t)i1.base * g.V + (int64_t)v * i1.stride + i1.rank];
          int32_t c2 = a.cost[(int64_t)i2.base * g.V + (int64_t)v * i2.stride + i2.rank];
          if (a.level < a.k) {
            c1 = light_or_inf(c1, ub_light);
            c2 = light_or_inf(c2, ub_light);
          }
          const int32_t c = c1 + c2;  // both <= kInf < 2^30: no wrap
          if (c1 < kInf && c2 < kInf) {
            if (c >= ovf_limit)
              acc[2] = 1;
            else if (c < best) {
              best = c;
              code = -(int32_t)s1;
            }
          }
          ++acc[1];
          if (sub == 0u) break;
        }
      }
      if (best < kInf && (best > cap || best > keep23)) {
        best = kInf;
        code = kLeaf;
      }
    }
    a.cost[a.base + idx] = best;
    a.par[a.base + idx] = code;
    if (ub > 0 || late) a.capt[idx] = cap;  // the growth of this wave prunes by it
    if (best < kInf) {
      flag2[v] = 1;
      ++acc[0];
    }
  }
  block_sum(acc);
  if (threadIdx.x == 0) {
    if (acc[0]) {
      atomicAdd(&a.ctl->changed[2], (int32_t)acc[0]);
      atomicAdd(&a.ctr->states, (unsigned long long)acc[0]);
    }
    if (a.params->stats_on) add_stat(a.stats, kStatSplits, acc[1]);
    if (acc[2]) atomicExch(&a.ctr->overflow, 1);
  }
}

// One thread per vertex (k <= kMergeTabK, at most kMergeTeamMinWords words
// of lower-level row per vertex, or a level of few masks over at most twice
// that: every wave of k <= 6, waves 2-3 of k = 7 and 8): the same states as k_merge, row by row. A thread copies its
// vertex's rows of levels 1..l-1 into shared memory once (light-filtered
// there when the merge uses light parts), a column per thread, and every
// split then reads two shared words at offsets precomputed into the block's
// copy of the split table (the level's split table, loaded once per block);
// the vertex's group mask is loaded once and its row written 16 bytes at a
// time. Blocks of NT = 128 threads (at most 64 KB of columns). Longer rows:
// k_merge_team.
constexpr int kMergeStagedWords = 256;  // the longest rows of k = 8 (teams of 4 up to here)

template <int NT>
__global__ void __launch_bounds__(NT) k_merge_staged(GraphDev g, LevelArgs a, MergeLevels ml) {
  extern __shared__ int32_t msm[];
  __shared__ int32_t loff[kMergeTabK + 1];  // level l's first word in a vertex's staged rows
  int32_t* sp = msm;                                            // m + 1
  int2* ss = reinterpret_cast<int2*>(msm + ((a.m + 2) & ~1));  // nsplits: staged word offsets x NT
  const int tn = a.k - a.level, te = tn + tn * (tn - 1) / 2;  // compact tour entries per mask
  int32_t* sct = reinterpret_cast<int32_t*>(ss + a.nsplits);    // a.m x te when a.tour
  int32_t* rows = sct + (a.tour ? a.m * te : 0);                // staged words x NT
  if (threadIdx.x == 0) {
    int32_t o = 0;
    for (int l = 1; l < a.level; ++l) {
      loff[l] = o;
      o += ml.stride[l];
    }
  }
  for (int i = threadIdx.x; i <= a.m; i += blockDim.x) sp[i] = a.msplit_ptr[i];
  __syncthreads();
  if (a.tour) {
    const int32_t* ct = a.tour + ((int64_t)a.k << a.k) * (a.k + 1);
    for (int i = threadIdx.x; i < a.m * te; i += blockDim.x) sct[i] = ct[i];
  }
  for (int i = threadIdx.x; i < a.nsplits; i += blockDim.x) {
    const int2 x = a.msplits[i];
    ss[i] = make_int2((loff[x.x >> 24] + (x.x & 0xffffff)) * NT, (loff[x.y >> 24] + (x.y & 0xffffff)) * NT);
  }
  __syncthreads();
  const int32_t ub = (a.level >= 2) ? a.params->ub : 0;
  const int32_t ub_light = a.params->ub;
  const int32_t ovf_limit = a.params->ovf_limit;
  const int32_t keep23 = merged_keep(a, ub);
  const bool late = a.params->late_bound != 0;
  const bool light_parts = a.level < a.k;
  uint8_t* flag2 = a.flags + 2 * (int64_t)a.vpad;
  long long acc[3] = {0, 0, 0};  // finite states, splits, overflow
  // staged costs are unsigned with "none" (kInf, or heavy when the merge
  // uses light parts) as kStagedInf = 3 * 2^30: a sum of two finite costs
  // (each below 2^30) stays below 2^31, any sum with a "none" is at least
  // 2^31, and no sum wraps, so a split is two loads, an add and a min
  constexpr uint32_t kStagedInf = 0xC0000000u;
  auto staged = [&](int32_t c) -> int32_t {
    return (int32_t)((light_parts ? light_or_inf(c, ub_light) : c) >= kInf ? kStagedInf : (uint32_t)c);
  };
  const int64_t v = (int64_t)blockIdx.x * NT + threadIdx.x;
  if (v < g.V) {
    int32_t* col = rows + threadIdx.x;
    const uint32_t* colu = reinterpret_cast<const uint32_t*>(col);
    for (int l = 1; l < a.level; ++l) {
      const int4* src = reinterpret_cast<const int4*>(a.cost + ml.off[l] + v * ml.stride[l]);
      int32_t* dst = col + loff[l] * NT;
      for (int q = 0; q < (ml.stride[l] >> 2); ++q) {
        const int4 t = src[q];
        dst[(4 * q) * NT] = staged(t.x);
        dst[(4 * q + 1) * NT] = staged(t.y);
        dst[(4 * q + 2) * NT] = staged(t.z);
        dst[(4 * q + 3) * NT] = staged(t.w);
      }
    }
    const uint32_t gm = __ldg(a.gmask + v);
    // the bounds read wave 1's distances from the staged level-1 row (words
    // 0..k-1): light ones are exact, the others exceed ub / 2, so
    // min(staged, ub / 2 + 1) is the capped one-label distance
    const uint32_t beyond = (uint32_t)(ub / 2 + 1);
    const uint32_t full = (1u << a.k) - 1u;
    int4* rowc = reinterpret_cast<int4*>(a.cost + a.base + v * a.stride);
    int4* rowp = reinterpret_cast<int4*>(a.par + a.base + v * a.stride);
    int4* rowk = reinterpret_cast<int4*>(a.capt + v * a.stride);
    bool any = false;
    for (int j0 = 0; j0 < a.stride; j0 += 4) {
      int32_t b4[4], c4[4], k4[4];
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        const int j = j0 + t;
        int32_t best = kInf, code = kLeaf;
        k4[t] = -1;  // padding slots: nothing fits
        if (j < a.m) {
          const uint32_t S = (uint32_t)__ldg(a.lmasks + j);
          if ((gm & S) == S) best = 0;
          const uint32_t X = full ^ S;
          // one-label bound: the farthest group of X (dmax)
          uint32_t dmax = 0u;
          if (ub > 0 && !(a.tour && __popc(X) >= 2))
            for (uint32_t xi = X; xi; xi &= xi - 1u) dmax = max(dmax, min(colu[(__ffs(xi) - 1) * NT], beyond));
          int32_t lb = (int32_t)dmax;
          if (ub > 0 && a.tour && __popc(X) >= 2) {
            // PrunedDP++'s tour bounds (graph_v_of_v_idealID_PrunedDPPlusPlus.h:
            // 268-386, 435-494): a tree joining v to the groups of X is at
            // least half a closed walk from v through all of them, over
            // lower bounds of every leg.
            //  lb1: the walk's first and last groups i != j, taken as
            //       unordered pairs i < j (the path table is symmetric, a
            //       path reversed; its i = j entries are no walks);
            //  lb2: the walk passes through every group i of X, so it costs
            //       at least d(v,i) + W2[i][X] (the cheapest order from i
            //       over X) + the distance back from the nearest group of X
            //  (halving is monotone, so each side halves its extreme sum once;
            //  every sum is at most ub / 2 + 1 + ub + ub / 2 + 1: unsigned, no wrap)
            // The path and W2 values of this mask come from the level's compact
            // table in shared memory, in the order its loops visit them.
            uint32_t p1 = 0xffffffffu, p2 = 0u, dmin = 0xffffffffu;
            const int32_t* tj = sct + j * te;
            int ai = 0, pi = tn;
            for (uint32_t xi = X; xi; xi &= xi - 1u, ++ai) {
              const int i = __ffs(xi) - 1;
              const uint32_t di = min(colu[i * NT], beyond);
              dmin = min(dmin, di);
              dmax = max(dmax, di);
              p2 = max(p2, di + (uint32_t)tj[ai]);
              for (uint32_t xj = xi & (xi - 1u); xj; xj &= xj - 1u, ++pi) {
                const int i2 = __ffs(xj) - 1;
                p1 = min(p1, di + (uint32_t)tj[pi] + min(colu[i2 * NT], beyond));
              }
            }
            lb = (int32_t)max(dmax, max(p1 >> 1, (p2 + dmin) >> 1));
          }
          const int32_t cap = ub > 0 ? ub - lb : kInf;
          k4[t] = cap < 0 ? -1 : cap;
          if (cap < 0) {
            best = kInf;
          } else if (best != 0) {
            uint32_t bu = 0xffffffffu;
            int win = -1;
            const int i1 = sp[j + 1];
            for (int i = sp[j]; i < i1; ++i) {
              const int2 x = ss[i];
              const uint32_t c = colu[x.x] + colu[x.y];
              if (c < bu) {
                bu = c;
                win = i;
              }
            }
            acc[1] += i1 - sp[j];
            if (bu < 0x80000000u) {  // both parts finite
              if (bu >= (uint32_t)ovf_limit) {
                acc[2] = 1;  // the cheapest tree reaches the cost limit
              } else {
                best = (int32_t)bu;
                const int2 x = a.msplits[win];
                code = -__ldg(ml.lmasks_all + ml.mbase[x.x >> 24] + (x.x & 0xffffff));
              }
            }
          }
          if (best < kInf && (best > cap || best > keep23)) {
            best = kInf;
            code = kLeaf;
          }
        }
        b4[t] = best;
        c4[t] = code;
        if (best < kInf) {
          any = true;
          ++acc[0];
        }
      }
      rowc[j0 >> 2] = make_int4(b4[0], b4[1], b4[2], b4[3]);
      rowp[j0 >> 2] = make_int4(c4[0], c4[1], c4[2], c4[3]);
      if (ub > 0 || late) rowk[j0 >> 2] = make_int4(k4[0], k4[1], k4[2], k4[3]);  // the growth of this wave prunes by it
    }
    if (any) flag2[v] = 1;
  }
  block_sum(acc);
  if (threadIdx.x == 0) {
    if (acc[0]) {
      atomicAdd(&a.ctl->changed[2], (int32_t)acc[0]);
      atomicAdd(&a.ctr->states, (unsigned long long)acc[0]);
    }
    if (a.params->stats_on) add_stat(a.stats, kStatSplits, acc[1]);
    if (acc[2]) atomicExch(&a.ctr->overflow, 1);
  }
}

// A team of T lanes per vertex, for the merges whose lower-level rows are
// too long to stage a thread per vertex at a useful occupancy: more than
// kMergeTeamMinWords words (waves 4 and up of k = 7 and 8, and k = 9, 10),
// where k_merge_staged keeps 8-16 warps per SM, unless the level has fewer
// than kMergeTeamMinMasks masks and at most twice that many words (the last
// merge of k = 6: one mask over 68 words, faster by a thread per vertex).
// The team copies its vertex's rows of levels 1..l-1 into its own slice of
// shared memory (consecutive words by consecutive lanes, light-filtered as
// in k_merge_staged), then evaluates the level's states. LANE_MASKS (a
// level of at least T masks): lane t of the team takes masks t, t + T, ...
// and scans each mask's splits alone. Otherwise the team takes the masks
// one by one and its lanes share each mask's splits; a minimum over
// (cost, split index) keeps the first cheapest split, as a sequential scan
// does. Bounds, caps, the 2/3 rule and the written rows are those of
// k_merge_staged. T = 4 up to 256 words (k <= 8: each lane keeps a
// quarter of the states, so lanes stay busy on levels of 7 to 70 masks,
// and a quarter of the staging per lane quadruples the blocks per SM),
// 32 beyond. Persistent blocks of kMergeTeamThreads threads stride over
// the vertices.
constexpr int kMergeTeamMinWords = 64;
constexpr int kMergeTeamMinMasks = 4;
constexpr int kMergeTeamThreads = 256;

template <int T, bool LANE_MASKS>
__global__ void __launch_bounds__(kMergeTeamThreads) k_merge_team(GraphDev g, LevelArgs a, MergeLevels ml,
                                                                  int32_t words) {
  static_assert(T >= 1 && T <= 32 && (T & (T - 1)) == 0, "teams are powers of two within a warp");
  constexpr int kTeams = kMergeTeamThreads / T;
  extern __shared__ int32_t msm[];
  __shared__ int32_t loff[kMergeTabK + 1];  // level l's first word in a vertex's staged rows
  int32_t* sp = msm;                                             // m + 1
  int2* ss = reinterpret_cast<int2*>(msm + ((a.m + 2) & ~1));   // nsplits: staged word offsets
  const int tn = a.k - a.level, te = tn + tn * (tn - 1) / 2;  // compact tour entries per mask
  int32_t* sct = reinterpret_cast<int32_t*>(ss + a.nsplits);    // a.m x te when a.tour
  uint32_t* rows = reinterpret_cast<uint32_t*>(sct + (a.tour ? a.m * te : 0));  // kTeams slices of (words | 1) words
  if (threadIdx.x == 0) {
    int32_t o = 0;
    for (int l = 1; l < a.level; ++l) {
      loff[l] = o;
      o += ml.stride[l];
    }
  }
  for (int i = threadIdx.x; i <= a.m; i += blockDim.x) sp[i] = a.msplit_ptr[i];
  __syncthreads();
  if (a.tour) {
    const int32_t* ct = a.tour + ((int64_t)a.k << a.k) * (a.k + 1);
    for (int i = threadIdx.x; i < a.m * te; i += blockDim.x) sct[i] = ct[i];
  }
  for (int i = threadIdx.x; i < a.nsplits; i += blockDim.x) {
    const int2 x = a.msplits[i];
    ss[i] = make_int2(loff[x.x >> 24] + (x.x & 0xffffff), loff[x.y >> 24] + (x.y & 0xffffff));
  }
  __syncthreads();
  const int32_t ub = a.params->ub;  // merges are waves >= 2
  const int32_t ovf_limit = a.params->ovf_limit;
  const int32_t keep23 = merged_keep(a, ub);
  const bool late = a.params->late_bound != 0;
  const bool light_parts = a.level < a.k;
  uint8_t* flag2 = a.flags + 2 * (int64_t)a.vpad;
  long long acc[3] = {0, 0, 0};  // finite states, splits, overflow
  constexpr uint32_t kStagedInf = 0xC0000000u;  // as in k_merge_staged
  const int team = threadIdx.x / T, lane = threadIdx.x % T;
  const unsigned tmask = T == 32 ? 0xffffffffu : ((1u << T) - 1u) << ((threadIdx.x & 31) & ~(T - 1));
  // an odd slice length puts the same word of the warp's teams in distinct banks
  uint32_t* col = rows + (int64_t)team * (words | 1);
  const uint32_t beyond = (uint32_t)(ub / 2 + 1);
  const uint32_t full = (1u << a.k) - 1u;
  // the cap of state S (mask rank j) at the staged vertex: ub minus the
  // one-label bound (wave 1's distances, words 0..k-1 of the staged rows)
  // or, with the tour tables (the level's compact table in shared memory),
  // the largest of the one-label and the two tour bounds; kInf without a
  // bound
  auto state_cap = [&](uint32_t S, int j) -> int32_t {
    if (ub <= 0) return kInf;
    const uint32_t X = full ^ S;
    uint32_t dmax = 0u;
    if (!(a.tour && __popc(X) >= 2)) {
      for (uint32_t xi = X; xi; xi &= xi - 1u) dmax = max(dmax, min(col[__ffs(xi) - 1], beyond));
      return ub - (int32_t)dmax;
    }
    uint32_t p1 = 0xffffffffu, p2 = 0u, dmin = 0xffffffffu;
    const int32_t* tj = sct + j * te;
    int ai = 0, pi = tn;
    for (uint32_t xi = X; xi; xi &= xi - 1u, ++ai) {
      const int i = __ffs(xi) - 1;
      const uint32_t di = min(col[i], beyond);
      dmin = min(dmin, di);
      dmax = max(dmax, di);
      p2 = max(p2, di + (uint32_t)tj[ai]);
      for (uint32_t xj = xi & (xi - 1u); xj; xj &= xj - 1u, ++pi) {
        const int i2 = __ffs(xj) - 1;
        p1 = min(p1, di + (uint32_t)tj[pi] + min(col[i2], beyond));
      }
    }
    return ub - (int32_t)max(dmax, max(p1 >> 1, (p2 + dmin) >> 1));
  };
  for (int64_t v = (int64_t)blockIdx.x * kTeams + team; v < g.V; v += (int64_t)gridDim.x * kTeams) {
    for (int l = 1; l < a.level; ++l) {
      const int32_t* src = a.cost + ml.off[l] + v * ml.stride[l];
      uint32_t* dst = col + loff[l];
      for (int w = lane; w < ml.stride[l]; w += T) {
        const int32_t c = src[w];
        dst[w] = (light_parts ? light_or_inf(c, ub) : c) >= kInf ? kStagedInf : (uint32_t)c;
      }
    }
    __syncwarp(tmask);
    const uint32_t gm = __ldg(a.gmask + v);
    int32_t* rowc = a.cost + a.base + v * a.stride;
    int32_t* rowp = a.par + a.base + v * a.stride;
    int32_t* rowk = a.capt + v * a.stride;
    bool any = false;
    if constexpr (LANE_MASKS) {
      for (int j = lane; j < a.stride; j += T) {
        int32_t best = kInf, code = kLeaf, capv = -1;  // padding slots: nothing fits
        if (j < a.m) {
          const uint32_t S = (uint32_t)__ldg(a.lmasks + j);
          if ((gm & S) == S) best = 0;
          const int32_t cap = state_cap(S, j);
          capv = cap < 0 ? -1 : cap;
          if (cap < 0) {
            best = kInf;
          } else if (best != 0) {
            uint32_t bu = 0xffffffffu;
            int win = -1;
            const int i1 = sp[j + 1];
            for (int i = sp[j]; i < i1; ++i) {
              const int2 x = ss[i];
              const uint32_t c = col[x.x] + col[x.y];
              if (c < bu) {
                bu = c;
                win = i;
              }
            }
            acc[1] += i1 - sp[j];
            if (bu < 0x80000000u) {  // both parts finite
              if (bu >= (uint32_t)ovf_limit) {
                acc[2] = 1;
              } else {
                best = (int32_t)bu;
                const int2 x = a.msplits[win];
                code = -__ldg(ml.lmasks_all + ml.mbase[x.x >> 24] + (x.x & 0xffffff));
              }
            }
          }
          if (best < kInf && (best > cap || best > keep23)) {
            best = kInf;
            code = kLeaf;
          }
        }
        rowc[j] = best;
        rowp[j] = code;
        if (ub > 0 || late) rowk[j] = capv;  // the growth of this wave prunes by it
        if (best < kInf) {
          any = true;
          ++acc[0];
        }
      }
    } else {
      for (int j = 0; j < a.stride; ++j) {  // the same j on every lane of the team
        int32_t best = kInf, code = kLeaf, capv = -1;
        if (j < a.m) {
          const uint32_t S = (uint32_t)__ldg(a.lmasks + j);
          if ((gm & S) == S) best = 0;
          const int32_t cap = state_cap(S, j);
          capv = cap < 0 ? -1 : cap;
          if (cap < 0) {
            best = kInf;
          } else if (best != 0) {
            unsigned long long key = ~0ull;
            const int i0 = sp[j], i1 = sp[j + 1];
            for (int i = i0 + lane; i < i1; i += T) {
              const int2 x = ss[i];
              const unsigned long long kk = ((unsigned long long)(col[x.x] + col[x.y]) << 32) | (uint32_t)i;
              key = kk < key ? kk : key;
            }
#pragma unroll
            for (int o = T / 2; o > 0; o >>= 1) {
              const unsigned long long y = __shfl_xor_sync(tmask, key, o);
              key = y < key ? y : key;
            }
            if (lane == 0) acc[1] += i1 - i0;
            const uint32_t bu = (uint32_t)(key >> 32);
            if (key != ~0ull && bu < 0x80000000u) {  // both parts finite
              if (bu >= (uint32_t)ovf_limit) {
                acc[2] = 1;
              } else {
                best = (int32_t)bu;
                const int2 x = a.msplits[(int)(key & 0xffffffffull)];
                code = -__ldg(ml.lmasks_all + ml.mbase[x.x >> 24] + (x.x & 0xffffff));
              }
            }
          }
          if (best < kInf && (best > cap || best > keep23)) {
            best = kInf;
            code = kLeaf;
          }
        }
        if (lane == 0) {
          rowc[j] = best;
          rowp[j] = code;
          if (ub > 0 || late) rowk[j] = capv;
          if (best < kInf) ++acc[0];
        }
        any = any || best < kInf;
      }
    }
    any = __any_sync(tmask, any);
    if (lane == 0 && any) flag2[v] = 1;
    __syncwarp(tmask);  // the slice is rewritten for the next vertex
  }
  block_sum(acc);
  if (threadIdx.x == 0) {
    if (acc[0]) {
      atomicAdd(&a.ctl->changed[2], (int32_t)acc[0]);
      atomicAdd(&a.ctr->states, (unsigned long long)acc[0]);
    }
    if (a.params->stats_on) add_stat(a.stats, kStatSplits, acc[1]);
    if (acc[2]) atomicExch(&a.ctr->overflow, 1);
  }
}


// ------------------------------------------------------------------- grow --
// One label-correcting round for every mask of the level, pull form: each
// candidate vertex u takes min over neighbours v changed in the previous
// round of T(v,S) + w(u,v), for all masks S of the level at once (a row is
// contiguous). Only u's thread(s) write u's row, so a state's cost and its
// parent are always written together (the reference writes the parent after
// a separate atomicMin, DPQ.cu:269-272).
//
// Sparse rounds: an improved vertex marks its neighbours as the next round's
// candidates and only candidates are processed. Dense rounds (the previous
// round changed more than V/8 vertices): every vertex is processed, every
// neighbour row is gathered without consulting the change flags, and no
// candidates are marked (the next round then sweeps every vertex).
//
// Mappings:
//   k_grow_thread<MP>  waves with row stride MP <= 24: one thread per
//                      vertex holds its whole row in registers and gathers
//                      U neighbour rows at a time with int4 loads;
//   k_grow_group<G,L>  wider waves: G lanes per vertex, lane j holding masks
//                      j, j+G, ... (L per lane), neighbour rows gathered four
//                      at a time;
//   hubs (degree > g.deg_big) in both: 32-entry chunks of hub rows taken by
//                      any warp, minima folded into a per-hub scratch row,
//                      applied by the warp that finishes the hub's last chunk.
// The last block to finish publishes the round's change count, advances
// the round and, inside a captured CUDA graph, sets the while condition.
namespace {

constexpr int kGatherUnroll = 4;
constexpr int kDenseGrab = 32;  // sweep positions a warp takes at a time in dense rounds (one per lane)

struct RoundState {
  int32_t r;
  int32_t prev;  // vertices the previous round changed
  bool dense, all_cand, stats;
  int32_t ub;        // pruning bound (waves >= 2; states are capped by the wave's cap table)
  int32_t ub_light;  // only states with 2 * cost <= ub_light grow (all waves)
  int32_t ovf_limit;  // stored costs must stay below this (kInf - largest weight)
  const uint8_t* cur_flag;
  uint8_t* next_flag;
  uint8_t* clear_flag;
  const uint8_t* cand_cur;
  uint8_t* cand_next;
  uint8_t* cand_clear;
};

// Per-thread counters: changed rows, improved entries, vertices, CSR
// entries, rows gathered, candidate marks, overflow.
enum { kAccChanged, kAccImproved, kAccVert, kAccEnt, kAccRows, kAccMarks, kAccOverflow, kAccN };

__device__ __forceinline__ bool round_begin(const GraphDev& g, const LevelArgs& a, RoundState& rs) {
  const GrowCtl* ctl = a.ctl;
  // the round and every rotating slot load together (one step), then the
  // previous round's slots are selected
  rs.r = ctl->round;
  const int32_t c0 = ctl->changed[0], c1 = ctl->changed[1], c2 = ctl->changed[2];
  const int32_t d0 = ctl->dense[0], d1 = ctl->dense[1], d2 = ctl->dense[2];
  const int32_t timeout = ctl->timeout;
  const int32_t dense_shift = a.params->dense_shift, stats_on = a.params->stats_on, ub = a.params->ub,
                ovf_limit = a.params->ovf_limit;
  const int pi = (rs.r + 2) % 3;
  const int32_t prev = pi == 0 ? c0 : pi == 1 ? c1 : c2;
  const int32_t prev_dense = pi == 0 ? d0 : pi == 1 ? d1 : d2;
  rs.prev = prev;
  // converged (nothing changed in the previous round), or out of rounds: a
  // later kernel of the same pass must not run another round
  if ((prev == 0) | (timeout != 0)) {
    if (a.use_cond && blockIdx.x == 0 && threadIdx.x == 0) cudaGraphSetConditional(a.cond, 0);
    return false;
  }
  rs.dense = prev > (g.V >> dense_shift);
  rs.all_cand = rs.dense || prev_dense != 0;
  rs.stats = stats_on != 0;
  rs.ub = a.level >= 2 ? ub : 0;  // wave 1 is the bound's own input: not pruned by it
  rs.ub_light = ub;
  rs.ovf_limit = ovf_limit;
  const int64_t P = a.vpad;  // flag arrays are padded to keep word atomics aligned
  rs.cur_flag = a.flags + (int64_t)((rs.r + 2) % 3) * P;
  rs.next_flag = a.flags + (int64_t)(rs.r % 3) * P;
  rs.clear_flag = a.flags + (int64_t)((rs.r + 1) % 3) * P;
  rs.cand_cur = a.cand + (int64_t)(rs.r % 3) * P;
  rs.cand_next = a.cand + (int64_t)((rs.r + 1) % 3) * P;
  rs.cand_clear = a.cand + (int64_t)((rs.r + 2) % 3) * P;
  return true;
}

// Zeroes the change flags of two rounds back and the candidate flags of the
// last round (vpad bytes each, 16-byte aligned) with 16-byte stores.
__device__ __forceinline__ void clear_flags(const LevelArgs& a, const RoundState& rs, int64_t t0, int64_t nthreads) {
  uint4* f = reinterpret_cast<uint4*>(rs.clear_flag);
  uint4* c = reinterpret_cast<uint4*>(rs.cand_clear);
  const uint4 z = make_uint4(0u, 0u, 0u, 0u);
  for (int64_t i = t0; i < ((int64_t)a.vpad >> 4); i += nthreads) {
    f[i] = z;
    c[i] = z;
  }
}

// Makes v a candidate of the next round (an idempotent byte store).
__device__ __forceinline__ void mark_candidate(uint8_t* cand, int32_t v, uint32_t (&acc)[kAccN]) {
  cand[v] = 1;
  ++acc[kAccMarks];
}

// Does some entry j of vals (light-filtered costs of the marking vertex,
// edge weight w still to add) improve vertex v's entry y(j)? With a bound
// the improved value must also pass v's cap for mask j (the wave's cap
// table). Masks go in passes of 32: the comparisons of a pass are
// independent (their loads overlap) and leave a bit set per improved mask;
// v's caps are loaded only for set bits.
template <class Vals, class Row>
__device__ __forceinline__ bool improves_row(const LevelArgs& a, int32_t ub, int32_t v, int32_t w, const Vals& vals,
                                             const Row& y, int m) {
  for (int j0 = 0; j0 < m; j0 += 32) {
    const int n = min(32, m - j0);
    uint32_t bits = 0;
#pragma unroll 8
    for (int jj = 0; jj < n; ++jj) bits |= (vals(j0 + jj) + w < y(j0 + jj) ? 1u : 0u) << jj;
    if (!bits) continue;
    if (ub <= 0) return true;
    bool ok = false;  // the caps of the improved masks, loaded together
#pragma unroll 8
    for (int jj = 0; jj < n; ++jj)
      if ((bits >> jj) & 1u) ok |= vals(j0 + jj) + w <= cap_at(a, v, j0 + jj);
    if (ok) return true;
  }
  return false;
}

// Block-level accumulators of a growth round: every warp folds its counters
// in and the last warp of the block to arrive publishes them, so no warp of
// the block waits at a barrier for the slowest one.
struct BlockAcc {
  unsigned long long v[kAccN];
  unsigned int warps_done;
};

__device__ __forceinline__ void block_acc_init(BlockAcc& ba) {
  if (threadIdx.x < kAccN) ba.v[threadIdx.x] = 0ull;
  if (threadIdx.x == 0) ba.warps_done = 0u;
  __syncthreads();
}

// Folds the block's counters into the round totals; true in the one thread
// of the block that did so (after every warp of the block has arrived).
__device__ __forceinline__ bool round_flush(const LevelArgs& a, const RoundState& rs, uint32_t (&acc)[kAccN],
                                            BlockAcc& ba) {
  const int lane = threadIdx.x & 31;
  long long tot[kAccN];
#pragma unroll
  for (int i = 0; i < kAccN; ++i) tot[i] = warp_sum_ll((long long)acc[i]);
  int last = 0;
  if (lane == 0) {
#pragma unroll
    for (int i = 0; i < kAccN; ++i)
      if (tot[i]) atomicAdd(&ba.v[i], (unsigned long long)tot[i]);
    __threadfence_block();
    last = atomicAdd(&ba.warps_done, 1u) == (blockDim.x >> 5) - 1;
  }
  if (!last) return false;
  __threadfence_block();
#pragma unroll
  for (int i = 0; i < kAccN; ++i) tot[i] = (long long)atomicAdd(&ba.v[i], 0ull);
  GrowCtl* ctl = a.ctl;
  if (tot[kAccChanged]) atomicAdd(&ctl->changed[rs.r % 3], (int32_t)tot[kAccChanged]);
  if (tot[kAccImproved]) atomicAdd(&a.ctr->states, (unsigned long long)tot[kAccImproved]);
  if (tot[kAccOverflow]) atomicExch(&a.ctr->overflow, 1);
  if (rs.stats) {
    const long long m = a.m, s = a.stride;
    add_stat(a.stats, kStatVertices, tot[kAccVert]);
    add_stat(a.stats, kStatEntries, tot[kAccEnt]);
    add_stat(a.stats, kStatRows, tot[kAccRows]);
    add_stat(a.stats, kStatGathered, tot[kAccRows] * m);
    add_stat(a.stats, kStatImproved, tot[kAccImproved]);
    // algorithmic bytes: per processed vertex the row_ptr pair, its own row
    // and its candidate byte; per CSR entry scanned (col,w) and, in sparse
    // rounds, the change flag; one neighbour row per gather; the parent per
    // improved entry, the row rewritten and a change flag per changed row;
    // (col,w) + a candidate byte per mark
    const long long flag_bytes = rs.dense ? 0 : 1;
    add_stat(a.stats, kStatBytes,
             tot[kAccVert] * (9 + 4 * s) + tot[kAccEnt] * (8 + flag_bytes) + tot[kAccRows] * 4 * s +
                 tot[kAccImproved] * 4 + tot[kAccChanged] * (4 * s + 1) + tot[kAccMarks] * 9);
  }
  return true;
}

// round_flush, then the last block of the round kernel publishes the
// round's change count and advances the round.
__device__ __forceinline__ void round_end(const LevelArgs& a, const RoundState& rs, uint32_t (&acc)[kAccN],
                                          BlockAcc& ba) {
  if (!round_flush(a, rs, acc, ba)) return;
  GrowCtl* ctl = a.ctl;
  __threadfence();
  const uint32_t t = atomicAdd(&ctl->done, 1u);
  if (t != gridDim.x - 1) return;
  // last block of the round
  __threadfence();
  const int32_t total = atomicAdd(&ctl->changed[rs.r % 3], 0);
  ctl->dense[rs.r % 3] = rs.dense ? 1 : 0;
  ctl->last_changed = total;
  ctl->changed[(rs.r + 1) % 3] = 0;
  ctl->work[(rs.r + 1) % 3] = 0u;
  ctl->done = 0u;
  ctl->round = rs.r + 1;
  atomicAdd(&a.ctr->rounds_total, 1);
  if (rs.stats) add_stat(a.stats, kStatRounds, 1);
  const bool more = total > 0 && rs.r + 1 < a.params->max_rounds;
  if (total > 0 && !more) {
    ctl->timeout = 1;
    a.ctr->timeout = 1;
  }
  if (a.use_cond) cudaGraphSetConditional(a.cond, more ? 1u : 0u);
}

// Relaxes a group's running minima against CSR entries [e0, e0 + G) of the
// current row (mask chunk jc).
template <int G, int L>
__device__ __forceinline__ void group_relax(const GraphDev& g, const LevelArgs& a, const RoundState& rs, int32_t e0,
                                            int32_t end, int jc, int glane, int gbase, unsigned gmask_lanes,
                                            unsigned gbits, int32_t (&best)[L], int32_t (&code)[L],
                                            uint32_t (&acc)[kAccN]) {
  const int32_t e = e0 + glane;
  int32_t nv = 0, nw = 0;
  bool act = false;
  if (e < end) {
    const int2 x = g.adj[e];
    nv = x.x;
    nw = x.y;
    act = rs.dense || rs.cur_flag[nv] != 0;
  }
  unsigned bal = (__ballot_sync(gmask_lanes, act) >> gbase) & gbits;
  if (glane == 0) acc[kAccRows] += __popc(bal);
  const int32_t s = a.stride;
  while (bal) {
    int src[kGatherUnroll];
#pragma unroll
    for (int i = 0; i < kGatherUnroll; ++i) {
      src[i] = bal ? __ffs(bal) - 1 : -1;
      bal &= bal - 1u;
    }
    int32_t vv[kGatherUnroll], ww[kGatherUnroll];
#pragma unroll
    for (int i = 0; i < kGatherUnroll; ++i) {
      const int sl = src[i] < 0 ? 0 : src[i];
      vv[i] = __shfl_sync(gmask_lanes, nv, sl, G);
      ww[i] = __shfl_sync(gmask_lanes, nw, sl, G);
    }
    // every load is issued unconditionally at an address inside row vv[i]
    // (entries past the row's end read its last entry; slots without a
    // source read the row of the group's first lane), so all of them are in
    // flight together whatever registers the compiler assigns; the unwanted
    // values are masked afterwards
    int32_t c[kGatherUnroll][L];
#pragma unroll
    for (int i = 0; i < kGatherUnroll; ++i) {
      const int32_t* rowv = a.cost + a.base + (int64_t)vv[i] * s;
#pragma unroll
      for (int t = 0; t < L; ++t) c[i][t] = rowv[min(jc + glane + t * G, s - 1)];
    }
#pragma unroll
    for (int i = 0; i < kGatherUnroll; ++i) {
#pragma unroll
      for (int t = 0; t < L; ++t)
        c[i][t] = (src[i] >= 0 && jc + glane + t * G < s) ? light_or_inf(c[i][t], rs.ub_light) : kInf;
    }
#pragma unroll
    for (int i = 0; i < kGatherUnroll; ++i) {
#pragma unroll
      for (int t = 0; t < L; ++t) {
        int32_t x = c[i][t];
        if (x < kInf) {
          x += ww[i];  // both < 2^30: no wrap
          if (x >= rs.ovf_limit)
            acc[kAccOverflow] = 1;
          else if (x < best[t]) {
            best[t] = x;
            code[t] = e0 + src[i];
          }
        }
      }
    }
  }
}

// Hub rows (degree > g.deg_big) are cut into 32-entry chunks that any warp
// may take. A warp relaxes its chunk for every mask (lane j holds masks
// j, j+32, ...), folds each lane's minimum into the hub's scratch row with
// a 64-bit atomicMin of (cost << 32 | CSR entry), and counts the chunk as
// done; the warp that finishes a hub's last chunk applies the scratch row
// to the hub's state row (its single writer), clears the scratch row and
// the counter for the next round and flags the hub as changed. No warp
// ever waits for another. This runs as a kernel of its own before the
// round kernel, which then marks the changed hubs' neighbours chunk by
// chunk (hub_mark), so no single warp walks a whole hub row.
template <int L>
__device__ __forceinline__ void hub_chunk_relax(const GraphDev& g, const LevelArgs& a, const RoundState& rs,
                                                int64_t c, uint32_t (&acc)[kAccN]) {
  constexpr int G = 32;
  constexpr int CH = G * L;
  const int lane = threadIdx.x & 31;
  const int32_t s = a.stride;
  const int32_t u = g.chunk_vtx[c];
  const int2 hc = g.hub_chunk[c];  // (hub index, first CSR entry of the chunk)
  const int32_t beg = g.row_ptr[u], end = g.row_ptr[u + 1];
  const int32_t cend = min(end, hc.y + G);
  unsigned long long* hm = g.hub_min + (int64_t)hc.x * g.hub_stride;
  bool folded = false;  // this lane folded a minimum into the scratch row
  for (int jc = 0; jc < s; jc += CH) {
    int32_t best[L], code[L];
#pragma unroll
    for (int t = 0; t < L; ++t) {
      best[t] = kInf;
      code[t] = -1;
    }
    group_relax<G, L>(g, a, rs, hc.y, cend, jc, lane, 0, 0xffffffffu, 0xffffffffu, best, code, acc);
#pragma unroll
    for (int t = 0; t < L; ++t) {
      const int j = jc + lane + t * G;
      if (j < s && best[t] < kInf) {
        atomicMin(hm + j, ((unsigned long long)(uint32_t)best[t] << 32) | (uint32_t)code[t]);
        folded = true;
      }
    }
  }
  if (lane == 0) acc[kAccEnt] += cend - hc.y;
  // the folded minima must be visible before the chunk counts as done; a
  // chunk that folded nothing has nothing to order
  if (__any_sync(0xffffffffu, folded)) __threadfence();
  int last = 0;
  if (lane == 0) last = atomicAdd(g.hub_cnt + hc.x, 1) == (end - beg + G - 1) / G - 1;
  last = __shfl_sync(0xffffffffu, last, 0);
  if (!last) return;
  __threadfence();
  const int64_t rowu = a.base + (int64_t)u * s;
  bool imp = false;
  for (int j = lane; j < s; j += G) {
    const unsigned long long r = atomicExch(hm + j, ~0ull);  // read and clear
    if (j >= a.m || r == ~0ull) continue;
    const int32_t c2 = (int32_t)(r >> 32);
    const int32_t own = a.cost[rowu + j];
    if (c2 >= own) continue;
    if (rs.ub > 0 && c2 > cap_at(a, u, j)) continue;
    a.cost[rowu + j] = c2;
    a.par[rowu + j] = (int32_t)(uint32_t)(r & 0xffffffffull);
    imp = true;
    ++acc[kAccImproved];
  }
  if (lane == 0) {
    atomicExch(g.hub_cnt + hc.x, 0);
    ++acc[kAccVert];
  }
  if (__ballot_sync(0xffffffffu, imp) && lane == 0) {
    rs.next_flag[u] = 1;
    ++acc[kAccChanged];
  }
}

// A warp takes chunks warp, warp + W, warp + 2W, ... (W warps in the
// grid); its lanes test 32 of them for candidacy at once and the warp
// relaxes the candidate ones in turn.
template <int L>
__device__ __forceinline__ void hub_relax(const GraphDev& g, const LevelArgs& a, const RoundState& rs,
                                          uint32_t (&acc)[kAccN]) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t c0 = warp; c0 < g.nchunks; c0 += 32 * nwarps) {
    const int64_t cl = c0 + lane * nwarps;
    const bool want = cl < g.nchunks && (rs.all_cand || rs.cand_cur[g.chunk_vtx[cl]] != 0);
    unsigned bal = __ballot_sync(0xffffffffu, want);
    while (bal) {
      const int64_t c = c0 + (int64_t)(__ffs(bal) - 1) * nwarps;
      bal &= bal - 1u;
      hub_chunk_relax<L>(g, a, rs, c, acc);
    }
  }
}

// Hub rows of waves with stride 4G <= kMaxTeamStride, relaxed a segment of
// up to kHubSeg entries per warp. The warp compacts the segment's active
// entries into shared memory 32 at a time (dense rounds: all of them, in
// order; sparse rounds: those whose neighbour changed, found after loading
// every entry of the segment and its change flag at once), then splits into 32/GP
// teams of GP lanes (GP = G rounded up to a power of two; lanes G .. GP-1
// of a team idle); team t takes active entries t, t + T, ... four at a
// time, lane q loading the 16-byte quarter q of each neighbour's row, so up
// to 32 rows are in flight, and folds them into running minima held in
// registers. At the end the teams' minima are combined by shuffles. A hub
// of one segment (degree <= kHubSeg: almost every hub) is then applied to
// its row directly by team 0, its only writer; the segments of a larger
// hub fold into the hub's scratch row and the last one to finish applies
// it, as in hub_chunk_relax.
template <int GP, bool DENSE>
__device__ __forceinline__ void hub_seg_team(const GraphDev& g, const LevelArgs& a, const RoundState& rs,
                                             int64_t sidx, int4* wbuf, uint32_t (&acc)[kAccN]) {
  constexpr int T = 32 / GP;
  const int lane = threadIdx.x & 31;
  const int team = lane / GP, glane = lane - team * GP;
  const int G = a.stride >> 2;
  const int32_t s = a.stride;
  const int4 sg = g.hub_seg[sidx];  // (hub vertex, hub index, first entry, segments of the hub)
  const int32_t u = sg.x;
  const int32_t e1 = min(g.row_ptr[u + 1], sg.z + kHubSeg);
  int32_t best[4] = {kInf, kInf, kInf, kInf};
  int32_t code[4] = {-1, -1, -1, -1};
  const bool on = glane < G;
  const int4* tab = reinterpret_cast<const int4*>(a.cost + a.base);
  int32_t rows = 0;
  // folds the n entries compacted in wbuf into the teams' minima
  auto gather = [&](int n) {
    for (int i0 = team; i0 < n; i0 += 4 * T) {
      int4 it[4], r[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) it[q] = wbuf[min(i0 + q * T, n - 1)];
#pragma unroll
      for (int q = 0; q < 4; ++q) r[q] = on ? tab[(int64_t)it[q].x * G + glane] : make_int4(kInf, kInf, kInf, kInf);
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        if (i0 + q * T >= n) continue;
        const int32_t rv[4] = {r[q].x, r[q].y, r[q].z, r[q].w};
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          const int32_t cc = light_or_inf(rv[t], rs.ub_light) + it[q].y;  // both < 2^30: no wrap
          if (cc < best[t]) {
            best[t] = cc;
            code[t] = it[q].z;
          }
        }
      }
    }
    __syncwarp();  // wbuf is rewritten next
  };
  if (DENSE) {
    for (int32_t e0 = sg.z; e0 < e1; e0 += 32) {
      const int32_t e = e0 + lane;
      if (e < e1) {
        const int2 x = g.adj[e];
        wbuf[lane] = make_int4(x.x, x.y, e, 0);
      }
      __syncwarp();
      const int n = min(32, e1 - e0);
      rows += n;
      gather(n);
    }
  } else {
    // a sparse round: the segment's CSR entries and their change flags are
    // loaded for the whole segment first (lane l holds entries l, l + 32,
    // ...), then only the changed neighbours are compacted, up to 32 at a
    // time, and gathered: a segment with few changed neighbours costs two
    // loads deep instead of two per 32 entries
    constexpr int NI = kHubSeg / 32;
    int2 xs[NI];
#pragma unroll
    for (int i = 0; i < NI; ++i) {
      const int32_t e = sg.z + 32 * i + lane;
      xs[i] = e < e1 ? g.adj[e] : make_int2(-1, 0);
    }
    uint32_t am = 0;
#pragma unroll
    for (int i = 0; i < NI; ++i)
      if (xs[i].x >= 0 && rs.cur_flag[xs[i].x] != 0) am |= 1u << i;
    int n = 0;
#pragma unroll
    for (int i = 0; i < NI; ++i) {
      const bool act = (am >> i) & 1u;
      const unsigned bal = __ballot_sync(0xffffffffu, act);
      if (!bal) continue;
      const int c = __popc(bal);
      if (n + c > 32) {
        gather(n);
        n = 0;
      }
      if (act) wbuf[n + __popc(bal & ((1u << lane) - 1u))] = make_int4(xs[i].x, xs[i].y, sg.z + 32 * i + lane, 0);
      __syncwarp();
      n += c;
      rows += c;
    }
    if (n) gather(n);
  }
#pragma unroll
  for (int off = GP; off < 32; off <<= 1) {
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int32_t ob = __shfl_xor_sync(0xffffffffu, best[t], off);
      const int32_t oc = __shfl_xor_sync(0xffffffffu, code[t], off);
      if (ob < best[t] || (ob == best[t] && (uint32_t)oc < (uint32_t)code[t])) {
        best[t] = ob;
        code[t] = oc;
      }
    }
  }
  if (lane == 0) {
    acc[kAccEnt] += e1 - sg.z;
    acc[kAccRows] += rows;
  }
  const int64_t rowu = a.base + (int64_t)u * s;
  if (sg.w == 1) {
    // the whole row in this warp: apply it directly (team 0 holds the minima)
    bool imp = false;
    if (team == 0 && on) {
      const int4 own4 = tab[(int64_t)u * G + glane];
      const int32_t own[4] = {own4.x, own4.y, own4.z, own4.w};
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        const int j = 4 * glane + t;
        if (j >= a.m || best[t] >= own[t]) continue;
        if (best[t] >= rs.ovf_limit) acc[kAccOverflow] = 1;
        if (rs.ub > 0 && best[t] > cap_at(a, u, j)) continue;
        a.cost[rowu + j] = best[t];
        a.par[rowu + j] = code[t];
        imp = true;
        ++acc[kAccImproved];
      }
    }
    if (lane == 0) ++acc[kAccVert];
    if (__ballot_sync(0xffffffffu, imp) && lane == 0) {
      rs.next_flag[u] = 1;
      ++acc[kAccChanged];
    }
    return;
  }
  unsigned long long* hm = g.hub_min + (int64_t)sg.y * g.hub_stride;
  bool folded = false;
  if (team == 0 && on) {
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      if (best[t] >= kInf) continue;
      if (best[t] >= rs.ovf_limit) acc[kAccOverflow] = 1;
      atomicMin(hm + 4 * glane + t, ((unsigned long long)(uint32_t)best[t] << 32) | (uint32_t)code[t]);
      folded = true;
    }
  }
  // the folded minima must be visible before the segment counts as done; a
  // segment that folded nothing has nothing to order
  if (__any_sync(0xffffffffu, folded)) __threadfence();
  int last = 0;
  if (lane == 0) last = atomicAdd(g.hub_cnt + sg.y, 1) == sg.w - 1;
  last = __shfl_sync(0xffffffffu, last, 0);
  if (!last) return;
  __threadfence();
  bool imp = false;
  for (int j = lane; j < s; j += 32) {
    const unsigned long long r = atomicExch(hm + j, ~0ull);  // read and clear
    if (j >= a.m || r == ~0ull) continue;
    const int32_t c2 = (int32_t)(r >> 32);
    const int32_t own = a.cost[rowu + j];
    if (c2 >= own) continue;
    if (rs.ub > 0 && c2 > cap_at(a, u, j)) continue;
    a.cost[rowu + j] = c2;
    a.par[rowu + j] = (int32_t)(uint32_t)(r & 0xffffffffull);
    imp = true;
    ++acc[kAccImproved];
  }
  if (lane == 0) {
    atomicExch(g.hub_cnt + sg.y, 0);
    ++acc[kAccVert];
  }
  if (__ballot_sync(0xffffffffu, imp) && lane == 0) {
    rs.next_flag[u] = 1;
    ++acc[kAccChanged];
  }
}

// hub_relax for waves with stride <= kMaxTeamStride: a warp takes segments
// warp, warp + W, ... (W warps in the grid), its lanes test 32 of them for
// candidacy at once and the warp relaxes the candidate ones in turn.
template <int GP, bool DENSE>
__device__ __forceinline__ void hub_relax_team(const GraphDev& g, const LevelArgs& a, const RoundState& rs,
                                               uint32_t (&acc)[kAccN]) {
  __shared__ int4 hbuf[kGrowThreads / 32][32];
  int4* wbuf = hbuf[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t c0 = warp; c0 < g.nsegs; c0 += 32 * nwarps) {
    const int64_t cl = c0 + lane * nwarps;
    const bool want = cl < g.nsegs && (rs.all_cand || rs.cand_cur[g.hub_seg[cl].x] != 0);
    unsigned bal = __ballot_sync(0xffffffffu, want);
    while (bal) {
      const int64_t c = c0 + (int64_t)(__ffs(bal) - 1) * nwarps;
      bal &= bal - 1u;
      hub_seg_team<GP, DENSE>(g, a, rs, c, wbuf, acc);
    }
  }
}

// Sparse rounds: for every hub that changed in this round's hub kernel, the
// warp that takes one of its 32-entry chunks marks the chunk's neighbours
// that the hub's new row improves (within their bound). Lanes read the
// hub's row at the same addresses (broadcast loads).
__device__ __forceinline__ void hub_mark(const GraphDev& g, const LevelArgs& a, const RoundState& rs,
                                         uint32_t (&acc)[kAccN]) {
  if (rs.dense) return;
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int32_t s = a.stride;
  for (int64_t c0 = warp; c0 < g.nchunks; c0 += 32 * nwarps) {  // chunks taken as in hub_relax
    const int64_t cl = c0 + lane * nwarps;
    const bool want = cl < g.nchunks && rs.next_flag[g.chunk_vtx[cl]] != 0;
    unsigned bal = __ballot_sync(0xffffffffu, want);
    while (bal) {
      const int64_t c = c0 + (int64_t)(__ffs(bal) - 1) * nwarps;
      bal &= bal - 1u;
      const int32_t u = g.chunk_vtx[c];
      const int2 hc = g.hub_chunk[c];
      const int32_t e = hc.y + lane;
      if (e >= g.row_ptr[u + 1]) continue;
      const int2 x = g.adj[e];
      const int32_t* hv = a.cost + a.base + (int64_t)u * s;
      const int32_t* yv = a.cost + a.base + (int64_t)x.x * s;
      if (improves_row(a, rs.ub, x.x, x.y, [&](int j) { return light_or_inf(hv[j], rs.ub_light); },
                       [&](int j) { return yv[j]; }, a.m))
        mark_candidate(rs.cand_next, x.x, acc);
    }
  }
}

}  // namespace

// --------------------------------------------------------------- seeding --
// Chooses how round 0 of a wave starts. When the merge left more than
// V >> dense_shift vertices with a finite state, round 0 is dense.
// Otherwise only neighbours that a light finite merged state can improve
// (within their bound) become round 0's candidates. Hub rows are walked a
// 32-entry chunk per warp; the other vertices 32 at a time per warp, which
// finds those with a light state by ballot and walks each one's (at most
// g.deg_big) neighbours with its 32 lanes.
__global__ void __launch_bounds__(kGrowThreads) k_seed(GraphDev g, LevelArgs a) {
  GrowCtl* ctl = a.ctl;
  if (ctl->changed[2] > (g.V >> a.params->dense_shift)) {
    if (blockIdx.x == 0 && threadIdx.x == 0) ctl->dense[2] = 1;
    return;
  }
  const int32_t ub_light = a.params->ub;
  const int32_t ub = a.level >= 2 ? a.params->ub : 0;
  uint8_t* cand0 = a.cand;  // candidates of round 0
  uint32_t acc[kAccN] = {0, 0, 0, 0, 0, 0, 0};
  const int32_t s = a.stride;
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  auto seed_entry = [&](const int32_t* hv, int32_t e) {
    const int2 x = g.adj[e];
    const int32_t* yu = a.cost + a.base + (int64_t)x.x * s;
    if (improves_row(a, ub, x.x, x.y, [&](int j) { return light_or_inf(hv[j], ub_light); },
                     [&](int j) { return yu[j]; }, a.m))
      mark_candidate(cand0, x.x, acc);
  };
  // the merge flagged every vertex with a finite state (flag array 2): only
  // those rows are read
  const uint8_t* merged = a.flags + 2 * (int64_t)a.vpad;
  for (int64_t c = warp; c < g.nchunks; c += nwarps) {
    const int32_t u = g.chunk_vtx[c];
    if (!merged[u]) continue;
    const int2 hc = g.hub_chunk[c];
    const int32_t* hv = a.cost + a.base + (int64_t)u * s;
    bool light = false;
    for (int j = lane; j < a.m; j += 32) light |= light_or_inf(hv[j], ub_light) < kInf;
    if (!__any_sync(0xffffffffu, light)) continue;
    const int32_t e = hc.y + lane;
    if (e < g.row_ptr[u + 1]) seed_entry(hv, e);
  }
  for (int64_t vbase = warp * 32; vbase < g.V; vbase += nwarps * 32) {
    const int64_t vl = vbase + lane;
    bool light = false;
    if (vl < g.V && merged[vl] && g.row_ptr[vl + 1] - g.row_ptr[vl] <= g.deg_big) {
      const int32_t* hv = a.cost + a.base + vl * s;
      for (int j = 0; j < a.m; ++j) light |= light_or_inf(hv[j], ub_light) < kInf;
    }
    unsigned lm = __ballot_sync(0xffffffffu, light);
    while (lm) {
      const int32_t v = (int32_t)(vbase + __ffs(lm) - 1);
      lm &= lm - 1u;
      const int32_t* hv = a.cost + a.base + (int64_t)v * s;
      const int32_t end = g.row_ptr[v + 1];
      for (int32_t e = g.row_ptr[v] + lane; e < end; e += 32) seed_entry(hv, e);
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) ctl->dense[2] = 0;
}

// Hub relaxation of a sparse round (hub_relax), ahead of the round kernel,
// which then marks the changed hubs' neighbours. Dense rounds mark nothing
// and relax the hubs inside the round kernel, beside the other vertices.
template <int L>
__global__ void __launch_bounds__(kGrowThreads) k_grow_hubs(GraphDev g, LevelArgs a) {
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&a.ctr->grow_launches, 1);
  RoundState rs;
  if (!round_begin(g, a, rs) || rs.dense) return;
  __shared__ BlockAcc ba;
  block_acc_init(ba);
  uint32_t acc[kAccN] = {0, 0, 0, 0, 0, 0, 0};
  hub_relax<L>(g, a, rs, acc);
  round_flush(a, rs, acc, ba);
}

// The hub kernel of sparse rounds for waves with stride <= kMaxTeamStride.
template <int GP>
__global__ void __launch_bounds__(kGrowThreads) k_grow_hubs_team(GraphDev g, LevelArgs a) {
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&a.ctr->grow_launches, 1);
  RoundState rs;
  if (!round_begin(g, a, rs) || rs.dense) return;
  __shared__ BlockAcc ba;
  block_acc_init(ba);
  uint32_t acc[kAccN] = {0, 0, 0, 0, 0, 0, 0};
  hub_relax_team<GP, false>(g, a, rs, acc);
  round_flush(a, rs, acc, ba);
}

// Thread per vertex: the vertex's MP-entry row lives in registers. True
// when the row changed (the caller's warp then marks its neighbours,
// warp_mark).
template <int MP>
__device__ __forceinline__ bool thread_vertex(const GraphDev& g, const LevelArgs& a, const RoundState& rs,
                                              int32_t u, int32_t& beg_out, int32_t& deg_out,
                                              uint32_t (&acc)[kAccN]) {
  constexpr int U = MP <= 8 ? 4 : 2;
  constexpr int Q = MP / 4;
  const int32_t beg = g.row_ptr[u], end = g.row_ptr[u + 1];
  beg_out = beg;
  deg_out = end - beg;
  if (end - beg > g.deg_big) return false;  // hub: handled in 32-entry chunks
  int4* rowc = reinterpret_cast<int4*>(a.cost + a.base + (int64_t)u * MP);
  int32_t best[MP];
  // parent of entry j as (CSR entry - beg), one byte each (rows are at most
  // kDegBigMax long); 0xff = unchanged
  uint32_t code[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int4 x = rowc[q];
    best[4 * q] = x.x;
    best[4 * q + 1] = x.y;
    best[4 * q + 2] = x.z;
    best[4 * q + 3] = x.w;
    code[q] = 0xffffffffu;
  }
  bool live = false;
#pragma unroll
  for (int j = 0; j < MP; ++j) live |= j < a.m && best[j] != 0;  // cost-0 states cannot improve
  ++acc[kAccVert];
  acc[kAccEnt] += end - beg;
  if (!live) return false;
  // gathers the rows of up to U neighbours (slot i: ok, vertex, weight, CSR
  // entry - beg) and folds them into best / code. A kInf (or heavy) row
  // entry gives c >= kInf and never wins; rows hold values below ovf_limit
  // (checked when stored), so c cannot wrap or reach kInf from a finite entry
  auto relax_batch = [&](const bool (&ok)[U], const int32_t (&nvx)[U], const int32_t (&nwx)[U],
                         const uint32_t (&rel)[U]) {
    int32_t rows[U][MP];
#pragma unroll
    for (int i = 0; i < U; ++i) {
      if (ok[i]) {
        ++acc[kAccRows];
        const int4* rv = reinterpret_cast<const int4*>(a.cost + a.base + (int64_t)nvx[i] * MP);
#pragma unroll
        for (int q = 0; q < Q; ++q) {
          const int4 x = rv[q];
          rows[i][4 * q] = x.x;
          rows[i][4 * q + 1] = x.y;
          rows[i][4 * q + 2] = x.z;
          rows[i][4 * q + 3] = x.w;
        }
      } else {
#pragma unroll
        for (int j = 0; j < MP; ++j) rows[i][j] = kInf;
      }
    }
#pragma unroll
    for (int i = 0; i < U; ++i) {
#pragma unroll
      for (int j = 0; j < MP; ++j) {
        const int32_t c = light_or_inf(rows[i][j], rs.ub_light) + nwx[i];
        const bool lt = c < best[j];
        best[j] = lt ? c : best[j];
        const int sh = 8 * (j & 3);
        code[j >> 2] = lt ? ((code[j >> 2] & ~(0xffu << sh)) | (rel[i] << sh)) : code[j >> 2];
      }
    }
  };
  // sparse rounds only (dense rounds run in k_grow_team): first the change
  // flags of every CSR entry (8
  // independent loads at a time) into a bit mask, then only the changed
  // neighbours' rows, U at a time: the loop no longer waits on a flag
  // load per pair of entries
  uint64_t actm = 0;  // rows are at most kDegBigMax = 64 entries long
  for (int32_t e0 = beg; e0 < end; e0 += 8) {
    int32_t nb[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) nb[i] = e0 + i < end ? g.adj[e0 + i].x : -1;
#pragma unroll
    for (int i = 0; i < 8; ++i)
      if (nb[i] >= 0 && rs.cur_flag[nb[i]] != 0) actm |= 1ull << (e0 + i - beg);  // e0 + i < end: shift < 64
  }
  while (actm) {
    bool ok[U];
    uint32_t rel[U];
    int32_t nvx[U], nwx[U];
#pragma unroll
    for (int i = 0; i < U; ++i) {
      ok[i] = actm != 0ull;
      rel[i] = ok[i] ? (uint32_t)(__ffsll((long long)actm) - 1) : 0u;
      if (ok[i]) actm &= actm - 1ull;
      nvx[i] = 0;
      nwx[i] = 0;
    }
#pragma unroll
    for (int i = 0; i < U; ++i) {
      if (ok[i]) {
        const int2 x = g.adj[beg + (int32_t)rel[i]];
        nvx[i] = x.x;
        nwx[i] = x.y;
      }
    }
    relax_batch(ok, nvx, nwx, rel);
  }
  bool any = false;
#pragma unroll
  for (int j = 0; j < MP; ++j) {
    const int sh = 8 * (j & 3);
    const bool imp = ((code[j >> 2] >> sh) & 0xffu) != 0xffu;
    if (imp && best[j] >= rs.ovf_limit) acc[kAccOverflow] = 1;
    if (imp && rs.ub > 0 && best[j] > cap_at(a, u, j)) {
      best[j] = a.cost[a.base + (int64_t)u * MP + j];  // keep the stored value
      code[j >> 2] |= 0xffu << sh;
    }
    any |= ((code[j >> 2] >> sh) & 0xffu) != 0xffu;
  }
  if (!any) return false;
#pragma unroll
  for (int q = 0; q < Q; ++q) rowc[q] = make_int4(best[4 * q], best[4 * q + 1], best[4 * q + 2], best[4 * q + 3]);
  int32_t* rowp = a.par + a.base + (int64_t)u * MP;
#pragma unroll
  for (int j = 0; j < MP; ++j) {
    const uint32_t rel = (code[j >> 2] >> (8 * (j & 3))) & 0xffu;
    if (rel != 0xffu) {
      rowp[j] = beg + (int32_t)rel;
      ++acc[kAccImproved];
    }
  }
  rs.next_flag[u] = 1;
  ++acc[kAccChanged];
  return true;
}

// Marks, for every vertex of the warp whose row changed this round (chg),
// the neighbours that the new row improves (within their bound). The CSR
// entries of the warp's changed rows are taken as one list, 32 at a time,
// a lane per entry (the entry's row found by a binary search over the
// lanes' entry offsets), so a step costs a few loads whatever the number
// of changed rows: the entry, the neighbour's and the changed row's masks
// (16 bytes at a time), and with a bound the neighbour's caps, all at
// once. A neighbour is marked only if the new row improves it for some
// mask: its row can only decrease later, so an unmarked neighbour never
// needs this row. Every lane of the warp must call it; dense rounds mark
// nothing (the next round sweeps every vertex).
template <int MP>
__device__ __forceinline__ void warp_mark(const GraphDev& g, const LevelArgs& a, const RoundState& rs, int32_t u,
                                          int32_t beg, int32_t deg, bool chg, uint32_t (&acc)[kAccN]) {
  constexpr int Q = MP / 4;
  if (rs.dense) return;
  if (!__ballot_sync(0xffffffffu, chg)) return;
  __syncwarp();  // the changed rows' stores are visible to the whole warp
  const int lane = threadIdx.x & 31;
  const int32_t d = chg ? deg : 0;
  int32_t incl = d;  // inclusive prefix of the changed rows' lengths over the lanes
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int32_t y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  const int32_t pre = incl - d;
  const int32_t total = __shfl_sync(0xffffffffu, incl, 31);
  for (int32_t p0 = 0; p0 < total; p0 += 32) {
    const int32_t p = p0 + lane;
    int src = 0;  // the last lane whose entries start at or before p
#pragma unroll
    for (int st = 16; st >= 1; st >>= 1) {
      const int c = src + st;
      const int32_t pc = __shfl_sync(0xffffffffu, pre, c & 31);
      if (c <= 31 && pc <= p) src = c;
    }
    const int32_t w = __shfl_sync(0xffffffffu, u, src);
    const int32_t wb = __shfl_sync(0xffffffffu, beg, src);
    const int32_t wp = __shfl_sync(0xffffffffu, pre, src);
    if (p >= total) continue;
    const int2 x = g.adj[wb + (p - wp)];
    // w's new row (light-filtered) against x's row
    const int4* wr = reinterpret_cast<const int4*>(a.cost + a.base + (int64_t)w * MP);
    const int4* rv = reinterpret_cast<const int4*>(a.cost + a.base + (int64_t)x.x * MP);
    int32_t val[MP];
    uint32_t bits = 0;  // masks the new row improves at x
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const int4 t = rv[q], h = wr[q];
      val[4 * q] = light_or_inf(h.x, rs.ub_light) + x.y;
      val[4 * q + 1] = light_or_inf(h.y, rs.ub_light) + x.y;
      val[4 * q + 2] = light_or_inf(h.z, rs.ub_light) + x.y;
      val[4 * q + 3] = light_or_inf(h.w, rs.ub_light) + x.y;
      bits |= (val[4 * q] < t.x ? 1u : 0u) << (4 * q);
      bits |= (val[4 * q + 1] < t.y ? 1u : 0u) << (4 * q + 1);
      bits |= (val[4 * q + 2] < t.z ? 1u : 0u) << (4 * q + 2);
      bits |= (val[4 * q + 3] < t.w ? 1u : 0u) << (4 * q + 3);
    }
    bool better = bits != 0;
    if (better && rs.ub > 0) {  // the same test under x's caps, all masks at once
      const int4* cv = reinterpret_cast<const int4*>(a.capt + (int64_t)x.x * MP);
      better = false;
#pragma unroll
      for (int q = 0; q < Q; ++q) {
        const int4 c = __ldg(cv + q);
        better |= ((bits >> (4 * q)) & 1u) && val[4 * q] <= c.x;
        better |= ((bits >> (4 * q + 1)) & 1u) && val[4 * q + 1] <= c.y;
        better |= ((bits >> (4 * q + 2)) & 1u) && val[4 * q + 2] <= c.z;
        better |= ((bits >> (4 * q + 3)) & 1u) && val[4 * q + 3] <= c.w;
      }
    }
    if (better) mark_candidate(rs.cand_next, x.x, acc);
  }
}

// A sparse round of a wave with row stride MP <= kMaxThreadMasks, after its
// hub chunks ran (k_grow_hubs_team): flags of two rounds back cleared, the
// changed hubs' neighbours marked, then every candidate (or, in the round
// after a dense one, every vertex) relaxed by a thread and the neighbours
// its new row improves marked (warp_mark).
template <int MP>
__device__ __forceinline__ void thread_round_body(const GraphDev& g, const LevelArgs& a, const RoundState& rs,
                                                  uint32_t (&acc)[kAccN]) {
  const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
  clear_flags(a, rs, t0, nthreads);
  hub_mark(g, a, rs, acc);
  // warps take their work from the round's counter, so blocks that draw
  // cheap vertices (or tiles without candidates) take more of them and no
  // SM idles while another finishes a fixed share
  const int lane = threadIdx.x & 31;
  uint32_t* work = &a.ctl->work[rs.r % 3];
  if (rs.all_cand) {
    // every vertex, kDenseGrab sweep positions per take; odd rounds sweep
    // backwards, so in-place updates also carry along the order in the
    // other direction within one round
    static_assert(kDenseGrab == 32, "one sweep position per lane");
    for (;;) {
      uint32_t base = 0;
      if (lane == 0) base = atomicAdd(work, (uint32_t)kDenseGrab);
      base = __shfl_sync(0xffffffffu, base, 0);
      if ((int64_t)base >= g.nsmall) break;
      const int64_t i = (int64_t)base + lane;
      const int32_t u = i < g.nsmall ? g.order[(rs.r & 1) ? g.nsmall - 1 - i : i] : -1;
      int32_t beg = 0, deg = 0;
      const bool chg = u >= 0 && thread_vertex<MP>(g, a, rs, u, beg, deg, acc);
      warp_mark<MP>(g, a, rs, u, beg, deg, chg, acc);
    }
  } else {
    // candidates only: a warp reads kCandTile candidate bytes at a time (8
    // per lane), compacts the set ones in shared memory and its lanes take
    // them in turn
    __shared__ int32_t tile[kGrowThreads / 32][kCandTile];
    const int wib = threadIdx.x >> 5;
    static_assert(kCandTile == 8 * 32, "a lane reads 8 flag bytes");
    for (;;) {
      uint32_t ti = 0;
      if (lane == 0) ti = atomicAdd(work, 1u);
      ti = __shfl_sync(0xffffffffu, ti, 0);
      const int64_t base = (int64_t)ti * kCandTile;
      if (base >= g.V) break;
      const int64_t v0 = base + 8 * lane;
      uint2 f = make_uint2(0u, 0u);
      if (v0 < g.V) f = *reinterpret_cast<const uint2*>(rs.cand_cur + v0);  // arrays padded to 16 bytes
      const uint32_t w2[2] = {f.x, f.y};
      int cnt = 0;
#pragma unroll
      for (int b = 0; b < 8; ++b) cnt += ((w2[b >> 2] >> (8 * (b & 3))) & 0xffu) != 0;
      int pre = cnt;  // inclusive prefix over lanes
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, pre, o);
        if (lane >= o) pre += t;
      }
      const int total = __shfl_sync(0xffffffffu, pre, 31);
      int pos = pre - cnt;
#pragma unroll
      for (int b = 0; b < 8; ++b)
        if (((w2[b >> 2] >> (8 * (b & 3))) & 0xffu) != 0) tile[wib][pos++] = (int32_t)(v0 + b);
      __syncwarp();
      for (int i0 = 0; i0 < total; i0 += 32) {
        const int32_t u = i0 + lane < total ? tile[wib][i0 + lane] : -1;
        int32_t beg = 0, deg = 0;
        const bool chg = u >= 0 && thread_vertex<MP>(g, a, rs, u, beg, deg, acc);
        warp_mark<MP>(g, a, rs, u, beg, deg, chg, acc);
      }
      __syncwarp();
    }
  }
}

template <int G>
__device__ __forceinline__ void sparse_team_body(const GraphDev& g, const LevelArgs& a, const RoundState& rs,
                                                 uint32_t (&acc)[kAccN]);

template <int MP>
__global__ void __launch_bounds__(kGrowThreads, (MP <= 16 ? 3 : 2)) k_grow_thread(GraphDev g, LevelArgs a) {
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&a.ctr->grow_launches, 1);
  RoundState rs;
  if (!round_begin(g, a, rs)) return;
  if (rs.dense) return;  // dense rounds run in k_grow_team
  __shared__ BlockAcc ba;
  block_acc_init(ba);
  uint32_t acc[kAccN] = {0, 0, 0, 0, 0, 0, 0};
  // a small frontier (at most V/32 rows changed) of a wide wave: teams, whose
  // lanes read a candidate's change flags together; otherwise a thread per
  // candidate, which holds more candidates in flight per warp
  bool teams = false;
  if constexpr (MP >= 16) teams = !rs.all_cand && rs.prev <= (g.V >> 5);
  if (teams) {
    if constexpr (MP >= 16) sparse_team_body<MP / 4>(g, a, rs, acc);
  } else {
    thread_round_body<MP>(g, a, rs, acc);
  }
  round_end(a, rs, acc, ba);
}

// Dense rounds of waves with row stride 4G <= kMaxTeamStride: a team of G
// lanes relaxes one vertex, lane q holding masks 4q .. 4q+3 of its row.
// Per neighbour a lane issues one 16-byte load (its quarter, half, ... of
// the neighbour's row; the team's loads together read the row's
// contiguous 16G bytes) after loading the CSR entry, which every lane of
// the team reads at the same address. UNR neighbours are in flight at a
// time: their CSR entries are loaded unconditionally at clamped addresses,
// then their rows, then folded, then the next UNR entries are loaded. The
// caller passes the vertex's row bounds (looked up for 32 vertices at once
// by the warp). A team holds 8 best / parent registers,
// not the whole row, so more warps stay resident than with a thread per
// vertex, and a neighbour costs a team one load and three integer
// operations per mask instead of a thread's serial chain. LIGHT: the solve
// prunes, only light neighbour states grow (light_or_inf).
template <int G, int UNR, bool LIGHT>
__device__ __forceinline__ void team_vertex(const GraphDev& g, const LevelArgs& a, const RoundState& rs, int32_t u,
                                            int32_t beg, int32_t end, int glane, unsigned tmask,
                                            uint32_t (&acc)[kAccN]) {
  constexpr int S = 4 * G;
  if (end - beg > g.deg_big) return;  // hub: relaxed in segments (hub_relax_team)
  const int64_t rowu = a.base + (int64_t)u * S;
  const int4 own4 = reinterpret_cast<const int4*>(a.cost + rowu)[glane];
  const int32_t own[4] = {own4.x, own4.y, own4.z, own4.w};
  int32_t best[4] = {own4.x, own4.y, own4.z, own4.w};
  int32_t code[4] = {-1, -1, -1, -1};
  bool live = false;
#pragma unroll
  for (int t = 0; t < 4; ++t) live |= 4 * glane + t < a.m && own[t] != 0;  // cost-0 states cannot improve
  if (glane == 0) {
    ++acc[kAccVert];
    acc[kAccEnt] += end - beg;
  }
  if (!(__ballot_sync(tmask, live) & tmask)) return;
  const int4* tab = reinterpret_cast<const int4*>(a.cost + a.base);
  int2 x[UNR];
  if (beg < end) {
#pragma unroll
    for (int i = 0; i < UNR; ++i) x[i] = g.adj[min(beg + i, end - 1)];
  }
  for (int32_t e0 = beg; e0 < end; e0 += UNR) {
    int4 r[UNR];
#pragma unroll
    for (int i = 0; i < UNR; ++i) r[i] = tab[(int64_t)x[i].x * G + glane];
#pragma unroll
    for (int i = 0; i < UNR; ++i) {
      if (e0 + i < end) {
        const int32_t rv[4] = {r[i].x, r[i].y, r[i].z, r[i].w};
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          // a kInf (or, pruning, heavy) entry gives c >= kInf and never wins;
          // stored costs stay below ovf_limit, so c cannot wrap
          const int32_t c = (LIGHT ? light_or_inf(rv[t], rs.ub_light) : rv[t]) + x[i].y;
          if (c < best[t]) {
            best[t] = c;
            code[t] = e0 + i;
          }
        }
      }
    }
    if (e0 + UNR < end) {
#pragma unroll
      for (int i = 0; i < UNR; ++i) x[i] = g.adj[min(e0 + UNR + i, end - 1)];
    }
  }
  if (glane == 0) acc[kAccRows] += end - beg;
  bool imp = false;
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    if (code[t] < 0) continue;
    if (best[t] >= rs.ovf_limit) acc[kAccOverflow] = 1;
    if (rs.ub > 0 && best[t] > cap_at(a, u, 4 * glane + t)) {  // over the state's cap: keep the stored value
      best[t] = own[t];
      code[t] = -1;
      continue;
    }
    imp = true;
  }
  if (imp) {
    reinterpret_cast<int4*>(a.cost + rowu)[glane] = make_int4(best[0], best[1], best[2], best[3]);
#pragma unroll
    for (int t = 0; t < 4; ++t)
      if (code[t] >= 0) {
        a.par[rowu + 4 * glane + t] = code[t];
        ++acc[kAccImproved];
      }
  }
  if ((__ballot_sync(tmask, imp) & tmask) && glane == 0) {
    rs.next_flag[u] = 1;
    ++acc[kAccChanged];
  }
}

// Sparse rounds by vertex teams (row stride 4G): a team of G lanes takes a
// candidate, lane q holding masks 4q .. 4q+3. The team reads the change
// flags of the candidate's CSR entries first (lane q takes entries q,
// q+G, ..., all at once), then gathers only the changed neighbours' rows,
// UNR at a time, each lane its 16-byte quarter. True (in every lane of the
// team) when the candidate's row changed.
template <int G, int UNR, bool LIGHT>
__device__ __forceinline__ bool team_sparse_vertex(const GraphDev& g, const LevelArgs& a, const RoundState& rs,
                                                   int32_t u, int glane, int team, unsigned tmask, int32_t& beg_out,
                                                   int32_t& deg_out, uint32_t (&acc)[kAccN]) {
  constexpr int S = 4 * G;
  constexpr int NE = (kDegBigMax + G - 1) / G;  // entries per lane, enough for any non-hub row
  const int32_t beg = g.row_ptr[u], end = g.row_ptr[u + 1];
  beg_out = beg;
  deg_out = end - beg;
  if (end - beg > g.deg_big) return false;  // hub: relaxed in segments
  const int32_t deg = end - beg;
  const int64_t rowu = a.base + (int64_t)u * S;
  const int4 own4 = reinterpret_cast<const int4*>(a.cost + rowu)[glane];
  const int32_t own[4] = {own4.x, own4.y, own4.z, own4.w};
  int32_t best[4] = {own4.x, own4.y, own4.z, own4.w};
  int32_t code[4] = {-1, -1, -1, -1};
  bool live = false;
#pragma unroll
  for (int t = 0; t < 4; ++t) live |= 4 * glane + t < a.m && own[t] != 0;  // cost-0 states cannot improve
  if (glane == 0) {
    ++acc[kAccVert];
    acc[kAccEnt] += deg;
  }
  if (!(__ballot_sync(tmask, live) & tmask)) return false;
  // change flags: lane q takes entries q, q + G, ...
  int32_t nb[NE];
#pragma unroll
  for (int i = 0; i < NE; ++i) {
    const int e = glane + i * G;
    nb[i] = e < deg ? g.adj[beg + e].x : -1;
  }
  uint64_t chm = 0;  // bit e: entry e's neighbour changed in the previous round
#pragma unroll
  for (int i = 0; i < NE; ++i) {
    const bool c = nb[i] >= 0 && rs.cur_flag[nb[i]] != 0;
    const unsigned b = (__ballot_sync(tmask, c) >> (team * G)) & ((1u << G) - 1u);
    chm |= (uint64_t)b << (i * G);
    if (i * G + G >= deg) break;  // team-uniform: deg is the same in every lane of the team
  }
  const int4* tab = reinterpret_cast<const int4*>(a.cost + a.base);
  int rows = 0;
  while (chm) {
    int rel[UNR];
    bool ok[UNR];
#pragma unroll
    for (int i = 0; i < UNR; ++i) {
      ok[i] = chm != 0ull;
      rel[i] = ok[i] ? __ffsll((long long)chm) - 1 : 0;
      if (ok[i]) chm &= chm - 1ull;
    }
    int2 x[UNR];
#pragma unroll
    for (int i = 0; i < UNR; ++i) x[i] = g.adj[beg + rel[i]];
    int4 r[UNR];
#pragma unroll
    for (int i = 0; i < UNR; ++i) r[i] = ok[i] ? tab[(int64_t)x[i].x * G + glane] : make_int4(kInf, kInf, kInf, kInf);
#pragma unroll
    for (int i = 0; i < UNR; ++i) {
      if (!ok[i]) continue;
      ++rows;
      const int32_t rv[4] = {r[i].x, r[i].y, r[i].z, r[i].w};
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        const int32_t c = (LIGHT ? light_or_inf(rv[t], rs.ub_light) : rv[t]) + x[i].y;
        if (c < best[t]) {
          best[t] = c;
          code[t] = beg + rel[i];
        }
      }
    }
  }
  if (glane == 0) acc[kAccRows] += rows;
  bool imp = false;
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    if (code[t] < 0) continue;
    if (best[t] >= rs.ovf_limit) acc[kAccOverflow] = 1;
    if (rs.ub > 0 && best[t] > cap_at(a, u, 4 * glane + t)) {  // over the state's cap: keep the stored value
      best[t] = own[t];
      code[t] = -1;
      continue;
    }
    imp = true;
  }
  if (imp) {
    reinterpret_cast<int4*>(a.cost + rowu)[glane] = make_int4(best[0], best[1], best[2], best[3]);
#pragma unroll
    for (int t = 0; t < 4; ++t)
      if (code[t] >= 0) {
        a.par[rowu + 4 * glane + t] = code[t];
        ++acc[kAccImproved];
      }
  }
  const bool chg = (__ballot_sync(tmask, imp) & tmask) != 0;
  if (chg && glane == 0) {
    rs.next_flag[u] = 1;
    ++acc[kAccChanged];
  }
  return chg;
}

// A sparse round over candidates (not the round after a dense one) of a
// wave with row stride 4G, by vertex teams: flags cleared, the changed
// hubs' neighbours marked, then the candidates relaxed a team each, T =
// 32 / G per warp step, and the neighbours of the changed ones marked.
template <int G>
__device__ __forceinline__ void sparse_team_body(const GraphDev& g, const LevelArgs& a, const RoundState& rs,
                                                 uint32_t (&acc)[kAccN]) {
  constexpr int MP = 4 * G;
  constexpr int UNR = 4;
  const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
  clear_flags(a, rs, t0, nthreads);
  hub_mark(g, a, rs, acc);
  constexpr int T = 32 / G;
  const int lane = threadIdx.x & 31;
  const int team = lane / G, glane = lane - team * G;
  const unsigned tmask = team < T ? (G == 32 ? 0xffffffffu : ((1u << G) - 1u) << (team * G)) : 0u;
  uint32_t* work = &a.ctl->work[rs.r % 3];
  const bool light = rs.ub_light > 0;
  // relaxes up to T candidates (list entries i0 + team) and marks the
  // neighbours of the changed ones; every lane of the warp calls it
  auto step = [&](const int32_t* list, int i0, int n) {
    const int idx = i0 + team;
    const int32_t u = (team < T && idx < n) ? list[idx] : -1;
    int32_t beg = 0, deg = 0;
    bool chg = false;
    if (u >= 0)
      chg = light ? team_sparse_vertex<G, UNR, true>(g, a, rs, u, glane, team, tmask, beg, deg, acc)
                  : team_sparse_vertex<G, UNR, false>(g, a, rs, u, glane, team, tmask, beg, deg, acc);
    __syncwarp();
    warp_mark<MP>(g, a, rs, u, beg, deg, chg && glane == 0, acc);
  };
  // candidate tiles as in thread_round_body
  __shared__ int32_t tile[kGrowThreads / 32][kCandTile];
  const int wib = threadIdx.x >> 5;
  static_assert(kCandTile == 8 * 32, "a lane reads 8 flag bytes");
  for (;;) {
    uint32_t ti = 0;
    if (lane == 0) ti = atomicAdd(work, 1u);
    ti = __shfl_sync(0xffffffffu, ti, 0);
    const int64_t base = (int64_t)ti * kCandTile;
    if (base >= g.V) break;
    const int64_t v0 = base + 8 * lane;
    uint2 f = make_uint2(0u, 0u);
    if (v0 < g.V) f = *reinterpret_cast<const uint2*>(rs.cand_cur + v0);  // arrays padded to 16 bytes
    const uint32_t w2[2] = {f.x, f.y};
    int cnt = 0;
#pragma unroll
    for (int b = 0; b < 8; ++b) cnt += ((w2[b >> 2] >> (8 * (b & 3))) & 0xffu) != 0;
    int pre = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, pre, o);
      if (lane >= o) pre += t;
    }
    const int total = __shfl_sync(0xffffffffu, pre, 31);
    int pos = pre - cnt;
#pragma unroll
    for (int b = 0; b < 8; ++b)
      if (((w2[b >> 2] >> (8 * (b & 3))) & 0xffu) != 0) tile[wib][pos++] = (int32_t)(v0 + b);
    __syncwarp();
    for (int i0 = 0; i0 < total; i0 += T) step(tile[wib], i0, total);
    __syncwarp();
  }
}

// The dense rounds of waves whose stride is 4G (sparse rounds return at
// once: k_grow_thread runs them). Hubs first (segments of up to kHubSeg
// entries), then the other vertices in growth order: a warp takes 32 sweep
// positions at a time from the round's counter, its 32/G teams take them in
// turn. Odd rounds sweep backwards.
template <int G, int UNR>
__global__ void __launch_bounds__(kGrowThreads, (G <= 4 ? 4 : 3)) k_grow_team(GraphDev g, LevelArgs a) {
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&a.ctr->grow_launches, 1);
  RoundState rs;
  if (!round_begin(g, a, rs)) return;
  if (!rs.dense) return;
  __shared__ BlockAcc ba;
  block_acc_init(ba);
  uint32_t acc[kAccN] = {0, 0, 0, 0, 0, 0, 0};
  const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
  clear_flags(a, rs, t0, nthreads);
  hub_relax_team<(G <= 1 ? 1 : G <= 2 ? 2 : G <= 4 ? 4 : G <= 8 ? 8 : G <= 16 ? 16 : 32), true>(g, a, rs, acc);
  constexpr int T = 32 / G;  // teams per warp; lanes T*G .. 31 idle
  const int lane = threadIdx.x & 31;
  const int team = lane / G, glane = lane - team * G;
  const unsigned tmask = team < T ? (G == 32 ? 0xffffffffu : ((1u << G) - 1u) << (team * G)) : 0u;
  uint32_t* work = &a.ctl->work[rs.r % 3];
  const bool light = rs.ub_light > 0;
  static_assert(kDenseGrab == 32, "one sweep position per lane");
  for (;;) {
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(work, (uint32_t)kDenseGrab);
    base = __shfl_sync(0xffffffffu, base, 0);
    if ((int64_t)base >= g.nsmall) break;
    // lane j looks up the take's j-th vertex and its row bounds (one
    // coalesced step for the whole warp), so a team starts each of its
    // vertices at the CSR entries
    const int64_t ij = (int64_t)base + lane;
    int32_t uj = -1, bj = 0, ej = 0;
    if (ij < g.nsmall) {
      uj = g.order[(rs.r & 1) ? g.nsmall - 1 - ij : ij];
      bj = g.row_ptr[uj];
      ej = g.row_ptr[uj + 1];
    }
    for (int p0 = 0; p0 < kDenseGrab; p0 += T) {  // the same trip count in every lane
      const int src = min(p0 + team, 31);
      const int32_t u = __shfl_sync(0xffffffffu, uj, src);
      const int32_t beg = __shfl_sync(0xffffffffu, bj, src);
      const int32_t end = __shfl_sync(0xffffffffu, ej, src);
      if (team < T && p0 + team < kDenseGrab && u >= 0) {
        if (light)
          team_vertex<G, UNR, true>(g, a, rs, u, beg, end, glane, tmask, acc);
        else
          team_vertex<G, UNR, false>(g, a, rs, u, beg, end, glane, tmask, acc);
      }
      __syncwarp();
    }
  }
  round_end(a, rs, acc, ba);
}

// G lanes per vertex for waves wider than kMaxThreadMasks. Each warp takes
// 32 consecutive vertices at a time, finds the candidates among them with
// one ballot, and its 32/G groups take the candidates in turn. SPARSE_ONLY:
// the wave's dense rounds run in k_grow_team (strides 28, 36, 56, 72: the
// waves of k = 7 and 8), this kernel its sparse rounds.
template <int G, int L, bool SPARSE_ONLY>
__global__ void __launch_bounds__(kGrowThreads, (L >= 3 ? 3 : 4)) k_grow_group(GraphDev g, LevelArgs a) {
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&a.ctr->grow_launches, 1);
  RoundState rs;
  if (!round_begin(g, a, rs)) return;
  if (SPARSE_ONLY && rs.dense) return;  // dense rounds of this wave run in k_grow_team
  __shared__ BlockAcc ba;
  block_acc_init(ba);
  uint32_t acc[kAccN] = {0, 0, 0, 0, 0, 0, 0};
  {
    const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
    clear_flags(a, rs, t0, nthreads);
  }
  if (!SPARSE_ONLY && rs.dense)
    hub_relax<((G * L + 31) / 32 < 4 ? (G * L + 31) / 32 : 4)>(g, a, rs, acc);
  else
    hub_mark(g, a, rs, acc);
  {
    const int tid = threadIdx.x, lane = tid & 31;
    const int glane = lane & (G - 1), gbase = lane & ~(G - 1);
    const unsigned gmask_lanes = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << gbase);
    const unsigned gbits = (G == 32) ? 0xffffffffu : ((1u << G) - 1u);
    constexpr int CH = G * L;
    constexpr int NGW = 32 / G;
    const int gw = lane / G;
    const int32_t s = a.stride;
    uint32_t* work = &a.ctl->work[rs.r % 3];
    for (;;) {  // 32 consecutive vertices per take from the round's counter
      uint32_t wt = 0;
      if (lane == 0) wt = atomicAdd(work, 1u);
      wt = __shfl_sync(0xffffffffu, wt, 0);
      const int64_t vbase = (int64_t)wt * 32;
      if (vbase >= g.V) break;
      const int64_t vl = vbase + lane;
      const bool cnd = vl < g.V && (rs.all_cand || rs.cand_cur[vl] != 0);
      unsigned cm = __ballot_sync(0xffffffffu, cnd);
      for (int i = 0; i < gw && cm; ++i) cm &= cm - 1u;
      while (cm) {
        const int32_t u = (int32_t)(vbase + __ffs(cm) - 1);
        for (int i = 0; i < NGW && cm; ++i) cm &= cm - 1u;
        const int32_t beg = g.row_ptr[u], end = g.row_ptr[u + 1];
        if (end - beg > g.deg_big) continue;  // handled in 32-entry chunks
        const int64_t rowu = a.base + (int64_t)u * s;
        bool imp_any = false;
        for (int jc = 0; jc < s; jc += CH) {
          int32_t own[L], best[L], code[L];
          bool live = false;
#pragma unroll
          for (int t = 0; t < L; ++t) {
            const int j = jc + glane + t * G;
            own[t] = (j < s) ? a.cost[rowu + j] : kInf;
            best[t] = own[t];
            code[t] = -1;
            live |= j < a.m && own[t] != 0;
          }
          if (!(__ballot_sync(gmask_lanes, live) & gmask_lanes)) continue;
          for (int32_t e0 = beg; e0 < end; e0 += G)
            group_relax<G, L>(g, a, rs, e0, end, jc, glane, gbase, gmask_lanes, gbits, best, code, acc);
          bool imp = false;
#pragma unroll
          for (int t = 0; t < L; ++t) {
            const int j = jc + glane + t * G;
            if (j < a.m && best[t] < own[t]) {
              if (rs.ub > 0 && best[t] > cap_at(a, u, j)) continue;
              a.cost[rowu + j] = best[t];
              a.par[rowu + j] = code[t];
              imp = true;
              ++acc[kAccImproved];
            }
          }
          imp_any |= (__ballot_sync(gmask_lanes, imp) & gmask_lanes) != 0;
        }
        if (imp_any && !rs.dense) {
          for (int32_t e = beg + glane; e < end; e += G) mark_candidate(rs.cand_next, g.adj[e].x, acc);
        }
        if (glane == 0) {
          ++acc[kAccVert];
          acc[kAccEnt] += end - beg;
          if (imp_any) {
            rs.next_flag[u] = 1;
            ++acc[kAccChanged];
          }
        }
      }
    }
  }
  round_end(a, rs, acc, ba);
}

// ------------------------------------------------------------ bound update --
// The cost of a feasible subgraph for every state: T(v,S) plus v's wave-1
// states T(v,{g}) for the groups g outside S (each stored cost is that of
// an actual tree or path, so the sum bounds the union's cost and hence the
// optimum from above). The cheapest one lowers params->ub (0 = none yet).
// A zero-cost tree is no bound in that encoding (0 reads as "none", and a
// later, costlier candidate would then raise the bound): it is skipped,
// and the bound stays what it was (still valid, only less tight).
// The restatement, over all states of a wave at once, of PrunedDP++'s
// update of its best solution (graph_v_of_v_idealID_PrunedDPPlusPlus.h:668-711).
__global__ void __launch_bounds__(kGrowThreads) k_ub_refine(GraphDev g, LevelArgs a) {
  if (!a.params->refine) return;
  __shared__ long long sbest[kGrowThreads / 32];
  long long best = LLONG_MAX;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < g.V; v += (int64_t)gridDim.x * blockDim.x) {
    const int32_t* d = a.cost + v * a.stride1;
    int32_t dd[16];
#pragma unroll
    for (int gg = 0; gg < 16; ++gg) dd[gg] = gg < a.k ? d[gg] : 0;
    const int4* row = reinterpret_cast<const int4*>(a.cost + a.base + v * a.stride);  // rows are 16-byte aligned
    for (int j0 = 0; j0 < a.m; j0 += 4) {
      const int4 q = row[j0 >> 2];
      const int32_t c4[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        const int j = j0 + t;
        const int32_t c = c4[t];
        if (j >= a.m || c >= kInf) continue;
        const uint32_t S = (uint32_t)__ldg(a.lmasks + j);
        long long sum = c;
        bool ok = true;
#pragma unroll
        for (int gg = 0; gg < 16; ++gg)
          if (gg < a.k && !((S >> gg) & 1u)) {
            ok &= dd[gg] < kInf;
            sum += dd[gg];
          }
        if (ok && sum < best) best = sum;
      }
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const long long x = __shfl_xor_sync(0xffffffffu, best, o);
    best = x < best ? x : best;
  }
  if ((threadIdx.x & 31) == 0) sbest[threadIdx.x >> 5] = best;
  __syncthreads();
  if (threadIdx.x != 0) return;
  for (int w = 1; w < (int)(blockDim.x >> 5); ++w) best = sbest[w] < best ? sbest[w] : best;
  if (best >= (long long)kInf || best <= 0) return;
  int32_t* ub = const_cast<int32_t*>(&a.params->ub);
  const int32_t cand = (int32_t)best;
  int32_t old = *reinterpret_cast<volatile int32_t*>(ub);
  while (old <= 0 || cand < old) {
    const int32_t prev = atomicCAS(ub, old, cand);
    if (prev == old) break;
    old = prev;
  }
}

// ----------------------------------------------------------------- argmin --
// ------------------------------------------------------------ tour table --
// Lower bounds of the group-to-group distances: D[a][b] = the smallest
// min(T(m,{a}), ub/2 + 1) over the members m of group b (wave 1's
// distances; light ones are exact and heavy ones exceed ub/2, so the min
// bounds the distance from below either way), made symmetric with the
// larger of D[a][b] and D[b][a] (both bound the same distance). Then
// path[i][X][j] = the cheapest order of visiting every group of X from
// group i to group j over legs D, by subsets of growing size, clamped at
// ub (a clamp only lowers the bound); orders that do not exist keep the
// clamp. The tables of PrunedDP++'s tour bound
// (graph_v_of_v_idealID_PrunedDPPlusPlus.h:268-386) for this query's
// groups, rebuilt before every merge because the bound may have dropped.
__global__ void __launch_bounds__(1024) k_tour_table(LevelArgs a, const int32_t* __restrict__ group_ptr,
                                                    const int32_t* __restrict__ members,
                                                    const int32_t* __restrict__ perm, int32_t* __restrict__ tour) {
  constexpr int KM = kTourMaxK;
  __shared__ int32_t D[KM][KM];
  extern __shared__ int32_t Fs[];  // k x 2^k x k (64 KB at k = 8), up to kTourSmemMaxK groups
  // no bound: the merge does not read the table, unless one may still
  // arrive before it (late_bound). Then no wave has grown under a bound yet
  // (bounds only drop), wave 1's distances are exact, and the table is
  // built with the open clamp kTourOpen; the merge caps distances at its own
  // bound, and the entries stay lower bounds either way.
  constexpr int32_t kTourOpen = 1 << 28;
  int32_t ub = a.params->ub;
  if (ub <= 0) {
    if (!a.params->late_bound) return;
    ub = kTourOpen;
  }
  const int k = a.k, W = 1 << k, kk = k * k;
  int32_t* F = k <= kTourSmemMaxK ? Fs : tour;  // beyond: the path table is built in place
  const int32_t beyond = ub / 2 + 1;
  for (int t = threadIdx.x; t < KM * KM; t += blockDim.x) D[t / KM][t % KM] = beyond;
  for (int t = threadIdx.x; t < k * W * k; t += blockDim.x) F[t] = ub;
  __syncthreads();
  // every member of every group at once: member i belongs to the last group
  // whose first member is at or before i
  __shared__ int32_t gstart[KM + 1];
  if (threadIdx.x <= k) gstart[threadIdx.x] = group_ptr[threadIdx.x];
  __syncthreads();
  for (int32_t i = gstart[0] + threadIdx.x; i < gstart[k]; i += blockDim.x) {
    int b = 0;
    for (int bb = 1; bb < k; ++bb) b = i >= gstart[bb] ? bb : b;
    const int32_t* d = a.cost + (int64_t)perm[members[i]] * a.stride1;  // wave 1: rank of {g} is g
    for (int g2 = 0; g2 < k; ++g2) atomicMin(&D[g2][b], min(d[g2], beyond));
  }
  __syncthreads();
  int32_t sym = 0;
  if (threadIdx.x < kk) sym = max(D[threadIdx.x / k][threadIdx.x % k], D[threadIdx.x % k][threadIdx.x / k]);
  __syncthreads();
  if (threadIdx.x < kk) D[threadIdx.x / k][threadIdx.x % k] = sym;
  if (threadIdx.x < k) F[((threadIdx.x << k) | (1 << threadIdx.x)) * k + threadIdx.x] = 0;
  __syncthreads();
  for (int p = 2; p <= k; ++p) {  // subsets of p groups from those of p - 1
    for (int t = threadIdx.x; t < W * kk; t += blockDim.x) {
      const int X = t / kk, i = (t / k) % k, j = t % k;
      if (__popc(X) != p || !((X >> i) & 1) || !((X >> j) & 1) || i == j) continue;
      const int prev = X ^ (1 << j);
      int32_t best = ub;
      for (int l = 0; l < k; ++l)
        if ((prev >> l) & 1) best = min(best, F[((i << k) | prev) * k + l] + D[l][j]);  // both <= ub < 2^30
      F[((i << k) | X) * k + j] = best;
    }
    __syncthreads();
  }
  if (F != tour)
    for (int t = threadIdx.x; t < k * W * k; t += blockDim.x) tour[t] = F[t];
  // W2[i][X] = the cheapest order visiting X from i, ending at any group
  // j != i (0 for X = {i}): PrunedDP++'s W2 (PrunedDPPlusPlus.h:565-585)
  for (int t = threadIdx.x; t < k * W; t += blockDim.x) {
    const int i = t / W, X = t % W;
    int32_t best = ub;
    if (X == (1 << i)) {
      best = 0;
    } else if ((X >> i) & 1) {
      for (int j = 0; j < k; ++j)
        if (j != i && ((X >> j) & 1)) best = min(best, F[((i << k) | X) * k + j]);
    }
    tour[k * W * k + t] = best;
  }
  // the level's compact tables (after W2): for mask rank j, X = the groups
  // outside S_j (n = k - level of them, in increasing order): W2[i][X] of
  // each, then path[i][X][i2] of each pair i < i2 in order
  __syncthreads();
  const int n = k - a.level, E = n + n * (n - 1) / 2;
  int32_t* ct = tour + k * W * k + k * W;
  for (int j = threadIdx.x; j < a.m; j += blockDim.x) {
    const uint32_t X = (uint32_t)(W - 1) ^ (uint32_t)a.lmasks[j];
    int32_t* e = ct + j * E;
    int ai = 0, p = n;
    for (uint32_t xi = X; xi; xi &= xi - 1u, ++ai) {
      const int i = __ffs(xi) - 1;
      e[ai] = tour[k * W * k + i * W + (int)X];
      for (uint32_t xj = xi & (xi - 1u); xj; xj &= xj - 1u, ++p) e[p] = F[((i << k) | (int)X) * k + __ffs(xj) - 1];
    }
  }
}

__global__ void k_argmin(int32_t V, const int32_t* __restrict__ full_slice, int32_t stride, Counters* ctr) {
  unsigned long long best = ~0ull;
  for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    const int32_t c = full_slice[(int64_t)v * stride];
    if (c < kInf) {
      const unsigned long long p = ((unsigned long long)(uint32_t)c << 32) | (uint32_t)v;
      best = p < best ? p : best;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long x = __shfl_xor_sync(0xffffffffu, best, o);
    best = x < best ? x : best;
  }
  if ((threadIdx.x & 31) == 0 && best != ~0ull) atomicMin(&ctr->best, best);
}

// -------------------------------------------------------------- backtrack --
// One CTA walks the parent records from (root, full) level by level: a
// frontier of states is expanded in parallel (grow -> child state through
// the recorded CSR entry, merge -> both halves), emitting tree vertices and
// edges. Every read is bounds-checked and the walk stops after `cap`
// states, so a corrupt record cannot fault or loop.
__global__ void __launch_bounds__(256) k_backtrack(GraphDev g, int64_t nnz, const int32_t* __restrict__ par,
                                                   const MaskInfo* __restrict__ minfo, int32_t full,
                                                   Counters* ctr, int2* qa, int2* qb, int32_t* out_v,
                                                   int3* out_e, int32_t cap) {
  __shared__ int32_t na, nb, processed;
  const unsigned long long best = ctr->best;
  if (threadIdx.x == 0) {
    na = 0;
    nb = 0;
    processed = 0;
    ctr->bt_nv = 0;
    ctr->bt_ne = 0;
    if (best != ~0ull && (int32_t)(best >> 32) < kInf && cap > 0) {
      qa[0] = make_int2((int32_t)(best & 0xffffffffull), (int32_t)full);
      na = 1;
    }
  }
  __syncthreads();
  int2* cur = qa;
  int2* nxt = qb;
  while (na > 0) {
    for (int32_t i = threadIdx.x; i < na; i += blockDim.x) {
      const int2 st = cur[i];
      const int32_t v = st.x;
      const uint32_t S = (uint32_t)st.y;
      if (v < 0 || v >= g.V || S == 0u || S > (uint32_t)full) {
        atomicExch(&ctr->bt_overflow, 2);
        continue;
      }
      const int32_t vi = atomicAdd(&ctr->bt_nv, 1);
      if (vi < cap) out_v[vi] = v;
      const MaskInfo mi = minfo[S];
      const int32_t c = par[(int64_t)mi.base * g.V + (int64_t)v * mi.stride + mi.rank];
      if (c == kLeaf) continue;
      if (c >= 0) {
        if ((int64_t)c >= nnz || c < g.row_ptr[v] || c >= g.row_ptr[v + 1]) {
          atomicExch(&ctr->bt_overflow, 2);
          continue;
        }
        const int2 x = g.adj[c];
        const int32_t ei = atomicAdd(&ctr->bt_ne, 1);
        if (ei < cap) out_e[ei] = make_int3(v, x.x, x.y);
        const int32_t p = atomicAdd(&nb, 1);
        if (p < cap) nxt[p] = make_int2(x.x, (int32_t)S);
      } else {
        const uint32_t s1 = (uint32_t)(-c);
        if (s1 == 0u || (s1 & ~S) != 0u || s1 == S) {
          atomicExch(&ctr->bt_overflow, 2);
          continue;
        }
        const int32_t p = atomicAdd(&nb, 2);
        if (p + 1 < cap) {
          nxt[p] = make_int2(v, (int32_t)s1);
          nxt[p + 1] = make_int2(v, (int32_t)(S ^ s1));
        }
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      processed += na;
      int32_t n = nb;
      if (n > cap || processed > cap) {
        atomicExch(&ctr->bt_overflow, 1);
        n = 0;
      }
      na = n;
      nb = 0;
    }
    __syncthreads();
    int2* t = cur;
    cur = nxt;
    nxt = t;
  }
  if (threadIdx.x == 0) ctr->bt_states = processed;
}

// ---------------------------------------------------------------- launchers --
cudaError_t launch_group_masks(const int32_t* group_ptr, const int32_t* members, const int32_t* perm, int32_t k,
                               uint32_t* gmask, cudaStream_t stream) {
  k_group_masks<<<64, 256, 0, stream>>>(group_ptr, members, perm, k, gmask);
  return cudaGetLastError();
}

// Dynamic shared memory a launch may take without opting in: 48 KB less
// the kernel's static shared memory (under 1 KB for the merge kernels).
constexpr size_t kSmemNoOptIn = 47 * 1024;

cudaError_t launch_merge(const GraphDev& g, const LevelArgs& a, const MergeLevels& ml, cudaStream_t stream) {
  if (a.k <= kMergeTabK && a.msplit_ptr) {
    int32_t words = 0;  // lower-level row words per vertex
    for (int l = 1; l < a.level; ++l) words += ml.stride[l];
    const int tn = a.k - a.level;
    const int64_t tour_words = a.tour ? (int64_t)a.m * (tn + tn * (tn - 1) / 2) : 0;  // compact tour tables
    if (words > kMergeTeamMinWords && (a.m >= kMergeTeamMinMasks || words > 2 * kMergeTeamMinWords)) {  // a team
      const int t = words <= kMergeStagedWords ? 4 : 32;
      const size_t smem = (size_t)((a.m + 2) & ~1) * sizeof(int32_t) + (size_t)a.nsplits * sizeof(int2) +
                          (size_t)tour_words * sizeof(int32_t) +
                          (size_t)(kMergeTeamThreads / t) * (words | 1) * sizeof(int32_t);
      const bool lane_masks = a.m >= t;
      const void* fn = t == 4 ? (lane_masks ? (const void*)k_merge_team<4, true> : (const void*)k_merge_team<4, false>)
                              : (lane_masks ? (const void*)k_merge_team<32, true> : (const void*)k_merge_team<32, false>);
      if (smem > kSmemNoOptIn) {  // up to ~75 KB (set on the current device every time)
        const cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
      }
      const int teams = kMergeTeamThreads / t;
      const int64_t blocks = std::min<int64_t>(((int64_t)g.V + teams - 1) / teams, 4096);
      const dim3 grid((unsigned)blocks), block(kMergeTeamThreads);
      if (t == 4 && lane_masks)
        k_merge_team<4, true><<<grid, block, smem, stream>>>(g, a, ml, words);
      else if (t == 4)
        k_merge_team<4, false><<<grid, block, smem, stream>>>(g, a, ml, words);
      else if (lane_masks)
        k_merge_team<32, true><<<grid, block, smem, stream>>>(g, a, ml, words);
      else
        k_merge_team<32, false><<<grid, block, smem, stream>>>(g, a, ml, words);
      return cudaGetLastError();
    }
    // a thread per vertex (at most kMergeTeamMinWords words, or the short single-mask merges)
    const size_t smem = (size_t)((a.m + 2) & ~1) * sizeof(int32_t) + (size_t)a.nsplits * sizeof(int2) +
                        (size_t)tour_words * sizeof(int32_t) + (size_t)words * 128 * sizeof(int32_t);
    if (smem > kSmemNoOptIn) {  // up to ~75 KB (set on the current device every time)
      const cudaError_t e =
          cudaFuncSetAttribute(k_merge_staged<128>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
    }
    const int64_t blocks = ((int64_t)g.V + 127) / 128;
    k_merge_staged<128><<<(unsigned)blocks, 128, smem, stream>>>(g, a, ml);
    return cudaGetLastError();
  }
  const int64_t total = (int64_t)g.V * a.stride;
  int64_t blocks = (total + kGrowThreads - 1) / kGrowThreads;
  if (blocks > (1 << 20)) blocks = 1 << 20;
  k_merge<<<(unsigned)blocks, kGrowThreads, 0, stream>>>(g, a);
  return cudaGetLastError();
}

namespace {
template <class Kernel>
int resident_blocks(Kernel kern) {
  int o = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, kern, kGrowThreads, 0) != cudaSuccess || o < 1) o = 2;
  return o;
}

// Every block of a round is resident at once (grid-stride loops inside).
template <class Kernel>
cudaError_t launch_round(Kernel kern, int occ, const GraphDev& g, const LevelArgs& a, int num_sms,
                         int vertices_per_block, cudaStream_t stream) {
  const int64_t needed = ((int64_t)g.V + vertices_per_block - 1) / vertices_per_block;
  int64_t blocks = (int64_t)num_sms * occ;
  if (blocks > needed) blocks = needed;
  if (blocks < 1) blocks = 1;
  kern<<<(unsigned)blocks, kGrowThreads, 0, stream>>>(g, a);
  return cudaGetLastError();
}

template <int L>
cudaError_t hub_round(const GraphDev& g, const LevelArgs& a, int num_sms, cudaStream_t stream, int64_t* launches) {
  if (g.nchunks == 0) return cudaSuccess;
  static const int occ = resident_blocks(k_grow_hubs<L>);
  const int64_t warps_per_block = kGrowThreads / 32;
  int64_t blocks = (g.nchunks + warps_per_block - 1) / warps_per_block;
  if (blocks > (int64_t)num_sms * occ) blocks = (int64_t)num_sms * occ;
  k_grow_hubs<L><<<(unsigned)blocks, kGrowThreads, 0, stream>>>(g, a);
  ++*launches;
  return cudaGetLastError();
}

template <int GP>
cudaError_t hub_team_round(const GraphDev& g, const LevelArgs& a, int num_sms, cudaStream_t stream,
                           int64_t* launches) {
  if (g.nsegs == 0) return cudaSuccess;
  static const int occ = resident_blocks(k_grow_hubs_team<GP>);
  const int64_t warps_per_block = kGrowThreads / 32;
  int64_t blocks = (g.nsegs + warps_per_block - 1) / warps_per_block;
  if (blocks > (int64_t)num_sms * occ) blocks = (int64_t)num_sms * occ;
  k_grow_hubs_team<GP><<<(unsigned)blocks, kGrowThreads, 0, stream>>>(g, a);
  ++*launches;
  return cudaGetLastError();
}

template <int MP>
cudaError_t thread_round(const GraphDev& g, const LevelArgs& a, int num_sms, cudaStream_t stream) {
  static const int occ = resident_blocks(k_grow_thread<MP>);
  return launch_round(k_grow_thread<MP>, occ, g, a, num_sms, kGrowThreads, stream);
}

template <int G, int L, bool SPARSE_ONLY = false>
cudaError_t group_round(const GraphDev& g, const LevelArgs& a, int num_sms, cudaStream_t stream) {
  static const int occ = resident_blocks(k_grow_group<G, L, SPARSE_ONLY>);
  return launch_round(k_grow_group<G, L, SPARSE_ONLY>, occ, g, a, num_sms, kGrowThreads / G, stream);
}
}  // namespace

template <int G>
cudaError_t team_round(const GraphDev& g, const LevelArgs& a, int num_sms, cudaStream_t stream) {
  constexpr int UNR = 4;
  static const int occ = resident_blocks(k_grow_team<G, UNR>);
  return launch_round(k_grow_team<G, UNR>, occ, g, a, num_sms, kGrowThreads / G, stream);
}

cudaError_t launch_grow_round(const GraphDev& g, const LevelArgs& a, int num_sms, cudaStream_t stream,
                              int64_t* launches) {
  const int lanes = (a.stride + 31) / 32;  // masks per lane in the hub kernel, in passes of at most 4
  const int G = a.stride >> 2;
  const cudaError_t he = a.stride <= kMaxThreadMasks
                             ? (G <= 1   ? hub_team_round<1>(g, a, num_sms, stream, launches)
                                : G <= 2 ? hub_team_round<2>(g, a, num_sms, stream, launches)
                                : G <= 4 ? hub_team_round<4>(g, a, num_sms, stream, launches)
                                         : hub_team_round<8>(g, a, num_sms, stream, launches))
                         : lanes <= 1 ? hub_round<1>(g, a, num_sms, stream, launches)
                         : lanes == 2 ? hub_round<2>(g, a, num_sms, stream, launches)
                         : lanes == 3 ? hub_round<3>(g, a, num_sms, stream, launches)
                                      : hub_round<4>(g, a, num_sms, stream, launches);
  if (he != cudaSuccess) return he;
  ++*launches;
  // waves with a thread kernel: sparse rounds there, then dense rounds in the
  // team kernel (each of the two returns at once in the other's rounds; a
  // dense round that follows a sparse one in the same pass runs right away)
  cudaError_t te = cudaSuccess;
  switch (a.stride) {
    case 4: te = thread_round<4>(g, a, num_sms, stream); break;
    case 8: te = thread_round<8>(g, a, num_sms, stream); break;
    case 12: te = thread_round<12>(g, a, num_sms, stream); break;
    case 16: te = thread_round<16>(g, a, num_sms, stream); break;
    case 20: te = thread_round<20>(g, a, num_sms, stream); break;
    case 24: te = thread_round<24>(g, a, num_sms, stream); break;
    default: te = cudaErrorNotSupported; break;
  }
  if (te != cudaErrorNotSupported) {
    if (te != cudaSuccess) return te;
    ++*launches;
    switch (a.stride) {
      case 4: te = team_round<1>(g, a, num_sms, stream); break;
      case 8: te = team_round<2>(g, a, num_sms, stream); break;
      case 12: te = team_round<3>(g, a, num_sms, stream); break;
      case 16: te = team_round<4>(g, a, num_sms, stream); break;
      case 20: te = team_round<5>(g, a, num_sms, stream); break;
      default: te = team_round<6>(g, a, num_sms, stream); break;
    }
    return te;
  }
  // strides of the waves of k = 7 and 8: sparse rounds by lane groups, dense
  // rounds by teams of stride/4 lanes (16-byte quarters of the rows)
  cudaError_t ge = cudaErrorNotSupported;
  switch (a.stride) {
    case 28: ge = group_round<16, 2, true>(g, a, num_sms, stream); break;
    case 36: ge = group_round<32, 2, true>(g, a, num_sms, stream); break;
    case 56: ge = group_round<32, 2, true>(g, a, num_sms, stream); break;
    case 72: ge = group_round<32, 3, true>(g, a, num_sms, stream); break;
    default: break;
  }
  if (ge != cudaErrorNotSupported) {
    if (ge != cudaSuccess) return ge;
    ++*launches;
    switch (a.stride) {
      case 28: return team_round<7>(g, a, num_sms, stream);
      case 36: return team_round<9>(g, a, num_sms, stream);
      case 56: return team_round<14>(g, a, num_sms, stream);
      default: return team_round<18>(g, a, num_sms, stream);
    }
  }
  if (a.stride <= 32) return group_round<16, 2>(g, a, num_sms, stream);
  if (a.stride <= 64) return group_round<32, 2>(g, a, num_sms, stream);
  if (a.stride <= 96) return group_round<32, 3>(g, a, num_sms, stream);
  return group_round<32, 4>(g, a, num_sms, stream);
}

cudaError_t launch_tour_table(const LevelArgs& a, const int32_t* group_ptr, const int32_t* members,
                              const int32_t* perm, int32_t* tour, cudaStream_t stream) {
  if (a.k > kTourMaxK) return cudaErrorInvalidValue;
  const size_t smem = a.k <= kTourSmemMaxK ? (size_t)a.k * ((size_t)1 << a.k) * a.k * sizeof(int32_t) : 0;
  if (smem > kSmemNoOptIn) {  // k = 8 (set on the current device every time)
    const cudaError_t e = cudaFuncSetAttribute(k_tour_table, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  k_tour_table<<<1, 1024, smem, stream>>>(a, group_ptr, members, perm, tour);
  return cudaGetLastError();
}

cudaError_t launch_seed(const GraphDev& g, const LevelArgs& a, int num_sms, cudaStream_t stream) {
  int64_t blocks = ((int64_t)g.V + kGrowThreads - 1) / kGrowThreads;  // >= one warp per 32 vertices
  if (blocks > (int64_t)num_sms * 8) blocks = (int64_t)num_sms * 8;
  k_seed<<<(unsigned)blocks, kGrowThreads, 0, stream>>>(g, a);
  return cudaGetLastError();
}

namespace {
// Lowers the solve's bound to cand (a bound <= 0 is none yet): the learned
// proposal's cost, injected while the solve's graph runs.
__global__ void k_bound_min(SolveParams* p, int32_t cand) {
  int32_t* ub = &p->ub;
  int32_t old = *reinterpret_cast<volatile int32_t*>(ub);
  while (old <= 0 || cand < old) {
    const int32_t prev = atomicCAS(ub, old, cand);
    if (prev == old) break;
    old = prev;
  }
}
}  // namespace

cudaError_t launch_bound_min(SolveParams* params, int32_t cand, cudaStream_t stream) {
  k_bound_min<<<1, 1, 0, stream>>>(params, cand);
  return cudaGetLastError();
}

cudaError_t launch_ub_refine(const GraphDev& g, const LevelArgs& a, int num_sms, cudaStream_t stream) {
  int64_t blocks = ((int64_t)g.V + kGrowThreads - 1) / kGrowThreads;
  if (blocks > (int64_t)num_sms * 8) blocks = (int64_t)num_sms * 8;
  k_ub_refine<<<(unsigned)blocks, kGrowThreads, 0, stream>>>(g, a);
  return cudaGetLastError();
}

cudaError_t launch_argmin(const GraphDev& g, const int32_t* full_slice, int32_t stride, Counters* ctr,
                          cudaStream_t stream) {
  int blocks = (g.V + 255) / 256;
  if (blocks > 4096) blocks = 4096;
  k_argmin<<<blocks, 256, 0, stream>>>(g.V, full_slice, stride, ctr);
  return cudaGetLastError();
}

cudaError_t launch_backtrack(const GraphDev& g, int64_t nnz, const int32_t* par, const MaskInfo* minfo,
                             int32_t full, Counters* ctr, int2* qa, int2* qb, int32_t* out_v, int3* out_e,
                             int32_t cap, cudaStream_t stream) {
  k_backtrack<<<1, 256, 0, stream>>>(g, nnz, par, minfo, full, ctr, qa, qb, out_v, out_e, cap);
  return cudaGetLastError();
}

}  // namespace gst
