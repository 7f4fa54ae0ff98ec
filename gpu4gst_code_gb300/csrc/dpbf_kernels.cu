// DPBF kernels for sm_103a: group masks, merge, growth round, argmin and
// backtrack. Plain SIMT integer code: the DP is min-plus over int32 costs
// and is bound by HBM traffic (growth) and the INT32 pipe (merge); nothing
// here is a contraction, so no tensor-core path applies.
//
// What each kernel replaces in the reference (src/DPQ.cu):
//   k_group_masks   set_max_ID / get_max (:22-47) — groups(v) as a bit mask
//   k_merge         the merge half of Relax (:286-314) and the seeding of
//                   T(v,p)=0 for p inside groups(v) (:638-659), done as one
//                   pass per DP wave over every vertex's submask splits
//   k_grow          dis0_init (:404-433) and the grow half of Relax
//                   (:259-282): one label-correcting round, pull form
//   k_argmin        host min scan over T(v,full) (:712-721)
//   k_backtrack     host BFS over parent records (:729-758)
#include <cstdint>

#include "dpbf.cuh"

namespace gst {

namespace {

__device__ __forceinline__ long long warp_sum_ll(long long x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

__device__ __forceinline__ void flush_stat(long long* stats, int slot, long long x) {
  x = warp_sum_ll(x);
  if ((threadIdx.x & 31) == 0 && x != 0) atomicAdd(reinterpret_cast<unsigned long long*>(stats + slot),
                                                   static_cast<unsigned long long>(x));
}

__device__ __forceinline__ void flush_count(int32_t* dst, int x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  if ((threadIdx.x & 31) == 0 && x != 0) atomicAdd(dst, x);
}

// Largest cost allowed for state (v,S) under the bound: ub - LB(v, full^S)
// with LB = max over groups g outside S of T(v,{g}) (one-label bound,
// src/DPQ.cu:361-403, applied per remaining group set). -1 = state dead.
__device__ __forceinline__ int32_t prune_cap(const LevelArgs& a, int32_t v, uint32_t S) {
  const int32_t* d = a.cost + a.base1 + (int64_t)v * a.k;
  int32_t lb = 0;
  for (int g = 0; g < a.k; ++g)
    if (!((S >> g) & 1u)) lb = max(lb, __ldg(d + g));
  const int32_t cap = a.ub - lb;
  return cap < 0 ? -1 : cap;
}

}  // namespace

// ------------------------------------------------------------ group masks --
__global__ void k_group_masks(const int32_t* __restrict__ group_ptr, const int32_t* __restrict__ members,
                              int32_t k, int32_t n, uint32_t* __restrict__ gmask) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int32_t g = 0;
  while (g + 1 < k && group_ptr[g + 1] <= i) ++g;
  atomicOr(gmask + members[i], 1u << g);
}

// ------------------------------------------------------------------ merge --
// One thread per (v, S) of the level: T(v,S) = 0 when S is inside groups(v),
// else the best split T(v,S1) + T(v,S^S1) over S1 holding the lowest bit of
// S (each unordered split once). Writes every entry of the level slice and
// marks vertices with a finite entry as the first growth frontier.
__global__ void __launch_bounds__(kGrowThreads) k_merge(GraphDev g, LevelArgs a) {
  const int64_t total = (int64_t)g.V * a.m;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int finite = 0, overflow = 0;
  long long splits = 0;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += stride) {
    const int32_t v = (int32_t)(idx / a.m);
    const int32_t j = (int32_t)(idx - (int64_t)v * a.m);
    const uint32_t S = (uint32_t)__ldg(a.lmasks + j);
    int32_t best = ((__ldg(a.gmask + v) & S) == S) ? 0 : kInf;
    int32_t code = kLeaf;
    if (a.level >= 2 && best != 0) {
      const uint32_t low = S & (0u - S), rest = S ^ low;
      for (uint32_t sub = (rest - 1u) & rest;; sub = (sub - 1u) & rest) {
        const uint32_t s1 = sub | low, s2 = S ^ s1;
        const MaskInfo i1 = a.minfo[s1], i2 = a.minfo[s2];
        const int32_t c1 = a.cost[(int64_t)i1.base * g.V + (int64_t)v * i1.m + i1.rank];
        const int32_t c2 = a.cost[(int64_t)i2.base * g.V + (int64_t)v * i2.m + i2.rank];
        const int32_t c = c1 + c2;  // both <= kInf < 2^30: no wrap
        if (c < best) {
          if (c >= kInf) {
            overflow = 1;
          } else {
            best = c;
            code = -(int32_t)s1;
          }
        } else if (c >= kInf && c1 < kInf && c2 < kInf) {
          overflow = 1;
        }
        ++splits;
        if (sub == 0u) break;
      }
    }
    if (a.ub > 0 && best < kInf && a.level >= 2) {
      const int32_t cap = prune_cap(a, v, S);
      if (best > cap) {
        best = kInf;
        code = kLeaf;
      }
    }
    a.cost[a.base + idx] = best;
    a.par[a.base + idx] = code;
    if (best < kInf) {
      a.next_flag[v] = 1;
      ++finite;
    }
  }
  flush_count(a.cur_changed, finite);
  if (a.stats) {
    flush_stat(a.stats, kStatSplits, splits);
  }
  if (overflow) atomicExch(&a.ctr->overflow, 1);
  {
    long long f = warp_sum_ll(finite);
    if ((threadIdx.x & 31) == 0 && f) atomicAdd(&a.ctr->states, (unsigned long long)f);
  }
}

// ------------------------------------------------------------------- grow --
// One label-correcting round for every mask of the level, pull form: each
// vertex u takes min over neighbours v changed in the previous round of
// T(v,S) + w(u,v), for all masks S of the level at once (the m entries of a
// row are contiguous). Only u writes u's entries, so a state's cost and its
// parent are always written together by one thread (the reference writes
// the parent after a separate atomicMin, DPQ.cu:269-272).
//
// Rows with degree <= kDegBig: a group of G lanes per vertex; lanes load G
// CSR entries at once, then broadcast each changed neighbour and gather its
// row (lane j holds masks j, j+G, ...). Rows with degree > kDegBig: one CTA
// per vertex (blocks [0, nbig)), partial minima combined in shared memory.
template <int G, int MPL>
__global__ void __launch_bounds__(kGrowThreads) k_grow(GraphDev g, LevelArgs a) {
  if (*a.prev_changed == 0) {
    // converged: keep the rotation consistent so later rounds also see 0
    if (blockIdx.x == 0 && threadIdx.x == 0) *a.zero_changed = 0;
    return;
  }
  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int glane = lane & (G - 1);
  const int gbase = lane & ~(G - 1);
  const unsigned gmask_lanes = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << gbase);
  const unsigned gbits = (G == 32) ? 0xffffffffu : ((1u << G) - 1u);
  const int m = a.m;
  constexpr int CH = G * MPL;  // masks per pass
  const bool prune = a.ub > 0;
  const bool stats = a.stats != nullptr;
  long long st_vert = 0, st_ent = 0, st_rows = 0, st_imp = 0;
  int changed = 0, overflow = 0;

  if ((int)blockIdx.x < g.nbig) {
    // ---------------------------------------------- one CTA, one big row --
    __shared__ unsigned long long red[CH];
    __shared__ int32_t cap_s[CH];
    __shared__ int any_imp;
    constexpr int NG = kGrowThreads / G;
    const int gi = tid / G;
    const int32_t u = g.big[blockIdx.x];
    const int32_t beg = g.row_ptr[u], end = g.row_ptr[u + 1];
    const int64_t rowu = a.base + (int64_t)u * m;
    if (tid == 0) any_imp = 0;
    for (int jc = 0; jc < m; jc += CH) {
      __syncthreads();
      if (tid < CH) {
        const int j = jc + tid;
        const int32_t own = (j < m) ? a.cost[rowu + j] : -1;
        red[tid] = ((unsigned long long)(uint32_t)own << 32) | 0xffffffffull;
        int32_t cap = kInf - 1;
        if (j < m && prune) cap = prune_cap(a, u, (uint32_t)__ldg(a.lmasks + j));
        cap_s[tid] = (j < m) ? cap : -1;
      }
      __syncthreads();
      int32_t best[MPL], code[MPL], capl[MPL];
#pragma unroll
      for (int t = 0; t < MPL; ++t) {
        best[t] = kInf;
        code[t] = -1;
        capl[t] = cap_s[glane + t * G];
      }
      for (int32_t e0 = beg + gi * G; e0 < end; e0 += NG * G) {
        const int32_t e = e0 + glane;
        int32_t nv = 0, nw = 0;
        bool act = false;
        if (e < end) {
          const int2 x = g.adj[e];
          nv = x.x;
          nw = x.y;
          act = a.cur_flag[nv] != 0;
        }
        unsigned bal = (__ballot_sync(gmask_lanes, act) >> gbase) & gbits;
        if (stats && glane == 0) st_rows += __popc(bal);
        while (bal) {
          const int src = __ffs(bal) - 1;
          bal &= bal - 1u;
          const int32_t v = __shfl_sync(gmask_lanes, nv, src, G);
          const int32_t w = __shfl_sync(gmask_lanes, nw, src, G);
          const int64_t rowv = a.base + (int64_t)v * m + jc;
#pragma unroll
          for (int t = 0; t < MPL; ++t) {
            const int j = glane + t * G;
            if (jc + j < m) {
              int32_t c = a.cost[rowv + j];
              if (c < kInf) {
                c += w;
                if (c >= kInf) overflow = 1;
                if (c < best[t] && c <= capl[t]) {
                  best[t] = c;
                  code[t] = e0 + src;
                }
              }
            }
          }
        }
      }
#pragma unroll
      for (int t = 0; t < MPL; ++t) {
        const int j = glane + t * G;
        if (jc + j < m && best[t] < kInf)
          atomicMin(&red[j], ((unsigned long long)(uint32_t)best[t] << 32) | (uint32_t)code[t]);
      }
      __syncthreads();
      if (tid < CH && jc + tid < m) {
        const unsigned long long r = red[tid];
        const int32_t c = (int32_t)(r >> 32);
        const int32_t own = a.cost[rowu + jc + tid];
        if (c < own) {
          a.cost[rowu + jc + tid] = c;
          a.par[rowu + jc + tid] = (int32_t)(uint32_t)(r & 0xffffffffull);
          any_imp = 1;
          ++st_imp;
        }
      }
    }
    __syncthreads();
    if (tid == 0) {
      st_vert = 1;
      st_ent = end - beg;
      if (any_imp) {
        a.next_flag[u] = 1;
        changed = 1;
      }
    }
  } else {
    // ------------------------------------------- groups over small rows --
    const int32_t sblock = blockIdx.x - g.nbig;
    const int32_t nsblocks = gridDim.x - g.nbig;
    const int64_t sthread = (int64_t)sblock * blockDim.x + tid;
    const int64_t nsthreads = (int64_t)nsblocks * blockDim.x;
    for (int64_t i = sthread; i < g.V; i += nsthreads) a.clear_flag[i] = 0;
    if (sthread == 0) {
      *a.zero_changed = 0;
      if (stats) atomicAdd(reinterpret_cast<unsigned long long*>(a.stats + kStatRounds), 1ull);
    }
    const int64_t ngroups = nsthreads / G;
    for (int64_t uu = sthread / G; uu < g.V; uu += ngroups) {
      const int32_t u = (int32_t)uu;
      const int32_t beg = g.row_ptr[u], end = g.row_ptr[u + 1];
      if (end - beg > kDegBig) continue;
      const int64_t rowu = a.base + (int64_t)u * m;
      bool imp_any = false;
      for (int jc = 0; jc < m; jc += CH) {
        int32_t own[MPL], best[MPL], code[MPL], capl[MPL];
        bool live = false;
#pragma unroll
        for (int t = 0; t < MPL; ++t) {
          const int j = jc + glane + t * G;
          own[t] = (j < m) ? a.cost[rowu + j] : -1;
          best[t] = own[t];
          code[t] = -1;
          capl[t] = (j < m) ? kInf - 1 : -1;
          if (j < m && prune) capl[t] = prune_cap(a, u, (uint32_t)__ldg(a.lmasks + j));
          live |= capl[t] >= 0 && own[t] != 0;
        }
        // no lane can improve: skip the row scan
        if (!(__ballot_sync(gmask_lanes, live) & gmask_lanes)) continue;
        for (int32_t e0 = beg; e0 < end; e0 += G) {
          const int32_t e = e0 + glane;
          int32_t nv = 0, nw = 0;
          bool act = false;
          if (e < end) {
            const int2 x = g.adj[e];
            nv = x.x;
            nw = x.y;
            act = a.cur_flag[nv] != 0;
          }
          unsigned bal = (__ballot_sync(gmask_lanes, act) >> gbase) & gbits;
          if (stats && glane == 0) st_rows += __popc(bal);
          while (bal) {
            const int src = __ffs(bal) - 1;
            bal &= bal - 1u;
            const int32_t v = __shfl_sync(gmask_lanes, nv, src, G);
            const int32_t w = __shfl_sync(gmask_lanes, nw, src, G);
            const int64_t rowv = a.base + (int64_t)v * m + jc;
#pragma unroll
            for (int t = 0; t < MPL; ++t) {
              const int j = glane + t * G;
              if (jc + j < m) {
                int32_t c = a.cost[rowv + j];
                if (c < kInf) {
                  c += w;
                  if (c >= kInf) overflow = 1;
                  if (c < best[t] && c <= capl[t]) {
                    best[t] = c;
                    code[t] = e0 + src;
                  }
                }
              }
            }
          }
        }
        bool imp = false;
#pragma unroll
        for (int t = 0; t < MPL; ++t) {
          const int j = jc + glane + t * G;
          if (j < m && best[t] < own[t]) {
            a.cost[rowu + j] = best[t];
            a.par[rowu + j] = code[t];
            imp = true;
            ++st_imp;
          }
        }
        imp_any |= (__ballot_sync(gmask_lanes, imp) & gmask_lanes) != 0;
      }
      if (glane == 0) {
        st_vert += 1;
        st_ent += end - beg;
        if (imp_any) {
          a.next_flag[u] = 1;
          ++changed;
        }
      }
    }
  }
  flush_count(a.cur_changed, changed);
  if (stats) {
    flush_stat(a.stats, kStatVertices, st_vert);
    flush_stat(a.stats, kStatEntries, st_ent);
    flush_stat(a.stats, kStatRows, st_rows);
    flush_stat(a.stats, kStatGathered, st_rows * m);
    flush_stat(a.stats, kStatImproved, st_imp);
    // algorithmic bytes: row_ptr pair + own row per scanned vertex, (col,w)
    // + frontier byte per scanned entry, one m-entry row per changed
    // neighbour, cost + parent per improved entry, one flag per changed row
    flush_stat(a.stats, kStatBytes,
               st_vert * (8 + 4LL * m) + st_ent * 9 + st_rows * 4LL * m + st_imp * 8 + changed);
  }
  {
    long long imp = warp_sum_ll(st_imp);
    if (lane == 0 && imp) atomicAdd(&a.ctr->states, (unsigned long long)imp);
  }
  if (overflow) atomicExch(&a.ctr->overflow, 1);
}

// ----------------------------------------------------------------- argmin --
__global__ void k_argmin(int32_t V, const int32_t* __restrict__ full_slice, Counters* ctr) {
  unsigned long long best = ~0ull;
  for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    const int32_t c = full_slice[v];
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
      const int32_t c = par[(int64_t)mi.base * g.V + (int64_t)v * mi.m + mi.rank];
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
cudaError_t launch_group_masks(const int32_t* group_ptr, const int32_t* members, int32_t k, int32_t nmembers,
                               uint32_t* gmask, cudaStream_t stream) {
  if (nmembers <= 0) return cudaSuccess;
  k_group_masks<<<(nmembers + 255) / 256, 256, 0, stream>>>(group_ptr, members, k, nmembers, gmask);
  return cudaGetLastError();
}

cudaError_t launch_merge(const GraphDev& g, const LevelArgs& a, cudaStream_t stream) {
  const int64_t total = (int64_t)g.V * a.m;
  int64_t blocks = (total + kGrowThreads - 1) / kGrowThreads;
  if (blocks > (1 << 20)) blocks = 1 << 20;
  k_merge<<<(unsigned)blocks, kGrowThreads, 0, stream>>>(g, a);
  return cudaGetLastError();
}

namespace {
template <int G, int MPL>
cudaError_t grow_instance(const GraphDev& g, const LevelArgs& a, int num_sms, cudaStream_t stream) {
  static int occ = 0;  // resident blocks per SM for this instance
  if (occ == 0) {
    int o = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k_grow<G, MPL>, kGrowThreads, 0) != cudaSuccess || o < 1)
      o = 4;
    occ = o;
  }
  const int64_t small_blocks_needed = ((int64_t)g.V * G + kGrowThreads - 1) / kGrowThreads;
  int64_t small_blocks = (int64_t)num_sms * occ;
  if (small_blocks > small_blocks_needed) small_blocks = small_blocks_needed;
  if (small_blocks < 1) small_blocks = 1;
  k_grow<G, MPL><<<(unsigned)(g.nbig + small_blocks), kGrowThreads, 0, stream>>>(g, a);
  return cudaGetLastError();
}
}  // namespace

cudaError_t launch_grow_round(const GraphDev& g, const LevelArgs& a, int num_sms, cudaStream_t stream) {
  const int m = a.m;
  if (m <= 8) return grow_instance<8, 1>(g, a, num_sms, stream);
  if (m <= 16) return grow_instance<16, 1>(g, a, num_sms, stream);
  if (m <= 32) return grow_instance<32, 1>(g, a, num_sms, stream);
  if (m <= 64) return grow_instance<32, 2>(g, a, num_sms, stream);
  if (m <= 96) return grow_instance<32, 3>(g, a, num_sms, stream);
  return grow_instance<32, 4>(g, a, num_sms, stream);
}

cudaError_t launch_argmin(const GraphDev& g, const int32_t* full_slice, Counters* ctr, cudaStream_t stream) {
  int blocks = (g.V + 255) / 256;
  if (blocks > 4096) blocks = 4096;
  k_argmin<<<blocks, 256, 0, stream>>>(g.V, full_slice, ctr);
  return cudaGetLastError();
}

cudaError_t launch_backtrack(const GraphDev& g, int64_t nnz, const int32_t* par, const MaskInfo* minfo,
                             int32_t full, Counters* ctr, int2* qa, int2* qb, int32_t* out_v, int3* out_e,
                             int32_t cap, cudaStream_t stream) {
  k_backtrack<<<1, 256, 0, stream>>>(g, nnz, par, minfo, full, ctr, qa, qb, out_v, out_e, cap);
  return cudaGetLastError();
}

}  // namespace gst
