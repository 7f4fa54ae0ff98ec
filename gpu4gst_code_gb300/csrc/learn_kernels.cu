// Kernels of the learned upper-bound proposal (declared in learn.cuh):
// query features, bf16 inference with tcgen05 tensor-core GEMMs over
// 128-vertex tiles (TMA-staged operands, tensor-memory accumulators), fp32 forward/backward training kernels and the Adam update.
//
// Query features x[v][0..15] (internal vertex IDs, k groups):
//   0  1                          6  all k groups within 1 hop
//   1  log(1 + deg) / 8           7  all k groups within 2 hops
//   2  groups v belongs to / k    8  all k groups within 3 hops
//   3  groups within 1 hop / k    9  neighbours in some group / deg
//   4  groups within 2 hops / k   10 v belongs to some group
//   5  groups within 3 hops / k   11..15 zero
// ("within h hops" includes v itself.)
#include <algorithm>
#include <cstdint>

#include "learn.cuh"

namespace gst {
namespace {

__device__ __forceinline__ int64_t gwarp() { return ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; }
__device__ __forceinline__ int64_t nwarps() { return ((int64_t)gridDim.x * blockDim.x) >> 5; }

int grid_for(int64_t items, int per_block, int cap = 152 * 16) {
  int64_t b = (items + per_block - 1) / per_block;
  if (b < 1) b = 1;
  if (b > cap) b = cap;
  return (int)b;
}

// -------------------------------------------------------------- features --
// out (zeroed by the caller) = in | OR over neighbours. Hub rows go one
// 32-entry chunk per warp (atomicOr); the other vertices a thread each.
__global__ void k_reach(GraphDev g, const int32_t* __restrict__ hub_of, const uint32_t* __restrict__ in,
                        uint32_t* __restrict__ out, int32_t* __restrict__ member_nbrs) {
  const int lane = threadIdx.x & 31;
  for (int64_t c = gwarp(); c < g.nchunks; c += nwarps()) {
    const int2 hc = g.hub_chunk[c];
    const int32_t u = g.big[hc.x];
    const int32_t e = hc.y + lane;
    uint32_t m = 0;
    if (e < g.row_ptr[u + 1]) m = in[g.adj[e].x];
    const uint32_t acc = __reduce_or_sync(0xffffffffu, m);
    const uint32_t cnt = __reduce_add_sync(0xffffffffu, m != 0u ? 1u : 0u);
    if (lane == 0) {
      atomicOr(out + u, acc | in[u]);
      if (member_nbrs && cnt) atomicAdd(member_nbrs + u, (int32_t)cnt);
    }
  }
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < g.V; v += (int64_t)gridDim.x * blockDim.x) {
    if (hub_of[v] >= 0) continue;
    const int32_t beg = g.row_ptr[v], end = g.row_ptr[v + 1];
    uint32_t acc = in[v];
    int32_t cnt = 0;
    for (int32_t e = beg; e < end; ++e) {
      const uint32_t m = in[g.adj[e].x];
      acc |= m;
      cnt += m != 0u;
    }
    out[v] = acc;
    if (member_nbrs) member_nbrs[v] = cnt;
  }
}

__global__ void k_features(GraphDev g, const uint32_t* __restrict__ m0, const uint32_t* __restrict__ r1,
                           const uint32_t* __restrict__ r2, const uint32_t* __restrict__ r3,
                           const int32_t* __restrict__ member_nbrs, int32_t k, float* __restrict__ x) {
  const float ik = 1.0f / (float)k;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < g.V; v += (int64_t)gridDim.x * blockDim.x) {
    const int32_t deg = g.row_ptr[v + 1] - g.row_ptr[v];
    const int c0 = __popc(m0[v]), c1 = __popc(r1[v]), c2 = __popc(r2[v]), c3 = __popc(r3[v]);
    float f[kFeat];
    f[0] = 1.0f;
    f[1] = log1pf((float)deg) * 0.125f;
    f[2] = c0 * ik;
    f[3] = c1 * ik;
    f[4] = c2 * ik;
    f[5] = c3 * ik;
    f[6] = c1 == k ? 1.0f : 0.0f;
    f[7] = c2 == k ? 1.0f : 0.0f;
    f[8] = c3 == k ? 1.0f : 0.0f;
    f[9] = deg > 0 ? (float)member_nbrs[v] / (float)deg : 0.0f;
    f[10] = c0 > 0 ? 1.0f : 0.0f;
#pragma unroll
    for (int i = 11; i < kFeat; ++i) f[i] = 0.0f;
    float4* xo = reinterpret_cast<float4*>(x + v * kFeat);
#pragma unroll
    for (int q = 0; q < kFeat / 4; ++q) xo[q] = make_float4(f[4 * q], f[4 * q + 1], f[4 * q + 2], f[4 * q + 3]);
  }
}

// ------------------------------------------------------------- inference --
__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
  const __nv_bfloat162 b = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&b);
}

__device__ __forceinline__ void add_bf16x8(float (&a)[8], const uint4 x) {
  const uint32_t w[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const float2 f = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&w[q]));
    a[2 * q] += f.x;
    a[2 * q + 1] += f.y;
  }
}

__global__ void k_pack_bf16(const float* __restrict__ p, __nv_bfloat16* __restrict__ wcat) {
  const int64_t n = (int64_t)kMpLayers * kHid * 2 * kHid;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int l = (int)(i / (kHid * 2 * kHid)) + 1;
    const int r = (int)(i % (kHid * 2 * kHid));
    const int o = r / (2 * kHid), c = r % (2 * kHid);
    const float* base = p + layer_off(l);
    const float w = c < kHid ? base[o * kHid + c] : base[kHid * kHid + o * kHid + (c - kHid)];
    wcat[i] = __float2bfloat16_rn(w);
  }
}

// Thread per vertex: all 64 outputs of h0 = relu(W0 x + b0) from W0 in
// shared memory (broadcast reads), the 16 features in registers, the row
// written as eight 16-byte stores.
__global__ void __launch_bounds__(256) k_infer_l0(int32_t V, const float* __restrict__ x, const float* __restrict__ p,
                                                  __nv_bfloat16* __restrict__ h) {
  __shared__ float sw[kHid][kFeat];
  __shared__ float sb[kHid];
  for (int i = threadIdx.x; i < kHid * kFeat; i += blockDim.x) sw[i / kFeat][i % kFeat] = p[kOffW0 + i];
  if (threadIdx.x < kHid) sb[threadIdx.x] = p[kOffB0 + threadIdx.x];
  __syncthreads();
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (int64_t)gridDim.x * blockDim.x) {
    float f[kFeat];
    const float4* xv = reinterpret_cast<const float4*>(x + v * kFeat);
#pragma unroll
    for (int q = 0; q < kFeat / 4; ++q) {
      const float4 t = xv[q];
      f[4 * q] = t.x;
      f[4 * q + 1] = t.y;
      f[4 * q + 2] = t.z;
      f[4 * q + 3] = t.w;
    }
    uint4* out = reinterpret_cast<uint4*>(h + v * kHid);
#pragma unroll 1
    for (int o8 = 0; o8 < kHid / 8; ++o8) {
      float y[8];
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        float acc = sb[o8 * 8 + t];
#pragma unroll
        for (int c = 0; c < kFeat; ++c) acc = fmaf(sw[o8 * 8 + t][c], f[c], acc);
        y[t] = fmaxf(acc, 0.0f);
      }
      out[o8] = make_uint4(pack_bf16x2(y[0], y[1]), pack_bf16x2(y[2], y[3]), pack_bf16x2(y[4], y[5]),
                           pack_bf16x2(y[6], y[7]));
    }
  }
}

// The neighbour mean of one layer's input, bf16 in and out: eight threads
// per vertex, 16 bytes (8 channels) each, fp32 accumulation; hub rows take
// their sums from hub_sum. No shared memory, so many warps are resident to
// cover the gathers' latency.
__global__ void __launch_bounds__(256) k_mean_bf16(GraphDev g, const int32_t* __restrict__ hub_of,
                                                   const float* __restrict__ hub_sum,
                                                   const __nv_bfloat16* __restrict__ hin,
                                                   __nv_bfloat16* __restrict__ agg) {
  const int sl = threadIdx.x & 7;
  for (int64_t v = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 3; v < g.V;
       v += ((int64_t)gridDim.x * blockDim.x) >> 3) {
    const int32_t beg = g.row_ptr[v], end = g.row_ptr[v + 1];
    const float inv = end > beg ? 1.0f / (float)(end - beg) : 0.0f;
    float a[8] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    const int32_t hb = hub_of[v];
    if (hb >= 0) {
      const float4* hs = reinterpret_cast<const float4*>(hub_sum + (int64_t)hb * kHid + 8 * sl);
      const float4 p0 = hs[0], p1 = hs[1];
      a[0] = p0.x; a[1] = p0.y; a[2] = p0.z; a[3] = p0.w;
      a[4] = p1.x; a[5] = p1.y; a[6] = p1.z; a[7] = p1.w;
    } else {
      int32_t e = beg;
      for (; e + 4 <= end; e += 4) {
        uint4 r[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) r[j] = reinterpret_cast<const uint4*>(hin + (int64_t)g.adj[e + j].x * kHid)[sl];
#pragma unroll
        for (int j = 0; j < 4; ++j) add_bf16x8(a, r[j]);
      }
      for (; e < end; ++e) add_bf16x8(a, reinterpret_cast<const uint4*>(hin + (int64_t)g.adj[e].x * kHid)[sl]);
    }
    reinterpret_cast<uint4*>(agg + v * kHid)[sl] =
        make_uint4(pack_bf16x2(a[0] * inv, a[1] * inv), pack_bf16x2(a[2] * inv, a[3] * inv),
                   pack_bf16x2(a[4] * inv, a[5] * inv), pack_bf16x2(a[6] * inv, a[7] * inv));
  }
}

__global__ void k_hub_sum_bf16(GraphDev g, const __nv_bfloat16* __restrict__ hin, float* __restrict__ hub_sum) {
  const int lane = threadIdx.x & 31;
  const __nv_bfloat162* h2 = reinterpret_cast<const __nv_bfloat162*>(hin);
  for (int64_t c = gwarp(); c < g.nchunks; c += nwarps()) {
    const int2 hc = g.hub_chunk[c];
    const int32_t u = g.big[hc.x];
    const int32_t end = min(g.row_ptr[u + 1], hc.y + 32);
    float ax = 0.0f, ay = 0.0f;
    for (int32_t e = hc.y; e < end; ++e) {
      const float2 f = __bfloat1622float2(h2[(int64_t)g.adj[e].x * (kHid / 2) + lane]);
      ax += f.x;
      ay += f.y;
    }
    atomicAdd(hub_sum + (int64_t)hc.x * kHid + 2 * lane, ax);
    atomicAdd(hub_sum + (int64_t)hc.x * kHid + 2 * lane + 1, ay);
  }
}



// ------------------------------------------------- tcgen05 layer GEMM --
// One message-passing layer as a tensor-core GEMM per 128-vertex tile:
// D[128 x 64] = A[128 x 128] * B^T, A = [h(v) | mean_{u in N(v)} h(u)]
// (bf16, both halves streamed by TMA with 128-byte swizzle), B = the
// layer's [Ws | Wn] (64 x 128 bf16, K-major, staged once per CTA), D in
// tensor memory (fp32, 128 lanes x 64 columns). One thread issues the TMA
// loads and the eight K=16 MMAs of a tile; after the MMA's commit arrives,
// each warp reads its 32 rows of D (tcgen05.ld 32x32b), adds the bias,
// applies the ReLU and stores bf16 activations, or on the last layer
// reduces them against wo into scores. Every wait is bounded: a wait that
// runs out sets *err (1: TMA, 2: MMA) and the CTA leaves after freeing its
// tensor memory.
constexpr int kTcThreads = 128;
constexpr int kTcRows = 128;                    // vertices per tile (MMA M)
constexpr uint32_t kTcTileBytes = 2u * kTcRows * 128u;  // A: two 128-byte K halves of 128 rows
constexpr int kTcStages = 2;                    // A tiles in flight per CTA
constexpr int kTcSmem = kTcStages * 32768 + 16384 + 64 + 512 + 1024;  // A stages, B, barriers, bias/wo, alignment
constexpr int kTcCtasPerSm = 2;
static_assert(kTcCtasPerSm * (kTcSmem + 1024) <= 228 * 1024, "two CTAs' shared memory (and reserve) per SM");
static_assert(kTcCtasPerSm * 64 <= 512, "tensor memory columns per SM");
constexpr uint32_t kTcWaitLimit = 1u << 20;     // polls of 64+ ns: > 60 ms, against microseconds per tile
constexpr uint32_t kTmemCols = 64;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// Waits for the phase with the given parity to complete; false after
// `limit` polls.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t limit) {
  const uint32_t a = smem_u32(bar);
  for (uint32_t i = 0; i < limit; ++i) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
    __nanosleep(64);
  }
  return false;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int32_t x, int32_t y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
      ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// Shared-memory matrix descriptor of a K-major operand with 128-byte
// swizzle: rows of 128 bytes, 8-row groups 1024 bytes apart (the stride
// byte offset), start address in 16-byte units, bits 46-48 = 0b001, the
// swizzle mode (2 = 128 bytes) in bits 61-63. The leading byte offset is
// unused for this layout (set to 1). Atoms start 1024-byte aligned, so the
// base offset is 0; a K step of 16 elements inside the 128-byte row moves
// the start address by 32 bytes.
__device__ __forceinline__ uint64_t sw128_kmajor_desc(uint32_t saddr) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

// Instruction descriptor of kind::f16: D fp32 (bits 4-5 = 1), A and B bf16
// (bits 7-9, 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 in bits
// 17-22, M >> 4 in bits 24-28.
constexpr uint32_t kTcIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(64 >> 3) << 17) |
                              ((uint32_t)(kTcRows >> 4) << 24);

__device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
      ::"r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(kTcIdesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void tc_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 16 consecutive fp32 columns of this thread's tensor-memory lane
__device__ __forceinline__ void tc_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, "
      "[%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}

__device__ __forceinline__ void tc_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__global__ void __launch_bounds__(kTcThreads) k_infer_layer_tc(const __grid_constant__ CUtensorMap map_h,
                                                               const __grid_constant__ CUtensorMap map_a, int32_t V,
                                                               const __nv_bfloat16* __restrict__ wcat,
                                                               const float* __restrict__ bias,
                                                               const float* __restrict__ wo,
                                                               const float* __restrict__ bo_ptr,
                                                               __nv_bfloat16* __restrict__ hout,
                                                               float* __restrict__ scores, int32_t* __restrict__ err,
                                                               uint32_t extra_tx) {
  extern __shared__ uint8_t tc_dsm[];
  const uint32_t raw = smem_u32(tc_dsm);
  uint8_t* sm = tc_dsm + (((raw + 1023u) & ~1023u) - raw);  // swizzle atoms are 1024-byte aligned
  uint8_t* sA = sm;                                          // [stage][K half][128 rows][128 B]
  uint8_t* sB = sm + kTcStages * 32768;                      // [K half][64 rows][128 B]
  uint8_t* misc = sB + 16384;
  uint64_t* full = reinterpret_cast<uint64_t*>(misc);        // [stage]: the stage's A tile landed
  uint64_t* mma_done = full + kTcStages;                     // the tile's MMAs completed
  uint32_t* tslot = reinterpret_cast<uint32_t*>(mma_done + 1);
  int32_t* sabort = reinterpret_cast<int32_t*>(tslot + 1);
  float* sbias = reinterpret_cast<float*>(misc + 64);
  float* swo = sbias + kHid;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // B: row o = output o, 16-byte chunk c of its 128 K values, stored in the
  // 128-byte-swizzled K-major layout (chunk c & 7 of K half c >> 3 at
  // position (c & 7) ^ (o & 7) of row o)
  for (int i = tid; i < kHid * 16; i += kTcThreads) {
    const int o = i >> 4, c = i & 15;
    const uint4 v = reinterpret_cast<const uint4*>(wcat + (int64_t)o * 2 * kHid)[c];
    *reinterpret_cast<uint4*>(sB + (c >> 3) * 8192 + o * 128 + (((c & 7) ^ (o & 7)) << 4)) = v;
  }
  if (tid < kHid) {
    sbias[tid] = bias[tid];
    swo[tid] = wo ? wo[tid] : 0.0f;
  }
  if (tid == 0) {
    for (int st = 0; st < kTcStages; ++st) mbar_init(&full[st], 1);
    mbar_init(mma_done, 1);
    *sabort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // B's stores, seen by the tensor cores
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  const float bo = bo_ptr ? *bo_ptr : 0.0f;
  const uint32_t sa = smem_u32(sA), sb = smem_u32(sB);
  const int64_t ntiles = ((int64_t)V + kTcRows - 1) / kTcRows;
  // stage s of A holds the CTA's tiles i = s, s + 2, ...: tile i + 1 loads
  // while tile i is multiplied and written out (its stage was freed when
  // tile i - 1's MMAs completed)
  // extra_tx (0 but in the bounded-wait test) raises the byte count the
  // CTA's first tile waits for above what its loads deliver
  auto load_tile = [&](int64_t t, int st) {
    mbar_expect_tx(&full[st], kTcTileBytes + (t == blockIdx.x ? extra_tx : 0u));
    tma_load_2d(sA + st * 32768, &map_h, 0, (int32_t)(t * kTcRows), &full[st]);
    tma_load_2d(sA + st * 32768 + 16384, &map_a, 0, (int32_t)(t * kTcRows), &full[st]);
  };
  static_assert(kTcStages == 2, "stage bits below");
  uint32_t pending = 0u;  // thread 0: bit st = a load of stage st issued and not yet seen complete
  uint32_t parity = 0u;   // bit st = phase parity of stage st's next completion
  if (tid == 0 && blockIdx.x < ntiles) {
    load_tile(blockIdx.x, 0);
    pending |= 1u;
  }
  int64_t i = 0;
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x, ++i) {
    const int st = (int)(i & 1);
    if (tid == 0) {
      const int64_t tn = t + gridDim.x;
      if (tn < ntiles) {
        load_tile(tn, st ^ 1);
        pending |= 1u << (st ^ 1);
      }
      if (mbar_wait(&full[st], (parity >> st) & 1u, kTcWaitLimit)) {
        pending &= ~(1u << st);
        parity ^= 1u << st;
        tc_fence_after();
        const uint32_t a0 = sa + (uint32_t)st * 32768u;
#pragma unroll
        for (int kk = 0; kk < 2 * kHid / 16; ++kk) {
          const uint32_t off = (uint32_t)(kk >> 2) * 16384u + (uint32_t)(kk & 3) * 32u;
          const uint32_t boff = (uint32_t)(kk >> 2) * 8192u + (uint32_t)(kk & 3) * 32u;
          tc_mma(tmem, sw128_kmajor_desc(a0 + off), sw128_kmajor_desc(sb + boff), kk > 0 ? 1u : 0u);
        }
        tc_commit(mma_done);
      } else {
        *sabort = 1;
        atomicExch(err, 1);
      }
    }
    __syncthreads();
    if (*sabort) break;
    if (!mbar_wait(mma_done, (uint32_t)(i & 1), kTcWaitLimit)) {
      *sabort = 1;
      atomicExch(err, 2);
    }
    __syncthreads();
    if (*sabort) break;
    tc_fence_after();
    uint32_t r[4][16];
    const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll
    for (int q = 0; q < 4; ++q) tc_ld16(taddr + 16 * q, r[q]);
    tc_wait_ld();
    const int64_t v = t * kTcRows + warp * 32 + lane;  // this thread's row of D
    if (v < V) {
      if (scores) {
        float sc = bo;
#pragma unroll
        for (int q = 0; q < 4; ++q)
#pragma unroll
          for (int j = 0; j < 16; ++j) sc += fmaxf(__uint_as_float(r[q][j]) + sbias[16 * q + j], 0.0f) * swo[16 * q + j];
        scores[v] = sc;
      } else {
        uint4* out = reinterpret_cast<uint4*>(hout + v * kHid);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          uint32_t pk[8];
#pragma unroll
          for (int j = 0; j < 8; ++j)
            pk[j] = pack_bf16x2(fmaxf(__uint_as_float(r[q][2 * j]) + sbias[16 * q + 2 * j], 0.0f),
                                fmaxf(__uint_as_float(r[q][2 * j + 1]) + sbias[16 * q + 2 * j + 1], 0.0f));
          out[2 * q] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
          out[2 * q + 1] = make_uint4(pk[4], pk[5], pk[6], pk[7]);
        }
      }
    }
    tc_fence_before();
    __syncthreads();  // D read before the next tile's MMAs overwrite it
  }
  if (tid == 0) {
    // after a wait ran out: loads still in flight land (bounded) before the
    // CTA leaves, and so do MMAs that were issued
    for (int st = 0; st < kTcStages; ++st)
      if ((pending >> st) & 1u) mbar_wait(&full[st], (parity >> st) & 1u, kTcWaitLimit);
    if (*sabort) mbar_wait(mma_done, (uint32_t)(i & 1), kTcWaitLimit);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
}

__global__ void k_feature_score(int32_t V, const float* __restrict__ x, float* __restrict__ s) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (int64_t)gridDim.x * blockDim.x) {
    const float* f = x + v * kFeat;
    s[v] = 1000.0f * f[3] + 100.0f * f[4] + 10.0f * f[5] + f[1];
  }
}

__device__ __forceinline__ uint32_t order_key(float f) {
  const uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__global__ void k_score_hist(int32_t V, const float* __restrict__ s, uint32_t* __restrict__ hist) {
  __shared__ uint32_t h[kScoreBins];
  for (int i = threadIdx.x; i < kScoreBins; i += blockDim.x) h[i] = 0u;
  __syncthreads();
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (int64_t)gridDim.x * blockDim.x) {
    const float f = s[v];
    if (f == f) atomicAdd(&h[order_key(f) >> 20], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < kScoreBins; i += blockDim.x)
    if (h[i]) atomicAdd(hist + i, h[i]);
}

__global__ void k_score_select(int32_t V, const float* __restrict__ s, uint32_t bin_lo, uint2* __restrict__ out,
                               int32_t* count, int32_t cap) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (int64_t)gridDim.x * blockDim.x) {
    const float f = s[v];
    if (f != f) continue;
    const uint32_t key = order_key(f);
    if ((key >> 20) < bin_lo) continue;
    const int32_t i = atomicAdd(count, 1);
    if (i < cap) out[i] = make_uint2(key, (uint32_t)v);
  }
}

__global__ void k_argmax(int32_t V, const float* __restrict__ s, unsigned long long* best) {
  unsigned long long b = 0ull;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (int64_t)gridDim.x * blockDim.x) {
    const float f = s[v];
    if (f != f) continue;  // NaN never wins
    const unsigned long long key = ((unsigned long long)order_key(f) << 32) | (0xffffffffull - (uint64_t)v);
    b = key > b ? key : b;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long x = __shfl_xor_sync(0xffffffffu, b, o);
    b = x > b ? x : b;
  }
  if ((threadIdx.x & 31) == 0 && b) atomicMax(best, b);
}

// -------------------------------------------------------------- training --
// block: 4 vertices x 64 outputs; W rows padded by one float
__global__ void __launch_bounds__(256) k_dense_fwd(int32_t V, const float* __restrict__ x1, int k1,
                                                   const float* __restrict__ w1, const float* __restrict__ x2,
                                                   const float* __restrict__ w2, const float* __restrict__ b,
                                                   float* __restrict__ y) {
  __shared__ float sw1[kHid][kHid + 1], sw2[kHid][kHid + 1];
  __shared__ float sx1[4][kHid], sx2[4][kHid];
  for (int i = threadIdx.x; i < kHid * k1; i += blockDim.x) sw1[i / k1][i % k1] = w1[i];
  if (x2)
    for (int i = threadIdx.x; i < kHid * kHid; i += blockDim.x) sw2[i / kHid][i % kHid] = w2[i];
  const int o = threadIdx.x & (kHid - 1), vi = threadIdx.x >> 6;
  const float bo = b[o];
  for (int64_t vb = (int64_t)blockIdx.x * 4; vb < V; vb += (int64_t)gridDim.x * 4) {
    __syncthreads();
    const int64_t v = vb + vi;
    if (o < k1) sx1[vi][o] = v < V ? x1[v * k1 + o] : 0.0f;
    if (x2) sx2[vi][o] = v < V ? x2[v * kHid + o] : 0.0f;
    __syncthreads();
    if (v >= V) continue;
    float acc = bo;
    for (int c = 0; c < k1; ++c) acc = fmaf(sw1[o][c], sx1[vi][c], acc);
    if (x2)
      for (int c = 0; c < kHid; ++c) acc = fmaf(sw2[o][c], sx2[vi][c], acc);
    y[v * kHid + o] = fmaxf(acc, 0.0f);
  }
}

__global__ void __launch_bounds__(256) k_dense_bwd_data(int32_t V, const float* __restrict__ dz,
                                                        const float* __restrict__ w, float* __restrict__ y) {
  __shared__ float sw[kHid][kHid];
  __shared__ float sdz[4][kHid];
  for (int i = threadIdx.x; i < kHid * kHid; i += blockDim.x) sw[i / kHid][i % kHid] = w[i];
  const int c = threadIdx.x & (kHid - 1), vi = threadIdx.x >> 6;
  for (int64_t vb = (int64_t)blockIdx.x * 4; vb < V; vb += (int64_t)gridDim.x * 4) {
    __syncthreads();
    const int64_t v = vb + vi;
    sdz[vi][c] = v < V ? dz[v * kHid + c] : 0.0f;
    __syncthreads();
    if (v >= V) continue;
    float acc = 0.0f;
    for (int o = 0; o < kHid; ++o) acc = fmaf(sdz[vi][o], sw[o][c], acc);
    y[v * kHid + c] = acc;
  }
}

// thread t owns output row o = t / 4 and columns c = t % 4 + 4 j
__global__ void __launch_bounds__(256) k_dense_bwd_weight(int32_t V, const float* __restrict__ dz,
                                                          const float* __restrict__ x, int k, float* __restrict__ dw,
                                                          float* __restrict__ db) {
  constexpr int kChunk = 32;
  __shared__ float sdz[kChunk][kHid + 1];
  __shared__ float sx[kChunk][kHid + 1];
  const int o = threadIdx.x >> 2, cl = threadIdx.x & 3;
  const int nc = k / 4;  // columns per thread (k is a multiple of 4, at most kHid)
  float acc[kHid / 4];
#pragma unroll
  for (int j = 0; j < kHid / 4; ++j) acc[j] = 0.0f;
  float accb = 0.0f;
  for (int64_t vb = (int64_t)blockIdx.x * kChunk; vb < V; vb += (int64_t)gridDim.x * kChunk) {
    __syncthreads();
    for (int i = threadIdx.x; i < kChunk * kHid; i += blockDim.x) {
      const int r = i / kHid, c = i % kHid;
      const int64_t v = vb + r;
      sdz[r][c] = v < V ? dz[v * kHid + c] : 0.0f;
      if (c < k) sx[r][c] = v < V ? x[v * k + c] : 0.0f;
    }
    __syncthreads();
    for (int r = 0; r < kChunk; ++r) {
      const float d = sdz[r][o];
      accb += d;
#pragma unroll
      for (int j = 0; j < kHid / 4; ++j)
        if (j < nc) acc[j] = fmaf(d, sx[r][cl + 4 * j], acc[j]);
    }
  }
#pragma unroll
  for (int j = 0; j < kHid / 4; ++j)
    if (j < nc) atomicAdd(dw + o * k + cl + 4 * j, acc[j]);
  if (db && cl == 0) atomicAdd(db + o, accb);
}

__global__ void k_mean_agg(GraphDev g, const float* __restrict__ x, float* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const float2* x2 = reinterpret_cast<const float2*>(x);
  for (int64_t v = gwarp(); v < g.V; v += nwarps()) {
    const int32_t beg = g.row_ptr[v], end = g.row_ptr[v + 1];
    float ax = 0.0f, ay = 0.0f;
    for (int32_t e = beg; e < end; ++e) {
      const float2 f = x2[(int64_t)g.adj[e].x * (kHid / 2) + lane];
      ax += f.x;
      ay += f.y;
    }
    const float inv = end > beg ? 1.0f / (float)(end - beg) : 0.0f;
    reinterpret_cast<float2*>(out)[v * (kHid / 2) + lane] = make_float2(ax * inv, ay * inv);
  }
}

__global__ void k_agg_bwd(GraphDev g, const float* __restrict__ t, const float* __restrict__ add,
                          const float* __restrict__ h, float* __restrict__ dz_prev) {
  const int lane = threadIdx.x & 31;
  const float2* t2 = reinterpret_cast<const float2*>(t);
  for (int64_t u = gwarp(); u < g.V; u += nwarps()) {
    const int32_t beg = g.row_ptr[u], end = g.row_ptr[u + 1];
    float2 a = reinterpret_cast<const float2*>(add)[u * (kHid / 2) + lane];
    for (int32_t e = beg; e < end; ++e) {
      const int32_t v = g.adj[e].x;
      const int32_t dv = g.row_ptr[v + 1] - g.row_ptr[v];  // >= 1: v lists u
      const float inv = 1.0f / (float)dv;
      const float2 f = t2[(int64_t)v * (kHid / 2) + lane];
      a.x = fmaf(f.x, inv, a.x);
      a.y = fmaf(f.y, inv, a.y);
    }
    const float2 hh = reinterpret_cast<const float2*>(h)[u * (kHid / 2) + lane];
    reinterpret_cast<float2*>(dz_prev)[u * (kHid / 2) + lane] =
        make_float2(hh.x > 0.0f ? a.x : 0.0f, hh.y > 0.0f ? a.y : 0.0f);
  }
}

__global__ void k_score(int32_t V, const float* __restrict__ h, const float* __restrict__ p, float* __restrict__ s) {
  const int lane = threadIdx.x & 31;
  const float2 wo = reinterpret_cast<const float2*>(p + kOffWo)[lane];
  const float bo = p[kOffBo];
  for (int64_t v = gwarp(); v < V; v += nwarps()) {
    const float2 f = reinterpret_cast<const float2*>(h)[v * (kHid / 2) + lane];
    float acc = f.x * wo.x + f.y * wo.y;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) s[v] = acc + bo;
  }
}

__device__ __forceinline__ int32_t float_ord(float f) {
  const int32_t i = __float_as_int(f);
  return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float ord_float(int32_t i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }

__global__ void k_loss_init(float* red) {
  reinterpret_cast<int32_t*>(red)[0] = float_ord(-3.0e38f);
  red[1] = 0.0f;
}

__global__ void k_loss_max(int32_t V, const float* __restrict__ s, float* red) {
  float m = -3.0e38f;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (int64_t)gridDim.x * blockDim.x)
    m = fmaxf(m, s[v]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(reinterpret_cast<int32_t*>(red), float_ord(m));
}

__global__ void k_loss_sum(int32_t V, const float* __restrict__ s, float* red) {
  const float m = ord_float(reinterpret_cast<const int32_t*>(red)[0]);
  float acc = 0.0f;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (int64_t)gridDim.x * blockDim.x)
    acc += expf(s[v] - m);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(red + 1, acc);
}

__global__ void k_loss_grad(int32_t V, const float* __restrict__ s, const uint8_t* __restrict__ label, int32_t n,
                            const float* red, float* __restrict__ ds, float* loss) {
  const float m = ord_float(reinterpret_cast<const int32_t*>(red)[0]);
  const float sum = red[1];
  const float lse = m + logf(sum);
  const float inv_n = 1.0f / (float)n;
  float acc = 0.0f;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (int64_t)gridDim.x * blockDim.x) {
    const float p = expf(s[v] - m) / sum;
    const bool y = label[v] != 0;
    ds[v] = p - (y ? inv_n : 0.0f);
    if (y) acc -= (s[v] - lse) * inv_n;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0 && acc != 0.0f) atomicAdd(loss, acc);
}

// block: 4 vertex lanes x 64 channels
__global__ void __launch_bounds__(256) k_out_bwd(int32_t V, const float* __restrict__ ds, const float* __restrict__ h,
                                                 const float* __restrict__ p, float* __restrict__ grad,
                                                 float* __restrict__ dz) {
  __shared__ float red[4][kHid];
  __shared__ float redb[4];
  const int c = threadIdx.x & (kHid - 1), vi = threadIdx.x >> 6;
  const float wo = p[kOffWo + c];
  float acc = 0.0f, accb = 0.0f;
  for (int64_t v = (int64_t)blockIdx.x * 4 + vi; v < V; v += (int64_t)gridDim.x * 4) {
    const float d = ds[v];
    const float hv = h[v * kHid + c];
    acc = fmaf(d, hv, acc);
    if (c == 0) accb += d;
    dz[v * kHid + c] = hv > 0.0f ? d * wo : 0.0f;
  }
  red[vi][c] = acc;
  if (c == 0) redb[vi] = accb;
  __syncthreads();
  if (vi == 0) {
    atomicAdd(grad + kOffWo + c, red[0][c] + red[1][c] + red[2][c] + red[3][c]);
    if (c == 0) atomicAdd(grad + kOffBo, redb[0] + redb[1] + redb[2] + redb[3]);
  }
}

__global__ void k_adam(int64_t n, float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, float lr, float c1, float c2) {
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

__global__ void k_set_labels(const int32_t* __restrict__ ids, int32_t n, uint8_t* __restrict__ label) {
  for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) label[ids[i]] = 1;
}

__global__ void __launch_bounds__(256) k_ub_paths(GraphDev g, const int32_t* __restrict__ dist,
                                                  const int32_t* __restrict__ par, int32_t stride,
                                                  const int32_t* __restrict__ group_ptr,
                                                  const int32_t* __restrict__ members, const int32_t* __restrict__ perm,
                                                  int3* __restrict__ out_e, int32_t* out_n, int32_t cap) {
  __shared__ unsigned long long best;
  if (threadIdx.x == 0) best = ~0ull;
  __syncthreads();
  const int gi = blockIdx.x;
  unsigned long long b = ~0ull;
  for (int32_t i = group_ptr[gi] + threadIdx.x; i < group_ptr[gi + 1]; i += blockDim.x) {
    const int32_t v = perm[members[i]];
    const int32_t d = dist[(int64_t)v * stride];
    if (d < kInf) {
      const unsigned long long key = ((unsigned long long)(uint32_t)d << 32) | (uint32_t)v;
      b = key < b ? key : b;
    }
  }
  atomicMin(&best, b);
  __syncthreads();
  if (threadIdx.x != 0) return;
  if (best == ~0ull) {
    atomicExch(out_n + 2, 1);
    return;
  }
  int32_t v = (int32_t)(best & 0xffffffffull);
  for (int32_t step = 0; step <= g.V; ++step) {
    const int32_t e = par[(int64_t)v * stride];
    if (e == kLeaf) return;  // the root
    if (e < g.row_ptr[v] || e >= g.row_ptr[v + 1]) break;  // not a growth record: stop
    const int2 x = g.adj[e];
    const int32_t i = atomicAdd(out_n, 1);
    if (i >= cap) break;
    out_e[i] = make_int3(v, x.x, x.y);
    v = x.x;
  }
  atomicExch(out_n + 1, 1);
}

// The proposal's paths over a solve's own wave 1, whose entry (v, {g}) is
// the distance from v to group g with its growth record: one thread per
// group walks from (root, {g}) along the records to a leaf, emitting
// (v, next, w) edges. Every step must be a growth record of its row whose
// cost is the next state's plus the edge weight, and the leaf a member of
// g; anything else stops the walk (out_n[1]), so whatever the table's
// state, the emitted paths are real paths of the graph.
__global__ void k_root_paths(GraphDev g, const int32_t* __restrict__ cost, const int32_t* __restrict__ par,
                             int32_t stride1, const uint32_t* __restrict__ gmask, int32_t root, int32_t k,
                             int3* __restrict__ out_e, int32_t* out_n, int32_t cap) {
  const int gi = blockIdx.x * blockDim.x + threadIdx.x;
  if (gi >= k) return;
  int32_t v = root;
  int32_t c = cost[(int64_t)v * stride1 + gi];
  if (c >= kInf) {
    atomicExch(out_n + 2, 1);
    return;
  }
  for (int32_t step = 0; step <= g.V; ++step) {
    const int32_t e = par[(int64_t)v * stride1 + gi];
    if (e == kLeaf) {
      if (c == 0 && ((gmask[v] >> gi) & 1u)) return;
      break;
    }
    if (e < g.row_ptr[v] || e >= g.row_ptr[v + 1]) break;
    const int2 x = g.adj[e];
    const int32_t cn = cost[(int64_t)x.x * stride1 + gi];
    if (cn != c - x.y || cn < 0) break;
    const int32_t i = atomicAdd(out_n, 1);
    if (i >= cap) break;
    out_e[i] = make_int3(v, x.x, x.y);
    v = x.x;
    c = cn;
  }
  atomicExch(out_n + 1, 1);
}

}  // namespace

// -------------------------------------------------------------- launchers --
cudaError_t launch_reach(const GraphDev& g, const int32_t* hub_of, const uint32_t* in, uint32_t* out,
                         int32_t* member_nbrs, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(out, 0, (size_t)g.V * sizeof(uint32_t), s);
  if (e == cudaSuccess && member_nbrs) e = cudaMemsetAsync(member_nbrs, 0, (size_t)g.V * sizeof(int32_t), s);
  if (e != cudaSuccess) return e;
  k_reach<<<grid_for(g.V, 256), 256, 0, s>>>(g, hub_of, in, out, member_nbrs);
  return cudaGetLastError();
}

cudaError_t launch_features(const GraphDev& g, const uint32_t* m0, const uint32_t* r1, const uint32_t* r2,
                            const uint32_t* r3, const int32_t* member_nbrs, int32_t k, float* x, cudaStream_t s) {
  k_features<<<grid_for(g.V, 256), 256, 0, s>>>(g, m0, r1, r2, r3, member_nbrs, k, x);
  return cudaGetLastError();
}

cudaError_t launch_pack_bf16(const float* params, __nv_bfloat16* wcat, cudaStream_t s) {
  k_pack_bf16<<<96, 256, 0, s>>>(params, wcat);
  return cudaGetLastError();
}

cudaError_t launch_infer_l0(int32_t V, const float* x, const float* params, __nv_bfloat16* h0, cudaStream_t s) {
  k_infer_l0<<<grid_for(V, 256), 256, 0, s>>>(V, x, params, h0);
  return cudaGetLastError();
}

cudaError_t launch_hub_sum_bf16(const GraphDev& g, const __nv_bfloat16* hin, float* hub_sum, cudaStream_t s) {
  if (g.nchunks == 0) return cudaSuccess;
  k_hub_sum_bf16<<<grid_for(g.nchunks * 32, 256), 256, 0, s>>>(g, hin, hub_sum);
  return cudaGetLastError();
}

cudaError_t make_act_map(const __nv_bfloat16* buf, int32_t V, CUtensorMap* out) {
  using EncodeFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
  static EncodeFn encode = [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      fn = nullptr;
    return reinterpret_cast<EncodeFn>(fn);
  }();
  if (!encode) return cudaErrorNotSupported;
  const cuuint64_t dims[2] = {(cuuint64_t)kHid, (cuuint64_t)(V > 0 ? V : 1)};
  const cuuint64_t strides[1] = {(cuuint64_t)kHid * sizeof(__nv_bfloat16)};  // 128-byte rows
  const cuuint32_t box[2] = {(cuuint32_t)kHid, (cuuint32_t)kTcRows};       // 128 bytes x 128 rows
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = encode(out, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<__nv_bfloat16*>(buf), dims, strides,
                            box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

cudaError_t launch_infer_layer(const GraphDev& g, const int32_t* hub_of, const float* hub_sum,
                               const __nv_bfloat16* hin, const CUtensorMap& hin_map, __nv_bfloat16* agg,
                               const CUtensorMap& agg_map, const __nv_bfloat16* wcat_l, const float* params, int l,
                               __nv_bfloat16* hout, float* scores, int32_t* err, cudaStream_t s) {
  k_mean_bf16<<<grid_for((int64_t)g.V * 8, 256, 152 * 32), 256, 0, s>>>(g, hub_of, hub_sum, hin, agg);
  const cudaError_t me = cudaGetLastError();
  if (me != cudaSuccess) return me;
  return launch_layer_gemm(g.V, hin_map, agg_map, wcat_l, params, l, hout, scores, err, 0u, s);
}

cudaError_t launch_layer_gemm(int32_t V, const CUtensorMap& hin_map, const CUtensorMap& agg_map,
                              const __nv_bfloat16* wcat_l, const float* params, int l, __nv_bfloat16* hout,
                              float* scores, int32_t* err, uint32_t extra_tx, cudaStream_t s) {
  const float* bias = params + layer_off(l) + 2 * kHid * kHid;
  const float* wo = scores ? params + kOffWo : nullptr;
  const float* bo = scores ? params + kOffBo : nullptr;
  // kTcCtasPerSm CTAs per SM (shared memory allows two; their tensor memory,
  // 2 x 64 columns, is a quarter of an SM's), each with two tiles in flight
  static const int ctas = [] {
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaFuncSetAttribute(k_infer_layer_tc, cudaFuncAttributePreferredSharedMemoryCarveout,
                         (int)cudaSharedmemCarveoutMaxShared);
    return sms * kTcCtasPerSm;
  }();
  const cudaError_t ae = cudaFuncSetAttribute(k_infer_layer_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem);
  if (ae != cudaSuccess) return ae;
  const int64_t tiles = ((int64_t)V + kTcRows - 1) / kTcRows;
  const int grid = (int)std::min<int64_t>(tiles, ctas);
  k_infer_layer_tc<<<grid, kTcThreads, kTcSmem, s>>>(hin_map, agg_map, V, wcat_l, bias, wo, bo, hout, scores, err,
                                                     extra_tx);
  return cudaGetLastError();
}

cudaError_t launch_feature_score(int32_t V, const float* x, float* s, cudaStream_t st) {
  k_feature_score<<<grid_for(V, 256), 256, 0, st>>>(V, x, s);
  return cudaGetLastError();
}

cudaError_t launch_score_hist(int32_t V, const float* scores, uint32_t* hist, cudaStream_t s) {
  k_score_hist<<<grid_for(V, 256, 152 * 2), 256, 0, s>>>(V, scores, hist);
  return cudaGetLastError();
}

cudaError_t launch_score_select(int32_t V, const float* scores, uint32_t bin_lo, uint2* out, int32_t* count,
                                int32_t cap, cudaStream_t s) {
  k_score_select<<<grid_for(V, 256, 152 * 4), 256, 0, s>>>(V, scores, bin_lo, out, count, cap);
  return cudaGetLastError();
}

cudaError_t launch_argmax(int32_t V, const float* scores, unsigned long long* best, cudaStream_t s) {
  k_argmax<<<grid_for(V, 256, 152 * 4), 256, 0, s>>>(V, scores, best);
  return cudaGetLastError();
}

cudaError_t launch_dense_fwd(int32_t V, const float* x1, int k1, const float* w1, const float* x2, const float* w2,
                             const float* b, float* y, cudaStream_t s) {
  k_dense_fwd<<<grid_for(V, 4, 152 * 8), 256, 0, s>>>(V, x1, k1, w1, x2, w2, b, y);
  return cudaGetLastError();
}

cudaError_t launch_dense_bwd_data(int32_t V, const float* dz, const float* w, float* y, cudaStream_t s) {
  k_dense_bwd_data<<<grid_for(V, 4, 152 * 8), 256, 0, s>>>(V, dz, w, y);
  return cudaGetLastError();
}

cudaError_t launch_dense_bwd_weight(int32_t V, const float* dz, const float* x, int k, float* dw, float* db,
                                    cudaStream_t s) {
  k_dense_bwd_weight<<<grid_for(V, 32, 152 * 2), 256, 0, s>>>(V, dz, x, k, dw, db);
  return cudaGetLastError();
}

cudaError_t launch_mean_agg(const GraphDev& g, const float* x, float* out, cudaStream_t s) {
  k_mean_agg<<<grid_for((int64_t)g.V * 32, 256), 256, 0, s>>>(g, x, out);
  return cudaGetLastError();
}

cudaError_t launch_agg_bwd(const GraphDev& g, const float* t, const float* add, const float* h, float* dz_prev,
                           cudaStream_t s) {
  k_agg_bwd<<<grid_for((int64_t)g.V * 32, 256), 256, 0, s>>>(g, t, add, h, dz_prev);
  return cudaGetLastError();
}

cudaError_t launch_score(int32_t V, const float* h, const float* params, float* s, cudaStream_t st) {
  k_score<<<grid_for((int64_t)V * 32, 256), 256, 0, st>>>(V, h, params, s);
  return cudaGetLastError();
}

cudaError_t launch_softmax_loss(int32_t V, const float* s, const uint8_t* label, int32_t n, float* ds, float* loss,
                                float* red, cudaStream_t st) {
  const int gb = grid_for(V, 256, 152 * 4);
  k_loss_init<<<1, 1, 0, st>>>(red);
  k_loss_max<<<gb, 256, 0, st>>>(V, s, red);
  k_loss_sum<<<gb, 256, 0, st>>>(V, s, red);
  k_loss_grad<<<gb, 256, 0, st>>>(V, s, label, n, red, ds, loss);
  return cudaGetLastError();
}

cudaError_t launch_out_bwd(int32_t V, const float* ds, const float* h, const float* params, float* grad, float* dz,
                           cudaStream_t s) {
  k_out_bwd<<<grid_for(V, 4, 152 * 8), 256, 0, s>>>(V, ds, h, params, grad, dz);
  return cudaGetLastError();
}

cudaError_t launch_set_labels(const int32_t* ids, int32_t n, uint8_t* label, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_set_labels<<<grid_for(n, 256, 64), 256, 0, s>>>(ids, n, label);
  return cudaGetLastError();
}

cudaError_t launch_ub_paths(const GraphDev& g, const int32_t* dist, const int32_t* par, int32_t stride,
                            const int32_t* group_ptr, const int32_t* members, const int32_t* perm, int32_t k,
                            int3* out_e, int32_t* out_n, int32_t cap, cudaStream_t s) {
  k_ub_paths<<<k, 256, 0, s>>>(g, dist, par, stride, group_ptr, members, perm, out_e, out_n, cap);
  return cudaGetLastError();
}

cudaError_t launch_root_paths(const GraphDev& g, const int32_t* cost, const int32_t* par, int32_t stride1,
                              const uint32_t* gmask, int32_t root, int32_t k, int3* out_e, int32_t* out_n, int32_t cap,
                              cudaStream_t s) {
  k_root_paths<<<1, 32, 0, s>>>(g, cost, par, stride1, gmask, root, k, out_e, out_n, cap);
  return cudaGetLastError();
}

cudaError_t launch_adam(int64_t n, float* p, const float* g, float* m, float* v, float lr, int32_t t, cudaStream_t s) {
  double c1 = 1.0, c2 = 1.0;
  for (int32_t i = 0; i < t; ++i) {
    c1 *= 0.9;
    c2 *= 0.999;
  }
  k_adam<<<grid_for(n, 256, 256), 256, 0, s>>>(n, p, g, m, v, lr, (float)(1.0 - c1), (float)(1.0 - c2));
  return cudaGetLastError();
}

}  // namespace gst
