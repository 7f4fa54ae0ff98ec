// gst_group_distances_noalloc: shortest-path distance of every vertex to a
// vertex set (one group), for callers that cannot allocate device memory.
//
// Who cannot allocate: code that runs inside a host application or serving
// stack that owns all device memory through its own pool and forbids
// cudaMalloc/cudaFree (they would bypass its accounting and limits), code
// on latency-critical paths where cudaMalloc's implicit device
// synchronisation is not acceptable, and plugins loaded after such a
// process has fixed its memory budget. They hand in device buffers for the
// graph, the sources and the outputs; this entry point allocates nothing.
//
// It is the growth kernel of the DP (pull-form label-correcting rounds, one
// group set at a time) with its frontier flags and round counters kept in
// the file-scope array below instead of in a per-graph workspace.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "gst.h"

namespace {

constexpr int32_t kNaInf = GST_COST_LIMIT;
constexpr int32_t kNaMaxV = GST_NOALLOC_MAX_VERTICES;
constexpr size_t kNaCtlBytes = 256;  // control words, then three flag arrays
constexpr size_t kNaScratchBytes = kNaCtlBytes + 3 * (size_t)kNaMaxV;
constexpr int kNaThreads = 256;
constexpr int kNaPollEvery = 8;
constexpr int kNaMaxDevices = 64;

// The scratch: 3 MiB + 256 B on every device that loads the library, held
// until the process exits. Every call shares it and it keeps the last
// call's contents, so each call clears what it needs first; calls whose
// work overlaps on one GPU (different streams, or host threads racing)
// corrupt each other's frontier.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaScratchBytes];

struct NaCtl {
  int32_t changed[3];  // rotating per-round change counts
  int32_t overflow;    // a distance reached GST_COST_LIMIT
  int32_t bad_input;   // a source or an edge entry out of range
};

// In host code g_noalloc_scratch names a host-side stand-in, not device
// memory: the device address comes from cudaGetSymbolAddress, once per
// device, with that device current.
std::mutex g_na_mu;
unsigned char* g_na_ptr[kNaMaxDevices] = {};

gst_status scratch_of_current_device(unsigned char** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNaMaxDevices) return GST_CUDA_ERROR;
  std::lock_guard<std::mutex> lock(g_na_mu);
  if (!g_na_ptr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return GST_CUDA_ERROR;
    g_na_ptr[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_na_ptr[dev];
  return GST_OK;
}

__global__ void k_na_init(int32_t V, int32_t* __restrict__ dist, int32_t* __restrict__ pred,
                          unsigned char* __restrict__ scratch) {
  NaCtl* ctl = reinterpret_cast<NaCtl*>(scratch);
  unsigned char* flags = scratch + kNaCtlBytes;
  const int32_t stride = gridDim.x * blockDim.x;
  for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < V; i += stride) {
    dist[i] = kNaInf;
    pred[i] = -1;
    flags[i] = 0;
    flags[kNaMaxV + i] = 0;
    flags[2 * kNaMaxV + i] = 0;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    ctl->changed[0] = ctl->changed[1] = ctl->changed[2] = 0;
    ctl->overflow = 0;
    ctl->bad_input = 0;
  }
}

// Sources start at distance 0 and form the first frontier (flag array 2,
// count slot 2: "round -1").
__global__ void k_na_seed(const int32_t* __restrict__ sources, int32_t n, int32_t V, int32_t* __restrict__ dist,
                          unsigned char* __restrict__ scratch) {
  NaCtl* ctl = reinterpret_cast<NaCtl*>(scratch);
  unsigned char* f2 = scratch + kNaCtlBytes + 2 * (size_t)kNaMaxV;
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int32_t s = sources[i];
  if (s < 0 || s >= V) {
    atomicExch(&ctl->bad_input, 1);
    return;
  }
  dist[s] = 0;
  f2[s] = 1;
  atomicAdd(&ctl->changed[2], 1);
}

// One pull round: u takes min over neighbours v that changed in the
// previous round of dist[v] + w(u,v); only u's thread writes u's entries.
__global__ void __launch_bounds__(kNaThreads)
    k_na_round(const int32_t* __restrict__ row_ptr, const int32_t* __restrict__ col, const int32_t* __restrict__ w,
               int32_t V, int64_t nnz, int32_t* __restrict__ dist, int32_t* __restrict__ pred,
               unsigned char* __restrict__ scratch, int32_t r) {
  NaCtl* ctl = reinterpret_cast<NaCtl*>(scratch);
  unsigned char* flags = scratch + kNaCtlBytes;
  const unsigned char* cur = flags + (size_t)((r + 2) % 3) * kNaMaxV;
  unsigned char* next = flags + (size_t)(r % 3) * kNaMaxV;
  unsigned char* clear = flags + (size_t)((r + 1) % 3) * kNaMaxV;
  if (ctl->changed[(r + 2) % 3] == 0) {  // converged: keep the rotation at zero
    if (blockIdx.x == 0 && threadIdx.x == 0) ctl->changed[(r + 1) % 3] = 0;
    return;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) ctl->changed[(r + 1) % 3] = 0;
  int changed = 0, overflow = 0, bad = 0;
  const int32_t stride = gridDim.x * blockDim.x;
  for (int32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < V; u += stride) {
    clear[u] = 0;
    const int32_t own = dist[u];
    int32_t best = own, code = -1;
    const int32_t beg = row_ptr[u], end = row_ptr[u + 1];
    if (beg < 0 || end < beg || (int64_t)end > nnz) {
      bad = 1;
      continue;
    }
    for (int32_t e = beg; e < end; ++e) {
      const int32_t v = col[e];
      if (v < 0 || v >= V) {
        bad = 1;
        continue;
      }
      if (!cur[v]) continue;
      int32_t c = dist[v];
      const int32_t we = w[e];
      if (c >= kNaInf) continue;
      if (we < 0 || we >= kNaInf) {
        bad = 1;
        continue;
      }
      c += we;  // both < 2^30: no wrap
      if (c >= kNaInf) {
        overflow = 1;
        continue;
      }
      if (c < best) {
        best = c;
        code = e;
      }
    }
    if (best < own) {
      dist[u] = best;
      pred[u] = code;
      next[u] = 1;
      ++changed;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) changed += __shfl_xor_sync(0xffffffffu, changed, o);
  if ((threadIdx.x & 31) == 0 && changed) atomicAdd(&ctl->changed[r % 3], changed);
  if (overflow) atomicExch(&ctl->overflow, 1);
  if (bad) atomicExch(&ctl->bad_input, 1);
}

}  // namespace

extern "C" gst_status gst_group_distances_noalloc(const int32_t* row_ptr, const int32_t* col, const int32_t* w,
                                                  int32_t V, int64_t nnz, const int32_t* sources,
                                                  int32_t num_sources, int32_t* dist, int32_t* pred, void* stream) {
  if (V > kNaMaxV) return GST_TOO_LARGE;
  if (V < 1 || nnz < 0 || nnz >= INT32_MAX || num_sources < 0 || !row_ptr || !dist || !pred ||
      (nnz > 0 && (!col || !w)) || (num_sources > 0 && !sources))
    return GST_BAD_INPUT;
  // an error still pending from the caller's earlier work is theirs: leave
  // it pending and run nothing, rather than report it as this call's own
  if (cudaPeekAtLastError() != cudaSuccess) return GST_CUDA_ERROR;
  unsigned char* scratch = nullptr;
  gst_status st = scratch_of_current_device(&scratch);
  if (st != GST_OK) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int blocks = (V + kNaThreads - 1) / kNaThreads;
  if (blocks > 4096) blocks = 4096;
  k_na_init<<<blocks, kNaThreads, 0, s>>>(V, dist, pred, scratch);
  if (num_sources > 0)
    k_na_seed<<<(num_sources + kNaThreads - 1) / kNaThreads, kNaThreads, 0, s>>>(sources, num_sources, V, dist,
                                                                                  scratch);
  if (cudaGetLastError() != cudaSuccess) return GST_CUDA_ERROR;
  NaCtl host_ctl;  // on the stack: the polls copy into it
  const int64_t max_rounds = (int64_t)V + 1;
  int64_t r = 0;
  for (;;) {
    for (int i = 0; i < kNaPollEvery; ++i, ++r)
      k_na_round<<<blocks, kNaThreads, 0, s>>>(row_ptr, col, w, V, nnz, dist, pred, scratch, (int32_t)(r % 3));
    if (cudaGetLastError() != cudaSuccess) return GST_CUDA_ERROR;  // a round failed to launch
    if (cudaMemcpyAsync(&host_ctl, scratch, sizeof(NaCtl), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return GST_CUDA_ERROR;
    if (host_ctl.bad_input) return GST_BAD_INPUT;
    if (host_ctl.overflow) return GST_OVERFLOW;
    if (host_ctl.changed[(r - 1) % 3] == 0) break;
    if (r >= max_rounds) return GST_TIMEOUT;
  }
  return GST_OK;
}
