// core.cu -- core numbers on the GPU by level-synchronous peeling.
//
// The reference computes core numbers once at start-up with a serial
// bucket-list peeling on the host (src/Graph.h:82-109); for million-vertex
// graphs that and the loader dominate start-up.  Here level k removes, in
// any order, every remaining vertex whose remaining degree is at most k:
//
//   scan   -- every vertex not yet removed with deg <= k is removed at level
//             k (core = k) and enters the frontier;
//   peel   -- one warp per frontier vertex decrements the remaining degree of
//             its not-yet-removed neighbours; the neighbour whose degree goes
//             from k+1 to k is removed at level k too and enters the next
//             frontier.  A decrement that finds deg <= k (a neighbour already
//             claimed at this level) is undone, so degrees never fall below k.
//
// until the frontier is empty, then k+1.  Any removal order within a level
// gives the same (unique) core numbers, so the result equals the serial
// peeling exactly.  The host loop reads one 16-byte counter block per
// iteration.
#include <algorithm>
#include <cstdint>

#include "../../include/scs.h"
#include "scs_device.cuh"

namespace scs {

namespace {

constexpr uint32_t UNSET = 0xFFFFFFFFu;
constexpr int CORE_THREADS = 256;

struct CoreCounters {
  uint32_t frontier;   // vertices appended to the output frontier
  uint32_t remaining;  // scan: vertices left after this level's scan
  uint32_t pad[2];
};

__device__ __forceinline__ void append(bool want, uint32_t v, uint32_t *cnt, uint32_t *dst) {
  const int lane = threadIdx.x & 31;
  const unsigned m = __ballot_sync(0xffffffffu, want);
  if (!m) return;
  uint32_t base = 0;
  if (lane == __ffs(m) - 1) base = atomicAdd(cnt, (uint32_t)__popc(m));
  base = __shfl_sync(0xffffffffu, base, __ffs(m) - 1);
  if (want) dst[base + __popc(m & ((1u << lane) - 1u))] = v;
}

__global__ void __launch_bounds__(CORE_THREADS)
core_init_kernel(const uint32_t *off, uint32_t n, uint32_t *deg, uint32_t *core) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    deg[v] = off[v + 1] - off[v];
    core[v] = UNSET;
  }
}

// Remove every remaining vertex with deg <= k; count the rest.
__global__ void __launch_bounds__(CORE_THREADS)
core_scan_kernel(uint32_t n, uint32_t k, const uint32_t *deg, uint32_t *core,
                 uint32_t *frontier, CoreCounters *ctr) {
  const uint32_t stride = gridDim.x * blockDim.x;
  // the loop bound is rounded up to whole warps so every lane reaches the
  // ballot in append()
  const uint32_t n_pad = (n + 31) & ~31u;
  uint32_t left = 0;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n_pad; v += stride) {
    bool take = false;
    if (v < n && core[v] == UNSET) {
      if (deg[v] <= k) {
        core[v] = k;
        take = true;
      } else {
        left++;
      }
    }
    append(take, v, &ctr->frontier, frontier);
  }
  for (int o = 16; o; o >>= 1) left += __shfl_xor_sync(0xffffffffu, left, o);
  if ((threadIdx.x & 31) == 0 && left) atomicAdd(&ctr->remaining, left);
}

// One warp per frontier vertex: decrement the neighbours still present.
__global__ void __launch_bounds__(CORE_THREADS)
core_peel_kernel(const uint32_t *off, const uint32_t *adj, uint32_t k,
                 const uint32_t *fin, uint32_t nin, uint32_t *deg, uint32_t *core,
                 uint32_t *fout, CoreCounters *ctr) {
  const int lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * (blockDim.x / 32);
  for (uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) / 32; w < nin; w += warps) {
    const uint32_t v = fin[w];
    const uint32_t b = off[v], e = off[v + 1];
    for (uint32_t i0 = b; i0 < e; i0 += 32) {
      const uint32_t i = i0 + lane;
      bool take = false;
      uint32_t u = 0;
      if (i < e) {
        u = adj[i];
        if (*(volatile uint32_t *)&core[u] == UNSET) {
          const uint32_t old = atomicSub(&deg[u], 1u);
          if (old == k + 1) {
            core[u] = k;  // this thread moved u to k: it owns u's removal
            take = true;
          } else if (old <= k) {
            atomicAdd(&deg[u], 1u);  // u was already claimed at level k
          }
        }
      }
      append(take, u, &ctr->frontier, fout);
    }
  }
}

}  // namespace

// Core numbers of the CSR graph in device memory.  scratch needs 3n words;
// ctr_host is pinned host memory for one CoreCounters (16 bytes) and ctr_dev
// its device twin.  Returns 0 or a cudaError_t value.
int gpu_core_numbers(const uint32_t *d_off, const uint32_t *d_adj, uint32_t n,
                     uint32_t *d_core, uint32_t *d_scratch, void *ctr_dev,
                     void *ctr_host, int num_sms, cudaStream_t st) {
  if (n == 0) return 0;
  uint32_t *deg = d_scratch, *fa = d_scratch + n, *fb = d_scratch + 2 * (size_t)n;
  CoreCounters *dc = (CoreCounters *)ctr_dev;
  volatile CoreCounters *hc = (volatile CoreCounters *)ctr_host;
  const int grid = num_sms * 8;
  core_init_kernel<<<grid, CORE_THREADS, 0, st>>>(d_off, n, deg, d_core);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return (int)e;
  uint64_t removed = 0;
  for (uint32_t k = 0; removed < n; k++) {
    e = cudaMemsetAsync(dc, 0, sizeof(CoreCounters), st);
    if (e != cudaSuccess) return (int)e;
    core_scan_kernel<<<grid, CORE_THREADS, 0, st>>>(n, k, deg, d_core, fa, dc);
    if ((e = cudaMemcpyAsync((void *)hc, dc, sizeof(CoreCounters), cudaMemcpyDeviceToHost, st)) !=
        cudaSuccess)
      return (int)e;
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return (int)e;
    uint32_t nin = hc->frontier;
    removed += nin;
    while (nin) {
      if ((e = cudaMemsetAsync(dc, 0, sizeof(CoreCounters), st)) != cudaSuccess) return (int)e;
      const uint32_t blocks = (uint32_t)std::min<uint64_t>((nin + 7) / 8, (uint64_t)grid);
      core_peel_kernel<<<blocks, CORE_THREADS, 0, st>>>(d_off, d_adj, k, fa, nin, deg, d_core,
                                                        fb, dc);
      if ((e = cudaMemcpyAsync((void *)hc, dc, sizeof(CoreCounters), cudaMemcpyDeviceToHost,
                               st)) != cudaSuccess)
        return (int)e;
      if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return (int)e;
      nin = hc->frontier;
      removed += nin;
      uint32_t *t = fa;
      fa = fb;
      fb = t;
    }
    if (removed > n) return (int)cudaErrorUnknown;  // cannot happen: each vertex is claimed once
  }
  return (int)cudaGetLastError();
}

}  // namespace scs

using namespace scs;

extern "C" int scs_core_decompose_gpu(uint32_t n, const uint32_t *off, const uint32_t *adj,
                                      uint32_t *core, int device) {
  if (!off || !core || (n && !adj && off[n] > 0)) return SCS_EINVAL;
  for (uint32_t v = 0; v < n; v++)
    if (off[v + 1] < off[v]) return SCS_EINVAL;
  const uint64_t nnz = off[n];
  for (uint64_t i = 0; i < nnz; i++)
    if (adj[i] >= n) return SCS_EINVAL;
  if (n == 0) return 0;
  if (cudaSetDevice(device) != cudaSuccess) return SCS_ECUDA;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
    return SCS_ECUDA;
  cudaStream_t st = nullptr;
  uint32_t *d_off = nullptr, *d_adj = nullptr, *d_core = nullptr, *d_scr = nullptr;
  void *d_ctr = nullptr, *h_ctr = nullptr;
  int rc = SCS_ECUDA;
  do {
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) break;
    if (cudaMalloc((void **)&d_off, (n + 1) * 4ull) != cudaSuccess) break;
    if (cudaMalloc((void **)&d_adj, std::max<uint64_t>(nnz, 1) * 4ull) != cudaSuccess) break;
    if (cudaMalloc((void **)&d_core, n * 4ull) != cudaSuccess) break;
    if (cudaMalloc((void **)&d_scr, 3ull * n * 4ull) != cudaSuccess) break;
    if (cudaMalloc(&d_ctr, 16) != cudaSuccess) break;
    if (cudaMallocHost(&h_ctr, 16) != cudaSuccess) break;
    if (cudaMemcpyAsync(d_off, off, (n + 1) * 4ull, cudaMemcpyHostToDevice, st) != cudaSuccess)
      break;
    if (nnz && cudaMemcpyAsync(d_adj, adj, nnz * 4ull, cudaMemcpyHostToDevice, st) != cudaSuccess)
      break;
    if (gpu_core_numbers(d_off, d_adj, n, d_core, d_scr, d_ctr, h_ctr, sms, st) != 0) break;
    if (cudaMemcpyAsync(core, d_core, n * 4ull, cudaMemcpyDeviceToHost, st) != cudaSuccess) break;
    if (cudaStreamSynchronize(st) != cudaSuccess) break;
    rc = 0;
  } while (0);
  cudaFree(d_off);
  cudaFree(d_adj);
  cudaFree(d_core);
  cudaFree(d_scr);
  cudaFree(d_ctr);
  if (h_ctr) cudaFreeHost(h_ctr);
  if (st) cudaStreamDestroy(st);
  return rc;
}
