// noalloc.cu -- allocation-free variant of the per-query local-graph build.
//
// Some callers cannot call cudaMalloc: code running inside another
// framework's memory pool or allocator hook, plugins whose host forbids
// device allocations after start-up, and code that must not allocate once a
// latency-critical loop has started.  scs_local_graph_noalloc lets them run
// the preprocessing stage (bounded BFS, core/distance filter, q's component,
// compacted local CSR) with buffers they already own: the caller passes the
// graph and the outputs, and the kernel's scratch (distances, bitmaps,
// frontiers) lives in the file-scope array below, which every GPU that loads
// this library holds until the process exits.
//
// The array has a fixed size: graphs of up to SCS_NOALLOC_MAX_N vertices.
// All calls share it and it keeps the last call's contents; the kernel clears
// what must start at zero on every call.  Calls that overlap on the GPU (on
// different streams, or from several threads) race on the array and give
// undefined results: issue them one after another.
#include <cstdint>
#include <cstring>
#include <mutex>

#include "../../include/scs.h"
#include "prep_core.cuh"

namespace scs {

constexpr uint32_t NOALLOC_MAX_N = SCS_NOALLOC_MAX_N;
constexpr uint32_t NOALLOC_MAX_W = NOALLOC_MAX_N / 32 + 1;

// scratch layout (bytes, each part 256-byte aligned)
constexpr size_t NA_DIST = 0;                                       // u16[n]
constexpr size_t NA_VIS = (NA_DIST + 2ull * NOALLOC_MAX_N + 255) & ~255ull;
constexpr size_t NA_COMP = (NA_VIS + 4ull * NOALLOC_MAX_W + 255) & ~255ull;
constexpr size_t NA_WPRE = (NA_COMP + 4ull * NOALLOC_MAX_W + 255) & ~255ull;
constexpr size_t NA_FA = (NA_WPRE + 4ull * NOALLOC_MAX_W + 255) & ~255ull;
constexpr size_t NA_FB = (NA_FA + 4ull * NOALLOC_MAX_N + 255) & ~255ull;
constexpr size_t NA_LDIST = (NA_FB + 4ull * NOALLOC_MAX_N + 255) & ~255ull;  // u16[n]
constexpr size_t NA_BYTES = (NA_LDIST + 2ull * NOALLOC_MAX_N + 255) & ~255ull;

static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_BYTES];

__global__ void __launch_bounds__(PREP_THREADS)
local_graph_noalloc_kernel(DevGraph g, uint32_t q, uint32_t kl, uint32_t ubd,
                           unsigned char *scratch, uint32_t *gid,
                           uint32_t *dist_out, uint32_t *loff, uint32_t *ladj,
                           unsigned long long cap_adj, uint32_t *info) {
  __shared__ uint32_t sh_warp[PREP_WARPS];
  __shared__ uint32_t sh_cnt[4];
  __shared__ uint32_t sh_ql;
  __shared__ unsigned long long sh_bytes;
  uint16_t *dist = (uint16_t *)(scratch + NA_DIST);
  uint32_t *vis = (uint32_t *)(scratch + NA_VIS);
  uint32_t *comp = (uint32_t *)(scratch + NA_COMP);
  uint32_t *wpre = (uint32_t *)(scratch + NA_WPRE);
  uint32_t *fa = (uint32_t *)(scratch + NA_FA);
  uint32_t *fb = (uint32_t *)(scratch + NA_FB);
  uint16_t *ldist = (uint16_t *)(scratch + NA_LDIST);
  if (threadIdx.x == 0) sh_bytes = 0;
  __syncthreads();
  // build_local_graph clears dist/vis/comp itself before using them
  const uint32_t nl = build_local_graph(g, q, kl, ubd, dist, vis, comp, fa, fb,
                                        wpre, gid, ldist, loff, ladj, cap_adj,
                                        g.n, sh_warp, sh_cnt, &sh_bytes, &sh_ql);
  if (nl == UINT32_MAX) {
    if (threadIdx.x == 0) {
      info[0] = 0;
      info[1] = 0;
      info[2] = 0;
      info[3] = 1;  // the padded rows do not fit in cap_adj
    }
    return;
  }
  for (uint32_t i = threadIdx.x; i < nl; i += PREP_THREADS)
    dist_out[i] = ldist[i] == INF16 ? 1000000000u : (uint32_t)ldist[i];
  if (threadIdx.x == 0) {
    info[0] = nl;
    info[1] = sh_ql;
    info[2] = loff[nl];
    info[3] = 0;
  }
}

}  // namespace scs

using namespace scs;

namespace {
// Set-up state, one entry per device ordinal: the device address of the
// scratch array and the unique id of the CUDA context it was looked up in.
// A device reset (cudaDeviceReset) destroys that context; the next call sees
// a new context id and does the set-up again, so a stale address is never
// passed to the kernel.
constexpr int MAX_DEVICES = 64;
typedef int (*CtxGetCurrentFn)(void **);
typedef int (*CtxGetIdFn)(void *, unsigned long long *);
std::mutex g_mu;
bool g_fn_ready = false;
CtxGetCurrentFn g_ctx_current = nullptr;
CtxGetIdFn g_ctx_id = nullptr;
void *g_scratch_ptr[MAX_DEVICES];
unsigned long long g_scratch_ctx[MAX_DEVICES];  // 0: not set up

// Id of the context current on this thread (0 if none or unavailable).  The
// driver calls are reached through the runtime's entry-point table, so the
// library needs no link against the driver library.
unsigned long long current_ctx_id() {
  if (!g_fn_ready) {
    void *a = nullptr, *b = nullptr;
    cudaDriverEntryPointQueryResult qa, qb;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000,
                                         cudaEnableDefault, &qa) == cudaSuccess &&
        qa == cudaDriverEntryPointSuccess &&
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000,
                                         cudaEnableDefault, &qb) == cudaSuccess &&
        qb == cudaDriverEntryPointSuccess) {
      g_ctx_current = (CtxGetCurrentFn)a;
      g_ctx_id = (CtxGetIdFn)b;
    }
    cudaGetLastError();
    g_fn_ready = true;
  }
  if (!g_ctx_current || !g_ctx_id) return 0;
  void *ctx = nullptr;
  unsigned long long id = 0;
  if (g_ctx_current(&ctx) != 0 || !ctx) return 0;
  if (g_ctx_id(ctx, &id) != 0) return 0;
  return id + 1;  // never 0
}
}  // namespace

extern "C" {

int scs_local_graph_noalloc(const uint32_t *d_off, const uint32_t *d_adj,
                            const uint32_t *d_core, uint32_t n, uint32_t dmax,
                            uint32_t q, uint32_t kl, uint32_t ubd,
                            uint32_t *d_gid, uint32_t *d_dist,
                            uint32_t *d_loc_off, uint32_t *d_loc_adj,
                            uint64_t loc_adj_cap, uint32_t *d_info,
                            void *stream) {
  if (!d_off || !d_adj || !d_core || !d_gid || !d_dist || !d_loc_off ||
      !d_loc_adj || !d_info)
    return SCS_EINVAL;
  if (n == 0 || n > NOALLOC_MAX_N || q >= n) return SCS_EINVAL;
  // hop distances are kept as u16 with 0xFFFF meaning "not reached", so a
  // bound at or above 0xFFFF would let unreached vertices pass the filter
  if (ubd >= INF16) return SCS_EINVAL;
  // an error left pending by the caller's earlier work stays pending for the
  // caller: report it without consuming it
  if (cudaPeekAtLastError() != cudaSuccess) return SCS_ECUDA;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) {
    cudaGetLastError();
    return SCS_ECUDA;
  }
  void *scratch = nullptr;
  {
    // Set-up, once per device and context, with that device current: the
    // device address of the scratch array (the host-side symbol is only a
    // stand-in).  The first call on a device does it and loads this module
    // there, so make that call before any stream capture.
    std::lock_guard<std::mutex> lk(g_mu);
    unsigned long long ctx = current_ctx_id();
    if (ctx == 0) {  // no context current yet: make the device's current
      if (cudaSetDevice(dev) != cudaSuccess) {
        cudaGetLastError();
        return SCS_ECUDA;
      }
      ctx = current_ctx_id();
    }
    if (ctx == 0 || g_scratch_ctx[dev] != ctx) {
      void *p = nullptr;
      if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
        cudaGetLastError();  // the failed lookup's own error
        return SCS_ECUDA;
      }
      g_scratch_ptr[dev] = p;
      g_scratch_ctx[dev] = ctx;  // 0 (ids unavailable): look up every call
    }
    scratch = g_scratch_ptr[dev];
  }
  DevGraph g{n, dmax, d_off, d_adj, d_core};
  local_graph_noalloc_kernel<<<1, PREP_THREADS, 0, (cudaStream_t)stream>>>(
      g, q, kl, ubd, (unsigned char *)scratch, d_gid, d_dist, d_loc_off,
      d_loc_adj, loc_adj_cap, d_info);
  // no error was pending before the launch, so this one is the launch's own
  if (cudaGetLastError() != cudaSuccess) return SCS_ECUDA;
  return 0;
}

}  // extern "C"
