// prep_core.cuh -- per-query local-graph build shared by the engine's
// preprocessing kernel and the allocation-free entry point.
//
// Restates cal_query_dist (src/Graph.h:111-142, bounded at depth ubD),
// initialReductionRules (src/helpers.cc:207-248: keep core > kl and
// dist <= ubD) and CompressTask/NeighborUpdate (src/helpers.cc:250-368: the
// filtered CSR), restricted to q's component in G[kept], with local ids in
// ascending global id and rows padded to a multiple of 4 with SENT.
#pragma once
#include "scs_device.cuh"

namespace scs {

constexpr int PREP_WARPS = PREP_THREADS / 32;

static __device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t x = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += x;
  }
  return v;
}

// In-place exclusive scan of a[0..len) (global); returns the total.
static __device__ uint32_t block_excl_scan(uint32_t *a, uint32_t len,
                                    uint32_t *sh_warp) {
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
  uint32_t running = 0;
  for (uint32_t base = 0; base < len; base += PREP_THREADS) {
    uint32_t i = base + t;
    uint32_t v = i < len ? a[i] : 0;
    uint32_t x = warp_incl_scan(v);
    if (lane == 31) sh_warp[wid] = x;
    __syncthreads();
    if (wid == 0) {
      uint32_t w = lane < PREP_WARPS ? sh_warp[lane] : 0;
      w = warp_incl_scan(w);
      if (lane < PREP_WARPS) sh_warp[lane] = w;
    }
    __syncthreads();
    uint32_t woff = wid ? sh_warp[wid - 1] : 0;
    uint32_t total = sh_warp[PREP_WARPS - 1];
    if (i < len) a[i] = running + woff + x - v;
    running += total;
    __syncthreads();
  }
  return running;
}

static __device__ __forceinline__ bool bit_get(const uint32_t *bm, uint32_t v) {
  return (bm[v >> 5] >> (v & 31)) & 1u;
}

// local id of a vertex whose comp bit is set
static __device__ __forceinline__ uint32_t local_id(const uint32_t *comp,
                                             const uint32_t *wpre, uint32_t v) {
  uint32_t w = comp[v >> 5];
  return wpre[v >> 5] + __popc(w & ((1u << (v & 31)) - 1u));
}

// Level-synchronous BFS from q.  mode 0: whole graph, depth <= maxd, writes
// dist; mode 1: only vertices with keep (core > kl && dist <= ubd), any depth,
// marks visited in `vis`.
static __device__ void block_bfs(const DevGraph &g, uint32_t q, int mode,
                          uint32_t maxd, uint32_t kl, uint32_t ubd,
                          uint16_t *dist, uint32_t *vis, uint32_t *fa,
                          uint32_t *fb, uint32_t *sh_cnt,
                          unsigned long long *bytes) {
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
  if (t == 0) {
    vis[q >> 5] |= 1u << (q & 31);
    if (mode == 0) dist[q] = 0;
    fa[0] = q;
    sh_cnt[0] = 1;
  }
  __syncthreads();
  uint32_t fsize = sh_cnt[0];
  uint32_t level = 0;
  unsigned long long edges = 0;
  while (fsize > 0 && (mode == 1 || level < maxd)) {
    if (t == 0) sh_cnt[1] = 0;
    __syncthreads();
    for (uint32_t fi = wid; fi < fsize; fi += PREP_WARPS) {
      uint32_t v = fa[fi];
      uint32_t b = g.off[v], e = g.off[v + 1];
      edges += (lane == 0) ? (e - b) : 0;
      for (uint32_t k = b; k < e; k += 32) {
        bool fresh = false;
        uint32_t w = 0;
        if (k + lane < e) {
          w = g.adj[k + lane];
          bool ok = true;
          if (mode == 1) ok = g.core[w] > kl && dist[w] <= ubd;
          uint32_t bit = 1u << (w & 31);
          if (ok && !(vis[w >> 5] & bit)) {
            uint32_t old = atomicOr(&vis[w >> 5], bit);
            fresh = !(old & bit);
          }
        }
        unsigned m = __ballot_sync(0xffffffffu, fresh);
        uint32_t base = 0;
        if (lane == 0 && m) base = atomicAdd(&sh_cnt[1], __popc(m));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (fresh) {
          fb[base + __popc(m & ((1u << lane) - 1u))] = w;
          if (mode == 0) dist[w] = (uint16_t)(level + 1);
        }
      }
    }
    __syncthreads();
    fsize = sh_cnt[1];
    uint32_t *tmp = fa;
    fa = fb;
    fb = tmp;
    level++;
    __syncthreads();
  }
  if (lane == 0 && edges) atomicAdd(bytes, edges * 4ull);
}


// Build the local graph of one query (all threads of the block call this).
// Scratch: dist[n] (u16), vis/comp/wpre[nw+1], fa/fb[n].  Outputs lgid,
// ldist (u16), loff[nl+1], ladj (padded rows).  Returns the local vertex
// count, or UINT32_MAX when it exceeds max_local or the rows exceed cap_adj.
// On return fa[i] holds the unpadded local degree of local vertex i and
// *q_local (shared) the local id of q.
static __device__ uint32_t build_local_graph(
    const DevGraph &g, uint32_t q, uint32_t kl, uint32_t ubd, uint16_t *dist,
    uint32_t *vis, uint32_t *comp, uint32_t *fa, uint32_t *fb, uint32_t *wpre,
    uint32_t *lgid, uint16_t *ldist, uint32_t *loff, uint32_t *ladj,
    unsigned long long cap_adj, uint32_t max_local, uint32_t *sh_warp,
    uint32_t *sh_cnt, unsigned long long *bytes, uint32_t *q_local) {
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
  const uint32_t n = g.n, nw = (n + 31) / 32;
  for (uint32_t i = t; i < n; i += PREP_THREADS) dist[i] = (uint16_t)INF16;
  for (uint32_t i = t; i < nw; i += PREP_THREADS) {
    vis[i] = 0;
    comp[i] = 0;
  }
  __syncthreads();
  // 1. bounded BFS over the whole graph
  block_bfs(g, q, 0, ubd, kl, ubd, dist, vis, fa, fb, sh_cnt, bytes);
  __syncthreads();
  // 2. q's component inside the kept set
  block_bfs(g, q, 1, 0, kl, ubd, dist, comp, fa, fb, sh_cnt, bytes);
  __syncthreads();
  // 3. local ids: exclusive prefix of per-word popcounts
  for (uint32_t i = t; i < nw; i += PREP_THREADS) wpre[i] = __popc(comp[i]);
  __syncthreads();
  uint32_t nl = block_excl_scan(wpre, nw, sh_warp);
  __syncthreads();
  if (nl > max_local) return UINT32_MAX;
  // 4. gid, distance, local degree (padded) into loff[i]
  for (uint32_t wi = t; wi < nw; wi += PREP_THREADS) {
    uint32_t bits = comp[wi], base = wpre[wi];
    while (bits) {
      uint32_t b = __ffs(bits) - 1;
      bits &= bits - 1;
      uint32_t v = wi * 32 + b;
      lgid[base] = v;
      ldist[base] = dist[v];
      base++;
    }
  }
  if (t == 0) sh_cnt[2] = 0;
  __syncthreads();
  for (uint32_t i = wid; i < nl; i += PREP_WARPS) {
    uint32_t v = lgid[i];
    uint32_t b = g.off[v], e = g.off[v + 1], c = 0;
    for (uint32_t k = b + lane; k < e; k += 32)
      c += bit_get(comp, g.adj[k]) ? 1u : 0u;
    for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if (lane == 0) loff[i] = (c + 3u) & ~3u;
    if (lane == 0) fa[i] = c;  // unpadded local degree
    if (lane == 0 && c > DMASK) atomicOr(&sh_cnt[2], 1u);
  }
  __syncthreads();
  // the search's state words hold in-task degrees in 15 bits
  if (sh_cnt[2]) return UINT32_MAX;
  uint32_t total = block_excl_scan(loff, nl, sh_warp);
  if (t == 0) loff[nl] = total;
  __syncthreads();
  if (total > cap_adj) return UINT32_MAX;
  // 5. fill rows in ascending order (ordered warp compaction), pad with SENT
  unsigned long long pbytes = 0;
  for (uint32_t i = wid; i < nl; i += PREP_WARPS) {
    uint32_t v = lgid[i];
    uint32_t b = g.off[v], e = g.off[v + 1];
    uint32_t w0 = loff[i], wpos = 0;
    for (uint32_t k = b; k < e; k += 32) {
      uint32_t w = 0;
      bool in = false;
      if (k + lane < e) {
        w = g.adj[k + lane];
        in = bit_get(comp, w);
      }
      unsigned m = __ballot_sync(0xffffffffu, in);
      if (in) ladj[w0 + wpos + __popc(m & ((1u << lane) - 1u))] = local_id(comp, wpre, w);
      wpos += __popc(m);
    }
    uint32_t padded = loff[i + 1] - w0;
    for (uint32_t k = wpos + lane; k < padded; k += 32) ladj[w0 + k] = SENT;
    if (lane == 0) pbytes += 4ull * (e - b) + 4ull * padded + 12ull;
  }
  if (lane == 0 && pbytes) atomicAdd(bytes, pbytes);
  __syncthreads();
  if (t == 0) *q_local = local_id(comp, wpre, q);
  __syncthreads();
  return nl;
}

}  // namespace scs

