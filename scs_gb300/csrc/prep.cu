// prep.cu -- per-query preprocessing on the GPU, one thread-block cluster
// per query.
//
// Restates, for one query slot:
//   * cal_query_dist (src/Graph.h:111-142): BFS hop distance from q, here
//     bounded at depth ubD (deeper vertices are filtered out anyway);
//   * initialReductionRules (src/helpers.cc:207-248): keep v iff
//     core[v] > kl && dist[v] <= ubD;
//   * CompressTask + NeighborUpdate (src/helpers.cc:250-368): the root task
//     (C = {q}, R = kept) with dC/dR, and the filtered CSR.  Here the kept set
//     is restricted to q's component in G[kept] (other components have no
//     edge into any task containing q), vertices get local ids in ascending
//     global id, and every local row is ascending and padded to a multiple of
//     4 entries so the search kernel can read rows with 16-byte loads.
//
// The output is the one build_local_graph (prep_core.cuh) gives with a single
// CTA; here the CTAs of one cluster share the work of a query, so a graph
// with millions of vertices is not walked by one SM:
//   * BFS levels: frontier vertices go to warps, those of big_row or more
//     neighbours (PrepScratch::big_row) to whole CTAs; a level whose
//     frontier holds more than n/64 vertices runs bottom-up instead (every
//     unvisited vertex looks for a neighbour in the frontier); the frontier counters live in rank 0's shared
//     memory and are updated through distributed shared memory;
//   * the two prefix scans (local ids, row offsets) run over one segment per
//     CTA, offset by the segment totals the other CTAs hold;
//   * the component BFS counts each component vertex's local degree as it
//     walks the row (every kept neighbour of a component vertex is in the
//     component), so no separate counting pass reads the rows again;
//   * the ordered row fill goes warp per row, or CTA per row for rows of
//     big_row or more.
// Every phase ends in a cluster barrier (barrier.cluster, in hardware: no
// software wait).  Data another CTA wrote is read through L2 (__ldcg), so no
// stale L1 line is seen.  A CTA reads the other CTAs' shared memory only
// before the barrier that ends the phase, so none exits while it is read.
#include <cooperative_groups.h>

#include "prep_core.cuh"

namespace cg = cooperative_groups;

namespace scs {

namespace {


// Shared state of one CTA.  The cluster's counters are rank 0's copies.
struct PrepSh {
  uint32_t warp[PREP_WARPS];  // block reductions and scans
  uint32_t cnt[3][2];         // frontier (small, big) counts, by level mod 3
  uint32_t nbig;              // local rows of big_row or more entries
  uint32_t flag;              // a local degree does not fit the state word
  uint32_t seg_total;         // this CTA's segment sum in a cluster scan
  uint32_t q_local;
  unsigned long long root;    // root record offset
};

__device__ __forceinline__ uint32_t lane_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

__device__ __forceinline__ bool bit_cg(const uint32_t *bm, uint32_t v) {
  return (__ldcg(bm + (v >> 5)) >> (v & 31)) & 1u;
}

__device__ __forceinline__ uint32_t local_id_cg(const uint32_t *comp,
                                                const uint32_t *wpre, uint32_t v) {
  const uint32_t w = __ldcg(comp + (v >> 5));
  return __ldcg(wpre + (v >> 5)) + __popc(w & ((1u << (v & 31)) - 1u));
}

// Sum of v over the block (every thread gets it).
__device__ uint32_t block_sum_all(uint32_t v, uint32_t *warp_buf) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if (lane == 0) warp_buf[wid] = v;
  __syncthreads();
  uint32_t tot = 0;
#pragma unroll
  for (int w = 0; w < PREP_WARPS; w++) tot += warp_buf[w];
  __syncthreads();
  return tot;
}

// In-place exclusive scan of a[0..len) (global, read through L2) by one CTA,
// starting from base.
__device__ void block_scan_from(uint32_t *a, uint32_t len, uint32_t base,
                                uint32_t *warp_buf) {
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
  uint32_t running = base;
  for (uint32_t b0 = 0; b0 < len; b0 += PREP_THREADS) {
    const uint32_t i = b0 + t;
    const uint32_t v = i < len ? __ldcg(a + i) : 0;
    const uint32_t x = warp_incl_scan(v);
    if (lane == 31) warp_buf[wid] = x;
    __syncthreads();
    uint32_t woff = 0, total = 0;
#pragma unroll
    for (int w = 0; w < PREP_WARPS; w++) {
      const uint32_t c = warp_buf[w];
      woff += w < wid ? c : 0u;
      total += c;
    }
    if (i < len) a[i] = running + woff + x - v;
    running += total;
    __syncthreads();
  }
}

// Exclusive scan of a[0..len) over the cluster: CTA r scans the r-th segment
// from the sum of the segments before it.  Returns the total.  Ends with a
// cluster barrier.
__device__ uint32_t cluster_excl_scan(cg::cluster_group &cl, PrepSh &sh,
                                      uint32_t *a, uint32_t len) {
  const uint32_t R = cl.num_blocks(), r = cl.block_rank();
  const uint32_t seg = (len + R - 1) / R;
  const uint32_t lo = min(len, r * seg), hi = min(len, lo + seg);
  uint32_t s = 0;
  for (uint32_t i = lo + threadIdx.x; i < hi; i += PREP_THREADS) s += __ldcg(a + i);
  s = block_sum_all(s, sh.warp);
  if (threadIdx.x == 0) sh.seg_total = s;
  cl.sync();
  uint32_t base = 0, total = 0;
  for (uint32_t k = 0; k < R; k++) {
    const uint32_t v = *cl.map_shared_rank(&sh.seg_total, k);
    base += k < r ? v : 0u;
    total += v;
  }
  block_scan_from(a + lo, hi - lo, base, sh.warp);
  cl.sync();
  return total;
}

// Rows of at most GROUP_ROW entries are walked four at a time per warp, by
// groups of 8 lanes, so a warp has four rows' loads in flight.
constexpr uint32_t GROUP_ROW = 64;

// Each lane tests adjacency entry k of its row (none when k >= hi; the call
// is warp-wide).  Appends the newly reached vertices to the next frontier
// (small ones from the front, those of big_row or more neighbours from the
// back) and records distances in mode 0.  In mode 1 it returns 1 when the
// entry is a neighbour inside the local graph: kept, or q itself.  Every
// kept neighbour of a vertex of q's component is in the component, so
// summed over a component vertex's row this is its local degree.
__device__ __forceinline__ uint32_t bfs_visit(const DevGraph &g, uint32_t k,
                                              uint32_t hi, int mode, uint32_t level,
                                              uint32_t kl, uint32_t ubd, uint32_t big_row,
                                              uint32_t q, uint16_t *dist,
                                              uint32_t *vis, uint32_t *nxt, uint32_t *ncnt) {
  const int lane = threadIdx.x & 31;
  bool fresh = false, big = false, local = false;
  uint32_t w = 0;
  if (k < hi) {
    w = g.adj[k];
    bool ok = true;
    if (mode == 1) {
      ok = g.core[w] > kl && __ldcg(dist + w) <= ubd;
      local = ok || w == q;
    }
    const uint32_t bit = 1u << (w & 31);
    if (ok && !(__ldcg(vis + (w >> 5)) & bit)) {
      const uint32_t old = atomicOr(&vis[w >> 5], bit);
      fresh = !(old & bit);
    }
    big = fresh && g.off[w + 1] - g.off[w] >= big_row;
  }
  const unsigned ms = __ballot_sync(0xffffffffu, fresh && !big);
  const unsigned mb = __ballot_sync(0xffffffffu, big);
  uint32_t bs = 0, bb = 0;
  if (lane == 0) {
    if (ms) bs = atomicAdd(&ncnt[0], (uint32_t)__popc(ms));
    if (mb) bb = atomicAdd(&ncnt[1], (uint32_t)__popc(mb));
  }
  bs = __shfl_sync(0xffffffffu, bs, 0);
  bb = __shfl_sync(0xffffffffu, bb, 0);
  if (fresh) {
    if (big)
      nxt[g.n - 1u - (bb + __popc(mb & lane_lt()))] = w;
    else
      nxt[bs + __popc(ms & lane_lt())] = w;
    if (mode == 0) dist[w] = (uint16_t)(level + 1);
  }
  return local ? 1u : 0u;
}

// Level-synchronous BFS from q over the cluster.  mode 0: whole graph, depth
// <= maxd, writes dist; mode 1: only vertices with core > kl && dist <= ubd,
// any depth, marks `vis`.  Level L reads the counts cnt[L % 3], appends to
// cnt[(L+1) % 3] and rank 0 clears cnt[(L+2) % 3], which nobody reads or
// writes in level L: one barrier per level.
__device__ void cluster_bfs(cg::cluster_group &cl, PrepSh &sh, PrepSh *r0,
                            const DevGraph &g, uint32_t q, int mode, uint32_t maxd,
                            uint32_t kl, uint32_t ubd, uint32_t big_row, uint16_t *dist,
                            uint32_t *vis, uint32_t *fa, uint32_t *fb, uint32_t *ldeg,
                            unsigned long long *bytes) {
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
  const uint32_t R = cl.num_blocks(), r = cl.block_rank();
  if (r == 0 && t == 0) {
    atomicOr(&vis[q >> 5], 1u << (q & 31));
    if (mode == 0) dist[q] = 0;
    for (int c = 0; c < 3; c++) sh.cnt[c][0] = sh.cnt[c][1] = 0;
    const bool big = g.off[q + 1] - g.off[q] >= big_row;
    fa[big ? g.n - 1u : 0u] = q;
    sh.cnt[0][big ? 1 : 0] = 1;
  }
  cl.sync();
  uint32_t *cur = fa, *nxt = fb;
  unsigned long long edges = 0;
  for (uint32_t level = 0;; level++) {
    const uint32_t c = level % 3;
    const uint32_t ns = r0->cnt[c][0], nb = r0->cnt[c][1];
    if (ns + nb == 0 || (mode == 0 && level >= maxd)) break;
    if (r == 0 && t == 0) sh.cnt[(level + 2) % 3][0] = sh.cnt[(level + 2) % 3][1] = 0;
    uint32_t *ncnt = r0->cnt[(level + 1) % 3];
    if (mode == 0 && ns + nb > (g.n >> 6) + 32u) {
      // Large frontier: bottom-up.  Every unvisited vertex scans its row
      // for a neighbour at distance `level` and stops at the first one
      // (Beamer's direction-optimizing BFS).  Distances are the same as
      // top-down; far fewer edges are read when most of the graph is near.
      for (uint32_t b0 = r * PREP_THREADS + (uint32_t)wid * 32u; b0 < g.n;
           b0 += R * PREP_THREADS) {
        const uint32_t v = b0 + lane;
        bool fresh = false, big = false;
        if (v < g.n && !((__ldcg(vis + (v >> 5)) >> (v & 31)) & 1u)) {
          const uint32_t lo = g.off[v], hi = g.off[v + 1];
          uint32_t k = lo;
          for (; k < hi; k++)
            if (__ldcg(dist + g.adj[k]) == level) {
              fresh = true;
              break;
            }
          edges += (k < hi ? k + 1 : hi) - lo;
          if (fresh) {
            dist[v] = (uint16_t)(level + 1);
            big = hi - lo >= big_row;
          }
        }
        // the warp's 32 vertices share one visited word (b0 is a multiple of 32)
        const unsigned fm = __ballot_sync(0xffffffffu, fresh);
        if (lane == 0 && fm) atomicOr(&vis[b0 >> 5], fm);
        const unsigned ms = __ballot_sync(0xffffffffu, fresh && !big);
        const unsigned mb = __ballot_sync(0xffffffffu, big);
        uint32_t bs = 0, bb = 0;
        if (lane == 0) {
          if (ms) bs = atomicAdd(&ncnt[0], (uint32_t)__popc(ms));
          if (mb) bb = atomicAdd(&ncnt[1], (uint32_t)__popc(mb));
        }
        bs = __shfl_sync(0xffffffffu, bs, 0);
        bb = __shfl_sync(0xffffffffu, bb, 0);
        if (fresh) {
          if (big)
            nxt[g.n - 1u - (bb + __popc(mb & lane_lt()))] = v;
          else
            nxt[bs + __popc(ms & lane_lt())] = v;
        }
      }
      cl.sync();
      uint32_t *tmp = cur;
      cur = nxt;
      nxt = tmp;
      continue;
    }
    // frontier vertices with long rows: a CTA each
    for (uint32_t b = r; b < nb; b += R) {
      const uint32_t v = __ldcg(cur + (g.n - 1u - b));
      const uint32_t lo = g.off[v], hi = g.off[v + 1];
      if (t == 0) edges += hi - lo;
      uint32_t c = 0;
      for (uint32_t k0 = lo + (uint32_t)wid * 32u; k0 < hi; k0 += PREP_THREADS)
        c += bfs_visit(g, k0 + lane, hi, mode, level, kl, ubd, big_row, q, dist, vis, nxt, ncnt);
      if (mode == 1) {
        c = block_sum_all(c, sh.warp);
        if (t == 0) ldeg[v] = c;
      }
    }
    // the others: four per warp, by 8-lane groups when all four rows are
    // short, else one after the other by the whole warp
    for (uint32_t f0 = (r * PREP_WARPS + wid) * 4u; f0 < ns; f0 += R * PREP_WARPS * 4u) {
      const uint32_t grp = lane >> 3, sl = lane & 7;
      uint32_t lo = 0, hi = 0;
      if (f0 + grp < ns) {
        const uint32_t v = __ldcg(cur + f0 + grp);
        lo = g.off[v];
        hi = g.off[v + 1];
      }
      if (sl == 0) edges += hi - lo;
      uint32_t len = hi - lo;
      for (int o = 8; o < 32; o <<= 1) len = max(len, __shfl_xor_sync(0xffffffffu, len, o));
      uint32_t c = 0;  // this group's row: its local degree (mode 1)
      if (len <= GROUP_ROW) {
        for (uint32_t k0 = 0; k0 < len; k0 += 8)
          c += bfs_visit(g, lo + k0 + sl, hi, mode, level, kl, ubd, big_row, q, dist, vis,
                         nxt, ncnt);
        for (int o = 4; o; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
      } else {
        for (uint32_t x = 0; x < 4; x++) {
          const uint32_t lx = __shfl_sync(0xffffffffu, lo, x * 8), hx = __shfl_sync(0xffffffffu, hi, x * 8);
          uint32_t cx = 0;
          for (uint32_t k0 = lx; k0 < hx; k0 += 32)
            cx += bfs_visit(g, k0 + lane, hx, mode, level, kl, ubd, big_row, q, dist, vis,
                            nxt, ncnt);
          for (int o = 16; o; o >>= 1) cx += __shfl_xor_sync(0xffffffffu, cx, o);
          if (grp == x) c = cx;
        }
      }
      if (mode == 1 && sl == 0 && f0 + grp < ns) ldeg[__ldcg(cur + f0 + grp)] = c;
    }
    cl.sync();
    uint32_t *tmp = cur;
    cur = nxt;
    nxt = tmp;
  }
  if (edges) atomicAdd(bytes, edges * 4ull);
  cl.sync();  // every CTA has read the last counts
}

// The local graph of one query, built by the whole cluster (every thread of
// every CTA calls this).  Same contract and output as build_local_graph in
// prep_core.cuh: returns the local vertex count or UINT32_MAX (too large for
// max_local, a local degree above DMASK, or rows beyond cap_adj); fa[i] gets
// the unpadded local degree of local vertex i and sh.q_local q's local id.
__device__ uint32_t cluster_build_local_graph(
    cg::cluster_group &cl, PrepSh &sh, PrepSh *r0, const DevGraph &g, uint32_t q,
    uint32_t kl, uint32_t ubd, uint16_t *dist, uint32_t *vis, uint32_t *comp, uint32_t *fa,
    uint32_t *fb, uint32_t *ldeg, uint32_t *wpre, uint32_t *lgid, uint16_t *ldist, uint32_t *loff,
    uint32_t *ladj, unsigned long long cap_adj, uint32_t max_local, uint32_t big_row,
    unsigned long long *bytes) {
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
  const uint32_t R = cl.num_blocks(), r = cl.block_rank();
  const uint32_t gt = r * PREP_THREADS + t, gstride = R * PREP_THREADS;
  const uint32_t gw = r * PREP_WARPS + wid, gwstride = R * PREP_WARPS;
  const uint32_t n = g.n, nw = (n + 31) / 32;
  for (uint32_t i = gt; i < n; i += gstride) dist[i] = (uint16_t)INF16;
  for (uint32_t i = gt; i < nw; i += gstride) {
    vis[i] = 0;
    comp[i] = 0;
  }
  cl.sync();
  // 1. bounded BFS over the whole graph; 2. q's component in the kept set
  cluster_bfs(cl, sh, r0, g, q, 0, ubd, kl, ubd, big_row, dist, vis, fa, fb, nullptr, bytes);
  // the component BFS also counts each component vertex's local degree
  cluster_bfs(cl, sh, r0, g, q, 1, 0, kl, ubd, big_row, dist, comp, fa, fb, ldeg, bytes);
  // 3. local ids: exclusive prefix of per-word popcounts
  for (uint32_t i = gt; i < nw; i += gstride) wpre[i] = __popc(__ldcg(comp + i));
  if (r == 0 && t == 0) {
    sh.nbig = 0;
    sh.flag = 0;
  }
  cl.sync();
  const uint32_t nl = cluster_excl_scan(cl, sh, wpre, nw);
  if (nl > max_local) return UINT32_MAX;
  // 4. gid, distance and local degree (counted by the component BFS) per
  // local id: padded into loff[i], unpadded into fa[i].  Rows of big_row or
  // more entries are listed in fb for whole CTAs to fill.
  for (uint32_t wi = gt; wi < nw; wi += gstride) {
    uint32_t bits = __ldcg(comp + wi), base = __ldcg(wpre + wi);
    while (bits) {
      const uint32_t b = __ffs(bits) - 1;
      bits &= bits - 1;
      const uint32_t v = wi * 32 + b;
      lgid[base] = v;
      ldist[base] = __ldcg(dist + v);
      const uint32_t c = __ldcg(ldeg + v);
      loff[base] = (c + 3u) & ~3u;
      fa[base] = c;
      if (c > DMASK) atomicOr(&r0->flag, 1u);
      if (g.off[v + 1] - g.off[v] >= big_row) fb[atomicAdd(&r0->nbig, 1u)] = base;
      base++;
    }
  }
  cl.sync();
  const uint32_t nbig = r0->nbig;
  // the search's state words hold in-task degrees in DMASK
  const uint32_t bad = r0->flag;
  cl.sync();
  if (bad) return UINT32_MAX;
  const uint32_t total = cluster_excl_scan(cl, sh, loff, nl);
  if (total > cap_adj) return UINT32_MAX;
  if (r == 0 && t == 0) loff[nl] = total;
  cl.sync();
  // 5. fill rows in ascending order (ordered compaction), pad with SENT
  unsigned long long pbytes = 0;
  for (uint32_t b = r; b < nbig; b += R) {
    const uint32_t i = __ldcg(fb + b), v = __ldcg(lgid + i);
    const uint32_t lo = g.off[v], hi = g.off[v + 1];
    const uint32_t w0 = __ldcg(loff + i);
    uint32_t wpos = 0;
    for (uint32_t b0 = lo; b0 < hi; b0 += PREP_THREADS) {
      const uint32_t k = b0 + t;
      uint32_t w = 0;
      bool in = false;
      if (k < hi) {
        w = g.adj[k];
        in = bit_cg(comp, w);
      }
      const unsigned m = __ballot_sync(0xffffffffu, in);
      if (lane == 0) sh.warp[wid] = __popc(m);
      __syncthreads();
      uint32_t pre = 0, tot = 0;
#pragma unroll
      for (int x = 0; x < PREP_WARPS; x++) {
        const uint32_t cw = sh.warp[x];
        pre += x < wid ? cw : 0u;
        tot += cw;
      }
      if (in) ladj[w0 + wpos + pre + __popc(m & lane_lt())] = local_id_cg(comp, wpre, w);
      wpos += tot;
      __syncthreads();
    }
    const uint32_t padded = __ldcg(loff + i + 1) - w0;
    for (uint32_t k = wpos + t; k < padded; k += PREP_THREADS) ladj[w0 + k] = SENT;
    if (t == 0) pbytes += 4ull * (hi - lo) + 4ull * padded + 12ull;
  }
  for (uint32_t i0 = gw * 4u; i0 < nl; i0 += gwstride * 4u) {
    // four rows per warp as in the count above; long rows were filled above
    const uint32_t grp = lane >> 3, sl = lane & 7, i = i0 + grp;
    uint32_t lo = 0, hi = 0, w0 = 0, padded = 0;
    bool mine = false;
    if (i < nl) {
      const uint32_t v = __ldcg(lgid + i);
      lo = g.off[v];
      hi = g.off[v + 1];
      mine = hi - lo < big_row;
      if (!mine) {
        hi = lo;
      } else {
        w0 = __ldcg(loff + i);
        padded = __ldcg(loff + i + 1) - w0;
      }
    }
    uint32_t len = hi - lo;
    for (int o = 8; o < 32; o <<= 1) len = max(len, __shfl_xor_sync(0xffffffffu, len, o));
    if (len <= GROUP_ROW) {
      uint32_t wpos = 0;
      for (uint32_t k0 = 0; k0 < len; k0 += 8) {
        const uint32_t k = lo + k0 + sl;
        uint32_t w = 0;
        bool in = false;
        if (k < hi) {
          w = g.adj[k];
          in = bit_cg(comp, w);
        }
        const uint32_t gm = (__ballot_sync(0xffffffffu, in) >> (grp * 8u)) & 0xFFu;
        if (in) ladj[w0 + wpos + __popc(gm & ((1u << sl) - 1u))] = local_id_cg(comp, wpre, w);
        wpos += __popc(gm);
      }
      if (mine) {
        for (uint32_t k = wpos + sl; k < padded; k += 8) ladj[w0 + k] = SENT;
        if (sl == 0) pbytes += 4ull * (hi - lo) + 4ull * padded + 12ull;
      }
    } else {
      for (uint32_t x = 0; x < 4; x++) {
        const uint32_t src = x * 8u;
        if (!__shfl_sync(0xffffffffu, (uint32_t)mine, src)) continue;
        const uint32_t lx = __shfl_sync(0xffffffffu, lo, src);
        const uint32_t hx = __shfl_sync(0xffffffffu, hi, src);
        const uint32_t wx = __shfl_sync(0xffffffffu, w0, src);
        const uint32_t px = __shfl_sync(0xffffffffu, padded, src);
        uint32_t wpos = 0;
        for (uint32_t k = lx; k < hx; k += 32) {
          uint32_t w = 0;
          bool in = false;
          if (k + lane < hx) {
            w = g.adj[k + lane];
            in = bit_cg(comp, w);
          }
          const unsigned m = __ballot_sync(0xffffffffu, in);
          if (in) ladj[wx + wpos + __popc(m & lane_lt())] = local_id_cg(comp, wpre, w);
          wpos += __popc(m);
        }
        for (uint32_t k = wpos + lane; k < px; k += 32) ladj[wx + k] = SENT;
        if (lane == 0) pbytes += 4ull * (hx - lx) + 4ull * px + 12ull;
      }
    }
  }
  if (pbytes) atomicAdd(bytes, pbytes);
  if (t == 0) sh.q_local = local_id_cg(comp, wpre, q);
  cl.sync();
  return nl;
}

__global__ void __launch_bounds__(PREP_THREADS)
prep_kernel(DevGraph g, SlotArrays sa, Slot *slots, const PrepJob *jobs,
            int njobs, PrepScratch ps, Pool pool, Counters *ctr) {
  __shared__ PrepSh sh;
  cg::cluster_group cl = cg::this_cluster();
  const uint32_t R = cl.num_blocks(), r = cl.block_rank();
  const int t = threadIdx.x;
  const uint32_t gt = r * PREP_THREADS + t, gstride = R * PREP_THREADS;
  const int jb = (int)(blockIdx.x / R);
  if (jb >= njobs) return;  // the whole cluster
  PrepSh *r0 = cl.map_shared_rank(&sh, 0);
  const PrepJob job = jobs[jb];
  uint16_t *dist = ps.dist + (size_t)jb * ps.stride_n;
  uint32_t *vis = ps.vis + (size_t)jb * ps.stride_w;
  uint32_t *comp = ps.comp + (size_t)jb * ps.stride_w;
  uint32_t *fa = ps.fa + (size_t)jb * ps.stride_n;
  uint32_t *fb = ps.fb + (size_t)jb * ps.stride_n;
  uint32_t *wpre = ps.wpre + (size_t)jb * ps.stride_w;
  uint32_t *ldeg = ps.ldeg + (size_t)jb * ps.stride_n;
  Slot *sl = slots + job.slot;
  uint32_t *loff = sa.loc_off + (size_t)job.slot * (sa.stride_n + 1);
  uint32_t *ladj = sa.loc_adj + (size_t)job.slot * sa.cap_adj;
  uint16_t *ldist = sa.loc_dist + (size_t)job.slot * sa.stride_n;
  uint32_t *lgid = sa.loc_gid + (size_t)job.slot * sa.stride_n;

  const uint32_t nl = cluster_build_local_graph(
      cl, sh, r0, g, job.q, job.kl, job.ubd, dist, vis, comp, fa, fb, ldeg, wpre, lgid, ldist,
      loff, ladj, sa.cap_adj, min(sa.max_local, sa.stride_n), max(ps.big_row, 1u),
      &ctr->prep_bytes);
  if (nl == UINT32_MAX) {
    if (r == 0 && t == 0) {
      sl->status = RS_TOO_LARGE;
      sl->kl = job.kl;  // the answer is the incumbent
      sl->kl_heu = job.kl_heu;
      sl->pending = 0;
      __threadfence();
      sl->state = SLOT_DONE;
      atomicAdd(&ctr->done_count, 1);
    }
    return;
  }
  // 6. root task: C = {q}, R = the rest; dC = [v ~ q], dR = deg - dC
  const uint32_t ql = sh.q_local;
  // mark N(q) in vis (reuse): clear first
  for (uint32_t i = gt; i < (nl + 31) / 32; i += gstride) vis[i] = 0;
  cl.sync();
  {
    const uint32_t lo = __ldcg(loff + ql), hi = __ldcg(loff + ql + 1);
    for (uint32_t k = lo + gt; k < hi; k += gstride) {
      const uint32_t w = __ldcg(ladj + k);
      if (w != SENT) atomicOr(&vis[w >> 5], 1u << (w & 31));
    }
  }
  const uint32_t len = 2 * nl + 5;
  // root_to_pool 1: the root goes to the bump area and is published now;
  // 2: it is parked at the slot's fixed offset (root_off_lo/hi) at the head of
  // the arena and published later by release_kernel.
  const bool parked = job.root_to_pool == 2;
  if (r == 0 && t == 0) {
    unsigned long long off = 0;
    if (parked)
      off = (unsigned long long)job.root_off_lo | ((unsigned long long)job.root_off_hi << 32);
    else if (job.root_to_pool)
      off = atomicAdd(pool.arena_top, (unsigned long long)len);
    sh.root = off;
  }
  cl.sync();
  const unsigned long long roff = r0->root;
  cl.sync();  // rank 0's shared memory is read before anyone can return
  if (job.root_to_pool && roff + len > pool.arena_cap) {
    if (r == 0 && t == 0) {
      sl->status = RS_CAPACITY;
      sl->kl = job.kl;
      sl->pending = 0;
      __threadfence();
      sl->state = SLOT_DONE;
      atomicAdd(&ctr->done_count, 1);
      atomicOr(&ctr->error, ERR_POOL);
    }
    return;
  }
  uint32_t *rec = pool.arena + roff;
  for (uint32_t i = gt; i < nl && job.root_to_pool; i += gstride) {
    const uint32_t dc = (i == ql) ? 0u : ((__ldcg(vis + (i >> 5)) >> (i & 31)) & 1u);
    const uint32_t dr = __ldcg(fa + i) - dc;
    rec[REC_HDR + i] = (i << 1) | (i == ql ? 1u : 0u);
    rec[REC_HDR + nl + i] = (dc << DC_SHIFT) | dr;
  }
  if (r == 0 && t == 0) {
    if (job.root_to_pool) {
      rec[0] = job.slot;
      rec[1] = nl;
      rec[2] = 1;
      rec[3] = len;
      rec[REC_HDR + 2 * nl] = len;
    }
    sl->n_local = nl;
    sl->q_local = ql;
    sl->l = job.l;
    sl->h = job.h;
    sl->limit_doms = job.limit_doms;
    sl->rules = job.rules;
    sl->kl = job.kl;
    sl->kl_heu = job.kl_heu;
    sl->ubd = job.ubd;
    sl->wit_lock = 0;
    sl->wit_val = 0;
    sl->wit_n = 0;
    sl->q_global = job.q;
    sl->qtag = job.qtag;
    sl->abort = 0;
    sl->pending = 1;
    sl->nodes = 0;
    sl->node_budget = job.node_budget;
    sl->status = RS_DONE;
    unsigned long long now;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
    sl->t_admit = now;
    if (job.root_to_pool) {
      if (!parked) atomicAdd(&ctr->pending, 1ull);  // a parked root counts when released
      atomicAdd(&ctr->prep_bytes, 8ull * nl + 20ull);
    } else {
      sl->pending = 0;
    }
  }
  // every thread fences its own stores of the root record and slot fields
  // before the barrier; rank 0's thread 0 then publishes (a fence orders only
  // the calling thread's writes)
  __threadfence();
  cl.sync();
  if (r == 0 && t == 0) {
    sl->state = SLOT_SEARCH;
    if (job.root_to_pool == 1) {
      uint32_t tk = atomicAdd(pool.tail, 1u);
      if (tk < pool.desc_cap) {
        __threadfence();
        atomicExch(&pool.desc[tk], roff + 1ull);
      } else {
        atomicOr(&ctr->error, ERR_POOL);
      }
    }
  }
}

}  // namespace

cudaError_t launch_prep(uint32_t cluster, cudaStream_t stream, DevGraph g,
                        SlotArrays sa, Slot *slots, const PrepJob *jobs,
                        int njobs, PrepScratch ps, Pool pool, Counters *ctr) {
  if (cluster != 1 && cluster != 2 && cluster != 4 && cluster != 8 && cluster != 16)
    return cudaErrorInvalidValue;
  if (njobs <= 0) return cudaSuccess;
  if (cluster > 8) {
    // 16 CTAs is above the portable cluster size: allowed per kernel
    const cudaError_t e =
        cudaFuncSetAttribute(prep_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return e;
  }
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3((unsigned)njobs * cluster);
  cfg.blockDim = dim3(PREP_THREADS);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, prep_kernel, g, sa, slots, jobs, njobs, ps, pool, ctr);
}

// Publish the parked roots of the given slots (one thread; a few per
// slice).  A slot whose preprocessing failed is already done and is skipped.
// The query's task is counted before its descriptor becomes visible.
__global__ void release_kernel(Slot *slots, const uint32_t *cand, uint32_t n,
                               unsigned long long root_stride, Pool pool,
                               Counters *ctr) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  for (uint32_t i = 0; i < n; i++) {
    const uint32_t slot = cand[i];
    Slot *sl = slots + slot;
    if (*(volatile uint32_t *)&sl->state != SLOT_SEARCH) continue;
    unsigned long long now;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
    sl->t_admit = now;  // search time runs from activation
    atomicAdd(&ctr->pending, 1ull);
    const uint32_t tk = atomicAdd(pool.tail, 1u);
    if (tk >= pool.desc_cap) {
      atomicOr(&ctr->error, ERR_POOL);
      continue;
    }
    __threadfence();
    atomicExch(&pool.desc[tk], (unsigned long long)slot * root_stride + 1ull);
  }
}

}  // namespace scs
