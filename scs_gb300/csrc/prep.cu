// prep.cu -- per-query preprocessing on the GPU, one CTA per query.
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
// Bitmaps and frontiers live in per-CTA scratch; all scans are block-wide.
#include "scs_device.cuh"

namespace scs {

constexpr int PREP_WARPS = PREP_THREADS / 32;

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t x = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += x;
  }
  return v;
}

// In-place exclusive scan of a[0..len) (global); returns the total.
__device__ uint32_t block_excl_scan(uint32_t *a, uint32_t len,
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

__device__ __forceinline__ bool bit_get(const uint32_t *bm, uint32_t v) {
  return (bm[v >> 5] >> (v & 31)) & 1u;
}

// local id of a vertex whose comp bit is set
__device__ __forceinline__ uint32_t local_id(const uint32_t *comp,
                                             const uint32_t *wpre, uint32_t v) {
  uint32_t w = comp[v >> 5];
  return wpre[v >> 5] + __popc(w & ((1u << (v & 31)) - 1u));
}

// Level-synchronous BFS from q.  mode 0: whole graph, depth <= maxd, writes
// dist; mode 1: only vertices with keep (core > kl && dist <= ubd), any depth,
// marks visited in `vis`.
__device__ void block_bfs(const DevGraph &g, uint32_t q, int mode,
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

__global__ void __launch_bounds__(PREP_THREADS)
prep_kernel(DevGraph g, SlotArrays sa, Slot *slots, const PrepJob *jobs,
            int njobs, PrepScratch ps, Pool pool, Counters *ctr) {
  __shared__ uint32_t sh_warp[PREP_WARPS];
  __shared__ uint32_t sh_cnt[4];
  __shared__ unsigned long long sh_root;
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
  const int jb = blockIdx.x;
  if (jb >= njobs) return;
  const PrepJob job = jobs[jb];
  const uint32_t n = g.n, nw = (n + 31) / 32;
  uint16_t *dist = ps.dist + (size_t)jb * ps.stride_n;
  uint32_t *vis = ps.vis + (size_t)jb * ps.stride_w;
  uint32_t *comp = ps.comp + (size_t)jb * ps.stride_w;
  uint32_t *fa = ps.fa + (size_t)jb * ps.stride_n;
  uint32_t *fb = ps.fb + (size_t)jb * ps.stride_n;
  uint32_t *wpre = ps.wpre + (size_t)jb * ps.stride_w;
  Slot *sl = slots + job.slot;
  uint32_t *loff = sa.loc_off + (size_t)job.slot * (sa.stride_n + 1);
  uint32_t *ladj = sa.loc_adj + (size_t)job.slot * sa.cap_adj;
  uint16_t *ldist = sa.loc_dist + (size_t)job.slot * sa.stride_n;
  uint32_t *lgid = sa.loc_gid + (size_t)job.slot * sa.stride_n;

  for (uint32_t i = t; i < n; i += PREP_THREADS) dist[i] = (uint16_t)INF16;
  for (uint32_t i = t; i < nw; i += PREP_THREADS) {
    vis[i] = 0;
    comp[i] = 0;
  }
  __syncthreads();
  // 1. bounded BFS over the whole graph
  block_bfs(g, job.q, 0, job.ubd, job.kl, job.ubd, dist, vis, fa, fb, sh_cnt,
            &ctr->prep_bytes);
  __syncthreads();
  // 2. q's component inside the kept set
  block_bfs(g, job.q, 1, 0, job.kl, job.ubd, dist, comp, fa, fb, sh_cnt,
            &ctr->prep_bytes);
  __syncthreads();
  // 3. local ids: exclusive prefix of per-word popcounts
  for (uint32_t i = t; i < nw; i += PREP_THREADS) wpre[i] = __popc(comp[i]);
  __syncthreads();
  uint32_t nl = block_excl_scan(wpre, nw, sh_warp);
  __syncthreads();
  if (nl > MAX_LOCAL || nl > sa.stride_n) {
    if (t == 0) {
      sl->n_local = nl;
      sl->status = RS_TOO_LARGE;
      sl->pending = 0;
      __threadfence();
      sl->state = SLOT_DONE;
      uint32_t k = atomicAdd(&ctr->done_count, 1);
      (void)k;
    }
    return;
  }
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
  __syncthreads();
  for (uint32_t i = wid; i < nl; i += PREP_WARPS) {
    uint32_t v = lgid[i];
    uint32_t b = g.off[v], e = g.off[v + 1], c = 0;
    for (uint32_t k = b + lane; k < e; k += 32)
      c += bit_get(comp, g.adj[k]) ? 1u : 0u;
    for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if (lane == 0) loff[i] = (c + 3u) & ~3u;
    if (lane == 0) fa[i] = c;  // unpadded local degree
  }
  __syncthreads();
  uint32_t total = block_excl_scan(loff, nl, sh_warp);
  if (t == 0) loff[nl] = total;
  __syncthreads();
  if (total > sa.cap_adj) {  // cannot happen: cap_adj >= nnz + 3n
    if (t == 0) {
      sl->status = RS_TOO_LARGE;
      sl->pending = 0;
      __threadfence();
      sl->state = SLOT_DONE;
      atomicAdd(&ctr->done_count, 1);
    }
    return;
  }
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
  if (lane == 0 && pbytes) atomicAdd(&ctr->prep_bytes, pbytes);
  __syncthreads();
  // 6. root task: C = {q}, R = the rest; dC = [v ~ q], dR = deg - dC
  const uint32_t ql = local_id(comp, wpre, job.q);
  // mark N(q) in vis (reuse): clear first
  for (uint32_t i = t; i < (nl + 31) / 32; i += PREP_THREADS) vis[i] = 0;
  __syncthreads();
  for (uint32_t k = loff[ql] + t; k < loff[ql + 1]; k += PREP_THREADS) {
    uint32_t w = ladj[k];
    if (w != SENT) atomicOr(&vis[w >> 5], 1u << (w & 31));
  }
  __syncthreads();
  const uint32_t len = 2 * nl + 5;
  if (t == 0) {
    unsigned long long off = 0;
    if (job.root_to_pool) off = atomicAdd(pool.arena_top, (unsigned long long)len);
    sh_root = off;
  }
  __syncthreads();
  unsigned long long roff = sh_root;
  if (job.root_to_pool && roff + len > pool.arena_cap) {
    if (t == 0) {
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
  for (uint32_t i = t; i < nl && job.root_to_pool; i += PREP_THREADS) {
    uint32_t dc = (i == ql) ? 0u : ((vis[i >> 5] >> (i & 31)) & 1u);
    uint32_t dr = fa[i] - dc;
    rec[REC_HDR + i] = (i << 1) | (i == ql ? 1u : 0u);
    rec[REC_HDR + nl + i] = (dc << 16) | dr;
  }
  if (t == 0) {
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
    sl->abort = 0;
    sl->pending = 1;
    sl->nodes = 0;
    sl->node_budget = job.node_budget;
    sl->status = RS_DONE;
    unsigned long long now;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
    sl->t_admit = now;
    if (job.root_to_pool) {
      atomicAdd(&ctr->pending, 1ull);
      atomicAdd(&ctr->prep_bytes, 8ull * nl + 20ull);
    } else {
      sl->pending = 0;
    }
  }
  __syncthreads();
  __threadfence();
  if (t == 0) {
    sl->state = SLOT_SEARCH;
    if (job.root_to_pool) {
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

}  // namespace scs
