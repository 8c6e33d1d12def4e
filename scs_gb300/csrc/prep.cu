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
#include "prep_core.cuh"

namespace scs {

__global__ void __launch_bounds__(PREP_THREADS)
prep_kernel(DevGraph g, SlotArrays sa, Slot *slots, const PrepJob *jobs,
            int njobs, PrepScratch ps, Pool pool, Counters *ctr) {
  __shared__ uint32_t sh_warp[PREP_WARPS];
  __shared__ uint32_t sh_cnt[4];
  __shared__ unsigned long long sh_root;
  __shared__ uint32_t sh_ql;
  const int t = threadIdx.x;
  const int jb = blockIdx.x;
  if (jb >= njobs) return;
  const PrepJob job = jobs[jb];
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

  const uint32_t nl = build_local_graph(
      g, job.q, job.kl, job.ubd, dist, vis, comp, fa, fb, wpre, lgid, ldist,
      loff, ladj, sa.cap_adj, min(sa.max_local, sa.stride_n), sh_warp, sh_cnt,
      &ctr->prep_bytes, &sh_ql);
  if (nl == UINT32_MAX) {
    if (t == 0) {
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
  const uint32_t ql = sh_ql;
  // mark N(q) in vis (reuse): clear first
  for (uint32_t i = t; i < (nl + 31) / 32; i += PREP_THREADS) vis[i] = 0;
  __syncthreads();
  for (uint32_t k = loff[ql] + t; k < loff[ql + 1]; k += PREP_THREADS) {
    uint32_t w = ladj[k];
    if (w != SENT) atomicOr(&vis[w >> 5], 1u << (w & 31));
  }
  __syncthreads();
  const uint32_t len = 2 * nl + 5;
  // root_to_pool 1: the root goes to the bump area and is published now;
  // 2: it is parked at the slot's fixed offset (root_off_lo/hi) at the head of
  // the arena and published later by release_kernel.
  const bool parked = job.root_to_pool == 2;
  if (t == 0) {
    unsigned long long off = 0;
    if (parked)
      off = (unsigned long long)job.root_off_lo | ((unsigned long long)job.root_off_hi << 32);
    else if (job.root_to_pool)
      off = atomicAdd(pool.arena_top, (unsigned long long)len);
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
    rec[REC_HDR + nl + i] = (dc << DC_SHIFT) | dr;
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
  // before the barrier; thread 0 then publishes (a fence orders only the
  // calling thread's writes)
  __threadfence();
  __syncthreads();
  if (t == 0) {
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
