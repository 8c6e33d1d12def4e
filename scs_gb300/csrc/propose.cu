// propose.cu -- the learned incumbent proposal.
//
// After a query's local graph is built and before its root task is searched,
// one CTA grows a community from q: at each step the candidates are the
// vertices outside C with a neighbour in C; a shortlist of 16 (the two best
// per warp by connectivity to C) is scored by the network (mlp.cuh) and the
// best one joins C.  Every prefix C of size l..h is a connected community
// containing q; the one with the largest minimum degree is the proposal.
// Its minimum degree is computed exactly here (integer counts), and it
// replaces the incumbent only when it is larger, together with its vertices
// as the query's witness -- the same update the search makes when it finds a
// better community.  The network only decides the order of the growth; the
// degree it reports is the integer method's.
//
// The reference's incumbent is its greedy heuristics on the host
// (CSSC_heu, inc/heuristic.h:321-349, used at main.cu:122-133); the engine
// keeps them (their value is what the reference reports when the search
// finds nothing better) and runs this proposal on top when a model is
// loaded.
#include "scs_device.cuh"

namespace scs {

constexpr int PT = 256;
constexpr int PWARPS = PT / 32;
constexpr uint32_t IN_C = 1u << 31;

__device__ __forceinline__ bool better(float s2, uint32_t i2, float s, uint32_t i) {
  return s2 > s || (s2 == s && i2 < i);
}

struct PropShared {
  uint32_t order[CL_CAP];
  uint32_t sl_id[MLP_TILE];
  float sl_sc[MLP_TILE];
  float feat[MLP_TILE * (MLP_IN + 1)];
  uint32_t red[PWARPS];
  uint32_t pick, best_md, best_size, ok;
};

// One job; all threads of the CTA call it.  cw is this CTA's scratch row
// (zero on entry and on return).
__device__ void propose_one(const DevGraph &g, const SlotArrays &sa, Slot *slots,
                            const PrepJob &job, uint32_t *cw, const MlpDev &M,
                            Counters *ctr, PropShared &S) {
  uint32_t *s_order = S.order, *s_sl_id = S.sl_id, *s_red = S.red;
  float *s_sl_sc = S.sl_sc, *s_feat = S.feat;
  uint32_t &s_pick = S.pick, &s_best_md = S.best_md, &s_best_size = S.best_size, &s_ok = S.ok;
  Slot *sl = slots + job.slot;
  if (*(volatile uint32_t *)&sl->state != SLOT_SEARCH) return;
  const uint32_t n = sl->n_local, q = sl->q_local, l = sl->l, h = sl->h;
  const uint32_t kl0 = *(volatile uint32_t *)&sl->kl;
  if (n == 0 || n > sa.max_local || h >= CL_CAP || q >= n) return;
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
  const uint32_t *off = sa.loc_off + (size_t)job.slot * (sa.stride_n + 1);
  const uint32_t *adj = sa.loc_adj + (size_t)job.slot * sa.cap_adj;
  const uint16_t *dist = sa.loc_dist + (size_t)job.slot * sa.stride_n;
  const uint32_t *gid = sa.loc_gid + (size_t)job.slot * sa.stride_n;
  // per vertex: IN_C | number of neighbours in C (cw, zero on entry)
  if (t == 0) {
    s_best_md = 0;
    s_best_size = 0;
    s_pick = q;
  }
  __syncthreads();
  const uint32_t ku = min(__ldg(g.core + gid[q]), h - 1);
  const float ldm = (float)g.dmax;
  uint32_t csize = 0;
  for (;;) {
    // add s_pick to C
    const uint32_t v = s_pick;
    if (t == 0) {
      atomicOr(cw + v, IN_C);
      s_order[csize] = v;
    }
    for (uint32_t k = off[v] + t; k < off[v + 1]; k += PT) {
      const uint32_t w = adj[k];
      if (w != SENT) atomicAdd(cw + w, 1u);
    }
    csize++;
    __syncthreads();
    if (csize >= l) {
      // minimum degree inside C (exact integer counts)
      uint32_t md = UINT32_MAX;
      for (uint32_t i = t; i < csize; i += PT) md = min(md, cw[s_order[i]] & ~IN_C);
#pragma unroll
      for (int o = 16; o; o >>= 1) md = min(md, __shfl_xor_sync(0xffffffffu, md, o));
      if (lane == 0) s_red[wid] = md;
      __syncthreads();
      if (t == 0) {
        uint32_t m = s_red[0];
        for (int k = 1; k < PWARPS; k++) m = min(m, s_red[k]);
        if (m > s_best_md || s_best_size == 0) {
          s_best_md = m;
          s_best_size = csize;
        }
      }
      __syncthreads();
    }
    if (csize >= h || s_best_md >= ku) break;
    // candidates: outside C with a neighbour in C; per-thread best by
    // connectivity (C neighbours + a fraction for the other neighbours)
    float bs = -1.f;
    uint32_t bi = UINT32_MAX;
    for (uint32_t i = t; i < n; i += PT) {
      const uint32_t w = cw[i];
      if ((w & IN_C) || w == 0) continue;
      const float deg = (float)(off[i + 1] - off[i]);
      const float s = (float)w + (deg - (float)w) / (ldm + 1.f);
      if (better(s, i, bs, bi)) {
        bs = s;
        bi = i;
      }
    }
    // per-warp top two -> shortlist of 16
#pragma unroll
    for (int k = 0; k < 2; k++) {
      float s = bs;
      uint32_t i = bi;
#pragma unroll
      for (int o = 16; o; o >>= 1) {
        const float s2 = __shfl_xor_sync(0xffffffffu, s, o);
        const uint32_t i2 = __shfl_xor_sync(0xffffffffu, i, o);
        if (better(s2, i2, s, i)) {
          s = s2;
          i = i2;
        }
      }
      if (lane == 0) {
        s_sl_id[2 * wid + k] = i;
        s_sl_sc[2 * wid + k] = s;
      }
      if (i != UINT32_MAX && bi == i) {
        bs = -1.f;
        bi = UINT32_MAX;
      }
    }
    __syncthreads();
    if (wid == 0) {
      const uint32_t id = lane < MLP_TILE ? s_sl_id[lane] : UINT32_MAX;
      const float sc = lane < MLP_TILE ? s_sl_sc[lane] : -1.f;
      const unsigned m = __ballot_sync(0xffffffffu, id != UINT32_MAX);
      const uint32_t nsl = __popc(m);
      const uint32_t r = __popc(m & ((1u << lane) - 1u));
      __syncwarp();
      if (id != UINT32_MAX) {
        s_sl_id[r] = id;
        s_sl_sc[r] = sc;
      }
      __syncwarp();
      if (nsl == 0) {
        if (lane == 0) s_pick = UINT32_MAX;
      } else {
        float smax = 0.f;
        uint32_t sbest = UINT32_MAX;
        for (uint32_t j = 0; j < nsl; j++)
          if (better(s_sl_sc[j], s_sl_id[j], smax, sbest)) {
            smax = s_sl_sc[j];
            sbest = s_sl_id[j];
          }
        if (lane < MLP_TILE) {
          float *f = s_feat + lane * (MLP_IN + 1);
          if ((uint32_t)lane < nsl) {
            const uint32_t x = s_sl_id[lane];
            const uint32_t dc = cw[x] & ~IN_C;
            const uint32_t deg = off[x + 1] - off[x];
            FeatIn c;
            c.dC = dc;
            c.dR = deg > dc ? deg - dc : 0;
            c.dist = dist[x];
            c.core = __ldg(g.core + gid[x]);
            c.deg = deg;
            c.score = s_sl_sc[lane];
            c.score_max = smax;
            c.is_best = x == sbest;
            FeatTask k;
            k.s = n;
            k.csize = csize;
            k.n_local = n;
            k.l = l;
            k.h = h;
            k.kl = max(kl0, s_best_md);
            k.ub = ku;
            k.ubd = ubd_dev(k.kl, h);
            k.dmax = g.dmax;
            make_features(c, k, f);
          } else {
#pragma unroll
            for (int j = 0; j < MLP_IN; j++) f[j] = 0.f;
          }
        }
        __syncwarp();
        const float z = mlp_score16(M, s_feat, MLP_IN + 1);
        float bz = (uint32_t)lane < nsl ? z : -INFINITY;
        uint32_t bid = (uint32_t)lane < nsl ? s_sl_id[lane] : UINT32_MAX;
#pragma unroll
        for (int o = 16; o; o >>= 1) {
          const float z2 = __shfl_xor_sync(0xffffffffu, bz, o);
          const uint32_t i2 = __shfl_xor_sync(0xffffffffu, bid, o);
          if (better(z2, i2, bz, bid)) {
            bz = z2;
            bid = i2;
          }
        }
        if (lane == 0) s_pick = bid;
      }
    }
    __syncthreads();
    if (s_pick == UINT32_MAX) break;  // q's component is exhausted
  }
  // the search kernel expects its scratch state words zero between tasks
  __syncthreads();
  for (uint32_t i = t; i < n; i += PT) cw[i] = 0;
  // the proposal replaces the incumbent only when it is better
  if (t == 0) {
    s_ok = 0;
    atomicAdd(&ctr->proposals, 1ull);
    const uint32_t md = s_best_md;
    if (s_best_size >= l && md > kl0) {
      uint32_t spins = 0;
      while (atomicCAS(&sl->wit_lock, 0u, 1u) != 0u) {
        if (++spins > (1u << 22)) break;
        __nanosleep(64);
      }
      if (spins <= (1u << 22)) {
        if (*(volatile uint32_t *)&sl->wit_val < md + 1u)
          s_ok = 1;
        else
          atomicExch(&sl->wit_lock, 0u);
      }
    }
  }
  __syncthreads();
  if (s_ok) {
    uint32_t *wit = sa.witness + (size_t)job.slot * sa.wit_cap;
    for (uint32_t i = t; i < s_best_size; i += PT) wit[i] = gid[s_order[i]];
    __threadfence();
    __syncthreads();
    if (t == 0) {
      sl->wit_n = s_best_size;
      sl->wit_val = s_best_md + 1u;
      atomicMax(&sl->kl, s_best_md);
      atomicAdd(&ctr->proposals_better, 1ull);
      __threadfence();
      atomicExch(&sl->wit_lock, 0u);
    }
  }
  __syncthreads();
}

// Jobs are taken in a grid-stride loop, one CTA each; CTA b uses row b of
// the search CTAs' scratch state words (the grid is at most that many rows).
__global__ void __launch_bounds__(PT)
propose_kernel(DevGraph g, SlotArrays sa, Slot *slots, const PrepJob *jobs, int njobs,
               Scratch scr, MlpDev M, Counters *ctr) {
  __shared__ PropShared S;
  if (!M.w) return;
  uint32_t *cw = scr.word + (size_t)blockIdx.x * scr.stride;
  for (int j = blockIdx.x; j < njobs; j += gridDim.x) {
    const PrepJob job = jobs[j];
    propose_one(g, sa, slots, job, cw, M, ctr, S);
  }
}

}  // namespace scs
