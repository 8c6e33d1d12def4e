// bnb.cu -- branch-and-bound search, one CTA per task.
//
// One step on a task (C, R) restates the reference's per-task pipeline:
//   ProcessTask       src/helpers.cc:371-542  (min degree + incumbent,
//                     rule 3, rules 1/2, bounds P1/P2, ustar)
//   calculateMinimumDegree :893-930, reductionRule3 :932-968,
//   reductionRule1and2 :970-1028, calculateUpperBoundDegree :1030-1102,
//   selectUstar :1104-1168, FindDoms :545-670, Expand/writeTasks/
//   writeDomTasks :673-857, :1171-1391.
// The step is deterministic and identical to the CPU oracle's orc_step
// (rules 3 and 1/2 applied to a fixpoint in synchronous rounds, ties to the
// lowest local id, dominance inside the task, sequential score sums in
// ascending neighbour order).
//
// GB300 mapping: the per-vertex state word (status | dC | dR) of the task's
// query lives in shared memory, indexed by local vertex id; task records carry
// dC/dR so loading a task is one coalesced pass; adjacency rows are read
// with 16-byte loads; children are derived from the adjacency of u* and the
// dominated vertices only; the Include child continues in place (depth-first
// dive), the others go to the CTA's own LIFO stack in HBM, and the oldest
// stack entry is donated to a shared pool when other CTAs are idle.  Every
// spin-wait has an iteration bound and reports through Counters::error.
#include "mlp.cuh"
#include "scs_device.cuh"

namespace scs {

constexpr int BT = SEARCH_THREADS;

// implementation switches (both variants are exact; chosen by measurement)
#ifndef SCS_R12_BALANCED
#define SCS_R12_BALANCED 0
#endif
#ifndef SCS_MASK_SCORES
#define SCS_MASK_SCORES 1
#endif
#ifndef SCS_R12_RECOUNT
#define SCS_R12_RECOUNT 1
#endif
// list passes (rule-1/2 checks, ustar candidates): entries per thread whose
// loads are issued together
#ifndef SCS_LIST_UNROLL
#define SCS_LIST_UNROLL 4
#endif
// the same when writing a step's children (one pass writes all of them)
#ifndef SCS_CHILD_UNROLL
#define SCS_CHILD_UNROLL 8
#endif
// rule-1/2 removals: rows cut into chunks of this many words, 32 rows per
// warp batch (0: short rows per thread, long rows per warp).  16 measured
// 1.2 % above 32 on the bench once most row reads hit L2.
#ifndef SCS_CHUNK_WORDS
#define SCS_CHUNK_WORDS 16
#endif
static_assert(SCS_CHUNK_WORDS % 4 == 0, "chunks are whole 16-byte groups");
// dominance test: words of a candidate's row one thread checks before a warp
// takes over the rest
#ifndef SCS_LANE_DOM
#define SCS_LANE_DOM 32
#endif
static_assert(SCS_LANE_DOM % 8 == 0, "stage 1 checks whole 8-word groups");
// rows of at most this many words (padding included) are scanned by one
// thread in rule-1/2 removals and recounts; longer rows by a warp
#ifndef SCS_LANE_ROW
#define SCS_LANE_ROW 128
#endif
#ifndef SCS_ROW_UNROLL
#define SCS_ROW_UNROLL 8
#endif
// ustar argmax pass: candidates per thread whose loads are issued together
// (2 measured 0.5 % above 1 on the bench; 4 adds spills and loses it)
#ifndef SCS_ARGMAX_UNROLL
#define SCS_ARGMAX_UNROLL 2
#endif
constexpr int NWARP = BT / 32;

// What the four sub-phase counters of scs_profile measure (they cost a few
// per cent, so the default build leaves them at zero):
// 0 nothing,
// 1 rule-1/2 sub-phases (check passes, removal rounds, recount rounds;
//   removed vertices and recount rounds),
// 2 step cycles by task size at entry (s < 512, s < 4096, larger; step
//   counts of the first two buckets),
// 3 ustar sub-phases (candidate collection, score push, argmax; summed |C|
//   and candidate counts),
// 4 as 0, but the phase cycles count only steps on tasks of fewer than 512
//   entries,
// 5 dominated-vertex sub-phases (marking N(u*) + test stage 1, test stage
//   2, the rest up to the child marks; candidates passing the prefilters and
//   candidates reaching stage 2).
#ifndef SCS_PROF_MODE
#define SCS_PROF_MODE 0
#endif
constexpr bool PROF_R12 = SCS_PROF_MODE == 1;

struct Sh {
  uint32_t slot, s, csize, n_local, l, h, ldoms, rules, kl, q_local, dmax;
  uint32_t outcome;  // 0 branched, 1 size, 2 bound, 3 no ustar / small
  uint32_t best;     // best min degree evaluated this step
  uint32_t cnt[4];
  uint32_t p1, p2, nR;
  uint32_t ustar, us_idx;
  uint32_t ndoms, ndom_cand;
  uint32_t masked;  // this step's scores came from C-neighbour masks
  uint32_t bad_rec;  // load_record met an entry id outside the local graph
  uint32_t doms[MAX_DOMS];
  uint32_t doms_idx[MAX_DOMS];
  uint32_t wit_pending;
  uint32_t bt;
  unsigned long long bytes;  // algorithmic bytes accumulated by this CTA
  unsigned long long ph[8];  // clock cycles per phase (thread 0)
  unsigned long long t_ph;   // start of the current phase
  unsigned long long r12, r3;
  unsigned long long sub[4];   // rule12: check passes, removal scans, compaction, -
  unsigned long long cnt4[4];  // removed vertices, removed row words, survivors, -
  float mean_deg;            // local CSR entries per local vertex (this query)
  int have;
  int prof_small;  // profile mode 4: this step's task has < 512 entries
  int stop;
  unsigned long long rec;
  uint32_t red_u[NWARP];
  uint32_t red_u2[NWARP];
  uint32_t red4[SCS_LIST_UNROLL * NWARP];  // per-row warp counts (compaction)
  double red_d[NWARP];
  uint32_t cl[CL_CAP];
  uint32_t A[CL_CAP];
  uint32_t B[CL_CAP];
  uint32_t hist[CL_CAP + 1];
  double wtab[64];   // 1/dC of the r-th smallest C vertex (ustar terms)
  uint32_t stride;   // per-CTA scratch stride (words)
  uint32_t kid_len[MAX_DOMS + 2];
  unsigned long long kid_dst[MAX_DOMS + 2];
  unsigned long long kid_pool[MAX_DOMS + 2];
  // learned branching (mlp.cuh): lrn bit 0 = the network picks u* among the
  // shortlist, bit 1 = this step's shortlist goes to the trace
  uint32_t lrn;
  uint32_t nsl;      // shortlisted candidates (<= 16)
  uint32_t nstep;    // steps this CTA ran (trace sampling)
  uint32_t qtag;     // the query's tag (trace key)
  uint32_t sl_id[MLP_TILE], sl_pos[MLP_TILE];
  double sl_sc[MLP_TILE];
  float feat[MLP_TILE * (MLP_IN + 1)];
};

__device__ __forceinline__ uint32_t st_of(uint32_t w) { return w >> 30; }
__device__ __forceinline__ uint32_t dc_of(uint32_t w) { return (w >> DC_SHIFT) & DCMASK; }
__device__ __forceinline__ uint32_t dr_of(uint32_t w) { return w & DMASK; }
__device__ __forceinline__ bool live(uint32_t w) {
  uint32_t s = w >> 30;
  return s == ST_R || s == ST_C;
}

__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ uint32_t warp_min(uint32_t v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ uint32_t warp_sum(uint32_t v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ uint32_t block_min(uint32_t v, Sh &sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  v = warp_min(v);
  if (lane == 0) sh.red_u[wid] = v;
  __syncthreads();
  uint32_t r = UINT32_MAX;
  for (int i = 0; i < NWARP; i++) r = min(r, sh.red_u[i]);
  __syncthreads();
  return r;
}

__device__ uint32_t block_sum(uint32_t v, Sh &sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  v = warp_sum(v);
  if (lane == 0) sh.red_u[wid] = v;
  __syncthreads();
  uint32_t r = 0;
  for (int i = 0; i < NWARP; i++) r += sh.red_u[i];
  __syncthreads();
  return r;
}

// max score, ties to the smaller id; returns via sh.red_d[0]/sh.red_u[0]
__device__ void block_argmax(double sc, uint32_t id, Sh &sh, double &osc,
                             uint32_t &oid) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    double s2 = __shfl_xor_sync(0xffffffffu, sc, o);
    uint32_t i2 = __shfl_xor_sync(0xffffffffu, id, o);
    if (s2 > sc || (s2 == sc && i2 < id)) {
      sc = s2;
      id = i2;
    }
  }
  if (lane == 0) {
    sh.red_d[wid] = sc;
    sh.red_u2[wid] = id;
  }
  __syncthreads();
  double bs = sh.red_d[0];
  uint32_t bi = sh.red_u2[0];
  for (int i = 1; i < NWARP; i++) {
    double s2 = sh.red_d[i];
    uint32_t i2 = sh.red_u2[i];
    if (s2 > bs || (s2 == bs && i2 < bi)) {
      bs = s2;
      bi = i2;
    }
  }
  __syncthreads();
  osc = bs;
  oid = bi;
}

// Append `want` lanes' values to tmp[] with a shared counter.
__device__ __forceinline__ void warp_append(bool want, uint32_t val,
                                            uint32_t *cnt, uint32_t *dst) {
  const int lane = threadIdx.x & 31;
  unsigned m = __ballot_sync(0xffffffffu, want);
  if (!m) return;
  uint32_t base = 0;
  if (lane == __ffs(m) - 1) base = atomicAdd(cnt, __popc(m));
  base = __shfl_sync(0xffffffffu, base, __ffs(m) - 1);
  if (want) dst[base + __popc(m & ((1u << lane) - 1u))] = val;
}

// The same, appending a pair (val to dst, val2 to dst2 at the same index).
__device__ __forceinline__ void warp_append2(bool want, uint32_t val, uint32_t val2,
                                             uint32_t *cnt, uint32_t *dst, uint32_t *dst2) {
  const int lane = threadIdx.x & 31;
  unsigned m = __ballot_sync(0xffffffffu, want);
  if (!m) return;
  uint32_t base = 0;
  if (lane == __ffs(m) - 1) base = atomicAdd(cnt, __popc(m));
  base = __shfl_sync(0xffffffffu, base, __ffs(m) - 1);
  if (want) {
    const uint32_t o = base + __popc(m & ((1u << lane) - 1u));
    dst[o] = val;
    dst2[o] = val2;
  }
}

__device__ __forceinline__ void phase_mark(Sh &sh, int which) {
  // thread 0 only: charge the cycles since the last mark to phase `which`
  if (threadIdx.x == 0) {
    unsigned long long now = clock64();
    if (SCS_PROF_MODE != 4 || sh.prof_small) sh.ph[which] += now - sh.t_ph;
    sh.t_ph = now;
  }
}

// In-place exclusive scan of a[0..len) (any memory); writes the total to
// a[len] and returns it.  All threads call.
__device__ uint32_t block_excl_scan_bt(uint32_t *a, uint32_t len, Sh &sh);

struct Task {
  uint32_t *W;
  uint32_t *list;
  uint32_t *list2;  // second buffer for stable compaction
  uint32_t *aux;
  uint32_t *tmp;
  uint32_t *cpos;  // list position of the candidate at the same index of tmp
  double *ssc;   // pushed ustar scores, by local id (zero between uses)
  unsigned long long *cmask;  // C-neighbour masks of the candidates, by local id
  uint32_t *bits;  // N[u*] as a bitmap in shared memory after W (null: aux)
  double *dsc2;  // scores of dominated candidates, by position
  const uint32_t *off;
  const uint32_t *adj;
  const uint16_t *dist;
  const uint32_t *gid;
  uint32_t *witness;
  Slot *slot;
};

__device__ uint32_t block_excl_scan_bt(uint32_t *a, uint32_t len, Sh &sh) {
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
  uint32_t running = 0;
  for (uint32_t base = 0; base < len; base += BT) {
    uint32_t i = base + t;
    uint32_t v = i < len ? a[i] : 0;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) sh.red_u[wid] = x;
    __syncthreads();
    uint32_t woff = 0, tot = 0;
    for (int q = 0; q < NWARP; q++) {
      uint32_t c = sh.red_u[q];
      if (q < wid) woff += c;
      tot += c;
    }
    if (i < len) a[i] = running + woff + x - v;
    running += tot;
    __syncthreads();
  }
  if (t == 0) a[len] = running;
  __syncthreads();
  return running;
}

// Visit the padded adjacency rows of ids[0..cnt) as one flat range of 16-byte
// units split evenly over the CTA's threads (each thread a contiguous range),
// calling f(r, nb) for every neighbour nb != SENT of ids[r].  pre needs
// cnt+1 words of scratch.  All threads call.
template <class F>
__device__ void for_rows_balanced(Task &T, Sh &sh, const uint32_t *ids,
                                  uint32_t cnt, uint32_t *pre, F f) {
  const int t = threadIdx.x;
  for (uint32_t i = t; i < cnt; i += BT) {
    uint32_t x = ids[i];
    pre[i] = (T.off[x + 1] - T.off[x]) >> 2;
  }
  __syncthreads();
  const uint32_t total = block_excl_scan_bt(pre, cnt, sh);
  const uint32_t per = (total + BT - 1) / BT;
  uint32_t beg = min(total, t * per), end = min(total, beg + per);
  if (beg < end) {
    // row containing unit beg: last r with pre[r] <= beg
    uint32_t lo = 0, hi = cnt;
    while (hi - lo > 1) {
      uint32_t mid = (lo + hi) >> 1;
      if (pre[mid] <= beg) lo = mid;
      else hi = mid;
    }
    uint32_t r = lo;
    uint32_t row_end = pre[r + 1];
    uint32_t x = ids[r];
    const uint32_t *rowp = T.adj + T.off[x];
    uint32_t rbeg = pre[r];
    for (uint32_t u = beg; u < end; u++) {
      while (u >= row_end) {
        r++;
        row_end = pre[r + 1];
        rbeg = pre[r];
        x = ids[r];
        rowp = T.adj + T.off[x];
      }
      const uint4 q4 = *reinterpret_cast<const uint4 *>(rowp + 4 * (u - rbeg));
      if (q4.x != SENT) f(r, q4.x);
      if (q4.y != SENT) f(r, q4.y);
      if (q4.z != SENT) f(r, q4.z);
      if (q4.w != SENT) f(r, q4.w);
    }
  }
  __syncthreads();
}

// Warp-cooperative scan of one padded adjacency row with SCS_ROW_UNROLL
// independent 128-byte loads in flight (the scans are latency-bound: one load
// at a time left the SMs nearly idle).  f(nb) runs for every nb != SENT.
template <class F>
__device__ __forceinline__ void warp_row_scan(const Task &T, uint32_t x, F f) {
  const int lane = threadIdx.x & 31;
  const uint32_t b = T.off[x], e = T.off[x + 1];
  for (uint32_t k0 = b; k0 < e; k0 += 32 * SCS_ROW_UNROLL) {
    uint32_t nb[SCS_ROW_UNROLL];
#pragma unroll
    for (int j = 0; j < SCS_ROW_UNROLL; j++) {
      uint32_t k = k0 + 32 * j + lane;
      nb[j] = k < e ? T.adj[k] : SENT;
    }
#pragma unroll
    for (int j = 0; j < SCS_ROW_UNROLL; j++)
      if (nb[j] != SENT) f(nb[j]);
  }
}

// Row scans that update memory: pred(nb) is evaluated for all of a thread's
// SCS_ROW_UNROLL neighbours before any apply(nb) runs.  The compiler cannot
// tell that apply's stores miss the next neighbours' state words, so with
// one combined lambda each load waited for the previous update; rows are
// strictly ascending (no repeated neighbour), so hoisting the loads is exact.
template <class P, class A>
__device__ __forceinline__ void warp_row_update(const Task &T, uint32_t x, P pred, A apply) {
  const int lane = threadIdx.x & 31;
  const uint32_t b = T.off[x], e = T.off[x + 1];
  for (uint32_t k0 = b; k0 < e; k0 += 32 * SCS_ROW_UNROLL) {
    uint32_t nb[SCS_ROW_UNROLL];
    bool ok[SCS_ROW_UNROLL];
#pragma unroll
    for (int j = 0; j < SCS_ROW_UNROLL; j++) {
      uint32_t k = k0 + 32 * j + lane;
      nb[j] = k < e ? T.adj[k] : SENT;
    }
#pragma unroll
    for (int j = 0; j < SCS_ROW_UNROLL; j++) ok[j] = nb[j] != SENT && pred(nb[j]);
#pragma unroll
    for (int j = 0; j < SCS_ROW_UNROLL; j++)
      if (ok[j]) apply(nb[j]);
  }
}

template <class P, class A>
__device__ __forceinline__ void block_row_update(const Task &T, uint32_t x, P pred, A apply) {
  const int t = threadIdx.x;
  const uint32_t b = T.off[x], e = T.off[x + 1];
  for (uint32_t k0 = b; k0 < e; k0 += BT * SCS_ROW_UNROLL) {
    uint32_t nb[SCS_ROW_UNROLL];
    bool ok[SCS_ROW_UNROLL];
#pragma unroll
    for (int j = 0; j < SCS_ROW_UNROLL; j++) {
      uint32_t k = k0 + BT * j + t;
      nb[j] = k < e ? T.adj[k] : SENT;
    }
#pragma unroll
    for (int j = 0; j < SCS_ROW_UNROLL; j++) ok[j] = nb[j] != SENT && pred(nb[j]);
#pragma unroll
    for (int j = 0; j < SCS_ROW_UNROLL; j++)
      if (ok[j]) apply(nb[j]);
  }
}

// One thread walks a short padded row [b, e) with 16-byte loads (rows start
// 16-byte aligned and are padded to 4 words), 8 words per iteration; pred
// runs on all 8 before apply, as in warp_row_update.
template <class P, class A>
__device__ __forceinline__ void lane_row_update(const Task &T, uint32_t b, uint32_t e,
                                                P pred, A apply) {
  for (uint32_t k = b; k < e; k += 8) {
    const uint4 q4 = *reinterpret_cast<const uint4 *>(T.adj + k);
    const uint4 r4 = k + 4 < e ? *reinterpret_cast<const uint4 *>(T.adj + k + 4)
                               : make_uint4(SENT, SENT, SENT, SENT);
    const uint32_t nb8[8] = {q4.x, q4.y, q4.z, q4.w, r4.x, r4.y, r4.z, r4.w};
    bool ok[8];
#pragma unroll
    for (int j = 0; j < 8; j++) ok[j] = nb8[j] != SENT && pred(nb8[j]);
#pragma unroll
    for (int j = 0; j < 8; j++)
      if (ok[j]) apply(nb8[j]);
  }
}

// The rows of ids[0..cnt), taken 32 at a time by each warp (one per lane),
// cut into SCS_CHUNK_WORDS-word chunks that the warp's lanes share: a warp
// prefix of the chunk counts and a 5-step shuffle search give each lane its
// row, so every lane keeps SCS_CHUNK_WORDS / 4 16-byte loads in flight
// whatever the row lengths.  pred runs on a chunk's words before apply.
template <class P, class A>
__device__ __forceinline__ void warp_rows_chunked(const Task &T, const uint32_t *ids,
                                                  uint32_t cnt, P pred, A apply) {
  constexpr uint32_t CW = SCS_CHUNK_WORDS > 0 ? SCS_CHUNK_WORDS : 16;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (uint32_t base = wid * 32; base < cnt; base += NWARP * 32) {
    const uint32_t i = base + lane;
    uint32_t b = 0, len = 0;
    if (i < cnt) {
      const uint32_t x = ids[i];
      b = T.off[x];
      len = T.off[x + 1] - b;
    }
    const uint32_t c = (len + CW - 1) / CW;
    uint32_t incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
    const uint32_t excl = incl - c;
    for (uint32_t k0 = 0; k0 < total; k0 += 32) {
      const uint32_t k = k0 + lane;
      uint32_t r = 0;  // last lane whose first chunk is at or before k
#pragma unroll
      for (uint32_t step = 16; step; step >>= 1) {
        const uint32_t e2 = __shfl_sync(0xffffffffu, excl, r + step);
        if (e2 <= k) r += step;
      }
      const uint32_t rb = __shfl_sync(0xffffffffu, b, r);
      const uint32_t rex = __shfl_sync(0xffffffffu, excl, r);
      const uint32_t rlen = __shfl_sync(0xffffffffu, len, r);
      if (k < total) {
        const uint32_t start = rb + (k - rex) * CW, end = min(rb + rlen, start + CW);
        uint32_t nb[CW];
#pragma unroll
        for (uint32_t q = 0; q < CW / 4; q++) {
          const uint4 v = start + 4 * q < end
                              ? *reinterpret_cast<const uint4 *>(T.adj + start + 4 * q)
                              : make_uint4(SENT, SENT, SENT, SENT);
          nb[4 * q] = v.x;
          nb[4 * q + 1] = v.y;
          nb[4 * q + 2] = v.z;
          nb[4 * q + 3] = v.w;
        }
        bool ok[CW];
#pragma unroll
        for (uint32_t j = 0; j < CW; j++) ok[j] = nb[j] != SENT && pred(nb[j]);
#pragma unroll
        for (uint32_t j = 0; j < CW; j++)
          if (ok[j]) apply(nb[j]);
      }
    }
  }
}

// Block-wide scan of one padded row (all threads), SCS_ROW_UNROLL loads in
// flight per thread.
template <class F>
__device__ __forceinline__ void block_row_scan(const Task &T, uint32_t x, F f) {
  const int t = threadIdx.x;
  const uint32_t b = T.off[x], e = T.off[x + 1];
  for (uint32_t k0 = b; k0 < e; k0 += BT * SCS_ROW_UNROLL) {
    uint32_t nb[SCS_ROW_UNROLL];
#pragma unroll
    for (int j = 0; j < SCS_ROW_UNROLL; j++) {
      uint32_t k = k0 + BT * j + t;
      nb[j] = k < e ? T.adj[k] : SENT;
    }
#pragma unroll
    for (int j = 0; j < SCS_ROW_UNROLL; j++)
      if (nb[j] != SENT) f(nb[j]);
  }
}

// ---------------------------------------------------------------------------
// load a record into the state words / live list / C list
// ---------------------------------------------------------------------------
__device__ void load_record(const uint32_t *rec, Task &T, Sh &sh) {
  const int t = threadIdx.x;
  const uint32_t s = sh.s;
  const uint32_t *ent = rec + REC_HDR;
  const uint32_t *deg = rec + REC_HDR + s;
  if (t == 0) {
    sh.cnt[0] = 0;
    sh.bad_rec = 0;
  }
  __syncthreads();
  for (uint32_t i0 = 0; i0 < s; i0 += BT * SCS_LIST_UNROLL) {
    // records may have been written by another SM: read through L2 so no
    // stale L1 line of an earlier neighbour in the arena is used
    uint32_t e[SCS_LIST_UNROLL], dg[SCS_LIST_UNROLL];
#pragma unroll
    for (int j = 0; j < SCS_LIST_UNROLL; j++) {
      const uint32_t i = i0 + BT * j + t;
      e[j] = i < s ? __ldcg(ent + i) : SENT;
      dg[j] = i < s ? __ldcg(deg + i) : 0u;
    }
#pragma unroll
    for (int j = 0; j < SCS_LIST_UNROLL; j++) {
      if (e[j] == SENT) continue;
      const uint32_t i = i0 + BT * j + t;
      const uint32_t id = e[j] >> 1, c = e[j] & 1u;
      if (id >= sh.n_local) {  // never index state with it; the caller stops
        sh.bad_rec = 1;
        continue;
      }
      T.W[id] = ((c ? ST_C : ST_R) << 30) | (dg[j] & (ST_ONE - 1u));  // same field layout
      T.list[i] = id;
      if (c) {
        uint32_t k = atomicAdd(&sh.cnt[0], 1u);
        if (k < CL_CAP) sh.cl[k] = id;
      }
    }
  }
  __syncthreads();
}

__device__ void clear_state(Task &T, Sh &sh) {
  for (uint32_t i = threadIdx.x; i < sh.s; i += BT) T.W[T.list[i]] = 0;
  __syncthreads();
}

// ---------------------------------------------------------------------------
// minimum degree of C and incumbent update (src/helpers.cc:446-455)
// ---------------------------------------------------------------------------
__device__ void eval_mindeg(Task &T, Sh &sh, bool test, uint32_t *t_wit) {
  const int t = threadIdx.x;
  const uint32_t cs = sh.csize;
  // read before block_min's barriers: thread 0 overwrites sh.best below
  const uint32_t best0 = sh.best;
  uint32_t v = UINT32_MAX;
  for (uint32_t i = t; i < cs && i < CL_CAP; i += BT) v = min(v, dc_of(T.W[sh.cl[i]]));
  uint32_t md = block_min(v, sh);
  if (md == UINT32_MAX) return;
  bool improve_step = (best0 == UINT32_MAX || md > best0);
  if (improve_step && t == 0) sh.best = md;
  if (test) {
    if (md > sh.kl && t == 0) sh.kl = md;
    if (improve_step) {
      for (uint32_t i = t; i < cs; i += BT) t_wit[i] = sh.cl[i];
      if (t == 0) t_wit[CL_CAP] = cs;  // count stored past the list
    }
    __syncthreads();
    return;
  }
  // global incumbent + witness (bounded lock).  The slot's incumbent is never
  // below sh.kl (sh.kl only takes values already in the slot), so unless md
  // beats sh.kl the atomic cannot raise it.
  if (t == 0) {
    sh.wit_pending = 0;
    uint32_t old = UINT32_MAX;
    if (md > sh.kl) {
      sh.kl = md;
      old = atomicMax(&T.slot->kl, md);
    }
    if (old < md) {
      uint32_t spins = 0;
      while (atomicCAS(&T.slot->wit_lock, 0u, 1u) != 0u) {
        if (++spins > (1u << 22)) break;
        __nanosleep(64);
      }
      if (spins <= (1u << 22)) {
        if (*(volatile uint32_t *)&T.slot->wit_val < md + 1u)
          sh.wit_pending = 1;
        else
          atomicExch(&T.slot->wit_lock, 0u);
      }
    }
  }
  __syncthreads();
  if (sh.wit_pending) {
    for (uint32_t i = t; i < cs && i < CL_CAP; i += BT) T.witness[i] = T.gid[sh.cl[i]];
    __threadfence();
    __syncthreads();
    if (t == 0) {
      T.slot->wit_n = min(cs, (uint32_t)CL_CAP);
      T.slot->wit_val = md + 1u;  // stored +1 so that 0 means none
      __threadfence();
      atomicExch(&T.slot->wit_lock, 0u);
    }
  }
  __syncthreads();
}


// ---------------------------------------------------------------------------
// rule 3 to a fixpoint: every R neighbour of a C vertex with dC+dR == kl+1
// moves to C (src/helpers.cc:932-968)
// ---------------------------------------------------------------------------
__device__ void rule3(Task &T, Sh &sh) {
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
  for (;;) {
    if (t == 0) sh.cnt[2] = 0;
    __syncthreads();
    const uint32_t kl = sh.kl, cs = min(sh.csize, (uint32_t)CL_CAP);
    for (uint32_t ci = wid; ci < cs; ci += NWARP) {
      uint32_t u = sh.cl[ci];
      uint32_t wu = T.W[u];
      if (dc_of(wu) + dr_of(wu) != kl + 1u || dr_of(wu) == 0) continue;
      uint32_t b = T.off[u], e = T.off[u + 1];
      for (uint32_t k = b; k < e; k += 32) {
        bool want = false;
        uint32_t nb = SENT;
        if (k + lane < e) {
          nb = T.adj[k + lane];
          if (nb != SENT && st_of(T.W[nb]) == ST_R)
            want = atomicExch(&T.aux[nb], 1u) == 0u;
        }
        warp_append(want, nb, &sh.cnt[2], T.tmp);
      }
    }
    __syncthreads();
    const uint32_t np = sh.cnt[2];
    if (t == 0) sh.r3++;
    if (np == 0) break;
    if (sh.csize + np > sh.h) {
      // the task is pruned by size: C only grows here.  The degree updates
      // are skipped (dC is a 9-bit field, valid while |C| <= h); only the
      // size reaches the caller.
      for (uint32_t i = t; i < np; i += BT) T.aux[T.tmp[i]] = 0;
      __syncthreads();
      if (t == 0) sh.csize += np;
      __syncthreads();
      break;
    }
    for (uint32_t i = t; i < np; i += BT) {
      uint32_t x = T.tmp[i];
      T.aux[x] = 0;
      T.W[x] += ST_ONE;  // R -> C
      uint32_t k = sh.csize + i;
      if (k < CL_CAP) sh.cl[k] = x;
    }
    __syncthreads();
    if (t == 0) sh.csize += np;
    for (uint32_t pi = wid; pi < np; pi += NWARP) {
      uint32_t x = T.tmp[pi];
      uint32_t b = T.off[x], e = T.off[x + 1];
      for (uint32_t k = b + lane; k < e; k += 32) {
        uint32_t nb = T.adj[k];
        if (nb != SENT && live(T.W[nb])) atomicAdd(&T.W[nb], DC_ONE - 1u);
      }
    }
    __syncthreads();
    if (sh.csize > sh.h) break;
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// rules 1/2 to a fixpoint (src/helpers.cc:970-1028), then compact the list.
// Synchronous rounds, each a pass over the live entries; the list is
// compacted only when something was removed, and |R| = s - |C| afterwards.
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool r12_violates(uint32_t w, uint32_t dist,
                                             uint32_t rules, uint32_t kl,
                                             uint32_t h, uint32_t cs,
                                             uint32_t ubd) {
  uint32_t dc = dc_of(w), dr = dr_of(w);
  if (rules & R_RED1) {
    uint32_t a = dr + dc, b2 = dc + h - cs - 1u;
    if (min(a, b2) <= kl) return true;
  }
  return (rules & R_RED2) && dist > ubd;
}

// Stable compaction of the live list into the second list buffer, keeping
// entries whose state word satisfies keep(); swaps the buffers.
template <class Keep>
__device__ void compact_list(Task &T, Sh &sh, Keep keep) {
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
  const uint32_t s = sh.s;
  uint32_t out = 0;
  // SCS_LIST_UNROLL rows of BT entries per round, one barrier per round:
  // row j's survivors follow those of rows < j, so the order is kept
  for (uint32_t i0 = 0; i0 < s; i0 += BT * SCS_LIST_UNROLL) {
    uint32_t x[SCS_LIST_UNROLL];
    bool k[SCS_LIST_UNROLL];
    unsigned m[SCS_LIST_UNROLL];
#pragma unroll
    for (int j = 0; j < SCS_LIST_UNROLL; j++) {
      const uint32_t i = i0 + BT * j + t;
      x[j] = i < s ? T.list[i] : SENT;
    }
#pragma unroll
    for (int j = 0; j < SCS_LIST_UNROLL; j++) {
      k[j] = x[j] != SENT && keep(x[j]);
      m[j] = __ballot_sync(0xffffffffu, k[j]);
      if (lane == 0) sh.red4[j * NWARP + wid] = __popc(m[j]);
    }
    __syncthreads();
    uint32_t base = out;
#pragma unroll
    for (int j = 0; j < SCS_LIST_UNROLL; j++) {
      uint32_t before = 0, tot = 0;
      for (int q = 0; q < NWARP; q++) {
        const uint32_t c = sh.red4[j * NWARP + q];
        if (q < wid) before += c;
        tot += c;
      }
      if (k[j]) T.list2[base + before + __popc(m[j] & ((1u << lane) - 1u))] = x[j];
      base += tot;
    }
    out = base;
    __syncthreads();
  }
  uint32_t *tmpp = T.list;
  T.list = T.list2;
  T.list2 = tmpp;
  if (t == 0) sh.s = out;
  __syncthreads();
}

__device__ void rule12(Task &T, Sh &sh, bool test) {
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
  const uint32_t h = sh.h, rules = sh.rules;
  if (t == 0) {
    // algorithmic bytes of this visit: 16 B per entry (vertex, status, dR,
    // dC) plus one pass over the entries' local adjacency, estimated with the
    // query's mean local degree (local CSR entries / local vertices)
    sh.bytes += 16ull * sh.s + (unsigned long long)(4.0f * sh.s * sh.mean_deg);
  }
  uint32_t removed = 0;
  if (rules & (R_RED1 | R_RED2)) {
    for (;;) {
      const uint32_t kl = sh.kl, cs = sh.csize, s = sh.s;
      const uint32_t ubd = ubd_dev(kl, h);
      unsigned long long c0 = clock64();
      if (t == 0) {
        sh.cnt[1] = 0;
        sh.cnt[2] = 0;  // long rows of this round's removals / recounts
      }
      __syncthreads();
      for (uint32_t i0 = 0; i0 < s; i0 += BT * SCS_LIST_UNROLL) {
        uint32_t x[SCS_LIST_UNROLL], w[SCS_LIST_UNROLL], d[SCS_LIST_UNROLL];
#pragma unroll
        for (int j = 0; j < SCS_LIST_UNROLL; j++) {
          const uint32_t i = i0 + BT * j + t;
          x[j] = i < s ? T.list[i] : SENT;
        }
#pragma unroll
        for (int j = 0; j < SCS_LIST_UNROLL; j++) {
          const uint32_t xx = x[j] != SENT ? x[j] : 0u;
          w[j] = T.W[xx];
          d[j] = T.dist[xx];
        }
#pragma unroll
        for (int j = 0; j < SCS_LIST_UNROLL; j++) {
          const bool rm = x[j] != SENT && st_of(w[j]) == ST_R &&
                          r12_violates(w[j], d[j], rules, kl, h, cs, ubd);
          warp_append(rm, x[j], &sh.cnt[1], T.tmp);
        }
      }
      __syncthreads();
      const uint32_t nr = sh.cnt[1];
      if (PROF_R12 && t == 0) sh.sub[0] += clock64() - c0;
      if (nr == 0) break;
      c0 = clock64();
      if (t == 0) {
        sh.r12++;
        if (PROF_R12) {
          sh.cnt4[0] += nr;
          sh.cnt4[2] += s - nr;
        }
      }
      removed += nr;
      for (uint32_t i = t; i < nr; i += BT) T.W[T.tmp[i]] = ST_X << 30;
      __syncthreads();
      if (SCS_R12_RECOUNT && s - nr < nr) {
        // burst: fewer survivors than removals -- recount each survivor's R
        // neighbours (exact, cost sum deg(survivors) < sum deg(removed))
        // Short rows one thread each, long rows a warp each.  Writing W[y]
        // changes only y's dR bits; the other threads read status bits only.
        uint32_t *longs = T.tmp + sh.stride;
        for (uint32_t i0 = 0; i0 < s; i0 += BT) {
          const uint32_t i = i0 + t;
          bool lng = false;
          uint32_t y = 0;
          if (i < s) {
            y = T.list[i];
            const uint32_t wy = T.W[y];
            if (live(wy)) {
              const uint32_t b = T.off[y], e = T.off[y + 1];
              if (e - b > SCS_LANE_ROW) {
                lng = true;
              } else {
                uint32_t c = 0;
                lane_row_update(T, b, e, [&](uint32_t nb) { return st_of(T.W[nb]) == ST_R; },
                                [&](uint32_t) { c++; });
                T.W[y] = (wy & ~DMASK) | c;
              }
            }
          }
          warp_append(lng, y, &sh.cnt[2], longs);
        }
        __syncthreads();
        const uint32_t nl = sh.cnt[2];
        for (uint32_t i = wid; i < nl; i += NWARP) {
          const uint32_t y = longs[i];
          const uint32_t wy = T.W[y];
          uint32_t c = 0;
          warp_row_scan(T, y, [&](uint32_t nb) { c += st_of(T.W[nb]) == ST_R; });
          c = warp_sum(c);
          if (lane == 0) T.W[y] = (wy & ~DMASK) | c;
        }
        __syncthreads();
        if (PROF_R12 && t == 0) {
          sh.sub[2] += clock64() - c0;
          sh.cnt4[1]++;
        }
        continue;
      }
      // neighbours lose one R neighbour each (non-returning reductions)
#if SCS_R12_BALANCED
      for_rows_balanced(T, sh, T.tmp, nr, T.tmp + sh.stride, [&](uint32_t, uint32_t nb) {
        if (live(T.W[nb])) atomicSub(&T.W[nb], 1u);
      });
#else
      if (SCS_CHUNK_WORDS > 0) {
        warp_rows_chunked(T, T.tmp, nr, [&](uint32_t nb) { return live(T.W[nb]); },
                          [&](uint32_t nb) { atomicSub(&T.W[nb], 1u); });
        __syncthreads();
      } else {
        // short rows one thread each (16-byte loads), long rows a warp each
        uint32_t *longs = T.tmp + sh.stride;
        for (uint32_t i0 = 0; i0 < nr; i0 += BT) {
          const uint32_t i = i0 + t;
          bool lng = false;
          uint32_t x = 0;
          if (i < nr) {
            x = T.tmp[i];
            const uint32_t b = T.off[x], e = T.off[x + 1];
            if (e - b > SCS_LANE_ROW)
              lng = true;
            else
              lane_row_update(T, b, e, [&](uint32_t nb) { return live(T.W[nb]); },
                              [&](uint32_t nb) { atomicSub(&T.W[nb], 1u); });
          }
          warp_append(lng, x, &sh.cnt[2], longs);
        }
        __syncthreads();
        const uint32_t nl = sh.cnt[2];
        for (uint32_t ri = wid; ri < nl; ri += NWARP)
          warp_row_update(T, longs[ri], [&](uint32_t nb) { return live(T.W[nb]); },
                          [&](uint32_t nb) { atomicSub(&T.W[nb], 1u); });
        __syncthreads();
      }
#endif
      if (PROF_R12 && t == 0) sh.sub[1] += clock64() - c0;
    }
  }
  unsigned long long c1 = clock64();
  if (removed) {
    compact_list(T, sh, [&](uint32_t x) {
      uint32_t w = T.W[x];
      if (st_of(w) == ST_X) {
        T.W[x] = 0;
        return false;
      }
      return true;
    });
  }
  if (t == 0) {
    sh.nR = sh.s - sh.csize;
    if (PROF_R12) sh.sub[3] += clock64() - c1;
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// bounds P1/P2 (src/helpers.cc:1030-1102)
// ---------------------------------------------------------------------------
__device__ void bounds(Task &T, Sh &sh) {
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
  const uint32_t cs = min(sh.csize, (uint32_t)CL_CAP), h = sh.h;
  uint32_t p1 = UINT32_MAX;
  if (sh.rules & R_PRUN1) {
    for (uint32_t i = t; i < cs; i += BT) {
      uint32_t w = T.W[sh.cl[i]];
      uint32_t a = dc_of(w) + h - sh.csize, b = dr_of(w) + dc_of(w);
      p1 = min(p1, min(a, b));
    }
    p1 = block_min(p1, sh);
  }
  uint32_t p2 = UINT32_MAX;
  if (sh.rules & R_PRUN2) {
    for (uint32_t i = t; i <= cs; i += BT) sh.hist[i] = 0;
    __syncthreads();
    // Most R vertices fall into a few low bins: lanes with the same bin add
    // once through their leader.
    for (uint32_t i0 = 0; i0 < sh.s; i0 += BT * SCS_LIST_UNROLL) {
      uint32_t x[SCS_LIST_UNROLL], w[SCS_LIST_UNROLL];
#pragma unroll
      for (int j = 0; j < SCS_LIST_UNROLL; j++) {
        const uint32_t i = i0 + BT * j + t;
        x[j] = i < sh.s ? T.list[i] : SENT;
      }
#pragma unroll
      for (int j = 0; j < SCS_LIST_UNROLL; j++) w[j] = T.W[x[j] != SENT ? x[j] : 0u];
#pragma unroll
      for (int j = 0; j < SCS_LIST_UNROLL; j++) {
        const bool r = x[j] != SENT && st_of(w[j]) == ST_R;
        const uint32_t bin = r ? min(dc_of(w[j]), cs) : UINT32_MAX;
        const unsigned grp = __match_any_sync(0xffffffffu, bin);
        if (r && lane == __ffs(grp) - 1) atomicAdd(&sh.hist[bin], (uint32_t)__popc(grp));
      }
    }
    // rank sort of C degrees into A (ascending)
    for (uint32_t i = t; i < cs; i += BT) {
      uint32_t vi = dc_of(T.W[sh.cl[i]]), r = 0;
      for (uint32_t j = 0; j < cs; j++) {
        uint32_t vj = dc_of(T.W[sh.cl[j]]);
        r += (vj < vi) || (vj == vi && j < i);
      }
      sh.A[r] = vi;
    }
    __syncthreads();
    if (t == 0) {  // B: the top min(h-|C|, |R|) R degrees, descending
      uint32_t want = min(h - sh.csize, sh.nR), nb = 0;
      for (int v = (int)cs; v >= 0 && nb < want; v--) {
        uint32_t c = sh.hist[v];
        while (c-- && nb < want) sh.B[nb++] = (uint32_t)v;
      }
      sh.cnt[3] = nb;
    }
    __syncthreads();
    if (wid == 0) {
      const uint32_t nb = sh.cnt[3];
      for (uint32_t it = 0; it < nb; it++) {
        uint32_t k = min(sh.B[it], cs);
        if (k == 0) break;
        uint32_t v = sh.A[k - 1];
        uint32_t lt = 0, le = 0;
        for (uint32_t i = lane; i < cs; i += 32) {
          uint32_t a = sh.A[i];
          lt += a < v;
          le += a <= v;
        }
        lt = warp_sum(lt);
        le = warp_sum(le);
        __syncwarp();
        uint32_t bcount = k - lt, c = le - lt;
        for (uint32_t i = lane; i < cs; i += 32) {
          if (i < lt) sh.A[i] += 1u;
          else if (i < lt + c - bcount) sh.A[i] = v;
          else if (i < le) sh.A[i] = v + 1u;
        }
        __syncwarp();
      }
    }
    __syncthreads();
    p2 = cs ? sh.A[0] : UINT32_MAX;
  }
  if (t == 0) {
    sh.p1 = p1;
    sh.p2 = p2;
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// ustar (src/helpers.cc:1104-1168) and dominated vertices (:545-670)
//
// Scores are pushed from C: for each u in C in ascending id order, every R
// neighbour v gets += 1/dC(u) (1.0 when dC(u) == 0) into ssc[v].  Each v
// receives its terms in ascending u order -- the order the oracle sums them
// scanning N(v) -- so the doubles are bit-identical, and the work is
// sum deg(C) instead of sum deg(candidates).  The dominated-vertex score uses
// the same terms except that dC(u) == 0 contributes 0; C stays connected, so
// dC(u) == 0 happens only for |C| == 1 (the root), where that partial sum is
// 0 and ssc is not used for it.
// ---------------------------------------------------------------------------
// Returns true when ssc holds C-neighbour masks (summed by choose_ustar)
// instead of scores.
__device__ bool score_candidates(Task &T, Sh &sh) {
  const int t = threadIdx.x;
  const uint32_t cs = min(sh.csize, (uint32_t)CL_CAP);
  // C in ascending id order (rank sort into sh.A)
  for (uint32_t i = t; i < cs; i += BT) {
    uint32_t vi = sh.cl[i], r = 0;
    for (uint32_t j = 0; j < cs; j++) r += sh.cl[j] < vi;
    sh.A[r] = vi;
  }
  __syncthreads();
  if (SCS_MASK_SCORES && cs <= 64) {
    // Every C row at once: candidate v collects a mask of its C neighbours
    // (bit r = r-th smallest C id) with non-returning atomics; the argmax
    // pass then sums the terms in bit order, which is ascending neighbour
    // order, as the oracle does.  The rows are cut into chunks of one warp's
    // SCS_ROW_UNROLL x 32 entries and the warps take chunks round-robin, so
    // one barrier covers all of C.
    constexpr uint32_t CH = 32 * SCS_ROW_UNROLL;
    const int lane = t & 31, wid = t >> 5;
    for (uint32_t r = t; r < cs; r += BT) {
      const uint32_t u = sh.A[r];
      const uint32_t dc = dc_of(T.W[u]);
      sh.wtab[r] = dc ? __ddiv_rn(1.0, (double)dc) : 1.0;
      const uint32_t b = T.off[u], e = T.off[u + 1];
      sh.hist[r] = b;
      sh.hist[64 + r] = e;
      sh.B[r] = (e - b + CH - 1) / CH;
    }
    __syncthreads();
    if (wid == 0) {  // exclusive prefix of the chunk counts, two per lane
      const uint32_t a = 2 * lane < cs ? sh.B[2 * lane] : 0;
      const uint32_t c = 2 * lane + 1 < cs ? sh.B[2 * lane + 1] : 0;
      uint32_t x = a + c;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
      }
      const uint32_t ex = x - a - c;
      __syncwarp();
      if (2 * lane < cs) sh.B[2 * lane] = ex;
      if (2 * lane + 1 < cs) sh.B[2 * lane + 1] = ex + a;
      if (lane == 31) sh.B[64] = x;
    }
    __syncthreads();
    const uint32_t total = sh.B[64];
    unsigned long long *mask = reinterpret_cast<unsigned long long *>(T.ssc);
    for (uint32_t c = wid; c < total; c += NWARP) {
      uint32_t lo = 0, hi = cs;  // row of chunk c: last r with B[r] <= c
      while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (sh.B[mid] <= c) lo = mid;
        else hi = mid;
      }
      const uint32_t k0 = sh.hist[lo] + (c - sh.B[lo]) * CH, e = sh.hist[64 + lo];
      uint32_t nb[SCS_ROW_UNROLL];
      bool ok[SCS_ROW_UNROLL];
#pragma unroll
      for (int j = 0; j < SCS_ROW_UNROLL; j++) {
        const uint32_t k = k0 + 32 * j + lane;
        nb[j] = k < e ? T.adj[k] : SENT;
      }
#pragma unroll
      for (int j = 0; j < SCS_ROW_UNROLL; j++)
        ok[j] = nb[j] != SENT && st_of(T.W[nb[j]]) == ST_R;
#pragma unroll
      for (int j = 0; j < SCS_ROW_UNROLL; j++)
        if (ok[j]) atomicOr(&mask[nb[j]], 1ull << lo);
    }
    __syncthreads();
    return true;
  }
  for (uint32_t ci = 0; ci < cs; ci++) {
    const uint32_t u = sh.A[ci];
    const uint32_t dc = dc_of(T.W[u]);
    const double wu = dc ? __ddiv_rn(1.0, (double)dc) : 1.0;
    const uint32_t b = T.off[u], e = T.off[u + 1];
    for (uint32_t k0 = b; k0 < e; k0 += BT * SCS_ROW_UNROLL) {
      uint32_t nb[SCS_ROW_UNROLL];
#pragma unroll
      for (int j = 0; j < SCS_ROW_UNROLL; j++) {
        uint32_t k = k0 + BT * j + t;
        nb[j] = k < e ? T.adj[k] : SENT;
      }
      // all state words, then all scores, then the stores: the neighbours of
      // one row are distinct, so the loads need not wait for earlier stores
      bool ok[SCS_ROW_UNROLL];
      double sv[SCS_ROW_UNROLL];
#pragma unroll
      for (int j = 0; j < SCS_ROW_UNROLL; j++)
        ok[j] = nb[j] != SENT && st_of(T.W[nb[j]]) == ST_R;
#pragma unroll
      for (int j = 0; j < SCS_ROW_UNROLL; j++) sv[j] = ok[j] ? T.ssc[nb[j]] : 0.0;
#pragma unroll
      for (int j = 0; j < SCS_ROW_UNROLL; j++)
        if (ok[j]) T.ssc[nb[j]] = __dadd_rn(sv[j], wu);
    }
    __syncthreads();
  }
  return false;
}

// Shortlist for the network: the two best per-thread candidates of each warp
// (by the reference rule's score, ties to the smaller id), so the rule's own
// u* is always in it.  All threads call; slots without a candidate get
// UINT32_MAX.  sc/id/pos are each thread's best candidate.
static_assert(2 * NWARP == MLP_TILE, "two shortlist places per warp");
__device__ void shortlist(double sc, uint32_t id, uint32_t pos, Sh &sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 2; k++) {
    double s = sc;
    uint32_t i = id;
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      const double s2 = __shfl_xor_sync(0xffffffffu, s, o);
      const uint32_t i2 = __shfl_xor_sync(0xffffffffu, i, o);
      if (s2 > s || (s2 == s && i2 < i)) {
        s = s2;
        i = i2;
      }
    }
    const bool ok = i != UINT32_MAX && s > 0.0;
    const bool mine = ok && id == i;
    const unsigned m = __ballot_sync(0xffffffffu, mine);
    const uint32_t p = __shfl_sync(0xffffffffu, pos, m ? __ffs(m) - 1 : 0);
    if (lane == 0) {
      sh.sl_sc[2 * wid + k] = ok ? s : 0.0;
      sh.sl_id[2 * wid + k] = ok ? i : UINT32_MAX;
      sh.sl_pos[2 * wid + k] = p;
    }
    if (mine) {  // the next round looks for the warp's second best
      sc = 0.0;
      id = UINT32_MAX;
    }
  }
}

// The network's choice of u* among the shortlist (lrn bit 0), and the
// shortlist's trace records (bit 1).  Warp 0 works; all threads call.
// Features follow make_features (mlp.cuh); the choice is the largest
// logit, ties to the smaller local id.  Any shortlisted vertex is an R
// vertex with a C neighbour, which the branching rule accepts as u*.
__device__ void learned_choice(const SearchParams &P, Task &T, Sh &sh) {
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    // compact the shortlist (16 places, empty ones UINT32_MAX)
    const uint32_t id = lane < MLP_TILE ? sh.sl_id[lane] : UINT32_MAX;
    const uint32_t pos = lane < MLP_TILE ? sh.sl_pos[lane] : 0;
    const double sc = lane < MLP_TILE ? sh.sl_sc[lane] : 0.0;
    const unsigned m = __ballot_sync(0xffffffffu, id != UINT32_MAX);
    const uint32_t nsl = __popc(m);
    const uint32_t r = __popc(m & ((1u << lane) - 1u));
    __syncwarp();
    if (id != UINT32_MAX) {
      sh.sl_id[r] = id;
      sh.sl_pos[r] = pos;
      sh.sl_sc[r] = sc;
    }
    __syncwarp();
    const bool score = (sh.lrn & 1u) && nsl >= 2;
    const bool trace = (sh.lrn & 2u) && nsl >= 1;
    const bool tout = (sh.lrn & 4u) != 0;  // one-step test: shortlist out
    if (tout && lane == 0) P.t_sl[(size_t)blockIdx.x * (MLP_TILE + 1)] = nsl;
    if (score || trace || tout) {
      FeatTask k;
      k.s = sh.csize + sh.nR;
      k.csize = sh.csize;
      k.n_local = sh.n_local;
      k.l = sh.l;
      k.h = sh.h;
      k.kl = sh.kl;
      k.ub = min(sh.p1, sh.p2);
      k.ubd = ubd_dev(sh.kl, sh.h);
      k.dmax = sh.dmax;
      // the rule's best score (its u* is the first place of some warp)
      double smax = 0.0;
      for (uint32_t j = 0; j < nsl; j++) smax = fmax(smax, sh.sl_sc[j]);
      if (lane < MLP_TILE) {
        float *f = sh.feat + lane * (MLP_IN + 1);
        if ((uint32_t)lane < nsl) {
          const uint32_t v = sh.sl_id[lane];
          const uint32_t w = T.W[v];
          FeatIn c;
          c.dC = dc_of(w);
          c.dR = dr_of(w);
          c.dist = T.dist[v];
          c.core = __ldg(P.g.core + T.gid[v]);
          c.deg = T.off[v + 1] - T.off[v];
          c.score = (float)sh.sl_sc[lane];
          c.score_max = (float)smax;
          c.is_best = v == sh.ustar;
          make_features(c, k, f);
        } else {
#pragma unroll
          for (int j = 0; j < MLP_IN; j++) f[j] = 0.f;
        }
      }
      __syncwarp();
      if (score) {
        const float z = mlp_score16(P.mlp, sh.feat, MLP_IN + 1);
        float bz = (uint32_t)lane < nsl ? z : -INFINITY;
        uint32_t bi = (uint32_t)lane < nsl ? sh.sl_id[lane] : UINT32_MAX;
        uint32_t bp = (uint32_t)lane < nsl ? sh.sl_pos[lane] : 0;
#pragma unroll
        for (int o = 16; o; o >>= 1) {
          const float z2 = __shfl_xor_sync(0xffffffffu, bz, o);
          const uint32_t i2 = __shfl_xor_sync(0xffffffffu, bi, o);
          const uint32_t p2 = __shfl_xor_sync(0xffffffffu, bp, o);
          if (z2 > bz || (z2 == bz && i2 < bi)) {
            bz = z2;
            bi = i2;
            bp = p2;
          }
        }
        if (lane == 0) {
          sh.ustar = bi;
          sh.us_idx = bp;
        }
      }
      if (tout && (uint32_t)lane < nsl) {
        P.t_sl[(size_t)blockIdx.x * (MLP_TILE + 1) + 1 + lane] = sh.sl_id[lane];
        const float *f = sh.feat + lane * (MLP_IN + 1);
        float *dst = P.t_sl_feat + ((size_t)blockIdx.x * MLP_TILE + lane) * MLP_IN;
#pragma unroll
        for (int j = 0; j < MLP_IN; j++) dst[j] = f[j];
      }
      if (trace) {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(P.trace_count, (unsigned long long)nsl);
        base = __shfl_sync(0xffffffffu, base, 0);
        if ((uint32_t)lane < nsl && base + lane < P.trace_cap) {
          const float *f = sh.feat + lane * (MLP_IN + 1);
          float *dst = P.trace_feat + (base + lane) * MLP_IN;
#pragma unroll
          for (int j = 0; j < MLP_IN; j++) dst[j] = f[j];
          P.trace_key[2 * (base + lane)] = sh.qtag;
          P.trace_key[2 * (base + lane) + 1] = T.gid[sh.sl_id[lane]];
        }
      }
    }
  }
  __syncthreads();
}

template <bool LRN>
__device__ void choose_ustar(const SearchParams &P, Task &T, Sh &sh) {
  const int t = threadIdx.x;
  const uint32_t s = sh.s;
  unsigned long long c0 = SCS_PROF_MODE == 3 ? clock64() : 0;
  if (t == 0) sh.cnt[0] = 0;
  __syncthreads();
  for (uint32_t i0 = 0; i0 < s; i0 += BT * SCS_LIST_UNROLL) {
    uint32_t x[SCS_LIST_UNROLL], w[SCS_LIST_UNROLL];
#pragma unroll
    for (int j = 0; j < SCS_LIST_UNROLL; j++) {
      const uint32_t i = i0 + BT * j + t;
      x[j] = i < s ? T.list[i] : SENT;
    }
#pragma unroll
    for (int j = 0; j < SCS_LIST_UNROLL; j++) w[j] = T.W[x[j] != SENT ? x[j] : 0u];
#pragma unroll
    for (int j = 0; j < SCS_LIST_UNROLL; j++) {
      const uint32_t i = i0 + BT * j + t;
      const bool c = x[j] != SENT && st_of(w[j]) == ST_R && dc_of(w[j]) > 0;
      // candidates carry their list position (cpos, same index)
      warp_append2(c, x[j], i, &sh.cnt[0], T.tmp, T.cpos);
    }
  }
  __syncthreads();
  const uint32_t nc = sh.cnt[0];
  if (SCS_PROF_MODE == 3 && t == 0) {
    const unsigned long long c1 = clock64();
    sh.sub[0] += c1 - c0;
    c0 = c1;
    sh.cnt4[0] += min(sh.csize, (uint32_t)CL_CAP);
    sh.cnt4[1] += nc;
  }
  const bool masked = score_candidates(T, sh);
  if (SCS_PROF_MODE == 3 && t == 0) {
    const unsigned long long c1 = clock64();
    sh.sub[1] += c1 - c0;
    c0 = c1;
  }
  const double dmax = (double)sh.dmax;
  double best = 0.0;
  uint32_t bid = UINT32_MAX, bpos = 0;
  // SCS_ARGMAX_UNROLL candidates per thread at a time: their packed ids, then
  // their masks (or scores) and state words, are loaded together
  for (uint32_t c0 = 0; c0 < nc; c0 += BT * SCS_ARGMAX_UNROLL) {
    uint32_t pk[SCS_ARGMAX_UNROLL];
#pragma unroll
    for (int j = 0; j < SCS_ARGMAX_UNROLL; j++) {
      const uint32_t ci = c0 + BT * j + t;
      pk[j] = ci < nc ? T.tmp[ci] : SENT;
    }
    unsigned long long mv[SCS_ARGMAX_UNROLL];
    uint32_t wv[SCS_ARGMAX_UNROLL];
#pragma unroll
    for (int j = 0; j < SCS_ARGMAX_UNROLL; j++) {
      const uint32_t x = pk[j] != SENT ? pk[j] : 0u;
      mv[j] = reinterpret_cast<const unsigned long long *>(T.ssc)[x];
      wv[j] = T.W[x];
    }
#pragma unroll
    for (int j = 0; j < SCS_ARGMAX_UNROLL; j++) {
      if (pk[j] == SENT) continue;
      const uint32_t x = pk[j];
      double sc;
      if (masked) {
        unsigned long long m = mv[j];
        T.cmask[x] = m;  // kept for the dominance prefilter
        sc = 0.0;
        while (m) {
          const int r = __ffsll((long long)m) - 1;
          m &= m - 1;
          sc = __dadd_rn(sc, sh.wtab[r]);
        }
        T.ssc[x] = sc;  // the mask word becomes the pushed score
      } else {
        sc = __longlong_as_double((long long)mv[j]);
      }
      if (sc > 0.0) sc = __dadd_rn(sc, __ddiv_rn((double)dr_of(wv[j]), dmax));
      if (sc > best || (sc == best && sc > 0.0 && x < bid)) {
        best = sc;
        bid = x;
        bpos = T.cpos[c0 + BT * j + t];
      }
    }
  }
  if (LRN && sh.lrn) shortlist(best, bid, bpos, sh);  // read after block_argmax's barriers
  double osc;
  uint32_t oid;
  block_argmax(best, bid, sh, osc, oid);
  if (osc > 0.0 && bid == oid) sh.us_idx = bpos;  // the one thread holding u*
  if (t == 0) {
    sh.ustar = (osc > 0.0) ? oid : UINT32_MAX;
    sh.ndom_cand = nc;
    sh.masked = masked;
    if (SCS_PROF_MODE == 3) sh.sub[2] += clock64() - c0;
  }
  __syncthreads();
  if (LRN && sh.lrn && sh.ustar != UINT32_MAX) learned_choice(P, T, sh);
}

// reset the pushed scores (candidates are exactly the R vertices with C
// neighbours, i.e. every vertex that received a term)
__device__ void clear_scores(Task &T, Sh &sh) {
  for (uint32_t ci = threadIdx.x; ci < sh.ndom_cand; ci += BT) T.ssc[T.tmp[ci]] = 0.0;
  __syncthreads();
}

__device__ void find_doms(Task &T, Sh &sh) {
  const int t = threadIdx.x;
  const uint32_t u = sh.ustar;
  if (t == 0) {
    sh.ndoms = 0;
    sh.cnt[1] = 0;
    sh.cnt[2] = 0;
  }
  __syncthreads();
  if (sh.ldoms == 0) return;
  const uint32_t wu = T.W[u];
  const uint32_t degu = dc_of(wu) + dr_of(wu), dcu = dc_of(wu);
  // mark N_T(u*) and u*
  uint32_t *bits = T.bits;
  auto mark = [&](uint32_t nb) {
    if (bits) atomicOr(&bits[nb >> 5], 1u << (nb & 31));
    else T.aux[nb] = 1u;
  };
  auto marked = [&](uint32_t nb) -> bool {
    return bits ? (bits[nb >> 5] >> (nb & 31)) & 1u : T.aux[nb] != 0u;
  };
  block_row_update(T, u, [&](uint32_t nb) { return live(T.W[nb]); }, mark);
  if (t == 0) mark(u);
  __syncthreads();
  // candidates (R, dC > 0) are in tmp[0..nc); necessary conditions for
  // N_T(v) within N_T(u*)+u*: dC(v) <= dC(u*), deg_T(v) <= deg_T(u*) + 1.
  // One lane per candidate: most candidates fail at their first neighbours,
  // so 32 candidates per warp keep many independent loads in flight.
  const uint32_t nc = sh.ndom_cand;
  const double dmax = (double)sh.dmax;
  const bool root_c = sh.csize <= 1;  // dom partial sum is 0 when |C| == 1
  uint32_t *dom_id = T.tmp + sh.s;  // second half of tmp (s <= n): candidate indices
  // With masks: v's C neighbours must all be neighbours of u* (u* is in R),
  // so mask(v) within mask(u*) is necessary as well.
  const bool use_mask = sh.masked;
  const unsigned long long mu = use_mask ? T.cmask[u] : 0ull;
  auto record = [&](uint32_t ci) {
    const uint32_t x = T.tmp[ci];
    const double part = root_c ? 0.0 : T.ssc[x];
    const double sc = __dadd_rn(part, __ddiv_rn((double)dr_of(T.W[x]), dmax));
    const uint32_t k = atomicAdd(&sh.cnt[1], 1u);
    dom_id[k] = ci;  // the candidate's index (id in tmp, position in cpos)
    T.dsc2[k] = sc;
  };
  // Stage 1, one thread per candidate: the prefilters and the first
  // SCS_LANE_DOM words of the row, where most candidates fail.  Candidates
  // still undecided go to a list (list2 is free here) for stage 2.
  uint32_t *undec = T.list2;
  for (uint32_t i0 = 0; i0 < nc; i0 += BT) {
    const uint32_t ci = i0 + t;
    bool more = false;
    if (ci < nc) {
      const uint32_t x = T.tmp[ci];
      const uint32_t wx = T.W[x];
      bool dom = x != u && dc_of(wx) <= dcu && dc_of(wx) + dr_of(wx) <= degu + 1u &&
                 !(use_mask && (T.cmask[x] & ~mu));
      if (dom) {
        if (SCS_PROF_MODE == 5) atomicAdd(&sh.cnt4[0], 1ull);
        const uint32_t b = T.off[x], e = T.off[x + 1];
        const uint32_t stop = min(e, b + SCS_LANE_DOM);
        for (uint32_t k = b; k < stop && dom; k += 8) {
          const uint4 q4 = *reinterpret_cast<const uint4 *>(T.adj + k);
          const uint4 r4 = k + 4 < e ? *reinterpret_cast<const uint4 *>(T.adj + k + 4)
                                     : make_uint4(SENT, SENT, SENT, SENT);
          const uint32_t nb8[8] = {q4.x, q4.y, q4.z, q4.w, r4.x, r4.y, r4.z, r4.w};
#pragma unroll
          for (int j = 0; j < 8; j++) {
            const uint32_t nb = nb8[j];
            if (nb != SENT && live(T.W[nb]) && !marked(nb)) dom = false;
          }
        }
        if (dom) {
          if (stop < e) more = true;
          else record(ci);
        }
      }
    }
    warp_append(more, ci, &sh.cnt[2], undec);
  }
  __syncthreads();
#if SCS_PROF_MODE == 5
  unsigned long long c5 = clock64();
  if (t == 0) {
    sh.sub[0] += c5 - sh.t_ph;
    sh.cnt4[1] += sh.cnt[2];
  }
#endif
  // Stage 2, one warp per undecided candidate over the rest of its row.
  {
    const int lane = t & 31, wid = t >> 5;
    const uint32_t nu = sh.cnt[2];
    for (uint32_t j = wid; j < nu; j += NWARP) {
      const uint32_t ci = undec[j], x = T.tmp[ci];
      const uint32_t e = T.off[x + 1];
      bool dom = true;
      for (uint32_t k0 = T.off[x] + SCS_LANE_DOM; k0 < e && dom; k0 += 32 * SCS_ROW_UNROLL) {
        uint32_t nb[SCS_ROW_UNROLL];
#pragma unroll
        for (int q = 0; q < SCS_ROW_UNROLL; q++) {
          const uint32_t k = k0 + 32 * q + lane;
          nb[q] = k < e ? T.adj[k] : SENT;
        }
        bool bad = false;
#pragma unroll
        for (int q = 0; q < SCS_ROW_UNROLL; q++)
          bad |= nb[q] != SENT && live(T.W[nb[q]]) && !marked(nb[q]);
        dom = !__any_sync(0xffffffffu, bad);
      }
      if (dom && lane == 0) record(ci);
    }
  }
  __syncthreads();
#if SCS_PROF_MODE == 5
  if (t == 0) sh.sub[1] += clock64() - c5;
#endif
  // clear marks
  if (bits) {
    for (uint32_t i = t; i < (sh.n_local + 31) / 32; i += BT) bits[i] = 0;
  } else {
    block_row_scan(T, u, [&](uint32_t nb) { T.aux[nb] = 0u; });
    if (t == 0) T.aux[u] = 0u;
  }
  __syncthreads();
  const uint32_t nd = sh.cnt[1];
  const uint32_t k = min(nd, min(sh.ldoms, (uint32_t)MAX_DOMS));
  for (uint32_t r = 0; r < k; r++) {
    double bs = -1.0;
    uint32_t bi = UINT32_MAX, bpos = UINT32_MAX, bli = 0;
    for (uint32_t i = t; i < nd; i += BT) {
      double sc = T.dsc2[i];
      const uint32_t ci = dom_id[i], x = T.tmp[ci];
      if (sc > bs || (sc == bs && x < bi)) {
        bs = sc;
        bi = x;
        bpos = i;
        bli = T.cpos[ci];
      }
    }
    double osc;
    uint32_t oid;
    block_argmax(bs, bi, sh, osc, oid);
    if (bi == oid && bpos != UINT32_MAX && bs == osc) {
      T.dsc2[bpos] = -2.0;  // exclude from later rounds
      sh.doms[r] = oid;
      sh.doms_idx[r] = bli;
    }
    __syncthreads();
  }
  if (t == 0) sh.ndoms = k;
  __syncthreads();
}

// ---------------------------------------------------------------------------
// children.  aux[x] bit 0: x ~ u*, bit j+1: x ~ d_j; bits 16..20: rank+1 if
// x == d_rank; bit 21: x == u*.
// child code: 0 = Include, 1..k = Dom_{code-1}, k+1 = Exclude
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool child_skip(uint32_t a, uint32_t code,
                                           uint32_t k) {
  uint32_t rk = (a >> 16) & 31u;  // rank + 1 (0: not a dom)
  bool is_u = (a >> 21) & 1u;
  if (code == k + 1) return is_u || rk;           // Exclude drops u*, D
  if (code == 0) return rk != 0;                  // Include drops D
  return rk != 0 && rk < code;                    // Dom_i drops d_0..d_{i-1}
}

__device__ __forceinline__ void child_entry(uint32_t x, uint32_t w, uint32_t a,
                                            uint32_t code, uint32_t k,
                                            uint32_t &ent, uint32_t &deg) {
  uint32_t rk = (a >> 16) & 31u;
  bool is_u = (a >> 21) & 1u;
  uint32_t dc = dc_of(w), dr = dr_of(w);
  bool inC = st_of(w) == ST_C;
  uint32_t adj_u = a & 1u;
  uint32_t domadj = (a >> 1) & ((1u << k) - 1u);
  if (code == k + 1) {           // Exclude: u*, D removed
    dr -= adj_u + __popc(domadj);
  } else if (code == 0) {        // Include: u* -> C, D removed
    dc += adj_u;
    dr -= adj_u + __popc(domadj);
    inC = inC || is_u;
  } else {                       // Dom_i: u*, d_i -> C; d_0..d_{i-1} removed
    uint32_t i = code - 1;
    uint32_t adj_i = (domadj >> i) & 1u;
    uint32_t lower = domadj & ((1u << i) - 1u);
    dc += adj_u + adj_i;
    dr -= adj_u + adj_i + __popc(lower);
    inC = inC || is_u || (rk == i + 1);
  }
  ent = (x << 1) | (inC ? 1u : 0u);
  deg = (dc << DC_SHIFT) | dr;
}

__device__ void mark_children(Task &T, Sh &sh) {
  const int t = threadIdx.x, wid = t >> 5;
  const uint32_t k = sh.ndoms;
  // adjacency bits: warp per marked vertex
  for (uint32_t j = wid; j <= k; j += NWARP) {
    uint32_t v = j == 0 ? sh.ustar : sh.doms[j - 1];
    warp_row_update(T, v, [&](uint32_t nb) { return live(T.W[nb]); },
                    [&](uint32_t nb) { atomicOr(&T.aux[nb], 1u << j); });
  }
  __syncthreads();
  // list positions of u* (us_idx) and the d_j (doms_idx) came with the
  // candidates
  if (t == 0) atomicOr(&T.aux[sh.ustar], 1u << 21);
  if (t < k) atomicOr(&T.aux[sh.doms[t]], (t + 1u) << 16);
  __syncthreads();
}

// Which of u* and the d_j lie before list index i: bit j of the result is
// doms_idx[j] < i, bit 31 us_idx < i.  Computed once per entry for all of
// its children.
__device__ __forceinline__ uint32_t marks_before(const Sh &sh, uint32_t i) {
  const uint32_t k = sh.ndoms;
  uint32_t b = sh.us_idx < i ? 0x80000000u : 0u;
  for (uint32_t j = 0; j < k; j++) b |= (sh.doms_idx[j] < i ? 1u : 0u) << j;
  return b;
}

// Skipped list entries before index i for child `code`, from marks_before's
// bits: Exclude skips u* and every d_j, Include every d_j, Dom_c the d_j with
// j < c - 1
__device__ __forceinline__ uint32_t skipped_from_marks(uint32_t b, uint32_t code,
                                                       uint32_t k) {
  const uint32_t doms = b & 0x7FFFFFFFu;
  if (code == k + 1) return (b >> 31) + __popc(doms);
  if (code == 0) return __popc(doms);
  return __popc(doms & ((1u << (code - 1)) - 1u));
}

__device__ __forceinline__ void child_shape(const Sh &sh, uint32_t code,
                                            uint32_t &s2, uint32_t &c2) {
  const uint32_t k = sh.ndoms;
  if (code == 0) {
    s2 = sh.s - k;
    c2 = sh.csize + 1;
  } else if (code == k + 1) {
    s2 = sh.s - 1 - k;
    c2 = sh.csize;
  } else {
    s2 = sh.s - (code - 1);
    c2 = sh.csize + 2;
  }
}

__device__ __forceinline__ bool child_alive(const Sh &sh, uint32_t s2,
                                            uint32_t c2) {
  return c2 <= sh.h && s2 >= sh.l;
}

// write child `code`: entries to ent[], degrees to deg[]; when rec is not
// null also the record header and footer (ent == rec + REC_HDR, deg == ent+s2)
__device__ void write_child(Task &T, Sh &sh, uint32_t code, uint32_t *ent_dst,
                            uint32_t *deg_dst, uint32_t *rec) {
  const int t = threadIdx.x;
  uint32_t s2, c2;
  child_shape(sh, code, s2, c2);
  const uint32_t s = sh.s, k = sh.ndoms;
  for (uint32_t i = t; i < s; i += BT) {
    uint32_t x = T.list[i];
    uint32_t a = T.aux[x];
    if (child_skip(a, code, k)) continue;
    uint32_t o = i - skipped_from_marks(marks_before(sh, i), code, k);
    uint32_t ent, deg;
    child_entry(x, T.W[x], a, code, k, ent, deg);
    ent_dst[o] = ent;
    deg_dst[o] = deg;
  }
  if (t == 0 && rec) {
    rec[0] = sh.slot;
    rec[1] = s2;
    rec[2] = c2;
    rec[3] = 2 * s2 + 5;
    rec[REC_HDR + 2 * s2] = 2 * s2 + 5;
  }
}

// Write every child code in [code_lo, code_hi] in one pass over the entries:
// dst[code] is the record start (or null when the child is not written).
__device__ void write_children(Task &T, Sh &sh, uint32_t code_lo,
                               uint32_t code_hi, uint32_t *const *dst) {
  const int t = threadIdx.x;
  const uint32_t s = sh.s, k = sh.ndoms;
  for (uint32_t i0 = 0; i0 < s; i0 += BT * SCS_CHILD_UNROLL) {
    uint32_t xs[SCS_CHILD_UNROLL], as[SCS_CHILD_UNROLL], ws[SCS_CHILD_UNROLL];
#pragma unroll
    for (int j = 0; j < SCS_CHILD_UNROLL; j++) {
      const uint32_t i = i0 + BT * j + t;
      xs[j] = i < s ? T.list[i] : SENT;
    }
#pragma unroll
    for (int j = 0; j < SCS_CHILD_UNROLL; j++) {
      const uint32_t xx = xs[j] != SENT ? xs[j] : 0u;
      as[j] = T.aux[xx];
      ws[j] = T.W[xx];
    }
#pragma unroll
    for (int j = 0; j < SCS_CHILD_UNROLL; j++) {
      const uint32_t i = i0 + BT * j + t;
      if (xs[j] == SENT) continue;
      const uint32_t mb = marks_before(sh, i);
      for (uint32_t code = code_lo; code <= code_hi; code++) {
        uint32_t *d = dst[code];
        if (!d || child_skip(as[j], code, k)) continue;
        uint32_t s2, c2;
        child_shape(sh, code, s2, c2);
        uint32_t o = i - skipped_from_marks(mb, code, k);
        uint32_t ent, deg;
        child_entry(xs[j], ws[j], as[j], code, k, ent, deg);
        d[REC_HDR + o] = ent;
        d[REC_HDR + s2 + o] = deg;
      }
    }
  }
  if (t == 0) {
    for (uint32_t code = code_lo; code <= code_hi; code++) {
      uint32_t *d = dst[code];
      if (!d) continue;
      uint32_t s2, c2;
      child_shape(sh, code, s2, c2);
      d[0] = sh.slot;
      d[1] = s2;
      d[2] = c2;
      d[3] = 2 * s2 + 5;
      d[REC_HDR + 2 * s2] = 2 * s2 + 5;
    }
  }
}

// apply the Include child to the in-CTA state (continue depth-first)
__device__ void apply_include(Task &T, Sh &sh) {
  const int t = threadIdx.x;
  const uint32_t s = sh.s, k = sh.ndoms;
  for (uint32_t i = t; i < s; i += BT) {
    uint32_t x = T.list[i];
    uint32_t a = T.aux[x];
    uint32_t rk = (a >> 16) & 31u;
    if (rk) {
      T.W[x] = 0;
    } else {
      uint32_t adj_u = a & 1u;
      uint32_t domadj = (a >> 1) & ((1u << k) - 1u);
      uint32_t w = T.W[x];
      w += adj_u * DC_ONE;
      w -= adj_u + __popc(domadj);
      if ((a >> 21) & 1u) w += ST_ONE;
      T.W[x] = w;
    }
    T.aux[x] = 0;
  }
  __syncthreads();
  // compact the live list (drop D)
  if (k) compact_list(T, sh, [&](uint32_t x) { return T.W[x] != 0; });
  if (t == 0) {
    if (sh.csize < CL_CAP) sh.cl[sh.csize] = sh.ustar;
    sh.csize += 1;
  }
  __syncthreads();
}

__device__ void clear_aux_list(Task &T, Sh &sh) {
  for (uint32_t i = threadIdx.x; i < sh.s; i += BT) T.aux[T.list[i]] = 0;
  __syncthreads();
}

// ---------------------------------------------------------------------------
// one step on the loaded task (phases up to the choice of u* and doms)
// returns outcome in sh.outcome
// ---------------------------------------------------------------------------
template <bool LRN>
__device__ void step_core(const SearchParams &P, Task &T, Sh &sh, bool test,
                          uint32_t *t_wit) {
  const int t = threadIdx.x;
  if (t == 0) {
    sh.nstep++;
    sh.best = UINT32_MAX;
    sh.outcome = 0;
    sh.p1 = sh.p2 = UINT32_MAX;
    sh.ustar = UINT32_MAX;
    sh.ndoms = 0;
    sh.nR = 0;
  }
  __syncthreads();
  phase_mark(sh, 7);
  if (sh.csize > sh.h) {
    if (t == 0) sh.outcome = 1;
    __syncthreads();
    return;
  }
  if (sh.l <= sh.csize) eval_mindeg(T, sh, test, t_wit);
  if (sh.rules & R_RED3) {
    const uint32_t c0 = sh.csize;
    rule3(T, sh);
    if (sh.csize > sh.h) {
      if (t == 0) sh.outcome = 1;
      __syncthreads();
      return;
    }
    if (sh.csize != c0 && sh.l <= sh.csize) eval_mindeg(T, sh, test, t_wit);
  }
  phase_mark(sh, 1);
  if (sh.csize >= sh.h) {
    if (t == 0) sh.outcome = 1;
    __syncthreads();
    return;
  }
  rule12(T, sh, test);
  phase_mark(sh, 2);
  bounds(T, sh);
  phase_mark(sh, 3);
  uint32_t ub = min(sh.p1, sh.p2);
  if (ub <= sh.kl) {
    if (t == 0) sh.outcome = 2;
    __syncthreads();
    return;
  }
  if (sh.csize + sh.nR < sh.l) {
    if (t == 0) sh.outcome = 3;
    __syncthreads();
    return;
  }
  choose_ustar<LRN>(P, T, sh);
  if (test && P.t_force) {
    // one-step test: branch on the given vertex instead of the rule's u*
    // (the caller passes a candidate: an R vertex with a C neighbour)
    if (t == 0) {
      const uint32_t f = P.t_force[blockIdx.x];
      if (f != SENT && sh.ustar != UINT32_MAX) {
        uint32_t lo = 0, hi = sh.s;  // T.list ascends over the live entries
        while (lo < hi) {
          const uint32_t mid = (lo + hi) >> 1;
          if (T.list[mid] < f) lo = mid + 1;
          else hi = mid;
        }
        if (lo < sh.s && T.list[lo] == f) {
          sh.ustar = f;
          sh.us_idx = lo;
        }
      }
    }
    __syncthreads();
  }
  phase_mark(sh, 4);
  if (sh.ustar == UINT32_MAX) {
    clear_scores(T, sh);
    if (t == 0) sh.outcome = 3;
    __syncthreads();
    return;
  }
#if SCS_PROF_MODE == 5
  unsigned long long c5 = clock64();
#endif
  find_doms(T, sh);
  clear_scores(T, sh);
  mark_children(T, sh);
#if SCS_PROF_MODE == 5
  // everything but the two test stages
  if (t == 0) sh.sub[2] += clock64() - c5;
#endif
  phase_mark(sh, 5);
}

__device__ Task make_task(const SearchParams &P, Sh &sh, uint32_t *dyn,
                          uint32_t cta) {
  Task T;
  const uint32_t slot = sh.slot;
  const size_t st = P.scr.stride;
  T.W = (sh.n_local <= P.nw_smem) ? dyn : P.scr.word + (size_t)cta * st;
  // the dominance test's marks go to a bitmap behind the state words when
  // both fit (the dynamic region is all zero between tasks)
  T.bits = (sh.n_local + (sh.n_local + 31) / 32 <= P.nw_smem) ? dyn + sh.n_local : nullptr;
  T.list = P.scr.list + (size_t)cta * 2 * st;
  T.list2 = T.list + st;
  T.aux = P.scr.aux + (size_t)cta * st;
  T.tmp = P.scr.tmp + (size_t)cta * 2 * st;
  T.cpos = P.scr.cpos + (size_t)cta * st;
  T.ssc = P.scr.dsc + (size_t)cta * 3 * st;
  T.cmask = reinterpret_cast<unsigned long long *>(T.ssc + st);
  T.dsc2 = T.ssc + 2 * st;
  T.off = P.sa.loc_off + (size_t)slot * (P.sa.stride_n + 1);
  T.adj = P.sa.loc_adj + (size_t)slot * P.sa.cap_adj;
  T.dist = P.sa.loc_dist + (size_t)slot * P.sa.stride_n;
  T.gid = P.sa.loc_gid + (size_t)slot * P.sa.stride_n;
  T.witness = P.sa.witness + (size_t)slot * P.sa.wit_cap;
  T.slot = P.slots + slot;
  if (threadIdx.x == 0) sh.stride = (uint32_t)st;
  __syncthreads();
  return T;
}

__device__ void set_task_header(const SearchParams &P, Sh &sh,
                                const uint32_t *rec) {
  if (threadIdx.x == 0) {
    sh.slot = __ldcg(rec);
    sh.s = __ldcg(rec + 1);
    sh.csize = __ldcg(rec + 2);
    Slot *sl = P.slots + sh.slot;
    sh.n_local = sl->n_local;
    sh.l = sl->l;
    sh.h = sl->h;
    sh.ldoms = min(sl->limit_doms, (uint32_t)MAX_DOMS);
    sh.rules = sl->rules;
    sh.kl = *(volatile uint32_t *)&sl->kl;
    sh.wit_pending = *(volatile uint32_t *)&sl->abort;
    sh.q_local = sl->q_local;
    sh.qtag = sl->qtag;
    sh.dmax = P.g.dmax;
    // the step after this one's increment decides the trace sampling
    sh.lrn = (P.mlp.w ? 1u : 0u) |
             ((P.trace_cap && ((sh.nstep + 1) & P.trace_mask) == 0) ? 2u : 0u);
    sh.mean_deg = sl->n_local ? (float)P.sa.loc_off[(size_t)sh.slot * (P.sa.stride_n + 1) + sl->n_local] /
                                    (float)sl->n_local
                              : 0.0f;
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// test entry: one deterministic step per CTA, all children written in
// canonical order Include, Dom_0..Dom_{k-1}, Exclude (dead ones skipped)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(BT, SEARCH_MINB)
step_test_kernel(SearchParams P) {
  extern __shared__ uint32_t dyn[];
  __shared__ Sh sh;
  const uint32_t ti = blockIdx.x;
  if (ti >= P.t_ntasks) return;
  const uint32_t *rec = P.t_rec + P.t_rec_off[ti];
  set_task_header(P, sh, rec);
  if (threadIdx.x == 0) {
    sh.kl = P.t_kl[ti];
    sh.bytes = 0;
    sh.nstep = blockIdx.x;
    for (int i = 0; i < 8; i++) sh.ph[i] = 0;
    for (int i = 0; i < 4; i++) sh.sub[i] = sh.cnt4[i] = 0;
    sh.r12 = sh.r3 = 0;
    sh.t_ph = clock64();
  }
  __syncthreads();
  Task T = make_task(P, sh, dyn, ti);
  // state words and the bitmap behind them start at zero
  for (uint32_t i = threadIdx.x; i < P.nw_smem; i += BT) dyn[i] = 0;
  if (threadIdx.x == 0) sh.lrn = P.t_sl ? 4u : 0u;
  __syncthreads();
  load_record(rec, T, sh);
  uint32_t *wit = P.t_wit + (size_t)ti * P.t_wit_stride;
  step_core<true>(P, T, sh, true, wit);
  uint32_t *hdr = P.t_hdr + 16 * ti;
  uint32_t *kids = P.t_kids ? P.t_kids + (size_t)ti * P.t_kids_stride : nullptr;
  if (sh.outcome == 0 && kids) {
    const uint32_t k = sh.ndoms;
    uint64_t w = 0;
    uint32_t nk = 0;
    for (uint32_t code = 0; code <= k + 1; code++) {
      uint32_t s2, c2;
      child_shape(sh, code, s2, c2);
      if (!child_alive(sh, s2, c2)) continue;
      uint32_t *dst = kids + w;
      if (P.t_kids_rec) {
        // full task records, as the search stores them
        write_child(T, sh, code, dst + REC_HDR, dst + REC_HDR + s2, dst);
        __syncthreads();
        if (threadIdx.x == 0 && nk < MAX_DOMS + 2)
          P.t_kid_off[(size_t)ti * (MAX_DOMS + 3) + nk] = (uint32_t)w;
        __syncthreads();
        w += 2ull * s2 + 5;
      } else {
        // layout for the parity tests: [s, csize, entries(s), degrees(s)]
        write_child(T, sh, code, dst + 2, dst + 2 + s2, nullptr);
        __syncthreads();
        if (threadIdx.x == 0) {
          dst[0] = s2;
          dst[1] = c2;
        }
        __syncthreads();
        w += 2 + 2ull * s2;
      }
      nk++;
    }
    if (threadIdx.x == 0) {
      hdr[9] = nk;
      hdr[10] = (uint32_t)w;
    }
  }
  // the child marks of a branching step (aux words, zero between tasks) are
  // cleared whether or not the children were written
  if (sh.outcome == 0) clear_aux_list(T, sh);
  if (threadIdx.x == 0) {
    hdr[0] = sh.outcome;
    hdr[1] = sh.kl;
    hdr[2] = sh.best;
    hdr[3] = sh.csize;
    hdr[4] = sh.outcome >= 2 || sh.outcome == 0 ? sh.csize + sh.nR : 0;
    hdr[5] = sh.p1;
    hdr[6] = sh.p2;
    hdr[7] = sh.ustar;
    hdr[8] = sh.ndoms;
    hdr[11] = wit[CL_CAP];
    if (sh.outcome == 0 && !kids) hdr[9] = 0;
    for (uint32_t j = 0; j < sh.ndoms; j++)
      P.t_doms[(size_t)ti * P.t_doms_stride + j] = sh.doms[j];
  }
  clear_state(T, sh);
}

// ---------------------------------------------------------------------------
// search: persistent within a time slice
// ---------------------------------------------------------------------------
// The next parked root of the slice's release queue goes to the pool (thread
// 0 of the CTA whose step finished a query).  Its task is counted before its
// descriptor is visible, and before the finished query's last task leaves
// the global count, so idle CTAs never see zero outstanding work between the
// two and leave the slice early.
__device__ void release_next(const SearchParams &P) {
  if (!P.rel_count) return;
  for (;;) {
    const uint32_t i = atomicAdd(P.rel_next, 1u);
    if (i >= P.rel_count) return;
    const uint32_t slot = P.rel_queue[i];
    Slot *sl = P.slots + slot;
    if (*(volatile uint32_t *)&sl->state != SLOT_SEARCH) {  // preparation failed
      P.rel_flag[i] = 2;
      continue;
    }
    sl->t_admit = gtimer();  // search time runs from activation
    atomicAdd(&P.ctr->pending, 1ull);
    P.rel_flag[i] = 1;
    const uint32_t tk = atomicAdd(P.pool.tail, 1u);
    if (tk >= P.pool.desc_cap) {
      atomicOr(&P.ctr->error, ERR_POOL);
      return;
    }
    __threadfence();
    atomicExch(&P.pool.desc[tk], (unsigned long long)slot * P.root_stride + 1ull);
    return;
  }
}

__device__ void finish_tasks(const SearchParams &P, uint32_t slot, long long delta) {
  // delta = tasks created - tasks ended; runs on thread 0.  Only a decrease
  // can finish the query, so only then is the old count waited for.
  Slot *sl = P.slots + slot;
  if (delta >= 0) {
    atomicAdd(&P.ctr->pending, (unsigned long long)delta);
    atomicAdd(&sl->pending, (unsigned long long)delta);
    return;
  }
  unsigned long long old = atomicAdd(&sl->pending, (unsigned long long)delta);
  if ((long long)old + delta == 0) {
    sl->t_done = gtimer();
    __threadfence();
    atomicExch(&sl->state, SLOT_DONE);
    atomicAdd(&P.ctr->done_count, 1u);
    release_next(P);
  }
  atomicAdd(&P.ctr->pending, (unsigned long long)delta);
}

// reserve `len` words for a record: own stack, else the shared pool
__device__ uint32_t *reserve_record(const SearchParams &P, uint32_t cta,
                                    uint32_t len, unsigned long long &top,
                                    unsigned long long &bot, bool &to_pool,
                                    unsigned long long &pool_off) {
  uint32_t *base = P.stk.base + (size_t)cta * P.stk.words;
  to_pool = false;
  if (top + len <= P.stk.words) {
    uint32_t *d = base + top;
    top += len;
    return d;
  }
  // spill to the pool
  unsigned long long off = atomicAdd(P.pool.arena_top, (unsigned long long)len);
  if (off + len > P.pool.arena_cap) return nullptr;
  to_pool = true;
  pool_off = off;
  atomicAdd(&P.ctr->spills, 1ull);
  return P.pool.arena + off;
}

__device__ bool publish_pool(const SearchParams &P, unsigned long long off) {
  __threadfence();
  uint32_t tk = atomicAdd(P.pool.tail, 1u);
  if (tk >= P.pool.desc_cap) {
    atomicOr(&P.ctr->error, ERR_POOL);
    return false;
  }
  atomicExch(&P.pool.desc[tk], off + 1ull);
  return true;
}

// Header sanity of a task record (thread 0): slot in range and searching,
// 1 <= s <= n_local, csize <= s, len == 2s+5, the record inside the region
// it came from (room words: the length its stack footer gave, or what is
// left of the pool arena), footer == len, first and last entry ids in range.
// Returns 0 or a code naming the first failed check.  No word outside the
// region is read.
__device__ uint32_t check_record(const SearchParams &P, const uint32_t *rec,
                                 int from_pool, unsigned long long room) {
  if (room < REC_HDR + 1) return 10;
  uint32_t slot = __ldcg(rec), s = __ldcg(rec + 1), cs = __ldcg(rec + 2),
           len = __ldcg(rec + 3);
  if (slot >= P.nslots) return 1;
  const Slot *sl = P.slots + slot;
  if (*(const volatile uint32_t *)&sl->state != SLOT_SEARCH) return 2;
  uint32_t nl = *(const volatile uint32_t *)&sl->n_local;
  if (s == 0 || s > nl) return 3;
  if (cs > s) return 4;
  if (len != 2 * s + 5) return 5;
  if (len > room || (!from_pool && len != room)) return 9;
  if (__ldcg(rec + REC_HDR + 2 * s) != len) return 6;
  // first and last entry ids in range (the full ascending check is O(s) on
  // one thread and is not paid per task)
  if ((__ldcg(rec + REC_HDR) >> 1) >= nl) return 7;
  if ((__ldcg(rec + REC_HDR + s - 1) >> 1) >= nl) return 8;
  return 0;
}

// claim one pool record; returns arena offset+1 or 0
__device__ unsigned long long pool_take(const SearchParams &P) {
  for (int attempt = 0; attempt < 64; attempt++) {
    uint32_t h = *(volatile uint32_t *)P.pool.head;
    uint32_t tl = min(*(volatile uint32_t *)P.pool.tail, P.pool.desc_cap);
    if (h >= tl) return 0;
    if (atomicCAS(P.pool.head, h, h + 1) == h) {
      for (uint32_t spin = 0; spin < (1u << 24); spin++) {
        unsigned long long d = *(volatile unsigned long long *)&P.pool.desc[h];
        if (d) return d;
        __nanosleep(32);
      }
      atomicOr(&P.ctr->error, ERR_SPIN);
      return 0;
    }
  }
  return 0;
}

// When a record of `len` words would not fit above `top` but the stack has
// room below `bot` (left by donations), slide [bot, top) down to 0.  All
// threads call this; the copy runs in chunks no longer than the shift so no
// chunk overlaps its own destination.
__device__ void stack_make_room(const SearchParams &P, uint32_t *sbase,
                                uint32_t len, unsigned long long &top,
                                unsigned long long &bot) {
  unsigned long long t0 = top, b0 = bot;
  // Thread 0 reserves records (moving top and bot) as soon as this returns:
  // every thread must have read them first, or a late warp could see the new
  // top, decide on a slide alone and run the copy loop's barriers out of
  // step with the rest of the CTA.
  __syncthreads();
  if (t0 + len <= P.stk.words || b0 == 0) return;
  const unsigned long long used = t0 - b0, shift = b0;
  // A slide copies the whole live part in chunks of at most the gap, one
  // barrier each.  Slide only when the gap holds the record and is at least
  // an eighth of the live part; otherwise the record goes to the pool (not
  // sliding is always safe: reservations fall back to the pool).
  if (shift < len || 8 * shift < used) return;
  if (threadIdx.x == 0) atomicAdd(&P.ctr->slides, 1ull);
  for (unsigned long long base = 0; base < used; base += shift) {
    unsigned long long cnt = min(shift, used - base);
    for (unsigned long long i = threadIdx.x; i < cnt; i += BT)
      sbase[base + i] = __ldcg(sbase + b0 + base + i);
    // the next chunk and later reads use L2 loads: each thread's moved words
    // must have reached L2 (a barrier alone only orders them within the CTA)
    __threadfence();
    __syncthreads();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    top = used;
    bot = 0;
  }
  __syncthreads();
}

// The persistent search; LRN adds the learned branching choice and the
// trace (two kernels, so the plain one carries none of that code and keeps
// its registers for the step itself).
template <bool LRN>
__device__ __forceinline__ void search_body(const SearchParams &P) {
  extern __shared__ uint32_t dyn[];
  __shared__ Sh sh;
  __shared__ unsigned long long s_top, s_bot;
  __shared__ int s_hungry;
  __shared__ uint32_t *s_rec;
  __shared__ unsigned long long s_pool_off;
  __shared__ int s_pool_rec;
  __shared__ unsigned long long s_room;  // words of the popped stack record
  __shared__ unsigned long long s_deadline;
  __shared__ int s_bad;  // the record just obtained failed its header checks
  // Thread 0's view of the query and the slice, read together at each step's
  // start (one round trip instead of one per check): the node count and
  // budget decide the search budget, the idle-CTA count the donation, the
  // stop flag the slice exit.  Each is at most one step stale, which only
  // delays a budget stop or a donation by a step.  Shared, not registers:
  // only thread 0 uses them, and registers are the kernel's tight resource.
  __shared__ unsigned long long s_nodes_seen, s_budget_seen;
  __shared__ uint32_t s_abort_seen, s_hungry_seen, s_stop_seen;
  const uint32_t cta = blockIdx.x;
  const int t = threadIdx.x;
  uint32_t *sbase = P.stk.base + (size_t)cta * P.stk.words;
  for (uint32_t i = t; i < P.nw_smem; i += BT) dyn[i] = 0;
  if (t == 0) {
    unsigned long long want = gtimer() + P.slice_ns;
    unsigned long long d = atomicCAS(&P.ctr->deadline, 0ull, want);
    s_deadline = d ? d : want;
    s_top = P.stk.top[cta];
    s_bot = P.stk.bot[cta];
    s_hungry = 0;
    s_nodes_seen = s_budget_seen = 0;
    s_abort_seen = s_hungry_seen = s_stop_seen = 0;
    sh.have = 0;
    sh.stop = 0;
    sh.bytes = 0;
    sh.nstep = blockIdx.x;
    for (int i = 0; i < 8; i++) sh.ph[i] = 0;
    for (int i = 0; i < 4; i++) sh.sub[i] = sh.cnt4[i] = 0;
    sh.r12 = sh.r3 = 0;
    sh.prof_small = 0;
    sh.t_ph = clock64();
  }
  __syncthreads();
  Task T;
  unsigned long long local_nodes = 0;
  for (;;) {
    // ---------------- obtain a task ----------------
    if (!sh.have) {
      // Thread 0 rewrites s_rec and sh.stop below.  The idle path loops back
      // here right after every thread read them, and the slice-exit check
      // reads sh.stop just before: without this barrier a late warp could
      // read the next iteration's record pointer (or stop flag), take the
      // other branch and run one barrier out of step with the rest of the
      // CTA from then on.
      __syncthreads();
      if (t == 0) {
        s_rec = nullptr;
        s_pool_rec = 0;
        if (s_top > s_bot) {
          uint32_t len = __ldcg(sbase + s_top - 1);
          if (len < 5 || len > s_top - s_bot) {
            atomicOr(&P.ctr->error, ERR_RECORD);
            s_top = s_bot;
          } else {
            s_rec = sbase + (s_top - len);
            s_room = len;
            s_top -= len;
          }
        }
        if (!s_rec) {
          unsigned long long d = pool_take(P);
          if (d) {
            s_rec = P.pool.arena + (d - 1);
            s_pool_rec = 1;
            atomicAdd(&P.ctr->steals, 1ull);
          }
        }
        if (s_rec && s_hungry) {
          atomicSub(&P.ctr->hungry, 1u);
          s_hungry = 0;
        }
        if (!s_rec) {
          if (!s_hungry) {
            atomicAdd(&P.ctr->hungry, 1u);
            s_hungry = 1;
          }
          unsigned long long pend = *(volatile unsigned long long *)&P.ctr->pending;
          if (pend == 0 || gtimer() > s_deadline ||
              *(volatile uint32_t *)&P.ctr->stop)
            sh.stop = 1;
          else
            __nanosleep(2000);
        }
      }
      __syncthreads();
      if (sh.stop) break;
      if (!s_rec) continue;
      const uint32_t *rec = s_rec;
      if (t == 0) {
        // validate the record before trusting any index in it (a flag of its
        // own: other warps may still be reading sh.stop above)
        const unsigned long long room =
            s_pool_rec ? P.pool.arena_cap - (unsigned long long)(rec - P.pool.arena) : s_room;
        uint32_t bad = check_record(P, rec, s_pool_rec, room);
        s_bad = bad != 0;
        if (bad) {
          atomicOr(&P.ctr->error, ERR_RECORD);
          P.ctr->err_info[0] = bad;
          if (room >= REC_HDR) {
            P.ctr->err_info[1] = __ldcg(rec);
            P.ctr->err_info[2] = __ldcg(rec + 1);
            P.ctr->err_info[3] = __ldcg(rec + 3);
          }
        }
      }
      __syncthreads();
      if (s_bad) break;
      set_task_header(P, sh, rec);  // also reads the query's abort flag
      if (sh.wit_pending) {
        if (t == 0) finish_tasks(P, sh.slot, -1);
        __syncthreads();
        continue;
      }
      phase_mark(sh, 7);
      T = make_task(P, sh, dyn, cta);
      load_record(rec, T, sh);
      if (sh.bad_rec) {  // a damaged record: report it and leave the slice
        if (t == 0) {
          atomicOr(&P.ctr->error, ERR_RECORD);
          P.ctr->err_info[0] = 11;
          P.ctr->err_info[1] = sh.slot;
          P.ctr->err_info[2] = sh.s;
          P.ctr->err_info[3] = sh.n_local;
        }
        break;
      }
      if (t == 0) sh.have = 1;
      __syncthreads();
      phase_mark(sh, 0);
    }
    // ---------------- one step ----------------
    // The query's abort flag and incumbent, read together once per step: a
    // stale incumbent only prunes less, so the step does not re-read it.
    if (t == 0) {
      const volatile Slot *sl = P.slots + sh.slot;
      const uint32_t ab = sl->abort, g = sl->kl;
      s_nodes_seen = sl->nodes;
      s_budget_seen = sl->node_budget;
      s_hungry_seen = *(volatile uint32_t *)&P.ctr->hungry;
      s_stop_seen = *(volatile uint32_t *)&P.ctr->stop;
      s_abort_seen = ab;
      sh.wit_pending = ab;
      if (g > sh.kl) sh.kl = g;
    }
    __syncthreads();
    if (sh.wit_pending) {  // the query stopped (budget / capacity): drop
      if (t == 0) {
        finish_tasks(P, sh.slot, -1);
        sh.have = 0;
      }
      clear_state(T, sh);
      continue;
    }
#if SCS_PROF_MODE == 4
    if (t == 0) sh.prof_small = sh.s < 512;
#endif
#if SCS_PROF_MODE == 2
    const uint32_t s_in = sh.s;
    const unsigned long long c_step = clock64();
#endif
    step_core<LRN>(P, T, sh, false, nullptr);
#if SCS_PROF_MODE == 2
    if (t == 0) {
      const int b = s_in < 512 ? 0 : s_in < 4096 ? 1 : 2;
      sh.sub[b] += clock64() - c_step;
      if (b < 2) sh.cnt4[b]++;
    }
#endif
    local_nodes++;
    bool cont = false;
    if (sh.outcome == 0) {
      const uint32_t k = sh.ndoms;
      // reserve Exclude, Dom_{k-1} .. Dom_0 in push order (Dom_0 on top, so
      // it pops first after the dive), then write all of them in one pass.
      // Room is made once for all of them: a compaction between two
      // reservations would move the earlier ones.
      {
        unsigned long long total = 0;
        for (uint32_t code = 1; code <= k + 1; code++) {
          uint32_t s2, c2;
          child_shape(sh, code, s2, c2);
          if (child_alive(sh, s2, c2)) total += 2ull * s2 + 5;
        }
        if (total) stack_make_room(P, sbase, (uint32_t)min(total, 0xFFFFFFFFull), s_top, s_bot);
      }
      if (t == 0) {
        for (int code = (int)k + 1; code >= 1; code--) {
          uint32_t s2, c2;
          child_shape(sh, (uint32_t)code, s2, c2);
          sh.kid_dst[code] = 0;
          sh.kid_len[code] = 0;
          if (!child_alive(sh, s2, c2)) continue;
          uint32_t len = 2 * s2 + 5;
          bool tp;
          unsigned long long poff = 0;
          unsigned long long top = s_top, bot = s_bot;
          if (top == bot) { top = bot = 0; }
          uint32_t *d = reserve_record(P, cta, len, top, bot, tp, poff);
          s_top = top;
          s_bot = bot;
          sh.kid_dst[code] = (unsigned long long)d;
          sh.kid_len[code] = tp ? 0x80000000u : 1u;
          sh.kid_pool[code] = poff;
          if (!d) {
            atomicOr(&P.ctr->error, ERR_STACK);
            P.slots[sh.slot].abort = 1;
            P.slots[sh.slot].status = RS_CAPACITY;
          }
        }
        // Count the reserved children before any of them is published: a
        // child spilled to the pool can be taken and finished by another CTA
        // before this step ends, and the query must not reach zero
        // outstanding tasks (and be reported done) while its siblings are
        // still stored.  The same update ends the parent and counts the
        // in-place Include dive, so it can reach zero only when nothing of
        // this task remains.
        uint32_t nres = 0;
        for (uint32_t code = 1; code <= k + 1; code++) nres += sh.kid_dst[code] != 0;
        uint32_t s0, c0;
        child_shape(sh, 0, s0, c0);
        const long long delta = (long long)nres + (child_alive(sh, s0, c0) ? 1 : 0) - 1;
        if (delta) finish_tasks(P, sh.slot, delta);
      }
      __syncthreads();
      if (k + 1 >= 1) {
        write_children(T, sh, 1, k + 1, (uint32_t *const *)sh.kid_dst);
        // Every thread stored entries of the children.  A child spilled to
        // the pool is read by another SM once thread 0 publishes it, so each
        // thread fences its own stores before the barrier.  Children on the
        // stack are read back only by this CTA, after the barrier.
        bool spilled = false;
        for (uint32_t code = 1; code <= k + 1; code++)
          spilled |= sh.kid_dst[code] != 0 && (sh.kid_len[code] & 0x80000000u);
        if (spilled) __threadfence();
        __syncthreads();
        for (uint32_t code = 1; code <= k + 1; code++) {
          if (!sh.kid_dst[code]) continue;
          if (t == 0) {
            uint32_t s2, c2;
            child_shape(sh, code, s2, c2);
            if (sh.kid_len[code] & 0x80000000u) publish_pool(P, sh.kid_pool[code]);
            sh.bytes += 16ull * s2;
          }
        }
      }
      uint32_t s2, c2;
      child_shape(sh, 0, s2, c2);
      cont = child_alive(sh, s2, c2);
      if (cont) {
        if (t == 0) sh.bytes += 16ull * s2;
        apply_include(T, sh);
      } else {
        clear_aux_list(T, sh);
      }
    }
    phase_mark(sh, 6);
    if (t == 0) {
      // a task that did not branch ends here (a branching one was settled
      // with its children)
      if (sh.outcome != 0) finish_tasks(P, sh.slot, -1);
      Slot *sl = P.slots + sh.slot;
      atomicAdd(&sl->nodes, 1ull);  // no return value: a reduction, no wait
      if (s_budget_seen && s_nodes_seen + 1ull >= s_budget_seen && !s_abort_seen) {
        sl->status = RS_TIMEOUT;
        sl->abort = 1;
        s_abort_seen = 1;
      }
      sh.have = cont ? 1 : 0;
    }
    __syncthreads();
    if (!cont) clear_state(T, sh);
    // ---------------- donate the oldest stack record if others are idle ----
    if (t == 0) {
      s_rec = nullptr;
      if (s_hungry_seen > 0 && s_top > s_bot) {
        uint32_t len = __ldcg(sbase + s_bot + 3);
        if (len >= 5 && s_bot + len < s_top) {  // keep at least one record
          unsigned long long off = atomicAdd(P.pool.arena_top, (unsigned long long)len);
          if (off + len <= P.pool.arena_cap) {
            s_rec = P.pool.arena + off;
            s_pool_off = off;
          }
        }
      }
    }
    __syncthreads();
    if (s_rec) {
      const uint32_t *src = sbase + s_bot;
      const uint32_t len = __ldcg(src + 3);
      for (uint32_t i = t; i < len; i += BT) s_rec[i] = __ldcg(src + i);
      __threadfence();  // every copying thread, before thread 0 publishes
      __syncthreads();
      if (t == 0) {
        if (publish_pool(P, s_pool_off)) {
          s_bot += len;
          atomicAdd(&P.ctr->donations, 1ull);
        }
      }
      __syncthreads();
    }
    // ---------------- leave the slice? ----------------
    if (t == 0) {
      if (gtimer() > s_deadline || s_stop_seen) sh.stop = 1;
    }
    __syncthreads();
    if (sh.stop) {
      if (sh.have) {
        // save the in-place task to the own stack (it is already counted)
        uint32_t len = 2 * sh.s + 5;
        stack_make_room(P, sbase, len, s_top, s_bot);
        if (t == 0) {
          bool tp;
          unsigned long long poff = 0;
          unsigned long long top = s_top, bot = s_bot;
          if (top == bot) { top = bot = 0; }
          s_rec = reserve_record(P, cta, len, top, bot, tp, poff);
          s_top = top;
          s_bot = bot;
          s_pool_rec = tp ? 1 : 0;
          s_pool_off = poff;
        }
        __syncthreads();
        if (s_rec) {
          uint32_t *d = s_rec;
          for (uint32_t i = t; i < sh.s; i += BT) {
            uint32_t x = T.list[i];
            uint32_t w = T.W[x];
            d[REC_HDR + i] = (x << 1) | (st_of(w) == ST_C ? 1u : 0u);
            d[REC_HDR + sh.s + i] = w & (ST_ONE - 1u);  // dC and dR fields
          }
          if (t == 0) {
            d[0] = sh.slot;
            d[1] = sh.s;
            d[2] = sh.csize;
            d[3] = len;
            d[REC_HDR + 2 * sh.s] = len;
          }
          __threadfence();  // every writer: the record is read back with L2 loads
          __syncthreads();
          if (t == 0 && s_pool_rec) publish_pool(P, s_pool_off);
        } else if (t == 0) {
          atomicOr(&P.ctr->error, ERR_STACK);
          P.slots[sh.slot].abort = 1;
          P.slots[sh.slot].status = RS_CAPACITY;
          finish_tasks(P, sh.slot, -1);
        }
        clear_state(T, sh);
      }
      break;
    }
  }
  if (t == 0) {
    if (s_hungry) atomicSub(&P.ctr->hungry, 1u);
    if (s_top == s_bot) s_top = s_bot = 0;
    P.stk.top[cta] = s_top;
    P.stk.bot[cta] = s_bot;
    atomicAdd(&P.ctr->nodes, local_nodes);
    atomicAdd(&P.ctr->bytes, sh.bytes);
    for (int i = 0; i < 8; i++) atomicAdd(&P.ctr->phase_cycles[i], sh.ph[i]);
    atomicAdd(&P.ctr->r12_rounds, sh.r12);
    atomicAdd(&P.ctr->r3_rounds, sh.r3);
    atomicAdd(&P.ctr->steps, local_nodes);
    for (int i = 0; i < 4; i++) {
      atomicAdd(&P.ctr->sub_cycles[i], sh.sub[i]);
      atomicAdd(&P.ctr->sub_counts[i], sh.cnt4[i]);
    }
  }
}

__global__ void __launch_bounds__(BT, SEARCH_MINB)
search_kernel(SearchParams P) {
  search_body<false>(P);
}

__global__ void __launch_bounds__(BT, SEARCH_MINB)
search_kernel_learned(SearchParams P) {
  search_body<true>(P);
}

}  // namespace scs
