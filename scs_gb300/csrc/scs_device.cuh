// scs_device.cuh -- device data layout shared by the preprocessing and the
// branch-and-bound kernels.
//
// Layout in HBM (one engine, one GPU):
//   graph      : CSR off[n+1], adj[nnz] (ascending), core[n]    (resident)
//   slot i     : local graph of query i -- loc_off[n+1], loc_adj[cap_adj]
//                (rows padded to a multiple of 4 with SENT so rows can be read
//                with 16-byte loads), loc_dist[n] (u16), loc_gid[n], witness
//   CTA c      : task stack region (LIFO, records below), scratch arrays
//   pool       : shared arena + descriptor ring for tasks moved between CTAs
//
// Task record (u32 words):
//   [0] slot  [1] s  [2] csize  [3] len
//   [4 .. 4+s)      entries  (local_id << 1) | inC      (ascending id)
//   [4+s .. 4+2s)   degrees  (dC << 21) | dR            (within the task)
//   [4+2s]          footer = len = 2s + 5
// Per-vertex state word used while a CTA works on a task (shared memory):
//   bits 31..30 status (0 absent, 1 R, 2 C, 3 removed), 29..21 dC, 20..0 dR.
// dC counts neighbours in C, so dC <= |C| <= h < 512 (9 bits) whenever the
// task is kept; dR takes the other 21 bits (local degrees up to 2,097,151).
#pragma once
#include <cstdint>

#include <cuda_runtime.h>

#include "mlp.cuh"

namespace scs {

constexpr uint32_t SENT = 0xFFFFFFFFu;
constexpr uint32_t ST_ABSENT = 0, ST_R = 1, ST_C = 2, ST_X = 3;
constexpr uint32_t DC_SHIFT = 21;
constexpr uint32_t DC_ONE = 1u << DC_SHIFT;
constexpr uint32_t ST_ONE = 1u << 30;
constexpr uint32_t DMASK = DC_ONE - 1u;   // dR field (and the largest dR)
constexpr uint32_t DCMASK = 0x1FFu;        // dC field after the shift
// Largest local graph a query may search unless scs_config.max_local says
// otherwise (it sizes the per-CTA scratch and the parked roots).  In-task
// dR is a 21-bit field of the state word, so a local graph with a vertex of
// more than DMASK local neighbours is rejected whatever its size.
constexpr uint32_t MAX_LOCAL_DEFAULT = 1u << 21;
constexpr uint32_t CL_CAP = 512;       // max |C| tracked (h < CL_CAP)
constexpr uint32_t MAX_DOMS = 15;      // adjacency mask bits 1..15
constexpr uint32_t INF16 = 0xFFFFu;
constexpr uint32_t REC_HDR = 4;

// rule switches (same bits as the oracle): red1 red2 red3 prun1 prun2
constexpr uint32_t R_RED1 = 1, R_RED2 = 2, R_RED3 = 4, R_PRUN1 = 8,
                   R_PRUN2 = 16;

// slot states
constexpr uint32_t SLOT_FREE = 0, SLOT_SEARCH = 2, SLOT_DONE = 3;

// result status (mirrors scs.h)
constexpr uint32_t RS_DONE = 0, RS_HEURISTIC = 1, RS_CAPACITY = 2,
                   RS_TIMEOUT = 3, RS_BAD = 4, RS_TOO_LARGE = 5;

struct Slot {
  uint32_t state;
  uint32_t status;
  uint32_t n_local;
  uint32_t q_local;
  uint32_t l, h, limit_doms, rules;
  uint32_t kl;       // incumbent, atomicMax
  uint32_t kl_heu;
  uint32_t ubd;
  uint32_t wit_lock;
  uint32_t wit_val;  // min degree of the witness (0 = none)
  uint32_t wit_n;
  uint32_t q_global;
  uint32_t qtag;     // the host's tag of the query (trace records carry it)
  uint32_t abort;    // set when the query stops early (budget/capacity)
  unsigned long long pending;  // outstanding tasks of this query
  unsigned long long nodes;
  unsigned long long t_admit;
  unsigned long long t_done;
  unsigned long long node_budget;
};

struct DevGraph {
  uint32_t n;
  uint32_t dmax;
  const uint32_t *off;
  const uint32_t *adj;
  const uint32_t *core;
};

struct SlotArrays {
  uint32_t *loc_off;  // [slots][n+1]
  uint32_t *loc_adj;  // [slots][cap_adj]
  uint16_t *loc_dist; // [slots][n]
  uint32_t *loc_gid;  // [slots][n]
  uint32_t *witness;  // [slots][wit_cap]
  uint64_t cap_adj;
  uint32_t stride_n;
  uint32_t wit_cap;
  uint32_t max_local;  // largest local graph searched (vertices)
};

struct Pool {
  uint32_t *arena;
  unsigned long long arena_cap;   // words
  unsigned long long *arena_top;  // bump pointer (words)
  unsigned long long *desc;       // offset+1, 0 = not yet published
  uint32_t desc_cap;
  uint32_t *head;
  uint32_t *tail;
};

struct Counters {
  unsigned long long pending;  // outstanding tasks, all queries
  unsigned long long nodes;
  unsigned long long donations;
  unsigned long long steals;
  unsigned long long spills;
  unsigned long long bytes;
  unsigned long long prep_bytes;
  unsigned long long deadline; // set by the first CTA of a slice
  uint32_t hungry;
  uint32_t error;              // bit flags, see ERR_*
  uint32_t done_count;
  uint32_t stop;               // host asks CTAs to leave the slice
  uint32_t err_info[4];
  // profiling: clock cycles per step phase summed over CTAs, and rounds
  unsigned long long phase_cycles[8];  // load, mindeg+r3, r12, bounds, ustar, doms, kids, other
  unsigned long long r12_rounds, r3_rounds, steps;
  unsigned long long sub_cycles[4], sub_counts[4];
  unsigned long long slides;   // task-stack slides (live part moved down)
  unsigned long long proposals;         // learned incumbent proposals made
  unsigned long long proposals_better;  // ... that raised the incumbent
};

constexpr uint32_t ERR_SPIN = 1, ERR_POOL = 2, ERR_STACK = 4, ERR_RECORD = 8;

struct Stacks {
  uint32_t *base;                  // [ctas][words]
  unsigned long long words;        // per CTA
  unsigned long long *top;         // [ctas]
  unsigned long long *bot;         // [ctas]
};

struct Scratch {  // per search CTA, stride n words each
  uint32_t *word;  // fallback state words when n_local exceeds shared memory
  uint32_t *list;  // live ids of the current task (ascending)
  uint32_t *aux;   // marks (zero between uses)
  uint32_t *tmp;   // removal / promotion / candidate lists
  uint32_t *cpos;  // list positions of the candidates in tmp
  double *dsc;     // candidate scores
  uint32_t stride;
};

__host__ __device__ inline uint32_t ubd_dev(uint32_t kl, uint32_t h) {
  // distance bound of src/helpers.cc:974-990, u32 arithmetic as written
  uint32_t ubd = h - 1;
  for (uint32_t d = 1; d <= h; d++) {
    if (d == 1 || d == 2) {
      if (kl + d > h) { ubd = d - 1; break; }
    } else {
      uint32_t min_n = kl + d + 1 + (d / 3) * (kl - 2);
      if (h < min_n) { ubd = d - 1; break; }
    }
  }
  return ubd;
}


// ---- kernel parameter blocks and entry points ----
struct PrepJob {
  uint32_t slot, q, kl, ubd;
  uint32_t l, h, limit_doms, rules;
  uint32_t kl_heu;
  uint32_t root_to_pool;  // 0: no root; 1: root published now; 2: root parked
  uint32_t root_off_lo, root_off_hi;  // parked root's arena offset (words)
  unsigned long long node_budget;
  uint32_t qtag;
  uint32_t pad_;
};

struct PrepScratch {
  uint16_t *dist;  // [jobs][n]
  uint32_t *vis;   // [jobs][nw]
  uint32_t *comp;  // [jobs][nw]
  uint32_t *fa;    // [jobs][n]
  uint32_t *fb;    // [jobs][n]
  uint32_t *wpre;  // [jobs][nw+1]
  uint32_t *ldeg;  // [jobs][n] local degree by global id (prep.cu)
  uint32_t stride_n;
  uint32_t stride_w;
  uint32_t big_row;  // rows this long are walked by a whole CTA (prep.cu)
};

struct SearchParams {
  DevGraph g;
  SlotArrays sa;
  Slot *slots;
  Pool pool;
  Counters *ctr;
  Stacks stk;
  Scratch scr;
  uint32_t nw_smem;                 // state words that fit in shared memory
  uint32_t nslots;
  unsigned long long slice_ns;      // slice length (device clock)
  // parked roots the device releases itself, in order, one each time a
  // searched query finishes inside the slice (the host reads rel_next and
  // rel_flag after the slice: 1 released, 2 skipped because already done)
  const uint32_t *rel_queue;
  uint32_t rel_count;
  uint32_t *rel_next;
  uint32_t *rel_flag;
  unsigned long long root_stride;
  // test mode (one step per CTA)
  const uint32_t *t_rec;            // input records
  const unsigned long long *t_rec_off;
  uint32_t t_ntasks;
  uint32_t *t_hdr;                  // 16 per task
  uint32_t *t_doms;
  uint32_t t_doms_stride;
  uint32_t *t_kids;
  unsigned long long t_kids_stride;
  uint32_t *t_wit;
  uint32_t t_wit_stride;
  const uint32_t *t_kl;             // incumbent per test task
  const uint32_t *t_force;          // u* forced per test task (local id;
                                    // SENT: the rule's own), or null
  uint32_t *t_sl;                   // per test task: [count, 16 local ids] of
                                    // the shortlist, or null
  float *t_sl_feat;                 // per test task: 16 x 16 features
  uint32_t t_kids_rec;              // 1: children written as full task
                                    // records, their offsets in t_kid_off
  uint32_t *t_kid_off;              // per test task: 18 child offsets
  // learned branching: packed network (w == null: the plain method) and the
  // trace the exact solver emits for training (cap == 0: none)
  MlpDev mlp;
  float *trace_feat;                // [cap][16] features
  uint32_t *trace_key;              // [cap][2] query tag, global vertex id
  unsigned long long *trace_count;  // records written (may pass cap)
  unsigned long long trace_cap;
  uint32_t trace_mask;              // a CTA traces its steps with
                                    // (step & mask) == 0
};

constexpr int PREP_THREADS = 512;
// Search CTA shape: 256 threads, registers sized for 3 resident CTAs per SM
// (measured fastest of 128/256/384/512 threads on the R-MAT scale-15 queries)
#ifndef SCS_SEARCH_THREADS
#define SCS_SEARCH_THREADS 256
#endif
#ifndef SCS_SEARCH_MINB
#define SCS_SEARCH_MINB 3
#endif
constexpr int SEARCH_THREADS = SCS_SEARCH_THREADS;
constexpr int SEARCH_MINB = SCS_SEARCH_MINB;

// Per-query preparation: one thread-block cluster of `cluster` CTAs (1, 2, 4,
// 8 or 16) per job; prep.cu.  PREP_MAX_CLUSTER is the portable size the
// engine picks on large graphs.
constexpr uint32_t PREP_MAX_CLUSTER = 8;
cudaError_t launch_prep(uint32_t cluster, cudaStream_t stream, DevGraph g,
                        SlotArrays sa, Slot *slots, const PrepJob *jobs,
                        int njobs, PrepScratch ps, Pool pool, Counters *ctr);
__global__ void search_kernel(SearchParams P);
// the same search with the learned branching choice and the trace
__global__ void search_kernel_learned(SearchParams P);
__global__ void release_kernel(Slot *slots, const uint32_t *cand, uint32_t n,
                               unsigned long long root_stride, Pool pool,
                               Counters *ctr);
// core numbers of a device CSR by level-synchronous peeling (core.cu)
int gpu_core_numbers(const uint32_t *d_off, const uint32_t *d_adj, uint32_t n,
                     uint32_t *d_core, uint32_t *d_scratch, void *ctr_dev,
                     void *ctr_host, int num_sms, cudaStream_t st);
__global__ void step_test_kernel(SearchParams P);
// learned incumbent proposal, one CTA of 256 threads per prepared job
__global__ void propose_kernel(DevGraph g, SlotArrays sa, Slot *slots, const PrepJob *jobs,
                               int njobs, Scratch scr, MlpDev M, Counters *ctr);

}  // namespace scs
