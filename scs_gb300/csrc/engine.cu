// engine.cu -- the GB300 SCS engine behind include/scs.h.
//
// Host flow per query (the reference's processMessages, main.cu:80-473):
//   submit -> admission into a free slot: ku = min(core[q], h-1)
//   (inc/Intialize.h:207), greedy incumbent on host threads
//   (inc/heuristic.h:321-349), early answer when kl == ku (main.cu:122-133),
//   ubD (main.cu:154-172) -> preprocessing kernel (prep.cu), root task parked
//   -> released to the shared pool while fewer than active_queries queries
//   are searched -> time-sliced persistent search (bnb.cu) until
//   the query's outstanding-task count reaches zero -> result.
// Unlike the reference, admission happens between search slices while other
// queries keep their tasks on the device (continuous batching), the level
// loop with its ~15 small copies per level is replaced by one persistent
// launch per slice, and the engine returns the community itself.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <chrono>
#include <condition_variable>
#include <memory>
#include <cstdio>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/scs.h"
#include "host_graph.h"
#include "scs_device.cuh"

using namespace scs;

namespace {

uint64_t now_ns() {
  return (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(
             std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

struct Pending {
  scs_query q;
  uint64_t ticket;
  uint64_t t_submit;
};

// A submitted query and its greedy incumbent, computed in the background by
// the heuristic workers so that it overlaps the search of earlier queries.
struct Job {
  Pending p;
  bool bad = false;   // rejected at submission
  bool done = false;  // kl/H ready (guarded by scs_engine::heu_mu)
  uint32_t kl = 0, ku = 0;
  std::vector<uint32_t> H;
};

struct SlotHost {
  bool busy = false;
  bool parked = false;  // prepared, root not yet released to the search
  Pending p;
  uint32_t kl_heu = 0;
  std::vector<uint32_t> heuH;
};

struct Done {
  scs_result r{};
  std::vector<uint32_t> H;
  uint64_t t_submit = 0;
  bool check = true;  // verify H (not for rejected queries)
};

std::string g_create_error;

// Queries searched at once unless scs_config.active_queries says otherwise.
constexpr uint32_t SCS_DEFAULT_ACTIVE = 32;
// Search slice length unless scs_config.slice_us says otherwise.  A slice
// ends early when no work is left; a longer one spends less of its time on
// the CTAs that finish their last step after the deadline (bench: 20 ms
// 61.3 queries/s, 40 ms 62.7, 80 ms 63.4), but admits new queries later.
constexpr uint64_t SCS_DEFAULT_SLICE_US = 80000;

}  // namespace

struct scs_engine {
  scs_config cfg{};
  HostGraph g;
  std::string err;
  int dev = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev2 = nullptr, ev3 = nullptr;
  bool prep_pending = false;

  // device graph
  uint32_t *d_off = nullptr, *d_adj = nullptr, *d_core = nullptr;
  // slots
  uint32_t nslots = 0;
  Slot *d_slots = nullptr;
  std::vector<Slot> h_slots;
  SlotArrays sa{};
  std::vector<SlotHost> slots;
  // prep
  uint32_t prep_cap = 0;
  uint32_t prep_cluster = 1;  // CTAs per query in preparation (prep.cu)
  PrepScratch ps{};
  PrepJob *d_jobs = nullptr;
  // search
  uint32_t grid = 0;
  uint32_t nw_smem = 0;
  size_t smem_bytes = 0;
  Pool pool{};
  Stacks stk{};
  // Roots are parked at a fixed place per slot at the head of the pool arena
  // (root_stride words each, root_words in all) and released a few at a time
  // so that only active_target queries are searched at once.
  unsigned long long root_stride = 0, root_words = 0;
  std::deque<uint32_t> parked;  // release order (entries of collected slots are skipped)
  uint32_t n_parked = 0;
  uint32_t *d_rel = nullptr;
  // parked roots queued for release on the device during a slice
  std::vector<uint32_t> devq;
  uint32_t *d_relq = nullptr, *d_rel_next = nullptr, *d_rel_flag = nullptr;
  uint32_t active_target = 0;
  unsigned long long pool_free = ~0ull;  // pool words free after the last slice
  Scratch scr{};
  Counters *d_ctr = nullptr;
  uint32_t rules = 31;
  // host state
  std::deque<std::shared_ptr<Job>> queue;     // admission order
  std::deque<std::shared_ptr<Job>> heu_todo;  // incumbents not yet started
  std::mutex heu_mu;
  std::condition_variable heu_cv, heu_done_cv;
  std::vector<std::thread> heu_workers;
  bool heu_stop = false;
  // Finished queries wait in `verify_q` until the verifier thread has checked
  // their community against the graph, then move to `done` for scs_poll.
  // The check runs beside the next search slice instead of between slices.
  std::deque<Done> verify_q;
  std::deque<Done> done;
  std::mutex res_mu;  // verify_q, done, res_pending, res_stop
  std::condition_variable res_cv;
  size_t res_pending = 0;  // in verify_q or being checked
  bool res_stop = false;
  std::thread verifier;
  uint64_t next_ticket = 1;
  uint32_t running = 0;
  uint64_t stats[SCS_STAT_COUNT] = {0};
  uint64_t prof[16] = {0};
  std::vector<HeuWork> work;
  unsigned host_threads = 1;
  std::vector<void *> allocs;
  // learned branching: packed network (learned == false: the plain method)
  bool learned = false;
  uint2 *d_mlp_w = nullptr;
  float *d_mlp_b = nullptr;
  // trace of the shortlisted candidates for training (cap 0: off)
  float *d_trace_feat = nullptr;
  uint32_t *d_trace_key = nullptr;
  unsigned long long *d_trace_count = nullptr;
  uint64_t trace_cap = 0;
  uint32_t trace_mask = 0;

  int cuda_fail(cudaError_t e, const char *what) {
    err = std::string(what) + ": " + cudaGetErrorString(e);
    // consume a non-sticky error so that it is not reported again by a later
    // launch check (of this engine or another one in the process)
    cudaGetLastError();
    return SCS_ECUDA;
  }
  template <class T>
  int dalloc(T **p, size_t count, bool zero = true) {
    size_t bytes = std::max<size_t>(count * sizeof(T), 16);
    cudaError_t e = cudaMalloc((void **)p, bytes);
    if (e != cudaSuccess) {
      err = "cudaMalloc(" + std::to_string(bytes) + "): " + cudaGetErrorString(e);
      return SCS_ENOMEM;
    }
    allocs.push_back(*p);
    if (zero) {
      e = cudaMemsetAsync(*p, 0, bytes, stream);
      if (e != cudaSuccess) return cuda_fail(e, "cudaMemset");
    }
    return 0;
  }
};

#define CK(call)                                         \
  do {                                                   \
    cudaError_t e_ = (call);                             \
    if (e_ != cudaSuccess) return E->cuda_fail(e_, #call); \
  } while (0)
#define RC(call)            \
  do {                      \
    int r_ = (call);        \
    if (r_) return r_;      \
  } while (0)

// Background worker: greedy incumbents of submitted queries, in submission
// order (the graph is read-only after creation; work[tid] is this worker's).
static void heu_worker(scs_engine *E, unsigned tid) {
  for (;;) {
    std::shared_ptr<Job> j;
    {
      std::unique_lock<std::mutex> lk(E->heu_mu);
      E->heu_cv.wait(lk, [&] { return E->heu_stop || !E->heu_todo.empty(); });
      if (E->heu_stop) return;
      j = E->heu_todo.front();
      E->heu_todo.pop_front();
    }
    std::vector<uint32_t> H;
    const uint32_t kl = greedy_incumbent(E->g, j->p.q.l, j->p.q.h, j->p.q.q, E->work[tid], H);
    {
      std::lock_guard<std::mutex> lk(E->heu_mu);
      j->kl = kl;
      j->H.swap(H);
      j->done = true;
    }
    E->heu_done_cv.notify_all();
  }
}

static void verify_worker(scs_engine *E);

static int engine_init(scs_engine *E) {
  const scs_config &c = E->cfg;
  if (c.prep_ctas != 0 && c.prep_ctas != 1 && c.prep_ctas != 2 && c.prep_ctas != 4 &&
      c.prep_ctas != 8 && c.prep_ctas != 16) {
    E->err = "prep_ctas must be 0, 1, 2, 4, 8 or 16";
    return SCS_EINVAL;
  }
  E->dev = c.device;
  CK(cudaSetDevice(E->dev));
  CK(cudaDeviceGetAttribute(&E->num_sms, cudaDevAttrMultiProcessorCount, E->dev));
  CK(cudaStreamCreateWithFlags(&E->stream, cudaStreamNonBlocking));
  CK(cudaEventCreate(&E->ev0));
  CK(cudaEventCreate(&E->ev1));
  CK(cudaEventCreate(&E->ev2));
  CK(cudaEventCreate(&E->ev3));
  E->rules = c.rules_set ? ((c.red1 ? R_RED1 : 0) | (c.red2 ? R_RED2 : 0) |
                            (c.red3 ? R_RED3 : 0) | (c.prun1 ? R_PRUN1 : 0) |
                            (c.prun2 ? R_PRUN2 : 0))
                         : 31u;
  const HostGraph &g = E->g;
  const uint32_t n = g.n;
  const uint64_t nnz = g.adj.size();
  // graph
  RC(E->dalloc(&E->d_off, n + 1, false));
  RC(E->dalloc(&E->d_adj, nnz, false));
  RC(E->dalloc(&E->d_core, n, false));
  CK(cudaMemcpyAsync(E->d_off, g.off.data(), (n + 1) * 4ull, cudaMemcpyHostToDevice, E->stream));
  if (nnz) CK(cudaMemcpyAsync(E->d_adj, g.adj.data(), nnz * 4ull, cudaMemcpyHostToDevice, E->stream));
  {
    // core numbers by GPU peeling (core.cu), copied back for admission and
    // the host-side incumbent; the scratch is released right away
    uint32_t *scr = nullptr;
    void *ctr = nullptr, *hctr = nullptr;
    cudaError_t e0 = cudaMalloc((void **)&scr, std::max<size_t>(3ull * n, 1) * 4);
    if (e0 == cudaSuccess) e0 = cudaMalloc(&ctr, 16);
    if (e0 == cudaSuccess) e0 = cudaMallocHost(&hctr, 16);
    int ce = e0 == cudaSuccess ? gpu_core_numbers(E->d_off, E->d_adj, n, E->d_core, scr, ctr,
                                                   hctr, E->num_sms, E->stream)
                               : (int)e0;
    E->g.core.resize(n);
    if (ce == 0 && n)
      ce = (int)cudaMemcpyAsync(E->g.core.data(), E->d_core, n * 4ull, cudaMemcpyDeviceToHost,
                                E->stream);
    if (ce == 0) ce = (int)cudaStreamSynchronize(E->stream);
    cudaFree(scr);
    cudaFree(ctr);
    if (hctr) cudaFreeHost(hctr);
    if (ce) return E->cuda_fail((cudaError_t)ce, "core numbers");
  }
  // slots
  E->nslots = c.limit_queries ? c.limit_queries : 64;
  E->slots.resize(E->nslots);
  E->h_slots.resize(E->nslots);
  RC(E->dalloc(&E->d_slots, E->nslots));
  SlotArrays &sa = E->sa;
  sa.stride_n = n;
  // a multiple of 4 words: every slot's rows start 16-byte aligned (rows are
  // read with 16-byte loads)
  sa.cap_adj = (nnz + 3ull * n + 4 + 3) & ~3ull;
  sa.wit_cap = CL_CAP;
  sa.max_local = std::min<uint32_t>(n, c.max_local ? c.max_local : MAX_LOCAL_DEFAULT);
  RC(E->dalloc(&sa.loc_off, (size_t)E->nslots * (n + 1), false));
  RC(E->dalloc(&sa.loc_adj, (size_t)E->nslots * sa.cap_adj, false));
  RC(E->dalloc(&sa.loc_dist, (size_t)E->nslots * n, false));
  RC(E->dalloc(&sa.loc_gid, (size_t)E->nslots * n, false));
  RC(E->dalloc(&sa.witness, (size_t)E->nslots * sa.wit_cap, false));
  // prep scratch
  E->prep_cap = std::min<uint32_t>(E->nslots, 256);
  PrepScratch &ps = E->ps;
  ps.stride_n = n;
  ps.stride_w = (n + 31) / 32 + 1;
  ps.big_row = c.prep_big_row ? c.prep_big_row : 4096;
  // a cluster per query on large graphs, where one SM's BFS and compaction
  // over the CSR would take a large share of the query's time
  E->prep_cluster = c.prep_ctas ? c.prep_ctas : (n >= (1u << 18) ? PREP_MAX_CLUSTER : 1u);
  RC(E->dalloc(&ps.dist, (size_t)E->prep_cap * n, false));
  RC(E->dalloc(&ps.vis, (size_t)E->prep_cap * ps.stride_w, false));
  RC(E->dalloc(&ps.comp, (size_t)E->prep_cap * ps.stride_w, false));
  RC(E->dalloc(&ps.fa, (size_t)E->prep_cap * n, false));
  RC(E->dalloc(&ps.fb, (size_t)E->prep_cap * n, false));
  RC(E->dalloc(&ps.wpre, (size_t)E->prep_cap * ps.stride_w, false));
  RC(E->dalloc(&ps.ldeg, (size_t)E->prep_cap * n, false));
  RC(E->dalloc(&E->d_jobs, E->prep_cap));
  // search grid and shared memory
  int max_optin = 0;
  CK(cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, E->dev));
  // CTAs per SM: several CTAs keep several tasks in flight per SM so one
  // task's serial phases overlap with the others' work.  The default is as
  // many as the kernel's registers allow; the shared memory left per CTA
  // then decides how many state words stay on chip.
  int occ_regs = 0;
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_regs, search_kernel, SEARCH_THREADS, 0));
  uint32_t cps = c.ctas_per_sm ? c.ctas_per_sm : (uint32_t)SEARCH_MINB;
  if (occ_regs >= 1) cps = std::min<uint32_t>(cps, (uint32_t)occ_regs);
  // The dynamic region gets what is left of the SM's shared memory per CTA
  // after the kernel's own static shared memory (as built, not estimated: a
  // few bytes too many silently cost a whole CTA per SM) and the per-block
  // reservation.
  cudaFuncAttributes fattr{};
  CK(cudaFuncGetAttributes(&fattr, search_kernel));
  int per_sm_i = 0, reserved_i = 0;
  CK(cudaDeviceGetAttribute(&per_sm_i, cudaDevAttrMaxSharedMemoryPerMultiprocessor, E->dev));
  CK(cudaDeviceGetAttribute(&reserved_i, cudaDevAttrReservedSharedMemoryPerBlock, E->dev));
  const size_t stat = fattr.sharedSizeBytes;
  const size_t per_cta = (size_t)per_sm_i / cps;
  size_t budget = std::min((size_t)max_optin + (size_t)reserved_i, per_cta);
  budget = budget > (size_t)reserved_i ? budget - (size_t)reserved_i : 0;
  size_t words = budget > stat ? (budget - stat) / 4 : 0;
  E->nw_smem = (uint32_t)std::min<size_t>(words, sa.max_local);
  E->smem_bytes = (size_t)E->nw_smem * 4;
  for (const void *k : {(const void *)search_kernel, (const void *)search_kernel_learned}) {
    CK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            (int)E->smem_bytes));
    CK(cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout,
                            (int)cudaSharedmemCarveoutMaxShared));
  }
  CK(cudaFuncSetAttribute(step_test_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                          (int)E->smem_bytes));
  int occ = 0;
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, search_kernel, SEARCH_THREADS,
                                                   E->smem_bytes));
  {
    int occ_l = 0;  // the learned variant must fit the same grid
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_l, search_kernel_learned,
                                                     SEARCH_THREADS, E->smem_bytes));
    occ = std::min(occ, occ_l);
  }
  if (occ < 1) {
    E->err = "search kernel does not fit on an SM";
    return SCS_ECUDA;
  }
  cps = std::min<uint32_t>(cps, (uint32_t)occ);
  E->grid = (uint32_t)E->num_sms * cps;
  E->stats[SCS_STAT_CTAS] = E->grid;
  E->stats[SCS_STAT_SMEM_WORDS] = E->nw_smem;
  // per-CTA scratch
  Scratch &sc = E->scr;
  // every per-task index is a local id or a list position, both below
  // the largest local graph: size the per-CTA arrays by that, not by n
  const uint32_t n_loc = sa.max_local;
  sc.stride = n_loc + 4;
  RC(E->dalloc(&sc.word, (size_t)E->grid * sc.stride));
  RC(E->dalloc(&sc.list, (size_t)E->grid * 2 * sc.stride, false));
  RC(E->dalloc(&sc.aux, (size_t)E->grid * sc.stride));
  RC(E->dalloc(&sc.tmp, (size_t)E->grid * 2 * sc.stride, false));
  RC(E->dalloc(&sc.cpos, (size_t)E->grid * sc.stride, false));
  RC(E->dalloc(&sc.dsc, (size_t)E->grid * 3 * sc.stride));  // zeroed: scores
  // stacks and pool: the task store is the engine's main memory consumer;
  // stacks get most of what is free (DFS records of the largest local graph),
  // the shared pool a quarter of the rest
  size_t free_b = 0, total_b = 0;
  CK(cudaMemGetInfo(&free_b, &total_b));
  uint64_t sw = c.stack_words;
  uint64_t pw = c.pool_words;
  uint64_t avail_words = (uint64_t)(free_b * 0.85) / 4;
  if (!pw) pw = std::min<uint64_t>(avail_words / 4, 1ull << 33);
  if (!sw) {
    uint64_t want = std::max<uint64_t>(1ull << 20, (uint64_t)(2 * n_loc + 5) * 4096);
    uint64_t cap = (avail_words - std::min(pw, avail_words)) / E->grid;
    sw = std::min(want, cap);
  }
  E->stk.words = sw;
  RC(E->dalloc(&E->stk.base, (size_t)E->grid * sw, false));
  RC(E->dalloc(&E->stk.top, E->grid));
  RC(E->dalloc(&E->stk.bot, E->grid));
  E->root_stride = 2ull * n_loc + 5;
  E->root_words = (unsigned long long)E->nslots * E->root_stride;
  E->pool.arena_cap = pw + E->root_words;
  RC(E->dalloc(&E->pool.arena, E->pool.arena_cap, false));
  RC(E->dalloc(&E->pool.arena_top, 1));
  // the bump area starts after the parked roots
  CK(cudaMemcpyAsync(E->pool.arena_top, &E->root_words, 8, cudaMemcpyHostToDevice, E->stream));
  E->pool_free = pw;
  RC(E->dalloc(&E->d_rel, E->nslots, false));
  RC(E->dalloc(&E->d_relq, E->nslots, false));
  RC(E->dalloc(&E->d_rel_next, 1));
  RC(E->dalloc(&E->d_rel_flag, E->nslots));
  // Queries searched at once.  Fewer keep the active local graphs in L2 (the
  // search is bound by dependent loads); enough must stay to feed every CTA
  // through donations.
  E->active_target = c.active_queries ? c.active_queries : SCS_DEFAULT_ACTIVE;
  E->stats[SCS_STAT_ACTIVE] = E->active_target;
  E->pool.desc_cap = 1u << 24;
  RC(E->dalloc(&E->pool.desc, E->pool.desc_cap));
  RC(E->dalloc(&E->pool.head, 1));
  RC(E->dalloc(&E->pool.tail, 1));
  RC(E->dalloc(&E->d_ctr, 1));
  CK(cudaStreamSynchronize(E->stream));
  E->host_threads = c.host_threads ? c.host_threads
                                   : std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  E->work.resize(E->host_threads);
  // greedy incumbents of submitted queries are computed by these workers
  for (unsigned k = 0; k < E->host_threads; k++) E->heu_workers.emplace_back(heu_worker, E, k);
  E->verifier = std::thread(verify_worker, E);
  return 0;
}

static SearchParams make_params(scs_engine *E) {
  SearchParams P{};
  P.g = DevGraph{E->g.n, E->g.dmax, E->d_off, E->d_adj, E->d_core};
  P.sa = E->sa;
  P.slots = E->d_slots;
  P.pool = E->pool;
  P.ctr = E->d_ctr;
  P.stk = E->stk;
  P.scr = E->scr;
  P.nw_smem = E->nw_smem;
  P.nslots = E->nslots;
  P.mlp = E->learned ? MlpDev{E->d_mlp_w, E->d_mlp_b} : MlpDev{nullptr, nullptr};
  P.trace_feat = E->d_trace_feat;
  P.trace_key = E->d_trace_key;
  P.trace_count = E->d_trace_count;
  P.trace_cap = E->trace_cap;
  P.trace_mask = E->trace_mask;
  return P;
}

// Hand a finished query to the verifier thread.
static void post_result(scs_engine *E, Done &&d) {
  {
    std::lock_guard<std::mutex> lk(E->res_mu);
    E->verify_q.push_back(std::move(d));
    E->res_pending++;
  }
  E->res_cv.notify_one();
}

// Verifier thread: checks each finished query's community (connected,
// contains q, l <= |H| <= h, minimum degree equal to the answer), sets
// h_verified and the latency, and makes the result visible to scs_poll.
static void verify_worker(scs_engine *E) {
  std::unique_lock<std::mutex> lk(E->res_mu);
  for (;;) {
    E->res_cv.wait(lk, [&] { return E->res_stop || !E->verify_q.empty(); });
    if (E->verify_q.empty()) return;  // stopping, nothing left
    Done d = std::move(E->verify_q.front());
    E->verify_q.pop_front();
    lk.unlock();
    uint32_t md = 0;
    const bool ok = d.check && verify_community(E->g, d.H.data(), (uint32_t)d.H.size(),
                                                d.r.q, d.r.l, d.r.h, md);
    d.r.h_verified = (ok && md == d.r.degree) ? 1u : 0u;
    d.r.latency_ns = now_ns() - d.t_submit;
    lk.lock();
    E->done.push_back(std::move(d));
    E->res_pending--;
    E->res_cv.notify_all();
  }
}

static void finish_result(scs_engine *E, uint32_t si, uint32_t degree,
                          int32_t status, uint64_t nodes, uint64_t search_ns,
                          const std::vector<uint32_t> &H) {
  SlotHost &sh = E->slots[si];
  Done d;
  d.r.ticket = sh.p.ticket;
  d.r.l = sh.p.q.l;
  d.r.h = sh.p.q.h;
  d.r.q = sh.p.q.q;
  d.r.degree = degree;
  d.r.status = status;
  d.r.kl_heuristic = sh.kl_heu;
  d.r.nodes = nodes;
  d.r.search_ns = search_ns;
  d.H = H;
  d.r.h_size = (uint32_t)H.size();
  d.t_submit = sh.p.t_submit;
  post_result(E, std::move(d));
  sh.busy = false;
  if (sh.parked) {  // a query whose preparation failed is never released
    sh.parked = false;
    E->n_parked--;
  }
}

// Finish queries answered without a search (bad input, heuristic hit).
static void finish_now(scs_engine *E, const Pending &p, uint32_t degree,
                       int32_t status, uint32_t kl_heu,
                       const std::vector<uint32_t> &H) {
  Done d;
  d.r.ticket = p.ticket;
  d.r.l = p.q.l;
  d.r.h = p.q.h;
  d.r.q = p.q.q;
  d.r.degree = degree;
  d.r.status = status;
  d.r.kl_heuristic = kl_heu;
  d.H = H;
  d.r.h_size = (uint32_t)H.size();
  d.t_submit = p.t_submit;
  d.check = status != SCS_BAD_QUERY;
  post_result(E, std::move(d));
}

// Admit queued queries into free slots; returns the number of prep jobs.
static int admit(scs_engine *E) {
  std::vector<uint32_t> free_slots;
  for (uint32_t i = 0; i < E->nslots; i++)
    if (!E->slots[i].busy) free_slots.push_back(i);
  // Admit the queued queries whose incumbents are ready, in queue order;
  // the others keep computing in the background while the admitted ones
  // search.  Only with nothing on the GPU does admission wait (for one).
  std::vector<std::shared_ptr<Job>> batch;
  {
    std::unique_lock<std::mutex> lk(E->heu_mu);
    if (E->running == 0 && !E->queue.empty()) {
      const uint64_t t0 = now_ns();
      auto any_done = [&] {
        for (auto &j : E->queue)
          if (j->done) return true;
        return false;
      };
      if (!E->heu_done_cv.wait_for(lk, std::chrono::minutes(10), any_done)) {
        E->err = "greedy incumbent workers made no progress for 10 minutes";
        return SCS_ESTALL;
      }
      E->stats[SCS_STAT_HEUR_NS] += now_ns() - t0;
    }
    for (auto it = E->queue.begin();
         it != E->queue.end() && batch.size() < free_slots.size() && batch.size() < E->prep_cap;) {
      if ((*it)->done) {
        batch.push_back(*it);
        it = E->queue.erase(it);
      } else {
        ++it;
      }
    }
  }
  if (batch.empty()) return 0;
  std::vector<PrepJob> jobs;
  std::vector<std::shared_ptr<Job>> searched;  // the jobs behind `jobs`
  size_t fs = 0;
  for (size_t i = 0; i < batch.size(); i++) {
    const Pending &p = batch[i]->p;
    Job &a = *batch[i];
    if (a.bad) {
      finish_now(E, p, 0, SCS_BAD_QUERY, 0, {});
      continue;
    }
    if (a.kl == a.ku || E->g.core[p.q.q] <= a.kl) {
      // the incumbent is optimal (main.cu:122-133), or no community better
      // than kl can contain q (core[q] <= kl)
      finish_now(E, p, a.kl, a.kl == a.ku ? SCS_HEURISTIC : SCS_DONE, a.kl, a.H);
      continue;
    }
    const uint32_t si = free_slots[fs++];
    PrepJob j{};
    j.slot = si;
    j.q = p.q.q;
    j.kl = a.kl;
    j.ubd = ubd_host(a.kl, p.q.h);
    j.l = p.q.l;
    j.h = p.q.h;
    j.limit_doms = std::min<uint32_t>(p.q.limit_doms, MAX_DOMS);
    j.rules = E->rules;
    j.kl_heu = a.kl;
    j.root_to_pool = 2;  // parked; release_kernel publishes it
    const unsigned long long roff = (unsigned long long)si * E->root_stride;
    j.root_off_lo = (uint32_t)roff;
    j.root_off_hi = (uint32_t)(roff >> 32);
    j.node_budget = E->cfg.node_budget;
    j.qtag = (uint32_t)p.ticket;
    jobs.push_back(j);
    searched.push_back(batch[i]);
  }
  if (jobs.empty()) return 0;
  // The copy, the events and the launch come before any slot changes state:
  // if one fails, the jobs go back to the head of the queue in their order
  // and no slot is left marked busy without a preparation behind it.
  auto requeue = [&](cudaError_t e, const char *what) {
    {
      std::lock_guard<std::mutex> lk(E->heu_mu);
      for (size_t k = searched.size(); k-- > 0;) E->queue.push_front(searched[k]);
    }
    return E->cuda_fail(e, what);
  };
  cudaError_t e = cudaMemcpyAsync(E->d_jobs, jobs.data(), jobs.size() * sizeof(PrepJob),
                                  cudaMemcpyHostToDevice, E->stream);
  if (e != cudaSuccess) return requeue(e, "prep job copy");
  e = cudaEventRecord(E->ev2, E->stream);
  if (e != cudaSuccess) return requeue(e, "prep start event");
  e = launch_prep(E->prep_cluster, E->stream,
                  DevGraph{E->g.n, E->g.dmax, E->d_off, E->d_adj, E->d_core}, E->sa,
                  E->d_slots, E->d_jobs, (int)jobs.size(), E->ps, E->pool, E->d_ctr);
  if (e != cudaSuccess) return requeue(e, "prep_kernel launch");
  if (E->learned) {
    // the network's incumbent proposal on each new local graph (propose.cu)
    propose_kernel<<<(unsigned)std::min<size_t>(jobs.size(), E->grid), 256, 0, E->stream>>>(
        DevGraph{E->g.n, E->g.dmax, E->d_off, E->d_adj, E->d_core}, E->sa, E->d_slots,
        E->d_jobs, (int)jobs.size(), E->scr, MlpDev{E->d_mlp_w, E->d_mlp_b}, E->d_ctr);
    e = cudaGetLastError();
    if (e != cudaSuccess) return requeue(e, "propose_kernel launch");
    E->stats[SCS_STAT_LAUNCHES]++;
  }
  E->stats[SCS_STAT_H2D] += jobs.size() * sizeof(PrepJob);
  E->stats[SCS_STAT_LAUNCHES]++;
  for (size_t k = 0; k < jobs.size(); k++) {
    const uint32_t si = jobs[k].slot;
    SlotHost &sh = E->slots[si];
    sh.busy = true;
    sh.p = searched[k]->p;
    sh.kl_heu = searched[k]->kl;
    sh.heuH = searched[k]->H;
    sh.parked = true;
    E->h_slots[si].n_local = 0;  // unknown until the next read-back
    E->parked.push_back(si);
    E->n_parked++;
  }
  E->running += (uint32_t)jobs.size();
  // the launch is in flight: a failed end event only loses its timing
  E->prep_pending = cudaEventRecord(E->ev3, E->stream) == cudaSuccess;
  if (!E->prep_pending) cudaGetLastError();
  return (int)jobs.size();
}

// one search slice + collection of finished slots
static int slice(scs_engine *E) {
  uint64_t t_us = E->cfg.slice_us ? E->cfg.slice_us : SCS_DEFAULT_SLICE_US;
  // release parked roots up to the active target
  {
    const uint32_t active = E->running - std::min(E->running, E->n_parked);
    const uint32_t need = E->active_target > active ? E->active_target - active : 0;
    std::vector<uint32_t> rel;
    E->devq.clear();
    if (E->n_parked && (need || !E->cfg.host_release_only)) {
      // candidates in admission order (entries of collected slots dropped).
      // A slot collected and admitted again before the deque was compacted
      // has two entries: each slot is taken once.
      std::vector<uint32_t> cand;
      std::vector<char> seen(E->nslots, 0);
      cand.reserve(E->parked.size());
      for (uint32_t si : E->parked)
        if (E->slots[si].parked && !seen[si]) {
          seen[si] = 1;
          cand.push_back(si);
        }
      if (E->cfg.release_order == 0 && cand.size() > need) {
        // shortest job first: the smallest local graphs, as read back after
        // the slice that followed their preparation (0 until then, so a
        // just-prepared query is not held back); ties keep admission order
        std::stable_sort(cand.begin(), cand.end(), [&](uint32_t a, uint32_t b) {
          return E->h_slots[a].n_local < E->h_slots[b].n_local;
        });
      }
      // Admission by free task-store memory: each released query claims
      // release_headroom records of its root's size from the pool's free
      // words (read back after the last slice).  With nothing searched, one
      // query goes regardless, so the engine always progresses.
      const unsigned long long head = E->cfg.release_headroom ? E->cfg.release_headroom : 4;
      unsigned long long budget = E->pool_free;
      bool held = false;
      uint32_t i = 0;
      for (; i < cand.size() && rel.size() < need; i++) {
        const uint32_t nl = E->h_slots[cand[i]].n_local;
        const unsigned long long claim =
            head * (2ull * (nl ? nl : E->sa.max_local) + 5);
        if (claim > budget && !(active == 0 && rel.empty())) {
          held = true;
          break;
        }
        budget -= std::min(budget, claim);
        E->slots[cand[i]].parked = false;
        E->n_parked--;
        rel.push_back(cand[i]);
      }
      // The next ones, as far as the pool's room goes, are queued for the
      // device: each time a searched query finishes inside the slice, the
      // finishing CTA releases the next (release_next in bnb.cu), so the
      // active set stays full between host round trips.
      if (!E->cfg.host_release_only && !held) {
        for (; i < cand.size(); i++) {
          const uint32_t nl = E->h_slots[cand[i]].n_local;
          const unsigned long long claim =
              head * (2ull * (nl ? nl : E->sa.max_local) + 5);
          if (claim > budget) break;
          budget -= claim;
          E->devq.push_back(cand[i]);
        }
      }
      if (held) E->stats[SCS_STAT_HELD_MEMORY]++;
      std::deque<uint32_t> keep;
      std::fill(seen.begin(), seen.end(), 0);
      for (uint32_t si : E->parked)
        if (E->slots[si].parked && !seen[si]) {
          seen[si] = 1;
          keep.push_back(si);
        }
      E->parked.swap(keep);
    }
    if (!rel.empty()) {
      CK(cudaMemcpyAsync(E->d_rel, rel.data(), rel.size() * 4, cudaMemcpyHostToDevice,
                         E->stream));
      release_kernel<<<1, 32, 0, E->stream>>>(E->d_slots, E->d_rel, (uint32_t)rel.size(),
                                              E->root_stride, E->pool, E->d_ctr);
      CK(cudaGetLastError());
      E->stats[SCS_STAT_LAUNCHES]++;
      E->stats[SCS_STAT_RELEASES] += rel.size();
      E->stats[SCS_STAT_H2D] += rel.size() * 4;
    }
    if (!E->devq.empty()) {
      CK(cudaMemcpyAsync(E->d_relq, E->devq.data(), E->devq.size() * 4, cudaMemcpyHostToDevice,
                         E->stream));
      CK(cudaMemsetAsync(E->d_rel_next, 0, 4, E->stream));
      CK(cudaMemsetAsync(E->d_rel_flag, 0, E->devq.size() * 4, E->stream));
      E->stats[SCS_STAT_H2D] += E->devq.size() * 4 + 4;
    }
  }
  SearchParams P = make_params(E);
  P.rel_queue = E->d_relq;
  P.rel_count = (uint32_t)E->devq.size();
  P.rel_next = E->d_rel_next;
  P.rel_flag = E->d_rel_flag;
  P.root_stride = E->root_stride;
  P.slice_ns = t_us * 1000ull;
  // per-slice fields: deadline (set by the first CTA), hungry, error,
  // done_count, stop
  CK(cudaMemsetAsync(&E->d_ctr->deadline, 0, 8, E->stream));
  CK(cudaMemsetAsync(&E->d_ctr->hungry, 0, sizeof(uint32_t) * 4, E->stream));
  // the learned variant when a model is loaded or the trace is on
  void (*kern)(SearchParams) =
      (E->learned || E->trace_cap) ? search_kernel_learned : search_kernel;
  // the dynamic shared-memory limit is per function, not per engine
  CK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                          (int)E->smem_bytes));
  CK(cudaEventRecord(E->ev0, E->stream));
  kern<<<E->grid, SEARCH_THREADS, E->smem_bytes, E->stream>>>(P);
  CK(cudaGetLastError());
  CK(cudaEventRecord(E->ev1, E->stream));
  E->stats[SCS_STAT_LAUNCHES]++;
  E->stats[SCS_STAT_SLICES]++;
  // read back slots and counters
  CK(cudaMemcpyAsync(E->h_slots.data(), E->d_slots, E->nslots * sizeof(Slot),
                     cudaMemcpyDeviceToHost, E->stream));
  Counters hc;
  CK(cudaMemcpyAsync(&hc, E->d_ctr, sizeof(Counters), cudaMemcpyDeviceToHost, E->stream));
  uint32_t ph[2];
  unsigned long long arena_used = 0;
  CK(cudaMemcpyAsync(ph, E->pool.head, 4, cudaMemcpyDeviceToHost, E->stream));
  CK(cudaMemcpyAsync(ph + 1, E->pool.tail, 4, cudaMemcpyDeviceToHost, E->stream));
  CK(cudaMemcpyAsync(&arena_used, E->pool.arena_top, 8, cudaMemcpyDeviceToHost, E->stream));
  std::vector<uint32_t> rel_flag(E->devq.size());
  if (!E->devq.empty()) {
    CK(cudaMemcpyAsync(rel_flag.data(), E->d_rel_flag, rel_flag.size() * 4,
                       cudaMemcpyDeviceToHost, E->stream));
    E->stats[SCS_STAT_D2H] += rel_flag.size() * 4;
  }
  CK(cudaStreamSynchronize(E->stream));
  float ms = 0;
  cudaEventElapsedTime(&ms, E->ev0, E->ev1);
  E->stats[SCS_STAT_SEARCH_NS] += (uint64_t)(ms * 1e6);
  // roots the device released during the slice are no longer parked (before
  // collection: such a query may also have finished in this slice)
  for (size_t i = 0; i < rel_flag.size(); i++) {
    if (rel_flag[i] != 1) continue;
    SlotHost &rs = E->slots[E->devq[i]];
    if (rs.parked) {
      rs.parked = false;
      E->n_parked--;
      E->stats[SCS_STAT_RELEASES]++;
      E->stats[SCS_STAT_DEVICE_RELEASES]++;
    }
  }
  if (E->prep_pending) {
    float pm = 0;
    cudaEventElapsedTime(&pm, E->ev2, E->ev3);
    E->stats[SCS_STAT_PREP_NS] += (uint64_t)(pm * 1e6);
    E->prep_pending = false;
  }
  E->stats[SCS_STAT_BYTES] = hc.bytes;
  for (int i = 0; i < 8; i++) E->prof[i] = hc.phase_cycles[i];
  E->prof[8] = hc.r12_rounds;
  E->prof[9] = hc.r3_rounds;
  E->prof[10] = hc.steps;
  for (int i = 0; i < 3; i++) {
    E->prof[11 + i] = hc.sub_cycles[i];
  }
  E->prof[14] = hc.sub_counts[0];
  E->prof[15] = hc.sub_counts[1];
  E->stats[SCS_STAT_D2H] += E->nslots * sizeof(Slot) + sizeof(Counters) + 8;
  E->stats[SCS_STAT_H2D] += 24;
  E->stats[SCS_STAT_NODES] = hc.nodes;
  E->stats[SCS_STAT_DONATIONS] = hc.donations;
  E->stats[SCS_STAT_STEALS] = hc.steals;
  E->stats[SCS_STAT_SPILLS] = hc.spills;
  E->stats[SCS_STAT_SLIDES] = hc.slides;
  E->stats[SCS_STAT_PROPOSALS_BETTER] = hc.proposals_better;
  E->stats[SCS_STAT_PREP_BYTES] = hc.prep_bytes;
  if (hc.error) {
    E->err = "device error flags " + std::to_string(hc.error) + " info " +
             std::to_string(hc.err_info[0]) + "," + std::to_string(hc.err_info[1]) + "," +
             std::to_string(hc.err_info[2]) + "," + std::to_string(hc.err_info[3]);
    fprintf(stderr, "scs: %s\n", E->err.c_str());
    if (hc.error & (ERR_RECORD | ERR_SPIN)) return SCS_ECUDA;
    E->stats[SCS_STAT_ERRORS] |= hc.error;
  }
  // collect finished slots
  for (uint32_t i = 0; i < E->nslots; i++) {
    SlotHost &sh = E->slots[i];
    const Slot &s = E->h_slots[i];
    if (!sh.busy || s.state != SLOT_DONE) continue;
    uint32_t degree = s.kl;
    std::vector<uint32_t> H;
    uint32_t wv = s.wit_val ? s.wit_val - 1 : 0;
    if (s.wit_val && wv == degree && s.wit_n) {
      H.resize(s.wit_n);
      CK(cudaMemcpy(H.data(), E->sa.witness + (size_t)i * E->sa.wit_cap,
                    s.wit_n * 4ull, cudaMemcpyDeviceToHost));
      E->stats[SCS_STAT_D2H] += s.wit_n * 4ull;
    } else {
      H = sh.heuH;
    }
    int32_t st = (int32_t)s.status;
    uint64_t sns = s.t_done > s.t_admit ? s.t_done - s.t_admit : 0;
    finish_result(E, i, degree, st, s.nodes, sns, H);
    Slot clear{};
    CK(cudaMemcpyAsync(E->d_slots + i, &clear, sizeof(Slot), cudaMemcpyHostToDevice, E->stream));
    E->stats[SCS_STAT_H2D] += sizeof(Slot);
    E->running--;
  }
  // pool reset when fully drained: every published record taken, and
  // something allocated (failed reservations also advance arena_top, so a
  // full arena with nothing published is reset too)
  E->pool_free = E->pool.arena_cap > arena_used ? E->pool.arena_cap - arena_used : 0;
  if (ph[0] >= std::min(ph[1], E->pool.desc_cap) && (ph[1] > 0 || arena_used > E->root_words)) {
    uint32_t used = std::min(ph[1], E->pool.desc_cap);
    CK(cudaMemsetAsync(E->pool.desc, 0, used * 8ull, E->stream));
    // the bump area restarts after the parked roots, which stay in place
    CK(cudaMemcpyAsync(E->pool.arena_top, &E->root_words, 8, cudaMemcpyHostToDevice,
                       E->stream));
    E->pool_free = E->pool.arena_cap - E->root_words;
    CK(cudaMemsetAsync(E->pool.head, 0, 4, E->stream));
    CK(cudaMemsetAsync(E->pool.tail, 0, 4, E->stream));
  }
  E->stats[SCS_STAT_POOL_FREE] = E->pool_free;
  CK(cudaStreamSynchronize(E->stream));
  return 0;
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

static int create_common(scs_engine **out, scs_engine *E, const scs_config *cfg) {
  if (cfg) E->cfg = *cfg;
  int rc = engine_init(E);
  if (rc) {
    g_create_error = E->err;
    scs_destroy(E);
    *out = nullptr;
    return rc;
  }
  *out = E;
  return 0;
}

int scs_create(scs_engine **out, const char *path, const scs_config *cfg) {
  if (!out || !path) return SCS_EINVAL;
  scs_engine *E = new scs_engine();
  int rc = load_edge_list(path, E->g, E->err, /*with_core=*/false);
  if (rc) {
    g_create_error = E->err;
    delete E;
    *out = nullptr;
    return SCS_EIO;
  }
  return create_common(out, E, cfg);
}

int scs_create_csr(scs_engine **out, uint32_t n, const uint32_t *off,
                   const uint32_t *adj, const scs_config *cfg) {
  if (!out) return SCS_EINVAL;
  scs_engine *E = new scs_engine();
  if (adopt_csr(n, off, adj, E->g, E->err, /*with_core=*/false)) {
    g_create_error = E->err;
    delete E;
    *out = nullptr;
    return SCS_EINVAL;
  }
  return create_common(out, E, cfg);
}

int scs_graph_info(scs_engine *E, uint32_t *n, uint64_t *nnz, uint32_t *dmax) {
  if (!E) return SCS_EINVAL;
  if (n) *n = E->g.n;
  if (nnz) *nnz = E->g.adj.size();
  if (dmax) *dmax = E->g.dmax;
  return 0;
}

int scs_core_numbers(scs_engine *E, uint32_t *core) {
  if (!E || !core) return SCS_EINVAL;
  std::copy(E->g.core.begin(), E->g.core.end(), core);
  return 0;
}

int scs_submit(scs_engine *E, const scs_query *q, uint64_t *ticket) {
  if (!E || !q) return SCS_EINVAL;
  // May run on any thread while another one steps the engine: the ticket,
  // the admission queue and the workers' queue change under heu_mu, which
  // admission holds while it walks the queue.
  auto j = std::make_shared<Job>();
  j->p.q = *q;
  j->p.t_submit = now_ns();
  const bool bad = q->q >= E->g.n || q->h < 1 || q->h >= CL_CAP - 1 || q->l > q->h;
  bool work = false;
  if (bad) {
    j->bad = true;
    j->done = true;
  } else {
    j->ku = std::min(E->g.core[q->q], q->h - 1);
    if (!q->heuristic) j->done = true;  // kl = 0
    else work = true;
  }
  {
    std::lock_guard<std::mutex> lk(E->heu_mu);
    j->p.ticket = E->next_ticket++;
    if (work) E->heu_todo.push_back(j);
    E->queue.push_back(j);
  }
  if (work) E->heu_cv.notify_one();
  if (ticket) *ticket = j->p.ticket;
  return 0;
}

int scs_step(scs_engine *E) {
  if (!E) return SCS_EINVAL;
  int a = admit(E);
  if (a < 0) return a;
  if (E->running > 0) RC(slice(E));
  size_t queued, checking;
  {
    std::lock_guard<std::mutex> lk(E->heu_mu);
    queued = E->queue.size();
  }
  {
    std::unique_lock<std::mutex> lk(E->res_mu);
    // with nothing left to search, wait for the last checks so that a run
    // to completion ends with every result pollable
    if (queued + E->running == 0)
      E->res_cv.wait(lk, [&] { return E->res_pending == 0; });
    checking = E->res_pending;
  }
  return (int)(queued + E->running + checking);
}

int scs_run(scs_engine *E) {
  if (!E) return SCS_EINVAL;
  for (;;) {
    int r = scs_step(E);
    if (r < 0) return r;
    if (r == 0) return 0;
  }
}

int scs_poll(scs_engine *E, scs_result *out, int max, uint32_t *h_buf,
             uint32_t h_stride) {
  if (!E || (!out && max > 0)) return SCS_EINVAL;
  int k = 0;
  std::lock_guard<std::mutex> lk(E->res_mu);
  while (k < max && !E->done.empty()) {
    Done &d = E->done.front();
    out[k] = d.r;
    if (h_buf) {
      uint32_t c = std::min<uint32_t>(d.r.h_size, h_stride);
      std::copy(d.H.begin(), d.H.begin() + c, h_buf + (size_t)k * h_stride);
    }
    E->done.pop_front();
    k++;
  }
  return k;
}

int scs_stats(scs_engine *E, uint64_t *out) {
  if (!E || !out) return SCS_EINVAL;
  std::copy(E->stats, E->stats + SCS_STAT_COUNT, out);
  return 0;
}

int scs_profile(scs_engine *E, uint64_t *out) {
  if (!E || !out) return SCS_EINVAL;
  std::copy(E->prof, E->prof + 16, out);
  return 0;
}

const char *scs_last_error(scs_engine *E) {
  return E ? E->err.c_str() : g_create_error.c_str();
}

int scs_destroy(scs_engine *E) {
  if (!E) return SCS_EINVAL;
  {
    std::lock_guard<std::mutex> lk(E->heu_mu);
    E->heu_stop = true;
  }
  E->heu_cv.notify_all();
  for (auto &t : E->heu_workers) t.join();
  {
    std::lock_guard<std::mutex> lk(E->res_mu);
    E->res_stop = true;
  }
  E->res_cv.notify_all();
  if (E->verifier.joinable()) E->verifier.join();
  if (E->stream) cudaStreamSynchronize(E->stream);
  for (void *p : E->allocs) cudaFree(p);
  cudaFree(E->d_mlp_w);
  cudaFree(E->d_mlp_b);
  cudaFree(E->d_trace_feat);
  cudaFree(E->d_trace_key);
  cudaFree(E->d_trace_count);
  if (E->ev0) cudaEventDestroy(E->ev0);
  if (E->ev1) cudaEventDestroy(E->ev1);
  if (E->ev2) cudaEventDestroy(E->ev2);
  if (E->ev3) cudaEventDestroy(E->ev3);
  if (E->stream) cudaStreamDestroy(E->stream);
  delete E;
  return 0;
}

// ---- learned branching ----

int scs_load_model(scs_engine *E, const char *path) {
  if (!E) return SCS_EINVAL;
  if (E->running) {
    E->err = "scs_load_model needs an idle engine";
    return SCS_EBUSY;
  }
  if (!path) {  // back to the plain method
    E->learned = false;
    return 0;
  }
  FILE *f = fopen(path, "rb");
  if (!f) {
    E->err = std::string("cannot open model file ") + path;
    return SCS_EIO;
  }
  char magic[8] = {0};
  uint32_t dims[4] = {0, 0, 0, 0};
  std::vector<float> params(MLP_NPARAM);
  const bool ok = fread(magic, 1, 8, f) == 8 && memcmp(magic, "SCSMLP01", 8) == 0 &&
                  fread(dims, 4, 4, f) == 4 && dims[0] == (uint32_t)MLP_IN &&
                  dims[1] == (uint32_t)MLP_H && dims[2] == (uint32_t)MLP_H && dims[3] == 1 &&
                  fread(params.data(), 4, MLP_NPARAM, f) == (size_t)MLP_NPARAM;
  fclose(f);
  if (!ok) {
    E->err = std::string("not a 16-128-128-1 model file: ") + path;
    return SCS_EIO;
  }
  for (float x : params)
    if (!std::isfinite(x)) {
      E->err = "model file holds a non-finite parameter";
      return SCS_EINVAL;
    }
  std::vector<uint32_t> packed;
  std::vector<float> bias;
  mlp_pack(params.data(), packed, bias);
  CK(cudaSetDevice(E->dev));
  if (!E->d_mlp_w) CK(cudaMalloc((void **)&E->d_mlp_w, packed.size() * 4));
  if (!E->d_mlp_b) CK(cudaMalloc((void **)&E->d_mlp_b, bias.size() * 4));
  CK(cudaMemcpyAsync(E->d_mlp_w, packed.data(), packed.size() * 4, cudaMemcpyHostToDevice,
                     E->stream));
  CK(cudaMemcpyAsync(E->d_mlp_b, bias.data(), bias.size() * 4, cudaMemcpyHostToDevice,
                     E->stream));
  CK(cudaStreamSynchronize(E->stream));
  E->stats[SCS_STAT_H2D] += packed.size() * 4 + bias.size() * 4;
  E->learned = true;
  return 0;
}

int scs_trace_enable(scs_engine *E, uint64_t max_records, uint32_t sample_shift) {
  if (!E || sample_shift > 20) return SCS_EINVAL;
  if (E->running) return SCS_EBUSY;
  CK(cudaSetDevice(E->dev));
  CK(cudaStreamSynchronize(E->stream));
  cudaFree(E->d_trace_feat);
  cudaFree(E->d_trace_key);
  E->d_trace_feat = nullptr;
  E->d_trace_key = nullptr;
  E->trace_cap = 0;
  if (!max_records) return 0;
  CK(cudaMalloc((void **)&E->d_trace_feat, max_records * MLP_IN * 4ull));
  CK(cudaMalloc((void **)&E->d_trace_key, max_records * 8ull));
  if (!E->d_trace_count) CK(cudaMalloc((void **)&E->d_trace_count, 8));
  CK(cudaMemsetAsync(E->d_trace_count, 0, 8, E->stream));
  CK(cudaStreamSynchronize(E->stream));
  E->trace_cap = max_records;
  E->trace_mask = (1u << sample_shift) - 1u;
  return 0;
}

int scs_trace_read(scs_engine *E, float *feat, uint32_t *keys, uint64_t max,
                   uint64_t *written) {
  if (!E || !written) return SCS_EINVAL;
  *written = 0;
  if (!E->trace_cap) return 0;
  unsigned long long cnt = 0;
  CK(cudaMemcpyAsync(&cnt, E->d_trace_count, 8, cudaMemcpyDeviceToHost, E->stream));
  CK(cudaStreamSynchronize(E->stream));
  *written = cnt;
  const uint64_t n = std::min<uint64_t>(std::min<uint64_t>(cnt, E->trace_cap), max);
  if (n && feat)
    CK(cudaMemcpy(feat, E->d_trace_feat, n * MLP_IN * 4ull, cudaMemcpyDeviceToHost));
  if (n && keys) CK(cudaMemcpy(keys, E->d_trace_key, n * 8ull, cudaMemcpyDeviceToHost));
  return (int)std::min<uint64_t>(n, (uint64_t)INT32_MAX);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// test hooks
// ---------------------------------------------------------------------------
extern "C" {

int scs_debug_prepare(scs_engine *E, uint32_t nq, const scs_query *qs,
                      const uint32_t *kl, const uint32_t *ubd,
                      uint32_t *n_local, uint32_t *q_local) {
  if (!E || !qs || !kl || !ubd) return SCS_EINVAL;
  if (nq > E->nslots || nq > E->prep_cap || E->running) return SCS_EBUSY;
  std::vector<PrepJob> jobs(nq);
  for (uint32_t i = 0; i < nq; i++) {
    if (qs[i].q >= E->g.n || qs[i].h < 1 || qs[i].h >= CL_CAP - 1) return SCS_EINVAL;
    PrepJob &j = jobs[i];
    j = PrepJob{};
    j.slot = i;
    j.q = qs[i].q;
    j.kl = kl[i];
    j.ubd = ubd[i];
    j.l = qs[i].l;
    j.h = qs[i].h;
    j.limit_doms = std::min<uint32_t>(qs[i].limit_doms, MAX_DOMS);
    j.rules = E->rules;
    j.kl_heu = kl[i];
    j.root_to_pool = 0;
  }
  CK(cudaMemcpyAsync(E->d_jobs, jobs.data(), nq * sizeof(PrepJob),
                     cudaMemcpyHostToDevice, E->stream));
  CK(launch_prep(E->prep_cluster, E->stream,
                 DevGraph{E->g.n, E->g.dmax, E->d_off, E->d_adj, E->d_core}, E->sa,
                 E->d_slots, E->d_jobs, (int)nq, E->ps, E->pool, E->d_ctr));
  CK(cudaMemcpyAsync(E->h_slots.data(), E->d_slots, nq * sizeof(Slot),
                     cudaMemcpyDeviceToHost, E->stream));
  CK(cudaStreamSynchronize(E->stream));
  for (uint32_t i = 0; i < nq; i++) {
    if (n_local) n_local[i] = E->h_slots[i].n_local;
    if (q_local) q_local[i] = E->h_slots[i].q_local;
    if (E->h_slots[i].status == RS_TOO_LARGE) return SCS_EINVAL;
  }
  return 0;
}

// Local graph of a prepared slot with padding removed.
int scs_debug_local_graph(scs_engine *E, uint32_t slot, uint32_t *gid,
                          uint32_t *off, uint32_t *adj, uint32_t *dist) {
  if (!E || slot >= E->nslots) return SCS_EINVAL;
  CK(cudaMemcpy(&E->h_slots[slot], E->d_slots + slot, sizeof(Slot), cudaMemcpyDeviceToHost));
  const uint32_t nl = E->h_slots[slot].n_local;
  const uint32_t n = E->g.n;
  std::vector<uint32_t> loff(nl + 1);
  CK(cudaMemcpy(loff.data(), E->sa.loc_off + (size_t)slot * (n + 1), (nl + 1) * 4ull,
                cudaMemcpyDeviceToHost));
  std::vector<uint32_t> ladj(loff[nl]);
  if (loff[nl])
    CK(cudaMemcpy(ladj.data(), E->sa.loc_adj + (size_t)slot * E->sa.cap_adj,
                  loff[nl] * 4ull, cudaMemcpyDeviceToHost));
  if (gid)
    CK(cudaMemcpy(gid, E->sa.loc_gid + (size_t)slot * n, nl * 4ull, cudaMemcpyDeviceToHost));
  if (dist) {
    std::vector<uint16_t> d16(nl);
    CK(cudaMemcpy(d16.data(), E->sa.loc_dist + (size_t)slot * n, nl * 2ull,
                  cudaMemcpyDeviceToHost));
    for (uint32_t i = 0; i < nl; i++) dist[i] = d16[i] == INF16 ? 1000000000u : d16[i];
  }
  uint64_t w = 0;
  if (off) off[0] = 0;
  for (uint32_t i = 0; i < nl; i++) {
    for (uint32_t k = loff[i]; k < loff[i + 1]; k++)
      if (ladj[k] != SENT) {
        if (adj) adj[w] = ladj[k];
        w++;
      }
    if (off) off[i + 1] = (uint32_t)w;
  }
  return 0;
}

// One deterministic step per task on prepared slots.  Task entries are
// (local_id<<1)|inC, ascending; the input degrees are computed here from the
// slot's local graph.
}  // extern "C"

// Task records (with in-task degrees recounted on the host) for the given
// tasks of prepared slots, for the one-step test kernel.
static int build_test_records(scs_engine *E, uint32_t ntasks, const uint32_t *task_slot,
                              const uint64_t *task_off, const uint32_t *task_len,
                              const uint32_t *task_entries, std::vector<uint32_t> &recs,
                              std::vector<unsigned long long> &roff) {
  const uint32_t n = E->g.n;
  std::vector<std::vector<uint32_t>> loff(E->nslots), ladj(E->nslots);
  for (uint32_t t = 0; t < ntasks; t++) {
    uint32_t s = task_slot[t];
    if (s >= E->nslots) return SCS_EINVAL;
    if (!loff[s].empty()) continue;
    CK(cudaMemcpy(&E->h_slots[s], E->d_slots + s, sizeof(Slot), cudaMemcpyDeviceToHost));
    uint32_t nl = E->h_slots[s].n_local;
    std::vector<uint32_t> o(nl + 1);
    int rc = scs_debug_local_graph(E, s, nullptr, o.data(), nullptr, nullptr);
    if (rc) return rc;
    std::vector<uint32_t> aa(o[nl] + 1);
    rc = scs_debug_local_graph(E, s, nullptr, o.data(), aa.data(), nullptr);
    if (rc) return rc;
    loff[s] = o;
    ladj[s] = aa;
  }
  recs.clear();
  roff.assign(ntasks, 0);
  std::vector<int32_t> pos(n, -1);
  for (uint32_t t = 0; t < ntasks; t++) {
    uint32_t s = task_slot[t], len = task_len[t];
    const uint32_t *e = task_entries + task_off[t];
    roff[t] = recs.size();
    recs.resize(recs.size() + 2 * len + 5);
    uint32_t *r = recs.data() + roff[t];
    uint32_t cs = 0;
    for (uint32_t i = 0; i < len; i++) pos[e[i] >> 1] = (int32_t)i;
    for (uint32_t i = 0; i < len; i++) {
      uint32_t v = e[i] >> 1, dc = 0, dr = 0;
      cs += e[i] & 1u;
      for (uint32_t k = loff[s][v]; k < loff[s][v + 1]; k++) {
        int32_t jj = pos[ladj[s][k]];
        if (jj >= 0) {
          if (e[jj] & 1u) dc++;
          else dr++;
        }
      }
      r[REC_HDR + i] = e[i];
      r[REC_HDR + len + i] = (dc << DC_SHIFT) | dr;
    }
    for (uint32_t i = 0; i < len; i++) pos[e[i] >> 1] = -1;
    r[0] = s;
    r[1] = len;
    r[2] = cs;
    r[3] = 2 * len + 5;
    r[REC_HDR + 2 * len] = 2 * len + 5;
  }
  return 0;
}

// Device buffers of a one-step test run (freed on destruction).
struct TestBufs {
  std::vector<void *> p;
  template <class T>
  bool get(T **ptr, size_t count) {
    if (cudaMalloc((void **)ptr, std::max<size_t>(count, 1) * sizeof(T)) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    p.push_back(*ptr);
    return true;
  }
  ~TestBufs() {
    for (void *q : p) cudaFree(q);
  }
};

extern "C" {

int scs_debug_step(scs_engine *E, uint32_t ntasks, const uint32_t *task_slot,
                   const uint32_t *kl_in, const uint64_t *task_off,
                   const uint32_t *task_len, const uint32_t *task_entries,
                   uint32_t *out_hdr, uint32_t *out_doms, uint32_t doms_stride,
                   uint32_t *out_kids, uint64_t kids_stride, uint32_t *out_wit,
                   uint32_t wit_stride, const uint32_t *force, uint32_t *out_sl,
                   float *out_sl_feat) {
  if (!E || !ntasks) return SCS_EINVAL;
  if (wit_stride < CL_CAP + 1 || doms_stride < MAX_DOMS) return SCS_EINVAL;
  std::vector<uint32_t> recs;
  std::vector<unsigned long long> roff;
  RC(build_test_records(E, ntasks, task_slot, task_off, task_len, task_entries, recs, roff));
  const uint32_t chunk = E->grid;
  TestBufs B;
  uint32_t *d_rec, *d_hdr, *d_doms, *d_kids, *d_wit, *d_kl, *d_force = nullptr, *d_sl = nullptr;
  float *d_slf = nullptr;
  unsigned long long *d_roff;
  if (!B.get(&d_rec, recs.size()) || !B.get(&d_roff, ntasks) || !B.get(&d_hdr, 16ull * chunk) ||
      !B.get(&d_doms, (size_t)doms_stride * chunk) || !B.get(&d_kids, kids_stride * chunk) ||
      !B.get(&d_wit, (size_t)wit_stride * chunk) || !B.get(&d_kl, ntasks) ||
      (force && !B.get(&d_force, ntasks)) ||
      (out_sl && !B.get(&d_sl, (size_t)(MLP_TILE + 1) * chunk)) ||
      (out_sl_feat && !B.get(&d_slf, (size_t)MLP_TILE * MLP_IN * chunk))) {
    E->err = "debug step allocation failed";
    return SCS_ENOMEM;
  }
  CK(cudaMemcpy(d_rec, recs.data(), recs.size() * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_roff, roff.data(), ntasks * 8ull, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_kl, kl_in, ntasks * 4ull, cudaMemcpyHostToDevice));
  if (force) CK(cudaMemcpy(d_force, force, ntasks * 4ull, cudaMemcpyHostToDevice));
  for (uint32_t base = 0; base < ntasks; base += chunk) {
    uint32_t cnt = std::min(chunk, ntasks - base);
    CK(cudaMemset(d_hdr, 0, 16ull * chunk * 4));
    CK(cudaMemset(d_wit, 0, (size_t)wit_stride * chunk * 4));
    if (d_sl) CK(cudaMemset(d_sl, 0, (size_t)(MLP_TILE + 1) * chunk * 4));
    SearchParams P = make_params(E);
    P.t_rec = d_rec;
    P.t_rec_off = d_roff + base;
    P.t_ntasks = cnt;
    P.t_hdr = d_hdr;
    P.t_doms = d_doms;
    P.t_doms_stride = doms_stride;
    P.t_kids = d_kids;
    P.t_kids_stride = kids_stride;
    P.t_wit = d_wit;
    P.t_wit_stride = wit_stride;
    P.t_kl = d_kl + base;
    P.t_force = d_force ? d_force + base : nullptr;
    P.t_sl = d_sl;
    P.t_sl_feat = d_slf;
    if (d_sl && !d_slf) {
      E->err = "the shortlist needs its feature buffer";
      return SCS_EINVAL;
    }
    CK(cudaFuncSetAttribute(step_test_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            (int)E->smem_bytes));
    step_test_kernel<<<cnt, SEARCH_THREADS, E->smem_bytes, E->stream>>>(P);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(E->stream));
    CK(cudaMemcpy(out_hdr + 16ull * base, d_hdr, 16ull * cnt * 4, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(out_doms + (size_t)doms_stride * base, d_doms, (size_t)doms_stride * cnt * 4,
                  cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(out_kids + kids_stride * base, d_kids, kids_stride * cnt * 4,
                  cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(out_wit + (size_t)wit_stride * base, d_wit, (size_t)wit_stride * cnt * 4,
                  cudaMemcpyDeviceToHost));
    if (out_sl)
      CK(cudaMemcpy(out_sl + (size_t)(MLP_TILE + 1) * base, d_sl,
                    (size_t)(MLP_TILE + 1) * cnt * 4, cudaMemcpyDeviceToHost));
    if (out_sl_feat)
      CK(cudaMemcpy(out_sl_feat + (size_t)MLP_TILE * MLP_IN * base, d_slf,
                    (size_t)MLP_TILE * MLP_IN * cnt * 4, cudaMemcpyDeviceToHost));
  }
  return 0;
}

int scs_debug_lookahead(scs_engine *E, uint32_t ntasks, const uint32_t *task_slot,
                        const uint32_t *kl_in, const uint64_t *task_off,
                        const uint32_t *task_len, const uint32_t *task_entries,
                        const uint32_t *force, uint32_t *out_hdr, uint32_t *out_nkids,
                        uint32_t *out_branching, uint64_t *out_cost) {
  if (!E || !ntasks || !force || !out_hdr || !out_nkids || !out_branching || !out_cost)
    return SCS_EINVAL;
  std::vector<uint32_t> recs;
  std::vector<unsigned long long> roff;
  RC(build_test_records(E, ntasks, task_slot, task_off, task_len, task_entries, recs, roff));
  uint32_t maxlen = 1;
  for (uint32_t t = 0; t < ntasks; t++) maxlen = std::max(maxlen, task_len[t]);
  const uint64_t kstride = (uint64_t)(MAX_DOMS + 2) * (2ull * maxlen + 5);
  const uint32_t chunk = std::min<uint32_t>(E->grid, 128);
  const uint32_t koff_stride = MAX_DOMS + 3;
  TestBufs B;
  uint32_t *d_rec, *d_hdr, *d_doms, *d_kids, *d_wit, *d_kl, *d_force, *d_koff, *d_ckl,
      *d_chdr;
  unsigned long long *d_roff, *d_croff;
  const uint32_t cmax = chunk * (MAX_DOMS + 2);
  if (!B.get(&d_rec, recs.size()) || !B.get(&d_roff, ntasks) || !B.get(&d_hdr, 16ull * chunk) ||
      !B.get(&d_doms, (size_t)MAX_DOMS * cmax) || !B.get(&d_kids, kstride * chunk) ||
      !B.get(&d_wit, (size_t)(CL_CAP + 1) * cmax) || !B.get(&d_kl, ntasks) ||
      !B.get(&d_force, ntasks) || !B.get(&d_koff, (size_t)koff_stride * chunk) ||
      !B.get(&d_ckl, cmax) || !B.get(&d_chdr, 16ull * cmax) || !B.get(&d_croff, cmax)) {
    E->err = "lookahead allocation failed";
    return SCS_ENOMEM;
  }
  CK(cudaMemcpy(d_rec, recs.data(), recs.size() * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_roff, roff.data(), ntasks * 8ull, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_kl, kl_in, ntasks * 4ull, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_force, force, ntasks * 4ull, cudaMemcpyHostToDevice));
  CK(cudaFuncSetAttribute(step_test_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                          (int)E->smem_bytes));
  std::vector<uint32_t> hdr(16ull * chunk), koff((size_t)koff_stride * chunk);
  std::vector<unsigned long long> croff;
  std::vector<uint32_t> ckl, cparent, chdr;
  for (uint32_t base = 0; base < ntasks; base += chunk) {
    const uint32_t cnt = std::min(chunk, ntasks - base);
    CK(cudaMemset(d_hdr, 0, 16ull * chunk * 4));
    CK(cudaMemset(d_wit, 0, (size_t)(CL_CAP + 1) * chunk * 4));
    // 1. the forced step of each task, children written as task records
    SearchParams P = make_params(E);
    P.t_rec = d_rec;
    P.t_rec_off = d_roff + base;
    P.t_ntasks = cnt;
    P.t_hdr = d_hdr;
    P.t_doms = d_doms;
    P.t_doms_stride = MAX_DOMS;
    P.t_kids = d_kids;
    P.t_kids_stride = kstride;
    P.t_wit = d_wit;
    P.t_wit_stride = CL_CAP + 1;
    P.t_kl = d_kl + base;
    P.t_force = d_force + base;
    P.t_kids_rec = 1;
    P.t_kid_off = d_koff;
    step_test_kernel<<<cnt, SEARCH_THREADS, E->smem_bytes, E->stream>>>(P);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(E->stream));
    CK(cudaMemcpy(hdr.data(), d_hdr, 16ull * cnt * 4, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(koff.data(), d_koff, (size_t)koff_stride * cnt * 4, cudaMemcpyDeviceToHost));
    croff.clear();
    ckl.clear();
    cparent.clear();
    for (uint32_t i = 0; i < cnt; i++) {
      const uint32_t *h = hdr.data() + 16 * i;
      std::copy(h, h + 16, out_hdr + 16ull * (base + i));
      out_nkids[base + i] = h[0] == 0 ? h[9] : 0;
      out_branching[base + i] = 0;
      out_cost[base + i] = 0;
      if (h[0] != 0) continue;
      for (uint32_t j = 0; j < h[9] && j < MAX_DOMS + 2; j++) {
        croff.push_back((unsigned long long)i * kstride + koff[(size_t)koff_stride * i + j]);
        ckl.push_back(h[1]);  // the incumbent after the parent's step
        cparent.push_back(base + i);
      }
    }
    if (croff.empty()) continue;
    // 2. one step on every child (no children of theirs written)
    const uint32_t nc = (uint32_t)croff.size();
    CK(cudaMemcpy(d_croff, croff.data(), nc * 8ull, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_ckl, ckl.data(), nc * 4ull, cudaMemcpyHostToDevice));
    CK(cudaMemset(d_chdr, 0, 16ull * nc * 4));
    CK(cudaMemset(d_wit, 0, (size_t)(CL_CAP + 1) * std::min(nc, cmax) * 4));
    for (uint32_t cb = 0; cb < nc; cb += E->grid) {
      const uint32_t cc = std::min<uint32_t>(E->grid, nc - cb);
      SearchParams Q = make_params(E);
      Q.t_rec = d_kids;
      Q.t_rec_off = d_croff + cb;
      Q.t_ntasks = cc;
      Q.t_hdr = d_chdr + 16ull * cb;
      Q.t_doms = d_doms;
      Q.t_doms_stride = MAX_DOMS;
      Q.t_kids = nullptr;
      Q.t_wit = d_wit;
      Q.t_wit_stride = CL_CAP + 1;
      Q.t_kl = d_ckl + cb;
      step_test_kernel<<<cc, SEARCH_THREADS, E->smem_bytes, E->stream>>>(Q);
      CK(cudaGetLastError());
      CK(cudaStreamSynchronize(E->stream));
    }
    chdr.resize(16ull * nc);
    CK(cudaMemcpy(chdr.data(), d_chdr, 16ull * nc * 4, cudaMemcpyDeviceToHost));
    // 3. cost: the live size of every child that still branches
    for (uint32_t c = 0; c < nc; c++) {
      const uint32_t *h = chdr.data() + 16ull * c;
      if (h[0] != 0) continue;
      out_branching[cparent[c]]++;
      out_cost[cparent[c]] += h[4];
    }
  }
  return 0;
}

}  // extern "C"
