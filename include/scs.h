/*
 * scs.h -- C ABI of the GB300 size-bounded community search engine.
 *
 * The reference (wajidmanzoor/SCS) has no library interface: its boundary is
 * the server process.  Each entry point below replaces one piece of it:
 *
 *   scs_create / scs_create_csr  <- main.cu:475-585: graph load
 *        (src/Graph.h:5-67), core decomposition (src/Graph.h:82-109), device
 *        allocation (src/gpuMemoryAllocation.cc:22-165) from the 12 CLI args
 *        (main.cu:476-502), here carried by scs_config.
 *   scs_submit                   <- main.cu:62-78 + main.cu:84-119: one
 *        "<l> <h> <qid> <heuristic_flag> <limit_dominating_set>" message
 *        admitted into a query slot.
 *   scs_run / scs_poll           <- main.cu:261-463: the level loop that runs
 *        the search and writes one result row per finished query
 *        (main.cu:122-133, 317-339, 340-360, 444-463).
 *   scs_destroy                  <- main.cu:586-594 (free + device reset).
 *
 * Conventions: every call returns 0 or a negative SCS_E* code; nothing calls
 * exit().  Plain pointers and sizes only.  One engine drives one GPU.
 * scs_submit may be called from any number of threads, also while another
 * thread steps the engine; every other call on one engine must come from one
 * thread at a time (the one that steps it).
 */
#ifndef SCS_H
#define SCS_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define SCS_OK 0
#define SCS_EINVAL -1     /* bad argument */
#define SCS_EIO -2        /* graph file missing or malformed */
#define SCS_ECUDA -3      /* CUDA runtime error (message via scs_last_error) */
#define SCS_ENOMEM -4     /* device or host allocation failed */
#define SCS_EBUSY -5      /* no free query slot */
#define SCS_ENOTREADY -6  /* nothing finished yet */
#define SCS_ESTALL -7     /* a host worker made no progress (scs_last_error) */

/* ---- per-query result status (scs_result.status) ---- */
#define SCS_DONE 0          /* search finished: degree is the optimum */
#define SCS_HEURISTIC 1     /* answered by the greedy incumbent (kl == ku),
                               the reference's Heu=1 row (main.cu:122-133) */
#define SCS_CAPACITY 2      /* task store overflow: degree is the best found,
                               the reference's Overtime=2 (main.cu:340-360) */
#define SCS_TIMEOUT 3       /* stopped by the search budget: best found,
                               the reference's Overtime=1 (main.cu:444-463) */
#define SCS_BAD_QUERY 4     /* malformed query (main.cu:106-109) */
#define SCS_TOO_LARGE 5     /* filtered graph exceeds the engine's limits
                               (scs_config.max_local, 21-bit degrees) */

/* Engine configuration.  Field meanings follow the reference CLI where one
 * exists (main.cu:476-502); zero selects the default. */
typedef struct {
  uint32_t limit_queries; /* concurrent query slots (CLI limitQueries)  */
  uint32_t red1, red2, red3;  /* reduction rules on (1) / off (0)       */
  uint32_t prun1, prun2;      /* upper-bound rules on (1) / off (0)     */
  uint32_t rules_set;         /* 0: all rules on; 1: use the fields above */
  uint32_t ctas_per_sm;       /* search CTAs per SM (0: auto)            */
  uint32_t threads_per_cta;   /* 256 or 512 (0: auto)                    */
  uint64_t stack_words;       /* task-stack words per CTA (0: auto)      */
  uint64_t pool_words;        /* shared task-pool words (0: auto)        */
  uint32_t slice_us;          /* search time slice in microseconds (0: 80 ms;
                                 new queries are admitted between slices) */
  uint64_t node_budget;       /* per-query task budget, 0 = unlimited
                                 (stands in for the level cap main.cu:444) */
  uint32_t host_threads;      /* threads for the greedy incumbent (0: auto) */
  int32_t device;             /* CUDA device ordinal                      */
  uint32_t active_queries;    /* queries searched at once; the other admitted
                                 ones wait prepared (0: auto, 32). Fewer keep
                                 the searched local graphs in L2. */
  uint32_t release_order;     /* which prepared query is searched next:
                                 0 the smallest local graph (shortest job
                                 first), 1 admission order */
  uint32_t release_headroom;  /* admission by free task-store memory: a
                                 prepared query is released to the search
                                 only while the shared pool has room for this
                                 many records of its root's size beyond what
                                 earlier releases of the slice claimed
                                 (0: 4).  When nothing is being searched the
                                 next query is released regardless. */
  uint32_t max_local;         /* largest local (filtered) graph a query may
                                 search, in vertices (0: min(n, 2^21)); larger
                                 ones report SCS_TOO_LARGE.  Each search CTA
                                 keeps about 13 words of scratch per vertex of
                                 this size, and each slot a parked root of
                                 2*max_local+5 words.  A local graph with a
                                 vertex of more than 2,097,151 local
                                 neighbours is too large at any setting. */
  uint32_t host_release_only; /* 1: prepared queries are released only
                                 between slices; 0 (default): the slice's
                                 next ones are also queued for the device,
                                 which releases one each time a searched
                                 query finishes */
  uint32_t prep_ctas;         /* CTAs that build one query's local graph, as
                                 one thread-block cluster: 1, 2, 4, 8 or 16
                                 (16 is a non-portable cluster size; 0: 8 on
                                 graphs of 2^18 vertices or more, else 1).
                                 The output is the same for any. */
  uint32_t prep_big_row;      /* preparation walks rows of at least this
                                 many entries with a whole CTA, shorter ones
                                 with a warp (0: 4096) */
} scs_config;

/* One query: the reference's message fields (main.cu:92-119). */
typedef struct {
  uint32_t l;          /* lower size bound N1 */
  uint32_t h;          /* upper size bound N2 */
  uint32_t q;          /* query vertex QID */
  uint32_t heuristic;  /* 1: greedy incumbent on (isHeu) */
  uint32_t limit_doms; /* dominating-branch limit (limitDoms) */
} scs_query;

typedef struct {
  uint64_t ticket;      /* value returned by scs_submit */
  uint32_t l, h, q;     /* echo of the query */
  uint32_t degree;      /* maximum minimum degree (Degree column) */
  int32_t status;       /* SCS_DONE, SCS_HEURISTIC, ... */
  uint32_t kl_heuristic;/* greedy incumbent */
  uint32_t h_size;      /* vertices written to the community buffer */
  uint32_t h_verified;  /* 1: community connected, contains q, size within
                           [l,h] and min degree == degree */
  uint64_t nodes;       /* search tasks processed */
  uint64_t latency_ns;  /* submit -> result available */
  uint64_t search_ns;   /* device search time (admission -> finish) */
} scs_result;

typedef struct scs_engine scs_engine;

/* Create from an edge-list file in the reference format: a "<n> <m>" header
 * then "u v" pairs (src/Graph.h:5-67).  Self-loops dropped, duplicates
 * merged. */
int scs_create(scs_engine **out, const char *edge_list_path,
               const scs_config *cfg);

/* Create from a symmetric CSR with strictly ascending neighbour lists and no
 * self-loops (the form scs_read_edge_list returns).  Returns SCS_EINVAL when
 * the CSR breaks one of these, e.g. an edge listed in only one of its rows. */
int scs_create_csr(scs_engine **out, uint32_t n, const uint32_t *off,
                   const uint32_t *adj, const scs_config *cfg);

/* Graph facts: n, directed adjacency entries, max degree. */
int scs_graph_info(scs_engine *e, uint32_t *n, uint64_t *nnz, uint32_t *dmax);

/* Copy core numbers (n entries) computed at creation. */
int scs_core_numbers(scs_engine *e, uint32_t *core_out);

/* Queue a query; returns a ticket.  Admission into a slot happens inside
 * scs_run/scs_step as slots free up (continuous batching). */
int scs_submit(scs_engine *e, const scs_query *q, uint64_t *ticket);

/* Advance the engine: admit waiting queries into free slots (prepared on the
 * device together), release prepared queries to the search up to
 * active_queries, run one search slice, collect finished queries.  A
 * collected query's community is verified on a background thread, beside
 * the next slice, before its result reaches scs_poll.  Returns the number of
 * queries still outstanding (queued + admitted + being verified), or a
 * negative error.  With nothing left to search it waits for the last checks,
 * so a return of 0 means every result is pollable. */
int scs_step(scs_engine *e);

/* Run until every submitted query has a pollable result. */
int scs_run(scs_engine *e);

/* Drain up to max finished results.  For result i the community's global
 * vertex ids go to h_buf[i*h_stride ... i*h_stride + h_size) when h_buf is
 * not NULL (h_stride >= the query's h).  Returns the count written. */
int scs_poll(scs_engine *e, scs_result *out, int max, uint32_t *h_buf,
             uint32_t h_stride);

/* Engine counters (array of SCS_STAT_COUNT u64). */
#define SCS_STAT_COUNT 24
enum {
  SCS_STAT_NODES = 0,     /* tasks processed */
  SCS_STAT_SLICES = 1,    /* search slices launched */
  SCS_STAT_DONATIONS = 2, /* tasks moved into the shared pool */
  SCS_STAT_STEALS = 3,    /* tasks taken from the shared pool */
  SCS_STAT_SPILLS = 4,    /* stack overflows spilled to the pool */
  SCS_STAT_BYTES = 5,     /* algorithmic bytes moved by the search */
  SCS_STAT_PREP_BYTES = 6,/* algorithmic bytes moved by preprocessing */
  SCS_STAT_SEARCH_NS = 7, /* device time inside search slices */
  SCS_STAT_PREP_NS = 8,   /* device time inside preprocessing */
  SCS_STAT_LAUNCHES = 9,  /* kernel launches issued */
  SCS_STAT_H2D = 10,      /* host-to-device bytes copied by the engine */
  SCS_STAT_D2H = 11,      /* device-to-host bytes copied by the engine */
  SCS_STAT_HEUR_NS = 12,  /* time admission waited for a greedy incumbent with
                             the GPU idle (incumbents are computed by background
                             host threads; ready queries are admitted first) */
  SCS_STAT_CTAS = 13,     /* search CTAs resident per slice (SMs x CTAs per
                             SM after the occupancy check) */
  SCS_STAT_SMEM_WORDS = 14,/* task state words held in shared memory per CTA
                             (larger local graphs keep them in device memory) */
  SCS_STAT_ERRORS = 15,   /* device error flags seen so far (bits, OR-ed) */
  SCS_STAT_ACTIVE = 16,   /* queries searched at once (the active target) */
  SCS_STAT_RELEASES = 17, /* prepared queries released to the search */
  SCS_STAT_SLIDES = 18,   /* task-stack slides: a CTA's live records moved
                             down over the room donations left below them */
  SCS_STAT_PROPOSALS_BETTER = 19, /* learned incumbent proposals that raised
                             a query's incumbent (model loaded) */
  SCS_STAT_HELD_MEMORY = 20, /* slices in which a prepared query waited for
                             pool room (release_headroom) */
  SCS_STAT_POOL_FREE = 21, /* shared-pool words free after the last slice */
  SCS_STAT_DEVICE_RELEASES = 22 /* prepared queries the device released
                             inside a slice as searched ones finished */
};
int scs_stats(scs_engine *e, uint64_t *out);

/* Search-kernel profile (16 u64): clock cycles spent per step phase summed
 * over CTAs [0 load, 1 min degree + rule 3, 2 rules 1/2, 3 bounds, 4 ustar,
 * 5 doms, 6 children, 7 other], then rule-1/2 rounds, rule-3 rounds, steps,
 * then five sub-phase counters: with -DSCS_PROF_MODE=1, rule-1/2 cycles in
 * [check passes, removal rounds, recount rounds], removed vertices and
 * recount rounds (modes 2-5 of bnb.cu measure other splits; the default
 * build leaves them zero). */
int scs_profile(scs_engine *e, uint64_t *out);

/* Text of the last error on this engine (or the last creation failure). */
const char *scs_last_error(scs_engine *e);

int scs_destroy(scs_engine *e);

/* ---- host-only utilities (no GPU needed) ---- */

/* Edge-list load (src/Graph.h:5-67) into a CSR allocated with malloc; free
 * both arrays with scs_free. */
int scs_read_edge_list(const char *path, uint32_t *n, uint64_t *nnz,
                       uint32_t **off, uint32_t **adj);
void scs_free(void *p);

/* Core numbers (src/Graph.h:82-109). */
int scs_core_decompose(uint32_t n, const uint32_t *off, const uint32_t *adj,
                       uint32_t *core);

/* The same core numbers computed on GPU `device` by level-synchronous
 * peeling (replaces the serial start-up peeling, src/Graph.h:82-109; the
 * engine uses it at creation).  Allocates its own device buffers.  Returns
 * 0, SCS_EINVAL for an invalid CSR or SCS_ECUDA. */
int scs_core_decompose_gpu(uint32_t n, const uint32_t *off, const uint32_t *adj,
                           uint32_t *core, int device);

/* Greedy incumbent kl = max(heu2, heu3, heu4) and its community
 * (CSSC_heu, inc/heuristic.h:321-349).  H needs room for max(h, deg(q)+1).
 * The CSR is checked as for scs_create_csr (SCS_EINVAL).  The counts and
 * scores the reference recomputes by rescanning neighbour rows are kept up to
 * date instead, with the same values and pop order, so kl and H are the
 * reference's. */
int scs_greedy_incumbent(uint32_t n, const uint32_t *off, const uint32_t *adj,
                         uint32_t l, uint32_t h, uint32_t q, uint32_t *kl,
                         uint32_t *H, uint32_t *hsize);

/* Distance bound ubD from n(k, D) (main.cu:154-172). */
uint32_t scs_distance_bound(uint32_t kl, uint32_t h);

/* Layout of the public structs as compiled, for bindings to check theirs:
 * out[0..7] = sizeof(scs_config), offsetof(scs_config, node_budget),
 * offsetof(scs_config, device), offsetof(scs_config, active_queries),
 * sizeof(scs_query), sizeof(scs_result), offsetof(scs_result, nodes),
 * offsetof(scs_result, search_ns).  Returns the count written (<= max). */
int scs_abi_layout(uint64_t *out, int max);

/* Check an answer community H[0..hs) of query (l, h, q) against a CSR graph
 * (the checks the reference's results imply but never perform: it reports
 * only the degree, main.cu:328-334).  Returns SCS_CHECK_OK when every id is
 * below n, no id repeats, q is in H, l <= |H| <= h and H is connected;
 * otherwise the first failed check.  *md receives the minimum degree inside
 * H whenever the ids are valid (0 otherwise). */
enum {
  SCS_CHECK_OK = 0,
  SCS_CHECK_EMPTY = 1,
  SCS_CHECK_RANGE = 2,      /* an id >= n */
  SCS_CHECK_REPEAT = 3,     /* an id listed twice */
  SCS_CHECK_NO_QUERY = 4,   /* q not in H */
  SCS_CHECK_SIZE = 5,       /* |H| outside [l, h] */
  SCS_CHECK_DISCONNECTED = 6
};
int scs_check_community(uint32_t n, const uint32_t *off, const uint32_t *adj,
                        const uint32_t *H, uint32_t hs, uint32_t q, uint32_t l,
                        uint32_t h, uint32_t *md);

/* ---- server surface (host only) ---- */

/* Parse one queue message (main.cu:92-109): returns 0 and fills q for
 * "<l> <h> <qid> <heuristic_flag> <limit_dominating_set>", 1 for
 * "server_exit" (main.cu:51-60), SCS_EINVAL otherwise. */
int scs_parse_message(const char *text, scs_query *q);

/* Format a result as the reference's results-file row
 * N1|N2|QID|Time|Degree|Overtime|Heu|TotalTime (main.cu:124-128, 328-333,
 * 348-352, 451-454).  Returns the length or SCS_EINVAL. */
int scs_format_result_row(const scs_result *r, char *buf, uint32_t cap);

/* ---- allocation-free preprocessing (no counterpart in the reference) ----
 * For callers that cannot call cudaMalloc -- code running inside another
 * framework's memory pool or allocator hook, plugins whose host forbids
 * device allocations after start-up, latency-critical loops that must not
 * allocate.  Builds the filtered local graph of one query (bounded BFS from
 * q, keep core > kl && dist <= ubd, q's component, local CSR) exactly like
 * the engine's preprocessing, but allocates nothing: the caller passes the
 * device graph (off[n+1], adj, core[n], max degree) and device outputs
 * gid[n], dist[n], loc_off[n+1], loc_adj[loc_adj_cap] (rows ascending,
 * padded to a multiple of 4 with 0xFFFFFFFF) and info[4] = {n_local,
 * q_local, padded entries used, status: 0 ok, 1 loc_adj_cap too small}.
 * Scratch is a fixed array inside the library for graphs of at most
 * SCS_NOALLOC_MAX_N vertices (about 6 MB, held on every GPU that loads the
 * library until exit); larger n is rejected with SCS_EINVAL, and so is a
 * distance bound ubd >= 65535 (hop distances are held as 16-bit values).  The
 * first call on a device looks up the array's device address there, so make
 * it before any stream capture; after a device reset the next call looks it
 * up again.  An error already pending from the caller's earlier CUDA work is
 * reported as SCS_ECUDA and left pending.  All calls share the array: calls
 * that overlap on the GPU race.  The kernel is enqueued on `stream` (a
 * cudaStream_t, NULL for the default stream); results are ready when the
 * stream is. */
#define SCS_NOALLOC_MAX_N (1u << 19)
int scs_local_graph_noalloc(const uint32_t *d_off, const uint32_t *d_adj,
                            const uint32_t *d_core, uint32_t n, uint32_t dmax,
                            uint32_t q, uint32_t kl, uint32_t ubd,
                            uint32_t *d_gid, uint32_t *d_dist,
                            uint32_t *d_loc_off, uint32_t *d_loc_adj,
                            uint64_t loc_adj_cap, uint32_t *d_info,
                            void *stream);

/* ---- learned branching (no counterpart in the reference) ----
 * A small network (16 candidate features -> 128 -> 128 -> 1, ReLU) scores
 * the branching candidates of each search step: the engine takes u* from a
 * shortlist of the candidates the reference's rule accepts (selectUstar,
 * src/helpers.cc:1104-1168), by the largest network score instead of the
 * rule's score.  Every pruning rule and the optimality proof stay the
 * integer method, so answers are the same with or without a model.  The
 * network runs on the tensor cores in BF16 with FP32 accumulation; its FP32
 * weights are trained by the engine's own GPU kernels (scs_mlp_train) on
 * traces the exact solver emits (scs_trace_enable / scs_trace_read). */

/* Load a model file ("SCSMLP01", u32 dims {16,128,128,1}, then the FP32
 * parameters W1[16][128], b1[128], W2[128][128], b2[128], W3[128], b3);
 * NULL returns the engine to the plain method.  Needs an idle engine. */
int scs_load_model(scs_engine *e, const char *path);

/* Record the shortlisted candidates of sampled search steps: per record 16
 * FP32 features and the key {query tag (low 32 bits of the ticket), global
 * vertex id}.  A CTA records its steps whose step count has the low
 * sample_shift bits zero.  max_records = 0 turns the trace off.  Needs an
 * idle engine; resets the record count. */
int scs_trace_enable(scs_engine *e, uint64_t max_records, uint32_t sample_shift);

/* Copy up to max records (feat: max*16 floats, keys: max*2 words; either may
 * be NULL); *written gets the records the search produced, which can exceed
 * the capacity (the excess was dropped).  Returns the count copied. */
int scs_trace_read(scs_engine *e, float *feat, uint32_t *keys, uint64_t max,
                   uint64_t *written);

#define SCS_MLP_NPARAM 18817
typedef struct {
  uint32_t epochs;     /* passes over the samples (0: 20) */
  uint32_t batch;      /* samples per step (0: 4096) */
  float lr;            /* Adam step size (0: 1e-3) */
  float weight_decay;  /* L2 term added to the gradient */
  uint64_t seed;       /* shuffling */
} scs_mlp_train_cfg;

/* Train on the GPU (hand-written FP32 kernels, Adam, weighted binary
 * cross-entropy on the logit) from X[n][16], labels y[n] in {0,1} and
 * weights w[n] (NULL: all 1).  params (SCS_MLP_NPARAM floats, file order)
 * holds the initial values and receives the result; epoch_loss (may be
 * NULL) gets the mean loss of each epoch. */
int scs_mlp_train(const float *X, const float *y, const float *w, uint64_t n,
                  const scs_mlp_train_cfg *cfg, float *params, float *epoch_loss,
                  int device);

/* Weighted mean loss and its gradient (file order) on one batch, computed by
 * the training kernels (for checking them against a CPU restatement). */
int scs_mlp_grad(const float *params, const float *X, const float *y, const float *w,
                 uint64_t n, double *loss, float *grad, int device);

/* Logits of n feature rows by the tensor-core BF16 inference the search
 * kernel uses (one warp per 16 rows). */
int scs_mlp_infer(const float *params, const float *X, uint64_t n, float *out,
                  int device);

/* Text of the last error of the scs_mlp_* calls. */
const char *scs_mlp_last_error(void);

/* ---- test hooks (used by the parity tests; no reference counterpart) ----
 * These expose single stages of the pipeline so they can be compared with
 * the CPU oracle.  They need an idle engine (no queries running). */

/* Build the local (filtered) graphs of nq queries into slots 0..nq-1 with the
 * given incumbents kl[i] and distance bounds ubd[i]; the stage restated from
 * initialReductionRules/CompressTask/NeighborUpdate (src/helpers.cc:207-368).
 * Writes each slot's local vertex count and local id of q. */
int scs_debug_prepare(scs_engine *e, uint32_t nq, const scs_query *queries,
                      const uint32_t *kl, const uint32_t *ubd,
                      uint32_t *n_local, uint32_t *q_local);

/* Copy a prepared slot's local graph: local->global ids, CSR without the
 * row padding, and full-graph hop distances.  Any pointer may be NULL. */
int scs_debug_local_graph(scs_engine *e, uint32_t slot, uint32_t *gid,
                          uint32_t *off, uint32_t *adj, uint32_t *dist);

/* Run ONE deterministic branch-and-bound step per task on the GPU with the
 * search kernel's own step code (ProcessTask + FindDoms + Expand,
 * src/helpers.cc:371-857).  Task t lives in slot task_slot[t], has incumbent
 * kl_in[t] and entries (local_id<<1)|inC at task_entries[task_off[t] ..
 * + task_len[t]), ascending.  Per task: out_hdr[16*t] gets the step header
 * (same layout as the CPU oracle's orc_step), out_doms the kept dominated
 * vertices, out_kids the children [s, csize, entries(s), degrees(s)] in the
 * order Include, Dom_0.., Exclude, out_wit the witness C (count at index
 * 512).  Strides: doms >= 15, wit >= 513. */
int scs_debug_step(scs_engine *e, uint32_t ntasks, const uint32_t *task_slot,
                   const uint32_t *kl_in, const uint64_t *task_off,
                   const uint32_t *task_len, const uint32_t *task_entries,
                   uint32_t *out_hdr, uint32_t *out_doms, uint32_t doms_stride,
                   uint32_t *out_kids, uint64_t kids_stride, uint32_t *out_wit,
                   uint32_t wit_stride, const uint32_t *force, uint32_t *out_sl,
                   float *out_sl_feat);
/* (scs_debug_step, continued) force (may be NULL): per task the local id
 * of u* to branch on instead of the rule's choice (a candidate: an R vertex
 * with a C neighbour; 0xFFFFFFFF keeps the rule's).  out_sl / out_sl_feat
 * (both or neither): per task the learned-branching shortlist, [count, 16
 * local ids] and 16 x 16 features. */

/* Strong-branching lookahead for training the branching network (no
 * reference counterpart): for each task, one step that branches on
 * force[t], then one step on each of its children.  out_hdr gets the forced
 * step's header (16 per task), out_nkids its children, out_branching how
 * many of them still branch after their own reductions and bounds, and
 * out_cost the sum of those children's live sizes (the work left below this
 * choice of u*, one level down). */
int scs_debug_lookahead(scs_engine *e, uint32_t ntasks, const uint32_t *task_slot,
                        const uint32_t *kl_in, const uint64_t *task_off,
                        const uint32_t *task_len, const uint32_t *task_entries,
                        const uint32_t *force, uint32_t *out_hdr, uint32_t *out_nkids,
                        uint32_t *out_branching, uint64_t *out_cost);

#ifdef __cplusplus
}
#endif
#endif
