/*
 * oracle.h -- CPU restatement of the size-bounded community search (SCS)
 * hot path of wajidmanzoor/SCS.  TEST INFRASTRUCTURE ONLY: only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline legs load this library,
 * always to check or time against, never as the measured or shipped path.
 *
 * Parity status: the graph loader, core numbers, BFS and the three greedy
 * heuristics are pinned bit-exactly against the reference's own CPU code
 * (src/Graph.h, inc/heuristic.h) compiled from its sources into oracle/_ref
 * and against committed golden vectors (tests/golden/).  The branch-and-bound
 * objective is pinned against an exhaustive brute-force solver on small graphs
 * (the reference ships no serial branch-and-bound).
 */
#ifndef SCS_ORACLE_H
#define SCS_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_INF 1000000000u /* inc/Utility.h:33 (INF for unreachable) */

/* Whole-graph view (CSR with ascending neighbour lists). */
typedef struct {
  uint32_t n;
  const uint32_t *off;    /* n+1 */
  const uint32_t *adj;    /* off[n] entries */
  const uint32_t *degree; /* n */
  const uint32_t *core;   /* n */
  uint32_t dmax;
} orc_graph;

/* Rule switches, same meaning as the reference CLI args red1..prun2
 * (main.cu:498-502). */
enum {
  ORC_RED1 = 1, ORC_RED2 = 2, ORC_RED3 = 4, ORC_PRUN1 = 8, ORC_PRUN2 = 16,
  ORC_ALL_RULES = 31
};

typedef struct {
  uint32_t degree;  /* reported maximum minimum degree */
  uint32_t kl_heu;  /* heuristic incumbent (0 when heuristic off) */
  uint32_t ku;      /* min(core[q], h-1) */
  uint32_t heu_hit; /* 1: answered by the heuristic (kl == ku) */
  uint32_t ubd;     /* distance bound used by the initial filter */
  uint32_t n_kept;  /* vertices passing core>kl && dist<=ubD */
  uint32_t n_local; /* of those, the ones in q's component */
  uint32_t status;  /* 0 ok, 1 node limit reached, 2 time limit reached */
  uint64_t nodes;   /* tasks processed */
  uint64_t max_task;
  uint64_t sum_task;
  uint32_t h_size;     /* size of the returned community */
  uint32_t h_from_bnb; /* 1 if the community came from the search */
  uint64_t size_hist[8]; /* tasks by size: <=32,64,128,256,512,1024,2048,more */
} orc_result;

/* ---- graph layer ---- */
int orc_load_edgelist(const char *path, uint32_t *n_out, uint64_t *m_header,
                      uint32_t **off_out, uint32_t **adj_out);
void orc_free(void *p);
void orc_degrees(uint32_t n, const uint32_t *off, uint32_t *degree,
                 uint32_t *dmax);
void orc_core(uint32_t n, const uint32_t *off, const uint32_t *adj,
              uint32_t *core);
void orc_bfs(uint32_t n, const uint32_t *off, const uint32_t *adj, uint32_t q,
             uint32_t *dist);

/* ---- bounds ---- */
uint32_t orc_ubd_host(uint32_t kl, uint32_t h);
uint32_t orc_ubd_dev(uint32_t kl, uint32_t h);

/* ---- heuristics: return kl, write H (capacity >= h) ---- */
uint32_t orc_heu2(const orc_graph *g, uint32_t l, uint32_t h, uint32_t q,
                  uint32_t *H, uint32_t *hsize);
uint32_t orc_heu3(const orc_graph *g, uint32_t l, uint32_t h, uint32_t q,
                  uint32_t *H, uint32_t *hsize);
uint32_t orc_heu4(const orc_graph *g, uint32_t l, uint32_t h, uint32_t q,
                  uint32_t *H, uint32_t *hsize);
uint32_t orc_cssc_heu(const orc_graph *g, uint32_t l, uint32_t h, uint32_t q,
                      uint32_t *H, uint32_t *hsize);

/* ---- full query ---- */
/* Wall-clock cap per orc_solve call (seconds, 0 = none; per process). */
void orc_set_time_limit(double seconds);

int orc_solve(const orc_graph *g, uint32_t l, uint32_t h, uint32_t q,
              uint32_t heur, uint32_t limit_doms, uint32_t rules,
              uint64_t node_limit, orc_result *res, uint32_t *H,
              uint32_t h_cap);

/* As orc_solve, with the incumbent raised to at least kl_floor before the
 * search (measures the proof part of a search when kl_floor is the optimum;
 * the result is then max(optimum, kl_floor)). */
int orc_solve_from(const orc_graph *g, uint32_t l, uint32_t h, uint32_t q,
                   uint32_t heur, uint32_t limit_doms, uint32_t rules,
                   uint64_t node_limit, uint32_t kl_floor, orc_result *res,
                   uint32_t *H, uint32_t h_cap);

/* Exhaustive solver for small components: max over connected S containing q
 * with l <= |S| <= h of min degree (0 if none).  Returns UINT32_MAX when the
 * component of q has more than `max_comp` vertices. */
uint32_t orc_bruteforce(const orc_graph *g, uint32_t l, uint32_t h,
                        uint32_t q, uint32_t max_comp);

/* ---- per-query preprocessing (local graph) ---- */
typedef struct {
  uint32_t n;       /* local vertices */
  uint32_t *off;    /* n+1 */
  uint32_t *adj;    /* local ids, ascending */
  uint32_t *dist;   /* full-graph BFS distance per local vertex */
  uint32_t *gid;    /* local -> global id */
  uint32_t q_local;
  uint32_t l, h, limit_doms, dmax, rules;
  int32_t *pos; /* scratch, n entries, all -1 between calls */
} orc_qctx;

int orc_prepare(const orc_graph *g, uint32_t q, uint32_t kl, uint32_t ubd,
                uint32_t component_only, orc_qctx *ctx, uint32_t *n_kept);
void orc_qctx_free(orc_qctx *ctx);

/* One branch-and-bound step on a task.  Task entries are (local_id<<1)|inC,
 * ascending.  hdr (16 words) receives:
 *   [0] status (0 branched, 1 dropped by size, 2 dropped by bound,
 *       3 dropped: no ustar or too few vertices)
 *   [1] kl after the step   [2] best min degree evaluated (UINT32_MAX none)
 *   [3] |C| after rule 3     [4] |C|+|R| after rules 1/2
 *   [5] P1  [6] P2  [7] ustar local id (UINT32_MAX none)  [8] #doms
 *   [9] #children  [10] words written to `kids`
 *   [11] size of the witness C written to `wit` (local ids) for [2]
 * doms (limit_doms entries) receives the kept dominated vertices in order.
 * kids receives children as [s, csize, entries...] in the order Include,
 * Dom_0..Dom_{k-1}, Exclude.  Returns 0, or -1 if kids_cap is too small. */
int orc_step(orc_qctx *ctx, const uint32_t *task, uint32_t s, uint32_t kl,
             uint32_t *hdr, uint32_t *doms, uint32_t *kids, uint64_t kids_cap,
             uint32_t *wit);

#ifdef __cplusplus
}
#endif
#endif
