/*
 * oracle.c -- CPU restatement of the SCS hot path (test infrastructure only;
 * see oracle.h).  Every function names the reference code it restates.
 */
#define _POSIX_C_SOURCE 199309L
#include "oracle.h"

#include <ctype.h>
#include <time.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ */
/* graph loader: src/Graph.h:5-67 (load_graph).  Header "<n> <m>", then
 * "u v" pairs until the first token that is not an unsigned integer.
 * Self-loops are dropped, both directions inserted into a set per vertex,
 * neighbour lists are ascending (std::set order).                       */
/* ------------------------------------------------------------------ */
static int cmp_u64(const void *a, const void *b) {
  uint64_t x = *(const uint64_t *)a, y = *(const uint64_t *)b;
  return (x > y) - (x < y);
}

static int next_uint(const char **p, const char *end, uint64_t *out) {
  const char *s = *p;
  while (s < end && isspace((unsigned char)*s)) s++;
  if (s >= end || !isdigit((unsigned char)*s)) return 0;
  uint64_t v = 0;
  while (s < end && isdigit((unsigned char)*s)) {
    v = v * 10 + (uint64_t)(*s - '0');
    s++;
  }
  *p = s;
  *out = v;
  return 1;
}

int orc_load_edgelist(const char *path, uint32_t *n_out, uint64_t *m_header,
                      uint32_t **off_out, uint32_t **adj_out) {
  FILE *f = fopen(path, "rb");
  if (!f) return -1;
  fseek(f, 0, SEEK_END);
  long sz = ftell(f);
  fseek(f, 0, SEEK_SET);
  char *buf = (char *)malloc((size_t)sz + 1);
  if (!buf) { fclose(f); return -2; }
  size_t rd = fread(buf, 1, (size_t)sz, f);
  fclose(f);
  buf[rd] = 0;
  const char *p = buf, *end = buf + rd;
  uint64_t n64, m64;
  if (!next_uint(&p, end, &n64) || !next_uint(&p, end, &m64)) {
    free(buf);
    return -3;
  }
  uint32_t n = (uint32_t)n64;
  size_t cap = 1024, cnt = 0;
  uint64_t *e = (uint64_t *)malloc(cap * sizeof(uint64_t));
  uint64_t u, v;
  for (;;) {
    if (!next_uint(&p, end, &u)) break;
    if (!next_uint(&p, end, &v)) break;
    if (u == v) continue;
    if (u >= n || v >= n) { free(e); free(buf); return -4; }
    if (cnt + 2 > cap) {
      cap *= 2;
      e = (uint64_t *)realloc(e, cap * sizeof(uint64_t));
    }
    e[cnt++] = (u << 32) | v;
    e[cnt++] = (v << 32) | u;
  }
  free(buf);
  qsort(e, cnt, sizeof(uint64_t), cmp_u64);
  size_t w = 0;
  for (size_t i = 0; i < cnt; i++)
    if (w == 0 || e[w - 1] != e[i]) e[w++] = e[i];
  uint32_t *off = (uint32_t *)calloc((size_t)n + 1, sizeof(uint32_t));
  uint32_t *adj = (uint32_t *)malloc((w ? w : 1) * sizeof(uint32_t));
  for (size_t i = 0; i < w; i++) {
    off[(e[i] >> 32) + 1]++;
    adj[i] = (uint32_t)(e[i] & 0xffffffffu);
  }
  for (uint32_t i = 0; i < n; i++) off[i + 1] += off[i];
  free(e);
  *n_out = n;
  *m_header = m64;
  *off_out = off;
  *adj_out = adj;
  return 0;
}

void orc_free(void *p) { free(p); }

/* degree and dMAX: src/Graph.h:36-45 */
void orc_degrees(uint32_t n, const uint32_t *off, uint32_t *degree,
                 uint32_t *dmax) {
  uint32_t mx = 0;
  for (uint32_t i = 0; i < n; i++) {
    degree[i] = off[i + 1] - off[i];
    if (degree[i] > mx) mx = degree[i];
  }
  *dmax = mx;
}

/* core numbers: src/Graph.h:82-109 peels with a bucket list; core numbers are
 * unique, so the standard O(m) bin-sort peeling yields the same array. */
void orc_core(uint32_t n, const uint32_t *off, const uint32_t *adj,
              uint32_t *core) {
  if (n == 0) return;
  uint32_t md = 0;
  uint32_t *deg = (uint32_t *)malloc(n * sizeof(uint32_t));
  for (uint32_t i = 0; i < n; i++) {
    deg[i] = off[i + 1] - off[i];
    if (deg[i] > md) md = deg[i];
  }
  uint32_t *bin = (uint32_t *)calloc((size_t)md + 2, sizeof(uint32_t));
  uint32_t *vert = (uint32_t *)malloc(n * sizeof(uint32_t));
  uint32_t *pos = (uint32_t *)malloc(n * sizeof(uint32_t));
  for (uint32_t i = 0; i < n; i++) bin[deg[i]]++;
  uint32_t start = 0;
  for (uint32_t d = 0; d <= md; d++) {
    uint32_t c = bin[d];
    bin[d] = start;
    start += c;
  }
  for (uint32_t v = 0; v < n; v++) {
    pos[v] = bin[deg[v]];
    vert[pos[v]] = v;
    bin[deg[v]]++;
  }
  for (uint32_t d = md; d >= 1; d--) bin[d] = bin[d - 1];
  bin[0] = 0;
  for (uint32_t i = 0; i < n; i++) {
    uint32_t v = vert[i];
    for (uint32_t k = off[v]; k < off[v + 1]; k++) {
      uint32_t u = adj[k];
      if (deg[u] > deg[v]) {
        uint32_t du = deg[u], pu = pos[u], pw = bin[du], w = vert[pw];
        if (u != w) {
          pos[u] = pw;
          vert[pu] = w;
          pos[w] = pu;
          vert[pw] = u;
        }
        bin[du]++;
        deg[u]--;
      }
    }
  }
  for (uint32_t i = 0; i < n; i++) core[i] = deg[i];
  free(deg);
  free(bin);
  free(vert);
  free(pos);
}

/* BFS hop distance over the whole graph: src/Graph.h:111-142 */
void orc_bfs(uint32_t n, const uint32_t *off, const uint32_t *adj, uint32_t q,
             uint32_t *dist) {
  for (uint32_t i = 0; i < n; i++) dist[i] = ORC_INF;
  uint32_t *Q = (uint32_t *)malloc((n ? n : 1) * sizeof(uint32_t));
  uint32_t head = 0, tail = 0;
  dist[q] = 0;
  Q[tail++] = q;
  while (head < tail) {
    uint32_t v = Q[head++];
    for (uint32_t i = off[v]; i < off[v + 1]; i++) {
      uint32_t w = adj[i];
      if (dist[w] == ORC_INF) {
        dist[w] = dist[v] + 1;
        Q[tail++] = w;
      }
    }
  }
  free(Q);
}

/* ------------------------------------------------------------------ */
/* distance bound from n(k,D).  Host form main.cu:154-172 (kl<=1 gives h-1;
 * the loop always breaks for kl>=2).  Device form src/helpers.cc:974-990 uses
 * u32 arithmetic, in which (kl-2) wraps for kl<2; both agree on every input
 * (checked exhaustively by the tests), but each is restated as written.   */
/* ------------------------------------------------------------------ */
uint32_t orc_ubd_host(uint32_t kl, uint32_t h) {
  uint32_t ubd = 0;
  if (kl <= 1) return h - 1;
  for (uint32_t d = 1; d <= h; d++) {
    if (d == 1 || d == 2) {
      if (kl + d > h) { ubd = d - 1; break; }
    } else {
      double mn = (double)kl + (double)d + 1.0 + (double)(d / 3) * (double)(kl - 2);
      uint32_t min_n = (uint32_t)mn;
      if (h < min_n) { ubd = d - 1; break; }
    }
  }
  return ubd;
}

uint32_t orc_ubd_dev(uint32_t kl, uint32_t h) {
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

/* ------------------------------------------------------------------ */
/* binary heap over (key, id) pairs with lexicographic order, standing in for
 * std::priority_queue<pair<...>>.  Pairs are totally ordered, so every
 * correct heap pops the same sequence as the reference's.              */
/* ------------------------------------------------------------------ */
typedef struct { double k; uint32_t id; } hent;
typedef struct { hent *a; size_t n, cap; int is_min; } heap_t;

static int h_before(const heap_t *h, hent x, hent y) { /* x pops before y */
  if (h->is_min) return (x.k < y.k) || (x.k == y.k && x.id < y.id);
  return (x.k > y.k) || (x.k == y.k && x.id > y.id);
}
static void h_push(heap_t *h, double k, uint32_t id) {
  if (h->n == h->cap) {
    h->cap = h->cap ? h->cap * 2 : 64;
    h->a = (hent *)realloc(h->a, h->cap * sizeof(hent));
  }
  size_t i = h->n++;
  hent x = {k, id};
  while (i > 0) {
    size_t p = (i - 1) / 2;
    if (!h_before(h, x, h->a[p])) break;
    h->a[i] = h->a[p];
    i = p;
  }
  h->a[i] = x;
}
static hent h_pop(heap_t *h) {
  hent top = h->a[0];
  hent x = h->a[--h->n];
  size_t i = 0;
  for (;;) {
    size_t c = 2 * i + 1;
    if (c >= h->n) break;
    if (c + 1 < h->n && h_before(h, h->a[c + 1], h->a[c])) c++;
    if (!h_before(h, h->a[c], x)) break;
    h->a[i] = h->a[c];
    i = c;
  }
  if (h->n) h->a[i] = x;
  return top;
}

/* heu2: inc/heuristic.h:8-120 (priority = neighbours inside H) */
uint32_t orc_heu2(const orc_graph *g, uint32_t N1, uint32_t N2, uint32_t q,
                  uint32_t *H, uint32_t *hsize) {
  const uint32_t *pstart = g->off, *edges = g->adj;
  uint32_t n = g->n;
  uint32_t *sta = (uint32_t *)calloc(n, sizeof(uint32_t));
  uint32_t *deg = (uint32_t *)calloc(n, sizeof(uint32_t));
  uint32_t *tH = (uint32_t *)malloc((n ? n : 1) * sizeof(uint32_t));
  uint32_t tn = 0, tkl = 0, tH_size = 0;
  heap_t Q = {0};
  Q.is_min = 0;
  h_push(&Q, 0.0, q);
  sta[q] = 1;
  while (Q.n) {
    uint32_t v = h_pop(&Q).id;
    if (sta[v] == 2) continue;
    tH[tn++] = v;
    sta[v] = 2;
    for (uint32_t j = pstart[v]; j < pstart[v + 1]; j++) {
      uint32_t nei = edges[j];
      if (sta[nei] == 0) {
        uint32_t d = 0;
        for (uint32_t w = pstart[nei]; w < pstart[nei + 1]; w++)
          if (sta[edges[w]] == 2) ++d;
        h_push(&Q, (double)d, nei);
        sta[nei] = 1;
      } else if (sta[nei] == 1) {
        uint32_t d = 0;
        for (uint32_t w = pstart[nei]; w < pstart[nei + 1]; w++)
          if (sta[edges[w]] == 2) ++d;
        h_push(&Q, (double)d, nei);
      } else {
        ++deg[nei];
        ++deg[v];
      }
    }
    if (tn >= N1) {
      uint32_t mindeg = ORC_INF;
      for (uint32_t i = 0; i < tn; i++)
        if (deg[tH[i]] < mindeg) mindeg = deg[tH[i]];
      if (mindeg >= tkl) {
        tkl = mindeg;
        tH_size = tn;
      }
    }
    if (tn == N2) break;
  }
  for (uint32_t i = 0; i < tH_size; i++) H[i] = tH[i];
  *hsize = tH_size;
  free(Q.a);
  free(sta);
  free(deg);
  free(tH);
  return tkl;
}

/* heu3: inc/heuristic.h:125-239 (priority = connection score, double) */
uint32_t orc_heu3(const orc_graph *g, uint32_t N1, uint32_t N2, uint32_t q,
                  uint32_t *H, uint32_t *hsize) {
  const uint32_t *pstart = g->off, *edges = g->adj, *degree = g->degree;
  uint32_t n = g->n;
  double dMAX = (double)g->dmax;
  uint32_t *sta = (uint32_t *)calloc(n, sizeof(uint32_t));
  uint32_t *deg = (uint32_t *)calloc(n, sizeof(uint32_t));
  uint32_t *tH = (uint32_t *)malloc((n ? n : 1) * sizeof(uint32_t));
  uint32_t tn = 0, tkl = 0, tH_size = 0;
  heap_t Q = {0};
  Q.is_min = 0;
  h_push(&Q, 0.0, q);
  sta[q] = 1;
  while (Q.n) {
    uint32_t v = h_pop(&Q).id;
    if (sta[v] == 2) continue;
    tH[tn++] = v;
    sta[v] = 2;
    for (uint32_t nei = pstart[v]; nei < pstart[v + 1]; nei++)
      if (sta[edges[nei]] == 2) {
        ++deg[edges[nei]];
        ++deg[v];
      }
    for (uint32_t nei = pstart[v]; nei < pstart[v + 1]; nei++) {
      uint32_t x = edges[nei];
      if (!sta[x] || sta[x] == 1) {
        double score = 0;
        for (uint32_t w = pstart[x]; w < pstart[x + 1]; w++)
          if (sta[edges[w]] == 2 && deg[edges[w]] != 0)
            score += (double)1 / deg[edges[w]];
        score += (double)degree[x] / dMAX;
        h_push(&Q, score, x);
        sta[x] = 1;
      }
    }
    if (tn >= N1) {
      uint32_t mindeg = ORC_INF;
      for (uint32_t i = 0; i < tn; i++)
        if (deg[tH[i]] < mindeg) mindeg = deg[tH[i]];
      if (mindeg >= tkl) {
        tkl = mindeg;
        tH_size = tn;
      }
    }
    if (tn == N2) break;
  }
  for (uint32_t i = 0; i < tH_size; i++) H[i] = tH[i];
  *hsize = tH_size;
  free(Q.a);
  free(sta);
  free(deg);
  free(tH);
  return tkl;
}

/* heu4: inc/heuristic.h:242-317 (peel q and its neighbours by min degree;
 * q starts with one extra degree, as in the reference) */
uint32_t orc_heu4(const orc_graph *g, uint32_t N1, uint32_t N2, uint32_t q,
                  uint32_t *H, uint32_t *hsize) {
  const uint32_t *pstart = g->off, *edges = g->adj, *degree = g->degree;
  uint32_t n = g->n;
  *hsize = 0;
  if (degree[q] < N1 - 1) return 0;
  uint32_t ssz = degree[q] + 1;
  uint32_t *S = (uint32_t *)malloc(ssz * sizeof(uint32_t));
  uint8_t *inS = (uint8_t *)calloc(n, 1);
  uint32_t *deg = (uint32_t *)calloc(n, sizeof(uint32_t));
  uint32_t sn = 0;
  S[sn++] = q;
  inS[q] = 1;
  ++deg[q];
  for (uint32_t j = pstart[q]; j < pstart[q + 1]; j++) {
    uint32_t x = edges[j];
    S[sn++] = x;
    inS[x] = 1;
    for (uint32_t w = pstart[x]; w < pstart[x + 1]; w++)
      if (inS[edges[w]]) {
        ++deg[edges[w]];
        ++deg[x];
      }
  }
  heap_t Q = {0};
  Q.is_min = 1;
  for (uint32_t i = 0; i < sn; i++) h_push(&Q, (double)deg[S[i]], S[i]);
  uint32_t *rmv = (uint32_t *)malloc(sn * sizeof(uint32_t));
  uint32_t rn = 0, rmv_idx = 0, mindeg = 0;
  while (Q.n) {
    hent t = h_pop(&Q);
    uint32_t d = (uint32_t)t.k, v = t.id;
    if (inS[v] == 0) continue;
    uint32_t remain = sn - rn;
    if (remain >= N1 && remain <= N2) {
      if (d > mindeg) {
        mindeg = d;
        rmv_idx = rn;
      }
    }
    if (remain == N1) break;
    inS[v] = 0;
    rmv[rn++] = v;
    for (uint32_t j = pstart[v]; j < pstart[v + 1]; j++)
      if (inS[edges[j]]) {
        --deg[edges[j]];
        h_push(&Q, (double)deg[edges[j]], edges[j]);
      }
  }
  memset(inS, 0, n);
  for (uint32_t i = 0; i < sn; i++) inS[S[i]] = 1;
  for (uint32_t i = 0; i < rmv_idx; i++) inS[rmv[i]] = 0;
  uint32_t hn = 0;
  for (uint32_t i = 0; i < sn; i++)
    if (inS[S[i]]) H[hn++] = S[i];
  *hsize = hn;
  free(Q.a);
  free(S);
  free(inS);
  free(deg);
  free(rmv);
  return mindeg;
}

/* CSSC_heu: inc/heuristic.h:321-349 (ties prefer heu4, then heu3) */
uint32_t orc_cssc_heu(const orc_graph *g, uint32_t l, uint32_t h, uint32_t q,
                      uint32_t *H, uint32_t *hsize) {
  uint32_t n = g->n ? g->n : 1;
  uint32_t *H2 = (uint32_t *)malloc(n * sizeof(uint32_t));
  uint32_t *H3 = (uint32_t *)malloc(n * sizeof(uint32_t));
  uint32_t *H4 = (uint32_t *)malloc(n * sizeof(uint32_t));
  uint32_t s2, s3, s4;
  uint32_t k2 = orc_heu2(g, l, h, q, H2, &s2);
  uint32_t k3 = orc_heu3(g, l, h, q, H3, &s3);
  uint32_t k4 = orc_heu4(g, l, h, q, H4, &s4);
  uint32_t *src, sz, kl;
  if (k4 >= k3 && k4 >= k2) { src = H4; sz = s4; kl = k4; }
  else if (k3 >= k2) { src = H3; sz = s3; kl = k3; }
  else { src = H2; sz = s2; kl = k2; }
  if (H) memcpy(H, src, sz * sizeof(uint32_t));
  *hsize = sz;
  free(H2);
  free(H3);
  free(H4);
  return kl;
}

/* ------------------------------------------------------------------ */
/* per-query preprocessing.  Filter: src/helpers.cc:207-248
 * (initialReductionRules: keep v iff core[v] > kl && dist[v] <= ubD).  The
 * root task and kept-neighbour counts: src/helpers.cc:250-313 (CompressTask)
 * and the filtered CSR: src/helpers.cc:317-368 (NeighborUpdate).  Local ids
 * are assigned in ascending global id and neighbour lists are ascending.
 * With component_only the kept set is further restricted to q's connected
 * component in G[kept]; no rule, bound or score of a task containing q can
 * see a vertex of another component (they have no edges to it), so the
 * search is unchanged apart from shorter task lists.                   */
/* ------------------------------------------------------------------ */
int orc_prepare(const orc_graph *g, uint32_t q, uint32_t kl, uint32_t ubd,
                uint32_t component_only, orc_qctx *ctx, uint32_t *n_kept) {
  uint32_t n = g->n;
  uint32_t *dist = (uint32_t *)malloc(n * sizeof(uint32_t));
  orc_bfs(n, g->off, g->adj, q, dist);
  uint8_t *keep = (uint8_t *)calloc(n, 1);
  uint32_t nk = 0;
  for (uint32_t v = 0; v < n; v++)
    if (g->core[v] > kl && dist[v] <= ubd) {
      keep[v] = 1;
      nk++;
    }
  *n_kept = nk;
  if (!keep[q]) { /* cannot happen when kl < ku; guard anyway */
    keep[q] = 1;
  }
  if (component_only) {
    uint8_t *comp = (uint8_t *)calloc(n, 1);
    uint32_t *Q = (uint32_t *)malloc(n * sizeof(uint32_t));
    uint32_t hd = 0, tl = 0;
    comp[q] = 1;
    Q[tl++] = q;
    while (hd < tl) {
      uint32_t v = Q[hd++];
      for (uint32_t i = g->off[v]; i < g->off[v + 1]; i++) {
        uint32_t w = g->adj[i];
        if (keep[w] && !comp[w]) {
          comp[w] = 1;
          Q[tl++] = w;
        }
      }
    }
    free(Q);
    free(keep);
    keep = comp;
  }
  uint32_t *lid = (uint32_t *)malloc(n * sizeof(uint32_t));
  uint32_t nl = 0;
  for (uint32_t v = 0; v < n; v++) lid[v] = keep[v] ? nl++ : UINT32_MAX;
  ctx->n = nl;
  ctx->gid = (uint32_t *)malloc((nl ? nl : 1) * sizeof(uint32_t));
  ctx->dist = (uint32_t *)malloc((nl ? nl : 1) * sizeof(uint32_t));
  ctx->off = (uint32_t *)calloc((size_t)nl + 1, sizeof(uint32_t));
  ctx->pos = (int32_t *)malloc((nl ? nl : 1) * sizeof(int32_t));
  for (uint32_t i = 0; i < nl; i++) ctx->pos[i] = -1;
  uint64_t ecount = 0;
  for (uint32_t v = 0; v < n; v++)
    if (keep[v]) {
      uint32_t c = 0;
      for (uint32_t i = g->off[v]; i < g->off[v + 1]; i++)
        if (keep[g->adj[i]]) c++;
      ctx->gid[lid[v]] = v;
      ctx->dist[lid[v]] = dist[v];
      ctx->off[lid[v] + 1] = c;
      ecount += c;
    }
  for (uint32_t i = 0; i < nl; i++) ctx->off[i + 1] += ctx->off[i];
  ctx->adj = (uint32_t *)malloc((ecount ? ecount : 1) * sizeof(uint32_t));
  for (uint32_t v = 0; v < n; v++)
    if (keep[v]) {
      uint32_t w = ctx->off[lid[v]];
      for (uint32_t i = g->off[v]; i < g->off[v + 1]; i++)
        if (keep[g->adj[i]]) ctx->adj[w++] = lid[g->adj[i]];
    }
  ctx->q_local = lid[q];
  free(lid);
  free(keep);
  free(dist);
  return 0;
}

void orc_qctx_free(orc_qctx *ctx) {
  free(ctx->off);
  free(ctx->adj);
  free(ctx->dist);
  free(ctx->gid);
  free(ctx->pos);
  memset(ctx, 0, sizeof(*ctx));
}

/* ------------------------------------------------------------------ */
/* One task step.  Order of the reference's ProcessTask
 * (src/helpers.cc:443-512): min degree of C and incumbent update (:446-455),
 * reduction rule 3 (:457-470, rule :932-968), rules 1/2 (:474, rule
 * :970-1028), bounds P1/P2 (:475-487, bound :1030-1102), ustar (:488-500,
 * score :1104-1168); then FindDoms (:545-670) and the branching of
 * Expand/writeTasks/writeDomTasks (:673-857, :1171-1391).
 *
 * Deterministic restatement (the reference applies rules 1-3 in one racy
 * in-place warp pass): rule 3 and rules 1/2 are each applied to a fixpoint
 * in synchronous rounds; ustar and doms ties go to the lowest local id;
 * doms are ordered by (score desc, id asc); the dominance test is the
 * intended N(v) subset-of N(u*)+u* taken inside the task (C+R), which keeps
 * the exchange argument of dominating branching valid; the size test
 * "total >= l" counts live vertices; P2 sorts correctly for any |C|.
 * Children that can never be evaluated (|C| > h, or |C|+|R| < l) are not
 * emitted.  Every change only tightens pruning with sound rules, fixes an
 * order, or skips dead work, so the optimum is unchanged.            */
/* ------------------------------------------------------------------ */
enum { ST_R = 0, ST_C = 1, ST_X = 2 };

static int cmp_u32(const void *a, const void *b) {
  uint32_t x = *(const uint32_t *)a, y = *(const uint32_t *)b;
  return (x > y) - (x < y);
}

typedef struct { double sc; uint32_t i; } dent;
static int cmp_dom(const void *a, const void *b) {
  const dent *x = (const dent *)a, *y = (const dent *)b;
  if (x->sc > y->sc) return -1;
  if (x->sc < y->sc) return 1;
  return (x->i > y->i) - (x->i < y->i);
}

static int adj_has(const orc_qctx *c, uint32_t v, uint32_t w) {
  uint32_t lo = c->off[v], hi = c->off[v + 1];
  while (lo < hi) {
    uint32_t mid = lo + (hi - lo) / 2;
    if (c->adj[mid] < w) lo = mid + 1;
    else hi = mid;
  }
  return lo < c->off[v + 1] && c->adj[lo] == w;
}

int orc_step(orc_qctx *ctx, const uint32_t *task, uint32_t s, uint32_t kl,
             uint32_t *hdr, uint32_t *doms_out, uint32_t *kids,
             uint64_t kids_cap, uint32_t *wit) {
  const uint32_t h = ctx->h, l = ctx->l, rules = ctx->rules;
  const double dmax = (double)ctx->dmax;
  uint32_t *v = (uint32_t *)malloc((s ? s : 1) * sizeof(uint32_t));
  uint8_t *st = (uint8_t *)malloc(s ? s : 1);
  uint32_t *dC = (uint32_t *)calloc(s ? s : 1, sizeof(uint32_t));
  uint32_t *dR = (uint32_t *)calloc(s ? s : 1, sizeof(uint32_t));
  uint8_t *mark = (uint8_t *)calloc(s ? s : 1, 1);
  uint32_t csize = 0;
  int rc = 0;
  for (int i = 0; i < 16; i++) hdr[i] = 0;
  hdr[2] = UINT32_MAX;
  hdr[5] = hdr[6] = hdr[7] = UINT32_MAX;
  for (uint32_t i = 0; i < s; i++) {
    v[i] = task[i] >> 1;
    st[i] = (task[i] & 1) ? ST_C : ST_R;
    csize += st[i] == ST_C;
    ctx->pos[v[i]] = (int32_t)i;
  }
  for (uint32_t i = 0; i < s; i++)
    for (uint32_t k = ctx->off[v[i]]; k < ctx->off[v[i] + 1]; k++) {
      int32_t j = ctx->pos[ctx->adj[k]];
      if (j >= 0) {
        if (st[j] == ST_C) dC[i]++;
        else dR[i]++;
      }
    }
  uint32_t best = UINT32_MAX;
#define MINDEG_UPDATE()                                      \
  do {                                                       \
    uint32_t md = UINT32_MAX;                                \
    for (uint32_t i = 0; i < s; i++)                         \
      if (st[i] == ST_C && dC[i] < md) md = dC[i];           \
    if (md != UINT32_MAX) {                                  \
      if (best == UINT32_MAX || md > best) {                 \
        best = md;                                           \
        uint32_t wn = 0;                                     \
        for (uint32_t i = 0; i < s; i++)                     \
          if (st[i] == ST_C) wit[wn++] = v[i];               \
        hdr[11] = wn;                                        \
      }                                                      \
      if (md > kl) kl = md;                                  \
    }                                                        \
  } while (0)

  if (csize > h) { hdr[0] = 1; goto done; }
  if (l <= csize) MINDEG_UPDATE();
  if (rules & ORC_RED3) {
    uint32_t c0 = csize;
    for (;;) {
      /* promote every R neighbour of a tight C vertex (dC+dR == kl+1) */
      uint32_t np = 0;
      memset(mark, 0, s);
      for (uint32_t i = 0; i < s; i++) {
        if (st[i] != ST_C || dC[i] + dR[i] != kl + 1) continue;
        for (uint32_t k = ctx->off[v[i]]; k < ctx->off[v[i] + 1]; k++) {
          int32_t j = ctx->pos[ctx->adj[k]];
          if (j >= 0 && st[j] == ST_R && !mark[j]) { mark[j] = 1; np++; }
        }
      }
      if (!np) break;
      for (uint32_t j = 0; j < s; j++)
        if (mark[j]) { st[j] = ST_C; csize++; }
      for (uint32_t j = 0; j < s; j++)
        if (mark[j])
          for (uint32_t k = ctx->off[v[j]]; k < ctx->off[v[j] + 1]; k++) {
            int32_t x = ctx->pos[ctx->adj[k]];
            if (x >= 0 && st[x] != ST_X) { dC[x]++; dR[x]--; }
          }
      if (csize > h) break;
    }
    if (csize > h) { hdr[3] = csize; hdr[0] = 1; goto done; }
    if (csize != c0 && l <= csize && csize <= h) MINDEG_UPDATE();
  }
  hdr[3] = csize;
  if (csize >= h) { hdr[0] = 1; goto done; }
  if (rules & (ORC_RED1 | ORC_RED2)) {
    uint32_t ubd = orc_ubd_dev(kl, h);
    for (;;) {
      uint32_t nr = 0;
      memset(mark, 0, s);
      for (uint32_t i = 0; i < s; i++) {
        if (st[i] != ST_R) continue;
        int chk = 0;
        if (rules & ORC_RED1) {
          uint32_t a = dR[i] + dC[i], b = dC[i] + h - csize - 1;
          if ((a < b ? a : b) <= kl) chk = 1;
        }
        if ((rules & ORC_RED2) && ctx->dist[v[i]] > ubd) chk = 1;
        if (chk) { mark[i] = 1; nr++; }
      }
      if (!nr) break;
      for (uint32_t i = 0; i < s; i++)
        if (mark[i]) { st[i] = ST_X; dC[i] = dR[i] = 0; }
      for (uint32_t i = 0; i < s; i++)
        if (mark[i])
          for (uint32_t k = ctx->off[v[i]]; k < ctx->off[v[i] + 1]; k++) {
            int32_t x = ctx->pos[ctx->adj[k]];
            if (x >= 0 && st[x] != ST_X) dR[x]--;
          }
    }
  }
  uint32_t nR = 0;
  for (uint32_t i = 0; i < s; i++) nR += st[i] == ST_R;
  hdr[4] = csize + nR;
  /* bounds */
  uint32_t p1 = UINT32_MAX, p2 = UINT32_MAX;
  if (rules & ORC_PRUN1) {
    for (uint32_t i = 0; i < s; i++)
      if (st[i] == ST_C) {
        uint32_t a = dC[i] + h - csize, b = dR[i] + dC[i];
        uint32_t x = a < b ? a : b;
        if (x < p1) p1 = x;
      }
  }
  if (rules & ORC_PRUN2) {
    uint32_t *A = (uint32_t *)malloc((csize ? csize : 1) * sizeof(uint32_t));
    uint32_t *B = (uint32_t *)malloc((nR ? nR : 1) * sizeof(uint32_t));
    uint32_t na = 0, nb = 0;
    for (uint32_t i = 0; i < s; i++) {
      if (st[i] == ST_C) A[na++] = dC[i];
      else if (st[i] == ST_R) B[nb++] = dC[i];
    }
    qsort(A, na, sizeof(uint32_t), cmp_u32);
    qsort(B, nb, sizeof(uint32_t), cmp_u32); /* ascending; read from end */
    uint32_t t = h - csize;
    if (t > nb) t = nb;
    for (uint32_t it = 0; it < t; it++) {
      uint32_t x = B[nb - 1 - it];
      uint32_t k = x < na ? x : na;
      for (uint32_t i = 0; i < k; i++) A[i]++;
      qsort(A, na, sizeof(uint32_t), cmp_u32);
    }
    if (na) p2 = A[0];
    free(A);
    free(B);
  }
  hdr[5] = p1;
  hdr[6] = p2;
  /* with both bounds switched off the reference reads an uninitialised
   * limit (src/helpers.cc:476-487); here "off" means no pruning */
  uint32_t ub = p1 < p2 ? p1 : p2;
  if (ub <= kl) { hdr[0] = 2; goto done; }
  if (csize + nR < l) { hdr[0] = 3; goto done; }
  /* ustar */
  double bs = 0;
  int32_t us = -1;
  for (uint32_t i = 0; i < s; i++) {
    if (st[i] != ST_R) continue;
    double sc = 0;
    for (uint32_t k = ctx->off[v[i]]; k < ctx->off[v[i] + 1]; k++) {
      int32_t j = ctx->pos[ctx->adj[k]];
      if (j >= 0 && st[j] == ST_C) sc += dC[j] != 0 ? (double)1 / dC[j] : 1.0;
    }
    if (sc > 0) sc += (double)dR[i] / dmax;
    if (sc > bs) { bs = sc; us = (int32_t)i; }
  }
  if (us < 0) { hdr[0] = 3; goto done; }
  hdr[7] = v[us];
  /* dominated vertices */
  uint32_t nd = 0;
  dent *D = NULL;
  if (ctx->limit_doms > 0) {
    D = (dent *)malloc((s ? s : 1) * sizeof(dent));
    uint32_t u = v[us];
    for (uint32_t i = 0; i < s; i++) {
      if (st[i] != ST_R || (int32_t)i == us || dC[i] == 0) continue;
      int dom = 1;
      double sc = 0;
      for (uint32_t k = ctx->off[v[i]]; k < ctx->off[v[i] + 1]; k++) {
        uint32_t w = ctx->adj[k];
        int32_t j = ctx->pos[w];
        if (j < 0 || st[j] == ST_X) continue; /* not in the task */
        if (w != u && !adj_has(ctx, u, w)) { dom = 0; break; }
        if (st[j] == ST_C && dC[j] != 0) sc += (double)1 / dC[j];
      }
      if (!dom) continue;
      sc += (double)dR[i] / dmax;
      D[nd].sc = sc;
      D[nd].i = i;
      nd++;
    }
    qsort(D, nd, sizeof(dent), cmp_dom);
    if (nd > ctx->limit_doms) nd = ctx->limit_doms;
  }
  hdr[8] = nd;
  for (uint32_t i = 0; i < nd; i++) doms_out[i] = v[D[i].i];
  /* children: Include, Dom_0..Dom_{nd-1}, Exclude */
  {
    memset(mark, 0, s); /* 1: in D, value = rank+1 stored separately */
    uint32_t *rank = (uint32_t *)malloc((s ? s : 1) * sizeof(uint32_t));
    for (uint32_t i = 0; i < s; i++) rank[i] = UINT32_MAX;
    for (uint32_t r = 0; r < nd; r++) rank[D[r].i] = r;
    uint64_t w = 0;
    uint32_t nk = 0;
    for (int32_t child = -1; child <= (int32_t)nd; child++) {
      /* child -1: Include; 0..nd-1: Dom_child; nd: Exclude */
      uint64_t need = 2 + (uint64_t)s;
      if (w + need > kids_cap) { rc = -1; break; }
      uint64_t hdrpos = w;
      w += 2;
      uint32_t cs = 0, cnt = 0;
      for (uint32_t i = 0; i < s; i++) {
        uint32_t inC;
        if (st[i] == ST_X) continue;
        if (st[i] == ST_C) inC = 1;
        else if ((int32_t)i == us) {
          if (child == (int32_t)nd) continue; /* Exclude drops u* */
          inC = 1;
        } else if (rank[i] != UINT32_MAX) {
          if (child < 0 || child == (int32_t)nd) continue;
          if (rank[i] < (uint32_t)child) continue;
          inC = rank[i] == (uint32_t)child;
        } else inC = 0;
        kids[w++] = (v[i] << 1) | inC;
        cnt++;
        cs += inC;
      }
      if (cs > h || cnt < l) { w = hdrpos; continue; } /* never evaluated */
      kids[hdrpos] = cnt;
      kids[hdrpos + 1] = cs;
      nk++;
    }
    free(rank);
    hdr[9] = nk;
    hdr[10] = (uint32_t)w;
  }
  free(D);
  hdr[0] = rc == 0 ? 0 : hdr[0];
done:
#undef MINDEG_UPDATE
  hdr[1] = kl;
  hdr[3] = csize;
  hdr[2] = best;
  for (uint32_t i = 0; i < s; i++) ctx->pos[v[i]] = -1;
  free(v);
  free(st);
  free(dC);
  free(dR);
  free(mark);
  return rc;
}

/* ------------------------------------------------------------------ */
/* serial DFS branch-and-bound over orc_step (LIFO; Include on top).
 * Per-query flow of main.cu:110-258: ku = min(core[q], h-1)
 * (inc/Intialize.h:207), heuristic incumbent, early answer when kl == ku
 * (main.cu:122-133), ubD (main.cu:154-172), filter + root task.       */
/* ------------------------------------------------------------------ */
typedef struct { uint32_t *e; uint32_t s; } stk_ent;

static double g_time_limit = 0.0; /* seconds per solve, 0 = none */
void orc_set_time_limit(double seconds) { g_time_limit = seconds; }
static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

int orc_solve(const orc_graph *g, uint32_t l, uint32_t h, uint32_t q,
              uint32_t heur, uint32_t limit_doms, uint32_t rules,
              uint64_t node_limit, orc_result *res, uint32_t *H,
              uint32_t h_cap) {
  return orc_solve_from(g, l, h, q, heur, limit_doms, rules, node_limit, 0,
                        res, H, h_cap);
}

int orc_solve_from(const orc_graph *g, uint32_t l, uint32_t h, uint32_t q,
                   uint32_t heur, uint32_t limit_doms, uint32_t rules,
                   uint64_t node_limit, uint32_t kl_floor, orc_result *res,
                   uint32_t *H, uint32_t h_cap) {
  memset(res, 0, sizeof(*res));
  uint32_t ku = g->core[q] < h - 1 ? g->core[q] : h - 1;
  uint32_t kl = 0, hs = 0;
  uint32_t *Hh = (uint32_t *)malloc((g->n ? g->n : 1) * sizeof(uint32_t));
  if (heur) kl = orc_cssc_heu(g, l, h, q, Hh, &hs);
  if (kl_floor > kl) kl = kl_floor; /* a known lower bound (proof-only runs) */
  res->kl_heu = kl;
  res->ku = ku;
  if (kl == ku) {
    res->heu_hit = 1;
    res->degree = kl;
    res->h_size = hs;
    if (H) for (uint32_t i = 0; i < hs && i < h_cap; i++) H[i] = Hh[i];
    free(Hh);
    return 0;
  }
  uint32_t ubd = orc_ubd_host(kl, h);
  res->ubd = ubd;
  orc_qctx ctx;
  memset(&ctx, 0, sizeof(ctx));
  uint32_t nk = 0;
  orc_prepare(g, q, kl, ubd, 1, &ctx, &nk);
  ctx.l = l;
  ctx.h = h;
  ctx.limit_doms = limit_doms;
  ctx.dmax = g->dmax;
  ctx.rules = rules;
  res->n_kept = nk;
  res->n_local = ctx.n;
  uint32_t best_val = kl;
  uint32_t *bestC = (uint32_t *)malloc((ctx.n + 2) * sizeof(uint32_t));
  uint32_t *wit = (uint32_t *)malloc((ctx.n + 2) * sizeof(uint32_t));
  uint32_t bestn = 0;
  int from_bnb = 0;
  size_t scap = 64, sn = 0;
  stk_ent *stk = (stk_ent *)malloc(scap * sizeof(stk_ent));
  stk[0].s = ctx.n;
  stk[0].e = (uint32_t *)malloc((ctx.n ? ctx.n : 1) * sizeof(uint32_t));
  for (uint32_t i = 0; i < ctx.n; i++)
    stk[0].e[i] = (i << 1) | (i == ctx.q_local);
  sn = 1;
  uint32_t hdr[16];
  uint32_t *doms = (uint32_t *)malloc((limit_doms + 1) * sizeof(uint32_t));
  uint64_t kcap = 0;
  uint32_t *kids = NULL;
  const double t_start = now_s();
  while (sn) {
    if (node_limit && res->nodes >= node_limit) { res->status = 1; break; }
    if (g_time_limit > 0 && (res->nodes & 15) == 0 &&
        now_s() - t_start > g_time_limit) { res->status = 2; break; }
    stk_ent t = stk[--sn];
    res->nodes++;
    res->sum_task += t.s;
    if (t.s > res->max_task) res->max_task = t.s;
    {
      uint32_t b = 0, lim = 32;
      while (b < 7 && t.s > lim) { b++; lim <<= 1; }
      res->size_hist[b]++;
    }
    uint64_t need = (uint64_t)(t.s + 2) * (limit_doms + 2);
    if (need > kcap) {
      kcap = need;
      kids = (uint32_t *)realloc(kids, kcap * sizeof(uint32_t));
    }
    orc_step(&ctx, t.e, t.s, kl, hdr, doms, kids, kcap, wit);
    kl = hdr[1];
    if (hdr[2] != UINT32_MAX && hdr[2] > best_val) {
      best_val = hdr[2];
      from_bnb = 1;
      bestn = hdr[11];
      for (uint32_t i = 0; i < bestn; i++) bestC[i] = ctx.gid[wit[i]];
    }
    if (hdr[0] == 0) {
      /* push children in reverse so Include is on top */
      uint32_t nkids = hdr[9];
      uint64_t *offs = (uint64_t *)malloc((nkids ? nkids : 1) * sizeof(uint64_t));
      uint64_t w = 0;
      for (uint32_t c = 0; c < nkids; c++) {
        offs[c] = w;
        w += 2 + kids[w];
      }
      for (int32_t c = (int32_t)nkids - 1; c >= 0; c--) {
        if (sn == scap) {
          scap *= 2;
          stk = (stk_ent *)realloc(stk, scap * sizeof(stk_ent));
        }
        uint32_t cnt = kids[offs[c]];
        stk[sn].s = cnt;
        stk[sn].e = (uint32_t *)malloc((cnt ? cnt : 1) * sizeof(uint32_t));
        memcpy(stk[sn].e, kids + offs[c] + 2, cnt * sizeof(uint32_t));
        sn++;
      }
      free(offs);
    }
    free(t.e);
  }
  while (sn) free(stk[--sn].e);
  free(stk);
  free(kids);
  free(doms);
  res->degree = kl;
  if (from_bnb && best_val == kl) {
    res->h_from_bnb = 1;
    res->h_size = bestn;
    if (H) for (uint32_t i = 0; i < bestn && i < h_cap; i++) H[i] = bestC[i];
  } else {
    res->h_size = hs;
    if (H) for (uint32_t i = 0; i < hs && i < h_cap; i++) H[i] = Hh[i];
  }
  free(bestC);
  free(wit);
  free(Hh);
  orc_qctx_free(&ctx);
  return 0;
}

/* ------------------------------------------------------------------ */
/* exhaustive ground truth for small components                        */
/* ------------------------------------------------------------------ */
uint32_t orc_bruteforce(const orc_graph *g, uint32_t l, uint32_t h,
                        uint32_t q, uint32_t max_comp) {
  uint32_t n = g->n;
  uint32_t *dist = (uint32_t *)malloc(n * sizeof(uint32_t));
  orc_bfs(n, g->off, g->adj, q, dist);
  uint32_t comp[64], nc = 0;
  for (uint32_t v = 0; v < n; v++)
    if (dist[v] != ORC_INF) {
      if (nc >= max_comp || nc >= 64) { free(dist); return UINT32_MAX; }
      comp[nc++] = v;
    }
  free(dist);
  uint32_t qi = 0;
  for (uint32_t i = 0; i < nc; i++) if (comp[i] == q) qi = i;
  uint64_t am[64];
  for (uint32_t i = 0; i < nc; i++) {
    am[i] = 0;
    for (uint32_t j = 0; j < nc; j++)
      for (uint32_t k = g->off[comp[i]]; k < g->off[comp[i] + 1]; k++)
        if (g->adj[k] == comp[j]) am[i] |= 1ull << j;
  }
  uint32_t best = 0;
  uint64_t total = 1ull << nc;
  for (uint64_t S = 0; S < total; S++) {
    if (!((S >> qi) & 1)) continue;
    uint32_t sz = (uint32_t)__builtin_popcountll(S);
    if (sz < l || sz > h) continue;
    /* connectivity */
    uint64_t seen = 1ull << qi, fr = seen;
    while (fr) {
      uint64_t nx = 0;
      for (uint32_t i = 0; i < nc; i++)
        if ((fr >> i) & 1) nx |= am[i] & S;
      nx &= ~seen;
      seen |= nx;
      fr = nx;
    }
    if (seen != S) continue;
    uint32_t md = UINT32_MAX;
    for (uint32_t i = 0; i < nc; i++)
      if ((S >> i) & 1) {
        uint32_t d = (uint32_t)__builtin_popcountll(am[i] & S);
        if (d < md) md = d;
      }
    if (md > best) best = md;
  }
  return best;
}
