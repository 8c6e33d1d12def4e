// ref_driver.cu -- exposes the reference's OWN CPU code (graph loader, core
// decomposition, BFS and greedy heuristics, compiled from its sources where
// they lie) through a small C ABI so tests can pin the oracle against it.
// TEST INFRASTRUCTURE ONLY.  Built by oracle/build_ref.py into oracle/_ref/
// (git-ignored); the reference headers are included by path (SCS_REF_DIR).
//
// Reference entry points used:
//   load_graph                     src/Graph.h:5-67
//   core_decomposition_linear_list src/Graph.h:82-109
//   cal_query_dist                 src/Graph.h:111-142
//   heu2 / heu3 / heu4 / CSSC_heu  inc/heuristic.h:8-349
#include SCS_REF_HEURISTIC_H

#include <cstdint>
#include <cstring>

extern "C" {

int ref_load(const char *path) {
  load_graph(path);
  core_decomposition_linear_list();
  q_dist = new ui[n];
  queries = new queryData[1];
  return 0;
}

void ref_sizes(uint32_t *n_out, uint64_t *m_header, uint64_t *nnz,
               uint32_t *dmax) {
  *n_out = n;
  *m_header = m;
  *nnz = pstart[n];
  *dmax = dMAX;
}

void ref_copy(uint32_t *off, uint32_t *adj, uint32_t *deg, uint32_t *cor) {
  memcpy(off, pstart, (size_t)(n + 1) * sizeof(ui));
  memcpy(adj, edges, (size_t)pstart[n] * sizeof(ui));
  memcpy(deg, degree, (size_t)n * sizeof(ui));
  memcpy(cor, core, (size_t)n * sizeof(ui));
}

void ref_bfs(uint32_t q, uint32_t *dist) {
  cal_query_dist(q);
  memcpy(dist, q_dist, (size_t)n * sizeof(ui));
}

// which: 2, 3, 4 for heu2/heu3/heu4, 0 for CSSC_heu (the max of the three).
uint32_t ref_heu(uint32_t which, uint32_t l, uint32_t h, uint32_t q,
                 uint32_t *H, uint32_t *hsize) {
  vector<ui> out;
  ui kl = 0;
  if (which == 2) heu2(out, kl, l, h, q);
  else if (which == 3) heu3(out, kl, l, h, q);
  else if (which == 4) heu4(out, kl, l, h, q);
  else {
    queries[0].N1 = l;
    queries[0].N2 = h;
    queries[0].QID = q;
    queries[0].kl = 0;
    CSSC_heu(0);
    kl = queries[0].kl;
    out = ::H;
  }
  for (size_t i = 0; i < out.size(); i++) H[i] = out[i];
  *hsize = (uint32_t)out.size();
  return kl;
}

}  // extern "C"
