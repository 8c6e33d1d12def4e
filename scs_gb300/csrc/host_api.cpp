// host_api.cpp -- host-only entry points of include/scs.h (no GPU needed).
#include <cstdlib>
#include <cstring>
#include <string>

#include "../../include/scs.h"
#include "host_graph.h"

using namespace scs;

extern "C" {

int scs_read_edge_list(const char *path, uint32_t *n, uint64_t *nnz,
                       uint32_t **off, uint32_t **adj) {
  if (!path || !n || !nnz || !off || !adj) return SCS_EINVAL;
  HostGraph g;
  std::string err;
  if (load_edge_list(path, g, err)) return SCS_EIO;
  *n = g.n;
  *nnz = g.adj.size();
  *off = (uint32_t *)malloc((g.off.size()) * 4);
  *adj = (uint32_t *)malloc(std::max<size_t>(g.adj.size(), 1) * 4);
  if (!*off || !*adj) return SCS_ENOMEM;
  memcpy(*off, g.off.data(), g.off.size() * 4);
  if (!g.adj.empty()) memcpy(*adj, g.adj.data(), g.adj.size() * 4);
  return 0;
}

void scs_free(void *p) { free(p); }

int scs_core_decompose(uint32_t n, const uint32_t *off, const uint32_t *adj,
                       uint32_t *core) {
  if (!core) return SCS_EINVAL;
  HostGraph g;
  std::string err;
  if (adopt_csr(n, off, adj, g, err)) return SCS_EINVAL;
  memcpy(core, g.core.data(), (size_t)n * 4);
  return 0;
}

int scs_greedy_incumbent(uint32_t n, const uint32_t *off, const uint32_t *adj,
                         uint32_t l, uint32_t h, uint32_t q, uint32_t *kl,
                         uint32_t *H, uint32_t *hsize) {
  if (!kl || q >= n) return SCS_EINVAL;
  HostGraph g;
  std::string err;
  if (adopt_csr(n, off, adj, g, err)) return SCS_EINVAL;
  HeuWork w;
  std::vector<uint32_t> out;
  *kl = greedy_incumbent(g, l, h, q, w, out);
  if (hsize) *hsize = (uint32_t)out.size();
  if (H) memcpy(H, out.data(), out.size() * 4);
  return 0;
}

uint32_t scs_distance_bound(uint32_t kl, uint32_t h) { return ubd_host(kl, h); }

}  // extern "C"
