// host_api.cpp -- host-only entry points of include/scs.h (no GPU needed).
#include <algorithm>
#include <cstddef>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

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

int scs_check_community(uint32_t n, const uint32_t *off, const uint32_t *adj,
                        const uint32_t *H, uint32_t hs, uint32_t q, uint32_t l,
                        uint32_t h, uint32_t *md) {
  if (md) *md = 0;
  if (!off || !adj || (hs && !H)) return SCS_EINVAL;
  if (hs == 0) return SCS_CHECK_EMPTY;
  std::vector<uint32_t> mem(H, H + hs);
  for (uint32_t v : mem)
    if (v >= n) return SCS_CHECK_RANGE;
  std::sort(mem.begin(), mem.end());
  if (std::adjacent_find(mem.begin(), mem.end()) != mem.end()) return SCS_CHECK_REPEAT;
  auto index = [&](uint32_t v) -> int64_t {
    auto it = std::lower_bound(mem.begin(), mem.end(), v);
    return (it != mem.end() && *it == v) ? (int64_t)(it - mem.begin()) : -1;
  };
  // minimum degree inside H, and connectivity by a DFS over H
  uint32_t mind = UINT32_MAX;
  for (uint32_t v : mem) {
    uint32_t d = 0;
    for (uint32_t k = off[v]; k < off[v + 1]; k++) d += index(adj[k]) >= 0;
    mind = std::min(mind, d);
  }
  if (md) *md = mind;
  if (index(q) < 0) return SCS_CHECK_NO_QUERY;
  if (mem.size() < l || mem.size() > h) return SCS_CHECK_SIZE;
  std::vector<char> vis(mem.size(), 0);
  std::vector<uint32_t> stack{mem[0]};
  vis[0] = 1;
  size_t cnt = 1;
  while (!stack.empty()) {
    const uint32_t v = stack.back();
    stack.pop_back();
    for (uint32_t k = off[v]; k < off[v + 1]; k++) {
      const int64_t i = index(adj[k]);
      if (i >= 0 && !vis[i]) {
        vis[i] = 1;
        cnt++;
        stack.push_back(adj[k]);
      }
    }
  }
  return cnt == mem.size() ? SCS_CHECK_OK : SCS_CHECK_DISCONNECTED;
}

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
  if (adopt_csr(n, off, adj, g, err, /*with_core=*/false)) return SCS_EINVAL;
  HeuWork w;
  std::vector<uint32_t> out;
  *kl = greedy_incumbent(g, l, h, q, w, out);
  if (hsize) *hsize = (uint32_t)out.size();
  if (H) memcpy(H, out.data(), out.size() * 4);
  return 0;
}

uint32_t scs_distance_bound(uint32_t kl, uint32_t h) { return ubd_host(kl, h); }

int scs_abi_layout(uint64_t *out, int max) {
  if (!out || max < 0) return SCS_EINVAL;
  const uint64_t v[8] = {sizeof(scs_config),        offsetof(scs_config, node_budget),
                         offsetof(scs_config, device), offsetof(scs_config, active_queries),
                         sizeof(scs_query),         sizeof(scs_result),
                         offsetof(scs_result, nodes), offsetof(scs_result, search_ns)};
  const int n = max < 8 ? max : 8;
  for (int i = 0; i < n; i++) out[i] = v[i];
  return n;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// server surface helpers
// ---------------------------------------------------------------------------
#include <cctype>
#include <sstream>

#include "server_format.h"

bool scs_is_server_exit(const std::string &str) {
  std::string t = str;
  size_t e = t.find_last_not_of(" \n\r\t");
  if (e == std::string::npos) return false;
  t.erase(e + 1);
  t.erase(0, t.find_first_not_of(" \n\r\t"));
  for (auto &c : t) c = (char)tolower((unsigned char)c);
  return t == "server_exit";
}

bool scs_parse_query(const std::string &s, scs_query &q) {
  std::istringstream iss(s);
  std::vector<unsigned long long> v;
  std::string tok;
  while (iss >> tok) {
    if (tok.empty() || tok.size() > 10) return false;
    for (char c : tok)
      if (!isdigit((unsigned char)c)) return false;
    v.push_back(std::stoull(tok));
  }
  if (v.size() != 5) return false;
  for (auto x : v)
    if (x > 0xFFFFFFFFull) return false;
  q.l = (uint32_t)v[0];
  q.h = (uint32_t)v[1];
  q.q = (uint32_t)v[2];
  q.heuristic = (uint32_t)v[3];
  q.limit_doms = (uint32_t)v[4];
  return true;
}

std::string scs_group_thousands(long long number) {
  std::vector<unsigned> seq;
  if (number <= 0) seq.push_back(0);
  while (number > 0) {
    seq.push_back((unsigned)(number % 1000));
    number /= 1000;
  }
  std::string res;
  char buf[8];
  for (size_t i = seq.size(); i > 0; i--) {
    snprintf(buf, sizeof(buf), i == seq.size() ? "%u" : ",%03u", seq[i - 1]);
    res += buf;
  }
  return res;
}

std::string scs_format_row(const scs_result &r) {
  std::ostringstream os;
  os << r.l << "|" << r.h << "|" << r.q << "|"
     << scs_group_thousands((long long)(r.latency_ns / 1000)) << "|" << r.degree << "|";
  switch (r.status) {
    case SCS_HEURISTIC: os << "0|1|0"; break;  // main.cu:127
    case SCS_TIMEOUT: os << "1|0"; break;      // main.cu:454 (7 fields)
    case SCS_CAPACITY: os << "2|0|0"; break;   // main.cu:351
    default: os << "0|0|0"; break;             // main.cu:332
  }
  return os.str();
}

extern "C" {

int scs_parse_message(const char *text, scs_query *q) {
  if (!text || !q) return SCS_EINVAL;
  if (scs_is_server_exit(text)) return 1;
  return scs_parse_query(text, *q) ? 0 : SCS_EINVAL;
}

int scs_format_result_row(const scs_result *r, char *buf, uint32_t cap) {
  if (!r || !buf || !cap) return SCS_EINVAL;
  std::string s = scs_format_row(*r);
  if (s.size() + 1 > cap) return SCS_EINVAL;
  memcpy(buf, s.c_str(), s.size() + 1);
  return (int)s.size();
}

}  // extern "C"
