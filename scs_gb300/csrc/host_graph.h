// host_graph.h -- host-side graph and greedy incumbent of the engine.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace scs {

struct HostGraph {
  uint32_t n = 0;
  uint64_t m_header = 0;
  uint32_t dmax = 0;
  std::vector<uint32_t> off;     // n+1
  std::vector<uint32_t> adj;     // ascending per row
  std::vector<uint32_t> degree;  // n
  std::vector<uint32_t> core;    // n
};

// Edge-list load with the reference's semantics (src/Graph.h:5-67).
// Returns 0, or a negative code with a message in err.
// with_core = false leaves g.core empty (the engine computes it on the GPU).
int load_edge_list(const char *path, HostGraph &g, std::string &err, bool with_core = true);
// Validate a caller CSR (rows strictly ascending, no self-loops, every edge in
// both rows) and adopt it.
int adopt_csr(uint32_t n, const uint32_t *off, const uint32_t *adj,
              HostGraph &g, std::string &err, bool with_core = true);
// Degrees, dmax and (with_core) core numbers by bin-sort peeling.
void finish_graph(HostGraph &g, bool with_core = true);

// heu3's per-candidate record: its members of H in ascending id order
// (inline up to INLINE, else in HeuWork::spills[spill - 1]), the best score
// it holds in the queue, and its degree/dMAX term.  One cache line.
struct alignas(64) HeuRec {
  static constexpr uint32_t INLINE = 10;
  uint32_t len, spill;
  double best, dterm;
  uint32_t ids[INLINE];
};

// Per-thread work arrays for the greedy incumbent; reused across queries.
struct HeuWork {
  std::vector<uint32_t> sta, deg, tH, touched;
  std::vector<uint32_t> slot;  // heu3: 0 untouched, 1 in H, r + 2 record r
  std::vector<uint32_t> cand;  // heu3: (candidate, record) pairs of one pop
  std::vector<HeuRec> recs;
  std::vector<std::vector<uint32_t>> spills;
  std::vector<uint8_t> inS;
  void ensure(uint32_t n);
};

// kl = max(heu2, heu3, heu4) with the reference's tie order
// (inc/heuristic.h:321-349); H receives the chosen community.
uint32_t greedy_incumbent(const HostGraph &g, uint32_t l, uint32_t h,
                          uint32_t q, HeuWork &w, std::vector<uint32_t> &H);

// distance bound main.cu:154-172 (host form)
uint32_t ubd_host(uint32_t kl, uint32_t h);

// Check a community: connected, contains q, l <= |H| <= h; returns its min
// degree in `md` (0 for empty).
bool verify_community(const HostGraph &g, const uint32_t *H, uint32_t hs,
                      uint32_t q, uint32_t l, uint32_t h, uint32_t &md);

}  // namespace scs
