// verify.cpp -- scs_verify: checks answer communities against the graph.
//
//   scs_verify <graph edge list> <communities file>
//
// The communities file is the one scs_server writes when SCS_COMMUNITIES is
// set (a header line, then "QID|N1|N2|Degree|Status|v1 v2 ..." rows).  For
// each row the community must have valid, distinct vertex ids, contain the
// query vertex, have between N1 and N2 vertices, be connected, and have a
// minimum internal degree equal to the reported Degree.  One line per row
// goes to stdout ("QID|N1|N2|Degree|<min degree found>|OK" or "...|FAIL
// <reason>"), then a summary.  Exit status: 0 all rows verified, 1 some row
// failed, 2 usage, I/O or format error.
//
// The reference reports only the degree (main.cu:328-334) and never its
// community, so it has no counterpart of this tool; the graph is read with
// the reference's edge-list semantics (src/Graph.h:5-67).
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/scs.h"

namespace {

const char *reason(int c) {
  switch (c) {
    case SCS_CHECK_EMPTY: return "empty community";
    case SCS_CHECK_RANGE: return "vertex id out of range";
    case SCS_CHECK_REPEAT: return "repeated vertex id";
    case SCS_CHECK_NO_QUERY: return "query vertex missing";
    case SCS_CHECK_SIZE: return "size outside [N1, N2]";
    case SCS_CHECK_DISCONNECTED: return "not connected";
    default: return "invalid arguments";
  }
}

// Parse an unsigned decimal field; false on anything else.
bool parse_u32(const std::string &t, uint32_t &v) {
  if (t.empty() || t.size() > 10) return false;
  uint64_t x = 0;
  for (char c : t) {
    if (c < '0' || c > '9') return false;
    x = x * 10 + (uint64_t)(c - '0');
  }
  if (x > 0xFFFFFFFFull) return false;
  v = (uint32_t)x;
  return true;
}

}  // namespace

int main(int argc, char **argv) {
  if (argc != 3) {
    std::cerr << "usage: scs_verify <graph edge list> <communities file>" << std::endl;
    return 2;
  }
  uint32_t n = 0, *off = nullptr, *adj = nullptr;
  uint64_t nnz = 0;
  if (scs_read_edge_list(argv[1], &n, &nnz, &off, &adj) != 0) {
    std::cerr << "scs_verify: cannot read graph " << argv[1] << std::endl;
    return 2;
  }
  std::ifstream in(argv[2]);
  if (!in) {
    std::cerr << "scs_verify: cannot open " << argv[2] << std::endl;
    scs_free(off);
    scs_free(adj);
    return 2;
  }
  std::string line;
  size_t rows = 0, ok = 0, lineno = 0;
  bool format_error = false;
  while (std::getline(in, line)) {
    lineno++;
    if (!line.empty() && line.back() == '\r') line.pop_back();
    if (line.empty() || line.rfind("QID|", 0) == 0) continue;  // blank or header
    std::vector<std::string> f;
    std::stringstream ss(line);
    std::string tok;
    while (std::getline(ss, tok, '|')) f.push_back(tok);
    if (line.back() == '|') f.push_back("");
    uint32_t qid = 0, l = 0, h = 0, degree = 0, status = 0;
    if (f.size() != 6 || !parse_u32(f[0], qid) || !parse_u32(f[1], l) ||
        !parse_u32(f[2], h) || !parse_u32(f[3], degree) || !parse_u32(f[4], status)) {
      std::cerr << "scs_verify: line " << lineno << ": malformed row" << std::endl;
      format_error = true;
      continue;
    }
    std::vector<uint32_t> H;
    std::stringstream hs(f[5]);
    bool bad_id = false;
    while (hs >> tok) {
      uint32_t v = 0;
      if (!parse_u32(tok, v)) bad_id = true;
      H.push_back(v);
    }
    rows++;
    std::cout << qid << "|" << l << "|" << h << "|" << degree << "|";
    if (bad_id) {
      std::cout << "-|FAIL malformed vertex id" << std::endl;
      continue;
    }
    uint32_t md = 0;
    const int c = scs_check_community(n, off, adj, H.data(), (uint32_t)H.size(), qid, l, h, &md);
    std::cout << md << "|";
    if (c != SCS_CHECK_OK) {
      std::cout << "FAIL " << reason(c) << std::endl;
    } else if (md != degree) {
      std::cout << "FAIL minimum degree " << md << " != reported " << degree << std::endl;
    } else {
      std::cout << "OK" << std::endl;
      ok++;
    }
  }
  std::cout << "verified " << ok << " of " << rows << " rows" << std::endl;
  scs_free(off);
  scs_free(adj);
  if (format_error) return 2;
  return ok == rows ? 0 : 1;
}
