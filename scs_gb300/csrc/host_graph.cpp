// host_graph.cpp -- graph load, core numbers and the greedy incumbent.
//
// load_edge_list follows src/Graph.h:5-67: "<n> <m>" header, then pairs,
// self-loops dropped, both directions merged into ascending unique rows.
// The parse is split over threads at line boundaries; a file whose lines do
// not all hold exactly two integers is parsed token by token instead, which
// is the reference's own semantics (stop at the first non-integer token).
//
// greedy_incumbent restates CSSC_heu (inc/heuristic.h:321-349) and its three
// greedy growers heu2 (:8-120), heu3 (:125-239) and heu4 (:242-317).  The
// priority queues hold totally ordered pairs, so the pop order -- and hence
// kl and H -- is the reference's exactly.
#include "host_graph.h"

#include <algorithm>
#include <atomic>
#include <cctype>
#include <cstdio>
#include <cstring>
#include <functional>
#include <queue>
#include <thread>
#include <utility>

namespace scs {

namespace {

struct Reader {
  const char *p, *end;
  bool next(uint64_t &v) {
    while (p < end && isspace((unsigned char)*p)) p++;
    if (p >= end || !isdigit((unsigned char)*p)) return false;
    uint64_t x = 0;
    while (p < end && isdigit((unsigned char)*p)) x = x * 10 + (uint64_t)(*p++ - '0');
    v = x;
    return true;
  }
};

// Parse "u v" lines of [b, e); returns false if any line is not two integers.
bool parse_lines(const char *b, const char *e, std::vector<uint64_t> &out) {
  const char *p = b;
  while (p < e) {
    const char *le = (const char *)memchr(p, '\n', (size_t)(e - p));
    if (!le) le = e;
    Reader r{p, le};
    uint64_t u, v, extra;
    bool any = false;
    {  // blank line?
      const char *q = p;
      while (q < le && isspace((unsigned char)*q)) q++;
      any = q < le;
    }
    if (any) {
      if (!r.next(u) || !r.next(v) || r.next(extra)) return false;
      while (r.p < le && isspace((unsigned char)*r.p)) r.p++;
      if (r.p != le) return false;
      out.push_back((u << 32) | v);
    }
    p = le + 1;
  }
  return true;
}

int build_csr(uint32_t n, std::vector<std::vector<uint64_t>> &parts,
              HostGraph &g, std::string &err) {
  std::vector<uint64_t> cnt(n + 1, 0);
  for (auto &pp : parts)
    for (uint64_t e : pp) {
      uint64_t u = e >> 32, v = e & 0xffffffffu;
      if (u == v) continue;
      if (u >= n || v >= n) {
        err = "vertex id out of range";
        return -2;
      }
      cnt[u + 1]++;
      cnt[v + 1]++;
    }
  for (uint32_t i = 0; i < n; i++) cnt[i + 1] += cnt[i];
  std::vector<uint32_t> raw(cnt[n]);
  std::vector<uint64_t> fill(cnt.begin(), cnt.end() - 1);
  for (auto &pp : parts) {
    for (uint64_t e : pp) {
      uint32_t u = (uint32_t)(e >> 32), v = (uint32_t)(e & 0xffffffffu);
      if (u == v) continue;
      raw[fill[u]++] = v;
      raw[fill[v]++] = u;
    }
    std::vector<uint64_t>().swap(pp);
  }
  // sort + unique each row, in parallel
  std::vector<uint32_t> rowlen(n, 0);
  unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  std::vector<std::thread> th;
  for (unsigned k = 0; k < nt; k++)
    th.emplace_back([&, k]() {
      for (uint32_t i = k; i < n; i += nt) {
        auto b = raw.begin() + (long)cnt[i], e = raw.begin() + (long)cnt[i + 1];
        std::sort(b, e);
        rowlen[i] = (uint32_t)(std::unique(b, e) - b);
      }
    });
  for (auto &t : th) t.join();
  g.off.assign(n + 1, 0);
  for (uint32_t i = 0; i < n; i++) g.off[i + 1] = g.off[i] + rowlen[i];
  g.adj.resize(g.off[n]);
  for (uint32_t i = 0; i < n; i++)
    std::copy(raw.begin() + (long)cnt[i], raw.begin() + (long)cnt[i] + rowlen[i],
              g.adj.begin() + g.off[i]);
  g.n = n;
  return 0;
}

}  // namespace

int load_edge_list(const char *path, HostGraph &g, std::string &err, bool with_core) {
  FILE *f = fopen(path, "rb");
  if (!f) {
    err = std::string("cannot open ") + path;
    return -1;
  }
  fseek(f, 0, SEEK_END);
  long sz = ftell(f);
  fseek(f, 0, SEEK_SET);
  std::string buf;
  buf.resize((size_t)std::max(sz, 0L));
  size_t rd = fread(&buf[0], 1, buf.size(), f);
  fclose(f);
  buf.resize(rd);
  Reader hr{buf.data(), buf.data() + buf.size()};
  uint64_t n64, m64;
  if (!hr.next(n64) || !hr.next(m64) || n64 > 0xFFFFFFF0ull) {
    err = "bad header";
    return -3;
  }
  const char *body = hr.p;
  const char *end = buf.data() + buf.size();
  // chunk at line boundaries
  unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  if ((size_t)(end - body) < (1u << 20)) nt = 1;
  std::vector<const char *> cut(nt + 1);
  cut[0] = body;
  cut[nt] = end;
  for (unsigned k = 1; k < nt; k++) {
    const char *c = body + (size_t)(end - body) * k / nt;
    if (c < cut[k - 1]) c = cut[k - 1];
    const char *nl = (const char *)memchr(c, '\n', (size_t)(end - c));
    cut[k] = nl ? nl + 1 : end;
  }
  std::vector<std::vector<uint64_t>> parts(nt);
  std::vector<char> ok(nt, 1);
  {
    std::vector<std::thread> th;
    for (unsigned k = 0; k < nt; k++)
      th.emplace_back([&, k]() { ok[k] = parse_lines(cut[k], cut[k + 1], parts[k]); });
    for (auto &t : th) t.join();
  }
  bool all_ok = true;
  for (char c : ok) all_ok = all_ok && c;
  if (!all_ok) {  // token-by-token, stopping at the first non-integer
    parts.assign(1, {});
    Reader r{body, end};
    uint64_t u, v;
    while (r.next(u) && r.next(v)) parts[0].push_back((u << 32) | v);
  }
  int rc = build_csr((uint32_t)n64, parts, g, err);
  if (rc) return rc;
  g.m_header = m64;
  finish_graph(g, with_core);
  return 0;
}

int adopt_csr(uint32_t n, const uint32_t *off, const uint32_t *adj,
              HostGraph &g, std::string &err, bool with_core) {
  if (!off || (n && !adj)) {
    err = "null CSR";
    return -1;
  }
  if (off[0] != 0) {
    err = "off[0] != 0";
    return -1;
  }
  for (uint32_t i = 0; i < n; i++) {
    if (off[i + 1] < off[i]) {
      err = "offsets not monotone";
      return -1;
    }
    for (uint32_t k = off[i]; k < off[i + 1]; k++) {
      if (adj[k] >= n || adj[k] == i) {
        err = "bad neighbour id or self-loop";
        return -1;
      }
      if (k > off[i] && adj[k] <= adj[k - 1]) {
        err = "rows must be strictly ascending";
        return -1;
      }
    }
  }
  // Every edge must be listed in both of its rows: the counts of the greedy
  // incumbent and of the search are taken from either side.
  std::atomic<bool> asym{false};
  unsigned nt = off[n] < (1u << 20) ? 1u
                                    : std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  std::vector<std::thread> th;
  for (unsigned k = 0; k < nt; k++)
    th.emplace_back([&, k]() {
      for (uint32_t i = k; i < n && !asym.load(std::memory_order_relaxed); i += nt)
        for (uint32_t e = off[i]; e < off[i + 1]; e++) {
          uint32_t j = adj[e];
          if (!std::binary_search(adj + off[j], adj + off[j + 1], i)) {
            asym.store(true, std::memory_order_relaxed);
            break;
          }
        }
    });
  for (auto &t : th) t.join();
  if (asym.load()) {
    err = "CSR not symmetric: an edge is missing from one of its rows";
    return -1;
  }
  g.n = n;
  g.off.assign(off, off + n + 1);
  g.adj.assign(adj, adj + off[n]);
  g.m_header = off[n] / 2;
  finish_graph(g, with_core);
  return 0;
}

void finish_graph(HostGraph &g, bool with_core) {
  const uint32_t n = g.n;
  g.degree.resize(n);
  g.dmax = 0;
  for (uint32_t i = 0; i < n; i++) {
    g.degree[i] = g.off[i + 1] - g.off[i];
    g.dmax = std::max(g.dmax, g.degree[i]);
  }
  // bin-sort peeling (core numbers are unique; src/Graph.h:82-109 computes
  // the same array with a bucket list)
  if (!with_core) {
    g.core.clear();
    return;
  }
  g.core.assign(n, 0);
  if (!n) return;
  std::vector<uint32_t> deg(g.degree), bin(g.dmax + 2, 0), vert(n), pos(n);
  for (uint32_t v = 0; v < n; v++) bin[deg[v]]++;
  uint32_t start = 0;
  for (uint32_t d = 0; d <= g.dmax; d++) {
    uint32_t c = bin[d];
    bin[d] = start;
    start += c;
  }
  for (uint32_t v = 0; v < n; v++) {
    pos[v] = bin[deg[v]];
    vert[pos[v]] = v;
    bin[deg[v]]++;
  }
  for (uint32_t d = g.dmax; d >= 1; d--) bin[d] = bin[d - 1];
  bin[0] = 0;
  for (uint32_t i = 0; i < n; i++) {
    uint32_t v = vert[i];
    for (uint32_t k = g.off[v]; k < g.off[v + 1]; k++) {
      uint32_t u = g.adj[k];
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
  for (uint32_t v = 0; v < n; v++) g.core[v] = deg[v];
}

void HeuWork::ensure(uint32_t n) {
  if (sta.size() < n) {
    sta.assign(n, 0);
    deg.assign(n, 0);
    slot.assign(n, 0);
    inS.assign(n, 0);
  }
  touched.clear();
}

uint32_t ubd_host(uint32_t kl, uint32_t h) {
  if (kl <= 1) return h - 1;
  uint32_t ubd = 0;
  for (uint32_t d = 1; d <= h; d++) {
    if (d == 1 || d == 2) {
      if (kl + d > h) {
        ubd = d - 1;
        break;
      }
    } else {
      uint64_t min_n = (uint64_t)kl + d + 1 + (uint64_t)(d / 3) * (kl - 2);
      if (h < min_n) {
        ubd = d - 1;
        break;
      }
    }
  }
  return ubd;
}

namespace {

constexpr uint32_t HEU_INF = 1000000000u;

// heu2: grow from q, always taking the frontier vertex with most neighbours
// inside H (ties to the larger id).
//
// The reference recounts |N(x) & H| by a scan of N(x) for every neighbour x
// of every vertex that joins H, which costs sum deg(v) * deg(x) and takes
// seconds per query on graphs with hubs.  Here cnt[x] = |N(x) & H| is kept
// for every vertex: a vertex joining H adds one to each of its neighbours
// (the graph is symmetric with unique rows, which adopt_csr and the loader
// guarantee), so the count pushed for x is the same number the scan gives.
// For a member of H the same count is its degree inside H.  The queue holds
// the same (count, id) pairs, so the pop order, kl and H are unchanged.
uint32_t heu2(const HostGraph &g, uint32_t N1, uint32_t N2, uint32_t q,
              HeuWork &w, std::vector<uint32_t> &H) {
  const uint32_t *off = g.off.data(), *adj = g.adj.data();
  auto &sta = w.sta;
  auto &cnt = w.deg;
  auto &touched = w.touched;
  auto &tH = w.tH;
  touched.clear();
  tH.clear();
  uint32_t tkl = 0, tsz = 0;
  std::priority_queue<std::pair<uint32_t, uint32_t>> Q;
  Q.push({0, q});
  sta[q] = 1;
  touched.push_back(q);
  while (!Q.empty()) {
    uint32_t v = Q.top().second;
    Q.pop();
    if (sta[v] == 2) continue;
    tH.push_back(v);
    sta[v] = 2;
    for (uint32_t j = off[v]; j < off[v + 1]; j++) ++cnt[adj[j]];
    for (uint32_t j = off[v]; j < off[v + 1]; j++) {
      uint32_t x = adj[j];
      if (sta[x] == 2) continue;
      Q.push({cnt[x], x});
      if (sta[x] == 0) {
        sta[x] = 1;
        touched.push_back(x);
      }
    }
    if (tH.size() >= N1) {
      uint32_t md = HEU_INF;
      for (uint32_t x : tH) md = std::min(md, cnt[x]);
      if (md >= tkl) {
        tkl = md;
        tsz = (uint32_t)tH.size();
      }
    }
    if (tH.size() == N2) break;
  }
  H.assign(tH.begin(), tH.begin() + tsz);
  for (uint32_t x : touched) {
    sta[x] = 0;
    cnt[x] = 0;
  }
  return tkl;
}

// heu3: as heu2 with the connection score sum 1/deg_H(y) over the members y
// of H adjacent to x, plus degree/dMAX.
//
// The reference rescans N(x) for each candidate x, summing in adjacency
// order, i.e. by ascending y (rows are ascending).  Here each candidate keeps
// its members of H in ascending order in a 64-byte record (spilling to a
// vector past HeuRec::INLINE), extended when a neighbour joins H, and the sum
// runs over that list: the same terms added in the same order, so every score
// is bit-identical.  A candidate enters the queue only when its score beats
// the best one it already holds there: an entry at or below that is popped
// after it (the pairs order by score, then id), when the candidate is already
// in H, so the pop order is the reference's.
uint32_t heu3(const HostGraph &g, uint32_t N1, uint32_t N2, uint32_t q,
              HeuWork &w, std::vector<uint32_t> &H) {
  const uint32_t *off = g.off.data(), *adj = g.adj.data();
  const double dM = (double)g.dmax;
  constexpr uint32_t IN_H = 1;  // st[x]: 0 untouched, 1 in H, r + 2 record r
  auto &st = w.slot;
  auto &deg = w.deg;
  auto &recs = w.recs;
  auto &touched = w.touched;
  auto &tH = w.tH;
  auto &cand = w.cand;
  touched.clear();
  tH.clear();
  uint32_t nrec = 0, nspill = 0;
  auto new_record = [&](uint32_t x) {
    if (nrec == recs.size()) recs.emplace_back();
    HeuRec &r = recs[nrec];
    r.len = 0;
    r.spill = 0;
    r.best = -1.0;
    r.dterm = (double)g.degree[x] / dM;
    st[x] = nrec + 2;
    touched.push_back(x);
    return nrec++;
  };
  uint32_t tkl = 0, tsz = 0;
  std::priority_queue<std::pair<double, uint32_t>> Q;
  Q.push({0.0, q});
  new_record(q);
  while (!Q.empty()) {
    uint32_t v = Q.top().second;
    Q.pop();
    if (st[v] == IN_H) continue;
    tH.push_back(v);
    st[v] = IN_H;
    // degrees inside H first: every score below reads them
    cand.clear();
    for (uint32_t j = off[v]; j < off[v + 1]; j++) {
      uint32_t x = adj[j], sx = st[x];
      if (sx == IN_H) {
        ++deg[x];
        ++deg[v];
      } else {
        cand.push_back(x);
        cand.push_back(sx ? sx - 2 : new_record(x));
      }
    }
    for (size_t c = 0; c < cand.size(); c += 2) {
      uint32_t x = cand[c];
      HeuRec &r = recs[cand[c + 1]];
      double sc = 0;
      if (!r.spill && r.len < HeuRec::INLINE) {
        uint32_t i = r.len++;
        while (i > 0 && r.ids[i - 1] > v) {
          r.ids[i] = r.ids[i - 1];
          i--;
        }
        r.ids[i] = v;
        for (uint32_t k = 0; k < r.len; k++)
          if (deg[r.ids[k]] != 0) sc += (double)1 / deg[r.ids[k]];
      } else {
        if (!r.spill) {
          if (nspill == w.spills.size()) w.spills.emplace_back();
          w.spills[nspill].assign(r.ids, r.ids + r.len);
          r.spill = ++nspill;
        }
        auto &L = w.spills[r.spill - 1];
        L.insert(std::upper_bound(L.begin(), L.end(), v), v);
        for (uint32_t y : L)
          if (deg[y] != 0) sc += (double)1 / deg[y];
      }
      sc += r.dterm;
      if (sc > r.best) {
        r.best = sc;
        Q.push({sc, x});
      }
    }
    if (tH.size() >= N1) {
      uint32_t md = HEU_INF;
      for (uint32_t x : tH) md = std::min(md, deg[x]);
      if (md >= tkl) {
        tkl = md;
        tsz = (uint32_t)tH.size();
      }
    }
    if (tH.size() == N2) break;
  }
  H.assign(tH.begin(), tH.begin() + tsz);
  for (uint32_t x : touched) st[x] = 0;
  for (uint32_t x : tH) deg[x] = 0;
  return tkl;
}

// heu4: peel {q} + N(q) by minimum degree (q counted with one extra degree)
uint32_t heu4(const HostGraph &g, uint32_t N1, uint32_t N2, uint32_t q,
              HeuWork &w, std::vector<uint32_t> &H) {
  H.clear();
  const uint32_t *off = g.off.data(), *adj = g.adj.data();
  if (g.degree[q] < N1 - 1u) return 0;
  auto &inS = w.inS;
  auto &deg = w.deg;
  std::vector<uint32_t> S;
  S.reserve(g.degree[q] + 1);
  S.push_back(q);
  inS[q] = 1;
  ++deg[q];
  for (uint32_t j = off[q]; j < off[q + 1]; j++) {
    uint32_t x = adj[j];
    S.push_back(x);
    inS[x] = 1;
    for (uint32_t k = off[x]; k < off[x + 1]; k++)
      if (inS[adj[k]]) {
        ++deg[adj[k]];
        ++deg[x];
      }
  }
  std::priority_queue<std::pair<uint32_t, uint32_t>,
                      std::vector<std::pair<uint32_t, uint32_t>>,
                      std::greater<std::pair<uint32_t, uint32_t>>>
      Q;
  for (uint32_t x : S) Q.push({deg[x], x});
  std::vector<uint32_t> rmv;
  uint32_t rmv_idx = 0, mindeg = 0;
  while (!Q.empty()) {
    uint32_t d = Q.top().first, v = Q.top().second;
    Q.pop();
    if (!inS[v]) continue;
    uint32_t remain = (uint32_t)S.size() - (uint32_t)rmv.size();
    if (remain >= N1 && remain <= N2 && d > mindeg) {
      mindeg = d;
      rmv_idx = (uint32_t)rmv.size();
    }
    if (remain == N1) break;
    inS[v] = 0;
    rmv.push_back(v);
    for (uint32_t j = off[v]; j < off[v + 1]; j++)
      if (inS[adj[j]]) {
        --deg[adj[j]];
        Q.push({deg[adj[j]], adj[j]});
      }
  }
  for (uint32_t x : S) inS[x] = 1;
  for (uint32_t i = 0; i < rmv_idx; i++) inS[rmv[i]] = 0;
  for (uint32_t x : S)
    if (inS[x]) H.push_back(x);
  for (uint32_t x : S) {
    inS[x] = 0;
    deg[x] = 0;
  }
  return mindeg;
}

}  // namespace

uint32_t greedy_incumbent(const HostGraph &g, uint32_t l, uint32_t h,
                          uint32_t q, HeuWork &w, std::vector<uint32_t> &H) {
  w.ensure(g.n);
  std::vector<uint32_t> H2, H3, H4;
  uint32_t k2 = heu2(g, l, h, q, w, H2);
  uint32_t k3 = heu3(g, l, h, q, w, H3);
  uint32_t k4 = heu4(g, l, h, q, w, H4);
  if (k4 >= k3 && k4 >= k2) {
    H.swap(H4);
    return k4;
  }
  if (k3 >= k2) {
    H.swap(H3);
    return k3;
  }
  H.swap(H2);
  return k2;
}

bool verify_community(const HostGraph &g, const uint32_t *H, uint32_t hs,
                      uint32_t q, uint32_t l, uint32_t h, uint32_t &md) {
  md = 0;
  if (hs == 0) return false;
  std::vector<uint32_t> mem(H, H + hs);
  std::sort(mem.begin(), mem.end());
  mem.erase(std::unique(mem.begin(), mem.end()), mem.end());
  if (mem.back() >= g.n) return false;
  // Membership by stamp (one array per thread, reused across calls): a row
  // scan costs one lookup per neighbour, not a binary search.  A hub in H
  // with thousands of neighbours is common, and results are verified
  // between search slices.
  thread_local std::vector<uint32_t> stamp, pos;
  thread_local uint32_t epoch = 0;
  if (stamp.size() < g.n) {
    stamp.assign(g.n, 0);
    pos.assign(g.n, 0);
    epoch = 0;
  }
  if (++epoch == 0) {
    std::fill(stamp.begin(), stamp.end(), 0u);
    epoch = 1;
  }
  for (uint32_t i = 0; i < (uint32_t)mem.size(); i++) {
    stamp[mem[i]] = epoch;
    pos[mem[i]] = i;
  }
  const uint32_t *off = g.off.data(), *adj = g.adj.data();
  auto in = [&](uint32_t v) { return stamp[v] == epoch; };
  uint32_t mind = UINT32_MAX;
  for (uint32_t v : mem) {
    uint32_t d = 0;
    for (uint32_t k = off[v]; k < off[v + 1]; k++) d += in(adj[k]);
    mind = std::min(mind, d);
  }
  md = mind;
  std::vector<uint32_t> stack{mem[0]};
  std::vector<char> vis(mem.size(), 0);
  vis[0] = 1;
  size_t cnt = 1;
  while (!stack.empty()) {
    uint32_t v = stack.back();
    stack.pop_back();
    for (uint32_t k = off[v]; k < off[v + 1]; k++) {
      const uint32_t w = adj[k];
      if (in(w) && !vis[pos[w]]) {
        vis[pos[w]] = 1;
        cnt++;
        stack.push_back(w);
      }
    }
  }
  bool conn = cnt == mem.size();
  return conn && q < g.n && in(q) && mem.size() >= l && mem.size() <= h;
}

}  // namespace scs
