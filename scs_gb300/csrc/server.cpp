// server.cpp -- scs_server: the reference's server surface on the GB300
// engine.
//
// CLI (main.cu:476-502, same 12 positional arguments):
//   scs_server <graph> <partitionSize> <bufferSize> <copyLimit> <readLimit>
//              <limitQueries> <factor> <red1> <red2> <red3> <prun1> <prun2>
// Queries arrive on the System V message queue of the reference
// (ipc/msgtool.h: key ftok("/tmp", 'g'), mtype 1, text of at most 80 bytes)
// as "<l> <h> <qid> <heuristic_flag> <limit_dominating_set>"; "server_exit"
// ends the server once every admitted query has finished (main.cu:96-99,
// 465-466).  Results go to results/results_<graph file name> with the
// reference's header and rows (main.cu:124-128, 328-333, 348-352, 451-454,
// 469-472).  partitionSize, bufferSize, copyLimit, readLimit and factor are
// validated and reported but the engine sizes its task store from device
// memory.  The listener blocks in msgrcv instead of polling.
//
// SCS_IPC_PROJ (environment) overrides the ftok project character (tests).
// SCS_COMMUNITIES (environment, any non-empty value) also writes each answer
// community to results/communities_<graph file name>, one row per query:
// "QID|N1|N2|Degree|Status|v1 v2 ..." (global vertex ids, status as in
// include/scs.h); scs_verify checks that file against the graph.  The
// reference computes these communities but never outputs them.
#include <sys/ipc.h>
#include <sys/msg.h>
#include <sys/stat.h>

#include <algorithm>
#include <atomic>
#include <cctype>
#include <cerrno>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <fstream>
#include <iostream>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/scs.h"
#include "server_format.h"

namespace {

struct MsgBuf {
  long mtype;
  char mtext[SCS_MSG_MAX];
};

std::mutex g_mu;
std::condition_variable g_cv;
std::deque<std::string> g_inbox;
bool g_exit_seen = false;

void listener(int qid) {
  MsgBuf m;
  for (;;) {
    ssize_t r = msgrcv(qid, &m, SCS_MSG_MAX, 1, 0);  // blocking
    if (r < 0) {
      if (errno == EINTR) continue;
      if (errno != EIDRM && errno != EINVAL) perror("scs_server: msgrcv");
      std::lock_guard<std::mutex> lk(g_mu);
      g_exit_seen = true;
      g_cv.notify_all();
      return;
    }
    std::string text(m.mtext, strnlen(m.mtext, (size_t)r));
    bool ex = scs_is_server_exit(text);
    {
      std::lock_guard<std::mutex> lk(g_mu);
      g_inbox.push_back(text);
      if (ex) g_exit_seen = true;
    }
    g_cv.notify_all();
    if (ex) return;
  }
}

bool file_exists(const std::string &p) {
  struct stat st;
  return stat(p.c_str(), &st) == 0;
}

void append_line(const std::string &path, const std::string &line) {
  std::ofstream f(path, std::ios::app);
  if (!f) {
    std::cerr << "Unable to open the file." << std::endl;
    return;
  }
  f << line << std::endl;
}

}  // namespace

int main(int argc, const char *argv[]) {
  if (argc != 13) {
    std::cout << "Server wrong input parameters!" << std::endl;
    return 1;
  }
  const char *graph = argv[1];
  long partition_size = atol(argv[2]), buffer_size = atol(argv[3]);
  double copy_limit = atof(argv[4]);
  long read_limit = atol(argv[5]), limit_queries = atol(argv[6]), factor = atol(argv[7]);
  int red1 = atoi(argv[8]), red2 = atoi(argv[9]), red3 = atoi(argv[10]);
  int prun1 = atoi(argv[11]), prun2 = atoi(argv[12]);
  if (limit_queries <= 0 || factor <= 0 || partition_size <= 0 || buffer_size <= 0) {
    std::cout << "Server wrong input parameters!" << std::endl;
    return 1;
  }
  std::string gp = graph;
  size_t pos = gp.find_last_of("/\\");
  std::string fname = "results/results_" + (pos == std::string::npos ? gp : gp.substr(pos + 1));
  mkdir("results", 0775);
  if (!file_exists(fname)) append_line(fname, "N1|N2|QID|Time|Degree|Overtime|Heu|TotalTime");
  const char *want_h = getenv("SCS_COMMUNITIES");
  const bool write_h = want_h && *want_h;
  const std::string hname =
      "results/communities_" + (pos == std::string::npos ? gp : gp.substr(pos + 1));
  if (write_h && !file_exists(hname)) append_line(hname, "QID|N1|N2|Degree|Status|Community");

  scs_config cfg{};
  cfg.limit_queries = (uint32_t)limit_queries;
  cfg.rules_set = 1;
  cfg.red1 = red1;
  cfg.red2 = red2;
  cfg.red3 = red3;
  cfg.prun1 = prun1;
  cfg.prun2 = prun2;
  cfg.slice_us = 5000;
  if (const char *b = getenv("SCS_NODE_BUDGET")) cfg.node_budget = strtoull(b, nullptr, 10);
  scs_engine *E = nullptr;
  int rc = scs_create(&E, graph, &cfg);
  if (rc) {
    std::cerr << "scs_server: " << scs_last_error(nullptr) << std::endl;
    return 2;
  }
  uint32_t n = 0, dmax = 0;
  uint64_t nnz = 0;
  scs_graph_info(E, &n, &nnz, &dmax);
  std::cout << "n=" << n << ",m=" << nnz / 2 << ",dMAX=" << dmax << std::endl;
  std::cout << "task store sized from device memory (partitionSize=" << partition_size
            << " bufferSize=" << buffer_size << " copyLimit=" << copy_limit
            << " readLimit=" << read_limit << " factor=" << factor << " accepted)" << std::endl;

  const char *proj = getenv("SCS_IPC_PROJ");
  key_t key = ftok(SCS_MSG_DIR, proj && *proj ? proj[0] : 'g');
  int qid = msgget(key, IPC_CREAT | 0660);
  if (qid < 0) {
    perror("scs_server: msgget");
    scs_destroy(E);
    return 3;
  }
  std::thread lt(listener, qid);
  auto t_start = std::chrono::steady_clock::now();
  std::unordered_map<uint64_t, int> qid_of_ticket;
  uint64_t outstanding = 0;
  uint64_t next_query_id = 0;
  std::vector<scs_result> res(256);
  const uint32_t h_stride = 512;  // queries need h < 510
  std::vector<uint32_t> hbuf(write_h ? res.size() * h_stride : 0);
  bool quit = false;
  for (;;) {
    // take messages
    std::vector<std::string> batch;
    {
      std::unique_lock<std::mutex> lk(g_mu);
      if (outstanding == 0 && g_inbox.empty() && !quit)
        g_cv.wait_for(lk, std::chrono::milliseconds(50));
      while (!g_inbox.empty()) {
        batch.push_back(g_inbox.front());
        g_inbox.pop_front();
      }
    }
    for (auto &text : batch) {
      next_query_id++;
      if (scs_is_server_exit(text)) {
        quit = true;
        continue;
      }
      scs_query q{};
      if (!scs_parse_query(text, q)) {
        std::cout << "Client wrong input parameters! Query ID: " << next_query_id - 1
                  << ", Query String: " << text << std::endl;
        continue;
      }
      uint64_t t;
      if (scs_submit(E, &q, &t) == 0) {
        qid_of_ticket[t] = (int)q.q;
        outstanding++;
      }
    }
    if (outstanding) {
      int r = scs_step(E);
      if (r < 0) {
        std::cerr << "scs_server: " << scs_last_error(E) << std::endl;
        break;
      }
    }
    int k;
    while ((k = scs_poll(E, res.data(), (int)res.size(), write_h ? hbuf.data() : nullptr,
                         h_stride)) > 0) {
      for (int i = 0; i < k; i++) {
        const scs_result &r = res[i];
        if (r.status == SCS_BAD_QUERY) {
          std::cout << "Client wrong input parameters! Query ID: " << r.ticket << std::endl;
        } else {
          append_line(fname, scs_format_row(r));
          if (write_h) {
            std::string row = std::to_string(r.q) + "|" + std::to_string(r.l) + "|" +
                              std::to_string(r.h) + "|" + std::to_string(r.degree) + "|" +
                              std::to_string(r.status) + "|";
            for (uint32_t j = 0; j < std::min(r.h_size, h_stride); j++) {
              if (j) row += ' ';
              row += std::to_string(hbuf[(size_t)i * h_stride + j]);
            }
            append_line(hname, row);
          }
          std::cout << "Found Solution : " << "QID = " << r.q << ", N1 = " << r.l
                    << ", N2 = " << r.h << ", kl = " << r.degree << std::endl;
        }
        outstanding--;
      }
    }
    if (quit && outstanding == 0) break;
  }
  long long total_us = std::chrono::duration_cast<std::chrono::microseconds>(
                           std::chrono::steady_clock::now() - t_start)
                           .count();
  append_line(fname, "-1|-1|-1|-1|-1|-1|-1|" + scs_group_thousands(total_us));
  msgctl(qid, IPC_RMID, nullptr);  // the reference removes its queue on exit;
  lt.join();                       // this also wakes a listener still blocked
  scs_destroy(E);
  std::cout << "End" << std::endl;
  return 0;
}
