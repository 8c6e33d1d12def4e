// client.cpp -- scs_client: batch query sender for scs_server (and for the
// reference's server: same queue protocol, ipc/msgtool.h:127-168).
//
//   scs_client <query file>
// Sends each line ("<l> <h> <qid> <heuristic_flag> <limit_dominating_set>")
// as one mtype-1 message, retrying while the queue is full; a line
// "server_exit" stops reading and is sent last (the batch-client behaviour
// of the reference, client/batchClient.cpp).  SCS_IPC_PROJ overrides the
// ftok project character.
#include <sys/ipc.h>
#include <sys/msg.h>
#include <unistd.h>

#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "server_format.h"

namespace {
struct MsgBuf {
  long mtype;
  char mtext[SCS_MSG_MAX];
};

bool send(int qid, const std::string &text) {
  MsgBuf m;
  m.mtype = 1;
  size_t len = std::min(text.size(), (size_t)SCS_MSG_MAX - 1);
  memcpy(m.mtext, text.data(), len);
  m.mtext[len] = 0;
  for (int tries = 0; tries < 10000000; tries++) {
    if (msgsnd(qid, &m, len + 1, IPC_NOWAIT) == 0) return true;
    if (errno != EAGAIN) {
      perror("scs_client: msgsnd");
      return false;
    }
    usleep(1);
  }
  return false;
}
}  // namespace

int main(int argc, char *argv[]) {
  if (argc != 2) {
    std::cerr << "usage: scs_client <query file>" << std::endl;
    return 1;
  }
  std::ifstream fin(argv[1]);
  if (!fin) {
    std::cerr << "scs_client: cannot open " << argv[1] << std::endl;
    return 1;
  }
  std::vector<std::string> lines;
  bool exit_after = false;
  std::string line;
  while (std::getline(fin, line)) {
    if (!line.empty() && line.back() == '\r') line.pop_back();
    if (line == "server_exit") {
      exit_after = true;
      break;
    }
    lines.push_back(line);
  }
  const char *proj = getenv("SCS_IPC_PROJ");
  key_t key = ftok(SCS_MSG_DIR, proj && *proj ? proj[0] : 'g');
  int qid = -1;
  for (int i = 0; i < 3000 && qid < 0; i++) {  // wait up to 30 s for the server
    qid = msgget(key, 0);
    if (qid < 0) usleep(10000);
  }
  if (qid < 0) {
    perror("scs_client: msgget");
    return 2;
  }
  for (auto &l : lines)
    if (!send(qid, l)) return 3;
  if (exit_after && !send(qid, "server_exit")) return 3;
  return 0;
}
