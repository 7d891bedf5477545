// Implementation of the single-rank MPI stub (test infrastructure).
#include "mpi.h"

#include <chrono>
#include <condition_variable>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <vector>

namespace {
struct Msg {
  int comm, tag;
  std::vector<char> data;
};
struct PendingRecv {
  void* buf;
  size_t bytes;
  int src, tag, comm;
  bool done;
  MPI_Status st;
};
std::mutex mu;
std::condition_variable cv;
std::deque<Msg> box;
std::map<int, PendingRecv> pending;
int next_req = 1;
int next_comm = 2;

bool matches(const Msg& m, int src, int tag, int comm) {
  (void)src;  // the only rank is 0
  return m.comm == comm && (tag == MPI_ANY_TAG || tag == m.tag);
}
std::deque<Msg>::iterator find_msg(int src, int tag, int comm) {
  for (auto it = box.begin(); it != box.end(); ++it)
    if (matches(*it, src, tag, comm)) return it;
  return box.end();
}
void fill(MPI_Status* st, const Msg& m) {
  if (!st) return;
  st->MPI_SOURCE = 0;
  st->MPI_TAG = m.tag;
  st->MPI_ERROR = 0;
  st->sg_bytes = (int)m.data.size();
}
// completes pending receives that now have a matching message (lock held)
void progress() {
  for (auto& kv : pending) {
    PendingRecv& p = kv.second;
    if (p.done) continue;
    auto it = find_msg(p.src, p.tag, p.comm);
    if (it == box.end()) continue;
    const size_t nb = std::min(p.bytes, it->data.size());
    if (nb) std::memcpy(p.buf, it->data.data(), nb);
    fill(&p.st, *it);
    p.done = true;
    box.erase(it);
  }
}
}  // namespace

extern "C" {
int MPI_Init(int*, char***) { return 0; }
int MPI_Init_thread(int*, char***, int, int* provided) {
  if (provided) *provided = MPI_THREAD_MULTIPLE;
  return 0;
}
int MPI_Initialized(int* f) { *f = 1; return 0; }
int MPI_Finalize(void) { return 0; }
int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return 0; }
int MPI_Comm_size(MPI_Comm, int* s) { *s = 1; return 0; }
int MPI_Comm_dup(MPI_Comm, MPI_Comm* out) {
  std::lock_guard<std::mutex> g(mu);
  *out = next_comm++;
  return 0;
}
int MPI_Comm_free(MPI_Comm* c) { *c = MPI_COMM_NULL; return 0; }
int MPI_Comm_split(MPI_Comm c, int, int, MPI_Comm* out) { return MPI_Comm_dup(c, out); }
int MPI_Barrier(MPI_Comm) { return 0; }
int MPI_Send(const void* buf, int count, MPI_Datatype t, int, int tag, MPI_Comm comm) {
  Msg m;
  m.comm = comm;
  m.tag = tag;
  const size_t nb = (size_t)count * (size_t)t;
  m.data.resize(nb);
  if (nb) std::memcpy(m.data.data(), buf, nb);
  {
    std::lock_guard<std::mutex> g(mu);
    box.push_back(std::move(m));
    progress();
  }
  cv.notify_all();
  return 0;
}
int MPI_Isend(const void* buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm comm,
              MPI_Request* req) {
  MPI_Send(buf, count, t, dest, tag, comm);
  if (req) *req = MPI_REQUEST_NULL;
  return 0;
}
int MPI_Recv(void* buf, int count, MPI_Datatype t, int src, int tag, MPI_Comm comm,
             MPI_Status* st) {
  std::unique_lock<std::mutex> g(mu);
  std::deque<Msg>::iterator it;
  cv.wait(g, [&] { return (it = find_msg(src, tag, comm)) != box.end(); });
  const size_t nb = std::min((size_t)count * (size_t)t, it->data.size());
  if (nb) std::memcpy(buf, it->data.data(), nb);
  fill(st, *it);
  box.erase(it);
  return 0;
}
int MPI_Irecv(void* buf, int count, MPI_Datatype t, int src, int tag, MPI_Comm comm,
              MPI_Request* req) {
  std::lock_guard<std::mutex> g(mu);
  const int id = next_req++;
  pending[id] = PendingRecv{buf, (size_t)count * (size_t)t, src, tag, comm, false, {}};
  progress();
  *req = id;
  return 0;
}
int MPI_Probe(int src, int tag, MPI_Comm comm, MPI_Status* st) {
  std::unique_lock<std::mutex> g(mu);
  std::deque<Msg>::iterator it;
  cv.wait(g, [&] { return (it = find_msg(src, tag, comm)) != box.end(); });
  fill(st, *it);
  return 0;
}
int MPI_Iprobe(int src, int tag, MPI_Comm comm, int* flag, MPI_Status* st) {
  std::lock_guard<std::mutex> g(mu);
  auto it = find_msg(src, tag, comm);
  *flag = it != box.end();
  if (*flag) fill(st, *it);
  return 0;
}
int MPI_Get_count(const MPI_Status* st, MPI_Datatype t, int* count) {
  *count = st->sg_bytes / (int)t;
  return 0;
}
int MPI_Test(MPI_Request* req, int* flag, MPI_Status* st) {
  if (*req == MPI_REQUEST_NULL) {
    *flag = 1;
    return 0;
  }
  std::lock_guard<std::mutex> g(mu);
  progress();
  auto it = pending.find(*req);
  *flag = (it == pending.end()) || it->second.done;
  if (*flag && it != pending.end()) {
    if (st) *st = it->second.st;
    pending.erase(it);
    *req = MPI_REQUEST_NULL;
  }
  return 0;
}
int MPI_Wait(MPI_Request* req, MPI_Status* st) {
  for (;;) {
    int flag = 0;
    MPI_Test(req, &flag, st);
    if (flag) return 0;
    std::unique_lock<std::mutex> g(mu);
    cv.wait_for(g, std::chrono::milliseconds(1));
  }
}
int MPI_Waitall(int n, MPI_Request* reqs, MPI_Status* sts) {
  for (int i = 0; i < n; ++i) MPI_Wait(&reqs[i], sts ? &sts[i] : nullptr);
  return 0;
}
int MPI_Waitany(int n, MPI_Request* reqs, int* index, MPI_Status* st) {
  for (;;) {
    for (int i = 0; i < n; ++i) {
      if (reqs[i] == MPI_REQUEST_NULL) continue;
      int flag = 0;
      MPI_Test(&reqs[i], &flag, st);
      if (flag) {
        *index = i;
        return 0;
      }
    }
    bool any = false;
    for (int i = 0; i < n; ++i) any |= reqs[i] != MPI_REQUEST_NULL;
    if (!any) {
      *index = -1;
      return 0;
    }
    std::unique_lock<std::mutex> g(mu);
    cv.wait_for(g, std::chrono::milliseconds(1));
  }
}
int MPI_Cancel(MPI_Request* req) {
  std::lock_guard<std::mutex> g(mu);
  auto it = pending.find(*req);
  if (it != pending.end()) it->second.done = true;
  return 0;
}
int MPI_Allreduce(const void* sb, void* rb, int count, MPI_Datatype t, MPI_Op, MPI_Comm) {
  if (sb != MPI_IN_PLACE && sb != rb) std::memcpy(rb, sb, (size_t)count * (size_t)t);
  return 0;
}
int MPI_Reduce(const void* sb, void* rb, int count, MPI_Datatype t, MPI_Op, int, MPI_Comm) {
  if (sb != MPI_IN_PLACE && sb != rb && rb) std::memcpy(rb, sb, (size_t)count * (size_t)t);
  return 0;
}
int MPI_Allgather(const void* sb, int sc, MPI_Datatype st, void* rb, int, MPI_Datatype, MPI_Comm) {
  if (sb != MPI_IN_PLACE) std::memcpy(rb, sb, (size_t)sc * (size_t)st);
  return 0;
}
int MPI_Allgatherv(const void* sb, int sc, MPI_Datatype st, void* rb, const int*,
                   const int* displs, MPI_Datatype rt, MPI_Comm) {
  if (sb != MPI_IN_PLACE)
    std::memcpy((char*)rb + (size_t)displs[0] * (size_t)rt, sb, (size_t)sc * (size_t)st);
  return 0;
}
int MPI_Gather(const void* sb, int sc, MPI_Datatype st, void* rb, int, MPI_Datatype, int,
               MPI_Comm) {
  if (sb != MPI_IN_PLACE && rb) std::memcpy(rb, sb, (size_t)sc * (size_t)st);
  return 0;
}
int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm) { return 0; }
int MPI_Get_processor_name(char* name, int* len) {
  std::strcpy(name, "localhost");
  *len = 9;
  return 0;
}
double MPI_Wtime(void) {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}
int MPI_Abort(MPI_Comm, int code) { std::exit(code); }
}
