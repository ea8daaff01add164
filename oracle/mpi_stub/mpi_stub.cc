// Thread-per-rank MPI stand-in (see mpi.h).  Test infrastructure only.
#include "mpi.h"

#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

namespace {

struct Message {
  int source, tag;
  std::vector<char> data;
};

struct Mailbox {
  std::mutex mu;
  std::condition_variable cv;
  std::deque<Message> queue;
};

int g_size = 1;
std::vector<Mailbox> *g_boxes = nullptr;
thread_local int t_rank = 0;

size_t type_size(MPI_Datatype t) { return t == MPI_DOUBLE ? sizeof(double) : sizeof(int); }

}  // namespace

struct mpistub_request {
  bool recv;
  void *buf;
  size_t bytes;
  int source, tag;
};

extern "C" {

int MPI_Comm_rank(MPI_Comm, int *rank)
{
  *rank = t_rank;
  return MPI_SUCCESS;
}

int MPI_Comm_size(MPI_Comm, int *size)
{
  *size = g_size;
  return MPI_SUCCESS;
}

int MPI_Irecv(void *buf, int count, MPI_Datatype type, int source, int tag, MPI_Comm,
              MPI_Request *req)
{
  if (source == MPI_PROC_NULL) {
    *req = nullptr;
    return MPI_SUCCESS;
  }
  *req = new mpistub_request{true, buf, count * type_size(type), source, tag};
  return MPI_SUCCESS;
}

int MPI_Isend(const void *buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm,
              MPI_Request *req)
{
  *req = nullptr;
  if (dest == MPI_PROC_NULL) return MPI_SUCCESS;
  Message m;
  m.source = t_rank;
  m.tag = tag;
  m.data.resize(count * type_size(type));
  std::memcpy(m.data.data(), buf, m.data.size());
  Mailbox &box = (*g_boxes)[dest];
  {
    std::lock_guard<std::mutex> lock(box.mu);
    box.queue.push_back(std::move(m));
  }
  box.cv.notify_all();
  return MPI_SUCCESS;
}

int MPI_Waitall(int count, MPI_Request reqs[], MPI_Status *)
{
  Mailbox &box = (*g_boxes)[t_rank];
  for (int k = 0; k < count; k++) {
    mpistub_request *r = reqs[k];
    reqs[k] = nullptr;
    if (!r) continue;
    if (r->recv) {
      std::unique_lock<std::mutex> lock(box.mu);
      for (;;) {
        auto it = box.queue.begin();
        for (; it != box.queue.end(); ++it)
          if (it->source == r->source && it->tag == r->tag) break;
        if (it != box.queue.end()) {
          std::memcpy(r->buf, it->data.data(), std::min(r->bytes, it->data.size()));
          box.queue.erase(it);
          break;
        }
        box.cv.wait(lock);
      }
    }
    delete r;
  }
  return MPI_SUCCESS;
}

void mpistub_run(int size, void (*fn)(int, void *), void *arg)
{
  std::vector<Mailbox> boxes(size);
  g_boxes = &boxes;
  g_size = size;
  std::vector<std::thread> threads;
  for (int r = 0; r < size; r++)
    threads.emplace_back([=] {
      t_rank = r;
      fn(r, arg);
    });
  for (auto &t : threads) t.join();
  g_boxes = nullptr;
  g_size = 1;
}

}  // extern "C"
