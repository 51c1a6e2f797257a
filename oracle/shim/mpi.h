/*
 * Single-rank loopback stand-in for <mpi.h>, used ONLY to compile the Gemini
 * reference toolkits (core/mpi.hpp, core/graph.hpp) on a host without MPI.
 * Test infrastructure: nothing in the product links against this file.
 *
 * Semantics: one process, rank 0 of size 1.  MPI_Send to rank 0 enqueues a
 * copy of the buffer; MPI_Probe / MPI_Recv dequeue in FIFO order per tag.
 * The reference's loaders send edge chunks to themselves even with one rank
 * (core/graph.hpp:569,592,597) from the main thread while a receiver thread
 * probes, so the queue is guarded by a mutex + condition variable.
 * Collectives reduce over one rank, i.e. they copy.
 */
#ifndef GG_SHIM_MPI_H
#define GG_SHIM_MPI_H

#include <stddef.h>
#include <stdint.h>
#include <string.h>
#include <sys/time.h>

#include <condition_variable>
#include <deque>
#include <mutex>
#include <vector>

typedef int MPI_Datatype;
typedef int MPI_Comm;
typedef int MPI_Op;

struct MPI_Status {
  int MPI_SOURCE;
  int MPI_TAG;
  int MPI_ERROR;
  long gg_bytes;
};

#define MPI_COMM_WORLD 0
#define MPI_ANY_SOURCE (-1)
#define MPI_ANY_TAG (-1)
#define MPI_SUCCESS 0
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_IN_PLACE ((void *)1)

#define MPI_THREAD_SINGLE 0
#define MPI_THREAD_FUNNELED 1
#define MPI_THREAD_SERIALIZED 2
#define MPI_THREAD_MULTIPLE 3

#define MPI_CHAR 1
#define MPI_UNSIGNED_CHAR 2
#define MPI_INT 3
#define MPI_UNSIGNED 4
#define MPI_LONG 5
#define MPI_UNSIGNED_LONG 6
#define MPI_FLOAT 7
#define MPI_DOUBLE 8

#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3

static inline size_t gg_shim_type_size(MPI_Datatype t) {
  switch (t) {
    case MPI_CHAR: case MPI_UNSIGNED_CHAR: return 1;
    case MPI_INT: case MPI_UNSIGNED: case MPI_FLOAT: return 4;
    case MPI_LONG: case MPI_UNSIGNED_LONG: case MPI_DOUBLE: return 8;
    default: return 1;
  }
}

struct GgShimMessage {
  int tag;
  std::vector<char> bytes;
};

struct GgShimQueue {
  std::mutex mu;
  std::condition_variable cv;
  std::deque<GgShimMessage> q;
};

static inline GgShimQueue &gg_shim_queue() {
  static GgShimQueue queue;
  return queue;
}

static inline int MPI_Init_thread(int *, char ***, int, int *provided) {
  if (provided) *provided = MPI_THREAD_MULTIPLE;
  return MPI_SUCCESS;
}
static inline int MPI_Finalize() { return MPI_SUCCESS; }
static inline int MPI_Comm_rank(MPI_Comm, int *rank) { *rank = 0; return MPI_SUCCESS; }
static inline int MPI_Comm_size(MPI_Comm, int *size) { *size = 1; return MPI_SUCCESS; }
static inline int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }
static inline double MPI_Wtime() {
  struct timeval tv;
  gettimeofday(&tv, NULL);
  return tv.tv_sec + tv.tv_usec / 1e6;
}

static inline int MPI_Allreduce(const void *sendbuf, void *recvbuf, int count,
                                MPI_Datatype type, MPI_Op, MPI_Comm) {
  if (sendbuf != MPI_IN_PLACE && sendbuf != recvbuf) {
    memcpy(recvbuf, sendbuf, (size_t)count * gg_shim_type_size(type));
  }
  return MPI_SUCCESS;
}

static inline int MPI_Send(const void *buf, int count, MPI_Datatype type, int,
                           int tag, MPI_Comm) {
  GgShimQueue &sq = gg_shim_queue();
  GgShimMessage m;
  m.tag = tag;
  size_t n = (size_t)count * gg_shim_type_size(type);
  m.bytes.assign((const char *)buf, (const char *)buf + n);
  {
    std::lock_guard<std::mutex> lk(sq.mu);
    sq.q.push_back(std::move(m));
  }
  sq.cv.notify_all();
  return MPI_SUCCESS;
}

static inline int MPI_Probe(int, int tag, MPI_Comm, MPI_Status *status) {
  GgShimQueue &sq = gg_shim_queue();
  std::unique_lock<std::mutex> lk(sq.mu);
  for (;;) {
    for (auto &m : sq.q) {
      if (tag == MPI_ANY_TAG || m.tag == tag) {
        if (status) {
          status->MPI_SOURCE = 0;
          status->MPI_TAG = m.tag;
          status->MPI_ERROR = 0;
          status->gg_bytes = (long)m.bytes.size();
        }
        return MPI_SUCCESS;
      }
    }
    sq.cv.wait(lk);
  }
}

static inline int MPI_Get_count(const MPI_Status *status, MPI_Datatype type, int *count) {
  *count = (int)(status->gg_bytes / (long)gg_shim_type_size(type));
  return MPI_SUCCESS;
}

static inline int MPI_Recv(void *buf, int count, MPI_Datatype type, int, int tag,
                           MPI_Comm, MPI_Status *status) {
  GgShimQueue &sq = gg_shim_queue();
  std::unique_lock<std::mutex> lk(sq.mu);
  for (;;) {
    for (auto it = sq.q.begin(); it != sq.q.end(); ++it) {
      if (tag == MPI_ANY_TAG || it->tag == tag) {
        size_t cap = (size_t)count * gg_shim_type_size(type);
        size_t n = it->bytes.size() < cap ? it->bytes.size() : cap;
        memcpy(buf, it->bytes.data(), n);
        if (status) {
          status->MPI_SOURCE = 0;
          status->MPI_TAG = it->tag;
          status->MPI_ERROR = 0;
          status->gg_bytes = (long)n;
        }
        sq.q.erase(it);
        return MPI_SUCCESS;
      }
    }
    sq.cv.wait(lk);
  }
}

#endif
