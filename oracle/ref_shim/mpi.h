/*
 * mpi.h -- one-rank stand-in for the MPI calls of ptersnow/mestrado.
 *
 * TEST INFRASTRUCTURE ONLY.  It lets the reference's own SpeciesBlock.cpp
 * (the neighbor-joining code that serves as the NJ oracle) compile and run in
 * a single process.  With one rank every collective is a copy and every
 * point-to-point message is a self-send: a posted receive is matched by tag
 * when the send arrives (readFasta posts its Irecv before rank 0 sends to
 * itself, buildBins posts all Irecvs before the Isends), otherwise the message
 * waits in a queue for the receive.
 *
 * Covers exactly the calls listed in the reference's call sites:
 * wnj.cpp:25-52 and SpeciesBlock.cpp:277-1577.
 */
#ifndef NWG_ORACLE_MPI_SHIM_H
#define NWG_ORACLE_MPI_SHIM_H

#include <cstring>
#include <cstdlib>
#include <vector>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Errhandler;
typedef int MPI_Request;

struct MPI_Status {
  int MPI_SOURCE;
  int MPI_TAG;
  int MPI_ERROR;
};

typedef void(MPI_User_function)(void*, void*, int*, MPI_Datatype*);
typedef void(MPI_Comm_errhandler_function)(MPI_Comm*, int*, ...);

#define MPI_COMM_WORLD 0
#define MPI_SUCCESS 0
#define MPI_ERR_OTHER 15
#define MPI_REQUEST_NULL (-1)

/* Datatype handles carry their byte size (user types are registered). */
#define MPI_CHAR 1
#define MPI_BYTE 2
#define MPI_INT 3
#define MPI_LONG 4
#define MPI_FLOAT 5
#define MPI_DOUBLE 6
#define MPI_SUM 1
#define MPI_MAX 2

namespace nwg_mpi_shim {

struct Pending {
  int req;
  void* buf;
  int bytes;
  int tag;
  bool done;
  int got_tag;
};

struct Queued {
  std::vector<char> data;
  int tag;
};

struct State {
  std::vector<Pending> recvs;
  std::vector<Queued> queue;
  std::vector<int> user_type_bytes;
  int next_req = 0;
};

inline State& st() {
  static State s;
  return s;
}

inline int type_bytes(MPI_Datatype t) {
  switch (t) {
    case MPI_CHAR: case MPI_BYTE: return 1;
    case MPI_INT: return (int)sizeof(int);
    case MPI_LONG: return (int)sizeof(long);
    case MPI_FLOAT: return (int)sizeof(float);
    case MPI_DOUBLE: return (int)sizeof(double);
    default: break;
  }
  int k = t - 100;
  if (k >= 0 && k < (int)st().user_type_bytes.size()) return st().user_type_bytes[k];
  std::abort();
}

inline Pending* find_req(int r) {
  for (auto& p : st().recvs)
    if (p.req == r) return &p;
  return nullptr;
}

inline void deliver(const void* buf, int bytes, int tag) {
  for (auto& p : st().recvs) {
    if (!p.done && p.tag == tag) {
      std::memcpy(p.buf, buf, (size_t)(bytes < p.bytes ? bytes : p.bytes));
      p.done = true;
      p.got_tag = tag;
      return;
    }
  }
  Queued q;
  q.data.assign((const char*)buf, (const char*)buf + bytes);
  q.tag = tag;
  st().queue.push_back(q);
}

}  // namespace nwg_mpi_shim

inline int MPI_Init(int*, char***) { return MPI_SUCCESS; }
inline int MPI_Finalize() { return MPI_SUCCESS; }
inline int MPI_Comm_size(MPI_Comm, int* n) { *n = 1; return MPI_SUCCESS; }
inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return MPI_SUCCESS; }
inline int MPI_Abort(MPI_Comm, int code) { std::exit(code); }
inline int MPI_Comm_create_errhandler(MPI_Comm_errhandler_function*, MPI_Errhandler* e) { *e = 1; return MPI_SUCCESS; }
inline int MPI_Comm_set_errhandler(MPI_Comm, MPI_Errhandler) { return MPI_SUCCESS; }
inline int MPI_Errhandler_free(MPI_Errhandler*) { return MPI_SUCCESS; }

inline int MPI_Type_contiguous(int count, MPI_Datatype old, MPI_Datatype* out) {
  nwg_mpi_shim::st().user_type_bytes.push_back(count * nwg_mpi_shim::type_bytes(old));
  *out = 100 + (int)nwg_mpi_shim::st().user_type_bytes.size() - 1;
  return MPI_SUCCESS;
}
inline int MPI_Type_commit(MPI_Datatype*) { return MPI_SUCCESS; }
inline int MPI_Type_free(MPI_Datatype*) { return MPI_SUCCESS; }
inline int MPI_Op_create(MPI_User_function*, int, MPI_Op* op) { *op = 3; return MPI_SUCCESS; }
inline int MPI_Op_free(MPI_Op*) { return MPI_SUCCESS; }

/* One rank: the root's buffer already holds the data. */
inline int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm) { return MPI_SUCCESS; }

inline int MPI_Allreduce(const void* in, void* out, int count, MPI_Datatype t, MPI_Op, MPI_Comm) {
  std::memmove(out, in, (size_t)count * nwg_mpi_shim::type_bytes(t));
  return MPI_SUCCESS;
}

inline int MPI_Allgather(const void* in, int scount, MPI_Datatype st_, void* out, int, MPI_Datatype, MPI_Comm) {
  std::memmove(out, in, (size_t)scount * nwg_mpi_shim::type_bytes(st_));
  return MPI_SUCCESS;
}

inline int MPI_Alltoallv(const void* sbuf, const int* scnt, const int* sdisp, MPI_Datatype st_,
                         void* rbuf, const int*, const int* rdisp, MPI_Datatype, MPI_Comm) {
  int b = nwg_mpi_shim::type_bytes(st_);
  std::memmove((char*)rbuf + (size_t)rdisp[0] * b, (const char*)sbuf + (size_t)sdisp[0] * b,
               (size_t)scnt[0] * b);
  return MPI_SUCCESS;
}

inline int MPI_Irecv(void* buf, int count, MPI_Datatype t, int, int tag, MPI_Comm, MPI_Request* req) {
  using namespace nwg_mpi_shim;
  int bytes = count * type_bytes(t);
  int r = st().next_req++;
  Pending p{r, buf, bytes, tag, false, tag};
  auto& q = st().queue;
  for (size_t k = 0; k < q.size(); ++k) {
    if (q[k].tag == tag) {
      std::memcpy(buf, q[k].data.data(), (size_t)(bytes < (int)q[k].data.size() ? bytes : (int)q[k].data.size()));
      p.done = true;
      q.erase(q.begin() + (long)k);
      break;
    }
  }
  st().recvs.push_back(p);
  *req = r;
  return MPI_SUCCESS;
}

inline int MPI_Recv(void* buf, int count, MPI_Datatype t, int src, int tag, MPI_Comm c, MPI_Status* s) {
  MPI_Request r;
  MPI_Irecv(buf, count, t, src, tag, c, &r);
  nwg_mpi_shim::Pending* p = nwg_mpi_shim::find_req(r);
  if (!p || !p->done) std::abort();   /* nothing can arrive later with one rank */
  if (s) { s->MPI_TAG = p->got_tag; s->MPI_SOURCE = 0; s->MPI_ERROR = 0; }
  return MPI_SUCCESS;
}

inline int MPI_Send(const void* buf, int count, MPI_Datatype t, int, int tag, MPI_Comm) {
  nwg_mpi_shim::deliver(buf, count * nwg_mpi_shim::type_bytes(t), tag);
  return MPI_SUCCESS;
}

inline int MPI_Isend(const void* buf, int count, MPI_Datatype t, int dst, int tag, MPI_Comm c, MPI_Request* req) {
  MPI_Send(buf, count, t, dst, tag, c);
  *req = MPI_REQUEST_NULL;
  return MPI_SUCCESS;
}

inline int MPI_Wait(MPI_Request* req, MPI_Status* s) {
  if (*req == MPI_REQUEST_NULL) return MPI_SUCCESS;
  nwg_mpi_shim::Pending* p = nwg_mpi_shim::find_req(*req);
  if (!p || !p->done) std::abort();
  if (s) { s->MPI_TAG = p->got_tag; s->MPI_SOURCE = 0; s->MPI_ERROR = 0; }
  *req = MPI_REQUEST_NULL;
  return MPI_SUCCESS;
}

inline int MPI_Waitany(int count, MPI_Request* reqs, int* index, MPI_Status* s) {
  for (int k = 0; k < count; ++k) {
    if (reqs[k] == MPI_REQUEST_NULL) continue;
    nwg_mpi_shim::Pending* p = nwg_mpi_shim::find_req(reqs[k]);
    if (p && p->done) {
      *index = k;
      if (s) { s->MPI_TAG = p->got_tag; s->MPI_SOURCE = 0; s->MPI_ERROR = 0; }
      reqs[k] = MPI_REQUEST_NULL;
      return MPI_SUCCESS;
    }
  }
  std::abort();
}

inline int MPI_Waitall(int count, MPI_Request* reqs, MPI_Status*) {
  for (int k = 0; k < count; ++k) reqs[k] = MPI_REQUEST_NULL;
  return MPI_SUCCESS;
}

#endif
