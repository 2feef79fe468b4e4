/* Stand-in for the MPI library, written for this project so that the reference's
 * unmodified headers compile and run without MPI.
 *
 * One rank (the default): rank 0 of 1; collectives are copies, splits the identity.
 * QSF_SHIM_NP=<p> (p <= 16): MPI_Init forks p - 1 more processes, which run the rest
 * of the program as ranks 1 .. p-1.  Before the fork it maps one shared anonymous
 * region that holds the synchronisation state, the exchange buffers of the
 * collectives and one allocation slice per rank (fftw_malloc draws from it, see
 * qsf_shim_arena.h), so every rank reads every other rank's wavefunction at the same
 * address: MPI_Get on a window is a copy, and MPI_Win_fence a barrier of the
 * window's communicator.  Communicators are member lists (ranks of MPI_COMM_WORLD);
 * their collectives synchronise through a slot chosen by the member set.  What the
 * reference calls for its multi-region grids is covered: Comm_split, Intercomm_create
 * / _merge, Win_create / _fence / Get, Barrier, Allreduce, Reduce, Bcast.  Point to
 * point calls, and gathers over more than one rank, abort.  The parent waits for the
 * other ranks at exit.  Every wait gives up (and aborts) after QSF_SHIM_TIMEOUT
 * seconds (default 300).
 *
 * Test infrastructure for the oracle harness only. */
#pragma once
#include <sched.h>
#include <sys/mman.h>
#include <sys/wait.h>
#include <time.h>
#include <unistd.h>

#include <algorithm>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <utility>
#include <vector>

#include "qsf_shim_arena.h"

constexpr int kShimMaxRanks = 16;

struct qsf_shim_comm {
  int size = 1, rank = 0;
  int pids[kShimMaxRanks] = {0};  // world rank of each member, in rank order
  bool inter = false;
  int rsize = 0;
  int rpids[kShimMaxRanks] = {0};  // inter-communicators: the remote group
};
struct qsf_shim_win {
  qsf_shim_comm* comm;
  int entry;
};
typedef qsf_shim_comm* MPI_Comm;
typedef int MPI_Group;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Info;
typedef qsf_shim_win* MPI_Win;
typedef long long MPI_Offset;
typedef long long MPI_Aint;
typedef FILE* MPI_File;
struct MPI_Status { int MPI_SOURCE, MPI_TAG, MPI_ERROR; };

#define MPI_INFO_NULL 0
#define MPI_SUM 1
#define MPI_IN_PLACE ((void*)1)
#define MPI_BOTTOM ((void*)0)
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_MAX_PROCESSOR_NAME 64
#define MPI_MAX_LIBRARY_VERSION_STRING 64
#define MPI_MODE_RDONLY 1
#define MPI_MODE_WRONLY 2
#define MPI_MODE_CREATE 4
#define MPI_MODE_NOSUCCEED 8
#define MPI_MODE_NOPRECEDE 16
#define MPI_MODE_NOSTORE 32
#define MPI_MODE_NOPUT 64
#define MPI_SEEK_SET SEEK_SET

enum : int {
  MPI_INT = 4, MPI_DOUBLE = 8, MPI_CXX_DOUBLE_COMPLEX = 16, MPI_CXX_BOOL = 1, MPI_UNSIGNED_CHAR = 1,
  MPI_OFFSET = 8, MPI_BYTE = 1, MPI_INT64_T = 8
};

static inline size_t qsf_shim_type_size(MPI_Datatype t) { return (size_t)t; }
[[noreturn]] static inline void qsf_shim_fatal(const char* what) {
  fprintf(stderr, "MPI stand-in: %s\n", what);
  fflush(stderr);
  abort();
}

// ---------------------------------------------------------------- shared state
constexpr int kShimSlots = 64;
constexpr size_t kShimSlotBytes = 1 << 16;  // exchange buffer per member of a slot
constexpr int kShimWins = 64;
constexpr int kShimTags = 16;

struct qsf_shim_slot {
  unsigned mask;  // member set (bit = world rank); 0 = free
  int count, gen;
  alignas(64) unsigned char buf[kShimMaxRanks][kShimSlotBytes];
};
struct qsf_shim_wentry {
  unsigned mask;
  int seq;
  void* base[kShimMaxRanks];
  long long unit[kShimMaxRanks];
};
struct qsf_shim_shared {
  int np;
  int inter_ready[kShimMaxRanks][kShimTags];
  unsigned inter_mask[kShimMaxRanks][kShimTags];
  qsf_shim_wentry wins[kShimWins];
  qsf_shim_slot slots[kShimSlots];
};

inline qsf_shim_shared* qsf_shim_sh = nullptr;
inline int qsf_shim_pid = 0, qsf_shim_np = 1;
inline qsf_shim_comm qsf_shim_world_comm;
inline std::vector<pid_t> qsf_shim_children;
inline std::map<unsigned, int> qsf_shim_win_seq;  // windows created per member set (this rank)

static inline MPI_Comm qsf_shim_world() { return &qsf_shim_world_comm; }
#define MPI_COMM_WORLD (qsf_shim_world())

static inline double qsf_shim_timeout() {
  const char* t = getenv("QSF_SHIM_TIMEOUT");
  return t ? atof(t) : 300.0;
}
static inline double qsf_shim_now() {
  timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}
// waits until pred() holds, yielding; aborts after the timeout
template <class P>
static inline void qsf_shim_wait(P pred, const char* what) {
  const double t0 = qsf_shim_now(), lim = qsf_shim_timeout();
  for (long it = 0; !pred(); ++it) {
    sched_yield();
    if ((it & 1023) == 0 && qsf_shim_now() - t0 > lim) qsf_shim_fatal(what);
  }
}

static inline unsigned qsf_shim_mask(const qsf_shim_comm* c) {
  unsigned m = 0;
  for (int i = 0; i < c->size; ++i) m |= 1u << c->pids[i];
  return m;
}
static inline qsf_shim_slot* qsf_shim_slot_for(unsigned mask) {
  for (int i = 0; i < kShimSlots; ++i) {
    qsf_shim_slot* s = &qsf_shim_sh->slots[i];
    unsigned cur = __atomic_load_n(&s->mask, __ATOMIC_ACQUIRE);
    if (cur == mask) return s;
    if (cur == 0) {
      unsigned expected = 0;
      if (__atomic_compare_exchange_n(&s->mask, &expected, mask, false, __ATOMIC_ACQ_REL, __ATOMIC_ACQUIRE))
        return s;
      if (expected == mask) return s;
    }
  }
  qsf_shim_fatal("out of collective slots");
}
static inline void qsf_shim_barrier(qsf_shim_comm* c) {
  if (c->size <= 1) return;
  qsf_shim_slot* s = qsf_shim_slot_for(qsf_shim_mask(c));
  const int gen = __atomic_load_n(&s->gen, __ATOMIC_ACQUIRE);
  if (__atomic_add_fetch(&s->count, 1, __ATOMIC_ACQ_REL) == c->size) {
    __atomic_store_n(&s->count, 0, __ATOMIC_RELAXED);
    __atomic_add_fetch(&s->gen, 1, __ATOMIC_RELEASE);
  } else {
    qsf_shim_wait([&] { return __atomic_load_n(&s->gen, __ATOMIC_ACQUIRE) != gen; }, "barrier timed out");
  }
}
static inline qsf_shim_comm* qsf_shim_new_comm(const std::vector<int>& pids) {
  qsf_shim_comm* c = new qsf_shim_comm();
  c->size = (int)pids.size();
  c->rank = -1;
  for (int i = 0; i < c->size; ++i) {
    c->pids[i] = pids[(size_t)i];
    if (pids[(size_t)i] == qsf_shim_pid) c->rank = i;
  }
  return c;
}

static inline void qsf_shim_wait_children() {
  if (qsf_shim_pid != 0) return;
  fflush(nullptr);
  for (pid_t c : qsf_shim_children) {
    int st = 0;
    if (waitpid(c, &st, 0) < 0 || !WIFEXITED(st) || WEXITSTATUS(st) != 0) {
      fprintf(stderr, "MPI stand-in: rank process %d failed (status %d)\n", (int)c, st);
      _exit(3);
    }
  }
  qsf_shim_children.clear();
}

// ---------------------------------------------------------------- environment
static inline int MPI_Init(int*, char***) {
  const char* e = getenv("QSF_SHIM_NP");
  const int np = e ? atoi(e) : 1;
  if (np < 1 || np > kShimMaxRanks) qsf_shim_fatal("QSF_SHIM_NP out of range");
  qsf_shim_np = np;
  qsf_shim_world_comm = qsf_shim_comm();
  qsf_shim_world_comm.size = np;
  for (int i = 0; i < np; ++i) qsf_shim_world_comm.pids[i] = i;
  if (np == 1) return 0;
  const size_t slice = (size_t)1 << 30;  // allocation space per rank (reserved, not committed)
  const size_t bytes = sizeof(qsf_shim_shared) + slice * (size_t)np;
  void* mem = mmap(nullptr, bytes, PROT_READ | PROT_WRITE, MAP_SHARED | MAP_ANONYMOUS | MAP_NORESERVE, -1, 0);
  if (mem == MAP_FAILED) qsf_shim_fatal("mmap of the shared region failed");
  qsf_shim_sh = static_cast<qsf_shim_shared*>(mem);
  qsf_shim_sh->np = np;
  for (int i = 0; i < kShimWins; ++i) qsf_shim_sh->wins[i].seq = -1;
  char* arena = static_cast<char*>(mem) + ((sizeof(qsf_shim_shared) + 4095) & ~(size_t)4095);
  qsf_shim_arena_lo = arena;
  qsf_shim_arena_hi = static_cast<char*>(mem) + bytes;
  fflush(nullptr);
  int me = 0;
  for (int r = 1; r < np; ++r) {
    pid_t c = fork();
    if (c < 0) qsf_shim_fatal("fork failed");
    if (c == 0) {
      me = r;
      qsf_shim_children.clear();
      break;
    }
    qsf_shim_children.push_back(c);
  }
  qsf_shim_pid = me;
  qsf_shim_world_comm.rank = me;
  const size_t per = (size_t)(qsf_shim_arena_hi - arena) / (size_t)np & ~(size_t)4095;
  qsf_shim_arena_cur = arena + per * (size_t)me;
  qsf_shim_arena_end = qsf_shim_arena_cur + per;
  if (me == 0) atexit(qsf_shim_wait_children);
  return 0;
}
static inline int MPI_Finalize() {
  qsf_shim_barrier(MPI_COMM_WORLD);
  if (qsf_shim_pid != 0) {
    fflush(nullptr);
    _exit(0);
  }
  qsf_shim_wait_children();
  return 0;
}
static inline int MPI_Comm_rank(MPI_Comm c, int* r) { *r = c ? c->rank : 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm c, int* s) { *s = c ? c->size : 1; return 0; }
static inline int MPI_Comm_group(MPI_Comm, MPI_Group* g) { *g = 0; return 0; }
static inline int MPI_Comm_remote_size(MPI_Comm c, int* s) { *s = c && c->inter ? c->rsize : 0; return 0; }
static inline int MPI_Barrier(MPI_Comm c) { qsf_shim_barrier(c); return 0; }
static inline int MPI_Get_processor_name(char* n, int* l) { strcpy(n, "oracle"); *l = 6; return 0; }
static inline int MPI_Get_version(int* v, int* s) { *v = 3; *s = 1; return 0; }
static inline int MPI_Get_library_version(char* v, int* l) { strcpy(v, "process stand-in"); *l = 16; return 0; }

// new communicators of the members with the same colour, ordered by (key, old rank)
static inline int MPI_Comm_split(MPI_Comm c, int color, int key, MPI_Comm* out) {
  if (c->size <= 1) {
    *out = qsf_shim_new_comm(std::vector<int>(c->pids, c->pids + c->size));
    return 0;
  }
  qsf_shim_slot* s = qsf_shim_slot_for(qsf_shim_mask(c));
  int mine[2] = {color, key};
  memcpy(s->buf[c->rank], mine, sizeof(mine));
  qsf_shim_barrier(c);
  std::vector<std::pair<std::pair<int, int>, int>> sel;
  for (int r = 0; r < c->size; ++r) {
    int v[2];
    memcpy(v, s->buf[r], sizeof(v));
    if (v[0] == color) sel.push_back({{v[1], r}, c->pids[r]});
  }
  qsf_shim_barrier(c);
  std::sort(sel.begin(), sel.end());
  std::vector<int> pids;
  for (auto& x : sel) pids.push_back(x.second);
  *out = qsf_shim_new_comm(pids);
  return 0;
}
// the local group is `local`; the remote group is the local communicator its leader
// (world rank remote_leader) passed with the same tag
static inline int MPI_Intercomm_create(MPI_Comm local, int, MPI_Comm, int remote_leader, int tag, MPI_Comm* out) {
  if (tag < 0 || tag >= kShimTags) qsf_shim_fatal("Intercomm_create tag out of range");
  __atomic_store_n(&qsf_shim_sh->inter_mask[qsf_shim_pid][tag], qsf_shim_mask(local), __ATOMIC_RELAXED);
  __atomic_store_n(&qsf_shim_sh->inter_ready[qsf_shim_pid][tag], 1, __ATOMIC_RELEASE);
  qsf_shim_wait([&] { return __atomic_load_n(&qsf_shim_sh->inter_ready[remote_leader][tag], __ATOMIC_ACQUIRE) != 0; },
                "Intercomm_create timed out");
  const unsigned rm = __atomic_load_n(&qsf_shim_sh->inter_mask[remote_leader][tag], __ATOMIC_RELAXED);
  qsf_shim_comm* c = qsf_shim_new_comm(std::vector<int>(local->pids, local->pids + local->size));
  c->inter = true;
  c->rsize = 0;
  for (int p = 0; p < kShimMaxRanks; ++p)
    if (rm & (1u << p)) c->rpids[c->rsize++] = p;
  *out = c;
  return 0;
}
// intra-communicator of both groups, the group that passed high = 0 first
static inline int MPI_Intercomm_merge(MPI_Comm inter, int high, MPI_Comm* out) {
  if (!inter || !inter->inter) qsf_shim_fatal("Intercomm_merge needs an inter-communicator");
  std::vector<int> loc(inter->pids, inter->pids + inter->size), rem(inter->rpids, inter->rpids + inter->rsize);
  std::vector<int> all = high ? rem : loc;
  const std::vector<int>& second = high ? loc : rem;
  all.insert(all.end(), second.begin(), second.end());
  *out = qsf_shim_new_comm(all);
  return 0;
}

// ---------------------------------------------------------------- collectives
static inline void qsf_shim_sum(void* r, const void* s, int n, MPI_Datatype t) {
  if (t == MPI_DOUBLE) {
    for (int i = 0; i < n; ++i) ((double*)r)[i] += ((const double*)s)[i];
  } else if (t == MPI_CXX_DOUBLE_COMPLEX) {
    for (int i = 0; i < 2 * n; ++i) ((double*)r)[i] += ((const double*)s)[i];
  } else if (t == MPI_INT) {
    for (int i = 0; i < n; ++i) ((int*)r)[i] += ((const int*)s)[i];
  } else {
    qsf_shim_fatal("reduction of this type is not available");
  }
}
// sum over the members in rank order into r on every member (root < 0) or on root
static inline void qsf_shim_reduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Comm c, int root) {
  const size_t bytes = (size_t)n * qsf_shim_type_size(t);
  const void* src = s == MPI_IN_PLACE ? r : s;
  if (c->size <= 1) {
    if (src != r) memcpy(r, src, bytes);
    return;
  }
  if (bytes > kShimSlotBytes) qsf_shim_fatal("reduction larger than the exchange buffer");
  qsf_shim_slot* sl = qsf_shim_slot_for(qsf_shim_mask(c));
  memcpy(sl->buf[c->rank], src, bytes);
  qsf_shim_barrier(c);
  if (root < 0 || c->rank == root) {
    std::vector<unsigned char> acc(bytes);
    memcpy(acc.data(), sl->buf[0], bytes);
    for (int k = 1; k < c->size; ++k) qsf_shim_sum(acc.data(), sl->buf[k], n, t);
    memcpy(r, acc.data(), bytes);
  }
  qsf_shim_barrier(c);
}
static inline int MPI_Allreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, MPI_Comm c) {
  qsf_shim_reduce(s, r, n, t, c, -1);
  return 0;
}
static inline int MPI_Reduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, int root, MPI_Comm c) {
  qsf_shim_reduce(s, r, n, t, c, root);
  return 0;
}
static inline int MPI_Bcast(void* b, int n, MPI_Datatype t, int root, MPI_Comm c) {
  if (c->size <= 1) return 0;
  const size_t bytes = (size_t)n * qsf_shim_type_size(t);
  if (bytes > kShimSlotBytes) qsf_shim_fatal("broadcast larger than the exchange buffer");
  qsf_shim_slot* sl = qsf_shim_slot_for(qsf_shim_mask(c));
  if (c->rank == root) memcpy(sl->buf[root], b, bytes);
  qsf_shim_barrier(c);
  if (c->rank != root) memcpy(b, sl->buf[root], bytes);
  qsf_shim_barrier(c);
  return 0;
}
static inline int MPI_Gather(const void* s, int n, MPI_Datatype t, void* r, int, MPI_Datatype, int, MPI_Comm c) {
  if (c->size > 1) qsf_shim_fatal("MPI_Gather over more than one rank is not available");
  if (s != MPI_IN_PLACE && s != r) memcpy(r, s, (size_t)n * qsf_shim_type_size(t));
  return 0;
}
static inline int MPI_Allgather(const void* s, int n, MPI_Datatype t, void* r, int, MPI_Datatype, MPI_Comm c) {
  if (c->size > 1) qsf_shim_fatal("MPI_Allgather over more than one rank is not available");
  if (s != MPI_IN_PLACE && s != r) memcpy(r, s, (size_t)n * qsf_shim_type_size(t));
  return 0;
}
static inline int MPI_Scatter(const void* s, int n, MPI_Datatype t, void* r, int, MPI_Datatype, int, MPI_Comm c) {
  if (c->size > 1) qsf_shim_fatal("MPI_Scatter over more than one rank is not available");
  if (s != r) memcpy(r, s, (size_t)n * qsf_shim_type_size(t));
  return 0;
}
static inline int MPI_Send(const void*, int, MPI_Datatype, int, int, MPI_Comm) { qsf_shim_fatal("MPI_Send is not available"); }
static inline int MPI_Recv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status*) {
  qsf_shim_fatal("MPI_Recv is not available");
}

static inline int MPI_Type_contiguous(int, MPI_Datatype, MPI_Datatype*) { qsf_shim_fatal("MPI_Type_contiguous is not available"); }
static inline int MPI_Type_create_struct(int, const int*, const MPI_Aint*, const MPI_Datatype*, MPI_Datatype*) {
  qsf_shim_fatal("MPI_Type_create_struct is not available");
}
static inline int MPI_Type_commit(MPI_Datatype*) { return 0; }

// ---------------------------------------------------------------- one-sided
static inline int MPI_Win_create(void* base, MPI_Aint size, int unit, MPI_Info, MPI_Comm c, MPI_Win* w) {
  qsf_shim_win* win = new qsf_shim_win();
  win->comm = c;
  win->entry = -1;
  *w = win;
  if (c->size <= 1) return 0;
  if (size > 0 && !qsf_shim_in_arena(base)) qsf_shim_fatal("window memory is not in the shared arena");
  const unsigned mask = qsf_shim_mask(c);
  const int seq = qsf_shim_win_seq[mask]++;
  for (int i = 0; i < kShimWins && win->entry < 0; ++i) {
    qsf_shim_wentry* e = &qsf_shim_sh->wins[i];
    unsigned cur = __atomic_load_n(&e->mask, __ATOMIC_ACQUIRE);
    if (cur == 0) {
      unsigned expected = 0;
      if (__atomic_compare_exchange_n(&e->mask, &expected, mask, false, __ATOMIC_ACQ_REL, __ATOMIC_ACQUIRE)) {
        __atomic_store_n(&e->seq, seq, __ATOMIC_RELEASE);
        win->entry = i;
        break;
      }
      cur = expected;
    }
    if (cur == mask) {
      qsf_shim_wait([&] { return __atomic_load_n(&e->seq, __ATOMIC_ACQUIRE) >= 0; }, "window table");
      if (e->seq == seq) win->entry = i;
    }
  }
  if (win->entry < 0) qsf_shim_fatal("out of window entries");
  qsf_shim_wentry* e = &qsf_shim_sh->wins[win->entry];
  e->base[qsf_shim_pid] = size > 0 ? base : nullptr;
  e->unit[qsf_shim_pid] = unit;
  qsf_shim_barrier(c);
  return 0;
}
static inline int MPI_Win_fence(int, MPI_Win w) {
  if (w) qsf_shim_barrier(w->comm);
  return 0;
}
static inline int MPI_Win_free(MPI_Win* w) {
  if (*w) qsf_shim_barrier((*w)->comm);
  return 0;
}
static inline int MPI_Get(void* origin, int count, MPI_Datatype t, int target, MPI_Aint disp, int, MPI_Datatype,
                          MPI_Win w) {
  if (!w || w->entry < 0) qsf_shim_fatal("MPI_Get on a window of one rank");
  const qsf_shim_wentry* e = &qsf_shim_sh->wins[w->entry];
  const int pid = w->comm->pids[target];
  const char* b = static_cast<const char*>(e->base[pid]);
  if (!b) qsf_shim_fatal("MPI_Get from a rank that exposes no memory");
  memcpy(origin, b + disp * e->unit[pid], (size_t)count * qsf_shim_type_size(t));
  return 0;
}

// ---------------------------------------------------------------- I/O (stdio)
static inline int MPI_File_open(MPI_Comm, const char* name, int mode, MPI_Info, MPI_File* fh) {
  *fh = fopen(name, (mode & MPI_MODE_RDONLY) ? "rb" : "wb");
  return *fh ? 0 : 1;
}
static inline int MPI_File_close(MPI_File* fh) { if (*fh) fclose(*fh); *fh = nullptr; return 0; }
static inline int MPI_File_delete(const char* name, MPI_Info) { remove(name); return 0; }
static inline int MPI_File_read(MPI_File fh, void* b, int n, MPI_Datatype t, MPI_Status*) {
  return fread(b, qsf_shim_type_size(t), (size_t)n, fh) == (size_t)n ? 0 : 1;
}
static inline int MPI_File_read_all(MPI_File fh, void* b, int n, MPI_Datatype t, MPI_Status* s) {
  return MPI_File_read(fh, b, n, t, s);
}
static inline int MPI_File_write(MPI_File fh, const void* b, int n, MPI_Datatype t, MPI_Status*) {
  return fwrite(b, qsf_shim_type_size(t), (size_t)n, fh) == (size_t)n ? 0 : 1;
}
static inline int MPI_File_seek(MPI_File fh, MPI_Offset o, int w) { return fseek(fh, (long)o, w); }
static inline int MPI_File_get_position(MPI_File fh, MPI_Offset* o) { *o = ftell(fh); return 0; }
static inline int MPI_File_set_view(MPI_File fh, MPI_Offset disp, MPI_Datatype, MPI_Datatype, const char*, MPI_Info) {
  return fseek(fh, (long)disp, SEEK_SET);
}
