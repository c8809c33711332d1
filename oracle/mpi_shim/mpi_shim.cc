// Thread-backed MPI stand-in for building the reference POREMAPS sources as a
// CPU oracle.  Test infrastructure only (see mpi.h).  Each MPI rank is a
// thread; collectives are deterministic (rank-ordered reductions).
#include "mpi.h"

#include <pthread.h>
#include <fcntl.h>
#include <unistd.h>
#include <time.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>
#include <algorithm>

// The reference program's own main().  Rank 0 is the process's main thread;
// MPI_Init on rank 0 starts ranks 1..P-1 as threads that enter main() again.
int main(int argc, char** argv);

namespace {

thread_local int tls_rank = 0;
int g_np = 1;
pthread_barrier_t g_barrier;

int g_dims[3] = {1, 1, 1};
int g_periods[3] = {0, 0, 0};

std::mutex g_mbox_mu;
std::condition_variable g_mbox_cv;
std::map<std::tuple<int, int, int>, std::deque<std::vector<char>>> g_mbox;

std::vector<const void*> g_slots;

struct Subarray {
  int sizes[3], subsizes[3], starts[3], order;
  MPI_Datatype old;
};
std::mutex g_types_mu;
std::vector<Subarray> g_types;

struct ShimFile {
  int fd;
  MPI_Offset disp;
  MPI_Datatype etype;
  MPI_Datatype filetype;
};

size_t type_size(MPI_Datatype t) {
  switch (t) {
    case MPI_C_BOOL: return sizeof(bool);
    case MPI_INT: return sizeof(int);
    case MPI_DOUBLE: return sizeof(double);
    default: fprintf(stderr, "mpi shim: unsupported datatype %d\n", t); abort();
  }
}

void barrier() { pthread_barrier_wait(&g_barrier); }

void coords_of(int rank, int* c) {
  c[2] = rank % g_dims[2];
  c[1] = (rank / g_dims[2]) % g_dims[1];
  c[0] = rank / (g_dims[2] * g_dims[1]);
}

int rank_of(const int* c) { return (c[0] * g_dims[1] + c[1]) * g_dims[2] + c[2]; }

Subarray subarray(MPI_Datatype t) {
  std::lock_guard<std::mutex> lk(g_types_mu);
  return g_types.at(t - PM_SHIM_FIRST_DERIVED);
}

// Visit the contiguous x-runs of a 3-D subarray (dim 0 fastest for Fortran
// order, as the reference always uses).  f(file_elem_offset, n_elems).
template <class F>
void for_each_run(const Subarray& s, F f) {
  if (s.order != MPI_ORDER_FORTRAN) { fprintf(stderr, "mpi shim: C order unsupported\n"); abort(); }
  for (int z = 0; z < s.subsizes[2]; ++z)
    for (int y = 0; y < s.subsizes[1]; ++y) {
      long long off = ((long long)(s.starts[2] + z) * s.sizes[1] + (s.starts[1] + y)) *
                          (long long)s.sizes[0] + s.starts[0];
      f(off, s.subsizes[0]);
    }
}

thread_local bool tls_started = false;
std::vector<pthread_t> g_threads;
int g_argc = 0;
char** g_argv = nullptr;

void* rank_thread(void* arg) {
  tls_rank = (int)(long)arg;
  tls_started = true;
  main(g_argc, g_argv);
  return nullptr;
}

}  // namespace

extern "C" {

int MPI_Init(int* argc, char*** argv) {
  if (tls_started) return 0;  // a rank thread re-entering main()
  tls_started = true;
  const char* np = getenv("PM_SHIM_NP");
  g_np = np ? atoi(np) : 1;
  if (g_np < 1) g_np = 1;
  g_slots.assign(g_np, nullptr);
  pthread_barrier_init(&g_barrier, nullptr, g_np);
  g_argc = argc ? *argc : 0;
  g_argv = argv ? *argv : nullptr;
  g_threads.resize(g_np);
  for (int r = 1; r < g_np; ++r) pthread_create(&g_threads[r], nullptr, rank_thread, (void*)(long)r);
  return 0;
}

int MPI_Finalize(void) {
  barrier();
  if (tls_rank == 0)
    for (int r = 1; r < g_np; ++r) pthread_join(g_threads[r], nullptr);
  return 0;
}
int MPI_Comm_rank(MPI_Comm, int* rank) { *rank = tls_rank; return 0; }
int MPI_Comm_size(MPI_Comm, int* size) { *size = g_np; return 0; }
int MPI_Barrier(MPI_Comm) { barrier(); return 0; }

int MPI_Dims_create(int nnodes, int ndims, int* dims) {
  // Balanced factorisation, largest first (as MPICH/OpenMPI produce).
  std::vector<int> primes;
  int n = nnodes;
  for (int p = 2; p * p <= n; ++p)
    while (n % p == 0) { primes.push_back(p); n /= p; }
  if (n > 1) primes.push_back(n);
  std::sort(primes.rbegin(), primes.rend());
  std::vector<int> d(ndims, 1);
  for (int p : primes) {
    int best = 0;
    for (int i = 1; i < ndims; ++i)
      if (d[i] < d[best]) best = i;
    d[best] *= p;
  }
  std::sort(d.rbegin(), d.rend());
  for (int i = 0; i < ndims; ++i) dims[i] = d[i];
  return 0;
}

int MPI_Cart_create(MPI_Comm, int ndims, const int* dims, const int* periods, int,
                    MPI_Comm* comm_cart) {
  for (int i = 0; i < ndims && i < 3; ++i) { g_dims[i] = dims[i]; g_periods[i] = periods[i]; }
  if (g_dims[0] * g_dims[1] * g_dims[2] != g_np) {
    fprintf(stderr, "mpi shim: dims %d %d %d do not match %d ranks\n", g_dims[0], g_dims[1],
            g_dims[2], g_np);
    abort();
  }
  barrier();
  *comm_cart = MPI_COMM_CART_BASE;
  return 0;
}

int MPI_Cart_coords(MPI_Comm, int rank, int, int* coords) { coords_of(rank, coords); return 0; }

int MPI_Cart_shift(MPI_Comm, int direction, int disp, int* source, int* dest) {
  int c[3];
  coords_of(tls_rank, c);
  int lo[3] = {c[0], c[1], c[2]}, hi[3] = {c[0], c[1], c[2]};
  lo[direction] -= disp;
  hi[direction] += disp;
  int d = g_dims[direction];
  auto fix = [&](int* cc) -> int {
    if (cc[direction] < 0 || cc[direction] >= d) {
      if (!g_periods[direction]) return MPI_PROC_NULL;
      cc[direction] = ((cc[direction] % d) + d) % d;
    }
    return rank_of(cc);
  };
  *source = fix(lo);
  *dest = fix(hi);
  return 0;
}

int MPI_Sendrecv(const void* sendbuf, int sendcount, MPI_Datatype sendtype, int dest,
                 int sendtag, void* recvbuf, int recvcount, MPI_Datatype recvtype,
                 int source, int recvtag, MPI_Comm, MPI_Status* status) {
  if (dest != MPI_PROC_NULL) {
    size_t n = (size_t)sendcount * type_size(sendtype);
    std::vector<char> msg((const char*)sendbuf, (const char*)sendbuf + n);
    std::lock_guard<std::mutex> lk(g_mbox_mu);
    g_mbox[std::make_tuple(tls_rank, dest, sendtag)].push_back(std::move(msg));
    g_mbox_cv.notify_all();
  }
  if (source != MPI_PROC_NULL) {
    auto key = std::make_tuple(source, tls_rank, recvtag);
    std::unique_lock<std::mutex> lk(g_mbox_mu);
    g_mbox_cv.wait(lk, [&] { auto it = g_mbox.find(key); return it != g_mbox.end() && !it->second.empty(); });
    std::vector<char> msg = std::move(g_mbox[key].front());
    g_mbox[key].pop_front();
    size_t n = std::min(msg.size(), (size_t)recvcount * type_size(recvtype));
    memcpy(recvbuf, msg.data(), n);
  }
  if (status) { status->MPI_SOURCE = source; status->MPI_TAG = recvtag; status->MPI_ERROR = 0; }
  return 0;
}

int MPI_Allreduce(const void* sendbuf, void* recvbuf, int count, MPI_Datatype type, MPI_Op op,
                  MPI_Comm) {
  const void* mine = (sendbuf == MPI_IN_PLACE) ? recvbuf : sendbuf;
  g_slots[tls_rank] = mine;
  barrier();
  size_t es = type_size(type);
  std::vector<char> acc((size_t)count * es);
  memcpy(acc.data(), g_slots[0], acc.size());
  for (int r = 1; r < g_np; ++r) {
    for (int i = 0; i < count; ++i) {
      if (type == MPI_DOUBLE) {
        double* a = (double*)acc.data() + i;
        double b = ((const double*)g_slots[r])[i];
        *a = (op == MPI_SUM) ? (*a + b) : (b > *a ? b : *a);
      } else if (type == MPI_INT) {
        int* a = (int*)acc.data() + i;
        int b = ((const int*)g_slots[r])[i];
        *a = (op == MPI_SUM) ? (*a + b) : (b > *a ? b : *a);
      } else {
        fprintf(stderr, "mpi shim: Allreduce type %d unsupported\n", type);
        abort();
      }
    }
  }
  barrier();
  memcpy(recvbuf, acc.data(), acc.size());
  return 0;
}

int MPI_Type_create_subarray(int ndims, const int* sizes, const int* subsizes, const int* starts,
                             int order, MPI_Datatype oldtype, MPI_Datatype* newtype) {
  if (ndims != 3) { fprintf(stderr, "mpi shim: only 3-D subarrays\n"); abort(); }
  Subarray s;
  for (int i = 0; i < 3; ++i) { s.sizes[i] = sizes[i]; s.subsizes[i] = subsizes[i]; s.starts[i] = starts[i]; }
  s.order = order;
  s.old = oldtype;
  std::lock_guard<std::mutex> lk(g_types_mu);
  g_types.push_back(s);
  *newtype = PM_SHIM_FIRST_DERIVED + (int)g_types.size() - 1;
  return 0;
}

int MPI_Type_commit(MPI_Datatype*) { return 0; }
int MPI_Type_free(MPI_Datatype*) { return 0; }

int MPI_File_open(MPI_Comm, const char* filename, int amode, MPI_Info, MPI_File* fh) {
  int flags = (amode & MPI_MODE_RDWR) ? O_RDWR : O_RDONLY;
  if (amode & MPI_MODE_CREATE) flags |= O_CREAT;
  int fd = open(filename, flags, 0644);
  if (fd < 0) { fprintf(stderr, "mpi shim: cannot open %s\n", filename); abort(); }
  ShimFile* f = new ShimFile{fd, 0, MPI_C_BOOL, MPI_C_BOOL};
  *fh = (MPI_File)f;
  barrier();
  return 0;
}

int MPI_File_set_view(MPI_File fh, MPI_Offset disp, MPI_Datatype etype, MPI_Datatype filetype,
                      const char*, MPI_Info) {
  ShimFile* f = (ShimFile*)fh;
  f->disp = disp;
  f->etype = etype;
  f->filetype = filetype;
  return 0;
}

int MPI_File_read_at_all(MPI_File fh, MPI_Offset offset, void* buf, int count, MPI_Datatype type,
                         MPI_Status*) {
  ShimFile* f = (ShimFile*)fh;
  size_t es = type_size(type);
  const Subarray s = subarray(f->filetype);
  char* out = (char*)buf;
  long long done = 0;
  for_each_run(s, [&](long long off, int n) {
    if (done >= count) return;
    ssize_t want = (ssize_t)n * es;
    ssize_t got = pread(f->fd, out, want, f->disp + (off + offset) * (long long)es);
    if (got < want) memset(out + (got > 0 ? got : 0), 0, want - (got > 0 ? got : 0));
    out += want;
    done += n;
  });
  barrier();
  return 0;
}

int MPI_File_write_at_all(MPI_File fh, MPI_Offset offset, const void* buf, int count,
                          MPI_Datatype type, MPI_Status*) {
  ShimFile* f = (ShimFile*)fh;
  size_t es = type_size(type);
  const Subarray s = subarray(f->filetype);
  const char* in = (const char*)buf;
  long long done = 0;
  for_each_run(s, [&](long long off, int n) {
    if (done >= count) return;
    ssize_t want = (ssize_t)n * es;
    if (pwrite(f->fd, in, want, f->disp + (off + offset) * (long long)es) != want) {
      fprintf(stderr, "mpi shim: short write\n");
      abort();
    }
    in += want;
    done += n;
  });
  barrier();
  return 0;
}

int MPI_File_close(MPI_File* fh) {
  ShimFile* f = (ShimFile*)*fh;
  close(f->fd);
  delete f;
  *fh = nullptr;
  barrier();
  return 0;
}

double MPI_Wtime(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

}  // extern "C"
