// Single-rank MPI stand-in (test infrastructure): implementation of the
// declarations in mpi.h.  Only used to compile and run the reference solver's
// own sources on one host core; see mpi.h for the contract.
#include "mpi.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

namespace {

struct SubarrayType {
  int ndims;
  int sizes[3];
  int subsizes[3];
  int starts[3];
  MPI_Datatype base;
};

std::vector<SubarrayType> g_types;  // handle h >= 16 -> g_types[h - 16]

struct PendingSend {
  int tag;
  std::vector<char> data;
};
struct PendingRecv {
  void *buf;
  size_t capacity;
  int tag;
  bool done;
};

std::vector<PendingSend> g_sends;   // self messages not yet received
std::vector<PendingRecv> g_recvs;   // request handle r -> g_recvs[r - 1]

void die(const char *what) {
  std::fprintf(stderr, "refshim MPI: %s\n", what);
  std::abort();
}

size_t base_size(MPI_Datatype t) {
  switch (t) {
    case MPI_BYTE: return 1;
    case MPI_INT: return sizeof(int);
    case MPI_DOUBLE: return sizeof(double);
    default: break;
  }
  if (t >= 16 && (size_t)(t - 16) < g_types.size()) {
    const SubarrayType &s = g_types[t - 16];
    size_t n = base_size(s.base);
    for (int d = 0; d < s.ndims; ++d) n *= (size_t)s.subsizes[d];
    return n;
  }
  die("unknown datatype");
  return 0;
}

// Byte offsets (relative to the type's origin) of every base element of a
// datatype, in the type-map order.
std::vector<size_t> type_map(MPI_Datatype t, size_t *elem) {
  std::vector<size_t> offs;
  if (t < 16) {
    *elem = base_size(t);
    offs.push_back(0);
    return offs;
  }
  const SubarrayType &s = g_types[t - 16];
  *elem = base_size(s.base);
  if (s.ndims != 3) die("only 3-D subarrays are supported");
  for (int a = 0; a < s.subsizes[0]; ++a)
    for (int b = 0; b < s.subsizes[1]; ++b)
      for (int c = 0; c < s.subsizes[2]; ++c) {
        size_t lin = ((size_t)(s.starts[0] + a) * s.sizes[1] + (s.starts[1] + b)) *
                         s.sizes[2] + (s.starts[2] + c);
        offs.push_back(lin * *elem);
      }
  return offs;
}

}  // namespace

struct tpm_shim_file {
  FILE *fp;
  MPI_Offset disp;
  MPI_Datatype filetype;  // 0 = default byte view
};

extern "C" {

int MPI_Init(int *, char ***) { return MPI_SUCCESS; }
int MPI_Finalize(void) { return MPI_SUCCESS; }
int MPI_Comm_rank(MPI_Comm, int *rank) { *rank = 0; return MPI_SUCCESS; }
int MPI_Comm_size(MPI_Comm, int *size) { *size = 1; return MPI_SUCCESS; }
int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }

int MPI_Isend(const void *buf, int count, MPI_Datatype type, int, int tag, MPI_Comm,
              MPI_Request *req) {
  size_t bytes = (size_t)count * base_size(type);
  for (auto &r : g_recvs) {
    if (!r.done && r.tag == tag) {
      if (bytes > r.capacity) die("message larger than posted receive");
      if (bytes) std::memcpy(r.buf, buf, bytes);
      r.done = true;
      *req = 0;
      return MPI_SUCCESS;
    }
  }
  PendingSend s;
  s.tag = tag;
  s.data.assign((const char *)buf, (const char *)buf + bytes);
  g_sends.push_back(std::move(s));
  *req = 0;
  return MPI_SUCCESS;
}

int MPI_Irecv(void *buf, int count, MPI_Datatype type, int, int tag, MPI_Comm,
              MPI_Request *req) {
  size_t cap = (size_t)count * base_size(type);
  for (size_t i = 0; i < g_sends.size(); ++i) {
    if (g_sends[i].tag == tag) {
      if (g_sends[i].data.size() > cap) die("message larger than posted receive");
      if (!g_sends[i].data.empty()) std::memcpy(buf, g_sends[i].data.data(), g_sends[i].data.size());
      g_sends.erase(g_sends.begin() + (long)i);
      *req = 0;
      return MPI_SUCCESS;
    }
  }
  PendingRecv r{buf, cap, tag, false};
  g_recvs.push_back(r);
  *req = (int)g_recvs.size();
  return MPI_SUCCESS;
}

int MPI_Send(const void *buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm c) {
  MPI_Request r;
  return MPI_Isend(buf, count, type, dest, tag, c, &r);
}

int MPI_Recv(void *buf, int count, MPI_Datatype type, int source, int tag, MPI_Comm c,
             MPI_Status *st) {
  MPI_Request r;
  MPI_Irecv(buf, count, type, source, tag, c, &r);
  return MPI_Waitall(1, &r, st);
}

int MPI_Waitall(int count, MPI_Request *reqs, MPI_Status *) {
  for (int i = 0; i < count; ++i) {
    if (reqs[i] > 0) {
      if (!g_recvs[reqs[i] - 1].done) die("receive never matched (would deadlock)");
      reqs[i] = 0;
    }
  }
  bool all_done = true;
  for (auto &r : g_recvs) all_done = all_done && r.done;
  if (all_done) g_recvs.clear();
  return MPI_SUCCESS;
}

int MPI_Reduce(const void *sendbuf, void *recvbuf, int count, MPI_Datatype type, MPI_Op, int,
               MPI_Comm) {
  if (sendbuf != recvbuf) std::memcpy(recvbuf, sendbuf, (size_t)count * base_size(type));
  return MPI_SUCCESS;
}

int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return MPI_SUCCESS; }

int MPI_Gather(const void *sendbuf, int sendcount, MPI_Datatype sendtype, void *recvbuf, int,
               MPI_Datatype, int, MPI_Comm) {
  if (sendbuf != recvbuf) std::memcpy(recvbuf, sendbuf, (size_t)sendcount * base_size(sendtype));
  return MPI_SUCCESS;
}

int MPI_Scatter(const void *sendbuf, int sendcount, MPI_Datatype sendtype, void *recvbuf, int,
                MPI_Datatype, int, MPI_Comm) {
  if (sendbuf != recvbuf) std::memcpy(recvbuf, sendbuf, (size_t)sendcount * base_size(sendtype));
  return MPI_SUCCESS;
}

int MPI_Type_create_subarray(int ndims, const int sizes[], const int subsizes[],
                             const int starts[], int order, MPI_Datatype oldtype,
                             MPI_Datatype *newtype) {
  if (order != MPI_ORDER_C || ndims != 3) die("only 3-D C-order subarrays are supported");
  SubarrayType s;
  s.ndims = ndims;
  for (int d = 0; d < 3; ++d) {
    s.sizes[d] = sizes[d];
    s.subsizes[d] = subsizes[d];
    s.starts[d] = starts[d];
  }
  s.base = oldtype;
  g_types.push_back(s);
  *newtype = 16 + (int)g_types.size() - 1;
  return MPI_SUCCESS;
}

int MPI_Type_commit(MPI_Datatype *) { return MPI_SUCCESS; }
int MPI_Type_free(MPI_Datatype *) { return MPI_SUCCESS; }

int MPI_File_open(MPI_Comm, const char *filename, int amode, MPI_Info, MPI_File *fh) {
  FILE *fp = nullptr;
  if (amode & MPI_MODE_RDONLY) {
    fp = std::fopen(filename, "rb");
  } else {
    fp = std::fopen(filename, "r+b");  // MPI_File_open never truncates
    if (!fp && (amode & MPI_MODE_CREATE)) fp = std::fopen(filename, "w+b");
  }
  if (!fp) {
    std::fprintf(stderr, "refshim MPI: cannot open %s\n", filename);
    std::abort();
  }
  *fh = new tpm_shim_file{fp, 0, 0};
  return MPI_SUCCESS;
}

int MPI_File_close(MPI_File *fh) {
  std::fclose((*fh)->fp);
  delete *fh;
  *fh = nullptr;
  return MPI_SUCCESS;
}

int MPI_File_set_view(MPI_File fh, MPI_Offset disp, MPI_Datatype, MPI_Datatype filetype,
                      const char *, MPI_Info) {
  fh->disp = disp;
  fh->filetype = filetype;
  return MPI_SUCCESS;
}

static void file_xfer(MPI_File fh, MPI_Offset start, char *mem, int count, MPI_Datatype memtype,
                      bool write) {
  size_t melem = 0, felem = 0;
  std::vector<size_t> moffs = type_map(memtype, &melem);
  std::vector<size_t> foffs;
  if (fh->filetype >= 16) {
    foffs = type_map(fh->filetype, &felem);
  }
  size_t nmem = moffs.size() * (size_t)count;
  size_t mext = (memtype >= 16) ? 0 : melem;  // contiguous repetition for base types
  auto offsets = [&](size_t e, size_t *moff, size_t *foff) {
    size_t rep = e / moffs.size();
    *moff = moffs[e % moffs.size()] + rep * mext;
    if (fh->filetype >= 16) {
      if (e >= foffs.size()) die("file view smaller than the transfer");
      *foff = (size_t)fh->disp + foffs[e];
    } else {
      *foff = (size_t)fh->disp + (size_t)start + e * melem;
    }
  };
  // transfer maximal runs that are contiguous both in memory and in the file
  size_t e = 0;
  while (e < nmem) {
    size_t m0, f0;
    offsets(e, &m0, &f0);
    size_t len = 1;
    while (e + len < nmem) {
      size_t m1, f1;
      offsets(e + len, &m1, &f1);
      if (m1 != m0 + len * melem || f1 != f0 + len * melem) break;
      ++len;
    }
    std::fseek(fh->fp, (long)f0, SEEK_SET);
    size_t bytes = len * melem;
    size_t n = write ? std::fwrite(mem + m0, 1, bytes, fh->fp)
                     : std::fread(mem + m0, 1, bytes, fh->fp);
    if (n != bytes) die(write ? "short write" : "short read (file too small)");
    e += len;
  }
}

int MPI_File_read_all(MPI_File fh, void *buf, int count, MPI_Datatype type, MPI_Status *) {
  file_xfer(fh, 0, (char *)buf, count, type, false);
  return MPI_SUCCESS;
}

int MPI_File_write_all(MPI_File fh, const void *buf, int count, MPI_Datatype type,
                       MPI_Status *) {
  file_xfer(fh, 0, (char *)buf, count, type, true);
  return MPI_SUCCESS;
}

int MPI_File_read_at_all(MPI_File fh, MPI_Offset offset, void *buf, int count,
                         MPI_Datatype type, MPI_Status *) {
  file_xfer(fh, offset, (char *)buf, count, type, false);
  return MPI_SUCCESS;
}

int MPI_File_write_at_all(MPI_File fh, MPI_Offset offset, const void *buf, int count,
                          MPI_Datatype type, MPI_Status *) {
  file_xfer(fh, offset, (char *)buf, count, type, true);
  return MPI_SUCCESS;
}

}  // extern "C"
