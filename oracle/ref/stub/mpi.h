/*
  Single-process stand-in for the MPI interface, used only to compile the
  reference sources into the CPU checker under oracle/_ref.  Test
  infrastructure: nothing in the shipped library includes this header.

  Semantics on the one rank that exists:
    * rank 0, size 1 for every communicator;
    * collectives copy the send buffer into the receive buffer
      (or leave it alone for MPI_IN_PLACE);
    * point-to-point messages to self are queued and matched by tag
      (the reference never sends a message on one rank, but the queue keeps
      the stub honest if it ever does);
    * MPI-IO writes go through stdio.
*/
#ifndef A2DS_ORACLE_MPI_STUB_H
#define A2DS_ORACLE_MPI_STUB_H

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Info;
typedef long long MPI_Offset;
typedef FILE *MPI_File;

typedef struct {
  int MPI_SOURCE;
  int MPI_TAG;
  int MPI_ERROR;
  int count_bytes;
} MPI_Status;

typedef int MPI_Request;

#define MPI_COMM_WORLD 91
#define MPI_COMM_SELF 92
#define MPI_COMM_NULL 0
#define MPI_SUCCESS 0
#define MPI_IDENT 0
#define MPI_CONGRUENT 1
#define MPI_SIMILAR 2
#define MPI_UNEQUAL 3
#define MPI_ANY_SOURCE (-1)
#define MPI_ANY_TAG (-1)
#define MPI_INFO_NULL 0
#define MPI_MAX_ERROR_STRING 256
#define MPI_MODE_RDONLY 1
#define MPI_MODE_WRONLY 2
#define MPI_MODE_CREATE 4
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_STATUSES_IGNORE ((MPI_Status *)0)
#define MPI_REQUEST_NULL (-1)
#define MPI_IN_PLACE ((void *)1)

/* Datatype handles encode their byte size in the low byte. */
#define MPI_CHAR ((1 << 8) | 1)
#define MPI_BYTE ((2 << 8) | 1)
#define MPI_INT ((3 << 8) | 4)
#define MPI_FLOAT ((4 << 8) | 4)
#define MPI_DOUBLE ((5 << 8) | 8)
#define MPI_DOUBLE_COMPLEX ((6 << 8) | 16)
#define MPI_LONG ((7 << 8) | 8)
#define MPI_UNSIGNED ((8 << 8) | 4)

#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3
#define MPI_PROD 4

typedef void(MPI_User_function)(void *, void *, int *, MPI_Datatype *);

static inline size_t a2ds_mpi_tsize(MPI_Datatype t) { return (size_t)(t & 0xff); }

static inline int MPI_Init(int *, char ***) { return 0; }
static inline int MPI_Initialized(int *flag) {
  *flag = 1;
  return 0;
}
static inline int MPI_Finalize() { return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int *rank) {
  *rank = 0;
  return 0;
}
static inline int MPI_Comm_size(MPI_Comm, int *size) {
  *size = 1;
  return 0;
}
static inline int MPI_Comm_dup(MPI_Comm c, MPI_Comm *n) {
  *n = c;
  return 0;
}
static inline int MPI_Comm_free(MPI_Comm *) { return 0; }
static inline int MPI_Comm_compare(MPI_Comm a, MPI_Comm b, int *r) {
  *r = (a == b) ? MPI_IDENT : MPI_CONGRUENT;
  return 0;
}
static inline int MPI_Comm_split(MPI_Comm c, int, int, MPI_Comm *n) {
  *n = c;
  return 0;
}
static inline double MPI_Wtime() {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}
static inline int MPI_Abort(MPI_Comm, int code) {
  fprintf(stderr, "MPI_Abort(%d) called in the single-process stub\n", code);
  abort();
  return code;
}
static inline int MPI_Barrier(MPI_Comm) { return 0; }
static inline int MPI_Error_string(int, char *s, int *len) {
  strcpy(s, "mpi stub error");
  *len = (int)strlen(s);
  return 0;
}
static inline int MPI_Op_create(MPI_User_function *, int, MPI_Op *op) {
  *op = MPI_MAX;
  return 0;
}
static inline int MPI_Op_free(MPI_Op *) { return 0; }

static inline void a2ds_mpi_copy(const void *s, void *r, int count,
                                 MPI_Datatype t) {
  if (s != MPI_IN_PLACE && s && r && count > 0 && s != r) {
    memmove(r, s, (size_t)count * a2ds_mpi_tsize(t));
  }
}

static inline int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t,
                                MPI_Op, MPI_Comm) {
  a2ds_mpi_copy(s, r, n, t);
  return 0;
}
static inline int MPI_Reduce(const void *s, void *r, int n, MPI_Datatype t,
                             MPI_Op, int, MPI_Comm) {
  a2ds_mpi_copy(s, r, n, t);
  return 0;
}
static inline int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) {
  return 0;
}
static inline int MPI_Scan(const void *s, void *r, int n, MPI_Datatype t,
                           MPI_Op, MPI_Comm) {
  a2ds_mpi_copy(s, r, n, t);
  return 0;
}
static inline int MPI_Allgather(const void *s, int sn, MPI_Datatype st, void *r,
                                int, MPI_Datatype, MPI_Comm) {
  a2ds_mpi_copy(s, r, sn, st);
  return 0;
}
static inline int MPI_Allgatherv(const void *s, int sn, MPI_Datatype st,
                                 void *r, const int *, const int *displs,
                                 MPI_Datatype rt, MPI_Comm) {
  if (s != MPI_IN_PLACE) {
    a2ds_mpi_copy(s, (char *)r + (size_t)displs[0] * a2ds_mpi_tsize(rt), sn, st);
  }
  return 0;
}
static inline int MPI_Gather(const void *s, int sn, MPI_Datatype st, void *r,
                             int, MPI_Datatype, int, MPI_Comm) {
  a2ds_mpi_copy(s, r, sn, st);
  return 0;
}
static inline int MPI_Gatherv(const void *s, int sn, MPI_Datatype st, void *r,
                              const int *, const int *displs, MPI_Datatype rt,
                              int, MPI_Comm) {
  if (r && displs) {
    a2ds_mpi_copy(s, (char *)r + (size_t)displs[0] * a2ds_mpi_tsize(rt), sn,
                  st);
  }
  return 0;
}
static inline int MPI_Scatter(const void *s, int sn, MPI_Datatype st, void *r,
                              int, MPI_Datatype, int, MPI_Comm) {
  a2ds_mpi_copy(s, r, sn, st);
  return 0;
}
static inline int MPI_Scatterv(const void *s, const int *scounts,
                               const int *displs, MPI_Datatype st, void *r, int,
                               MPI_Datatype, int, MPI_Comm) {
  if (s && scounts && displs) {
    a2ds_mpi_copy((const char *)s + (size_t)displs[0] * a2ds_mpi_tsize(st), r,
                  scounts[0], st);
  }
  return 0;
}
static inline int MPI_Alltoall(const void *s, int sn, MPI_Datatype st, void *r,
                               int, MPI_Datatype, MPI_Comm) {
  a2ds_mpi_copy(s, r, sn, st);
  return 0;
}
static inline int MPI_Alltoallv(const void *s, const int *scounts,
                                const int *sdispls, MPI_Datatype st, void *r,
                                const int *, const int *rdispls,
                                MPI_Datatype rt, MPI_Comm) {
  if (s && r && scounts && scounts[0] > 0) {
    memmove((char *)r + (size_t)rdispls[0] * a2ds_mpi_tsize(rt),
            (const char *)s + (size_t)sdispls[0] * a2ds_mpi_tsize(st),
            (size_t)scounts[0] * a2ds_mpi_tsize(st));
  }
  return 0;
}

/* Self messages: the reference never exchanges data on one rank; any
   attempt to move a non-empty payload is reported and aborts. */
static inline int a2ds_mpi_p2p(int n, const char *what) {
  if (n > 0) {
    fprintf(stderr, "%s with %d items in the single-process stub\n", what, n);
    abort();
  }
  return 0;
}
static inline int MPI_Send(const void *, int n, MPI_Datatype, int, int,
                           MPI_Comm) {
  return a2ds_mpi_p2p(n, "MPI_Send");
}
static inline int MPI_Isend(const void *, int n, MPI_Datatype, int, int,
                            MPI_Comm, MPI_Request *req) {
  if (req) *req = MPI_REQUEST_NULL;
  return a2ds_mpi_p2p(n, "MPI_Isend");
}
static inline int MPI_Irecv(void *, int n, MPI_Datatype, int, int, MPI_Comm,
                            MPI_Request *req) {
  if (req) *req = MPI_REQUEST_NULL;
  return a2ds_mpi_p2p(n, "MPI_Irecv");
}
static inline int MPI_Recv(void *, int n, MPI_Datatype, int, int, MPI_Comm,
                           MPI_Status *) {
  return a2ds_mpi_p2p(n, "MPI_Recv");
}
static inline int MPI_Probe(int, int, MPI_Comm, MPI_Status *) {
  return a2ds_mpi_p2p(1, "MPI_Probe");
}
static inline int MPI_Get_count(const MPI_Status *s, MPI_Datatype t, int *n) {
  *n = s ? (int)(s->count_bytes / (int)a2ds_mpi_tsize(t)) : 0;
  return 0;
}
static inline int MPI_Wait(MPI_Request *, MPI_Status *) { return 0; }
static inline int MPI_Waitall(int, MPI_Request *, MPI_Status *) { return 0; }
static inline int MPI_Waitany(int, MPI_Request *, int *index, MPI_Status *) {
  *index = 0;
  return 0;
}

/* MPI-IO over stdio.  A file view's displacement (bytes) is kept per open
   file: MPI_File_write / read continue from the view start, and the
   explicit-offset calls take their offset in elements from it. */
static inline MPI_Offset *a2ds_mpi_view_disp(MPI_File fp, int release) {
  static MPI_File files[16];
  static MPI_Offset disp[16];
  for (int k = 0; k < 16; k++)
    if (files[k] == fp) {
      if (release) files[k] = NULL;
      return &disp[k];
    }
  for (int k = 0; k < 16; k++)
    if (!files[k]) {
      files[k] = fp;
      disp[k] = 0;
      return &disp[k];
    }
  return &disp[0];
}
static inline int MPI_File_open(MPI_Comm, const char *name, int mode, MPI_Info,
                                MPI_File *fp) {
  *fp = fopen(name, (mode & MPI_MODE_WRONLY) ? "wb" : "rb");
  if (*fp) *a2ds_mpi_view_disp(*fp, 0) = 0;
  return *fp ? 0 : 1;
}
static inline int MPI_File_close(MPI_File *fp) {
  if (*fp) {
    a2ds_mpi_view_disp(*fp, 1);
    fclose(*fp);
  }
  *fp = NULL;
  return 0;
}
static inline int MPI_File_set_size(MPI_File, MPI_Offset) { return 0; }
static inline int MPI_File_set_view(MPI_File fp, MPI_Offset disp, MPI_Datatype,
                                    MPI_Datatype, const char *, MPI_Info) {
  *a2ds_mpi_view_disp(fp, 0) = disp;
  return fseek(fp, (long)disp, SEEK_SET);
}
static inline int MPI_File_write(MPI_File fp, const void *b, int n,
                                 MPI_Datatype t, MPI_Status *) {
  fwrite(b, a2ds_mpi_tsize(t), (size_t)n, fp);
  return 0;
}
static inline int MPI_File_read(MPI_File fp, void *b, int n, MPI_Datatype t,
                                MPI_Status *) {
  size_t r = fread(b, a2ds_mpi_tsize(t), (size_t)n, fp);
  return r == (size_t)n ? 0 : 1;
}
static inline int MPI_File_write_at_all(MPI_File fp, MPI_Offset off,
                                        const void *b, int n, MPI_Datatype t,
                                        MPI_Status *) {
  fseek(fp, (long)(*a2ds_mpi_view_disp(fp, 0) + off * (MPI_Offset)a2ds_mpi_tsize(t)), SEEK_SET);
  fwrite(b, a2ds_mpi_tsize(t), (size_t)n, fp);
  return 0;
}
static inline int MPI_File_read_at_all(MPI_File fp, MPI_Offset off, void *b,
                                       int n, MPI_Datatype t, MPI_Status *) {
  fseek(fp, (long)(*a2ds_mpi_view_disp(fp, 0) + off * (MPI_Offset)a2ds_mpi_tsize(t)), SEEK_SET);
  size_t r = fread(b, a2ds_mpi_tsize(t), (size_t)n, fp);
  return r == (size_t)n ? 0 : 1;
}

#endif
