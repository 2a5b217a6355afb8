/*
 * Single-process stand-in for the subset of the MPI-1/MPI-IO API that the
 * Voce reference sources call (init.c, evolution.c, constitutive.c, io.c,
 * testf.c).  TEST INFRASTRUCTURE ONLY: it exists so that the unmodified
 * reference C sources compile and run on one core as the parity oracle.
 *
 * Semantics: one rank by default (rank 0, size 1); VOCE_REF_RANKS=P runs P
 * forked ranks over shared memory (shim_mpi.c).  MPI_Allreduce sums in rank
 * order and, when the environment variable VOCE_REF_TRACE names a file,
 * rank 0 appends every reduced value with %.17g and a running call counter,
 * which gives a full-precision record of the reference's macro curve and
 * error trace.
 * MPI-IO writes go to the file at the view displacement with pwrite-style
 * positioning; derived struct types keep their holes, as MPI does.
 */
#ifndef VOCE_SHIM_MPI_H
#define VOCE_SHIM_MPI_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Info;
typedef long MPI_Aint;
typedef long long MPI_Offset;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR, count; } MPI_Status;
typedef struct shim_mpi_file *MPI_File;

#define MPI_COMM_WORLD 1
#define MPI_INFO_NULL 0
#define MPI_SUM 1
/* predefined datatypes; derived ones are numbered from 16 upwards */
#define MPI_INT 1
#define MPI_DOUBLE 2
#define MPI_FLOAT 3
#define MPI_MODE_CREATE 1
#define MPI_MODE_WRONLY 4
#define MPI_MODE_RDONLY 2
#define MPI_SUCCESS 0

int MPI_Init(int *argc, char ***argv);
int MPI_Finalize(void);
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Comm_rank(MPI_Comm comm, int *rank);
int MPI_Barrier(MPI_Comm comm);
int MPI_Abort(MPI_Comm comm, int errorcode);
int MPI_Allreduce(const void *sendbuf, void *recvbuf, int count,
                  MPI_Datatype datatype, MPI_Op op, MPI_Comm comm);
int MPI_Address(const void *location, MPI_Aint *address);
int MPI_Type_struct(int count, const int blocklens[], const MPI_Aint displs[],
                    const MPI_Datatype types[], MPI_Datatype *newtype);
int MPI_Type_commit(MPI_Datatype *type);
int MPI_File_open(MPI_Comm comm, const char *filename, int amode,
                  MPI_Info info, MPI_File *fh);
int MPI_File_set_view(MPI_File fh, MPI_Offset disp, MPI_Datatype etype,
                      MPI_Datatype filetype, const char *datarep,
                      MPI_Info info);
int MPI_File_write(MPI_File fh, const void *buf, int count,
                   MPI_Datatype datatype, MPI_Status *status);
int MPI_File_close(MPI_File *fh);

/* shim-only helpers (not MPI API) */
long shim_mpi_allreduce_calls(void);
void shim_mpi_trace_open(const char *path);
/* bytes of shared memory for the slab FFT's exchange buffer; call before
 * MPI_Init (the region is mapped before the ranks fork) */
void shim_mpi_reserve(size_t bytes);
void *shim_mpi_shared_buffer(void);
int shim_mpi_barrier(void);

#ifdef __cplusplus
}
#endif
#endif
