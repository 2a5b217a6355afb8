/*
 * Single-process MPI stand-in (see mpi.h).  TEST INFRASTRUCTURE ONLY.
 */
#include "mpi.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static FILE *g_trace = NULL;
static long g_allreduce_calls = 0;

#define MAX_TYPES 64
#define MAX_FIELDS 32
typedef struct {
    int nfields;
    long extent;
    long off[MAX_FIELDS];
    int size[MAX_FIELDS]; /* bytes of one field element */
    int count[MAX_FIELDS];
} shim_type;
static shim_type g_types[MAX_TYPES];
static int g_ntypes = 0;

struct shim_mpi_file {
    FILE *fp;
    long long disp;
    MPI_Datatype filetype;
};

static int basic_size(MPI_Datatype t)
{
    switch (t) {
    case MPI_INT: return (int)sizeof(int);
    case MPI_DOUBLE: return (int)sizeof(double);
    case MPI_FLOAT: return (int)sizeof(float);
    default: return 0;
    }
}

static long type_extent(MPI_Datatype t)
{
    int b = basic_size(t);
    if (b) return b;
    if (t >= 16 && t < 16 + g_ntypes) return g_types[t - 16].extent;
    return 0;
}

void shim_mpi_trace_open(const char *path)
{
    if (g_trace) fclose(g_trace);
    g_trace = path ? fopen(path, "w") : NULL;
}

long shim_mpi_allreduce_calls(void) { return g_allreduce_calls; }

int MPI_Init(int *argc, char ***argv)
{
    (void)argc; (void)argv;
    const char *tp = getenv("VOCE_REF_TRACE");
    if (tp && *tp) shim_mpi_trace_open(tp);
    return MPI_SUCCESS;
}

int MPI_Finalize(void)
{
    if (g_trace) { fclose(g_trace); g_trace = NULL; }
    return MPI_SUCCESS;
}

int MPI_Comm_size(MPI_Comm comm, int *size) { (void)comm; *size = 1; return 0; }
int MPI_Comm_rank(MPI_Comm comm, int *rank) { (void)comm; *rank = 0; return 0; }
int MPI_Barrier(MPI_Comm comm) { (void)comm; return 0; }

int MPI_Abort(MPI_Comm comm, int errorcode)
{
    (void)comm;
    fprintf(stderr, "MPI_Abort(%d)\n", errorcode);
    fflush(NULL);
    exit(errorcode ? errorcode : 1);
}

int MPI_Allreduce(const void *sendbuf, void *recvbuf, int count,
                  MPI_Datatype datatype, MPI_Op op, MPI_Comm comm)
{
    (void)op; (void)comm;
    int b = basic_size(datatype);
    memmove(recvbuf, sendbuf, (size_t)b * count);
    for (int i = 0; i < count; ++i) {
        ++g_allreduce_calls;
        if (!g_trace) continue;
        if (datatype == MPI_DOUBLE)
            fprintf(g_trace, "%ld d %.17g\n", g_allreduce_calls,
                    ((const double *)sendbuf)[i]);
        else if (datatype == MPI_INT)
            fprintf(g_trace, "%ld i %d\n", g_allreduce_calls,
                    ((const int *)sendbuf)[i]);
    }
    return MPI_SUCCESS;
}

int MPI_Address(const void *location, MPI_Aint *address)
{
    *address = (MPI_Aint)(size_t)location;
    return 0;
}

int MPI_Type_struct(int count, const int blocklens[], const MPI_Aint displs[],
                    const MPI_Datatype types[], MPI_Datatype *newtype)
{
    if (g_ntypes >= MAX_TYPES || count > MAX_FIELDS) MPI_Abort(0, 90);
    shim_type *t = &g_types[g_ntypes];
    t->nfields = count;
    t->extent = 0;
    for (int i = 0; i < count; ++i) {
        t->off[i] = displs[i];
        t->size[i] = basic_size(types[i]);
        t->count[i] = blocklens[i];
        long end = displs[i] + (long)t->size[i] * blocklens[i];
        if (end > t->extent) t->extent = end;
    }
    /* round the extent up to the largest member alignment, as C does */
    long al = 1;
    for (int i = 0; i < count; ++i) if (t->size[i] > al) al = t->size[i];
    t->extent = (t->extent + al - 1) / al * al;
    *newtype = 16 + g_ntypes;
    ++g_ntypes;
    return 0;
}

int MPI_Type_commit(MPI_Datatype *type) { (void)type; return 0; }

int MPI_File_open(MPI_Comm comm, const char *filename, int amode,
                  MPI_Info info, MPI_File *fh)
{
    (void)comm; (void)info;
    FILE *fp = NULL;
    if (amode & MPI_MODE_RDONLY) fp = fopen(filename, "rb");
    else {
        fp = fopen(filename, "r+b");
        if (!fp && (amode & MPI_MODE_CREATE)) fp = fopen(filename, "w+b");
    }
    if (!fp) return 1;
    struct shim_mpi_file *f = (struct shim_mpi_file *)calloc(1, sizeof(*f));
    f->fp = fp;
    f->filetype = MPI_DOUBLE;
    *fh = f;
    return 0;
}

int MPI_File_set_view(MPI_File fh, MPI_Offset disp, MPI_Datatype etype,
                      MPI_Datatype filetype, const char *datarep, MPI_Info info)
{
    (void)etype; (void)datarep; (void)info;
    fh->disp = disp;
    fh->filetype = filetype;
    return 0;
}

int MPI_File_write(MPI_File fh, const void *buf, int count,
                   MPI_Datatype datatype, MPI_Status *status)
{
    const char *src = (const char *)buf;
    long ext = type_extent(datatype);
    if (basic_size(datatype)) {
        fseeko(fh->fp, (off_t)fh->disp, SEEK_SET);
        fwrite(src, (size_t)ext, (size_t)count, fh->fp);
    } else {
        /* derived type: write each member at its displacement, keep holes */
        const shim_type *t = &g_types[datatype - 16];
        for (long e = 0; e < count; ++e) {
            for (int k = 0; k < t->nfields; ++k) {
                off_t pos = (off_t)(fh->disp + e * t->extent + t->off[k]);
                fseeko(fh->fp, pos, SEEK_SET);
                fwrite(src + e * t->extent + t->off[k], (size_t)t->size[k],
                       (size_t)t->count[k], fh->fp);
            }
        }
    }
    if (status) status->count = count;
    return 0;
}

int MPI_File_close(MPI_File *fh)
{
    if (fh && *fh) {
        fclose((*fh)->fp);
        free(*fh);
        *fh = NULL;
    }
    return 0;
}
