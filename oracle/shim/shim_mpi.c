/*
 * MPI stand-in (see mpi.h).  TEST INFRASTRUCTURE ONLY.
 *
 * One rank by default.  With VOCE_REF_RANKS=P (P > 1) MPI_Init forks P - 1
 * more processes that share one anonymous memory region (mapped before the
 * fork): a sense-reversing barrier, one reduction slot row per rank and the
 * exchange buffer of the slab FFT (shim_fftw.c).  MPI_Allreduce adds the
 * ranks' contributions in rank order, so every rank gets the same bits.
 * Rank 0 waits for the others in MPI_Finalize.
 */
#define _GNU_SOURCE
#include "mpi.h"

#include <sched.h>
#include <signal.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/mman.h>
#include <sys/wait.h>
#include <time.h>
#include <unistd.h>

static FILE *g_trace = NULL;
static long g_allreduce_calls = 0;

#define SHIM_MAX_RANKS 64
#define SHIM_MAX_COUNT 64
typedef struct {
    int count, sense, abort_flag, np;
    double slots[SHIM_MAX_RANKS][SHIM_MAX_COUNT];
} shim_ctl;
static shim_ctl *g_ctl = NULL;
static void *g_shared_buf = NULL;
static size_t g_reserve = 0;
static int g_rank = 0, g_size = 1, g_sense = 0;
static pid_t g_children[SHIM_MAX_RANKS];

void shim_mpi_reserve(size_t bytes) { g_reserve = bytes; }
void *shim_mpi_shared_buffer(void) { return g_shared_buf; }

/* all ranks meet; gives up (exit 3) when another rank has aborted or after
 * an hour, so that a failed rank cannot leave the others spinning */
static void shim_barrier(void)
{
    if (g_size == 1) return;
    g_sense = !g_sense;
    if (__atomic_add_fetch(&g_ctl->count, 1, __ATOMIC_ACQ_REL) == g_size) {
        __atomic_store_n(&g_ctl->count, 0, __ATOMIC_RELAXED);
        __atomic_store_n(&g_ctl->sense, g_sense, __ATOMIC_RELEASE);
        return;
    }
    const time_t t0 = time(NULL);
    for (long spin = 0; __atomic_load_n(&g_ctl->sense, __ATOMIC_ACQUIRE) != g_sense; ++spin) {
        if (__atomic_load_n(&g_ctl->abort_flag, __ATOMIC_RELAXED)) _exit(3);
        if ((spin & 1023) == 1023) {
            sched_yield();
            if (time(NULL) - t0 > 3600) { fprintf(stderr, "shim barrier timeout\n"); _exit(3); }
        }
    }
}

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
    const char *np = getenv("VOCE_REF_RANKS");
    int p = (np && *np) ? atoi(np) : 1;
    if (p < 1) p = 1;
    if (p > SHIM_MAX_RANKS) p = SHIM_MAX_RANKS;
    if (p > 1) {
        const size_t ctl = (sizeof(shim_ctl) + 4095) & ~(size_t)4095;
        void *m = mmap(NULL, ctl + g_reserve, PROT_READ | PROT_WRITE, MAP_SHARED | MAP_ANONYMOUS, -1, 0);
        if (m == MAP_FAILED) { perror("shim mmap"); exit(4); }
        g_ctl = (shim_ctl *)m;
        g_ctl->np = p;
        g_shared_buf = g_reserve ? (char *)m + ctl : NULL;
        fflush(NULL);
        for (int r = 1; r < p; ++r) {
            pid_t pid = fork();
            if (pid < 0) { perror("shim fork"); exit(4); }
            if (pid == 0) { g_rank = r; break; }
            g_children[r] = pid;
        }
        g_size = p;
    }
    const char *tp = getenv("VOCE_REF_TRACE");
    if (tp && *tp && g_rank == 0) shim_mpi_trace_open(tp);
    return MPI_SUCCESS;
}

int MPI_Finalize(void)
{
    shim_barrier();
    if (g_trace) { fclose(g_trace); g_trace = NULL; }
    if (g_rank > 0) {
        fflush(NULL);
        _exit(0);
    }
    int bad = 0;
    for (int r = 1; r < g_size; ++r) {
        int st = 0;
        if (waitpid(g_children[r], &st, 0) < 0 || !WIFEXITED(st) || WEXITSTATUS(st) != 0) bad = 1;
    }
    if (bad) { fprintf(stderr, "shim: a rank failed\n"); exit(5); }
    return MPI_SUCCESS;
}

int MPI_Comm_size(MPI_Comm comm, int *size) { (void)comm; *size = g_size; return 0; }
int MPI_Comm_rank(MPI_Comm comm, int *rank) { (void)comm; *rank = g_rank; return 0; }
int MPI_Barrier(MPI_Comm comm) { (void)comm; shim_barrier(); return 0; }
int shim_mpi_barrier(void) { shim_barrier(); return 0; }

int MPI_Abort(MPI_Comm comm, int errorcode)
{
    (void)comm;
    fprintf(stderr, "MPI_Abort(%d)\n", errorcode);
    fflush(NULL);
    if (g_ctl) __atomic_store_n(&g_ctl->abort_flag, 1, __ATOMIC_RELAXED);
    exit(errorcode ? errorcode : 1);
}

int MPI_Allreduce(const void *sendbuf, void *recvbuf, int count,
                  MPI_Datatype datatype, MPI_Op op, MPI_Comm comm)
{
    (void)op; (void)comm;
    int b = basic_size(datatype);
    if (g_size == 1) {
        memmove(recvbuf, sendbuf, (size_t)b * count);
    } else {
        if (count > SHIM_MAX_COUNT) MPI_Abort(0, 91);
        for (int i = 0; i < count; ++i)
            g_ctl->slots[g_rank][i] = datatype == MPI_INT ? (double)((const int *)sendbuf)[i]
                                                          : ((const double *)sendbuf)[i];
        shim_barrier();
        for (int i = 0; i < count; ++i) {
            double acc = g_ctl->slots[0][i];
            for (int r = 1; r < g_size; ++r) acc += g_ctl->slots[r][i];   /* rank order */
            if (datatype == MPI_INT) ((int *)recvbuf)[i] = (int)acc;
            else ((double *)recvbuf)[i] = acc;
        }
        shim_barrier();
    }
    for (int i = 0; i < count; ++i) {
        ++g_allreduce_calls;
        if (!g_trace) continue;
        if (datatype == MPI_DOUBLE)
            fprintf(g_trace, "%ld d %.17g\n", g_allreduce_calls,
                    ((const double *)recvbuf)[i]);
        else if (datatype == MPI_INT)
            fprintf(g_trace, "%ld i %d\n", g_allreduce_calls,
                    ((const int *)recvbuf)[i]);
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
    /* collective: rank 0 creates the file before the others open it */
    if (g_rank > 0) shim_barrier();
    if (amode & MPI_MODE_RDONLY) fp = fopen(filename, "rb");
    else {
        fp = fopen(filename, "r+b");
        if (!fp && (amode & MPI_MODE_CREATE)) fp = fopen(filename, "w+b");
    }
    if (g_rank == 0 && g_size > 1) shim_barrier();
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
    shim_barrier();   /* collective: every rank's part is written */
    return 0;
}
