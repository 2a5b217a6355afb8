/*
 * voce_gpu.h -- C ABI of the GB300 EVP-FFT solver step (libvoce_gpu.so).
 *
 * Drop-in boundary for the solver step of the Voce crystal-plasticity code:
 * the Green-operator fixed point with the per-voxel Newton-Raphson stress
 * update and the Voce hardening law.  One RVE (representative volume
 * element) lives whole on one GPU; every kernel on the solve path is
 * hand-written sm_103a code in this library.  Plain C types only: no CUDA or
 * C++ types cross this boundary.
 *
 * Reference interfaces each group replaces (file:line in the Voce sources):
 *   voce_namelist_read    GetNameList           io.c:54-122 (names io.c:25-52)
 *   voce_slip_read        PlasticInit's reader  init.c:51-186
 *   voce_mesh_read        InitMicroStruct's reader init.c:393-442
 *   voce_rve_create       SetupJob              init.c:617-828
 *   voce_rve_run          Evolution (istep loop) evolution.c:265-622
 *   voce_rve_destroy      DestroyJob            init.c:830-930
 *   voce_rve_get_field    the field globals Sig/Eps/Edot/DisGrad/... that
 *                         io.c's Write*MPI dump (evp.h:190-316, io.c:193-1003)
 *   voce_rve_get_increment the vm.out line     evolution.c:562-566
 *   voce_rve_get_iter_log  the err.out lines   evolution.c:424-429
 *   SetupJob/Evolution/DestroyJob (voce_legacy.h) keep the reference's own
 *                         void(void) entry points over its globals.
 *
 * Errors: every function returns VOCE_OK (0) or a VOCE_ERR_* code and never
 * exits the process (the reference calls MPI_Abort or exit(35) instead:
 * evp.h:42-43, kinematics.c:306-309).  voce_last_error() gives a message.
 * Non-convergence (IterMax reached, Newton cap of 100 reached) is reported
 * in the increment record, not as an error, as in the reference.
 *
 * Threading: one host thread per handle; handles are independent (each has
 * its own CUDA stream).
 */
#ifndef VOCE_GPU_H
#define VOCE_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define VOCE_ABI_VERSION 1

enum {
    VOCE_OK = 0,
    VOCE_ERR_ARG = 1,         /* bad argument / null pointer */
    VOCE_ERR_IO = 2,          /* file cannot be opened or read */
    VOCE_ERR_PARSE = 3,       /* malformed input (mesh index mismatch: init.c:420-423) */
    VOCE_ERR_BC = 4,          /* inconsistent boundary conditions (init.c:713-735) */
    VOCE_ERR_SINGULAR = 5,    /* near-zero matrix row (kinematics.c:306-309) */
    VOCE_ERR_UNSUPPORTED = 6, /* grid size or material the library does not handle */
    VOCE_ERR_NOMEM = 7,       /* device allocation failed */
    VOCE_ERR_CUDA = 8,        /* CUDA runtime error, or no GPU */
    VOCE_ERR_STATE = 9,       /* call out of order */
    VOCE_ERR_CANCELLED = 10,  /* request cancelled by the caller (voce_serve.h) */
    VOCE_ERR_DEADLINE = 11    /* request not done by its deadline (voce_serve.h) */
};

/* Precision forms.
 *   VOCE_PREC_FP64        the reference's arithmetic: FP64 throughout.
 *   VOCE_PREC_MIXED       spectrum and Green-operator convolution in FP32; the
 *                         Newton-Raphson (the FP64 form's own code), the Voce
 *                         hardening, the averages and the error norms in FP64.
 *   VOCE_PREC_MIXED_NR32  as VOCE_PREC_MIXED, and the Newton iterations in
 *                         FP32 ended by an acceptance step on the FP64
 *                         residual (relative update below 1e-5), FP32-only
 *                         while the Green error is above 1e-4; per-voxel error
 *                         norms in FP32 (their sums in FP64).  The Newton
 *                         iterations and the norms are not FP64 here.
 *   VOCE_PREC_MIXED_IR    spectrum and Green-operator convolution in FP32;
 *                         the Newton iterations that accept a stress
 *                         evaluate the residual and the flow rule (resolved
 *                         shears, power law, strain rate) in FP64 and take
 *                         the reference's stop test in FP64, with the
 *                         correction -- the Jacobian's assembly and its LDL^T
 *                         solve -- in FP32 (iterative refinement: the
 *                         accepted stress is a root of the FP64 residual);
 *                         they start from a point solved on the FP32 pipe
 *                         (voce_set_ir_predictor); hardening, averages and
 *                         the per-voxel error norms in FP64. */
enum { VOCE_PREC_FP64 = 0, VOCE_PREC_MIXED = 1, VOCE_PREC_MIXED_NR32 = 2, VOCE_PREC_MIXED_IR = 3 };

/* Every variable the reference's namelist reader knows (io.c:25-52), with
 * the reference's names, types and lengths. */
typedef struct {
    int CellDim[3];
    int N_phases;
    int Type_phases[2];          /* 0 crystal, 1 gas */
    double TimeStep;
    int N_steps;
    int Update_Flag, Hard_Flag, Tex_Flag, IterMax;
    int PrintControl[2];
    double Err;
    int VelGrad_BC_Flag[6];      /* Voigt order 11,22,33,23,13,12 */
    double VelGrad_BC[6];
    int Stress_BC_Flag[6];
    double Stress_BC[6];
    double ElastConst_PhaseI[4];  /* c11 c12 c44 nu (MPa) */
    double ElastConst_PhaseII[4];
    char Slip_PhaseI[100], Slip_PhaseII[100], initial_ms[100];
    double self[2], coplane[2], cross[2], glissile[2], hirth[2], lomer[2];
} voce_namelist;

/* One slip mode of a .sx single-crystal file (init.c:117-178), as read:
 * slip-plane normals bn and directions bb are NOT normalised here. */
typedef struct {
    int nsys;                    /* <= 12 */
    double nrs, gamd0;           /* rate-sensitivity exponent, reference rate */
    double tau0f, tau0b, tau1, thet0, thet1;  /* Voce parameters */
    double bn[12][3], bb[12][3];
} voce_slip;

/* Microstructure: per voxel (x slowest, z fastest) Bunge angles in degrees,
 * grain id and 1-based phase id -- the columns of the mesh file. */
typedef struct {
    int dims[3];
    const double *euler_deg;     /* 3 per voxel */
    const int *grain;
    const int *phase;
} voce_mesh;

/* One vm.out line (evolution.c:563-564) plus the full-precision macro values
 * behind it. */
typedef struct {
    int istep, iters, iter_total;
    int nr_max;                  /* largest Newton iteration count seen */
    double e_vm, evmp, d_vm, dvmp, s_vm, s_vm1;
    double sig_avg[9], sig_avg1[9], eps_avg[9], edot_avg[9];
    double disgrad_avg[9];       /* DisGradAvg_actual at increment end */
    double err_e, err_s;         /* last iteration's normalised errors */
    double rot_slip_avg, rot_loc_avg; /* update_orient's printed averages */
    double nr_iters_total;       /* Newton iterations summed over voxels and iterations */
} voce_increment;

/* Field ids for voce_rve_get_field.  Tensors come back as 9 doubles per
 * voxel (row-major 3x3) like the reference globals (evp.h:304-312). */
enum {
    VOCE_FIELD_SIG = 0,        /* Sig, 9 */
    VOCE_FIELD_EPS = 1,        /* Eps, 9 */
    VOCE_FIELD_EDOT = 2,       /* Edot (plastic strain rate), 9 */
    VOCE_FIELD_DISGRAD = 3,    /* DisGrad, 9 */
    VOCE_FIELD_TRANMAT = 4,    /* TranMat_xt2sa, 9 */
    VOCE_FIELD_CRSS = 5,       /* crss (forward), 12 */
    VOCE_FIELD_GAMDOT = 6,     /* gamdot, 12 */
    VOCE_FIELD_GAMACUM = 7,    /* gamacum, 1 */
    VOCE_FIELD_SVM = 8,        /* SVM, 1 */
    VOCE_FIELD_EVM = 9,        /* EVM, 1 */
    VOCE_FIELD_GAMMATOTAL = 10, /* gammatotal (shear summed over increments), 12 */
    VOCE_FIELD_TAUX = 11,      /* tau_x (constitutive.c:45), 12 */
    VOCE_FIELD_RHO_RSS = 12,   /* rho_rss  (evolution.c:509-529: updated by  */
    VOCE_FIELD_RHO_CRSS = 13,  /* rho_crss  each increment from the third on */
    VOCE_FIELD_WORK_P = 14,    /* work_p    when Hard_Flag is 1; 0 before), 1 */
    VOCE_FIELD_DISP_FLUCT = 15, /* displacement fluctuation u~ (voxel units of
                                  length), 3: the periodic field whose gradient
                                  is DisGrad minus its average, computed when
                                  asked for.  It stands in for the reference's
                                  displacement_fluct (evolution.c:532-560),
                                  which sums over voxels into one value per
                                  component and scales by g = xi/|xi| instead
                                  of xi/|xi|^2.  Terms along a Nyquist
                                  coordinate cancel, as in the Green
                                  operator.  Allocates a 9-component spectrum
                                  work array on first use (72 B per voxel in
                                  FP64, 36 B in the mixed forms); single-
                                  precision spectrum in the mixed forms.  Not
                                  available through voce_rve_get_field_noalloc */
    VOCE_FIELD_SIG_VOIGT = 20, /* Sig 11,22,33,23,13,12: the order of the
                                  sig_1..6 dumps (io.c:321-358), 6 */
    VOCE_FIELD_EDOT_VOIGT = 21 /* Edot in the same order (io.c:360-397), 6 */
};

typedef struct voce_rve voce_rve;

int voce_abi_version(void);
const char *voce_last_error(void);

/* Input readers, same formats and quirks as the reference's. */
int voce_namelist_read(const char *path, voce_namelist *out);
int voce_slip_read(const char *path, voce_slip *out);
int voce_mesh_read(const char *path, const int dims[3], double *euler_deg,
                   int *grain, int *phase);

/* Set an RVE up on the current CUDA device (SetupJob).  slip[p] is the
 * slip mode of phase p+1 and may be NULL for a gas phase. */
int voce_rve_create(const voce_namelist *nl, const voce_slip *slip[2],
                    const voce_mesh *mesh, int precision, voce_rve **out);
/* Same, reading the namelist, .sx and mesh files (relative names are taken
 * relative to the namelist's directory). */
int voce_rve_create_from_files(const char *namelist_path, int precision,
                               voce_rve **out);
/* Advance n strain increments (each: prelude, Green-operator iterations to
 * convergence or IterMax, epilogue with reorientation and hardening). */
int voce_rve_run(voce_rve *r, int n_increments);
int voce_rve_increments_done(const voce_rve *r);
int voce_rve_get_increment(const voce_rve *r, int k, voce_increment *out);
/* Normalised errors and s_vm of every iteration of increment k (0-based);
 * returns the number of iterations written (at most max), or < 0. */
int voce_rve_get_iter_log(const voce_rve *r, int k, double *err_e,
                          double *err_s, double *s_vm, int max);
/* Full-precision record of every iteration of increment k, 12 doubles per
 * iteration: normalised Err_e, Err_s, s_vm, Newton iterations summed over
 * voxels, the raw sums over voxels of the strain and stress error norms (the
 * values the reference reduces at evolution.c:406-409), and the sum over
 * voxels of the stress 6-vector.  Returns the number of rows written. */
int voce_rve_get_iter_detail(const voce_rve *r, int k, double *rows, int max);
int voce_rve_get_field(voce_rve *r, int field, double *host_out);

/* voce_rve_get_field_noalloc: voce_rve_get_field without any device
 * allocation.  It has no counterpart in the reference (whose fields are host
 * globals).  For callers that cannot allocate device memory at download time:
 * a server whose HBM budget is committed to admitted RVEs (it downloads a
 * finished request before freeing that request's memory), a host that
 * overlaps downloads with other RVEs' increments on other streams (cudaMalloc
 * and cudaFree can synchronise the whole device), a host whose device memory
 * all belongs to its own pool allocator.  It calls no cudaMalloc, cudaFree or
 * other allocating routine; the field is staged in a fixed array of
 * VOCE_NOALLOC_MAX_DOUBLES doubles (32 MiB) that every GPU loading this
 * library's device code holds until the process exits.
 *   - A field of more doubles (width x voxels) fails with
 *     VOCE_ERR_UNSUPPORTED; voce_rve_get_field has no such limit.  Every field
 *     of an RVE up to 64^3 fits, and 1-wide fields up to 4 Mi voxels.
 *   - The first call on a device does its set-up (looks up the array's device
 *     address); make that first call before any stream capture.  The address
 *     is kept for the life of the process: a device reset (cudaDeviceReset)
 *     after that first call is not supported.
 *   - All calls on a device share the array, which keeps the last call's
 *     contents.  Each call writes every value it reads back, so nothing needs
 *     clearing, but calls whose work overlaps on the GPU (threads downloading
 *     RVEs on different streams at once) race on it: serialise them.
 *   - Output, errors and the synchronisation on return are those of
 *     voce_rve_get_field. */
#define VOCE_NOALLOC_MAX_DOUBLES 4194304
int voce_rve_get_field_noalloc(voce_rve *r, int field, double *host_out);

/* Synthetic microstructure on the GPU (no counterpart in the reference,
 * whose microstructure comes from a mesh file): the periodic Voronoi
 * tessellation of the unit cube by n_seeds seeds (x, y, z in [0,1)) on a
 * dims[0] x dims[1] x dims[2] grid of voxel centres ((i + 0.5) / n), by
 * minimum-image distance in FP64, ties to the lowest seed.  Fills a mesh
 * ready for voce_rve_create: grain = seed index + 1, phase = 1, and the
 * Bunge angles (degrees) given for its grain.  A request can carry seeds and
 * grain orientations instead of a whole mesh file. */
int voce_mesh_voronoi(const int dims[3], int n_seeds, const double *seeds_xyz,
                      const double *grain_euler_deg, double *euler_deg, int *grain, int *phase);

/* Snapshot / restore (no counterpart in the reference, which has no resume:
 * its io.c dumps are write-only).  A snapshot holds everything an RVE
 * carries from one call to the next: the per-voxel fields, hardening and
 * orientation state, the macro state, the increment records, the
 * per-iteration log rows of an increment in progress and the namelist.  Taken between calls (not while the RVE is in a batch); restored
 * on the current CUDA device as a new handle that continues exactly as the
 * original would (bit-identical increments).  A snapshot is read only by the
 * same build of the library (VOCE_ERR_UNSUPPORTED otherwise); a damaged one
 * fails with VOCE_ERR_PARSE.  Before any of it reaches the GPU, restore
 * checks what sizes an array or bounds an index against what creation makes
 * for the same grid and form: the grid and spectrum sizes, the precision
 * flags, each axis' transform schedule and FFT tiles, the work split, the
 * slip-system count, IterMax, the phase ids and the increment and iteration
 * counters of the macro state. */
long long voce_rve_snapshot_size(voce_rve *r);
int voce_rve_snapshot(voce_rve *r, void *buf, long long size);
int voce_rve_restore(const void *buf, long long size, voce_rve **out);
int voce_rve_save(voce_rve *r, const char *path);
int voce_rve_load(const char *path, voce_rve **out);

int voce_rve_destroy(voce_rve *r);

/* Device-memory footprint of an RVE of the given grid and precision, in
 * bytes (what voce_rve_create allocates). */
long long voce_rve_footprint(const int dims[3], int precision);

#ifdef __cplusplus
}
#endif
#endif
