/*
 * CPU restatement of the Voce EVP-FFT solver step -- the parity ORACLE.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py may load or run it, and only as the checker
 * or the timed CPU baseline.  The product (voce_gb300, libvoce_gpu.so) never
 * links, loads or calls anything here.
 *
 * It restates, in plain C, what the reference computes for one RVE
 * (reference files cited per function in evp_oracle.c): the namelist, .sx
 * and mesh readers, SetupJob, the Evolution() increment loop with the
 * Green-operator fixed point, the per-voxel Newton-Raphson, the mixed
 * boundary-condition update, reorientation and Voce hardening.  It keeps the
 * reference's data layout (3x3 tensors per voxel, a 81-coefficient Green
 * operator table, nine complex FFTs each way) and its floating-point
 * operation order, and uses the same FFT code as the FFTW-2 shim, so a
 * single-process run reproduces the reference built against the shims bit
 * for bit.  Voxel loops run on OpenMP threads; every sum over voxels is
 * taken afterwards in voxel order, so the result does not depend on the
 * thread count.
 */
#ifndef VOCE_EVP_ORACLE_H
#define VOCE_EVP_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_job oracle_job;

/* Reads the namelist (and the .sx and mesh files it names; relative names
 * are taken relative to the namelist's directory) and sets the job up like
 * SetupJob.  When trace_path is given, the value of every reduction the
 * reference performs with MPI_Allreduce is written there, in its order and
 * in the MPI shim's trace format.  Returns NULL and fills err (if given,
 * 256 bytes) on failure. */
oracle_job *oracle_create(const char *namelist_path, int nthreads,
                          const char *trace_path, char *err);
void oracle_destroy(oracle_job *j);

/* Runs n increments (each: prelude, Green iterations, epilogue).  Returns
 * the number of increments done so far. */
int oracle_run(oracle_job *j, int n_increments);

/* Per-increment record (the vm.out line plus full-precision macro values). */
typedef struct {
    int istep, iters, iter_total;
    double e_vm, evmp, d_vm, dvmp, s_vm, s_vm1;
    double sig_avg[9], sig_avg1[9], eps_avg[9], edot_avg[9];
    double disgrad_avg[9];   /* DisGradAvg_actual at increment end */
    double err_e, err_s;     /* last iteration's normalised errors */
} oracle_incr;

int oracle_n_increments(const oracle_job *j);
int oracle_get_increment(const oracle_job *j, int k, oracle_incr *out);
/* per-iteration errors of increment k (0-based): arrays of length iters */
int oracle_get_iter_log(const oracle_job *j, int k, double *err_e,
                        double *err_s, double *s_vm);

/* Fields, voxel order (x slowest, z fastest).
 *   0 Sig, 1 Eps, 2 Edot, 3 DisGrad  : 9 doubles per voxel (3x3 row-major)
 *   4 TranMat_xt2sa                  : 9
 *   5 crss (forward)                 : 12
 *   6 gamdot                         : 12
 *   7 gamacum                        : 1
 *   8 SVM, 9 EVM                     : 1
 *   10 Schm_gr                       : 60 (12 systems x 5)
 *   11 C_gr                          : 36
 * Returns the number of doubles per voxel, or -1. */
int oracle_get_field(const oracle_job *j, int id, double *out);
long oracle_nvox(const oracle_job *j);
int oracle_dims(const oracle_job *j, int *dims3);
/* Displacement fluctuation (the corrected evolution.c:532-560), 3 doubles
 * per voxel, from the accumulated fluctuation (from_fluct 1) or from DisGrad
 * (0).  Uses the job's FFT buffer; returns 0, or -1 when out of memory. */
int oracle_disp_fluct(oracle_job *j, int from_fluct, double *out);
/* C066 (36), S066 (36), WGT, Wgt_ph1 */
int oracle_get_reference_medium(const oracle_job *j, double *c066,
                                double *s066, double *wgt_ph1);

/* ---- function-level entry points (each mirrors one reference function) */
void oracle_basis(double B[6][3][3]);
void oracle_chg_basis(double *v6, double *t2, double *c2, double *t4, int opt);
void oracle_chg_basis5(double *v5, double *t2, double *c2, double *t4, int opt);
/* returns 0, or 35 when a row is (near) zero (the reference exits with 35) */
int oracle_lu_inv66(double *c66);
void oracle_euler_to_transmatrix(double t1, double ph, double t2, double *a9);
/* StrainRate_eval for one voxel given its Schmid (12x5), crss (12x2) */
void oracle_strain_rate(int nsys, const double *stress6, const double *sch60,
                        const double *tau24, const double *nsrs,
                        const double *gam0, double *edot6, double *d_edot36,
                        double *gamdot12, double *taux12);
/* UpdateStress body for one solid voxel.  Inputs: C_gr (36), C066 (36),
 * Sig/Eps/DisGrad (3x3 each), Schmid (60), crss (24), nsrs/gam0 (12 each),
 * dt.  Outputs: new Sig (9), Edot (9), gamdot (12), SVM, EVM,
 * conv_istep_s, conv_istep_e, NR iteration count. */
int oracle_update_stress_voxel(int nsys, const double *cgr36,
                               const double *c066, const double *sig9,
                               const double *eps9, const double *disgrad9,
                               const double *sch60, const double *tau24,
                               const double *nsrs, const double *gam0,
                               double dt, double *sig_out9, double *edot_out9,
                               double *gamdot12, double *svm, double *evm,
                               double *conv_s, double *conv_e);
/* harden() for one voxel (constitutive.c:250-310) */
void oracle_harden_voxel(int nsys, const double *hard144, const double *tau3,
                         const double *thet2, double dt,
                         const double *gamdot12, double *gamacum,
                         double *gammatotal12, double *crss24);
/* Orientation() (constitutive.c:117-169): tran9 updated in place */
void oracle_orientation(double *tran9, const double *rot9);

#ifdef __cplusplus
}
#endif
#endif
