/*
 * voce_legacy.h -- the reference's own entry points over its globals
 * (libvoce_legacy.so, which links libvoce_gpu.so).
 *
 * Voce's main (evp.c:7-32) calls GetNameList, OpenFiles, SetupJob,
 * Evolution, DestroyJob and CloseFiles, and the state lives in the globals
 * that evp.h:77-316 defines (under EVP_GLOBALS_ONCE, in evp.c).  Linking the
 * reference's evp.o and io.o against libvoce_legacy.so and libvoce_gpu.so,
 * in place of init.o, evolution.o, constitutive.o and kinematics.o, runs the
 * same job on the GPU:
 *
 *   mpicxx evp.o io.o -L<lib> -lvoce_legacy -lvoce_gpu -o evp
 *
 * The library exports every symbol io.o and evp.o take from the replaced
 * objects, under both C and C++ linkage (the reference's Makefile compiles
 * with mpicxx):
 *   SetupJob      init.c:617-828    reads the namelist globals that GetNameList
 *                                   filled, the .sx and mesh files they name
 *                                   (relative to the working directory), sets
 *                                   the RVE up on the current CUDA device and
 *                                   writes the vm.out / err.out headers
 *                                   (init.c:539-540) to fp_vm / fp_err
 *   Evolution     evolution.c:265-622  runs N_steps increments; writes the
 *                                   err.out and vm.out lines and the .iout
 *                                   dumps PrintControl and Tex_Flag select
 *                                   (voce_io.h); sets the macro globals
 *   DestroyJob    init.c:830-930    frees the RVE and the globals SetupJob
 *                                   allocated
 *   chg_basis, EulerToTransMatrix   kinematics.c:14-93, 187-240 (io.o calls them)
 *
 * Globals read: CellDim, TimeStep, N_steps, Err, IterMax, PrintControl,
 * Update_Flag, Hard_Flag, Tex_Flag, VelGrad_BC_Flag, VelGrad_BC,
 * Stress_BC_Flag, Stress_BC, N_phases, Type_phases, ElastConst_PhaseI/II,
 * Slip_PhaseI/II, initial_ms, self, coplane, cross, glissile, hirth, lomer,
 * rank, fp_vm, fp_err.
 * Globals written: Nxyz, WGT, Wgt_ph1, lnx, lxs, lnyt, lyst, lsize, B;
 * grain_f, phase_f, Sig, Eps, Edot, DisGrad, TranMat_xt2sa (allocated by
 * SetupJob, holding the state after SetupJob and after Evolution); after
 * every increment s_vm, s_vm1, e_vm, d_vm, Err_e, Err_s, SigAvg, SigAvg1,
 * EpsAvg, EdotAvg, DisGradAvg.
 *
 * One grid runs on one GPU: under mpirun only rank 0 does the work and the
 * other ranks return at once.  VOCE_PRECISION=mixed, mixed_ir or mixed_nr32
 * in the environment selects that precision form (FP64 otherwise).  A failure prints "voce: <message>" on
 * stderr and exits, with status 35 for a singular matrix (the reference's
 * exit(35), kinematics.c:306-309) and 1 otherwise.
 */
#ifndef VOCE_LEGACY_H
#define VOCE_LEGACY_H

#ifdef __cplusplus
extern "C" {
#endif

void SetupJob(void);
void Evolution(void);
void DestroyJob(void);
void chg_basis(double V6[6], double T2[3][3], double C2[6][6], double T4[3][3][3][3], int opt);
void EulerToTransMatrix(double *t1, double *ph, double *t2, double a[3][3], int opt);

#ifdef __cplusplus
}
#endif
#endif
