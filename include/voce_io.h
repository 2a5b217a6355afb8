/*
 * voce_io.h -- the reference's output files, written from an RVE handle.
 *
 * The reference writes three kinds of output while Evolution() runs:
 *   vm.out    one line per increment          evolution.c:562-566, header init.c:539
 *   err.out   "STEP = n" and one line per     evolution.c:301-303, 424-429,
 *             Green-operator iteration        header init.c:540
 *   *.iout    binary field dumps through MPI-IO with the "native" view
 *             (io.c:193-1003), after increments that PrintControl selects
 *             and, with Tex_Flag 1, a final set (evolution.c:568-611).
 * These functions produce the same files, same names and same bytes layout:
 * raw native-endian doubles for the per-voxel scalar dumps (voxel order x
 * slowest, z fastest), and fixed-size records for the per-system and texture
 * dumps, including the padding holes that the reference's MPI struct types
 * leave (written as zero bytes, which is what a new file holds there).  Like
 * the reference (MPI_MODE_CREATE|MPI_MODE_WRONLY), an existing file is
 * overwritten from its start and not truncated.
 */
#ifndef VOCE_IO_H
#define VOCE_IO_H

#include <stdio.h>

#include "voce_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Kinds of .iout dump, named after the reference writer each follows.
 * <name> is the writer's first argument (it may start with a directory). */
enum {
    VOCE_IOUT_EPS = 0,      /* WriteEpsMPI  io.c:193-229: <name>_<1..6>_S%04d.iout,
                               Eps 11,22,33,23,13,12 */
    VOCE_IOUT_SIG = 1,      /* WriteSigMPI  io.c:321-358: <name>_<1..6>_S%04d.iout */
    VOCE_IOUT_ELS = 2,      /* WriteElsMPI  io.c:280-319: <name>_<1..6>_S%06d.iout,
                               sym(DisGrad) - Eps */
    VOCE_IOUT_EDOT = 3,     /* WriteEdotMPI io.c:360-397: <name>_<1..6>_S%04d.iout */
    VOCE_IOUT_SLIP = 4,     /* WriteSLIPMPI io.c:651-726: <name>_S%04d.iout, 104-byte
                               records: int grain, 4 pad bytes, 12 doubles gammatotal */
    VOCE_IOUT_TAUX = 5,     /* WritetauxMPI io.c:728-804: same records, tau_x */
    VOCE_IOUT_CRSS = 6,     /* WriteCRSSMPI io.c:860-937: same records, forward crss */
    VOCE_IOUT_TEX = 7,      /* WriteTextureMPI io.c:939-1003: <name>_S%04d.iout, 48-byte
                               records: Bunge angles (deg) of TranMat, 3 doubles;
                               x, y, z (1-based), grain, phase, 0: 6 ints */
    VOCE_IOUT_SVM = 8,      /* WriteSVMMPI  io.c:567-593: <name>_S%04d.iout */
    VOCE_IOUT_EVM = 9,      /* WriteEVMMPI  io.c:595-621: <name>_S%04d.iout */
    VOCE_IOUT_RHO_RSS = 10, /* WriteRhoRMPI io.c:426-452: <name>_S%04d.iout */
    VOCE_IOUT_RHO_CRSS = 11, /* WriteRhoCRMPI io.c:398-424: <name>_S%04d.iout */
    VOCE_IOUT_WORK_P = 12,  /* WriteWorkPMPI io.c:623-649: <name>_S%06d.iout */
    VOCE_IOUT_WORK_E = 13,  /* WriteWorkEMPI io.c:231-278: <name>_S%06d.iout,
                               0.5 Sig : T(els), T() reading the Voigt-ordered
                               elastic strain as basis coefficients as the
                               reference does */
    VOCE_IOUT_NEW_POSITION = 14 /* WriteNewPositionMPI io.c:806-858: <name>_S%04d.iout,
                               24-byte records of 3 doubles: the displacement
                               fluctuation VOCE_FIELD_DISP_FLUCT.  Same names and
                               layout as the reference's; the values are the
                               corrected field, where the reference's
                               (evolution.c:532-560) come out as
                               -fluctuation[i][2] */
};

/* One dump of the RVE's current state. */
int voce_rve_write_iout(voce_rve *r, int kind, const char *name, int step);

/* The dumps Evolution() writes after increment istep (1-based), under the
 * namelist the RVE was created from: with PrintControl[0] == 1 and istep a
 * multiple of PrintControl[1], eps, sig, els and edot, plus (Tex_Flag 1)
 * slip_sys, taux_sys, crss_sys, tex, rho_rss, rho_crss, work_p, SVM, EVM and
 * new_position (evolution.c:568-589).  Returns VOCE_OK without writing when istep is not
 * selected.  dir is prepended to the names ("" or NULL: current directory). */
int voce_rve_write_step_iout(voce_rve *r, int istep, const char *dir);
/* The final set Evolution() writes with Tex_Flag 1 (evolution.c:592-611),
 * step 0; nothing otherwise. */
int voce_rve_write_final_iout(voce_rve *r, const char *dir);

/* The header lines of vm.out and err.out (init.c:539-540). */
int voce_write_log_headers(FILE *fp_vm, FILE *fp_err);
/* The err.out lines and the vm.out line of increment k (0-based), in the
 * reference's formats; the "STEP = n" line only when n_steps != 1, as in
 * evolution.c:301.  Either file may be NULL. */
int voce_rve_write_log(const voce_rve *r, int k, int n_steps, FILE *fp_vm, FILE *fp_err);

/* Grain and phase ids of every voxel, as given at creation. */
int voce_rve_get_ids(const voce_rve *r, int *grain, int *phase);
/* The namelist the RVE was created from. */
int voce_rve_get_namelist(const voce_rve *r, voce_namelist *out);

#ifdef __cplusplus
}
#endif
#endif
