/*
 * Test host for libvoce_legacy.so: a stand-in for the reference's program
 * (evp.c:7-32 with GetNameList, io.c:54-122, and OpenFiles, io.c:171-180).
 * It defines the globals the legacy layer reads and writes, with the names
 * and types of evp.h:77-316, fills the namelist ones with voce_namelist_read
 * (the same reader semantics as GetNameList), opens vm.out / err.out and
 * calls SetupJob, Evolution and DestroyJob.  After Evolution it prints one
 * line with some of the globals the layer sets, for the tests to check.
 *
 * usage: host_main <namelist>     (run in the directory of the input files)
 */
#include <stdio.h>
#include <string.h>

#include "voce_gpu.h"
#include "voce_legacy.h"

typedef double real;
typedef real ten2nd[3][3];

int CellDim[3], Nxyz, N_steps, IterMax, PrintControl[2], Update_Flag, Hard_Flag, Tex_Flag;
real TimeStep, Err;
int VelGrad_BC_Flag[6], Stress_BC_Flag[6];
real VelGrad_BC[6], Stress_BC[6];
int N_phases, Type_phases[2];
real ElastConst_PhaseI[4], ElastConst_PhaseII[4];
char Slip_PhaseI[100], Slip_PhaseII[100], initial_ms[100];
real self[2], coplane[2], cross[2], glissile[2], hirth[2], lomer[2];
int rank, NumPE;
int lnx, lxs, lnyt, lyst, lsize;
FILE *fp_vm, *fp_err;
real WGT, Wgt_ph1;
real d_vm, s_vm, e_vm, s_vm1, Err_e, Err_s;
ten2nd SigAvg, EpsAvg, EdotAvg, SigAvg1, DisGradAvg;
ten2nd *Sig, *Eps, *Edot, *DisGrad, *TranMat_xt2sa;
int *grain_f, *phase_f;
ten2nd B[6];

int main(int argc, char **argv)
{
    if (argc < 2) {
        fprintf(stderr, "usage: %s <namelist>\n", argv[0]);
        return 2;
    }
    voce_namelist nl;
    if (voce_namelist_read(argv[1], &nl) != VOCE_OK) {
        fprintf(stderr, "namelist: %s\n", voce_last_error());
        return 1;
    }
    memcpy(CellDim, nl.CellDim, sizeof(CellDim));
    N_phases = nl.N_phases;
    memcpy(Type_phases, nl.Type_phases, sizeof(Type_phases));
    TimeStep = nl.TimeStep;
    N_steps = nl.N_steps;
    Update_Flag = nl.Update_Flag;
    Hard_Flag = nl.Hard_Flag;
    Tex_Flag = nl.Tex_Flag;
    IterMax = nl.IterMax;
    memcpy(PrintControl, nl.PrintControl, sizeof(PrintControl));
    Err = nl.Err;
    memcpy(VelGrad_BC_Flag, nl.VelGrad_BC_Flag, sizeof(VelGrad_BC_Flag));
    memcpy(VelGrad_BC, nl.VelGrad_BC, sizeof(VelGrad_BC));
    memcpy(Stress_BC_Flag, nl.Stress_BC_Flag, sizeof(Stress_BC_Flag));
    memcpy(Stress_BC, nl.Stress_BC, sizeof(Stress_BC));
    memcpy(ElastConst_PhaseI, nl.ElastConst_PhaseI, sizeof(ElastConst_PhaseI));
    memcpy(ElastConst_PhaseII, nl.ElastConst_PhaseII, sizeof(ElastConst_PhaseII));
    memcpy(Slip_PhaseI, nl.Slip_PhaseI, sizeof(Slip_PhaseI));
    memcpy(Slip_PhaseII, nl.Slip_PhaseII, sizeof(Slip_PhaseII));
    memcpy(initial_ms, nl.initial_ms, sizeof(initial_ms));
    memcpy(self, nl.self, sizeof(self));
    memcpy(coplane, nl.coplane, sizeof(coplane));
    memcpy(cross, nl.cross, sizeof(cross));
    memcpy(glissile, nl.glissile, sizeof(glissile));
    memcpy(hirth, nl.hirth, sizeof(hirth));
    memcpy(lomer, nl.lomer, sizeof(lomer));
    rank = 0;
    NumPE = 1;

    fp_vm = fopen("vm.out", "w+");
    fp_err = fopen("err.out", "w+");
    if (!fp_vm || !fp_err) {
        fprintf(stderr, "cannot open vm.out / err.out\n");
        return 1;
    }
    SetupJob();
    Evolution();
    printf("GLOBALS %d %.17g %.17g %.17g %.17g %.17g\n", Nxyz, s_vm, SigAvg[2][2], Sig[0][2][2],
           Sig[Nxyz - 1][0][1], DisGrad[Nxyz / 2][1][2]);
    DestroyJob();
    fclose(fp_vm);
    fclose(fp_err);
    return 0;
}
