// libvoce_legacy.so: SetupJob / Evolution / DestroyJob over the reference's
// globals (voce_legacy.h), C linkage.  The C++-linkage names the reference's
// own build binds are in voce_legacy_cxx.cpp and forward here.
#include "voce_legacy_impl.h"

#include "voce_gpu.h"
#include "voce_io.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

// ---- the reference's globals this layer uses (defined by the program,
// evp.h:77-316 under EVP_GLOBALS_ONCE); names and types must match ----------
typedef double real;
typedef real ten2nd[3][3];

extern int CellDim[3];
extern int Nxyz;
extern real TimeStep;
extern int N_steps;
extern real Err;
extern int IterMax;
extern int PrintControl[2];
extern int Update_Flag, Hard_Flag, Tex_Flag;
extern int VelGrad_BC_Flag[6];
extern real VelGrad_BC[6];
extern int Stress_BC_Flag[6];
extern real Stress_BC[6];
extern int N_phases;
extern int Type_phases[2];
extern real ElastConst_PhaseI[4], ElastConst_PhaseII[4];
extern char Slip_PhaseI[100], Slip_PhaseII[100], initial_ms[100];
extern real self[2], coplane[2], cross[2], glissile[2], hirth[2], lomer[2];
extern int rank, NumPE;
extern int lnx, lxs, lnyt, lyst, lsize;
extern FILE *fp_vm, *fp_err;
extern real WGT, Wgt_ph1;
extern real d_vm, s_vm, e_vm, s_vm1, Err_e, Err_s;
extern ten2nd SigAvg, EpsAvg, EdotAvg, SigAvg1, DisGradAvg;
extern ten2nd *Sig, *Eps, *Edot, *DisGrad, *TranMat_xt2sa;
extern int *grain_f, *phase_f;
extern ten2nd B[6];

namespace {

voce_rve *g_rve = nullptr;
bool g_owned = false;  // the field globals below were allocated here

[[noreturn]] void die(int rc)
{
    std::fprintf(stderr, "voce: %s\n", voce_last_error());
    std::exit(rc == VOCE_ERR_SINGULAR ? 35 : 1);
}

void check(int rc)
{
    if (rc != VOCE_OK) die(rc);
}

void namelist_from_globals(voce_namelist *nl)
{
    std::memset(nl, 0, sizeof(*nl));
    std::memcpy(nl->CellDim, CellDim, sizeof(nl->CellDim));
    nl->N_phases = N_phases;
    std::memcpy(nl->Type_phases, Type_phases, sizeof(nl->Type_phases));
    nl->TimeStep = TimeStep;
    nl->N_steps = N_steps;
    nl->Update_Flag = Update_Flag;
    nl->Hard_Flag = Hard_Flag;
    nl->Tex_Flag = Tex_Flag;
    nl->IterMax = IterMax;
    std::memcpy(nl->PrintControl, PrintControl, sizeof(nl->PrintControl));
    nl->Err = Err;
    std::memcpy(nl->VelGrad_BC_Flag, VelGrad_BC_Flag, sizeof(nl->VelGrad_BC_Flag));
    std::memcpy(nl->VelGrad_BC, VelGrad_BC, sizeof(nl->VelGrad_BC));
    std::memcpy(nl->Stress_BC_Flag, Stress_BC_Flag, sizeof(nl->Stress_BC_Flag));
    std::memcpy(nl->Stress_BC, Stress_BC, sizeof(nl->Stress_BC));
    std::memcpy(nl->ElastConst_PhaseI, ElastConst_PhaseI, sizeof(nl->ElastConst_PhaseI));
    std::memcpy(nl->ElastConst_PhaseII, ElastConst_PhaseII, sizeof(nl->ElastConst_PhaseII));
    std::memcpy(nl->Slip_PhaseI, Slip_PhaseI, sizeof(nl->Slip_PhaseI));
    std::memcpy(nl->Slip_PhaseII, Slip_PhaseII, sizeof(nl->Slip_PhaseII));
    std::memcpy(nl->initial_ms, initial_ms, sizeof(nl->initial_ms));
    std::memcpy(nl->self, self, sizeof(nl->self));
    std::memcpy(nl->coplane, coplane, sizeof(nl->coplane));
    std::memcpy(nl->cross, cross, sizeof(nl->cross));
    std::memcpy(nl->glissile, glissile, sizeof(nl->glissile));
    std::memcpy(nl->hirth, hirth, sizeof(nl->hirth));
    std::memcpy(nl->lomer, lomer, sizeof(nl->lomer));
}

void copy9(ten2nd dst, const double *src)
{
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) dst[a][b] = src[3 * a + b];
}

// Sig, Eps, Edot, DisGrad and TranMat_xt2sa from the device.
void fields_to_globals()
{
    ten2nd *dst[5] = {Sig, Eps, Edot, DisGrad, TranMat_xt2sa};
    const int ids[5] = {VOCE_FIELD_SIG, VOCE_FIELD_EPS, VOCE_FIELD_EDOT, VOCE_FIELD_DISGRAD,
                        VOCE_FIELD_TRANMAT};
    for (int f = 0; f < 5; ++f)
        if (dst[f]) check(voce_rve_get_field(g_rve, ids[f], reinterpret_cast<double *>(dst[f])));
}

void macro_to_globals(const voce_increment &rec)
{
    s_vm = rec.s_vm;
    s_vm1 = rec.s_vm1;
    e_vm = rec.e_vm;
    d_vm = rec.d_vm;
    Err_e = rec.err_e;
    Err_s = rec.err_s;
    copy9(SigAvg, rec.sig_avg);
    copy9(SigAvg1, rec.sig_avg1);
    copy9(EpsAvg, rec.eps_avg);
    copy9(EdotAvg, rec.edot_avg);
    copy9(DisGradAvg, rec.disgrad_avg);
}

template <class T>
T *alloc_n(long long n)
{
    T *p = static_cast<T *>(std::malloc(sizeof(T) * (size_t)n));
    if (!p) {
        std::fprintf(stderr, "voce: host allocation of %lld elements failed\n", n);
        std::exit(1);
    }
    return p;
}

}  // namespace

extern "C" {

void voce_legacy_setup(void)
{
    if (rank != 0) return;
    voce_namelist nl;
    namelist_from_globals(&nl);
    const long long nv = (long long)CellDim[0] * CellDim[1] * CellDim[2];
    if (nv <= 0) {
        std::fprintf(stderr, "voce: CellDim not set\n");
        std::exit(1);
    }
    voce_slip sx[2];
    const voce_slip *sp[2] = {nullptr, nullptr};
    for (int p = 0; p < N_phases && p < 2; ++p) {
        if (Type_phases[p]) continue;
        check(voce_slip_read(p == 0 ? Slip_PhaseI : Slip_PhaseII, &sx[p]));
        sp[p] = &sx[p];
    }
    std::vector<double> eul((size_t)(3 * nv));
    grain_f = alloc_n<int>(nv);
    phase_f = alloc_n<int>(nv);
    check(voce_mesh_read(initial_ms, CellDim, eul.data(), grain_f, phase_f));
    voce_mesh mesh;
    std::memcpy(mesh.dims, CellDim, sizeof(mesh.dims));
    mesh.euler_deg = eul.data();
    mesh.grain = grain_f;
    mesh.phase = phase_f;
    const char *pe = std::getenv("VOCE_PRECISION");
    int prec = VOCE_PREC_FP64;
    if (pe && std::strcmp(pe, "mixed") == 0) prec = VOCE_PREC_MIXED;
    else if (pe && std::strcmp(pe, "mixed_ir") == 0) prec = VOCE_PREC_MIXED_IR;
    else if (pe && std::strcmp(pe, "mixed_nr32") == 0) prec = VOCE_PREC_MIXED_NR32;
    check(voce_rve_create(&nl, sp, &mesh, prec, &g_rve));

    // one rank holds the whole grid (init.c:647 with one process)
    Nxyz = (int)nv;
    WGT = 1.0 / Nxyz;
    long long n1 = 0;
    for (long long v = 0; v < nv; ++v) n1 += phase_f[v] == 1;
    Wgt_ph1 = (1.0 * (double)n1) / Nxyz;
    lnx = CellDim[0];
    lxs = 0;
    lnyt = CellDim[1];
    lyst = 0;
    lsize = (int)nv;
    voce_legacy_chg_basis(nullptr, nullptr, nullptr, nullptr, 0);
    Sig = alloc_n<ten2nd>(nv);
    Eps = alloc_n<ten2nd>(nv);
    Edot = alloc_n<ten2nd>(nv);
    DisGrad = alloc_n<ten2nd>(nv);
    TranMat_xt2sa = alloc_n<ten2nd>(nv);
    g_owned = true;
    fields_to_globals();
    check(voce_write_log_headers(fp_vm, fp_err));
}

void voce_legacy_evolution(void)
{
    if (rank != 0) return;
    if (!g_rve) {
        std::fprintf(stderr, "voce: Evolution() before SetupJob()\n");
        std::exit(1);
    }
    voce_namelist nl;
    check(voce_rve_get_namelist(g_rve, &nl));
    const bool print = nl.PrintControl[0] == 1 && nl.PrintControl[1] > 0;
    int done = voce_rve_increments_done(g_rve);
    while (done < N_steps) {
        // run up to the next increment whose fields are dumped
        int target = N_steps;
        if (print) {
            const int pc = nl.PrintControl[1];
            const int next = ((done + 1 + pc - 1) / pc) * pc;
            if (next < target) target = next;
        }
        check(voce_rve_run(g_rve, target - done));
        for (int k = done; k < target; ++k) check(voce_rve_write_log(g_rve, k, N_steps, fp_vm, fp_err));
        voce_increment rec;
        check(voce_rve_get_increment(g_rve, target - 1, &rec));
        macro_to_globals(rec);
        check(voce_rve_write_step_iout(g_rve, target, ""));
        done = target;
    }
    check(voce_rve_write_final_iout(g_rve, ""));
    fields_to_globals();
    std::printf("-------------Simulation ends----------------\n");
    std::printf("======================================\n\n");
}

void voce_legacy_destroy(void)
{
    if (g_rve) {
        voce_rve_destroy(g_rve);
        g_rve = nullptr;
    }
    if (g_owned) {
        ten2nd **fs[5] = {&Sig, &Eps, &Edot, &DisGrad, &TranMat_xt2sa};
        for (ten2nd **f : fs) {
            std::free(*f);
            *f = nullptr;
        }
        std::free(grain_f);
        std::free(phase_f);
        grain_f = phase_f = nullptr;
        g_owned = false;
    }
}

// chg_basis (kinematics.c:14-93): the Lebensohn-Tome basis B, and the
// changes between 6-vectors / 3x3 tensors and 6x6 / 3x3x3x3 tensors in it.
void voce_legacy_chg_basis(double *V6, double (*T2)[3], double (*C2)[6], double (*T4)[3][3][3], int opt)
{
    if (opt == 0) {
        const double r2 = 0.70710678118654744, r3 = 0.57735026918962584, r6 = 0.40824829046386304;
        std::memset(B, 0, sizeof(ten2nd) * 6);
        B[1][0][0] = -r6; B[1][1][1] = -r6; B[1][2][2] = 2. * r6;
        B[0][0][0] = -r2; B[0][1][1] = r2;
        B[2][1][2] = r2; B[2][2][1] = r2;
        B[3][0][2] = r2; B[3][2][0] = r2;
        B[4][0][1] = r2; B[4][1][0] = r2;
        B[5][0][0] = r3; B[5][1][1] = r3; B[5][2][2] = r3;
    } else if (opt == 1) {
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                T2[a][b] = 0.0;
                for (int i = 0; i < 6; ++i) T2[a][b] += V6[i] * B[i][a][b];
            }
    } else if (opt == 2) {
        for (int i = 0; i < 6; ++i) {
            V6[i] = 0.0;
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) V6[i] += T2[a][b] * B[i][a][b];
        }
    } else if (opt == 3) {
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b)
                for (int c = 0; c < 3; ++c)
                    for (int e = 0; e < 3; ++e) {
                        T4[a][b][c][e] = 0.0;
                        for (int i = 0; i < 6; ++i)
                            for (int j = 0; j < 6; ++j) T4[a][b][c][e] += C2[i][j] * B[i][a][b] * B[j][c][e];
                    }
    } else if (opt == 4) {
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j < 6; ++j) {
                C2[i][j] = 0.0;
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b)
                        for (int c = 0; c < 3; ++c)
                            for (int e = 0; e < 3; ++e) C2[i][j] += T4[a][b][c][e] * B[i][a][b] * B[j][c][e];
            }
    } else {
        std::fprintf(stderr, "chg_basis: Wrong option!!\n");
        std::exit(4);
    }
}

// EulerToTransMatrix (kinematics.c:187-240): Bunge angles <-> the
// sample->crystal matrix.  opt 1: matrix -> angles in degrees (with the
// reference's pi, evp.h:52); opt 2: angles in radians -> matrix.
void voce_legacy_euler(double *p_t1, double *p_ph, double *p_t2, double (*a)[3], int opt)
{
    const double pi_ref = 3.14159265359;
    if (opt == 1) {
        double ph = std::acos(a[2][2]), t1, t2;
        if (std::fabs(a[2][2]) > 0.9999) {
            t2 = 0.;
            t1 = std::atan2(a[0][1], a[0][0]);
        } else {
            const double sph = std::sin(ph);
            t1 = std::atan2(a[2][0] / sph, -1.0 * a[2][1] / sph);
            t2 = std::atan2(a[0][2] / sph, a[1][2] / sph);
        }
        ph *= 180. / pi_ref;
        t1 *= 180. / pi_ref;
        t2 *= 180. / pi_ref;
        *p_ph = ph;
        *p_t1 = t1;
        *p_t2 = t2;
    } else if (opt == 2) {
        const double t1 = *p_t1, ph = *p_ph, t2 = *p_t2;
        const double c1 = std::cos(t1), s1 = std::sin(t1), cp = std::cos(ph), sp = std::sin(ph);
        const double c2 = std::cos(t2), s2 = std::sin(t2);
        a[0][0] = c1 * c2 - s1 * s2 * cp;
        a[0][1] = s1 * c2 + c1 * s2 * cp;
        a[0][2] = s2 * sp;
        a[1][0] = -1.0 * c1 * s2 - s1 * c2 * cp;
        a[1][1] = -1.0 * s1 * s2 + c1 * c2 * cp;
        a[1][2] = c2 * sp;
        a[2][0] = s1 * sp;
        a[2][1] = -1.0 * c1 * sp;
        a[2][2] = cp;
    } else {
        std::fprintf(stderr, "Wrong option for EulerToTransMatrix()!!\n");
        std::exit(604);
    }
}

// the C-linkage names (voce_legacy.h)
void SetupJob(void) { voce_legacy_setup(); }
void Evolution(void) { voce_legacy_evolution(); }
void DestroyJob(void) { voce_legacy_destroy(); }
void chg_basis(double V6[6], double T2[3][3], double C2[6][6], double T4[3][3][3][3], int opt)
{
    voce_legacy_chg_basis(V6, T2, C2, T4, opt);
}
void EulerToTransMatrix(double *t1, double *ph, double *t2, double a[3][3], int opt)
{
    voce_legacy_euler(t1, ph, t2, a, opt);
}

}  // extern "C"
