/*
 * CPU restatement of the Voce EVP-FFT solver step (the parity oracle).
 * TEST INFRASTRUCTURE ONLY -- see evp_oracle.h for what it is and who may
 * use it.  Each function names the reference file:line it restates.  The
 * floating-point operations are evaluated in the reference's order (the
 * same association of products and sums), so that single-process results
 * match the reference built against the shims bit for bit.
 */
#include "evp_oracle.h"
#include "fft_core.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define NS 12                    /* NSYSMX, evpFlags.h:5 */
#define PI_REF 3.14159265359     /* evp.h:57 (not M_PI) */
#define TWO_PI_REF 6.28318530718 /* evp.h:58 */

/* --------------------------------------------------------------------- */
/* basis of Lebensohn & Tome (kinematics.c:14-174)                        */
/* --------------------------------------------------------------------- */
static double Bt[6][3][3];
static int Bt_ready = 0;

static void basis_init(void)
{
    /* kinematics.c:33-35 literal constants and :346-364 layout */
    const double r2 = 0.70710678118654744, r3 = 0.57735026918962584,
                 r6 = 0.40824829046386304;
    if (Bt_ready) return;
    memset(Bt, 0, sizeof(Bt));
    Bt[1][0][0] = -1. * r6; Bt[1][1][1] = -1. * r6; Bt[1][2][2] = 2. * r6;
    Bt[0][0][0] = -1. * r2; Bt[0][1][1] = r2;
    Bt[2][1][2] = r2; Bt[2][2][1] = r2;
    Bt[3][0][2] = r2; Bt[3][2][0] = r2;
    Bt[4][0][1] = r2; Bt[4][1][0] = r2;
    Bt[5][0][0] = r3; Bt[5][1][1] = r3; Bt[5][2][2] = r3;
    Bt_ready = 1;
}

void oracle_basis(double B[6][3][3]) { basis_init(); memcpy(B, Bt, sizeof(Bt)); }

/* chg_basis opt 1: 6-vector -> symmetric 3x3 (kinematics.c:366-372) */
static void v6_to_t(const double *v, double t[3][3], int nb)
{
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            double s = 0.0;
            for (int i = 0; i < nb; ++i) s += v[i] * Bt[i][a][b];
            t[a][b] = s;
        }
}

/* chg_basis opt 2: 3x3 -> 6-vector (kinematics.c:373-380) */
static void t_to_v6(double t[3][3], double *v, int nb)
{
    for (int i = 0; i < nb; ++i) {
        double s = 0.0;
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) s += t[a][b] * Bt[i][a][b];
        v[i] = s;
    }
}

/* chg_basis opt 3: 6x6 -> 3x3x3x3 (kinematics.c:381-388) */
static void c66_to_t4(const double *c, double *t4)
{
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b)
            for (int k = 0; k < 3; ++k)
                for (int l = 0; l < 3; ++l) {
                    double s = 0.0;
                    for (int i = 0; i < 6; ++i)
                        for (int j = 0; j < 6; ++j)
                            s += c[i * 6 + j] * Bt[i][a][b] * Bt[j][k][l];
                    t4[((a * 3 + b) * 3 + k) * 3 + l] = s;
                }
}

/* chg_basis opt 4: 3x3x3x3 -> 6x6 (kinematics.c:389-398) */
static void t4_to_c66(const double *t4, double *c)
{
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) {
            double s = 0.0;
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b)
                    for (int k = 0; k < 3; ++k)
                        for (int l = 0; l < 3; ++l)
                            s += t4[((a * 3 + b) * 3 + k) * 3 + l] * Bt[i][a][b] * Bt[j][k][l];
            c[i * 6 + j] = s;
        }
}

void oracle_chg_basis(double *v6, double *t2, double *c2, double *t4, int opt)
{
    basis_init();
    if (opt == 1) v6_to_t(v6, (double (*)[3])t2, 6);
    else if (opt == 2) t_to_v6((double (*)[3])t2, v6, 6);
    else if (opt == 3) c66_to_t4(c2, t4);
    else if (opt == 4) t4_to_c66(t4, c2);
}

void oracle_chg_basis5(double *v5, double *t2, double *c2, double *t4, int opt)
{
    (void)c2; (void)t4;
    basis_init();
    if (opt == 1) v6_to_t(v5, (double (*)[3])t2, 5);
    else if (opt == 2) t_to_v6((double (*)[3])t2, v5, 5);
}

/* --------------------------------------------------------------------- */
/* 6x6 inverse: Crout LU with implicit scaling (kinematics.c:282-424)     */
/* --------------------------------------------------------------------- */
static int lu_dcmp6(double a[6][6], int indx[6])
{
    const int n = 6;
    double vv[6];
    int imax = 0;
    for (int i = 0; i < n; ++i) {
        double big = 0.0, t;
        for (int j = 0; j < n; ++j)
            if ((t = fabs(a[i][j])) > big) big = t;
        if (fabs(big) < 1E-5) return 35; /* kinematics.c:306-309 exit(35) */
        vv[i] = 1.0 / big;
    }
    for (int j = 0; j < n; ++j) {
        for (int i = 0; i < j; ++i) {
            double sum = a[i][j];
            for (int k = 0; k < i; ++k) sum -= a[i][k] * a[k][j];
            a[i][j] = sum;
        }
        double big = 0.0, dum;
        for (int i = j; i < n; ++i) {
            double sum = a[i][j];
            for (int k = 0; k < j; ++k) sum -= a[i][k] * a[k][j];
            a[i][j] = sum;
            if ((dum = vv[i] * fabs(sum)) >= big) { big = dum; imax = i; }
        }
        if (j != imax) {
            for (int k = 0; k < n; ++k) {
                dum = a[imax][k]; a[imax][k] = a[j][k]; a[j][k] = dum;
            }
            vv[imax] = vv[j];
        }
        indx[j] = imax;
        if (fabs(a[j][j]) < 1E-5) a[j][j] = 1.0E-20; /* TINY, kinematics.c:341 */
        if (j != n - 1) {
            dum = 1.0 / (a[j][j]);
            for (int i = j + 1; i < n; ++i) a[i][j] *= dum;
        }
    }
    return 0;
}

static void lu_bksb6(double a[6][6], const int indx[6], double b[6])
{
    const int n = 6;
    int ii = -1; /* first row with a non-negligible entry (kinematics.c:383) */
    for (int i = 0; i < n; ++i) {
        int ip = indx[i];
        double sum = b[ip];
        b[ip] = b[i];
        if (ii >= 0)
            for (int j = ii; j <= i - 1; ++j) sum -= a[i][j] * b[j];
        else if (fabs(sum) > 1E-5) ii = i;
        b[i] = sum;
    }
    for (int i = n - 1; i >= 0; --i) {
        double sum = b[i];
        for (int j = i + 1; j < n; ++j) sum -= a[i][j] * b[j];
        b[i] = sum / a[i][i];
    }
}

static int lu_inv6(double c[6][6])
{
    int indx[6];
    double y[6][6], col[6];
    int rc = lu_dcmp6(c, indx);
    if (rc) return rc;
    for (int j = 0; j < 6; ++j) {
        for (int i = 0; i < 6; ++i) col[i] = 0.0;
        col[j] = 1.0;
        lu_bksb6(c, indx, col);
        for (int i = 0; i < 6; ++i) y[i][j] = col[i];
    }
    memcpy(c, y, sizeof(y));
    return 0;
}

int oracle_lu_inv66(double *c66) { return lu_inv6((double (*)[6])c66); }

/* --------------------------------------------------------------------- */
/* rotations (kinematics.c:187-280)                                       */
/* --------------------------------------------------------------------- */
static void euler_to_a(double t1, double ph, double t2, double a[3][3])
{
    double ct1 = cos(t1), st1 = sin(t1), cph = cos(ph), sph = sin(ph),
           ct2 = cos(t2), st2 = sin(t2);
    a[0][0] = ct1 * ct2 - st1 * st2 * cph;
    a[0][1] = st1 * ct2 + ct1 * st2 * cph;
    a[0][2] = st2 * sph;
    a[1][0] = -1.0 * ct1 * st2 - st1 * ct2 * cph;
    a[1][1] = -1.0 * st1 * st2 + ct1 * ct2 * cph;
    a[1][2] = ct2 * sph;
    a[2][0] = st1 * sph;
    a[2][1] = -1.0 * ct1 * sph;
    a[2][2] = cph;
}

void oracle_euler_to_transmatrix(double t1, double ph, double t2, double *a9)
{
    euler_to_a(t1, ph, t2, (double (*)[3])a9);
}

/* Ten4thTransform opt 2: c1_ijkl = a_mi a_nj a_pk a_ql c2_mnpq (kinematics.c:243-280) */
static void ten4_back(double *c1, double a[3][3], const double *c2)
{
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            for (int k = 0; k < 3; ++k)
                for (int l = 0; l < 3; ++l) {
                    double s = 0.0;
                    for (int m = 0; m < 3; ++m)
                        for (int n = 0; n < 3; ++n)
                            for (int p = 0; p < 3; ++p)
                                for (int q = 0; q < 3; ++q)
                                    s += a[m][i] * a[n][j] * a[p][k] * a[q][l] *
                                         c2[((m * 3 + n) * 3 + p) * 3 + q];
                    c1[((i * 3 + j) * 3 + k) * 3 + l] = s;
                }
}

/* --------------------------------------------------------------------- */
/* flow rule: StrainRate_eval (constitutive.c:126-194)                    */
/* --------------------------------------------------------------------- */
static void strain_rate(int nsys, const double *stress, const double *sc,
                        const double *tau, const double *nsrs,
                        const double *gam0, double *edot, double d[6][6],
                        double *gamdot, double *taux)
{
    double rss1[NS], rss2[NS];
    for (int i = 0; i < nsys; ++i) {
        const double *s = sc + 5 * i;
        double r = s[0] * stress[0] + s[1] * stress[1] + s[2] * stress[2] +
                   s[3] * stress[3] + s[4] * stress[4];
        double x = 0.0; /* xkin: always 0 (init.c:793) */
        int isign = ((r - x) < 0) ? 1 : 0;
        r = (r - x) / tau[2 * i + isign];
        rss1[i] = gam0[i] * nsrs[i] * fabs(pow(r, nsrs[i] - 1.)) / tau[2 * i + isign];
        rss2[i] = gam0[i] * fabs(pow(r, nsrs[i])) * ((double)(2 * (r > 0) - 1));
        if (gamdot) gamdot[i] = rss2[i];
        if (taux) taux[i] = rss1[i];
    }
    for (int i = 0; i < 5; ++i) {
        double e = 0.;
        for (int j = 0; j < nsys; ++j) e += sc[5 * j + i] * rss2[j];
        edot[i] = e;
    }
    edot[5] = 0.0;
    for (int i = 0; i < 5; ++i)
        for (int j = 0; j < 5; ++j) {
            double s = 0.0;
            for (int k = 0; k < nsys; ++k) s += sc[5 * k + i] * sc[5 * k + j] * rss1[k];
            d[i][j] = s;
        }
    for (int i = 0; i < 6; ++i) { d[i][5] = 0.0; d[5][i] = 0.0; }
}

void oracle_strain_rate(int nsys, const double *stress6, const double *sch60,
                        const double *tau24, const double *nsrs,
                        const double *gam0, double *edot6, double *d_edot36,
                        double *gamdot12, double *taux12)
{
    strain_rate(nsys, stress6, sch60, tau24, nsrs, gam0, edot6,
                (double (*)[6])d_edot36, gamdot12, taux12);
}

/* --------------------------------------------------------------------- */
/* per-voxel stress update: UpdateStress body (evolution.c:25-158)        */
/* --------------------------------------------------------------------- */
typedef struct {
    double sig[3][3], edot[3][3];
    double svm, evm, conv_s, conv_e;
    int iters;
} nr_out;

static int update_stress_voxel(int nsys, const double *cgr, const double *c066,
                               double sigin[3][3], double epsin[3][3],
                               double dg[3][3], const double *sc,
                               const double *tau, const double *nsrs,
                               const double *gam0, double dt, double *gamdot,
                               double *taux, nr_out *o)
{
    double sg66[6][6], aux[3][3], strain_aux[3][3];
    double xl6[6], sig6[6], eps6[6], strain6[6], edot6[6], d66[6][6];
    double tot_eps[6] = {0}, sig6_old[6], res[6], jac[6][6];   /* set by the first Newton pass, which always runs */
    memcpy(sg66, cgr, sizeof(sg66));
    int rc = lu_inv6(sg66);
    if (rc) return rc;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b)
            strain_aux[a][b] = (dg[a][b] + dg[b][a]) / 2.0;
    t_to_v6(sigin, xl6, 6);
    t_to_v6(sigin, sig6, 6);
    t_to_v6(epsin, eps6, 6);
    t_to_v6(strain_aux, strain6, 6);
    double signorm = 0.0;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) signorm += sigin[a][b] * sigin[a][b];
    signorm = sqrt(signorm);

    const double erroral = 1E-7;
    int iterl = 0;
    double erral = 10 * erroral, conv_e = 0.0, conv_s = 0.0;
    while ((iterl < 100) && (fabs(erral) > fabs(erroral))) {
        iterl++;
        for (int i = 0; i < 6; ++i) sig6_old[i] = sig6[i];
        strain_rate(nsys, sig6, sc, tau, nsrs, gam0, edot6, d66, gamdot, taux);
        for (int i = 0; i < 6; ++i) {
            tot_eps[i] = eps6[i] + edot6[i] * dt;
            for (int j = 0; j < 6; ++j) tot_eps[i] += sg66[i][j] * sig6[j];
        }
        for (int i = 0; i < 6; ++i) {
            res[i] = sig6[i] - xl6[i];
            for (int j = 0; j < 6; ++j) res[i] += c066[i * 6 + j] * (tot_eps[j] - strain6[j]);
        }
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j < 6; ++j) {
                jac[i][j] = (double)(i == j);
                for (int k = 0; k < 6; ++k)
                    jac[i][j] += c066[i * 6 + k] * (sg66[k][j] + d66[k][j] * dt);
            }
        rc = lu_inv6(jac);
        if (rc) return rc;
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j < 6; ++j) sig6[i] -= jac[i][j] * res[j];
        double cnr = 0.0;
        conv_e = 0.0;
        conv_s = 0.0;
        for (int i = 0; i < 6; ++i) {
            cnr += (sig6[i] - sig6_old[i]) * (sig6[i] - sig6_old[i]);
            conv_e += (tot_eps[i] - strain6[i]) * (tot_eps[i] - strain6[i]);
            conv_s += (sig6[i] - xl6[i]) * (sig6[i] - xl6[i]);
        }
        erral = sqrt(cnr) / signorm;
        conv_e = sqrt(conv_e);
        conv_s = sqrt(conv_s);
    }
    double tot_e[3][3];
    v6_to_t(sig6, o->sig, 6);
    v6_to_t(edot6, o->edot, 6);
    v6_to_t(tot_eps, tot_e, 6);
    double tr = o->sig[0][0] + o->sig[1][1] + o->sig[2][2];
    double svm = 0.0;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            aux[a][b] = (o->sig[a][b] + o->sig[b][a]) / 2. - (double)(a == b) * tr / 3.0;
        }
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) svm += aux[a][b] * aux[a][b];
    o->svm = sqrt(3. / 2. * svm);
    tr = tot_e[0][0] + tot_e[1][1] + tot_e[2][2];
    double evm = 0.0;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b)
            aux[a][b] = (tot_e[a][b] + tot_e[b][a]) / 2. - (double)(a == b) * tr / 3.0;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) evm += aux[a][b] * aux[a][b];
    o->evm = sqrt(2. / 3. * evm);
    o->conv_s = conv_s;
    o->conv_e = conv_e;
    o->iters = iterl;
    return 0;
}

int oracle_update_stress_voxel(int nsys, const double *cgr36,
                               const double *c066, const double *sig9,
                               const double *eps9, const double *disgrad9,
                               const double *sch60, const double *tau24,
                               const double *nsrs, const double *gam0,
                               double dt, double *sig_out9, double *edot_out9,
                               double *gamdot12, double *svm, double *evm,
                               double *conv_s, double *conv_e)
{
    basis_init();
    nr_out o;
    double s[3][3], e[3][3], d[3][3];
    memcpy(s, sig9, sizeof(s));
    memcpy(e, eps9, sizeof(e));
    memcpy(d, disgrad9, sizeof(d));
    int rc = update_stress_voxel(nsys, cgr36, c066, s, e, d, sch60, tau24, nsrs,
                                 gam0, dt, gamdot12, NULL, &o);
    if (rc) return -rc;
    memcpy(sig_out9, o.sig, sizeof(o.sig));
    memcpy(edot_out9, o.edot, sizeof(o.edot));
    *svm = o.svm; *evm = o.evm; *conv_s = o.conv_s; *conv_e = o.conv_e;
    return o.iters;
}

/* --------------------------------------------------------------------- */
/* Voce hardening for one voxel: harden() body (constitutive.c:261-305)   */
/* --------------------------------------------------------------------- */
static void harden_voxel(int nsys, const double *hard, const double *tau3,
                         const double *thet2, double dt, const double *gamdot,
                         double *gamacum, double *gtot, double *crss,
                         double *trial)
{
    double gamtot = *gamacum, deltgam = 0.0;
    for (int i = 0; i < nsys; ++i) gtot[i] = gtot[i] + (gamdot[i]) * dt;
    for (int i = 0; i < nsys; ++i) deltgam += fabs(gamdot[i]) * dt;
    for (int i = 0; i < nsys; ++i) {
        double dtau = 0.;
        for (int j = 0; j < nsys; ++j) dtau += hard[i * NS + j] * fabs(gamdot[j]) * dt;
        double tau0 = tau3[3 * i + 0], tau1 = tau3[3 * i + 2];
        double th0 = thet2[2 * i + 0], th1 = thet2[2 * i + 1];
        double tiny = 1.E-4 * tau0, voce = 0.0;
        if (fabs(th0) > tiny) {
            voce = th1 * deltgam;
            if (fabs(tau1) > tiny) {
                double fact = fabs(th0 / tau1);
                double exp_ini = exp(-1.0 * gamtot * fact);
                double exp_del = exp(-1.0 * deltgam * fact);
                voce += -1. * (fact * tau1 - th1) / fact * exp_ini * (exp_del - 1.0) -
                        th1 / fact * exp_ini *
                            (exp_del * ((gamtot + deltgam) * fact + 1.0) - (gamtot * fact + 1.0));
            }
        }
        crss[2 * i + 0] += dtau * voce / deltgam;
        crss[2 * i + 1] += dtau * voce / deltgam;
        if (trial) {
            trial[2 * i + 0] = crss[2 * i + 0];
            trial[2 * i + 1] = crss[2 * i + 1];
        }
    }
    *gamacum = gamtot + deltgam;
}

void oracle_harden_voxel(int nsys, const double *hard144, const double *tau36,
                         const double *thet24, double dt,
                         const double *gamdot12, double *gamacum,
                         double *gammatotal12, double *crss24)
{
    harden_voxel(nsys, hard144, tau36, thet24, dt, gamdot12, gamacum,
                 gammatotal12, crss24, NULL);
}

/* Orientation() (constitutive.c:117-169) */
static void orientation(double tran[3][3], double rot[3][3])
{
    double w[3] = {rot[2][1], rot[0][2], rot[1][0]};
    double wn = 0.0;
    for (int i = 0; i < 3; ++i) wn += w[i] * w[i];
    wn = sqrt(wn);
    double wt = tan(wn / 2.0);
    if (fabs(wn) < 1E-6) wn = 1.0;
    for (int i = 0; i < 3; ++i) w[i] *= wt / wn;
    double om[3][3] = {{0., -1. * w[2], w[1]}, {w[2], 0., -1. * w[0]}, {-1. * w[1], w[0], 0.}};
    double om2[3][3], tn[3][3];
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            double s = 0.0;
            for (int i = 0; i < 3; ++i) s += om[a][i] * om[i][b];
            om2[a][b] = s;
        }
    wt = wt * wt;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b)
            rot[a][b] = (double)(a == b) + 2. * (om[a][b] + om2[a][b]) / (1. + wt);
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            double s = 0.0;
            for (int i = 0; i < 3; ++i) s += rot[a][i] * tran[i][b];
            tn[a][b] = s;
        }
    memcpy(tran, tn, sizeof(tn));
}

void oracle_orientation(double *tran9, const double *rot9)
{
    double r[3][3];
    memcpy(r, rot9, sizeof(r));
    orientation((double (*)[3])tran9, r);
}

/* --------------------------------------------------------------------- */
/* job state                                                              */
/* --------------------------------------------------------------------- */
struct oracle_job {
    int nthreads;
    /* namelist variables (io.c:25-52) */
    int CellDim[3], N_phases, Type_phases[2], N_steps, Update_Flag, Hard_Flag,
        Tex_Flag, IterMax, PrintControl[2], VelGrad_BC_Flag[6], Stress_BC_Flag[6];
    double TimeStep, Err, VelGrad_BC[6], Stress_BC[6], ElastConst[2][4];
    char Slip[2][100], initial_ms[100];
    double self_[2], coplane[2], cross_[2], glissile[2], hirth[2], lomer[2];
    /* material */
    int nsys[2];
    double nsrs[2][NS], gam0[2][NS], tau[2][NS][3], thet[2][NS][2];
    double bn[2][NS][3], bb[2][NS][3], schm_xt[2][NS][5], hard[2][NS * NS];
    double cijkl[2][81];
    /* grid and reference medium */
    long nv;
    int Nxyz;
    double WGT, Wgt_ph1, C066[36], S066[36], C0[81], S0[81];
    /* boundary conditions (init.c:713-745) */
    double Udot[3][3], Udot_s[3][3], Udot_a[3][3], d_vm, Scauchy[3][3];
    int CREEP_FLAG;
    /* fields */
    int *grain, *phase;
    double *gn;     /* 3 per voxel: unit frequency vector g/|g| */
    double *GAMMA;  /* 81 per voxel */
    double *Cgr, *Tm, *Sch, *Sig, *Eps, *Edot, *DG, *VG, *fluct;
    double *crss, *trial, *gamdot, *taux, *gtot, *gamacum, *SVM, *EVM;
    double *kr, *ki, *fft, *red_s, *red_e;
    /* macro state (evolution.c:265-290 locals and evp.h globals) */
    double DisGradAvg[3][3], dDisGradAvg[3][3], dDisGradAvg_acum[3][3],
        DisGradAvg_t[3][3], DisGradAvg_actual[3][3], SigAvg[3][3],
        SigAvg1[3][3], EpsAvg[3][3], EdotAvg[3][3], VelGradAvg[3][3];
    double s_vm, s_vm1, e_vm, Err_e, Err_s;
    int iter_total, istep;
    /* logs */
    oracle_incr *incr;
    int n_incr, cap_incr;
    double *it_e, *it_s, *it_v;
    int *it_start, it_n, it_cap;
    FILE *trace;
    long trace_n;
};

static void tr_d(oracle_job *j, double v)
{
    ++j->trace_n;
    if (j->trace) fprintf(j->trace, "%ld d %.17g\n", j->trace_n, v);
}

static void tr_i(oracle_job *j, int v)
{
    ++j->trace_n;
    if (j->trace) fprintf(j->trace, "%ld i %d\n", j->trace_n, v);
}

/* ---- readers ---------------------------------------------------------- */
typedef struct { const char *name; int type; int len; void *ptr; } nl_var;

static void join_path(char *out, size_t n, const char *dir, const char *name)
{
    if (name[0] == '/' || !dir[0]) snprintf(out, n, "%s", name);
    else snprintf(out, n, "%s/%s", dir, name);
}

/* GetNameList (io.c:54-122): fgets of 80, '#' or empty lines skipped, a line
 * whose first token is missing ends the read, case-sensitive keys, unknown
 * keys ignored, a repeated key keeps its first values. */
static int read_namelist(oracle_job *j, const char *path, char *err)
{
    nl_var vars[] = {
        {"CellDim", 0, 3, j->CellDim}, {"N_phases", 0, 1, &j->N_phases},
        {"Type_phases", 0, 2, j->Type_phases}, {"TimeStep", 1, 1, &j->TimeStep},
        {"N_steps", 0, 1, &j->N_steps}, {"Update_Flag", 0, 1, &j->Update_Flag},
        {"Hard_Flag", 0, 1, &j->Hard_Flag}, {"Tex_Flag", 0, 1, &j->Tex_Flag},
        {"IterMax", 0, 1, &j->IterMax}, {"PrintControl", 0, 2, j->PrintControl},
        {"Err", 1, 1, &j->Err}, {"VelGrad_BC_Flag", 0, 6, j->VelGrad_BC_Flag},
        {"VelGrad_BC", 1, 6, j->VelGrad_BC}, {"Stress_BC_Flag", 0, 6, j->Stress_BC_Flag},
        {"Stress_BC", 1, 6, j->Stress_BC}, {"ElastConst_PhaseI", 1, 4, j->ElastConst[0]},
        {"ElastConst_PhaseII", 1, 4, j->ElastConst[1]}, {"Slip_PhaseI", 2, 1, j->Slip[0]},
        {"Slip_PhaseII", 2, 1, j->Slip[1]}, {"initial_ms", 2, 1, j->initial_ms},
        {"self", 1, 2, j->self_}, {"coplane", 1, 2, j->coplane}, {"cross", 1, 2, j->cross_},
        {"glissile", 1, 2, j->glissile}, {"hirth", 1, 2, j->hirth}, {"lomer", 1, 2, j->lomer},
    };
    const int nvars = (int)(sizeof(vars) / sizeof(vars[0]));
    int seen[32] = {0};
    FILE *fp = fopen(path, "r");
    if (!fp) { snprintf(err, 256, "cannot open namelist %s", path); return 1; }
    char buf[80];
    while (1) {
        if (!fgets(buf, 80, fp)) break;
        if (feof(fp)) break;
        if (buf[0] == '#' || buf[0] == '\n') continue;
        char *tok = strtok(buf, " \t\n");
        if (!tok) break;
        for (int k = 0; k < nvars; ++k) {
            if (strcmp(tok, vars[k].name) != 0) continue;
            if (!seen[k]) {
                seen[k] = 1;
                for (int q = 0; q < vars[k].len; ++q) {
                    tok = strtok(NULL, ", \t\n");
                    if (!tok) continue;
                    if (vars[k].type == 0) ((int *)vars[k].ptr)[q] = (int)atol(tok);
                    else if (vars[k].type == 1) ((double *)vars[k].ptr)[q] = atof(tok);
                    else strcpy((char *)vars[k].ptr + q, tok);
                }
            }
            break;
        }
    }
    fclose(fp);
    return 0;
}

/* PlasticInit (init.c:51-391): fixed-position reads of the .sx file */
static int read_sx(oracle_job *j, const char *path, int ph, char *err)
{
    FILE *fp = fopen(path, "r");
    if (!fp) { snprintf(err, 256, "cannot open sx %s", path); return 1; }
    char buf[80] = {0};
    char xs[80];
    int nmax = 0, nmodes = 0, imode[16] = {0};
    double ax[3];
#define L() do { if (!fgets(buf, 80, fp)) buf[0] = 0; } while (0)
    L(); L(); sscanf(buf, "%s", xs); L(); L(); L(); sscanf(buf, "%lf %lf %lf", ax, ax + 1, ax + 2);
    L(); L(); L(); sscanf(buf, "%d", &nmax); L(); L(); L(); sscanf(buf, "%d", &nmodes);
    if (nmodes < 1 || nmodes > 16) { fclose(fp); snprintf(err, 256, "bad N_modes"); return 1; }
    L(); L();
    for (int i = 0; i < nmodes; ++i) { L(); sscanf(buf, "%d", &imode[i]); }
    L();
    int mx = 0, nsmx = 0;
    double nrsx = 0, gamd0x = 0, twshx, tau0xf = 0, tau0xb = 0, tau1x = 0, thet0 = 0, thet1 = 0, hs, hl;
    int isect;
    for (int i = 0; i < nmax; ++i) {
        L();
        sscanf(buf, "%*s %*s %d %*s", &mx);
        int match = 0;
        for (int q = 0; q < nmodes; ++q) if (mx == imode[q]) { match = 1; break; }
        if (match) {
            L(); L(); sscanf(buf, "%d %lf %lf %lf %d", &nsmx, &nrsx, &gamd0x, &twshx, &isect);
            if (nsmx > NS) { fclose(fp); snprintf(err, 256, "nsmx > 12"); return 1; }
            j->nsys[ph] = nsmx;
            L(); L(); sscanf(buf, "%lf %lf %lf %lf %lf", &tau0xf, &tau0xb, &tau1x, &thet0, &thet1);
            L(); L(); sscanf(buf, "%lf %lf", &hs, &hl);
            L();
            if (tau1x < 1.E-6) { tau1x = 1.E-6; thet0 = thet1; } /* init.c:141-144 */
            for (int s = 0; s < nsmx; ++s) {
                j->nsrs[ph][s] = nrsx;
                j->gam0[ph][s] = gamd0x;
                j->tau[ph][s][0] = tau0xf;
                j->tau[ph][s][1] = tau0xb;
                j->tau[ph][s][2] = tau1x;
                j->thet[ph][s][0] = thet0;
                j->thet[ph][s][1] = thet1;
                L();
                sscanf(buf, "%lf %lf %lf %lf %lf %lf", &j->bn[ph][s][0], &j->bn[ph][s][1],
                       &j->bn[ph][s][2], &j->bb[ph][s][0], &j->bb[ph][s][1], &j->bb[ph][s][2]);
            }
        } else {
            for (int q = 0; q < 24; ++q) L();
        }
    }
#undef L
    fclose(fp);
    /* normalise, check orthogonality, Schmid in crystal axes (init.c:189-226) */
    for (int s = 0; s < j->nsys[ph]; ++s) {
        double *n = j->bn[ph][s], *b = j->bb[ph][s], nrm;
        nrm = sqrt(pow(n[0], 2.0) + pow(n[1], 2.0) + pow(n[2], 2.0));
        for (int q = 0; q < 3; ++q) n[q] /= nrm;
        nrm = sqrt(pow(b[0], 2.0) + pow(b[1], 2.0) + pow(b[2], 2.0));
        for (int q = 0; q < 3; ++q) b[q] /= nrm;
        nrm = 0.0;
        for (int q = 0; q < 3; ++q) nrm += n[q] * b[q];
        if (nrm > 1E-3) { snprintf(err, 256, "slip system not orthogonal"); return 1; }
        double a[3][3];
        for (int p = 0; p < 3; ++p)
            for (int q = 0; q < 3; ++q) a[p][q] = (n[p] * b[q] + n[q] * b[p]) / 2.0;
        t_to_v6(a, j->schm_xt[ph][s], 5);
    }
    /* latent hardening table (init.c:283-381): which coefficient couples
     * which pair of the 12 systems; lower triangle by symmetry */
    static const char tbl[12][12] = {
        "SCCHGLXGGHLG", " SCGXGGHLLHG", "  SLGHGLHGGX", "   SCCHLGXGG",
        "    SCLHGGHL", "     SGGXGLH", "      SCCHGL", "       SCGXG",
        "        SLGH", "         SCC", "          SC", "           S"};
    double *H = j->hard[ph];
    for (int p = 0; p < 12; ++p)
        for (int q = p; q < 12; ++q) {
            double v = 0.0;
            switch (tbl[p][q]) {
            case 'S': v = j->self_[ph]; break;
            case 'C': v = j->coplane[ph]; break;
            case 'X': v = j->cross_[ph]; break;
            case 'G': v = j->glissile[ph]; break;
            case 'H': v = j->hirth[ph]; break;
            case 'L': v = j->lomer[ph]; break;
            }
            H[p * NS + q] = v;
        }
    for (int p = 1; p < 12; ++p)
        for (int q = 0; q < p; ++q) H[p * NS + q] = H[q * NS + p];
    return 0;
}

/* ElastStiffnessMatrix (init.c:9-49): cubic C_ijkl from c11, c12, c44 */
static void cubic_stiffness(const double *ec, double *c)
{
    memset(c, 0, 81 * sizeof(double));
#define CI(i, jj, k, l) c[((((i) - 1) * 3 + (jj) - 1) * 3 + (k) - 1) * 3 + (l) - 1]
    for (int i = 1; i <= 3; ++i) CI(i, i, i, i) = ec[0];
    for (int i = 1; i <= 3; ++i)
        for (int k = 1; k <= 3; ++k)
            if (i != k) {
                CI(i, i, k, k) = ec[1];
                CI(i, k, i, k) = ec[2];
                CI(i, k, k, i) = ec[2];
            }
#undef CI
}

/* ---- setup (SetupJob, init.c:617-828) ---------------------------------- */
static void alloc_fields(oracle_job *j)
{
    long n = j->nv;
#define A(p, k) j->p = (double *)calloc((size_t)n * (k), sizeof(double))
    A(gn, 3); A(GAMMA, 81); A(Cgr, 36); A(Tm, 9); A(Sch, 60); A(Sig, 9); A(Eps, 9);
    A(Edot, 9); A(DG, 9); A(VG, 9); A(fluct, 9); A(crss, 24); A(trial, 24);
    A(gamdot, 12); A(taux, 12); A(gtot, 12); A(gamacum, 1); A(SVM, 1); A(EVM, 1);
    A(kr, 9); A(ki, 9); A(fft, 2); A(red_s, 1); A(red_e, 1);
#undef A
    j->grain = (int *)calloc((size_t)n, sizeof(int));
    j->phase = (int *)calloc((size_t)n, sizeof(int));
}

static void update_schmid(oracle_job *j)
{
    /* kinematics.c:426-459 */
#pragma omp parallel for schedule(static) num_threads(j->nthreads)
    for (long v = 0; v < j->nv; ++v) {
        int ph = j->phase[v] - 1;
        if (j->Type_phases[ph]) continue;
        double (*T)[3] = (double (*)[3])(j->Tm + 9 * v);
        for (int s = 0; s < j->nsys[ph]; ++s) {
            double a[3][3], ar[3][3];
            v6_to_t(j->schm_xt[ph][s], a, 5);
            for (int p = 0; p < 3; ++p)
                for (int q = 0; q < 3; ++q) {
                    double acc = 0.0;
                    for (int pp = 0; pp < 3; ++pp)
                        for (int qq = 0; qq < 3; ++qq) acc += T[p][pp] * T[q][qq] * a[pp][qq];
                    ar[p][q] = acc;
                }
            t_to_v6(ar, j->Sch + 60 * v + 5 * s, 5);
        }
    }
}

static int setup(oracle_job *j, const char *nlpath, char *err)
{
    char dir[512] = {0}, p[1024];
    const char *sl = strrchr(nlpath, '/');
    if (sl) { memcpy(dir, nlpath, (size_t)(sl - nlpath)); }
    if (read_namelist(j, nlpath, err)) return 1;
    j->Nxyz = j->CellDim[0] * j->CellDim[1] * j->CellDim[2];
    j->nv = j->Nxyz;
    j->WGT = 1. / j->Nxyz;
    if (j->nv <= 0 || j->N_phases < 1 || j->N_phases > 2) { snprintf(err, 256, "bad dims/phases"); return 1; }
    alloc_fields(j);

    /* k-space (init.c:660-677) */
    for (int x = 0; x < j->CellDim[0]; ++x)
        for (int y = 0; y < j->CellDim[1]; ++y)
            for (int z = 0; z < j->CellDim[2]; ++z) {
                long v = ((long)x * j->CellDim[1] + y) * j->CellDim[2] + z;
                double t[3];
                t[0] = (double)(x) * (double)(1.0 / j->CellDim[0]);
                t[1] = (double)(y) * (double)(1.0 / j->CellDim[1]);
                t[2] = (double)(z) * (double)(1.0 / j->CellDim[2]);
                for (int m = 0; m < 3; ++m) { t[m] -= round(t[m]); t[m] *= TWO_PI_REF; }
                double g2 = sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
                if (x + y + z == 0) { g2 = 1.0; t[0] = t[1] = t[2] = 0.0; }
                for (int m = 0; m < 3; ++m) j->gn[3 * v + m] = t[m] * (1. / g2);
            }

    basis_init();
    int nsolid = 0;
    for (int ph = 0; ph < j->N_phases; ++ph) {
        if (j->Type_phases[ph]) continue;
        ++nsolid;
        if (nsolid > 1) { snprintf(err, 256, "more than one crystalline phase"); return 1; }
        cubic_stiffness(j->ElastConst[ph], j->cijkl[ph]);
        join_path(p, sizeof(p), dir, j->Slip[ph]);
        if (read_sx(j, p, ph, err)) return 1;
    }

    /* InitMicroStruct (init.c:393-483) */
    join_path(p, sizeof(p), dir, j->initial_ms);
    FILE *fp = fopen(p, "r");
    if (!fp) { snprintf(err, 256, "cannot open mesh %s", p); return 1; }
    char buf[80];
    int nph1 = 0;
    double c066l[36] = {0};
    for (long v = 0; v < j->nv; ++v) {
        double ph, th, om;
        int ii, jj, kk, jgr, jph;
        if (!fgets(buf, 80, fp) ||
            sscanf(buf, "%lf %lf %lf %d %d %d %d %d", &ph, &th, &om, &ii, &jj, &kk, &jgr, &jph) != 8) {
            fclose(fp); snprintf(err, 256, "mesh read error at voxel %ld", v); return 1;
        }
        long idx = ((long)(ii - 1) * j->CellDim[1] + jj - 1) * j->CellDim[2] + kk - 1;
        if (idx != v || jph < 1 || jph > j->N_phases) {
            fclose(fp); snprintf(err, 256, "mesh index mismatch at voxel %ld", v); return 1;
        }
        if (jph == 1) nph1++;
        j->grain[v] = jgr;
        j->phase[v] = jph;
        if (!j->Type_phases[jph - 1]) {
            ph *= PI_REF / 180.; th *= PI_REF / 180.; om *= PI_REF / 180.;
            double a[3][3], c4[81];
            euler_to_a(ph, th, om, a);
            for (int q = 0; q < 3; ++q)
                for (int r = 0; r < 3; ++r) j->Tm[9 * v + 3 * q + r] = a[r][q];
            ten4_back(c4, a, j->cijkl[jph - 1]);
            t4_to_c66(c4, j->Cgr + 36 * v);
            for (int q = 0; q < 36; ++q) c066l[q] += j->Cgr[36 * v + q];
        }
    }
    fclose(fp);
    tr_i(j, nph1);
    j->Wgt_ph1 = (1.0 * (double)nph1) / j->Nxyz;
    for (int q = 0; q < 36; ++q) { tr_d(j, c066l[q]); j->C066[q] = c066l[q] * j->WGT; }
    memcpy(j->S066, j->C066, sizeof(j->S066));
    if (lu_inv6((double (*)[6])j->S066)) { snprintf(err, 256, "singular C066"); return 1; }
    c66_to_t4(j->C066, j->C0);
    c66_to_t4(j->S066, j->S0);

    /* boundary conditions (init.c:713-745) */
    const double *vb = j->VelGrad_BC;
    int sf = j->VelGrad_BC_Flag[0] + j->VelGrad_BC_Flag[1] + j->VelGrad_BC_Flag[2];
    if (sf == 2) { snprintf(err, 256, "two deviatoric velgrad components"); return 1; }
    double U[3][3] = {{vb[0], vb[5], vb[4]}, {vb[5], vb[1], vb[3]}, {vb[4], vb[3], vb[2]}};
    memcpy(j->Udot, U, sizeof(U));
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            j->Udot_s[a][b] = (U[a][b] + U[b][a]) / 2.;
            j->Udot_a[a][b] = (U[a][b] - U[b][a]) / 2.;
        }
    double d6[6], dev[3][3];
    t_to_v6(j->Udot_s, d6, 6);
    v6_to_t(d6, dev, 5);
    j->d_vm = 0.0;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) j->d_vm += pow(dev[a][b], 2.0);
    j->d_vm = sqrt(2. / 3. * j->d_vm);
    for (int i = 0; i < 6; ++i)
        if ((j->Stress_BC_Flag[i] * j->VelGrad_BC_Flag[i] != 0) ||
            ((j->Stress_BC_Flag[i] + j->VelGrad_BC_Flag[i]) != 1)) {
            snprintf(err, 256, "inconsistent boundary conditions"); return 1;
        }
    j->CREEP_FLAG = 0;
    for (int i = 0; i < 6; ++i) j->CREEP_FLAG += j->Stress_BC_Flag[i];
    j->CREEP_FLAG /= 6;
    const double *sb = j->Stress_BC;
    double S[3][3] = {{sb[0], sb[5], sb[4]}, {sb[5], sb[1], sb[3]}, {sb[4], sb[3], sb[2]}};
    memcpy(j->Scauchy, S, sizeof(S));

    /* hardening state (init.c:747-796); gamacum and gammatotal are left
     * uninitialised by the reference (malloc): they start at zero here */
    for (long v = 0; v < j->nv; ++v) {
        int ph = j->phase[v] - 1;
        if (j->Type_phases[ph]) continue;
        for (int s = 0; s < j->nsys[ph]; ++s) {
            j->crss[24 * v + 2 * s] = j->tau[ph][s][0];
            j->crss[24 * v + 2 * s + 1] = j->tau[ph][s][1];
            j->trial[24 * v + 2 * s] = j->tau[ph][s][0];
            j->trial[24 * v + 2 * s + 1] = j->tau[ph][s][1];
        }
    }

    /* InitFields (init.c:486-544) */
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            j->DisGradAvg[a][b] = j->Udot[a][b] * j->TimeStep;
            j->dDisGradAvg[a][b] = 0.0;
            j->dDisGradAvg_acum[a][b] = 0.0;
        }
#pragma omp parallel for schedule(static) num_threads(j->nthreads)
    for (long v = 0; v < j->nv; ++v) {
        int ph = j->phase[v] - 1;
        double *sg = j->Sig + 9 * v;
        if (!j->Type_phases[ph]) {
            double cg[81];
            c66_to_t4(j->Cgr + 36 * v, cg);
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) {
                    double s = 0.0;
                    for (int k = 0; k < 3; ++k)
                        for (int l = 0; l < 3; ++l) s += cg[((a * 3 + b) * 3 + k) * 3 + l] * j->DisGradAvg[k][l];
                    if (j->CREEP_FLAG == 1) s += j->Scauchy[a][b];
                    sg[3 * a + b] = s;
                }
        }
    }
    j->e_vm = j->d_vm * j->TimeStep;

    /* CalcGAMMA (init.c:546-615) */
#pragma omp parallel for schedule(static) num_threads(j->nthreads)
    for (long v = 0; v < j->nv; ++v) {
        double *G = j->GAMMA + 81 * v;
        if (v == 0) { memset(G, 0, 81 * sizeof(double)); continue; }
        const double *n = j->gn + 3 * v;
        double io[3][3], om[3][3];
        for (int i = 0; i < 3; ++i)
            for (int k = 0; k < 3; ++k) {
                double s = 0.0;
                for (int jj = 0; jj < 3; ++jj)
                    for (int l = 0; l < 3; ++l) s += j->C0[((i * 3 + jj) * 3 + k) * 3 + l] * n[jj] * n[l];
                io[i][k] = s;
            }
        double det = io[0][0] * (io[1][1] * io[2][2] - io[1][2] * io[2][1]) -
                     io[0][1] * (io[1][0] * io[2][2] - io[1][2] * io[2][0]) +
                     io[0][2] * (io[1][0] * io[2][1] - io[2][0] * io[1][1]);
        om[0][0] = io[1][1] * io[2][2] - io[1][2] * io[2][1];
        om[0][1] = io[0][2] * io[2][1] - io[0][1] * io[2][2];
        om[0][2] = io[0][1] * io[1][2] - io[0][2] * io[1][1];
        om[1][0] = io[1][2] * io[2][0] - io[1][0] * io[2][2];
        om[1][1] = io[0][0] * io[2][2] - io[0][2] * io[2][0];
        om[1][2] = io[0][2] * io[1][0] - io[0][0] * io[1][2];
        om[2][0] = io[1][0] * io[2][1] - io[1][1] * io[2][0];
        om[2][1] = io[0][1] * io[2][0] - io[0][0] * io[2][1];
        om[2][2] = io[0][0] * io[1][1] - io[0][1] * io[1][0];
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) om[a][b] /= det;
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b)
                for (int c = 0; c < 3; ++c)
                    for (int d = 0; d < 3; ++d)
                        G[((a * 3 + b) * 3 + c) * 3 + d] = -1.0 * om[a][c] * n[b] * n[d];
    }
    return 0;
}

/* ---- the increment loop (Evolution, evolution.c:265-622) ------------- */
static void update_stress_all(oracle_job *j, double *Err_e_loc, double *Err_s_loc)
{
    /* UpdateStress (evolution.c:3-168) with per-voxel contributions summed
     * afterwards in voxel order */
    const double dt = j->TimeStep;
#pragma omp parallel for schedule(dynamic, 256) num_threads(j->nthreads)
    for (long v = 0; v < j->nv; ++v) {
        int ph = j->phase[v] - 1;
        double *sg = j->Sig + 9 * v, *ed = j->Edot + 9 * v;
        if (!j->Type_phases[ph]) {
            nr_out o;
            update_stress_voxel(j->nsys[ph], j->Cgr + 36 * v, j->C066,
                                (double (*)[3])sg, (double (*)[3])(j->Eps + 9 * v),
                                (double (*)[3])(j->DG + 9 * v), j->Sch + 60 * v,
                                j->trial + 24 * v, j->nsrs[ph], j->gam0[ph], dt,
                                j->gamdot + 12 * v, j->taux + 12 * v, &o);
            memcpy(sg, o.sig, sizeof(o.sig));
            memcpy(ed, o.edot, sizeof(o.edot));
            j->SVM[v] = o.svm;
            j->EVM[v] = o.evm;
            j->red_s[v] = o.conv_s;
            j->red_e[v] = o.conv_e;
        } else {
            memset(sg, 0, 9 * sizeof(double));
            memset(ed, 0, 9 * sizeof(double));
            j->red_s[v] = 0.0;
            j->red_e[v] = 0.0;
        }
    }
    double se = 0.0, ss = 0.0;
    for (long v = 0; v < j->nv; ++v) {
        int ph = j->phase[v] - 1;
        if (j->Type_phases[ph]) continue;
        ss += j->red_s[v];
        se += j->red_e[v];
    }
    *Err_e_loc = se;
    *Err_s_loc = ss;
}

static void get_smacro(oracle_job *j)
{
    /* evolution.c:170-241 */
    static const int IJV[2][6] = {{0, 1, 2, 1, 0, 0}, {0, 1, 2, 2, 2, 1}};
    double loc[9], loc1[9];
#pragma omp parallel for schedule(static) num_threads(j->nthreads)
    for (int c = 0; c < 9; ++c) {
        double s = 0.0, s1 = 0.0;
        for (long v = 0; v < j->nv; ++v) {
            s += j->Sig[9 * v + c];
            if (j->phase[v] == 1) s1 += j->Sig[9 * v + c];
        }
        loc[c] = s;
        loc1[c] = s1;
    }
    for (int c = 0; c < 9; ++c) {
        tr_d(j, loc[c]);
        tr_d(j, loc1[c]);
        j->SigAvg[c / 3][c % 3] = loc[c] * j->WGT;
        j->SigAvg1[c / 3][c % 3] = loc1[c] * (j->WGT / j->Wgt_ph1);
    }
    for (int i = 0; i < 6; ++i) {
        int ii = IJV[0][i], jj = IJV[1][i];
        j->dDisGradAvg[ii][jj] = 0.0;
        if (j->VelGrad_BC_Flag[i] == 0)
            for (int k = 0; k < 6; ++k) {
                int kk = IJV[0][k], ll = IJV[1][k];
                j->dDisGradAvg[ii][jj] += j->S0[((ii * 3 + jj) * 3 + kk) * 3 + ll] *
                                          j->Stress_BC_Flag[k] *
                                          (j->Scauchy[kk][ll] - j->SigAvg[kk][ll]);
            }
    }
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) j->dDisGradAvg_acum[a][b] += j->dDisGradAvg[a][b];
    double s6[6], dev[3][3];
    t_to_v6(j->SigAvg, s6, 6);
    v6_to_t(s6, dev, 5);
    j->s_vm = 0.0;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) j->s_vm += dev[a][b] * dev[a][b];
    j->s_vm = sqrt(3. / 2. * j->s_vm);
    t_to_v6(j->SigAvg1, s6, 6);
    v6_to_t(s6, dev, 5);
    j->s_vm1 = 0.0;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) j->s_vm1 += dev[a][b] * dev[a][b];
    j->s_vm1 = sqrt(3. / 2. * j->s_vm1);
}

static double von_mises_strain(double t[3][3])
{
    /* VonMises (evolution.c:243-262) */
    double tr = t[0][0] + t[1][1] + t[2][2], d[3][3], vm = 0.0;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) d[a][b] = (t[a][b] + t[b][a]) / 2. - (double)(a == b) * tr / 3.0;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) vm += d[a][b] * d[a][b];
    return sqrt(2. / 3. * vm);
}

static void update_orient(oracle_job *j)
{
    /* constitutive.c:171-248 */
    const double dt = j->TimeStep;
#pragma omp parallel for schedule(static) num_threads(j->nthreads)
    for (long v = 0; v < j->nv; ++v) {
        int ph = j->phase[v] - 1;
        if (j->Type_phases[ph]) { j->red_s[v] = 0.0; j->red_e[v] = 0.0; continue; }
        double RL[3][3], Lp[3][3], RS[3][3], Rot[3][3], tm[3][3];
        const double *VG = j->VG + 9 * v;
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                RL[a][b] = (VG[3 * a + b] - VG[3 * b + a]) / 2.;
                Lp[a][b] = 0.0;
                tm[a][b] = j->Tm[9 * v + 3 * a + b];
            }
        for (int s = 0; s < j->nsys[ph]; ++s) {
            double bs[3], ns[3];
            for (int a = 0; a < 3; ++a) {
                bs[a] = 0.0; ns[a] = 0.0;
                for (int b = 0; b < 3; ++b) {
                    bs[a] += tm[a][b] * j->bb[ph][s][b];
                    ns[a] += tm[a][b] * j->bn[ph][s][b];
                }
            }
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) Lp[a][b] += bs[a] * ns[b] * j->gamdot[12 * v + s];
        }
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) RS[a][b] = (Lp[a][b] - Lp[b][a]) / 2.;
        j->red_s[v] = sqrt(RS[2][1] * RS[2][1] + RS[0][2] * RS[0][2] + RS[1][0] * RS[1][0]) * j->WGT;
        j->red_e[v] = sqrt(RL[2][1] * RL[2][1] + RL[0][2] * RL[0][2] + RL[1][0] * RL[1][0]) * j->WGT;
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) Rot[a][b] = (j->Udot_a[a][b] + RL[a][b] - RS[a][b]) * dt;
        orientation(tm, Rot);
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) j->Tm[9 * v + 3 * a + b] = tm[a][b];
    }
    double rsl = 0.0, rlc = 0.0;
    for (long v = 0; v < j->nv; ++v) {
        int ph = j->phase[v] - 1;
        if (j->Type_phases[ph]) continue;
        rsl += j->red_s[v];
        rlc += j->red_e[v];
    }
    tr_d(j, rsl);
    tr_d(j, rlc);
}

static void log_iter(oracle_job *j)
{
    if (j->it_n == j->it_cap) {
        j->it_cap = j->it_cap ? 2 * j->it_cap : 1024;
        j->it_e = (double *)realloc(j->it_e, sizeof(double) * j->it_cap);
        j->it_s = (double *)realloc(j->it_s, sizeof(double) * j->it_cap);
        j->it_v = (double *)realloc(j->it_v, sizeof(double) * j->it_cap);
    }
    j->it_e[j->it_n] = j->Err_e;
    j->it_s[j->it_n] = j->Err_s;
    j->it_v[j->it_n] = j->s_vm;
    j->it_n++;
}

static void increment(oracle_job *j)
{
    const long nv = j->nv;
    const double dt = j->TimeStep;
    const int istep = ++j->istep;
    /* prelude (evolution.c:306-333) */
#pragma omp parallel for schedule(static) num_threads(j->nthreads)
    for (long v = 0; v < nv; ++v)
        for (int c = 0; c < 9; ++c) {
            j->VG[9 * v + c] = j->DG[9 * v + c];
            if (j->CREEP_FLAG == 1) j->DG[9 * v + c] = j->DisGradAvg_actual[c / 3][c % 3];
            else j->DG[9 * v + c] += j->Udot[c / 3][c % 3] * dt;
        }
    if (istep == 1 || j->Update_Flag == 1) update_schmid(j);
    memset(j->dDisGradAvg, 0, sizeof(j->dDisGradAvg));
    memset(j->dDisGradAvg_acum, 0, sizeof(j->dDisGradAvg_acum));

    if (j->n_incr == j->cap_incr) {
        j->cap_incr = j->cap_incr ? 2 * j->cap_incr : 64;
        j->incr = (oracle_incr *)realloc(j->incr, sizeof(oracle_incr) * j->cap_incr);
        j->it_start = (int *)realloc(j->it_start, sizeof(int) * j->cap_incr);
    }
    j->it_start[j->n_incr] = j->it_n;

    int iter = 0;
    j->Err_e = 2. * j->Err;
    j->Err_s = 2. * j->Err;
    const int nx = j->CellDim[0], ny = j->CellDim[1], nz = j->CellDim[2];
    double *F = j->fft;
    while ((iter < j->IterMax) && (fmax(fabs(j->Err_s), fabs(j->Err_e)) > fabs(j->Err))) {
        iter++;
        j->iter_total++;
        /* forward transforms of the nine stress components (evolution.c:350-361) */
        for (int c = 0; c < 9; ++c) {
#pragma omp parallel for schedule(static) num_threads(j->nthreads)
            for (long v = 0; v < nv; ++v) { F[2 * v] = j->Sig[9 * v + c]; F[2 * v + 1] = 0.0; }
            fftc_3d(nx, ny, nz, -1, F, j->nthreads);
#pragma omp parallel for schedule(static) num_threads(j->nthreads)
            for (long v = 0; v < nv; ++v) { j->kr[9 * v + c] = F[2 * v]; j->ki[9 * v + c] = F[2 * v + 1]; }
        }
        /* Green operator contraction (evolution.c:363-377) */
#pragma omp parallel for schedule(static) num_threads(j->nthreads)
        for (long v = 0; v < nv; ++v) {
            double ur[9], ui[9];
            const double *G = j->GAMMA + 81 * v, *kr = j->kr + 9 * v, *ki = j->ki + 9 * v;
            for (int c = 0; c < 9; ++c) {
                double sr = 0.0, si = 0.0;
                for (int d = 0; d < 9; ++d) {
                    sr += G[9 * c + d] * kr[d];
                    si += G[9 * c + d] * ki[d];
                }
                ur[c] = sr;
                ui[c] = si;
            }
            memcpy(j->kr + 9 * v, ur, sizeof(ur));
            memcpy(j->ki + 9 * v, ui, sizeof(ui));
        }
        /* inverse transforms and the displacement-gradient update (evolution.c:383-394) */
        for (int c = 0; c < 9; ++c) {
#pragma omp parallel for schedule(static) num_threads(j->nthreads)
            for (long v = 0; v < nv; ++v) { F[2 * v] = j->kr[9 * v + c]; F[2 * v + 1] = j->ki[9 * v + c]; }
            fftc_3d(nx, ny, nz, 1, F, j->nthreads);
            const double dd = j->dDisGradAvg[c / 3][c % 3];
#pragma omp parallel for schedule(static) num_threads(j->nthreads)
            for (long v = 0; v < nv; ++v) {
                j->DG[9 * v + c] += dd + F[2 * v] / j->Nxyz;
                j->fluct[9 * v + c] += F[2 * v] / j->Nxyz;
            }
        }
        double ee, es;
        update_stress_all(j, &ee, &es);
        tr_d(j, ee);
        tr_d(j, es);
        j->Err_e = ee;
        j->Err_s = es;
        j->Err_e *= j->WGT;
        j->Err_s *= j->WGT;
        get_smacro(j);
        if (fabs(j->e_vm) > 1E-5) j->Err_e /= j->e_vm;
        j->Err_s /= j->s_vm;
        log_iter(j);
    }

    /* epilogue (evolution.c:433-566) */
#pragma omp parallel for schedule(static) num_threads(j->nthreads)
    for (long v = 0; v < nv; ++v)
        for (int c = 0; c < 9; ++c) j->VG[9 * v + c] = (j->DG[9 * v + c] - j->VG[9 * v + c]) / dt;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            j->DisGradAvg_actual[a][b] = j->DisGradAvg[a][b] + j->dDisGradAvg_acum[a][b];
            j->VelGradAvg[a][b] = (j->DisGradAvg_actual[a][b] - j->DisGradAvg_t[a][b]) / dt;
        }
    j->e_vm = von_mises_strain(j->DisGradAvg_actual);
    double d_vm = von_mises_strain(j->VelGradAvg);
    memcpy(j->DisGradAvg_t, j->DisGradAvg_actual, sizeof(j->DisGradAvg_t));
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) j->DisGradAvg[a][b] = j->DisGradAvg_t[a][b] + j->Udot[a][b] * dt;
#pragma omp parallel for schedule(static) num_threads(j->nthreads)
    for (long v = 0; v < nv; ++v)
        for (int c = 0; c < 9; ++c) j->Eps[9 * v + c] += j->Edot[9 * v + c] * dt;
    double ea[9], da[9];
#pragma omp parallel for schedule(static) num_threads(j->nthreads)
    for (int c = 0; c < 9; ++c) {
        double s = 0.0, t = 0.0;
        for (long v = 0; v < nv; ++v) { s += j->Eps[9 * v + c]; t += j->Edot[9 * v + c]; }
        ea[c] = s;
        da[c] = t;
    }
    double evmp = 0.0, dvmp = 0.0;
    for (int c = 0; c < 9; ++c) {
        tr_d(j, ea[c]);
        tr_d(j, da[c]);
        j->EpsAvg[c / 3][c % 3] = ea[c] * j->WGT;
        j->EdotAvg[c / 3][c % 3] = da[c] * j->WGT;
    }
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            evmp += j->EpsAvg[a][b] * j->EpsAvg[a][b];
            dvmp += j->EdotAvg[a][b] * j->EdotAvg[a][b];
        }
    evmp = sqrt(2. / 3. * evmp);
    dvmp = sqrt(2. / 3. * dvmp);
    if (j->Update_Flag == 1 && istep > 1) update_orient(j);
    if (j->Hard_Flag == 1 && istep > 2) {
#pragma omp parallel for schedule(static) num_threads(j->nthreads)
        for (long v = 0; v < nv; ++v) {
            int ph = j->phase[v] - 1;
            if (j->Type_phases[ph]) continue;
            harden_voxel(j->nsys[ph], j->hard[ph], &j->tau[ph][0][0], &j->thet[ph][0][0], dt,
                         j->gamdot + 12 * v, j->gamacum + v, j->gtot + 12 * v,
                         j->crss + 24 * v, j->trial + 24 * v);
        }
    }
    oracle_incr *r = &j->incr[j->n_incr];
    memset(r, 0, sizeof(*r));
    r->istep = istep;
    r->iters = iter;
    r->iter_total = j->iter_total;
    r->e_vm = j->e_vm; r->evmp = evmp; r->d_vm = d_vm; r->dvmp = dvmp;
    r->s_vm = j->s_vm; r->s_vm1 = j->s_vm1;
    memcpy(r->sig_avg, j->SigAvg, sizeof(r->sig_avg));
    memcpy(r->sig_avg1, j->SigAvg1, sizeof(r->sig_avg1));
    memcpy(r->eps_avg, j->EpsAvg, sizeof(r->eps_avg));
    memcpy(r->edot_avg, j->EdotAvg, sizeof(r->edot_avg));
    memcpy(r->disgrad_avg, j->DisGradAvg_actual, sizeof(r->disgrad_avg));
    r->err_e = j->Err_e;
    r->err_s = j->Err_s;
    j->n_incr++;
}

/* --------------------------------------------------------------------- */
/* public API                                                             */
/* --------------------------------------------------------------------- */
oracle_job *oracle_create(const char *namelist_path, int nthreads,
                          const char *trace_path, char *err)
{
    char e[256] = {0};
    oracle_job *j = (oracle_job *)calloc(1, sizeof(*j));
    j->nthreads = nthreads > 0 ? nthreads : 1;
    if (trace_path && *trace_path) j->trace = fopen(trace_path, "w");
    if (setup(j, namelist_path, e)) {
        if (err) snprintf(err, 256, "%s", e);
        oracle_destroy(j);
        return NULL;
    }
    return j;
}

void oracle_destroy(oracle_job *j)
{
    if (!j) return;
    if (j->trace) fclose(j->trace);
    void *ps[] = {j->gn, j->GAMMA, j->Cgr, j->Tm, j->Sch, j->Sig, j->Eps, j->Edot, j->DG,
                  j->VG, j->fluct, j->crss, j->trial, j->gamdot, j->taux, j->gtot,
                  j->gamacum, j->SVM, j->EVM, j->kr, j->ki, j->fft, j->red_s, j->red_e,
                  j->grain, j->phase, j->incr, j->it_e, j->it_s, j->it_v, j->it_start};
    for (size_t k = 0; k < sizeof(ps) / sizeof(ps[0]); ++k) free(ps[k]);
    free(j);
}

int oracle_run(oracle_job *j, int n)
{
    for (int k = 0; k < n; ++k) increment(j);
    if (j->trace) fflush(j->trace);
    return j->n_incr;
}

int oracle_n_increments(const oracle_job *j) { return j->n_incr; }

int oracle_get_increment(const oracle_job *j, int k, oracle_incr *out)
{
    if (k < 0 || k >= j->n_incr) return -1;
    *out = j->incr[k];
    return 0;
}

int oracle_get_iter_log(const oracle_job *j, int k, double *ee, double *es, double *sv)
{
    if (k < 0 || k >= j->n_incr) return -1;
    int s = j->it_start[k], n = j->incr[k].iters;
    for (int i = 0; i < n; ++i) {
        if (ee) ee[i] = j->it_e[s + i];
        if (es) es[i] = j->it_s[s + i];
        if (sv) sv[i] = j->it_v[s + i];
    }
    return n;
}

int oracle_get_field(const oracle_job *j, int id, double *out)
{
    const double *src = NULL;
    int k = 0;
    switch (id) {
    case 0: src = j->Sig; k = 9; break;
    case 1: src = j->Eps; k = 9; break;
    case 2: src = j->Edot; k = 9; break;
    case 3: src = j->DG; k = 9; break;
    case 4: src = j->Tm; k = 9; break;
    case 5: k = 12; break;
    case 6: src = j->gamdot; k = 12; break;
    case 7: src = j->gamacum; k = 1; break;
    case 8: src = j->SVM; k = 1; break;
    case 9: src = j->EVM; k = 1; break;
    case 10: src = j->Sch; k = 60; break;
    case 11: src = j->Cgr; k = 36; break;
    default: return -1;
    }
    if (!out) return k;
    if (id == 5) {
        for (long v = 0; v < j->nv; ++v)
            for (int s = 0; s < 12; ++s) out[12 * v + s] = j->crss[24 * v + 2 * s];
    } else {
        memcpy(out, src, sizeof(double) * (size_t)k * (size_t)j->nv);
    }
    return k;
}

long oracle_nvox(const oracle_job *j) { return j->nv; }

int oracle_dims(const oracle_job *j, int *d)
{
    d[0] = j->CellDim[0]; d[1] = j->CellDim[1]; d[2] = j->CellDim[2];
    return 0;
}

int oracle_get_reference_medium(const oracle_job *j, double *c066, double *s066,
                                double *wgt_ph1)
{
    if (c066) memcpy(c066, j->C066, sizeof(j->C066));
    if (s066) memcpy(s066, j->S066, sizeof(j->S066));
    if (wgt_ph1) *wgt_ph1 = j->Wgt_ph1;
    return 0;
}

/* Displacement fluctuation, the computation evolution.c:532-560 sets out to
 * make, with its three faults corrected:
 *   - tmp_re/tmp_im are accumulated per frequency (the reference sums them
 *     over all voxels into one scalar per component, :545-546);
 *   - the inverse transform is taken of that accumulated spectrum (the
 *     reference stores the scalar at the stale index pIDX, :549-550, and
 *     transforms what is left of the last forward transform);
 *   - the weight is q = xi/|xi|^2, which makes the result an inverse gradient
 *     (the reference's g, init.c:660-676, is xi/|xi|).
 * Per component i: tmp(k) = sum_j i F^_ij(k) q_j(k), u_i = -Re(IFFT(tmp))/Nxyz,
 * with the reference's frequencies xi (init.c:660-667) and q(0) = 0.
 * from_fluct 1 transforms the accumulated `fluctuation` (evolution.c:392),
 * 0 transforms DisGrad (the same spectrum away from k = 0 while DisGrad is
 * never reset, i.e. without creep).  out: 3 doubles per voxel. */
int oracle_disp_fluct(oracle_job *j, int from_fluct, double *out)
{
    const int nx = j->CellDim[0], ny = j->CellDim[1], nz = j->CellDim[2];
    const long nv = j->nv;
    const double *src = from_fluct ? j->fluct : j->DG;
    double *q = (double *)malloc(sizeof(double) * 3 * (size_t)nv);
    double *tr = (double *)malloc(sizeof(double) * (size_t)nv);
    double *ti = (double *)malloc(sizeof(double) * (size_t)nv);
    double *F = j->fft;
    if (!q || !tr || !ti) { free(q); free(tr); free(ti); return -1; }
    for (int x = 0; x < nx; ++x)
        for (int y = 0; y < ny; ++y)
            for (int z = 0; z < nz; ++z) {
                long v = ((long)x * ny + y) * nz + z;
                double t[3];
                t[0] = (double)(x) * (double)(1.0 / nx);
                t[1] = (double)(y) * (double)(1.0 / ny);
                t[2] = (double)(z) * (double)(1.0 / nz);
                for (int m = 0; m < 3; ++m) { t[m] -= round(t[m]); t[m] *= TWO_PI_REF; }
                double s = t[0] * t[0] + t[1] * t[1] + t[2] * t[2];
                for (int m = 0; m < 3; ++m) q[3 * v + m] = (v == 0) ? 0.0 : t[m] / s;
            }
    for (int mi = 0; mi < 3; ++mi) {
        memset(tr, 0, sizeof(double) * (size_t)nv);
        memset(ti, 0, sizeof(double) * (size_t)nv);
        for (int mj = 0; mj < 3; ++mj) {
            for (long v = 0; v < nv; ++v) { F[2 * v] = src[9 * v + 3 * mi + mj]; F[2 * v + 1] = 0.0; }
            fftc_3d(nx, ny, nz, -1, F, j->nthreads);
            for (long v = 0; v < nv; ++v) {
                tr[v] += -F[2 * v + 1] * q[3 * v + mj];
                ti[v] += F[2 * v] * q[3 * v + mj];
            }
        }
        for (long v = 0; v < nv; ++v) { F[2 * v] = tr[v]; F[2 * v + 1] = ti[v]; }
        fftc_3d(nx, ny, nz, 1, F, j->nthreads);
        for (long v = 0; v < nv; ++v) out[3 * v + mi] = -F[2 * v] / j->Nxyz;
    }
    free(q); free(tr); free(ti);
    return 0;
}
