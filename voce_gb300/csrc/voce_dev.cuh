// Device-side data structures and math of the GB300 EVP-FFT solver step.
//
// Layout in HBM (one RVE, nv = nx*ny*nz voxels, x slowest / z fastest, SoA):
//   sig[6][nv]    stress in the Lebensohn-Tome 6-vector basis (the basis of
//                 the reference's chg_basis, kinematics.c:14-174)
//   sigp[5][nv]   stress before the last Newton update (the point at which
//                 the reference evaluates Edot/gamdot, evolution.c:67,126)
//   eps[5][nv]    total strain at time t in the same basis (6th comp is 0)
//   dgs[6][nv]    symmetric part of the displacement gradient, same basis
//   dga[3][nv]    antisymmetric part: (D12-D21)/2, (D02-D20)/2, (D01-D10)/2
//   tm[9][nv]     crystal->sample rotation TranMat_xt2sa (evp.h:240)
//   sch[60][nv]   Schmid 5-vectors of the 12 systems in sample axes
//   sg[21][nv]    grain compliance S_g = C_gr^-1, packed upper triangle
//   sgp[21][nv]   S_g + S0, packed (mixed_ir form only)
//   crss[24][nv]  critical resolved shear stress (system, +/- direction)
//   itau[24][nv]  1/crss
//   gamacum[nv], gtot[12][nv], edot[5][nv], gamdot[12][nv], taux[12][nv],
//   svm[nv], evm[nv], phase[nv]
//   diag[3][nv]   post-increment diagnostics rho_rss, rho_crss, work_p
//                 (evolution.c:509-529)
//   spec[6][nzh][nx][ny] half spectrum (kz = 0..nz/2), complex, y fastest
//   aacc[3][nzh][nx][ny] antisymmetric part of the Green update, summed
//                 over the iterations of the current increment
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define VOCE_NS 12
#define VOCE_NPART 16
#define VOCE_MAXRAD 12
#define VOCE_ITLOG 12   // doubles per logged iteration
// Mixed form: Green iterations whose predecessor's normalised error is above
// this (and the first of every increment) run the Newton solve in single
// precision only; the rest end it on the double-precision residual.
#define VOCE_POLISH_ERR 1e-4
// systems per unrolled step of the single-precision flow-rule loops (their
// loads issue together)
#ifndef VOCE_SYS_UNROLL
#define VOCE_SYS_UNROLL 2
#endif
constexpr int kSysUnroll = VOCE_SYS_UNROLL;

// Lebensohn-Tome basis constants, the literal values of kinematics.c:333-335
#define RSQ2 0.70710678118654744
#define RSQ3 0.57735026918962584
#define RSQ6 0.40824829046386304
#define VOCE_PI_REF 3.14159265359
#define VOCE_TWO_PI_REF 6.28318530718

// One axis's transform: Stockham radix stages rad[0..nst) (n1 = 0), or, in
// the single-precision spectrum only, the two-pass register FFT of
// L = n1 x (L / n1) (n1 > 0; rad then keeps the default Stockham stages).
struct FftPlan1 {
    int L, nst;
    int rad[VOCE_MAXRAD];
    int n1;
};

// Per-RVE macro state (device, written only by the single-thread
// finalisers).  Mirrors the reference's macro globals and Evolution locals.
struct MacroDev {
    double DisGradAvg[9], DisGradAvg_t[9], DisGradAvg_actual[9];
    double dDisGradAvg[9], dDisGradAvg_acum[9], VelGradAvg[9], DGA_prev[9];
    double SigAvg[9], SigAvg1[9], EpsAvg[9], EdotAvg[9];
    double s_vm, s_vm1, e_vm, d_vm, evmp, dvmp, Err_e, Err_s;
    double ddg6[6];      // B-basis sym(dDisGradAvg) used by the next c2r update
    double acum_a[3];    // antisym(dDisGradAvg_acum): A12, A02, A01
    double rsl, rlc, nr_total;
    int iter, iter_total, istep, converged, nr_max, first_iter, done;
    int active;          // 1 while increments remain (batched runs)
    int pending_prelude; // 1 after an increment ended inside a batch tick
    int target;          // last increment to run (batched runs)
    int pad;
};

// Per-increment record (device array, one per increment run)
struct IncrDev {
    int istep, iters, iter_total, nr_max;
    double e_vm, evmp, d_vm, dvmp, s_vm, s_vm1;
    double sig_avg[9], sig_avg1[9], eps_avg[9], edot_avg[9], disgrad_avg[9];
    double err_e, err_s, rsl, rlc, nr_total;
};

// Everything a kernel needs to know about one RVE.  Passed by value as a
// kernel parameter (it is ~3 KB; the limit is 32 KB).
struct RveDesc {
    int nx, ny, nz, nzh;
    long long nv, nspec;
    int solid[3];        // solid[phase id 1..2]
    int nsys, ipow_n;    // ipow_n >= 0: n integral, |r|^(n-1) by multiplication
    int update_flag, hard_flag, creep, iter_max;
    int mixed;           // spectrum precision: 0 double, 1 float
    int chord;           // FP64 Newton: reuse the last Jacobian once the update is below 1e-4
    int nr32;            // Newton iterations in float with an FP64 acceptance step
    int ir;              // Newton on the FP64 residual with a float Jacobian and solve
    int ir_pred;         // ir: the FP64 steps start from a single-precision / float-float solve
    double dt, wgt, wgt_ph1, err_tol, inv_nv;
    double wgt_ratio;    // wgt / wgt_ph1 (the same IEEE division, once on the host)
    int all_ph1;         // every voxel is phase 1 (the phase-1 sums equal the full ones)
    double gam0[VOCE_NS], nrs[VOCE_NS], g0n[VOCE_NS];
    float gam0f[VOCE_NS], nrsf[VOCE_NS];   // float copies for the mixed Newton
    float gam0l[VOCE_NS];                  // gam0 - gam0f, rounded to float
    float dth, dtl;                        // dt as a float pair: dth + dtl
    int gam0_uniform;    // every system has the same gam0
    double tau0[VOCE_NS], tau1[VOCE_NS], thet0[VOCE_NS], thet1[VOCE_NS];
    double hard[VOCE_NS * VOCE_NS];
    double bn[VOCE_NS * 3], bb[VOCE_NS * 3];
    double S0[36];       // S066 (B basis)
    float S0f[36];       // float copy (mixed-precision error norms)
    double S0t[81];      // S0 as 3x3x3x3 (get_smacro's dDisGradAvg)
    double Kq[36];       // acoustic tensor coefficients: K6 = Kq * nn6
    float Kqf[36];       // float copy (Green operator of the mixed forms)
    double inv_n[3];     // 1.0/nx, 1.0/ny, 1.0/nz
    float inv_nf[3];
    double Udot[9], Scauchy[9];
    double u6[6];        // B-basis sym(Udot)
    double ua[3];        // antisym(Udot): A12, A02, A01
    int vflag[6], sflag[6];
    FftPlan1 plx, ply, plz;
    // FFT tiles (lines per block) and the Newton-kernel work split
    int zrows, yxt, xkc, xkc3, zirows, zirows3;
    double schxt[VOCE_NS * 5];  // Schmid 5-vectors in crystal axes
    double tau0b[VOCE_NS];      // backward CRSS start value
    // fields
    double *sig, *sigp, *eps, *dgs, *dga, *tm, *sch, *sg, *crss, *itau;
    float *sch32;        // float copy of sch (float-Jacobian Newton forms only)
    float *itau32;       // float copy of itau (float-Jacobian Newton forms only)
    float *sgp32;        // float (S_g + S0), packed upper triangle (float-Jacobian Newton forms only)
    float *sch_lo, *itau_lo, *sgp_lo;   // x - (double)x32 rounded to float, for the same three
    double *sgp;         // S_g + S0 in FP64, packed upper triangle (the mixed_ir Newton's residual)
    double *gamacum, *gtot, *edot, *gamdot, *taux, *svm, *evm, *rotl, *diag;
    int *phase;
    void *spec, *aacc;
    const void *twx, *twy, *twz;  // exp(-2 pi i j / L), complex of the spectrum type
    double *part;        // [npart_blocks][VOCE_NPART]
    double *gstore;      // FP64 form: per frequency n(3) and omega(6), [9][nspec]
    int npart;
    MacroDev *macro;
    double *itlog;       // [iter_max][VOCE_ITLOG] for the current increment
    IncrDev *incr;       // [capacity]
    int incr_cap;
};

// ---------------------------------------------------------------------------
// small tensor helpers.  Symmetric 3x3 as 6 comps (00,11,22,12,02,01).
// ---------------------------------------------------------------------------
template <typename T>
__host__ __device__ __forceinline__ void t6_to_b(const T *t, T *b)
{
    b[0] = T(RSQ2) * (t[1] - t[0]);
    b[1] = T(RSQ6) * (T(2) * t[2] - t[0] - t[1]);
    b[2] = T(2.0 * RSQ2) * t[3];
    b[3] = T(2.0 * RSQ2) * t[4];
    b[4] = T(2.0 * RSQ2) * t[5];
    b[5] = T(RSQ3) * (t[0] + t[1] + t[2]);
}

template <typename T>
__host__ __device__ __forceinline__ void b_to_t6(const T *b, T *t)
{
    t[0] = -T(RSQ2) * b[0] - T(RSQ6) * b[1] + T(RSQ3) * b[5];
    t[1] = T(RSQ2) * b[0] - T(RSQ6) * b[1] + T(RSQ3) * b[5];
    t[2] = T(2.0 * RSQ6) * b[1] + T(RSQ3) * b[5];
    t[3] = T(RSQ2) * b[2];
    t[4] = T(RSQ2) * b[3];
    t[5] = T(RSQ2) * b[4];
}

// packed upper-triangle index of a symmetric 6x6
__host__ __device__ __forceinline__ int sym6(int i, int j)
{
    int a = i < j ? i : j, b = i < j ? j : i;
    return a * 6 - (a * (a - 1)) / 2 + (b - a);
}

// Newton-Raphson reciprocal: the hardware's approximate double reciprocal
// (rcp.approx.ftz.f64, about 20 correct bits) refined by two steps of
// r <- r + r(1 - x r), each of which squares the relative error (down to
// rounding); outside 2^-99 <= |x| < 2^99 it falls back to division.  The
// range test reads the exponent bits with integer operations, and the seed
// needs no conversions, which keeps both off the FP64 pipe.  It is used
// inside the 6x6 solve of the Newton step and for the Green operator's 3x3
// inverse.
__device__ __forceinline__ double rcp_nr(double x)
{
    const unsigned hi = (unsigned)__double2hiint(x) & 0x7fffffffu;
    if (hi - 0x39C00000u >= 0x46200000u - 0x39C00000u) return 1.0 / x;
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
    double e = fma(-x, r, 1.0);
    r = fma(r, e, r);
    e = fma(-x, r, 1.0);
    r = fma(r, e, r);
    return r;
}

// Newton-Raphson square root for the mixed_ir form's per-voxel error norms:
// the hardware's approximate double reciprocal square root r
// (rsqrt.approx.ftz.f64) gives y = x r, and one Heron step
// y <- y + (x - y^2) r / 2 (the residual exact by an FMA) squares its
// relative error, to about 1e-13; outside 2^-99 <= x < 2^99 (zero, tiny,
// huge, negative, not finite) it falls back to sqrt.  Four FP64-pipe
// operations instead of the correctly rounded square root's longer sequence.
__device__ __forceinline__ double sqrt_nr(double x)
{
    const unsigned hi = (unsigned)__double2hiint(x);
    if (hi - 0x39C00000u >= 0x46200000u - 0x39C00000u) return sqrt(x);
    double r;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
    const double y = x * r;
    return fma(fma(-y, y, x), 0.5 * r, y);
}

// single-precision LDL^T solve of the same system (mixed-precision Newton).
// The pivots' reciprocals are the hardware's approximate ones
// (rcp.approx.ftz.f32, within an ulp): the solve is a Newton correction whose
// accuracy is that of single precision anyway, and the pivots of this
// positive definite system are normal numbers.
__device__ __forceinline__ void ldlt_solve6f(const float (&M)[6][6], float (&b)[6])
{
    float L[6][6], w[6][6], dinv[6];
#pragma unroll
    for (int j = 0; j < 6; ++j) {
        float dj = M[j][j];
#pragma unroll
        for (int k = 0; k < j; ++k) dj = fmaf(-L[j][k], w[j][k], dj);
        asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(dinv[j]) : "f"(dj));
#pragma unroll
        for (int i = j + 1; i < 6; ++i) {
            float sv = M[i][j];
#pragma unroll
            for (int k = 0; k < j; ++k) sv = fmaf(-L[i][k], w[j][k], sv);
            w[i][j] = sv;
            L[i][j] = sv * dinv[j];
        }
    }
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        float sv = b[i];
#pragma unroll
        for (int k = 0; k < i; ++k) sv = fmaf(-L[i][k], b[k], sv);
        b[i] = sv;
    }
#pragma unroll
    for (int i = 0; i < 6; ++i) b[i] *= dinv[i];
#pragma unroll
    for (int i = 5; i >= 0; --i) {
        float sv = b[i];
#pragma unroll
        for (int k = i + 1; k < 6; ++k) sv = fmaf(-L[k][i], b[k], sv);
        b[i] = sv;
    }
}

// |r|^e by binary powering (e >= 0), exact integer exponent
__device__ __forceinline__ double ipow_abs(double a, int e)
{
    double res = 1.0, b = a;
    while (e) {
        if (e & 1) res *= b;
        e >>= 1;
        if (e) b *= b;
    }
    return res;
}

// |r|^e with a fixed multiplication chain for e = 19 (n = 20): 6 products
__device__ __forceinline__ double pow_abs_e(double a, int e)
{
    if (e == 19) {
        const double a2 = a * a, a4 = a2 * a2, a8 = a4 * a4, a16 = a8 * a8;
        return (a16 * a2) * a;
    }
    return ipow_abs(a, e);
}

// ---------------------------------------------------------------------------
// Flow rule: StrainRate_eval (constitutive.c:126-194) on a stress 5-vector.
// edot[5] = sum_k sch_k * gdot_k; D (packed 15, 5x5 sym) = sum_k rss1_k sch_k sch_k^T
// xkin is always zero in the reference (init.c:793) and is left out.
// ---------------------------------------------------------------------------
template <bool WANT_D, bool WANT_SYS, typename DT = double>
__device__ __forceinline__ void flow_rule(const RveDesc &d, long long v, const double *s,
                                          double *edot, DT *D, double *gd, double *tx)
{
    const long long nv = d.nv;
#pragma unroll
    for (int i = 0; i < 5; ++i) edot[i] = 0.0;
    if (WANT_D) {
#pragma unroll
        for (int i = 0; i < 15; ++i) D[i] = DT(0);
    }
    for (int k = 0; k < d.nsys; ++k) {
        double sc[5];
#pragma unroll
        for (int i = 0; i < 5; ++i) sc[i] = __ldg(d.sch + (long long)(5 * k + i) * nv + v);
        const double rss = sc[0] * s[0] + sc[1] * s[1] + sc[2] * s[2] + sc[3] * s[3] + sc[4] * s[4];
        // the sign bit by an integer test (for rss = -0 it picks the backward
        // CRSS, where a float compare picks the forward one; both give zero
        // shear rate and a zero tangent term)
        const int neg = __double2hiint(rss) < 0;
        const double it = __ldg(d.itau + (long long)(2 * k + neg) * nv + v);
        const double r = rss * it;
        double g1, g2;
        if (d.ipow_n >= 1) {
            // |r|^(n-1) and |r|^n sign(r) = q r with q = gam0 |r|^(n-1)
            const double q = d.gam0[k] * pow_abs_e(fabs(r), d.ipow_n - 1);
            g2 = q * r;                      // rss2 = gam0 |r^n| sign(r)
            g1 = (q * it) * d.nrs[k];        // rss1 = gam0 n |r^(n-1)| / tau
        } else {
            g1 = d.g0n[k] * fabs(pow(r, d.nrs[k] - 1.0)) * it;
            g2 = d.gam0[k] * fabs(pow(r, d.nrs[k])) * (r > 0.0 ? 1.0 : -1.0);
        }
        if (WANT_SYS) { gd[k] = g2; tx[k] = g1; }
#pragma unroll
        for (int i = 0; i < 5; ++i) edot[i] = fma(sc[i], g2, edot[i]);
        if (WANT_D) {
            DT scd[5], t[5];
            if (sizeof(DT) == 4) {
                // the single-precision Jacobian reads the float copy of the Schmid vectors
#pragma unroll
                for (int i = 0; i < 5; ++i) scd[i] = (DT)__ldg(d.sch32 + (long long)(5 * k + i) * nv + v);
            } else {
#pragma unroll
                for (int i = 0; i < 5; ++i) scd[i] = (DT)sc[i];
            }
            const DT gg = (DT)g1;
#pragma unroll
            for (int i = 0; i < 5; ++i) t[i] = gg * scd[i];
            int q = 0;
#pragma unroll
            for (int i = 0; i < 5; ++i)
#pragma unroll
                for (int j = i; j < 5; ++j) { D[q] = fma(t[i], scd[j], D[q]); ++q; }
        }
    }
}

// |a|^e in single precision: the same product chain as pow_abs_e.
__device__ __forceinline__ float pow_abs_ef(float a, int e)
{
    if (e == 19) {
        const float a2 = a * a, a4 = a2 * a2, a8 = a4 * a4, a16 = a8 * a8;
        return (a16 * a2) * a;
    }
    float res = 1.0f, b = a;
    while (e) {
        if (e & 1) res *= b;
        b *= b;
        e >>= 1;
    }
    return res;
}

// The single-precision Newton kernel stages each voxel's float Schmid
// vectors and 1/CRSS (both directions) in shared memory, one column per
// thread: st[c * VOCE_NR_THREADS], c = 5k+i for the Schmid vectors and
// VOCE_STAGE_ITAU + 2k + (rss < 0) for 1/CRSS.
#define VOCE_NR_THREADS 128
#define VOCE_STAGE_ITAU 60
#define VOCE_STAGE_FLOATS 84

// flow_rule entirely in single precision (mixed-precision Newton, integer
// exponent only): strain rate and its 5x5 Jacobian (packed upper triangle)
// at the stress s, from the staged column st.  Returns false when a resolved-shear ratio is too large
// for |r|^n in single precision, or not finite.
__device__ __forceinline__ bool flow_rule_f32(const RveDesc &d, const float *st, const float *s,
                                              float *edot, float *D)
{
#pragma unroll
    for (int i = 0; i < 5; ++i) edot[i] = 0.0f;
#pragma unroll
    for (int i = 0; i < 15; ++i) D[i] = 0.0f;
#pragma unroll kSysUnroll
    for (int k = 0; k < d.nsys; ++k) {
        float sc[5];
#pragma unroll
        for (int i = 0; i < 5; ++i) sc[i] = st[(5 * k + i) * VOCE_NR_THREADS];
        const float rss = sc[0] * s[0] + sc[1] * s[1] + sc[2] * s[2] + sc[3] * s[3] + sc[4] * s[4];
        const int neg = rss < 0.0f;
        const float it = st[(VOCE_STAGE_ITAU + 2 * k + neg) * VOCE_NR_THREADS];
        const float r = rss * it;
        const float ar = fabsf(r);
        if (!(ar < 60.0f)) return false;
        const float q = d.gam0f[k] * pow_abs_ef(ar, d.ipow_n - 1);
        const float g2 = q * r, g1 = (q * it) * d.nrsf[k];
        float t[5];
#pragma unroll
        for (int i = 0; i < 5; ++i) {
            edot[i] = fmaf(sc[i], g2, edot[i]);
            t[i] = g1 * sc[i];
        }
        int c = 0;
#pragma unroll
        for (int i = 0; i < 5; ++i)
#pragma unroll
            for (int j = i; j < 5; ++j) { D[c] = fmaf(t[i], sc[j], D[c]); ++c; }
    }
    return true;
}

// ---------------------------------------------------------------------------
// Float-float arithmetic for the mixed Newton's acceptance residual.  A value
// is the unevaluated sum h + l of two floats, about 48 significant bits.  The
// error-free transformations are Knuth's TwoSum and the FMA TwoProduct; the
// dot products accumulate as in Ogita, Rump and Oishi's Dot2 ("Accurate sum
// and dot product", SIAM J. Sci. Comput. 26, 2005).  Each step is written in
// the order it must be evaluated (no fast-math, nothing reassociated).  The
// residual only needs an absolute error far below 2^-24 of its largest term,
// so pairs are renormalised only where a product follows.
// ---------------------------------------------------------------------------
struct ff32 {
    float h, l;
};

// stores x as the float pair hi[i] + lo[i] (hi alone when lo is null)
__device__ __forceinline__ void put_pair(float *hi, float *lo, long long i, double x)
{
    const float h = (float)x;
    hi[i] = h;
    if (lo) lo[i] = (float)(x - (double)h);
}

__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// h + l with |l| below half an ulp of h (|h| >= |l| on entry)
__device__ __forceinline__ ff32 ff_norm(float h, float l)
{
    ff32 r;
    r.h = h + l;
    r.l = l - (r.h - h);
    return r;
}

// acc += (ah + al) * x
__device__ __forceinline__ void ff_acc(ff32 &acc, float ah, float al, float x)
{
    const float p = ah * x;
    const float pe = fmaf(ah, x, -p);
    float s, e;
    two_sum(acc.h, p, s, e);
    acc.h = s;
    acc.l += e + fmaf(al, x, pe);
}

// acc += (ah + al) * (bh + bl)
__device__ __forceinline__ void ff_acc2(ff32 &acc, float ah, float al, float bh, float bl)
{
    const float p = ah * bh;
    const float pe = fmaf(ah, bl, fmaf(al, bh, fmaf(ah, bh, -p)));
    float s, e;
    two_sum(acc.h, p, s, e);
    acc.h = s;
    acc.l += e + pe;
}

__device__ __forceinline__ ff32 ff_mul(ff32 a, float bh, float bl)
{
    const float p = a.h * bh;
    return ff_norm(p, fmaf(a.h, bl, fmaf(a.l, bh, fmaf(a.h, bh, -p))));
}

__device__ __forceinline__ ff32 ff_add(ff32 a, ff32 b)
{
    float s, e;
    two_sum(a.h, b.h, s, e);
    return ff_norm(s, e + (a.l + b.l));
}

// a^e for a float pair a >= 0 and an integer e >= 1, by binary powering
__device__ __forceinline__ ff32 ff_ipow(ff32 a, int e)
{
    if (e == 20) {   // a^16 a^4
        ff32 a2 = ff_mul(a, a.h, a.l), a4 = ff_mul(a2, a2.h, a2.l);
        ff32 a8 = ff_mul(a4, a4.h, a4.l), a16 = ff_mul(a8, a8.h, a8.l);
        return ff_mul(a16, a4.h, a4.l);
    }
    ff32 res, b = a;
    res.h = 1.0f;
    res.l = 0.0f;
    while (e) {
        if (e & 1) res = ff_mul(res, b.h, b.l);
        e >>= 1;
        if (e) b = ff_mul(b, b.h, b.l);
    }
    return res;
}

// The Newton residual of evolution.c:78-83 in the symmetric form used here,
//   x = cc + dt * edot(s) + (S_g + S0) s,
// at a single-precision stress s, in float-float: every model quantity is
// taken as its float pair (Schmid vectors, 1/CRSS, S_g + S0, gam0, dt), which
// is its double value to about 2^-48, so x is the double-precision residual.
// Ph holds the high halves of S_g + S0 (already loaded), st the staged
// column of the high halves of the Schmid vectors and 1/CRSS (flow_rule_f32).
// Returns false when a resolved-shear ratio leaves the single-precision range.
__device__ __forceinline__ bool residual_ff(const RveDesc &d, long long v, const float *st,
                                            const float (&s)[6], const double (&cc)[6],
                                            const float (&Ph)[21], float (&x)[6])
{
    const long long nv = d.nv;
    ff32 ed[5];
#pragma unroll
    for (int i = 0; i < 5; ++i) { ed[i].h = 0.0f; ed[i].l = 0.0f; }
    const bool uni = d.gam0_uniform != 0;
#pragma unroll kSysUnroll
    for (int k = 0; k < d.nsys; ++k) {
        float sh[5], sl[5];
#pragma unroll
        for (int i = 0; i < 5; ++i) {
            sh[i] = st[(5 * k + i) * VOCE_NR_THREADS];
            sl[i] = __ldg(d.sch_lo + (long long)(5 * k + i) * nv + v);
        }
        ff32 rss;
        rss.h = 0.0f;
        rss.l = 0.0f;
#pragma unroll
        for (int i = 0; i < 5; ++i) ff_acc(rss, sh[i], sl[i], s[i]);
        rss = ff_norm(rss.h, rss.l);
        const int neg = rss.h < 0.0f;
        const float ih = st[(VOCE_STAGE_ITAU + 2 * k + neg) * VOCE_NR_THREADS];
        ff32 a = ff_mul(rss, ih, __ldg(d.itau_lo + (long long)(2 * k + neg) * nv + v));
        if (neg) { a.h = -a.h; a.l = -a.l; }
        if (!(a.h < 60.0f)) return false;
        ff32 g = ff_ipow(a, d.ipow_n);   // |r|^n
        if (!uni) g = ff_mul(g, d.gam0f[k], d.gam0l[k]);
        if (neg) { g.h = -g.h; g.l = -g.l; }
#pragma unroll
        for (int i = 0; i < 5; ++i) ff_acc2(ed[i], sh[i], sl[i], g.h, g.l);
    }
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        const float ch = (float)cc[i];
        ff32 t;
        t.h = ch;
        t.l = (float)(cc[i] - (double)ch);
        if (i < 5) {
            ff32 e = ff_norm(ed[i].h, ed[i].l);
            if (uni) e = ff_mul(e, d.gam0f[0], d.gam0l[0]);
            t = ff_add(t, ff_mul(e, d.dth, d.dtl));
        }
#pragma unroll
        for (int j = 0; j < 6; ++j) {
            const int q = sym6(i, j);
            ff_acc(t, Ph[q], __ldg(d.sgp_lo + (long long)q * nv + v), s[j]);
        }
        x[i] = t.h + t.l;
    }
    return true;
}

// Solve M x = b for symmetric positive definite M (6x6, full storage, only
// the lower triangle read) by an LDL^T factorisation without pivoting.
// LDL^T factors of the symmetric 6x6 M (lower triangle read): L strictly
// below the diagonal, dinv = 1/D
__device__ __forceinline__ void ldlt_factor6(const double (&M)[6][6], double (&L)[6][6], double (&dinv)[6])
{
    double w[6][6];
#pragma unroll
    for (int j = 0; j < 6; ++j) {
        double dj = M[j][j];
#pragma unroll
        for (int k = 0; k < j; ++k) dj = fma(-L[j][k], w[j][k], dj);
        dinv[j] = rcp_nr(dj);
#pragma unroll
        for (int i = j + 1; i < 6; ++i) {
            double s = M[i][j];
#pragma unroll
            for (int k = 0; k < j; ++k) s = fma(-L[i][k], w[j][k], s);
            w[i][j] = s;
            L[i][j] = s * dinv[j];
        }
    }
}

// b := M^-1 b from the factors of ldlt_factor6
__device__ __forceinline__ void ldlt_apply6(const double (&L)[6][6], const double (&dinv)[6], double (&b)[6])
{
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        double s = b[i];
#pragma unroll
        for (int k = 0; k < i; ++k) s = fma(-L[i][k], b[k], s);
        b[i] = s;
    }
#pragma unroll
    for (int i = 0; i < 6; ++i) b[i] *= dinv[i];
#pragma unroll
    for (int i = 5; i >= 0; --i) {
        double s = b[i];
#pragma unroll
        for (int k = i + 1; k < 6; ++k) s = fma(-L[k][i], b[k], s);
        b[i] = s;
    }
}

__device__ __forceinline__ void ldlt_solve6(const double (&M)[6][6], double (&b)[6])
{
    double L[6][6], dinv[6];
    ldlt_factor6(M, L, dinv);
    ldlt_apply6(L, dinv, b);
}

// ---------------------------------------------------------------------------
// Green operator on the fly.  The reference tabulates
//   Gamma_ijkl(k) = -omega_ik n_j n_l,  omega = (C0_ijkl n_j n_l)^-1
// per frequency (init.c:546-615) and contracts it with the stress spectrum
// (evolution.c:363-377).  Here, per frequency: t = sig^ n, v = omega t,
// dU = -v (x) n, split into its symmetric part (6 comps, basis B) and its
// antisymmetric part (A12, A02, A01).
// The reference takes the real part of a complex inverse FFT of dU
// (evolution.c:389-392); that equals the inverse transform of the Hermitian
// part of dU, i.e. of (Gamma(k) + Gamma(-k))/2 applied to sig^(k).  Gamma is
// even in n except on the Nyquist planes, where n(-k) is not -n(k) because
// the reference maps index N/2 to -pi for both k and -k (init.c:661-666);
// there both operators are applied and averaged.
// ---------------------------------------------------------------------------
// Frequency of index i on an axis of n points (init.c:655-666): the
// reference's i/n - round(i/n), scaled by its 2 pi; inv_n = 1.0/n exactly as
// the host computes it.
__device__ __forceinline__ double kfreq(int i, double inv_n)
{
    double t = (double)i * inv_n;
    t -= round(t);
    return t * VOCE_TWO_PI_REF;
}

// The same in single precision, with the rounding done on the integer index
// (i in [0, n): i - n when 2i >= n, which is where round(i/n) is 1).
__device__ __forceinline__ float kfreqf(int i, int n, float inv_n)
{
    const int ii = (2 * i >= n) ? i - n : i;
    return ((float)ii * inv_n) * (float)VOCE_TWO_PI_REF;
}

// Unit frequency vector n = g/|g| (g != 0)
__device__ __forceinline__ void unit_freq(const RveDesc &d, int ix, int iy, int iz, double *n)
{
    const double g0 = kfreq(ix, d.inv_n[0]), g1 = kfreq(iy, d.inv_n[1]), g2 = kfreq(iz, d.inv_n[2]);
    const double s = rsqrt(g0 * g0 + g1 * g1 + g2 * g2);
    n[0] = g0 * s; n[1] = g1 * s; n[2] = g2 * s;
}

__device__ __forceinline__ void unit_freq(const RveDesc &d, int ix, int iy, int iz, float *n)
{
    const float g0 = kfreqf(ix, d.nx, d.inv_nf[0]), g1 = kfreqf(iy, d.ny, d.inv_nf[1]);
    const float g2 = kfreqf(iz, d.nz, d.inv_nf[2]);
    const float s = rsqrtf(g0 * g0 + g1 * g1 + g2 * g2);
    n[0] = g0 * s; n[1] = g1 * s; n[2] = g2 * s;
}

// Arithmetic type of the Green operator: double in the FP64 form, float with
// the single-precision spectrum (the mixed forms).
template <typename R> struct GreenT { typedef double T; };
template <> struct GreenT<float> { typedef float T; };

__device__ __forceinline__ double green_rcp(double x) { return rcp_nr(x); }
__device__ __forceinline__ float green_rcp(float x) { return __frcp_rn(x); }

// omega = (Kq nn)^-1 of unit frequency n: 00, 01, 02, 11, 12, 22
template <typename G>
__device__ __forceinline__ void green_omega(const G *Kq, const G *nd, G (&w)[6])
{
    // acoustic tensor K_ik = C0_ijkl n_j n_l (6 sym comps) = Kq * nn
    G nn[6] = {nd[0] * nd[0], nd[1] * nd[1], nd[2] * nd[2],
               nd[1] * nd[2], nd[0] * nd[2], nd[0] * nd[1]};
    G K[6];
#pragma unroll
    for (int a = 0; a < 6; ++a) {
        G s = G(0);
#pragma unroll
        for (int m = 0; m < 6; ++m) s = fma(Kq[a * 6 + m], nn[m], s);
        K[a] = s;
    }
    // omega = K^-1 by cofactors (M3Inverse, init.c:546-568); K symmetric
    G c00 = K[1] * K[2] - K[3] * K[3];
    G c01 = K[4] * K[3] - K[5] * K[2];
    G c02 = K[5] * K[3] - K[4] * K[1];
    G c11 = K[0] * K[2] - K[4] * K[4];
    G c12 = K[4] * K[5] - K[0] * K[3];
    G c22 = K[0] * K[1] - K[5] * K[5];
    G det = K[0] * c00 + K[5] * c01 + K[4] * c02;
    G id = green_rcp(det);
    w[0] = c00 * id; w[1] = c01 * id; w[2] = c02 * id;
    w[3] = c11 * id; w[4] = c12 * id; w[5] = c22 * id;
}

// dU -= wgt (omega sig^ n) (x) n, symmetric and antisymmetric parts
template <typename R, typename G>
__device__ __forceinline__ void green_update(const G (&w)[6], const G *nd,
                                             const R (&sr)[6], const R (&si)[6],
                                             R (&ur)[6], R (&ui)[6], R (&ar)[3], R (&ai)[3],
                                             R wgt)
{
    R w00 = R(w[0]), w01 = R(w[1]), w02 = R(w[2]);
    R w11 = R(w[3]), w12 = R(w[4]), w22 = R(w[5]);
    R n0 = R(nd[0]), n1 = R(nd[1]), n2 = R(nd[2]);
    // t = sig^ n (sig^ symmetric: 00,11,22,12,02,01)
    R t0r = sr[0] * n0 + sr[5] * n1 + sr[4] * n2, t0i = si[0] * n0 + si[5] * n1 + si[4] * n2;
    R t1r = sr[5] * n0 + sr[1] * n1 + sr[3] * n2, t1i = si[5] * n0 + si[1] * n1 + si[3] * n2;
    R t2r = sr[4] * n0 + sr[3] * n1 + sr[2] * n2, t2i = si[4] * n0 + si[3] * n1 + si[2] * n2;
    R v0r = w00 * t0r + w01 * t1r + w02 * t2r, v0i = w00 * t0i + w01 * t1i + w02 * t2i;
    R v1r = w01 * t0r + w11 * t1r + w12 * t2r, v1i = w01 * t0i + w11 * t1i + w12 * t2i;
    R v2r = w02 * t0r + w12 * t1r + w22 * t2r, v2i = w02 * t0i + w12 * t1i + w22 * t2i;
    // dU = -v (x) n ; weight wgt (1 or 1/2 on the Nyquist planes)
    R h = -wgt;
    R hh = R(0.5) * h;
    ur[0] += h * v0r * n0;                 ui[0] += h * v0i * n0;
    ur[1] += h * v1r * n1;                 ui[1] += h * v1i * n1;
    ur[2] += h * v2r * n2;                 ui[2] += h * v2i * n2;
    ur[3] += hh * (v1r * n2 + v2r * n1);   ui[3] += hh * (v1i * n2 + v2i * n1);
    ur[4] += hh * (v0r * n2 + v2r * n0);   ui[4] += hh * (v0i * n2 + v2i * n0);
    ur[5] += hh * (v0r * n1 + v1r * n0);   ui[5] += hh * (v0i * n1 + v1i * n0);
    ar[0] += hh * (v1r * n2 - v2r * n1);   ai[0] += hh * (v1i * n2 - v2i * n1);
    ar[1] += hh * (v0r * n2 - v2r * n0);   ai[1] += hh * (v0i * n2 - v2i * n0);
    ar[2] += hh * (v0r * n1 - v1r * n0);   ai[2] += hh * (v0i * n1 - v1i * n0);
}

template <typename R, typename G>
__device__ __forceinline__ void green_rank1(const G *Kq, const G *nd,
                                            const R (&sr)[6], const R (&si)[6],
                                            R (&ur)[6], R (&ui)[6], R (&ar)[3], R (&ai)[3],
                                            R wgt)
{
    G w[6];
    green_omega<G>(Kq, nd, w);
    green_update<R, G>(w, nd, sr, si, ur, ui, ar, ai, wgt);
}

__device__ __forceinline__ const double *green_kq(const RveDesc &d, double *) { return d.Kq; }
__device__ __forceinline__ const float *green_kq(const RveDesc &d, float *) { return d.Kqf; }

// Apply the Green operator at frequency (ix,iy,iz), spectral index o.  In:
// B-basis stress spectrum (br, bi).  Out: B-basis symmetric update in
// (br, bi) and the antisymmetric update (ar, ai).  With d.gstore (FP64 form)
// the frequency's n and omega are read, else computed.
template <typename R>
__device__ __forceinline__ void green_apply(const RveDesc &d, int ix, int iy, int iz, long long o,
                                            R (&br)[6], R (&bi)[6], R (&ar)[3], R (&ai)[3])
{
    R sr[6], si[6], ur[6], ui[6];
    b_to_t6<R>(br, sr);
    b_to_t6<R>(bi, si);
#pragma unroll
    for (int a = 0; a < 6; ++a) { ur[a] = R(0); ui[a] = R(0); }
#pragma unroll
    for (int a = 0; a < 3; ++a) { ar[a] = R(0); ai[a] = R(0); }
    if ((ix | iy | iz) != 0) {
        typedef typename GreenT<R>::T G;
        const G *kq = green_kq(d, (G *)nullptr);
        G n[3], w[6];
        if (sizeof(G) == 8 && d.gstore) {
            const double *gs = d.gstore + o;
            const long long ns = d.nspec;
#pragma unroll
            for (int q = 0; q < 3; ++q) n[q] = (G)__ldg(gs + q * ns);
#pragma unroll
            for (int q = 0; q < 6; ++q) w[q] = (G)__ldg(gs + (3 + q) * ns);
        } else {
            unit_freq(d, ix, iy, iz, n);
            green_omega<G>(kq, n, w);
        }
        bool nyq = ((d.nx % 2 == 0) && ix == d.nx / 2) || ((d.ny % 2 == 0) && iy == d.ny / 2) ||
                   ((d.nz % 2 == 0) && iz == d.nz / 2);
        if (!nyq) {
            green_update<R, G>(w, n, sr, si, ur, ui, ar, ai, R(1));
        } else {
            G n2[3];
            unit_freq(d, (d.nx - ix) % d.nx, (d.ny - iy) % d.ny, (d.nz - iz) % d.nz, n2);
            green_update<R, G>(w, n, sr, si, ur, ui, ar, ai, R(0.5));
            green_rank1<R, G>(kq, n2, sr, si, ur, ui, ar, ai, R(0.5));
        }
    }
    t6_to_b<R>(ur, br);
    t6_to_b<R>(ui, bi);
}

// ---------------------------------------------------------------------------
// Shared-memory Stockham FFT over NL lines of length L.  Element (line l,
// index i) lives at buf[i * ldl + l].  sign -1: exp(-2 pi i jk/L) (forward),
// +1: inverse; unnormalised.  Returns the buffer holding the result.
// ---------------------------------------------------------------------------
template <typename R> struct Cx;
template <> struct Cx<double> { typedef double2 T; };
template <> struct Cx<float> { typedef float2 T; };

template <typename R>
__device__ __forceinline__ typename Cx<R>::T cmul(typename Cx<R>::T a, typename Cx<R>::T b)
{
    typename Cx<R>::T c;
    c.x = a.x * b.x - a.y * b.y;
    c.y = a.x * b.y + a.y * b.x;
    return c;
}

// ---------------------------------------------------------------------------
// Register FFT of the single-precision spectrum.  A line of length
// L = N1 N2 runs as two passes of small DFTs held in registers (the
// four-step Cooley-Tukey split).  Pass 1: for each t < N2, the N1 elements
// t + N2 j are transformed over j and output k1 is multiplied by W_L^(t k1),
// in place.  Pass 2: for each k1 < N1, those values over t are transformed
// and X[k1 + N1 k2] is written to the other buffer.  An element crosses
// shared memory twice (once per radix stage in the Stockham kernel below),
// and the small DFTs -- composed the same way from radix 2, 3 and 4 -- carry
// their twiddles as constants, with every index fixed at compile time.
// ---------------------------------------------------------------------------

// the split N1 of the lengths the register FFT runs (0: the Stockham kernel)
__host__ __device__ inline int reg_fft_split(int L)
{
    switch (L) {
    case 16: return 4;    // 4 x 4
    case 24: return 4;    // 4 x 6
    case 32: return 4;    // 4 x 8
    case 48: return 6;    // 6 x 8
    case 64: return 8;    // 8 x 8
    case 96: return 8;    // 8 x 12
    case 128: return 8;   // 8 x 16
    case 192: return 12;  // 12 x 16
    case 256: return 16;  // 16 x 16
    default: return 0;
    }
}

// cos(2 pi a / 48) for 0 <= a <= 12.  The small DFTs (N dividing 48) meet
// only angles a that are multiples of 3 (N = 16) or 4 (N = 12); the values
// are cos 0, cos pi/8 = sqrt(2 + sqrt 2) / 2, cos pi/6 = sqrt 3 / 2,
// cos pi/4 = sqrt 2 / 2, cos pi/3, cos 3pi/8 = sqrt(2 - sqrt 2) / 2, cos pi/2.
__host__ __device__ constexpr double cos_q48(int a)
{
    return a == 0 ? 1.0 : a == 3 ? 0.92387953251128675613 : a == 4 ? 0.86602540378443864676
         : a == 6 ? 0.70710678118654752440 : a == 8 ? 0.5 : a == 9 ? 0.38268343236508977173 : 0.0;
}
__host__ __device__ constexpr double cos48(int a)
{
    a = ((a % 48) + 48) % 48;
    return a <= 12 ? cos_q48(a) : a <= 24 ? -cos_q48(24 - a) : a <= 36 ? -cos_q48(a - 24) : cos_q48(48 - a);
}
__host__ __device__ constexpr double sin48(int a) { return cos48(a - 12); }

template <int I> struct IC { static constexpr int v = I; };
// f(IC<B>), f(IC<B + 1>), ..., f(IC<E - 1>)
template <int B, int E, class F>
__device__ __forceinline__ void sfor(F &&f)
{
    if constexpr (B < E) {
        f(IC<B>{});
        sfor<B + 1, E>(f);
    }
}

// v W_N^E, W_N = exp(S 2 pi i / N)
template <int N, int E, int S>
__device__ __forceinline__ float2 rot(float2 v)
{
    static_assert(48 % N == 0, "small DFT lengths divide 48");
    constexpr int a = (48 / N * E) % 48;
    static_assert(a % 3 == 0 || a % 4 == 0, "angle without a constant");
    if constexpr (a == 0) {
        return v;
    } else if constexpr (a == 24) {
        return make_float2(-v.x, -v.y);
    } else if constexpr (a == 12 || a == 36) {
        // W = g i, g = +-1
        constexpr int g = (a == 12 ? 1 : -1) * S;
        if constexpr (g > 0) return make_float2(-v.y, v.x);
        else return make_float2(v.y, -v.x);
    } else {
        constexpr float c = (float)cos48(a), s = (float)(S * sin48(a));
        return make_float2(c * v.x - s * v.y, c * v.y + s * v.x);
    }
}

// The small DFTs run in place on a strided view of a register array, the
// view's element i being x[O + T i].  Output q of an N-point DFT is left in
// view element dft_pos(N, q) (the four-step split transposes; placing the
// outputs in the registers the inputs came from needs no temporaries, and
// the caller indexes the permutation at compile time).
__host__ __device__ constexpr int dft_pos(int N, int q)
{
    return N <= 4 ? q
                  : dft_pos(N / (N % 4 == 0 ? 4 : 2), q / (N % 4 == 0 ? 4 : 2)) +
                        N / (N % 4 == 0 ? 4 : 2) * dft_pos(N % 4 == 0 ? 4 : 2, q % (N % 4 == 0 ? 4 : 2));
}

// X[q] = sum_n x[n] exp(S 2 pi i n q / N) over the view, X[q] left in view
// element dft_pos(N, q); N = A B composes radix 2, 3 and 4: A-point DFTs
// over n = t + B j for each t, twiddles W_N^(t k), B-point DFTs over t
template <int N, int S, int O, int T, int M>
__device__ __forceinline__ void sdft(float2 (&x)[M])
{
    if constexpr (N == 2) {
        const float2 a = x[O], b = x[O + T];
        x[O] = make_float2(a.x + b.x, a.y + b.y);
        x[O + T] = make_float2(a.x - b.x, a.y - b.y);
    } else if constexpr (N == 3) {
        constexpr float s3 = (float)(S * 0.86602540378443864676);
        const float2 x0 = x[O], x1 = x[O + T], x2 = x[O + 2 * T];
        const float2 u = make_float2(x1.x + x2.x, x1.y + x2.y);
        const float2 w = make_float2(x1.x - x2.x, x1.y - x2.y);
        const float2 m = make_float2(x0.x - 0.5f * u.x, x0.y - 0.5f * u.y);
        x[O] = make_float2(x0.x + u.x, x0.y + u.y);
        x[O + T] = make_float2(m.x - s3 * w.y, m.y + s3 * w.x);
        x[O + 2 * T] = make_float2(m.x + s3 * w.y, m.y - s3 * w.x);
    } else if constexpr (N == 4) {
        const float2 x0 = x[O], x1 = x[O + T], x2 = x[O + 2 * T], x3 = x[O + 3 * T];
        const float2 t0 = make_float2(x0.x + x2.x, x0.y + x2.y);
        const float2 t1 = make_float2(x0.x - x2.x, x0.y - x2.y);
        const float2 t2 = make_float2(x1.x + x3.x, x1.y + x3.y);
        const float2 t3 = make_float2(x1.x - x3.x, x1.y - x3.y);
        x[O] = make_float2(t0.x + t2.x, t0.y + t2.y);
        x[O + 2 * T] = make_float2(t0.x - t2.x, t0.y - t2.y);
        if constexpr (S < 0) {   // t1 -/+ i t3
            x[O + T] = make_float2(t1.x + t3.y, t1.y - t3.x);
            x[O + 3 * T] = make_float2(t1.x - t3.y, t1.y + t3.x);
        } else {
            x[O + T] = make_float2(t1.x - t3.y, t1.y + t3.x);
            x[O + 3 * T] = make_float2(t1.x + t3.y, t1.y - t3.x);
        }
    } else {
        constexpr int A = N % 4 == 0 ? 4 : 2, B = N / A;
        sfor<0, B>([&](auto tc) { sdft<A, S, O + T * decltype(tc)::v, T * B>(x); });
        sfor<1, B>([&](auto tc) {
            constexpr int t = decltype(tc)::v;
            sfor<1, A>([&](auto kc) {
                constexpr int k = decltype(kc)::v, r = O + T * (t + B * dft_pos(A, k));
                x[r] = rot<N, t * k, S>(x[r]);
            });
        });
        sfor<0, A>([&](auto kc) { sdft<B, S, O + T * B * dft_pos(A, decltype(kc)::v), T>(x); });
    }
}

// NL lines of length N1 N2 from a (element (l, i) at a[i * ldl + l]) into b;
// tw[e] = exp(-2 pi i e / L), followed by the pass-1 twiddle matrix
// tw[L + k N2 + t] = exp(-2 pi i t k / L) (conjugated for S = +1).  Pass 1's tasks are
// (l, t), pass 2's (l, k1), l fastest: consecutive threads read consecutive
// words of shared memory.
template <int N1, int N2, int S>
__device__ float2 *fft_reg(float2 *a, float2 *b, int NL, int ldl, const float2 *__restrict__ tw)
{
    const int tid = threadIdx.x, nthr = blockDim.x;
    const int dl = nthr % NL, dq = nthr / NL;
    {
        const int st = N2 * ldl;
        int l = tid % NL, t = tid / NL;
        for (int task = tid; task < NL * N2; task += nthr) {
            float2 *p = a + t * ldl + l;
            float2 x[N1];
#pragma unroll
            for (int j = 0; j < N1; ++j) x[j] = p[j * st];
            sdft<N1, S, 0, 1>(x);
            if (t != 0) {
                const float2 *wm = tw + N1 * N2 + t;   // the pass-1 twiddle matrix
                sfor<1, N1>([&](auto kc) {
                    constexpr int k = decltype(kc)::v, r = dft_pos(N1, k);
                    float2 w = __ldg(wm + k * N2);
                    if (S > 0) w.y = -w.y;
                    x[r] = cmul<float>(x[r], w);
                });
            }
            sfor<0, N1>([&](auto kc) { p[decltype(kc)::v * st] = x[dft_pos(N1, decltype(kc)::v)]; });
            l += dl;
            t += dq;
            if (l >= NL) { l -= NL; ++t; }
        }
    }
    __syncthreads();
    {
        const int sb = N1 * ldl;
        int l = tid % NL, k1 = tid / NL;
        for (int task = tid; task < NL * N1; task += nthr) {
            const float2 *p = a + N2 * k1 * ldl + l;
            float2 x[N2];
#pragma unroll
            for (int t = 0; t < N2; ++t) x[t] = p[t * ldl];
            sdft<N2, S, 0, 1>(x);
            float2 *q = b + k1 * ldl + l;
            sfor<0, N2>([&](auto kc) { q[decltype(kc)::v * sb] = x[dft_pos(N2, decltype(kc)::v)]; });
            l += dl;
            k1 += dq;
            if (l >= NL) { l -= NL; ++k1; }
        }
    }
    __syncthreads();
    return b;
}

__device__ __forceinline__ float2 *fft_reg_lines(float2 *a, float2 *b, int NL, int ldl, int L,
                                                 const float2 *__restrict__ tw, int sign)
{
#define VOCE_REG_FFT(L_, N1_) \
    case L_: return sign < 0 ? fft_reg<N1_, L_ / N1_, -1>(a, b, NL, ldl, tw) : fft_reg<N1_, L_ / N1_, 1>(a, b, NL, ldl, tw);
    switch (L) {
    VOCE_REG_FFT(16, 4)
    VOCE_REG_FFT(24, 4)
    VOCE_REG_FFT(32, 4)
    VOCE_REG_FFT(48, 6)
    VOCE_REG_FFT(64, 8)
    VOCE_REG_FFT(96, 8)
    VOCE_REG_FFT(128, 8)
    VOCE_REG_FFT(192, 12)
    VOCE_REG_FFT(256, 16)
    default: return nullptr;
    }
#undef VOCE_REG_FFT
}

template <typename R>
__device__ typename Cx<R>::T *fft_lines(typename Cx<R>::T *a, typename Cx<R>::T *b, int NL,
                                        int ldl, const FftPlan1 &pl,
                                        const typename Cx<R>::T *__restrict__ tw, int sign)
{
    typedef typename Cx<R>::T C;
    if constexpr (sizeof(R) == 4) {
        // the plan's split always matches reg_fft_split (the host sets both);
        // an unknown length falls through to the Stockham stages, which the
        // plan also holds
        if (pl.n1 && reg_fft_split(pl.L) == pl.n1) {
            C *res = fft_reg_lines(a, b, NL, ldl, pl.L, tw, sign);
            if (res) return res;
        }
    }
    const int L = pl.L;
    const int tid = threadIdx.x, nthr = blockDim.x;
    int ncur = L, s = 1;
    C *src = a, *dst = b;
    const R sg = R(sign);
    for (int st = 0; st < pl.nst; ++st) {
        const int r = pl.rad[st];
        const int m = ncur / r;
        const int nb = NL * (L / r);
        // butterfly bi = (p s + q) NL + l: the thread's first (l, q, p) and the
        // step to its next one (bi + nthr) by two divisions per stage, then
        // carried forward, instead of three divisions per butterfly
        int l = tid % NL, q = tid / NL, p = q / s;
        q -= p * s;
        const int dl = nthr % NL, dt = nthr / NL, dp = dt / s, dq = dt - dp * s;
        for (int bi = tid; bi < nb; bi += nthr) {
            C x[4], y[4];
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if (j < r) x[j] = src[(q + s * (p + j * m)) * ldl + l];
            if (r == 4) {
                C t0, t1, t2, t3;
                t0.x = x[0].x + x[2].x; t0.y = x[0].y + x[2].y;
                t1.x = x[0].x - x[2].x; t1.y = x[0].y - x[2].y;
                t2.x = x[1].x + x[3].x; t2.y = x[1].y + x[3].y;
                t3.x = x[1].x - x[3].x; t3.y = x[1].y - x[3].y;
                y[0].x = t0.x + t2.x;       y[0].y = t0.y + t2.y;
                y[2].x = t0.x - t2.x;       y[2].y = t0.y - t2.y;
                y[1].x = t1.x - sg * t3.y;  y[1].y = t1.y + sg * t3.x;
                y[3].x = t1.x + sg * t3.y;  y[3].y = t1.y - sg * t3.x;
            } else if (r == 2) {
                y[0].x = x[0].x + x[1].x; y[0].y = x[0].y + x[1].y;
                y[1].x = x[0].x - x[1].x; y[1].y = x[0].y - x[1].y;
            } else {  // r == 3
                const R c3 = R(-0.5), s3 = sg * R(0.86602540378443864676);
                C u;
                u.x = x[1].x + x[2].x; u.y = x[1].y + x[2].y;
                C w;
                w.x = x[1].x - x[2].x; w.y = x[1].y - x[2].y;
                y[0].x = x[0].x + u.x; y[0].y = x[0].y + u.y;
                C m0;
                m0.x = x[0].x + c3 * u.x; m0.y = x[0].y + c3 * u.y;
                y[1].x = m0.x - s3 * w.y; y[1].y = m0.y + s3 * w.x;
                y[2].x = m0.x + s3 * w.y; y[2].y = m0.y - s3 * w.x;
            }
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                if (k >= r) break;
                const int e = p * k * s;  // < L
                C w = tw[e];
                if (sign > 0) w.y = -w.y;
                C z = (e == 0) ? y[k] : cmul<R>(y[k], w);
                dst[(q + s * (r * p + k)) * ldl + l] = z;
            }
            // (l, q, p) of bi + nthr
            l += dl;
            int c = 0;
            if (l >= NL) { l -= NL; c = 1; }
            q += dq + c;
            p += dp;
            if (q >= s) { q -= s; p += 1; }
        }
        __syncthreads();
        ncur = m;
        s *= r;
        C *tt = src; src = dst; dst = tt;
    }
    return src;
}
