/*
 * Own mixed-radix Stockham FFT (double precision).  TEST INFRASTRUCTURE ONLY
 * (see fft_core.h).  Stages use radix 4 first, then 2, 3, 5, 7; twiddles are
 * evaluated once per plan in long double and rounded to double.
 */
#include "fft_core.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

struct fftc_plan1d {
    int n, sign, nst;
    int rad[40];
    double *tw; /* tw[2j], tw[2j+1] = cos, sin of sign*2*pi*j/n */
};

fftc_plan1d *fftc_plan1d_create(int n, int sign)
{
    if (n < 1 || (sign != 1 && sign != -1)) return NULL;
    fftc_plan1d *p = (fftc_plan1d *)calloc(1, sizeof(*p));
    p->n = n;
    p->sign = sign;
    int m = n, k = 0;
    while (m % 4 == 0) { p->rad[k++] = 4; m /= 4; }
    while (m % 2 == 0) { p->rad[k++] = 2; m /= 2; }
    while (m % 3 == 0) { p->rad[k++] = 3; m /= 3; }
    while (m % 5 == 0) { p->rad[k++] = 5; m /= 5; }
    while (m % 7 == 0) { p->rad[k++] = 7; m /= 7; }
    if (m != 1) { free(p); return NULL; }
    p->nst = k;
    p->tw = (double *)malloc(sizeof(double) * 2 * (size_t)n);
    const long double two_pi = 6.283185307179586476925286766559005768L;
    for (int j = 0; j < n; ++j) {
        long double a = two_pi * (long double)j / (long double)n;
        p->tw[2 * j] = (double)cosl(a);
        p->tw[2 * j + 1] = (double)(sign * sinl(a));
    }
    return p;
}

void fftc_plan1d_destroy(fftc_plan1d *p)
{
    if (!p) return;
    free(p->tw);
    free(p);
}

/* one Stockham pass: src and dst hold n contiguous complex values */
static void pass(const fftc_plan1d *P, int r, int n_cur, int s,
                 const double *src, double *dst)
{
    const int n = P->n, m = n_cur / r;
    const double *tw = P->tw;
    const double sg = (double)P->sign;
    double ar[8], ai[8], br[8], bi[8];
    for (int p = 0; p < m; ++p) {
        for (int q = 0; q < s; ++q) {
            for (int j = 0; j < r; ++j) {
                long idx = q + (long)s * (p + j * m);
                ar[j] = src[2 * idx];
                ai[j] = src[2 * idx + 1];
            }
            if (r == 2) {
                br[0] = ar[0] + ar[1]; bi[0] = ai[0] + ai[1];
                br[1] = ar[0] - ar[1]; bi[1] = ai[0] - ai[1];
            } else if (r == 4) {
                double t0r = ar[0] + ar[2], t0i = ai[0] + ai[2];
                double t1r = ar[0] - ar[2], t1i = ai[0] - ai[2];
                double t2r = ar[1] + ar[3], t2i = ai[1] + ai[3];
                double t3r = ar[1] - ar[3], t3i = ai[1] - ai[3];
                /* sign*i*(t3) = (-sign*t3i, sign*t3r) */
                br[0] = t0r + t2r;       bi[0] = t0i + t2i;
                br[2] = t0r - t2r;       bi[2] = t0i - t2i;
                br[1] = t1r - sg * t3i;  bi[1] = t1i + sg * t3r;
                br[3] = t1r + sg * t3i;  bi[3] = t1i - sg * t3r;
            } else {
                /* direct DFT of radix r with the plan's own table:
                 * w_r^(jk) = tw[(jk mod r) * n / r] */
                int step = n / r;
                for (int k = 0; k < r; ++k) {
                    double sr = 0.0, si = 0.0;
                    for (int j = 0; j < r; ++j) {
                        int e = ((j * k) % r) * step;
                        double c = tw[2 * e], sn = tw[2 * e + 1];
                        sr += ar[j] * c - ai[j] * sn;
                        si += ar[j] * sn + ai[j] * c;
                    }
                    br[k] = sr;
                    bi[k] = si;
                }
            }
            for (int k = 0; k < r; ++k) {
                long e = (long)p * k * s; /* < n */
                double c = tw[2 * e], sn = tw[2 * e + 1];
                long o = q + (long)s * (r * p + k);
                dst[2 * o] = br[k] * c - bi[k] * sn;
                dst[2 * o + 1] = br[k] * sn + bi[k] * c;
            }
        }
    }
}

void fftc_line(const fftc_plan1d *P, double *data, long stride, double *scratch)
{
    const int n = P->n;
    if (n == 1) return;
    double *a = scratch;           /* n complex */
    double *b = scratch + 2 * n;   /* n complex */
    for (int j = 0; j < n; ++j) {
        a[2 * j] = data[2 * j * stride];
        a[2 * j + 1] = data[2 * j * stride + 1];
    }
    int n_cur = n, s = 1;
    double *src = a, *dst = b;
    for (int st = 0; st < P->nst; ++st) {
        int r = P->rad[st];
        pass(P, r, n_cur, s, src, dst);
        n_cur /= r;
        s *= r;
        double *t = src; src = dst; dst = t;
    }
    for (int j = 0; j < n; ++j) {
        data[2 * j * stride] = src[2 * j];
        data[2 * j * stride + 1] = src[2 * j + 1];
    }
}

int fftc_3d(int nx, int ny, int nz, int sign, double *data, int nthreads)
{
    fftc_plan1d *pz = fftc_plan1d_create(nz, sign);
    fftc_plan1d *py = fftc_plan1d_create(ny, sign);
    fftc_plan1d *px = fftc_plan1d_create(nx, sign);
    if (!pz || !py || !px) {
        fftc_plan1d_destroy(pz); fftc_plan1d_destroy(py); fftc_plan1d_destroy(px);
        return -1;
    }
    int nmax = nx > ny ? nx : ny;
    if (nz > nmax) nmax = nz;
    if (nthreads < 1) nthreads = 1;
    (void)nthreads;
    /* z lines: contiguous */
#pragma omp parallel num_threads(nthreads)
    {
        double *scr = (double *)malloc(sizeof(double) * 4 * (size_t)nmax);
#pragma omp for schedule(static)
        for (long l = 0; l < (long)nx * ny; ++l)
            fftc_line(pz, data + 2 * l * nz, 1, scr);
        /* y lines: stride nz */
#pragma omp for schedule(static)
        for (long l = 0; l < (long)nx * nz; ++l) {
            long x = l / nz, z = l % nz;
            fftc_line(py, data + 2 * (x * (long)ny * nz + z), nz, scr);
        }
        /* x lines: stride ny*nz */
#pragma omp for schedule(static)
        for (long l = 0; l < (long)ny * nz; ++l)
            fftc_line(px, data + 2 * l, (long)ny * nz, scr);
        free(scr);
    }
    fftc_plan1d_destroy(pz); fftc_plan1d_destroy(py); fftc_plan1d_destroy(px);
    return 0;
}
