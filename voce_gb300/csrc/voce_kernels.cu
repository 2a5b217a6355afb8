// sm_103a kernels of the EVP-FFT solver step.  See voce_dev.cuh for the
// data layout.  One Green-operator iteration is
//   k_fft_z_fwd  -> k_fft_y(-1) -> k_fft_x_green -> k_fft_y(+1) ->
//   k_fft_z_inv(update) -> k_nr -> k_finalize_iter
// and an increment ends with
//   k_fft_x(+1,aacc) -> k_fft_y(+1,aacc) -> k_fft_z_inv(rotl) ->
//   k_incr_end -> k_finalize_incr
#include "voce_dev.cuh"
#include "voce_kernels.h"

#include <math.h>

#include <algorithm>
#include <atomic>

namespace voce {

// ---------------------------------------------------------------------------
// deterministic block reduction of VOCE_NPART partial sums (entry 15 is a max)
// ---------------------------------------------------------------------------
__device__ void block_partials(double (&acc)[VOCE_NPART], double *out)
{
    __shared__ double red[32][VOCE_NPART];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < VOCE_NPART; ++q) {
        double x = acc[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            double y = __shfl_down_sync(0xffffffffu, x, o);
            x = (q == VOCE_NPART - 1) ? fmax(x, y) : x + y;
        }
        if (lane == 0) red[warp][q] = x;
    }
    __syncthreads();
    if (threadIdx.x < VOCE_NPART) {
        const int q = threadIdx.x, nw = (blockDim.x + 31) >> 5;
        double s = red[0][q];
        for (int w = 1; w < nw; ++w) s = (q == VOCE_NPART - 1) ? fmax(s, red[w][q]) : s + red[w][q];
        out[q] = s;
    }
    __syncthreads();
}

// sum the per-block partials of one kernel in a fixed order (one block of
// 256 threads): thread t takes quantity t % 16 over stripe t / 16, a run of
// consecutive blocks, with up to 32 loads in flight and a pairwise tree over
// them; the 16 stripe sums are then added pairwise too.  Entry 15 is a max
// (of non-negative counts, so 0 is its identity as for the sums).
__device__ void reduce_partials(const double *part, int npart, double (&tot)[VOCE_NPART])
{
    __shared__ double red[16][VOCE_NPART];
    const int t = threadIdx.x;  // blockDim.x == 256
    const int q = t % VOCE_NPART, stripe = t / VOCE_NPART;
    const bool mx = q == VOCE_NPART - 1;
    const int chunk = (npart + 15) / 16;
    const int b0 = stripe * chunk, b1 = min(npart, b0 + chunk);
    double s = 0.0;
    for (int b = b0; b < b1; b += 32) {
        double x[32];
#pragma unroll
        for (int k = 0; k < 32; ++k) x[k] = (b + k < b1) ? part[(long long)(b + k) * VOCE_NPART + q] : 0.0;
#pragma unroll
        for (int w = 16; w >= 1; w >>= 1)
#pragma unroll
            for (int k = 0; k < w; ++k) x[k] = mx ? fmax(x[k], x[k + w]) : x[k] + x[k + w];
        s = mx ? fmax(s, x[0]) : s + x[0];
    }
    red[stripe][q] = s;
    __syncthreads();
    if (t < VOCE_NPART) {
        double v[16];
#pragma unroll
        for (int k = 0; k < 16; ++k) v[k] = red[k][t];
#pragma unroll
        for (int w = 8; w >= 1; w >>= 1)
#pragma unroll
            for (int k = 0; k < w; ++k) v[k] = mx ? fmax(v[k], v[k + w]) : v[k] + v[k + w];
        red[0][t] = v[0];
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < VOCE_NPART; ++k) tot[k] = red[0][k];
    __syncthreads();
}

// rotation of the 6-vector basis: x_sample = Mr * x_crystal for the
// tensor map X -> a^T X a (a = sample->crystal matrix, TranMat = a^T):
// Mr[b][c] = <B_b, a^T B_c a>
__device__ void rotation_B(const double (&a)[3][3], double (&Mr)[6][6])
{
    for (int c = 0; c < 6; ++c) {
        double bc6[6] = {0, 0, 0, 0, 0, 0};
        bc6[c] = 1.0;
        double t6[6];
        b_to_t6<double>(bc6, t6);
        double X[3][3] = {{t6[0], t6[5], t6[4]}, {t6[5], t6[1], t6[3]}, {t6[4], t6[3], t6[2]}};
        double Y[3][3], Z[3][3];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                double s = 0.0;
                for (int m = 0; m < 3; ++m) s += X[i][m] * a[m][j];
                Y[i][j] = s;  // X a
            }
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                double s = 0.0;
                for (int m = 0; m < 3; ++m) s += a[m][i] * Y[m][j];
                Z[i][j] = s;  // a^T X a
            }
        double z6[6] = {Z[0][0], Z[1][1], Z[2][2], 0.5 * (Z[1][2] + Z[2][1]),
                        0.5 * (Z[0][2] + Z[2][0]), 0.5 * (Z[0][1] + Z[1][0])};
        double col[6];
        t6_to_b<double>(z6, col);
        for (int b = 0; b < 6; ++b) Mr[b][c] = col[b];
    }
}

// EulerToTransMatrix opt 2 (kinematics.c:529-545)
__device__ void euler_a(double t1, double ph, double t2, double (&a)[3][3])
{
    double ct1 = cos(t1), st1 = sin(t1), cph = cos(ph), sph = sin(ph), ct2 = cos(t2), st2 = sin(t2);
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

__device__ void schmid_from_tm(const RveDesc &d, long long v, const double (&T)[3][3])
{
    double a[3][3], Mr[6][6];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) a[i][j] = T[j][i];
    rotation_B(a, Mr);
    for (int s = 0; s < d.nsys; ++s)
        for (int i = 0; i < 5; ++i) {
            double acc = 0.0;
            for (int c = 0; c < 5; ++c) acc += Mr[i][c] * d.schxt[5 * s + c];
            d.sch[(long long)(5 * s + i) * d.nv + v] = acc;
            if (d.sch32) put_pair(d.sch32, d.sch_lo, (long long)(5 * s + i) * d.nv + v, acc);
        }
}

// ---------------------------------------------------------------------------
// setup: per-voxel rotation, grain stiffness/compliance, Schmid tensors,
// initial stress (InitMicroStruct init.c:393-442, InitFields init.c:486-534,
// update_schmid kinematics.c:426-459 for istep 1)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_setup(RveDesc d, SetupConst sc, const double *__restrict__ euler)
{
    double acc[VOCE_NPART];
    double cacc[36];
    for (int q = 0; q < VOCE_NPART; ++q) acc[q] = 0.0;
    for (int q = 0; q < 36; ++q) cacc[q] = 0.0;
    const long long nv = d.nv;
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < nv;
         v += (long long)gridDim.x * blockDim.x) {
        const int ph = d.phase[v];
        for (int c = 0; c < 6; ++c) {
            d.eps[c < 5 ? c * nv + v : v] = 0.0;
            d.dgs[c * nv + v] = 0.0;
        }
        for (int c = 0; c < 3; ++c) d.dga[c * nv + v] = 0.0;
        d.gamacum[v] = 0.0;
        for (int k = 0; k < VOCE_NS; ++k) {
            d.gtot[k * nv + v] = 0.0;
            d.gamdot[k * nv + v] = 0.0;
            d.taux[k * nv + v] = 0.0;
        }
        for (int c = 0; c < 5; ++c) d.edot[c * nv + v] = 0.0;
        d.svm[v] = 0.0;
        d.evm[v] = 0.0;
        for (int c = 0; c < 3; ++c) d.diag[c * nv + v] = 0.0;
        if (!d.solid[ph]) {
            for (int c = 0; c < 6; ++c) { d.sig[c * nv + v] = 0.0; d.sigp[c * nv + v] = 0.0; }
            for (int c = 0; c < 9; ++c) d.tm[c * nv + v] = (c % 4 == 0) ? 1.0 : 0.0;
            for (int c = 0; c < 21; ++c) d.sg[c * nv + v] = 0.0;
            for (int c = 0; c < 60; ++c) d.sch[c * nv + v] = 0.0;
            if (d.sch32)
                for (int c = 0; c < 60; ++c) put_pair(d.sch32, d.sch_lo, c * nv + v, 0.0);
            for (int c = 0; c < 24; ++c) { d.crss[c * nv + v] = 0.0; d.itau[c * nv + v] = 0.0; }
            if (d.itau32)
                for (int c = 0; c < 24; ++c) put_pair(d.itau32, d.itau_lo, c * nv + v, 0.0);
            continue;
        }
        acc[0] += 1.0;
        double a[3][3], Mr[6][6];
        const double f = VOCE_PI_REF / 180.;
        euler_a(euler[3 * v] * f, euler[3 * v + 1] * f, euler[3 * v + 2] * f, a);
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) d.tm[(3 * i + j) * nv + v] = a[j][i];
        rotation_B(a, Mr);
        // C_gr = Mr Cxt Mr^T, S_g = Mr Sxt Mr^T
        double Cg[6][6], Sg[6][6];
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j < 6; ++j) {
                double sC = 0.0, sS = 0.0;
                for (int k = 0; k < 6; ++k) {
                    double tC = 0.0, tS = 0.0;
                    for (int l = 0; l < 6; ++l) {
                        tC += sc.cxt[k * 6 + l] * Mr[j][l];
                        tS += sc.sxt[k * 6 + l] * Mr[j][l];
                    }
                    sC += Mr[i][k] * tC;
                    sS += Mr[i][k] * tS;
                }
                Cg[i][j] = sC;
                Sg[i][j] = sS;
            }
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j < 6; ++j) cacc[i * 6 + j] += Cg[i][j];
        for (int i = 0; i < 6; ++i)
            for (int j = i; j < 6; ++j) d.sg[(long long)sym6(i, j) * nv + v] = 0.5 * (Sg[i][j] + Sg[j][i]);
        // initial stress: C_gr : DisGradAvg (+ Scauchy under creep)
        for (int i = 0; i < 6; ++i) {
            double s = 0.0;
            for (int j = 0; j < 6; ++j) s += Cg[i][j] * sc.d6[j];
            if (d.creep) s += sc.sc6[i];
            d.sig[i * nv + v] = s;
            d.sigp[i * nv + v] = s;
        }
        for (int k = 0; k < d.nsys; ++k) {
            d.crss[(2 * k) * nv + v] = d.tau0[k];
            d.crss[(2 * k + 1) * nv + v] = d.tau0b[k];
            d.itau[(2 * k) * nv + v] = 1.0 / d.tau0[k];
            d.itau[(2 * k + 1) * nv + v] = 1.0 / d.tau0b[k];
            if (d.itau32) {
                put_pair(d.itau32, d.itau_lo, (2 * k) * nv + v, 1.0 / d.tau0[k]);
                put_pair(d.itau32, d.itau_lo, (2 * k + 1) * nv + v, 1.0 / d.tau0b[k]);
            }
        }
        double T[3][3];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) T[i][j] = a[j][i];
        schmid_from_tm(d, v, T);
    }
    // voxel count and C066 partial sums (37 values) in three passes of 15
    // (the 16th slot of block_partials is a max and stays unused)
    double tmp[VOCE_NPART];
    for (int pass = 0; pass < 3; ++pass) {
        for (int q = 0; q < VOCE_NPART - 1; ++q) {
            const int idx = pass * (VOCE_NPART - 1) + q;
            tmp[q] = (idx == 0) ? acc[0] : ((idx - 1 < 36) ? cacc[idx - 1] : 0.0);
        }
        tmp[VOCE_NPART - 1] = 0.0;
        block_partials(tmp, d.part + ((long long)pass * gridDim.x + blockIdx.x) * VOCE_NPART);
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Asynchronous global -> shared copies (cp.async): the data lands in shared
// memory without passing through registers, so a thread can have every
// element of its share of a tile in flight at once; cp_async_wait_all waits
// for all of this thread's outstanding copies (a __syncthreads then makes
// them visible to the block).  4 and 8 bytes are cached in L1 and L2, 16
// bytes in L2 only; both addresses aligned to the size.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void cp_async4(float *smem, const float *gmem)
{
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(sa), "l"(__cvta_generic_to_global(gmem)) : "memory");
}

__device__ __forceinline__ void cp_async8(void *smem, const void *gmem)
{
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(sa), "l"(__cvta_generic_to_global(gmem)) : "memory");
}

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem)
{
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sa), "l"(__cvta_generic_to_global(gmem)) : "memory");
}

__device__ __forceinline__ void cp_async_wait_all()
{
    asm volatile("cp.async.wait_all;" ::: "memory");
}

// ---------------------------------------------------------------------------
// FFT passes
// ---------------------------------------------------------------------------
// Position (a0, a1, a2) of a flat tile index i = a0 + n0 (a1 + n1 a2),
// carried from one element of a thread to its next (i += step) by additions
// and compares: a tile loop pays the integer divisions by the run-time tile
// extents once per thread instead of once per element (those divisions were
// most of the instructions of the FFT passes' load and store loops).
struct Idx3 {
    int a0, a1, a2, d0, d1, d2, n0, n1;
    __device__ __forceinline__ Idx3(int i, int step, int n0_, int n1_) : n0(n0_), n1(n1_)
    {
        int t = i / n0;
        a0 = i - t * n0;
        a1 = t % n1;
        a2 = t / n1;
        t = step / n0;
        d0 = step - t * n0;
        d1 = t % n1;
        d2 = t / n1;
    }
    __device__ __forceinline__ void next()
    {
        a0 += d0;
        int c = a0 >= n0;
        if (c) a0 -= n0;
        a1 += d1 + c;
        c = a1 >= n1;
        if (c) a1 -= n1;
        a2 += d2 + c;
    }
};
constexpr int kIdxUnbounded = 1 << 30;   // n1 of a two-level index (a2 stays 0)

// Tile copy of n elements by the block over a carried index: each thread
// first loads U elements (its i, i + nthr, ...) into registers, then stores
// them, so that U global loads per thread are in flight at once.
// ld(a0, a1, a2) returns an element, st(a0, a1, a2, value) places it.
template <int U, typename T, class LD, class ST>
__device__ __forceinline__ void staged_copy3(int n, int n0, int n1, LD ld, ST st)
{
    const int nt = blockDim.x;
    Idx3 il(threadIdx.x, nt, n0, n1), is = il;
    for (int b = threadIdx.x; b < n; b += U * nt) {
        T v[U];
#pragma unroll
        for (int j = 0; j < U; ++j) {
            if (b + j * nt < n) v[j] = ld(il.a0, il.a1, il.a2);
            il.next();
        }
#pragma unroll
        for (int j = 0; j < U; ++j) {
            if (b + j * nt < n) st(is.a0, is.a1, is.a2, v[j]);
            is.next();
        }
    }
}

// loads in flight per thread: the single-precision passes wait on memory, the
// double-precision ones on the FP64 pipe (there one at a time, as before,
// keeps their registers and occupancy)
template <typename R> struct CopyDepth { static constexpr int v = 8; };
template <> struct CopyDepth<double> { static constexpr int v = 1; };
// the z passes gather strided columns and convert: measured slower with
// deeper copies (more registers, fewer resident blocks), so one at a time
constexpr int kZCopyDepth = 1;

// the stress's six components into the spectrum (evolution.c:350-361)
template <typename R>
__device__ void fft_z_fwd_unit(const RveDesc &d, int rows, int unit)
{
    typedef typename Cx<R>::T C;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *bufA = reinterpret_cast<C *>(smem_raw);
    const int nx = d.nx, ny = d.ny, nz = d.nz, nzh = d.nzh;
    const long long nv = d.nv;
    const int NL = 3 * rows, ldl = NL | 1;
    C *bufB = bufA + nz * ldl;
    const int ytiles = ny / rows;
    const int x = unit / ytiles, y0 = (unit % ytiles) * rows;
    const long long vb = ((long long)x * ny + y0) * nz;
    if constexpr (sizeof(R) == 4) {
        // rows y0 .. y0 + rows - 1 of a component are one run of rows * nz
        // doubles (z fastest): the six runs are staged behind bufA by
        // 16-byte asynchronous copies, then converted into the line layout
        double *stage = reinterpret_cast<double *>(bufB);
        const int run = rows * nz, half_run = run / 2;   // nz is even
        Idx3 ic(threadIdx.x, blockDim.x, half_run, kIdxUnbounded);
        for (int i = threadIdx.x; i < 6 * half_run; i += blockDim.x, ic.next())
            cp_async16(stage + 2 * i, d.sig + ic.a1 * nv + vb + 2 * ic.a0);
        cp_async_wait_all();
        __syncthreads();
        // element (z, r, p): components 2p and 2p + 1 of row r
        Idx3 ix(threadIdx.x, blockDim.x, nz, rows);
        for (int i = threadIdx.x; i < 3 * run; i += blockDim.x, ix.next()) {
            const int z = ix.a0, r = ix.a1, p = ix.a2, q = r * nz + z;
            bufA[z * ldl + p * rows + r] = make_float2((float)stage[2 * p * run + q], (float)stage[(2 * p + 1) * run + q]);
        }
    } else {
        // element (z, r, c) is sig[c][vb + r * nz + z]
        staged_copy3<kZCopyDepth, double>(
            6 * rows * nz, nz, rows,
            [&](int z, int r, int c) { return __ldg(d.sig + c * nv + vb + (long long)r * nz + z); },
            [&](int z, int r, int c, double v) {
                C *e = &bufA[z * ldl + (c >> 1) * rows + r];
                if (c & 1) e->y = (R)v; else e->x = (R)v;
            });
    }
    __syncthreads();
    C *res = fft_lines<R>(bufA, bufB, NL, ldl, d.plz, (const C *)d.twz, -1);
    C *spec = (C *)d.spec;
    const long long plane = (long long)nx * ny;
    Idx3 ix(threadIdx.x, blockDim.x, rows, nzh);
    for (int idx = threadIdx.x; idx < 3 * rows * nzh; idx += blockDim.x, ix.next()) {
        const int r = ix.a0, k = ix.a1, p = ix.a2;
        const int l = p * rows + r;
        const C zk = res[k * ldl + l], zm = res[((nz - k) % nz) * ldl + l];
        C A, B;
        A.x = R(0.5) * (zk.x + zm.x);
        A.y = R(0.5) * (zk.y - zm.y);
        B.x = R(0.5) * (zk.y + zm.y);
        B.y = R(-0.5) * (zk.x - zm.x);
        const long long o = (long long)k * plane + (long long)x * ny + y0 + r;
        spec[(long long)(2 * p) * nzh * plane + o] = A;
        spec[(long long)(2 * p + 1) * nzh * plane + o] = B;
    }
}


// forward r2c along z of ncomp real fields src[c][nv] into the half
// spectrum dstp[c][nzh][nx][ny]: two fields per complex line (an odd count
// pads the last line with zeros), split by the Hermitian symmetry of each
template <typename R, int ncomp>
__device__ void fft_z_fwd_src(const RveDesc &d, const double *src, void *dstp, int rows, int unit)
{
    typedef typename Cx<R>::T C;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *bufA = reinterpret_cast<C *>(smem_raw);
    const int nx = d.nx, ny = d.ny, nz = d.nz, nzh = d.nzh;
    const long long nv = d.nv;
    const int np = (ncomp + 1) / 2;
    const int NL = np * rows, ldl = NL | 1;
    C *bufB = bufA + nz * ldl;
    const int ytiles = ny / rows;
    const int x = unit / ytiles, y0 = (unit % ytiles) * rows;
    const long long vb = ((long long)x * ny + y0) * nz;
    Idx3 iz(threadIdx.x, blockDim.x, nz, rows);
    for (int idx = threadIdx.x; idx < 2 * np * rows * nz; idx += blockDim.x, iz.next()) {
        const int z = iz.a0, r = iz.a1, c = iz.a2;
        const R val = (ncomp % 2 == 0 || c < ncomp) ? (R)__ldg(src + c * nv + vb + (long long)r * nz + z) : R(0);
        C *e = &bufA[z * ldl + (c >> 1) * rows + r];
        if (c & 1) e->y = val; else e->x = val;
    }
    __syncthreads();
    C *res = fft_lines<R>(bufA, bufB, NL, ldl, d.plz, (const C *)d.twz, -1);
    C *spec = (C *)dstp;
    const long long plane = (long long)nx * ny;
    Idx3 ix(threadIdx.x, blockDim.x, rows, nzh);
    for (int idx = threadIdx.x; idx < np * rows * nzh; idx += blockDim.x, ix.next()) {
        const int r = ix.a0, k = ix.a1, p = ix.a2;
        const int l = p * rows + r;
        const C zk = res[k * ldl + l], zm = res[((nz - k) % nz) * ldl + l];
        C A, B;
        A.x = R(0.5) * (zk.x + zm.x);
        A.y = R(0.5) * (zk.y - zm.y);
        B.x = R(0.5) * (zk.y + zm.y);
        B.y = R(-0.5) * (zk.x - zm.x);
        const long long o = (long long)k * plane + (long long)x * ny + y0 + r;
        spec[(long long)(2 * p) * nzh * plane + o] = A;
        if (ncomp % 2 == 0 || 2 * p + 1 < ncomp) spec[(long long)(2 * p + 1) * nzh * plane + o] = B;
    }
}



template <typename R>
__device__ void fft_y_unit(const RveDesc &d, void *specp, int sign, int xt, int unit)
{
    typedef typename Cx<R>::T C;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *bufA = reinterpret_cast<C *>(smem_raw);
    const int nx = d.nx, ny = d.ny;
    const int NL = xt, ldl = NL | 1;
    C *bufB = bufA + ny * ldl;
    const int xtiles = nx / xt;
    const int line = unit / xtiles;  // c * nzh + kz
    const int x0 = (unit % xtiles) * xt;
    C *spec = (C *)specp;
    const long long base = ((long long)line * nx + x0) * ny;
    // element (y, xl) is spec[base + xl * ny + y]
    if constexpr (sizeof(R) == 4) {
        Idx3 il(threadIdx.x, blockDim.x, ny, kIdxUnbounded);
        for (int i = threadIdx.x; i < xt * ny; i += blockDim.x, il.next())
            cp_async8(&bufA[il.a0 * ldl + il.a1], spec + base + i);
        cp_async_wait_all();
    } else {
        staged_copy3<CopyDepth<R>::v, C>(
            xt * ny, ny, kIdxUnbounded, [&](int y, int xl, int) { return spec[base + xl * ny + y]; },
            [&](int y, int xl, int, C v) { bufA[y * ldl + xl] = v; });
    }
    __syncthreads();
    C *res = fft_lines<R>(bufA, bufB, NL, ldl, d.ply, (const C *)d.twy, sign);
    Idx3 ix(threadIdx.x, blockDim.x, ny, kIdxUnbounded);
    for (int idx = threadIdx.x; idx < xt * ny; idx += blockDim.x, ix.next())
        spec[base + idx] = res[ix.a0 * ldl + ix.a1];
}


// ---------------------------------------------------------------------------
// The y pass of the single-precision spectrum as a stream over a block's
// units, for plans whose RVEs all run the register FFT along y.  A unit's
// tile (NL = yxt lines of L = ny contiguous coefficients) is held line by
// line at pos(l, i) = l LP + i + i / N2, LP = L + N1 + 1: pass 1 (tasks
// (t, l), t fastest) and pass 2 (tasks (k1, l), k1 fastest) then read rows
// of consecutive words, and pass 2 writes X[k1 + N1 k2] of line l straight
// to the spectrum, consecutive threads to consecutive coefficients.  The
// next unit's tile is staged by cp.async while this one transforms (two
// tile buffers of S complex floats, S >= NL LP of every RVE of the plan).
// ---------------------------------------------------------------------------
template <int N1, int N2, int S>
__device__ __forceinline__ void ystream_tile(float2 *A, int NL, float2 *g, const float2 *__restrict__ tw)
{
    constexpr int L = N1 * N2, LP = L + N1 + 1;
    const int tid = threadIdx.x, nthr = blockDim.x;
    for (int task = tid; task < NL * N2; task += nthr) {
        const int l = task / N2, t = task - l * N2;
        float2 *p = A + l * LP + t;
        float2 x[N1];
        sfor<0, N1>([&](auto jc) { x[decltype(jc)::v] = p[(N2 + 1) * decltype(jc)::v]; });
        sdft<N1, S, 0, 1>(x);
        if (t != 0) {
            const float2 *wm = tw + L + t;   // the pass-1 twiddle matrix
            sfor<1, N1>([&](auto kc) {
                constexpr int k = decltype(kc)::v, r = dft_pos(N1, k);
                float2 w = __ldg(wm + k * N2);
                if (S > 0) w.y = -w.y;
                x[r] = cmul<float>(x[r], w);
            });
        }
        sfor<0, N1>([&](auto kc) { p[(N2 + 1) * decltype(kc)::v] = x[dft_pos(N1, decltype(kc)::v)]; });
    }
    __syncthreads();
    for (int task = tid; task < NL * N1; task += nthr) {
        const int l = task / N1, k1 = task - l * N1;
        const float2 *p = A + l * LP + (N2 + 1) * k1;
        float2 x[N2];
#pragma unroll
        for (int t = 0; t < N2; ++t) x[t] = p[t];
        sdft<N2, S, 0, 1>(x);
        float2 *q = g + l * L + k1;
        sfor<0, N2>([&](auto kc) { q[N1 * decltype(kc)::v] = x[dft_pos(N2, decltype(kc)::v)]; });
    }
}

template <typename R>
__device__ void fft_x_green_unit(const RveDesc &d, int kc, int unit)
{
    typedef typename Cx<R>::T C;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *bufA = reinterpret_cast<C *>(smem_raw);
    const int nx = d.nx, ny = d.ny, nzh = d.nzh;
    const int NL = 6 * kc, ldl = NL | 1;
    C *bufB = bufA + nx * ldl;
    const int ytiles = ny / kc;
    const int kz = unit / ytiles, y0 = (unit % ytiles) * kc;
    C *spec = (C *)d.spec;
    C *aacc = (C *)d.aacc;
    const long long plane = (long long)nx * ny, cstride = (long long)nzh * plane;
    const long long kb = (long long)kz * plane + y0;
    // element (yl, x, c) is spec[c][kz][x][y0 + yl]
    if constexpr (sizeof(R) == 4) {
        Idx3 il(threadIdx.x, blockDim.x, kc, nx);
        for (int i = threadIdx.x; i < 6 * nx * kc; i += blockDim.x, il.next())
            cp_async8(&bufA[il.a0 + il.a1 * ldl + il.a2 * kc],
                      spec + il.a2 * cstride + kb + (long long)il.a1 * ny + il.a0);
        cp_async_wait_all();
    } else {
        staged_copy3<CopyDepth<R>::v, C>(
            6 * nx * kc, kc, nx,
            [&](int yl, int x, int c) { return spec[c * cstride + kb + (long long)x * ny + yl]; },
            [&](int yl, int x, int c, C v) { bufA[x * ldl + c * kc + yl] = v; });
    }
    __syncthreads();
    C *res = fft_lines<R>(bufA, bufB, NL, ldl, d.plx, (const C *)d.twx, -1);
    C *oth = (res == bufA) ? bufB : bufA;
    const int first = d.macro->first_iter;
    // single precision: the accumulator's tile, acc[(c nx + x) kc + yl], is
    // staged in the free line buffer while the Green loop's operands wait
    C *acc = oth;
    if constexpr (sizeof(R) == 4) {
        if (!first) {
            Idx3 il(threadIdx.x, blockDim.x, kc, nx);
            for (int i = threadIdx.x; i < 3 * nx * kc; i += blockDim.x, il.next())
                cp_async8(acc + i, aacc + il.a2 * cstride + kb + (long long)il.a1 * ny + il.a0);
            cp_async_wait_all();
            __syncthreads();
        }
    }
    Idx3 ig(threadIdx.x, blockDim.x, kc, kIdxUnbounded);
    for (int idx = threadIdx.x; idx < nx * kc; idx += blockDim.x, ig.next()) {
        const int yl = ig.a0, x = ig.a1;
        R br[6], bi[6], ar[3], ai[3];
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            const C e = res[x * ldl + c * kc + yl];
            br[c] = e.x;
            bi[c] = e.y;
        }
        green_apply<R>(d, x, y0 + yl, kz, kb + (long long)x * ny + yl, br, bi, ar, ai);
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            C e;
            e.x = br[c];
            e.y = bi[c];
            res[x * ldl + c * kc + yl] = e;
        }
        const long long o = kb + (long long)x * ny + yl;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            C e;
            if (first) { e.x = ar[c]; e.y = ai[c]; }
            else {
                if constexpr (sizeof(R) == 4) e = acc[(c * nx + x) * kc + yl];
                else e = aacc[c * cstride + o];
                e.x += ar[c];
                e.y += ai[c];
            }
            aacc[c * cstride + o] = e;
        }
    }
    __syncthreads();
    C *res2 = fft_lines<R>(res, oth, NL, ldl, d.plx, (const C *)d.twx, +1);
    Idx3 is(threadIdx.x, blockDim.x, kc, nx);
    for (int idx = threadIdx.x; idx < 6 * nx * kc; idx += blockDim.x, is.next()) {
        const int yl = is.a0, x = is.a1, c = is.a2;
        spec[c * cstride + kb + (long long)x * ny + yl] = res2[x * ldl + c * kc + yl];
    }
}


// ---------------------------------------------------------------------------
// The x pass with the Green operator for an RVE on the register FFT along x
// (single precision).  The tile's NL = 6 kc lines (line l = c kc + yl:
// component c, column y0 + yl) are held line by line at pos(l, i) = l LP +
// i + i / N2, LP = L + N1 + 1 (odd): the forward transform runs in place on
// A and leaves X[k] at pos(l, k) of B, the Green operator works on B, the
// inverse transform runs in place on B and its second pass writes straight
// to the spectrum.  Every shared-memory index inside the transforms is a
// compile-time offset from one base per task.
// ---------------------------------------------------------------------------
template <int N1, int N2, int S>
__device__ __forceinline__ void xg_pass1(float2 *A, int NL, const float2 *__restrict__ tw)
{
    constexpr int L = N1 * N2, LP = L + N1 + 1;
    for (int task = threadIdx.x; task < NL * N2; task += blockDim.x) {
        const int l = task / N2, t = task - l * N2;
        float2 *p = A + l * LP + t;
        float2 x[N1];
        sfor<0, N1>([&](auto jc) { x[decltype(jc)::v] = p[(N2 + 1) * decltype(jc)::v]; });
        sdft<N1, S, 0, 1>(x);
        if (t != 0) {
            const float2 *wm = tw + L + t;   // the pass-1 twiddle matrix
            sfor<1, N1>([&](auto kc) {
                constexpr int k = decltype(kc)::v, r = dft_pos(N1, k);
                float2 w = __ldg(wm + k * N2);
                if (S > 0) w.y = -w.y;
                x[r] = cmul<float>(x[r], w);
            });
        }
        sfor<0, N1>([&](auto kc) { p[(N2 + 1) * decltype(kc)::v] = x[dft_pos(N1, decltype(kc)::v)]; });
    }
}

template <int N1, int N2>
__device__ void xg_unit_f32(const RveDesc &d, int kc, int unit)
{
    constexpr int L = N1 * N2, LP = L + N1 + 1;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2 *A = reinterpret_cast<float2 *>(smem_raw);
    const int NL = 6 * kc;
    float2 *B = A + NL * LP;
    const int ny = d.ny, nzh = d.nzh;
    const int ytiles = ny / kc;
    const int kz = unit / ytiles, y0 = (unit % ytiles) * kc;
    float2 *spec = (float2 *)d.spec, *aacc = (float2 *)d.aacc;
    const long long plane = (long long)L * ny, cstride = (long long)nzh * plane;
    const long long kb = (long long)kz * plane + y0;
    const float2 *tw = (const float2 *)d.twx;
    const int tid = threadIdx.x, nthr = blockDim.x;
    {   // element (yl, x, c), yl fastest
        Idx3 il(tid, nthr, kc, L);
        for (int i = tid; i < NL * L; i += nthr, il.next()) {
            const int yl = il.a0, x = il.a1, c = il.a2;
            cp_async8(A + (c * kc + yl) * LP + x + x / N2, spec + c * cstride + kb + (long long)x * ny + yl);
        }
        cp_async_wait_all();
    }
    __syncthreads();
    xg_pass1<N1, N2, -1>(A, NL, tw);
    __syncthreads();
    for (int task = tid; task < NL * N1; task += nthr) {
        const int l = task / N1, k1 = task - l * N1;
        const float2 *p = A + l * LP + (N2 + 1) * k1;
        float2 x[N2];
#pragma unroll
        for (int t = 0; t < N2; ++t) x[t] = p[t];
        sdft<N2, -1, 0, 1>(x);
        float2 *q = B + l * LP;
        sfor<0, N2>([&](auto mc) {
            const int k = k1 + N1 * decltype(mc)::v;
            q[k + k / N2] = x[dft_pos(N2, decltype(mc)::v)];
        });
    }
    __syncthreads();
    // the accumulator's tile, acc[(c L + x) kc + yl], staged in the free A
    const int first = d.macro->first_iter;
    if (!first) {
        Idx3 il(tid, nthr, kc, L);
        for (int i = tid; i < 3 * L * kc; i += nthr, il.next())
            cp_async8(A + i, aacc + il.a2 * cstride + kb + (long long)il.a1 * ny + il.a0);
        cp_async_wait_all();
        __syncthreads();
    }
    // the Green operator at frequency (x, y0 + yl, kz), yl fastest
    Idx3 ig(tid, nthr, kc, kIdxUnbounded);
    for (int idx = tid; idx < L * kc; idx += nthr, ig.next()) {
        const int yl = ig.a0, x = ig.a1, px = x + x / N2;
        float br[6], bi[6], ar[3], ai[3];
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            const float2 e = B[(c * kc + yl) * LP + px];
            br[c] = e.x;
            bi[c] = e.y;
        }
        const long long o = kb + (long long)x * ny + yl;
        green_apply<float>(d, x, y0 + yl, kz, o, br, bi, ar, ai);
#pragma unroll
        for (int c = 0; c < 6; ++c) B[(c * kc + yl) * LP + px] = make_float2(br[c], bi[c]);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            float2 e = make_float2(ar[c], ai[c]);
            if (!first) {
                const float2 a = A[(c * L + x) * kc + yl];
                e.x += a.x;
                e.y += a.y;
            }
            aacc[c * cstride + o] = e;
        }
    }
    __syncthreads();
    xg_pass1<N1, N2, 1>(B, NL, tw);
    __syncthreads();
    // inverse pass 2: tasks (l, k1), l fastest, written to spectrum line l
    {
        const long long sN = (long long)N1 * ny;
        const int dl = nthr % NL, dk = nthr / NL;
        int l = tid % NL, k1 = tid / NL;
        for (int task = tid; task < NL * N1; task += nthr) {
            const float2 *p = B + l * LP + (N2 + 1) * k1;
            float2 x[N2];
#pragma unroll
            for (int t = 0; t < N2; ++t) x[t] = p[t];
            sdft<N2, 1, 0, 1>(x);
            const int c = l / kc, yl = l - c * kc;
            float2 *g = spec + c * cstride + kb + yl + (long long)k1 * ny;
            sfor<0, N2>([&](auto mc) { g[decltype(mc)::v * sN] = x[dft_pos(N2, decltype(mc)::v)]; });
            l += dl;
            k1 += dk;
            if (l >= NL) { l -= NL; ++k1; }
        }
    }
}

// smem of xg_unit_f32, bytes
__host__ __device__ inline size_t xg32_smem(int nx, int n1, int kc)
{
    return 2 * sizeof(float2) * (size_t)(6 * kc) * (size_t)(nx + n1 + 1);
}

template <typename R>
__device__ void fft_x_unit(const RveDesc &d, void *specp, int ncomp, int sign, int kc, int unit)
{
    typedef typename Cx<R>::T C;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *bufA = reinterpret_cast<C *>(smem_raw);
    const int nx = d.nx, ny = d.ny, nzh = d.nzh;
    const int NL = ncomp * kc, ldl = NL | 1;
    C *bufB = bufA + nx * ldl;
    const int ytiles = ny / kc;
    const int kz = unit / ytiles, y0 = (unit % ytiles) * kc;
    C *spec = (C *)specp;
    const long long plane = (long long)nx * ny, cstride = (long long)nzh * plane;
    const long long kb = (long long)kz * plane + y0;
    if constexpr (sizeof(R) == 4) {
        Idx3 il(threadIdx.x, blockDim.x, kc, nx);
        for (int i = threadIdx.x; i < ncomp * nx * kc; i += blockDim.x, il.next())
            cp_async8(&bufA[il.a0 + il.a1 * ldl + il.a2 * kc],
                      spec + il.a2 * cstride + kb + (long long)il.a1 * ny + il.a0);
        cp_async_wait_all();
    } else {
        staged_copy3<CopyDepth<R>::v, C>(
            ncomp * nx * kc, kc, nx,
            [&](int yl, int x, int c) { return spec[c * cstride + kb + (long long)x * ny + yl]; },
            [&](int yl, int x, int c, C v) { bufA[x * ldl + c * kc + yl] = v; });
    }
    __syncthreads();
    C *res = fft_lines<R>(bufA, bufB, NL, ldl, d.plx, (const C *)d.twx, sign);
    Idx3 is(threadIdx.x, blockDim.x, kc, nx);
    for (int idx = threadIdx.x; idx < ncomp * nx * kc; idx += blockDim.x, is.next()) {
        const int yl = is.a0, x = is.a1, c = is.a2;
        spec[c * cstride + kb + (long long)x * ny + yl] = res[x * ldl + c * kc + yl];
    }
}


// Shared memory of the single-precision z passes, in complex floats.  The
// forward pass stages the six stress runs (rows x nz doubles each) behind
// its first line buffer; the inverse one (mode 0) stages the raw half-spectrum
// columns there and the old displacement-gradient runs after both buffers.
__host__ __device__ inline long long zf32_lines(int nz, int rows) { return (long long)nz * ((3 * rows) | 1); }
__host__ __device__ inline long long zf32_fwd_size(int nz, int rows)
{
    const long long a = zf32_lines(nz, rows), st = 6LL * rows * nz;   // 6 runs of doubles
    return a + (a > st ? a : st);
}
__host__ __device__ inline long long zi32_bregion(int nz, int nzh, int rows)
{
    const long long a = zf32_lines(nz, rows), st = 6LL * nzh * rows;
    return a > st ? a : st;
}
__host__ __device__ inline long long zi32_size(int nz, int nzh, int rows)
{
    return zf32_lines(nz, rows) + zi32_bregion(nz, nzh, rows) + 6LL * rows * nz;   // + 6 runs of doubles
}

// Single-precision inverse z transform of the six stress-update components
// into the symmetric displacement gradient (mode 0 of fft_z_inv_unit, with
// the same arithmetic).  The raw columns S[(c nzh + ks) rows + r] and the
// old gradient runs D[c rows nz + r nz + z] are staged by asynchronous
// copies, the columns first: the block waits for them, and the gradient
// runs arrive while the lines transform.
__device__ void fft_z_inv_dgs_f32(const RveDesc &d, int rows, int unit)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2 *bufA = reinterpret_cast<float2 *>(smem_raw);
    const int nx = d.nx, ny = d.ny, nz = d.nz, nzh = d.nzh, half = nz / 2;
    const long long nv = d.nv;
    const int NL = 3 * rows, ldl = NL | 1;
    float2 *bufB = bufA + nz * ldl;
    float2 *S = bufB;
    double *D = reinterpret_cast<double *>(bufA + zf32_lines(nz, rows) + zi32_bregion(nz, nzh, rows));
    const int ytiles = ny / rows;
    const int x = unit / ytiles, y0 = (unit % ytiles) * rows;
    const float2 *spec = (const float2 *)d.spec;
    const long long plane = (long long)nx * ny, cstride = (long long)nzh * plane;
    const long long xy = (long long)x * ny + y0, vb = xy * nz;
    const int run = rows * nz, half_run = run / 2;
    {
        Idx3 is(threadIdx.x, blockDim.x, rows, nzh);   // (r, ks, c)
        for (int i = threadIdx.x; i < 6 * nzh * rows; i += blockDim.x, is.next())
            cp_async8(S + i, spec + is.a2 * cstride + (long long)is.a1 * plane + xy + is.a0);
        asm volatile("cp.async.commit_group;" ::: "memory");
    }
    {
        Idx3 ic(threadIdx.x, blockDim.x, half_run, kIdxUnbounded);
        for (int i = threadIdx.x; i < 6 * half_run; i += blockDim.x, ic.next())
            cp_async16(D + 2 * i, d.dgs + ic.a1 * nv + vb + 2 * ic.a0);
        asm volatile("cp.async.commit_group;" ::: "memory");
    }
    asm volatile("cp.async.wait_group 1;" ::: "memory");
    __syncthreads();
    // element (r, k, p): line p's coefficient k of row r (components 2p, 2p + 1)
    Idx3 ik(threadIdx.x, blockDim.x, rows, nz);
    for (int i = threadIdx.x; i < 3 * nz * rows; i += blockDim.x, ik.next()) {
        const int r = ik.a0, k = ik.a1, p = ik.a2;
        const int ks = k <= half ? k : nz - k;
        float2 A = S[(2 * p * nzh + ks) * rows + r], B = S[((2 * p + 1) * nzh + ks) * rows + r];
        if (k == 0 || k == half) { A.y = 0.f; B.y = 0.f; }
        if (k > half) { A.y = -A.y; B.y = -B.y; }
        bufA[k * ldl + p * rows + r] = make_float2(A.x - B.y, A.y + B.x);
    }
    __syncthreads();
    const float2 *res = fft_lines<float>(bufA, bufB, NL, ldl, d.plz, (const float2 *)d.twz, +1);
    cp_async_wait_all();
    __syncthreads();
    const MacroDev *m = d.macro;
    // the update val/N as a float product (exact for a power-of-two N):
    // one FP64-pipe operation fewer per value than a product in FP64
    const float inv = (float)d.inv_nv;
    // element (z, r, c) is dgs[c][vb + r * nz + z] = D[i]
    Idx3 iz(threadIdx.x, blockDim.x, nz, rows);
    for (int i = threadIdx.x; i < 6 * run; i += blockDim.x, iz.next()) {
        const int z = iz.a0, r = iz.a1, c = iz.a2;
        const float2 e = res[z * ldl + (c >> 1) * rows + r];
        const double val = (double)(((c & 1) ? e.y : e.x) * inv);
        d.dgs[(long long)c * nv + vb + (long long)r * nz + z] = D[i] + (m->ddg6[c] + val);
    }
}

// inverse z transform (Hermitian half spectrum -> real); mode 0 adds the
// result to the symmetric displacement gradient (evolution.c:383-394),
// mode 1 writes it (scaled by 1/N) to rotl, mode 2 (scaled by 1/N) to
// out[ncomp * v + c], voxel by voxel
template <typename R>
__device__ void fft_z_inv_unit(const RveDesc &d, void *specp, int ncomp, int rows, int mode, int unit,
                               double *out = nullptr)
{
    typedef typename Cx<R>::T C;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *bufA = reinterpret_cast<C *>(smem_raw);
    const int nx = d.nx, ny = d.ny, nz = d.nz, nzh = d.nzh;
    const long long nv = d.nv;
    const int np = (ncomp + 1) / 2;
    const int NL = np * rows, ldl = NL | 1;
    C *bufB = bufA + nz * ldl;
    const int ytiles = ny / rows;
    const int x = unit / ytiles, y0 = (unit % ytiles) * rows;
    const C *spec = (const C *)specp;
    const long long plane = (long long)nx * ny, cstride = (long long)nzh * plane;
    const long long xy = (long long)x * ny + y0;
    const int half = nz / 2;
    struct AB { C a, b; };
    // element (r, k, p): line p's coefficient k of row r
    staged_copy3<kZCopyDepth, AB>(
        np * nz * rows, rows, nz,
        [&](int r, int k, int p) {
            const int ca = 2 * p, cb = 2 * p + 1;
            const int ks = k <= half ? k : nz - k;
            const long long o = (long long)ks * plane + xy + r;
            AB v;
            v.a = spec[ca * cstride + o];
            if (cb < ncomp) v.b = spec[cb * cstride + o];
            else { v.b.x = R(0); v.b.y = R(0); }
            return v;
        },
        [&](int r, int k, int p, AB v) {
            const bool lo = k <= half;
            C A = v.a, B = v.b;
            if (k == 0 || k == half) { A.y = R(0); B.y = R(0); }
            if (!lo) { A.y = -A.y; B.y = -B.y; }
            C Z;
            Z.x = A.x - B.y;
            Z.y = A.y + B.x;
            bufA[k * ldl + p * rows + r] = Z;
        });
    __syncthreads();
    const C *res = fft_lines<R>(bufA, bufB, NL, ldl, d.plz, (const C *)d.twz, +1);
    const long long vb = xy * nz;
    const double inv = d.inv_nv;
    if (mode == 0) {
        const MacroDev *m = d.macro;
        // element (z, r, c) is dgs[c][vb + r * nz + z]
        staged_copy3<kZCopyDepth, double>(
            ncomp * rows * nz, nz, rows,
            [&](int z, int r, int c) { return d.dgs[(long long)c * nv + vb + (long long)r * nz + z]; },
            [&](int z, int r, int c, double old) {
                const C e = res[z * ldl + (c >> 1) * rows + r];
                const double val = (double)((c & 1) ? e.y : e.x);
                d.dgs[(long long)c * nv + vb + (long long)r * nz + z] = old + (m->ddg6[c] + val * inv);
            });
    } else if (mode == 1) {
        Idx3 iz(threadIdx.x, blockDim.x, nz, rows);
        for (int idx = threadIdx.x; idx < ncomp * rows * nz; idx += blockDim.x, iz.next()) {
            const int z = iz.a0, r = iz.a1, c = iz.a2;
            const C e = res[z * ldl + (c >> 1) * rows + r];
            const double val = (double)((c & 1) ? e.y : e.x);
            d.rotl[(long long)c * nv + vb + (long long)r * nz + z] = val * inv;
        }
    } else {
        for (int idx = threadIdx.x; idx < ncomp * rows * nz; idx += blockDim.x) {
            const int c = idx % ncomp, t = idx / ncomp, z = t % nz, r = t / nz;
            const C e = res[z * ldl + (c >> 1) * rows + r];
            const double val = (double)((c & 1) ? e.y : e.x);
            out[ncomp * (vb + (long long)r * nz + z) + c] = val * inv;
        }
    }
}


// ---------------------------------------------------------------------------
// per-voxel Newton-Raphson stress update (UpdateStress, evolution.c:3-168),
// solved in the equivalent symmetric form
//   (S0 + S_g + dt dEdot) dsig = S0 R
// where R is the reference's residual (evolution.c:78-83) and S0 = C0^-1.
// NR32 (the VOCE_PREC_MIXED_NR32 form): see mixed_newton below; otherwise
// the FP64 Newton of the reference, for the FP64 and VOCE_PREC_MIXED forms.
// ---------------------------------------------------------------------------

// P = S_g + S0 (packed upper triangle) of voxel v
__device__ __forceinline__ void load_P(const RveDesc &d, long long v, double (&P)[21])
{
#pragma unroll
    for (int q = 0; q < 21; ++q) P[q] = __ldg(d.sg + (long long)q * d.nv + v);
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
        for (int j = i; j < 6; ++j) P[sym6(i, j)] += d.S0[i * 6 + j];
}

// The same, with loads the compiler may not merge with earlier ones: a
// reload where keeping P live would cost registers.
__device__ __forceinline__ void reload_P(const RveDesc &d, long long v, double (&P)[21])
{
#pragma unroll
    for (int q = 0; q < 21; ++q) {
        const double *a = d.sg + (long long)q * d.nv + v;
        double x;
        asm volatile("ld.global.nc.f64 %0, [%1];" : "=d"(x) : "l"(a));
        P[q] = x;
    }
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
        for (int j = i; j < 6; ++j) P[sym6(i, j)] += d.S0[i * 6 + j];
}

// Newton steps on the FP64 residual with the stop test of evolution.c:112.
// NR32 (fallback of the single-precision form only): the Jacobian and its
// solve in FP32, an inexact Newton step converging to the same FP64 fixed
// point; otherwise all FP64.  With d.chord (the VOCE_PREC_MIXED form), an
// FP64 step whose predecessor moved the stress by less than 1e-4 relative
// reuses that predecessor's factored Jacobian (a chord step: the residual,
// the flow rule's strain rate and the stop test are evaluated as always, the
// Jacobian and its LDL^T factorisation are not).  Near the root the Jacobian
// then differs by about n x 1e-4 relative, so each chord step still divides
// the error by ~500; the converged stress moves by ~1e-14 relative against
// the exact-Jacobian Newton of the reference (evolution.c:85-110), the point
// before the last update (where the strain rate is evaluated) by up to 1e-8
// when the step count changes.
template <bool NR32, bool CHORD = false>
__device__ __forceinline__ void newton_fp64(const RveDesc &d, long long v, const double (&P)[21],
                                           const double (&cc)[6], double thr, double (&sig)[6],
                                           double (&sp)[6], double (&Rl)[6], int &it)
{
    const double dt = d.dt;
    bool go = true;
    // FP64 Jacobian factors, kept for chord steps (CHORD instances only)
    double L[6][6], dinv[6];
    bool fresh = true;
    (void)L; (void)dinv; (void)fresh;
    while (go && it < 100) {
        ++it;
        double ed[5];
#pragma unroll
        for (int c = 0; c < 6; ++c) sp[c] = sig[c];
        double R[6];
        if (NR32) {
            float D[15];
            flow_rule<true, false, float>(d, v, sig, ed, D, nullptr, nullptr);
            float M[6][6], x[6];
#pragma unroll
            for (int i = 0; i < 6; ++i) {
                double s = cc[i] + (i < 5 ? dt * ed[i] : 0.0);
#pragma unroll
                for (int j = 0; j < 6; ++j) s = fma(P[sym6(i, j)], sig[j], s);
                R[i] = s;
                Rl[i] = s;
                x[i] = (float)s;
            }
            const float dtf = (float)dt;
#pragma unroll
            for (int i = 0; i < 6; ++i)
#pragma unroll
                for (int j = 0; j <= i; ++j) {
                    float m = (float)P[sym6(i, j)];
                    if (i < 5 && j < 5) m = fmaf(dtf, D[j * 5 - (j * (j - 1)) / 2 + (i - j)], m);
                    M[i][j] = m;
                }
            ldlt_solve6f(M, x);
#pragma unroll
            for (int i = 0; i < 6; ++i) R[i] = (double)x[i];
        } else if (!CHORD) {
            double D[15];
            flow_rule<true, false, double>(d, v, sig, ed, D, nullptr, nullptr);
#pragma unroll
            for (int i = 0; i < 6; ++i) {
                double s = cc[i] + (i < 5 ? dt * ed[i] : 0.0);
#pragma unroll
                for (int j = 0; j < 6; ++j) s = fma(P[sym6(i, j)], sig[j], s);
                R[i] = s;
                Rl[i] = s;
            }
            double M[6][6];
#pragma unroll
            for (int i = 0; i < 6; ++i)
#pragma unroll
                for (int j = 0; j <= i; ++j) {
                    double m = P[sym6(i, j)];
                    if (i < 5 && j < 5) m = fma(dt, D[j * 5 - (j * (j - 1)) / 2 + (i - j)], m);
                    M[i][j] = m;
                }
            ldlt_solve6(M, R);
        } else {
            if (fresh) {
                double D[15];
                flow_rule<true, false, double>(d, v, sig, ed, D, nullptr, nullptr);
                double M[6][6];
#pragma unroll
                for (int i = 0; i < 6; ++i)
#pragma unroll
                    for (int j = 0; j <= i; ++j) {
                        double m = P[sym6(i, j)];
                        if (i < 5 && j < 5) m = fma(dt, D[j * 5 - (j * (j - 1)) / 2 + (i - j)], m);
                        M[i][j] = m;
                    }
                ldlt_factor6(M, L, dinv);
            } else {
                flow_rule<false, false, double>(d, v, sig, ed, (double *)nullptr, nullptr, nullptr);
            }
#pragma unroll
            for (int i = 0; i < 6; ++i) {
                double s = cc[i] + (i < 5 ? dt * ed[i] : 0.0);
#pragma unroll
                for (int j = 0; j < 6; ++j) s = fma(P[sym6(i, j)], sig[j], s);
                R[i] = s;
                Rl[i] = s;
            }
            ldlt_apply6(L, dinv, R);
        }
        double cnr = 0.0;
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            const double sn = sig[c] - R[c];
            const double dd = sn - sig[c];
            cnr = fma(dd, dd, cnr);
            sig[c] = sn;
        }
        go = cnr > thr;
        // the next step reuses this Jacobian (a chord step) once the update
        // is below 1e-4 relative (cnr <= 1e-8 sn2 = 1e6 thr)
        if (CHORD) fresh = !d.chord || cnr > 1e6 * thr;
    }
}

// Mixed form: Newton in single precision (residual, Jacobian and solve) down
// to a relative update of 1e-4, then one Newton step on the double-precision
// residual with the last single-precision matrix.  That residual is evaluated
// in float-float on the FP32 pipe (residual_ff), from float pairs of the
// model data: the double-precision model to about 2^-48, at a fraction of the
// cost of FP64 arithmetic on this part.  That step is accepted when
// its relative update is below 1e-5: Newton's quadratic term then puts the
// next update near 1e-9, under the 1e-7 test of the FP64 form, so the
// accepted stress is taken as the converged point (zero residual, and the
// point the strain rate is later evaluated at).  Anything else continues with
// newton_fp64 from where it stands.  Without polish (Green iterations whose
// predecessor's error is above VOCE_POLISH_ERR, and the first of an
// increment) the single-precision Newton runs down to 1e-5 and its point is
// taken as converged: its error, a few 1e-6 relative, is far below the
// change such an iteration makes.
__device__ __forceinline__ void mixed_newton(const RveDesc &d, long long v, const float *st,
                                             const double (&lam)[6], const double (&cc)[6], double sn2,
                                             bool polish, double (&sig)[6], double (&sp)[6],
                                             double (&Rl)[6], int &it)
{
    const double dt = d.dt;
    bool done = false;
    if (d.ipow_n >= 1) {
        float sf[6], Mf[6][6], Pf[21];
#pragma unroll
        for (int q = 0; q < 21; ++q) Pf[q] = __ldg(d.sgp32 + (long long)q * d.nv + v);
        float ccf[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) { sf[c] = (float)lam[c]; ccf[c] = (float)cc[c]; }
        // single precision alone stops at a relative update of 1e-5, before a
        // polish step at 1e-4
        const float thr32 = (float)((polish ? 1e-8 : 1e-10) * sn2);
        const float dtf = (float)dt;
        bool ok = true, conv = false;
        cp_async_wait_all();   // the staged column of this voxel
        while (it < 24) {
            ++it;
            float ed[5], D[15], x[6];
            if (!flow_rule_f32(d, st, sf, ed, D)) { ok = false; break; }
#pragma unroll
            for (int i = 0; i < 6; ++i) {
                float t = ccf[i] + (i < 5 ? dtf * ed[i] : 0.0f);
#pragma unroll
                for (int j = 0; j < 6; ++j) t = fmaf(Pf[sym6(i, j)], sf[j], t);
                x[i] = t;
            }
#pragma unroll
            for (int i = 0; i < 6; ++i)
#pragma unroll
                for (int j = 0; j <= i; ++j) {
                    float m = Pf[sym6(i, j)];
                    if (i < 5 && j < 5) m = fmaf(dtf, D[j * 5 - (j * (j - 1)) / 2 + (i - j)], m);
                    Mf[i][j] = m;
                }
            ldlt_solve6f(Mf, x);
            float dn = 0.0f;
#pragma unroll
            for (int c = 0; c < 6; ++c) { dn = fmaf(x[c], x[c], dn); sf[c] -= x[c]; }
            if (!(dn <= 3.0e38f)) { ok = false; break; }   // not finite
            if (dn < thr32) { conv = true; break; }
        }
        if (ok && conv && !polish) {
            done = true;
#pragma unroll
            for (int c = 0; c < 6; ++c) { sig[c] = (double)sf[c]; sp[c] = sig[c]; Rl[c] = 0.0; }
        } else if (ok && conv) {
            ++it;
            float x[6];
            if (residual_ff(d, v, st, sf, cc, Pf, x)) {
                ldlt_solve6f(Mf, x);
                float dn = 0.0f;
#pragma unroll
                for (int c = 0; c < 6; ++c) {
                    dn = fmaf(x[c], x[c], dn);
                    sig[c] = (double)sf[c] - (double)x[c];
                }
                if (dn <= (float)(1e-10 * sn2)) {
                    done = true;
#pragma unroll
                    for (int c = 0; c < 6; ++c) { sp[c] = sig[c]; Rl[c] = 0.0; }
                }
            } else {
#pragma unroll
                for (int c = 0; c < 6; ++c) sig[c] = (double)sf[c];
            }
        } else {
#pragma unroll
            for (int c = 0; c < 6; ++c) sig[c] = lam[c];
        }
    }
    if (!done) {
        double P[21];
        reload_P(d, v, P);
        newton_fp64<true>(d, v, P, cc, 1e-14 * sn2, sig, sp, Rl, it);
    }
}

// Newton iterations of the VOCE_PREC_MIXED_IR form: every iteration
// evaluates the reference's residual (evolution.c:78-83, in the symmetric
// form x = cc + dt edot(s) + (S_g + S0) s) and the flow rule
// (constitutive.c:126-194: resolved shears, |r|^n, strain rate) in FP64, and
// takes the stop test of evolution.c:112 in FP64; only the correction -- the
// Jacobian dt dEdot/ds + S_g + S0 and its LDL^T solve -- is assembled and
// solved in FP32, from float copies of the Schmid vectors, 1/CRSS and
// S_g + S0.  This is iterative refinement: each step solves for the FP64
// residual with an approximate matrix (relative error ~1e-7 times its
// condition number), so the iteration converges to the root of the FP64
// residual, near the root nearly as fast as the exact Newton.  A resolved
// shear ratio |r| >= 60 (where |r|^(n-1) could leave the float range) makes
// that iteration take the FP64 Jacobian instead.  gam0 is one value for all
// systems (one slip mode), so it is applied once to the strain-rate sums.
//
// With d.ir_pred the FP64 iterations start from a point computed on the FP32
// pipe (ir_start): single-precision Newton steps down to a relative update of
// 1e-4, then one step on the float-float residual (residual_ff, the model
// data as float pairs, about 48 bits) with the last single-precision matrix.
// That point lies within about 1e-9 relative of the FP64 residual's root, so
// the first FP64 step's update is already below the 1e-7 stop test: one FP64
// residual evaluation per voxel accepts it, against two to seven from the
// Green iterate.  The start never decides the result -- the accepted stress
// and the stop decision come from the FP64 steps.  A start that does not
// converge in single precision, meets a resolved-shear ratio too large for
// |r|^n in FP32 or a non-finite value is dropped (the FP64 steps then start
// from the Green iterate).  st is the voxel's staged column of float Schmid
// vectors and 1/CRSS (as in the single-precision Newton form).  The last
// single-precision matrix goes to the column mout (lower triangle packed,
// stride VOCE_NR_THREADS), where the FP64 steps read it.
__device__ __forceinline__ bool ir_start(const RveDesc &d, long long v, const float *st,
                                         const double (&lam)[6], const double (&cc)[6], double sn2,
                                         double (&sig)[6], int &it, float *mout)
{
    float sf[6], ccf[6], Pf[21], Mf[6][6];
#pragma unroll
    for (int q = 0; q < 21; ++q) Pf[q] = __ldg(d.sgp32 + (long long)q * d.nv + v);
#pragma unroll
    for (int c = 0; c < 6; ++c) { sf[c] = (float)lam[c]; ccf[c] = (float)cc[c]; }
    // single precision stops at a relative update of 1e-4 (its rounding
    // floor can lie near 1e-5); the float-float step then takes the point to
    // within Newton's quadratic term of that update (~1e-9)
    const float thr32 = 1e-8f * (float)sn2;
    const float dtf = d.dth;
    bool conv = false;
    cp_async_wait_all();   // the staged column of this voxel
    for (int p = 0; p < 12; ++p) {
        float ed[5], D[15], x[6];
        if (!flow_rule_f32(d, st, sf, ed, D)) return false;
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            float t = ccf[i] + (i < 5 ? dtf * ed[i] : 0.0f);
#pragma unroll
            for (int j = 0; j < 6; ++j) t = fmaf(Pf[sym6(i, j)], sf[j], t);
            x[i] = t;
#pragma unroll
            for (int j = 0; j <= i; ++j) {
                float m = Pf[sym6(i, j)];
                if (i < 5 && j < 5) m = fmaf(dtf, D[j * 5 - (j * (j - 1)) / 2 + (i - j)], m);
                Mf[i][j] = m;
            }
        }
        ldlt_solve6f(Mf, x);
        float dn = 0.0f;
#pragma unroll
        for (int c = 0; c < 6; ++c) { dn = fmaf(x[c], x[c], dn); sf[c] -= x[c]; }
        ++it;
        if (!(dn <= 3.0e38f)) return false;   // not finite
        if (dn < thr32) { conv = true; break; }
    }
    if (!conv) return false;
    float x[6];
    if (!residual_ff(d, v, st, sf, cc, Pf, x)) return false;
    ldlt_solve6f(Mf, x);
    ++it;
#pragma unroll
    for (int c = 0; c < 6; ++c) sig[c] = (double)sf[c] - (double)x[c];
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
        for (int j = 0; j <= i; ++j) mout[sym6(i, j) * VOCE_NR_THREADS] = Mf[i][j];
    return true;
}

// One FP64-Jacobian step of newton_ir, for the rare iteration whose
// resolved-shear ratio leaves the float range; kept out of line so that its
// registers do not weigh on the common path.
__device__ __noinline__ void ir_fp64_step(const RveDesc &d, long long v, const double *sig, double *R)
{
    double P[21], Dd[15], edd[5];
    for (int q = 0; q < 21; ++q) P[q] = d.sgp[(long long)q * d.nv + v];
    flow_rule<true, false, double>(d, v, sig, edd, Dd, nullptr, nullptr);
    double M[6][6], b[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        b[i] = R[i];
#pragma unroll
        for (int j = 0; j <= i; ++j) {
            double m = P[sym6(i, j)];
            if (i < 5 && j < 5) m = fma(d.dt, Dd[j * 5 - (j * (j - 1)) / 2 + (i - j)], m);
            M[i][j] = m;
        }
    }
    ldlt_solve6(M, b);
#pragma unroll
    for (int i = 0; i < 6; ++i) R[i] = b[i];
}

// mst (with START): the single-precision matrix of the start's last step,
// lower triangle packed, in the voxel's staged column; the FP64 steps solve
// with it instead of assembling the Jacobian again (near the root it is the
// Jacobian to about n x 1e-4 relative, so each step still divides the error
// by ~500 -- and from the start one step is usually the last).  S_g + S0 is
// read from d.sgp (FP64, stored at setup) where the residual needs it, rather
// than kept in registers across the iterations.
template <bool START>
__device__ __forceinline__ void newton_ir(const RveDesc &d, long long v, const double (&cc)[6],
                                          double thr, double (&sig)[6], double (&sp)[6],
                                          double (&Rl)[6], int &it, const float *mst)
{
    const long long nv = d.nv;
    const double dtg = d.dt * d.gam0[0];
    const float dtf = d.dth;
    const float g1c = d.gam0f[0] * d.nrsf[0];   // gam0 n
    const int e = d.ipow_n - 1;
    bool go = true;
    while (go && it < 100) {
        ++it;
#pragma unroll
        for (int c = 0; c < 6; ++c) sp[c] = sig[c];
        double ed[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
        float D[15];
#pragma unroll
        for (int q = 0; q < 15; ++q) D[q] = 0.0f;
        bool big = false;
#pragma unroll 2
        for (int k = 0; k < d.nsys; ++k) {
            double sc[5];
#pragma unroll
            for (int i = 0; i < 5; ++i) sc[i] = __ldg(d.sch + (long long)(5 * k + i) * nv + v);
            const double rss = sc[0] * sig[0] + sc[1] * sig[1] + sc[2] * sig[2] + sc[3] * sig[3] + sc[4] * sig[4];
            const int neg = __double2hiint(rss) < 0;
            const long long ti = (long long)(2 * k + neg) * nv + v;
            const double it0 = __ldg(d.itau + (long long)(2 * k) * nv + v);
            const double it1 = __ldg(d.itau + (long long)(2 * k + 1) * nv + v);
            const double r = rss * (neg ? it1 : it0);
            // |r| >= 60 (or not finite), tested on the high word: an
            // integer comparison instead of one on the FP64 pipe
            big = big || (__double2hiint(r) & 0x7fffffff) >= 0x404E0000;
            double g2;                                // |r|^n sign(r) / gam0
            float aef;                                // |r|^(n-1), for the float Jacobian
            if (e == 19) {
                // |r|^20 = ((r^2)^2 |r|)^2)^2: five products, the sign of r
                // put on the high word
                const double a2 = r * r, a4 = a2 * a2, a5 = a4 * fabs(r), a10 = a5 * a5, a20 = a10 * a10;
                g2 = __hiloint2double(__double2hiint(a20) | (__double2hiint(r) & (int)0x80000000),
                                      __double2loint(a20));
                if (!START) {
                    const float af = fabsf((float)r), af2 = af * af, af4 = af2 * af2, af8 = af4 * af4;
                    aef = af8 * af8 * af2 * af;
                }
            } else {
                const double ae = pow_abs_e(fabs(r), e);   // |r|^(n-1)
                g2 = ae * r;
                aef = (float)ae;
            }
#pragma unroll
            for (int i = 0; i < 5; ++i) ed[i] = fma(sc[i], g2, ed[i]);
            if (START) continue;
            // Jacobian term gam0 n |r|^(n-1) / tau m m^T, in single precision
            const float g1 = g1c * aef * __ldg(d.itau32 + ti);
            float sf[5], t[5];
#pragma unroll
            for (int i = 0; i < 5; ++i) {
                sf[i] = __ldg(d.sch32 + (long long)(5 * k + i) * nv + v);
                t[i] = g1 * sf[i];
            }
            int q = 0;
#pragma unroll
            for (int i = 0; i < 5; ++i)
#pragma unroll
                for (int j = i; j < 5; ++j) { D[q] = fmaf(t[i], sf[j], D[q]); ++q; }
        }
        double R[6];
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            double s = (i < 5) ? fma(dtg, ed[i], cc[i]) : cc[i];
#pragma unroll
            for (int j = 0; j < 6; ++j) s = fma(__ldg(d.sgp + (long long)sym6(i, j) * nv + v), sig[j], s);
            R[i] = s;
            Rl[i] = s;
        }
        if (!big) {
            float M[6][6], x[6];
#pragma unroll
            for (int i = 0; i < 6; ++i) {
                x[i] = (float)R[i];
#pragma unroll
                for (int j = 0; j <= i; ++j) {
                    float m;
                    if (START) {
                        m = mst[sym6(i, j) * VOCE_NR_THREADS];
                    } else {
                        m = __ldg(d.sgp32 + (long long)sym6(i, j) * nv + v);
                        if (i < 5 && j < 5) m = fmaf(dtf, D[j * 5 - (j * (j - 1)) / 2 + (i - j)], m);
                    }
                    M[i][j] = m;
                }
            }
            ldlt_solve6f(M, x);
#pragma unroll
            for (int i = 0; i < 6; ++i) R[i] = (double)x[i];
        } else {
            ir_fp64_step(d, v, sig, R);
        }
        // the stop test of evolution.c:112 on the update itself (the
        // reference's |sig_new - sig_old|^2 up to the rounding of one
        // subtraction)
        double cnr = 0.0;
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            cnr = fma(R[c], R[c], cnr);
            sig[c] -= R[c];
        }
        go = cnr > thr;
    }
}

template <bool NR32, bool CHORD = false, bool IR = false>
__device__ void nr_unit(const RveDesc &d, int unit, int nunits)
{
    // per-thread sums in shared memory (one slot per thread, the same
    // additions in the same order as register accumulators) keep them out of
    // the registers the Newton loop needs
    __shared__ double s_acc[VOCE_NPART][VOCE_NR_THREADS];
    // Newton iteration count (sum, max) as integers; entries 14 and 15 of
    // the partials receive them converted, the same values
    __shared__ int s_it[2][VOCE_NR_THREADS];
    const int tid = threadIdx.x;
    // NR32: this thread's column of the staged float model data
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float *st = reinterpret_cast<float *>(smem_raw) + tid;
    bool polish = true;
    if (NR32) {
        const MacroDev *m = d.macro;
        polish = !m->first_iter && fmax(fabs(m->Err_e), fabs(m->Err_s)) <= VOCE_POLISH_ERR;
    }
#pragma unroll
    for (int q = 0; q < VOCE_NPART; ++q) s_acc[q][tid] = 0.0;
    s_it[0][tid] = 0;
    s_it[1][tid] = 0;
    const long long nv = d.nv;
    for (long long v = (long long)unit * blockDim.x + threadIdx.x; v < nv;
         v += (long long)nunits * blockDim.x) {
        if (NR32 || IR) {
            // asynchronous copies of the voxel's float Schmid vectors and
            // 1/CRSS; every path below waits for them before the next voxel
#pragma unroll
            for (int c = 0; c < VOCE_STAGE_ITAU; ++c) cp_async4(st + c * VOCE_NR_THREADS, d.sch32 + c * nv + v);
#pragma unroll
            for (int c = 0; c < 24; ++c)
                cp_async4(st + (VOCE_STAGE_ITAU + c) * VOCE_NR_THREADS, d.itau32 + c * nv + v);
        }
        if ((IR && d.ir_pred) || (NR32 && polish)) {
            // the low halves the float-float step reads (the mixed_ir start's,
            // the mixed_nr32 acceptance step's), brought to L2 while the
            // single-precision steps run: one 128-byte line per row of the
            // warp's 32 voxels, the 105 rows shared out over the lanes (the
            // FP64 rows or the next voxel's rows as well: measured slower)
            const int lane = tid & 31;
            const long long vw = v - lane;
            for (int r = lane; r < 105; r += 32) {
                const float *b = r < 60 ? d.sch_lo + (long long)r * nv
                               : r < 84 ? d.itau_lo + (long long)(r - 60) * nv : d.sgp_lo + (long long)(r - 84) * nv;
                asm volatile("prefetch.global.L2 [%0];" ::"l"(b + vw));
            }
        }
        const int ph = d.phase[v];
        if (!d.solid[ph]) {
#pragma unroll
            for (int c = 0; c < 6; ++c) { d.sig[c * nv + v] = 0.0; d.sigp[c * nv + v] = 0.0; }
            if (NR32 || IR) cp_async_wait_all();
            continue;
        }
        double lam[6], cc[6];
        {
            double e6[6], ep[6];
#pragma unroll
            for (int c = 0; c < 6; ++c) {
                lam[c] = d.sig[c * nv + v];
                e6[c] = d.dgs[c * nv + v];
            }
#pragma unroll
            for (int c = 0; c < 5; ++c) ep[c] = d.eps[c * nv + v];
            ep[5] = 0.0;
#pragma unroll
            for (int i = 0; i < 6; ++i) {
                double s = ep[i] - e6[i];
#pragma unroll
                for (int j = 0; j < 6; ++j) s = fma(-d.S0[i * 6 + j], lam[j], s);
                cc[i] = s;
            }
        }
        double sn2 = 0.0;
#pragma unroll
        for (int c = 0; c < 6; ++c) sn2 = fma(lam[c], lam[c], sn2);
        double sig[6], sp[6], Rl[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) { sig[c] = lam[c]; sp[c] = lam[c]; Rl[c] = 0.0; }
        int it = 0;
        if (NR32) {
            mixed_newton(d, v, st, lam, cc, sn2, polish, sig, sp, Rl, it);
            cp_async_wait_all();   // (already done unless the float phase was skipped)
        } else if (IR && d.ipow_n >= 1) {
            // sqrt(cnr)/signorm > 1e-7 (evolution.c:112) tested as cnr > 1e-14 signorm^2
            bool started = false;
            if (d.ir_pred) {
                int it0 = it;
                // the staged column is read no more once the start ends: it
                // keeps the last matrix for the FP64 steps (st is this
                // thread's own column)
                started = ir_start(d, v, st, lam, cc, sn2, sig, it, const_cast<float *>(st));
                if (!started) {
#pragma unroll
                    for (int c = 0; c < 6; ++c) sig[c] = lam[c];
                    it = it0;
                }
            }
            if (started) newton_ir<true>(d, v, cc, 1e-14 * sn2, sig, sp, Rl, it, st);
            else newton_ir<false>(d, v, cc, 1e-14 * sn2, sig, sp, Rl, it, nullptr);
            cp_async_wait_all();
        } else {
            double P[21];
            load_P(d, v, P);
            // sqrt(cnr)/signorm > 1e-7 (evolution.c:112) tested as cnr > 1e-14 signorm^2
            newton_fp64<IR, CHORD>(d, v, P, cc, 1e-14 * sn2, sig, sp, Rl, it);
            if (IR) cp_async_wait_all();
        }
        double ncs, nce;   // |sig - lam| and the strain-compatibility norm (evolution.c:118-123)
        if (NR32) {
            // error norms in single precision: they only steer the Green
            // iteration's stop test at 1e-5
            float ds[6], dp[6], cs = 0.0f, ce = 0.0f;
#pragma unroll
            for (int i = 0; i < 6; ++i) {
                ds[i] = (float)(sig[i] - lam[i]);
                dp[i] = (float)(sp[i] - lam[i]);
                cs = fmaf(ds[i], ds[i], cs);
            }
#pragma unroll
            for (int i = 0; i < 6; ++i) {
                float te = (float)Rl[i];
#pragma unroll
                for (int j = 0; j < 6; ++j) te = fmaf(-d.S0f[i * 6 + j], dp[j], te);
                ce = fmaf(te, te, ce);
            }
            ncs = (double)sqrtf(cs);
            nce = (double)sqrtf(ce);
        } else {
            double cs = 0.0, ce = 0.0;
#pragma unroll
            for (int i = 0; i < 6; ++i) {
                const double ds = sig[i] - lam[i];
                cs = fma(ds, ds, cs);
                double te = Rl[i];
#pragma unroll
                for (int j = 0; j < 6; ++j) te = fma(-d.S0[i * 6 + j], sp[j] - lam[j], te);
                ce = fma(te, te, ce);
            }
            // the mixed_ir form's norms by a Newton-Raphson square root
            // (about 1e-13 relative); the other forms' correctly rounded
            ncs = IR ? sqrt_nr(cs) : sqrt(cs);
            nce = IR ? sqrt_nr(ce) : sqrt(ce);
        }
#pragma unroll
        for (int c = 0; c < 6; ++c) { d.sig[c * nv + v] = sig[c]; d.sigp[c * nv + v] = sp[c]; }
        s_acc[0][tid] += ncs;
        s_acc[1][tid] += nce;
#pragma unroll
        for (int c = 0; c < 6; ++c) s_acc[2 + c][tid] += sig[c];
        // phase-1 sums; when every voxel is phase 1 they would repeat the
        // sums above addition for addition, and are copied from them below
        if (ph == 1 && !d.all_ph1) {
#pragma unroll
            for (int c = 0; c < 6; ++c) s_acc[8 + c][tid] += sig[c];
        }
        s_it[0][tid] += it;
        s_it[1][tid] = max(s_it[1][tid], it);
    }
    double acc[VOCE_NPART];
#pragma unroll
    for (int q = 0; q < VOCE_NPART; ++q) acc[q] = s_acc[q][tid];
    if (d.all_ph1) {
#pragma unroll
        for (int c = 0; c < 6; ++c) acc[8 + c] = acc[2 + c];
    }
    acc[14] = (double)s_it[0][tid];
    acc[15] = (double)s_it[1][tid];
    block_partials(acc, d.part + (long long)unit * VOCE_NPART);
}


__device__ double vm_strain(const double *t)  // VonMises, evolution.c:243-262
{
    double tr = t[0] + t[4] + t[8], vm = 0.0;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            double x = (t[3 * a + b] + t[3 * b + a]) / 2. - (double)(a == b) * tr / 3.0;
            vm += x * x;
        }
    return sqrt(2. / 3. * vm);
}

__device__ void sym9_from_b(const double *b6, double *t9)
{
    double t[6];
    b_to_t6<double>(b6, t);
    t9[0] = t[0]; t9[4] = t[1]; t9[8] = t[2];
    t9[5] = t9[7] = t[3];
    t9[2] = t9[6] = t[4];
    t9[1] = t9[3] = t[5];
}

// s_vm of a symmetric tensor through the deviatoric 5-vector (get_smacro,
// evolution.c:218-238)
__device__ double svm_of(const double *t9)
{
    double t6[6] = {t9[0], t9[4], t9[8], t9[5], t9[2], t9[1]}, b6[6];
    t6_to_b<double>(t6, b6);
    b6[5] = 0.0;
    double dev[9];
    sym9_from_b(b6, dev);
    double s = 0.0;
    for (int q = 0; q < 9; ++q) s += dev[q] * dev[q];
    return sqrt(3. / 2. * s);
}

// Errors, volume averages, mixed-BC macro correction and the convergence
// decision (evolution.c:401-431, get_smacro :170-241), after the block's
// reduction of the partial sums, by the block's first warp.  Every value is
// computed by one lane with the operations, in the order, a single thread
// would use, so the results do not depend on the split; the lanes compute
// independent values side by side (the 9 + 9 stress averages, the 6 mixed-BC
// corrections, the two von Mises norms, the two error normalisations, the
// epilogue's 9 velocity-gradient divisions and its two norms), each step as
// one instruction stream for the warp.  That cuts the dependent chain of
// slow FP64 operations (~60-cycle DADD/DFMA latency, ~1500-cycle divisions)
// that bounds this kernel.  m is the block's shared-memory copy.
__device__ void finalize_iter_body(const RveDesc &d, MacroDev *m, int npart)
{
    double tot[VOCE_NPART];
    reduce_partials(d.part, npart, tot);
    const int lane = threadIdx.x;
    if (lane >= 32) return;
    __shared__ double s_dg[9], s_vm2[2], s_act[2][9];
    const int IJV0[6] = {0, 1, 2, 1, 0, 0}, IJV1[6] = {0, 1, 2, 2, 2, 1};
    const int first_iter = m->first_iter, it = m->iter, istep = m->istep;
    const double Err_e0 = m->Err_e, Err_s0 = m->Err_s, e_vm = m->e_vm;
    // the mixed form's Newton ran in single precision alone this iteration
    // (the predicate nr_unit used): it may not end the increment
    const bool fp32_only = d.nr32 && (first_iter || fmax(fabs(Err_e0), fabs(Err_s0)) > VOCE_POLISH_ERR);
    // lane q < 9: SigAvg[q]; lane 9 + q: SigAvg1[q] (phase 1)
    if (lane < 18) {
        double s9[9];
        sym9_from_b(tot + (lane < 9 ? 2 : 8), s9);
        const int q = lane < 9 ? lane : lane - 9;
        const double v = s9[q] * (lane < 9 ? d.wgt : d.wgt_ratio);
        if (lane < 9) m->SigAvg[q] = v;
        else m->SigAvg1[q] = v;
    }
    // entries get_smacro leaves alone keep their value
    if (lane < 9) s_dg[lane] = m->dDisGradAvg[lane];
    __syncwarp();
    // lane i < 6: dDisGradAvg at IJV(i) (get_smacro)
    if (lane < 6) {
        const int ii = IJV0[lane], jj = IJV1[lane];
        double s = 0.0;
        if (d.vflag[lane] == 0)
#pragma unroll
            for (int k = 0; k < 6; ++k) {
                const int kk = IJV0[k], ll = IJV1[k];
                s += d.S0t[((ii * 3 + jj) * 3 + kk) * 3 + ll] * d.sflag[k] *
                     (d.Scauchy[kk * 3 + ll] - m->SigAvg[kk * 3 + ll]);
            }
        s_dg[ii * 3 + jj] = s;
    }
    __syncwarp();
    if (lane < 9) {
        const double dg = s_dg[lane];
        m->dDisGradAvg[lane] = dg;
        m->dDisGradAvg_acum[lane] += dg;
    }
    // lane 0: s_vm, lane 1: s_vm1
    if (lane < 2) {
        const double v = svm_of(lane == 0 ? m->SigAvg : m->SigAvg1);
        if (lane == 0) m->s_vm = v;
        else m->s_vm1 = v;
        s_vm2[lane] = v;
    }
    __syncwarp();
    // lane 0: Err_s = sum / s_vm; lane 1: Err_e = sum / e_vm when e_vm > 1e-5
    // (x / 1.0 is x exactly, so the untaken division is a division by one)
    double err = 0.0;
    if (lane < 2) {
        const double num = tot[lane == 0 ? 0 : 1] * d.wgt;
        const double den = lane == 0 ? s_vm2[0] : (fabs(e_vm) > 1E-5 ? e_vm : 1.0);
        err = num / den;
    }
    const double Err_s = __shfl_sync(0xffffffffu, err, 0), Err_e = __shfl_sync(0xffffffffu, err, 1);
    if (lane == 0) {
        m->Err_e = Err_e;
        m->Err_s = Err_s;
    }
    if (it < d.iter_max && lane < VOCE_ITLOG) {
        const int slot = (istep - 1) % d.incr_cap;
        double *lg = d.itlog + ((long long)slot * d.iter_max + it) * VOCE_ITLOG;
        double v;
        switch (lane) {
        case 0: v = Err_e; break;
        case 1: v = Err_s; break;
        case 2: v = s_vm2[0]; break;
        case 3: v = tot[14]; break;
        case 4: v = tot[1]; break;   // raw sum of the strain-compatibility norms
        case 5: v = tot[0]; break;   // raw sum of the stress-change norms
        default: v = tot[2 + lane - 6]; break;   // sum of sigma (basis)
        }
        lg[lane] = v;
    }
    __syncwarp();
    const bool more = (it + 1 < d.iter_max) &&
                      (fp32_only || fmax(fabs(Err_s), fabs(Err_e)) > fabs(d.err_tol));
    if (lane == 0) {
        m->iter = it + 1;
        m->iter_total += 1;
        m->nr_total += tot[14];
        m->nr_max = max(m->nr_max, (int)tot[15]);
        const double *dg = s_dg;
        double t6[6] = {dg[0], dg[4], dg[8], 0.5 * (dg[5] + dg[7]), 0.5 * (dg[2] + dg[6]), 0.5 * (dg[1] + dg[3])};
        t6_to_b<double>(t6, m->ddg6);
        m->first_iter = 0;
        m->pending_prelude = 0;
        m->converged = more ? 0 : 1;
    }
    if (more) return;
    // epilogue macro bookkeeping (evolution.c:438-461); lane q < 9 entry q
    if (lane < 9) {
        const int q = lane;
        const double act = m->DisGradAvg[q] + m->dDisGradAvg_acum[q];
        const double vga = (act - m->DisGradAvg_t[q]) / d.dt;
        s_act[0][q] = act;
        s_act[1][q] = vga;
        m->VelGradAvg[q] = vga;
        m->DisGradAvg_t[q] = act;
        m->DisGradAvg[q] = act + d.Udot[q] * d.dt;
        // the prelude of this increment used the previous DisGradAvg_actual
        m->DGA_prev[q] = m->DisGradAvg_actual[q];
        m->DisGradAvg_actual[q] = act;
    }
    __syncwarp();
    // lane 0: e_vm of DisGradAvg_actual, lane 1: d_vm of VelGradAvg
    if (lane < 2) {
        const double v = vm_strain(s_act[lane]);
        if (lane == 0) m->e_vm = v;
        else m->d_vm = v;
    }
    if (lane == 0) {
        // the displacement gradient received every dDisGradAvg of this
        // increment except the last one, which get_smacro computes after the
        // final update (evolution.c:391 vs :418): only those enter VelGrad
        double a[9];
        for (int q = 0; q < 9; ++q) a[q] = m->dDisGradAvg_acum[q] - s_dg[q];
        m->acum_a[0] = 0.5 * (a[5] - a[7]);
        m->acum_a[1] = 0.5 * (a[2] - a[6]);
        m->acum_a[2] = 0.5 * (a[1] - a[3]);
    }
    __syncwarp();
}


// Harden one voxel: harden() body (constitutive.c:261-305)
__device__ void harden_voxel(const RveDesc &d, long long v, const double *gd)
{
    const long long nv = d.nv;
    const double dt = d.dt;
    const double gamtot = d.gamacum[v];
    double deltgam = 0.0;
    for (int i = 0; i < d.nsys; ++i) d.gtot[i * nv + v] = d.gtot[i * nv + v] + gd[i] * dt;
    for (int i = 0; i < d.nsys; ++i) deltgam += fabs(gd[i]) * dt;
    for (int i = 0; i < d.nsys; ++i) {
        double dtau = 0.;
        for (int j = 0; j < d.nsys; ++j) dtau += d.hard[i * VOCE_NS + j] * fabs(gd[j]) * dt;
        const double tau0 = d.tau0[i], tau1 = d.tau1[i], th0 = d.thet0[i], th1 = d.thet1[i];
        const double tiny = 1.E-4 * tau0;
        double voce = 0.0;
        if (fabs(th0) > tiny) {
            voce = th1 * deltgam;
            if (fabs(tau1) > tiny) {
                const double fact = fabs(th0 / tau1);
                const double exp_ini = exp(-1.0 * gamtot * fact);
                const double exp_del = exp(-1.0 * deltgam * fact);
                voce += -1. * (fact * tau1 - th1) / fact * exp_ini * (exp_del - 1.0) -
                        th1 / fact * exp_ini * (exp_del * ((gamtot + deltgam) * fact + 1.0) - (gamtot * fact + 1.0));
            }
        }
        const double inc = dtau * voce / deltgam;
        const double c0 = d.crss[(2 * i) * nv + v] + inc;
        const double c1 = d.crss[(2 * i + 1) * nv + v] + inc;
        d.crss[(2 * i) * nv + v] = c0;
        d.crss[(2 * i + 1) * nv + v] = c1;
        d.itau[(2 * i) * nv + v] = 1.0 / c0;
        d.itau[(2 * i + 1) * nv + v] = 1.0 / c1;
        if (d.itau32) {
            put_pair(d.itau32, d.itau_lo, (2 * i) * nv + v, 1.0 / c0);
            put_pair(d.itau32, d.itau_lo, (2 * i + 1) * nv + v, 1.0 / c1);
        }
    }
    d.gamacum[v] = gamtot + deltgam;
}

// Orientation() (constitutive.c:117-169)
__device__ void orientation(double (&tran)[3][3], double (&rot)[3][3])
{
    double w[3] = {rot[2][1], rot[0][2], rot[1][0]};
    double wn = sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
    double wt = tan(wn / 2.0);
    if (fabs(wn) < 1E-6) wn = 1.0;
    for (int i = 0; i < 3; ++i) w[i] *= wt / wn;
    const double om[3][3] = {{0., -1. * w[2], w[1]}, {w[2], 0., -1. * w[0]}, {-1. * w[1], w[0], 0.}};
    double om2[3][3], tn[3][3];
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            double s = 0.0;
            for (int i = 0; i < 3; ++i) s += om[a][i] * om[i][b];
            om2[a][b] = s;
        }
    wt = wt * wt;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) rot[a][b] = (double)(a == b) + 2. * (om[a][b] + om2[a][b]) / (1. + wt);
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            double s = 0.0;
            for (int i = 0; i < 3; ++i) s += rot[a][i] * tran[i][b];
            tn[a][b] = s;
        }
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) tran[a][b] = tn[a][b];
}

// increment epilogue (evolution.c:433-530; update_orient constitutive.c:171-248; harden :250-310;
// update_schmid kinematics.c:426-459)
__device__ void incr_end_unit(const RveDesc &d, int unit, int nunits)
{
    double acc[VOCE_NPART];
    for (int q = 0; q < VOCE_NPART; ++q) acc[q] = 0.0;
    const MacroDev *m = d.macro;
    const long long nv = d.nv;
    const double dt = d.dt;
    const int istep = m->istep;
    const bool upd = d.update_flag == 1 && istep > 1;
    const bool hrd = d.hard_flag == 1 && istep > 2;
    // under creep the prelude set DisGrad to the previous DisGradAvg_actual
    double dga_start_c[3];
    {
        const double *p = m->DGA_prev;
        dga_start_c[0] = 0.5 * (p[5] - p[7]);
        dga_start_c[1] = 0.5 * (p[2] - p[6]);
        dga_start_c[2] = 0.5 * (p[1] - p[3]);
    }
    for (long long v = (long long)unit * blockDim.x + threadIdx.x; v < nv;
         v += (long long)nunits * blockDim.x) {
        const int ph = d.phase[v];
        // antisymmetric displacement gradient bookkeeping
        double rl[3];
        for (int c = 0; c < 3; ++c) {
            const double prev = d.dga[c * nv + v];
            const double st = d.creep ? dga_start_c[c] : prev + d.ua[c] * dt;
            const double en = st + m->acum_a[c] + d.rotl[c * nv + v];
            rl[c] = (en - prev) / dt;
            d.dga[c * nv + v] = en;
        }
        double e5[5] = {0, 0, 0, 0, 0}, ed[5] = {0, 0, 0, 0, 0};
        for (int c = 0; c < 5; ++c) e5[c] = d.eps[c * nv + v];
        if (d.solid[ph]) {
            double sp[6], gd[VOCE_NS], tx[VOCE_NS];
            for (int c = 0; c < 6; ++c) sp[c] = d.sigp[c * nv + v];
            flow_rule<false, true, double>(d, v, sp, ed, (double *)nullptr, gd, tx);
            for (int k = 0; k < d.nsys; ++k) {
                d.gamdot[k * nv + v] = gd[k];
                d.taux[k * nv + v] = tx[k];
            }
            for (int c = 0; c < 5; ++c) d.edot[c * nv + v] = ed[c];
            // SVM from the new stress, EVM from the total strain of the last
            // Newton iteration (evolution.c:134-155)
            double s6[6], s9[9], te6[6], t9[9];
            for (int c = 0; c < 6; ++c) s6[c] = d.sig[c * nv + v];
            sym9_from_b(s6, s9);
            {
                double tr = s9[0] + s9[4] + s9[8], acc2 = 0.0;
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b) {
                        double x = s9[3 * a + b] - (double)(a == b) * tr / 3.0;
                        acc2 += x * x;
                    }
                d.svm[v] = sqrt(3. / 2. * acc2);
            }
            for (int i = 0; i < 6; ++i) {
                double s = (i < 5 ? e5[i] + ed[i] * dt : 0.0);
                for (int j = 0; j < 6; ++j) s += d.sg[(long long)sym6(i, j) * nv + v] * sp[j];
                te6[i] = s;
            }
            sym9_from_b(te6, t9);
            {
                double tr = t9[0] + t9[4] + t9[8], acc2 = 0.0;
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b) {
                        double x = t9[3 * a + b] - (double)(a == b) * tr / 3.0;
                        acc2 += x * x;
                    }
                d.evm[v] = sqrt(2. / 3. * acc2);
            }
            // Eps += Edot dt (evolution.c:464-468)
            for (int c = 0; c < 5; ++c) {
                e5[c] = e5[c] + ed[c] * dt;
                d.eps[c * nv + v] = e5[c];
            }
            // resolved shear stresses for the diagnostics, with the Schmid
            // tensors of this increment (the reorientation below replaces them)
            double rss[VOCE_NS];
            if (hrd)
                for (int k = 0; k < d.nsys; ++k) {
                    const double *sc = d.sch + (long long)(5 * k) * nv + v;
                    rss[k] = sc[0] * s6[0] + sc[nv] * s6[1] + sc[2 * nv] * s6[2] + sc[3 * nv] * s6[3] +
                             sc[4 * nv] * s6[4];
                }
            if (upd) {
                double T[3][3], RL[3][3], Lp[3][3], RS[3][3], Rot[3][3];
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b) {
                        T[a][b] = d.tm[(3 * a + b) * nv + v];
                        Lp[a][b] = 0.0;
                    }
                RL[0][0] = RL[1][1] = RL[2][2] = 0.0;
                RL[1][2] = rl[0]; RL[2][1] = -rl[0];
                RL[0][2] = rl[1]; RL[2][0] = -rl[1];
                RL[0][1] = rl[2]; RL[1][0] = -rl[2];
                for (int s = 0; s < d.nsys; ++s) {
                    double bs[3], ns[3];
                    for (int a = 0; a < 3; ++a) {
                        bs[a] = 0.0; ns[a] = 0.0;
                        for (int b = 0; b < 3; ++b) {
                            bs[a] += T[a][b] * d.bb[3 * s + b];
                            ns[a] += T[a][b] * d.bn[3 * s + b];
                        }
                    }
                    for (int a = 0; a < 3; ++a)
                        for (int b = 0; b < 3; ++b) Lp[a][b] += bs[a] * ns[b] * gd[s];
                }
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b) RS[a][b] = (Lp[a][b] - Lp[b][a]) / 2.;
                acc[12] += sqrt(RS[2][1] * RS[2][1] + RS[0][2] * RS[0][2] + RS[1][0] * RS[1][0]) * d.wgt;
                acc[13] += sqrt(RL[2][1] * RL[2][1] + RL[0][2] * RL[0][2] + RL[1][0] * RL[1][0]) * d.wgt;
                const double Ua[3][3] = {{0.0, d.ua[2], d.ua[1]}, {-d.ua[2], 0.0, d.ua[0]}, {-d.ua[1], -d.ua[0], 0.0}};
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b) Rot[a][b] = (Ua[a][b] + RL[a][b] - RS[a][b]) * dt;
                orientation(T, Rot);
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b) d.tm[(3 * a + b) * nv + v] = T[a][b];
                schmid_from_tm(d, v, T);
            }
            if (hrd) {
                harden_voxel(d, v, gd);
                // rho_rss, rho_crss, work_p (evolution.c:509-529)
                const double ref = 0.35 * 47.565 * 0.256;
                double rr = 0.0, rc = 0.0, wp = 0.0;
                for (int k = 0; k < d.nsys; ++k) {
                    const double a = rss[k] / ref, b = d.crss[(2 * k) * nv + v] / ref;
                    rr += a * a;
                    rc += b * b;
                    wp += fabs(d.gtot[k * nv + v] * rss[k]);
                }
                d.diag[v] = rr;
                d.diag[nv + v] = rc;
                d.diag[2 * nv + v] = wp;
            }
        } else {
            for (int c = 0; c < 5; ++c) d.edot[c * nv + v] = 0.0;
        }
        for (int c = 0; c < 5; ++c) { acc[c] += e5[c]; acc[6 + c] += ed[c]; }
    }
    block_partials(acc, d.part + (long long)unit * VOCE_NPART);
}


// increment prelude (evolution.c:306-318): DisGrad += Udot dt, or, under
// creep, DisGrad := DisGradAvg_actual of the previous increment
__device__ void prelude_unit(const RveDesc &d, int unit, int nunits)
{
    const MacroDev *m = d.macro;
    double set6[6];
    {
        const double *a = m->DisGradAvg_actual;
        double t6[6] = {a[0], a[4], a[8], 0.5 * (a[5] + a[7]), 0.5 * (a[2] + a[6]), 0.5 * (a[1] + a[3])};
        t6_to_b<double>(t6, set6);
    }
    const long long nv = d.nv;
    for (long long v = (long long)unit * blockDim.x + threadIdx.x; v < nv;
         v += (long long)nunits * blockDim.x)
        for (int c = 0; c < 6; ++c) {
            if (d.creep) d.dgs[c * nv + v] = set6[c];
            else d.dgs[c * nv + v] += d.u6[c] * d.dt;
        }
}


__device__ void finalize_incr_body(const RveDesc &d, MacroDev *m, int npart)
{
    double tot[VOCE_NPART];
    reduce_partials(d.part, npart, tot);
    if (threadIdx.x != 0) return;
    double e6[6] = {tot[0], tot[1], tot[2], tot[3], tot[4], 0.0};
    double d6[6] = {tot[6], tot[7], tot[8], tot[9], tot[10], 0.0};
    double e9[9], d9[9];
    sym9_from_b(e6, e9);
    sym9_from_b(d6, d9);
    double evmp = 0.0, dvmp = 0.0;
    for (int q = 0; q < 9; ++q) {
        m->EpsAvg[q] = e9[q] * d.wgt;
        m->EdotAvg[q] = d9[q] * d.wgt;
        evmp += m->EpsAvg[q] * m->EpsAvg[q];
        dvmp += m->EdotAvg[q] * m->EdotAvg[q];
    }
    m->evmp = sqrt(2. / 3. * evmp);
    m->dvmp = sqrt(2. / 3. * dvmp);
    m->rsl = tot[12];
    m->rlc = tot[13];
    const int k = m->istep - 1;
    if (k >= 0 && d.incr_cap > 0) {
        IncrDev *r = d.incr + (k % d.incr_cap);
        r->istep = m->istep;
        r->iters = m->iter;
        r->iter_total = m->iter_total;
        r->nr_max = m->nr_max;
        r->e_vm = m->e_vm; r->evmp = m->evmp; r->d_vm = m->d_vm; r->dvmp = m->dvmp;
        r->s_vm = m->s_vm; r->s_vm1 = m->s_vm1;
        for (int q = 0; q < 9; ++q) {
            r->sig_avg[q] = m->SigAvg[q];
            r->sig_avg1[q] = m->SigAvg1[q];
            r->eps_avg[q] = m->EpsAvg[q];
            r->edot_avg[q] = m->EdotAvg[q];
            r->disgrad_avg[q] = m->DisGradAvg_actual[q];
        }
        r->err_e = m->Err_e; r->err_s = m->Err_s;
        r->rsl = m->rsl; r->rlc = m->rlc;
        r->nr_total = m->nr_total;
    }
    // reset for the next increment (evolution.c:330-340)
    m->istep += 1;
    if (m->istep > m->target) { m->active = 0; m->pending_prelude = 0; }
    else m->pending_prelude = 1;
    m->iter = 0;
    m->converged = 0;
    m->first_iter = 1;
    m->nr_max = 0;
    m->nr_total = 0.0;
    m->Err_e = 2. * d.err_tol;
    m->Err_s = 2. * d.err_tol;
    for (int q = 0; q < 9; ++q) { m->dDisGradAvg[q] = 0.0; m->dDisGradAvg_acum[q] = 0.0; }
    for (int q = 0; q < 6; ++q) m->ddg6[q] = 0.0;
    for (int q = 0; q < 3; ++q) m->acum_a[q] = 0.0;
}


// fields in the reference's layouts, for download
__global__ void k_field_out(RveDesc d, int field, double *out)
{
    const long long nv = d.nv;
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < nv;
         v += (long long)gridDim.x * blockDim.x) {
        double b6[6] = {0, 0, 0, 0, 0, 0}, t9[9], t6[6];
        switch (field) {
        case 0: case 20:
            for (int c = 0; c < 6; ++c) b6[c] = d.sig[c * nv + v];
            break;
        case 1:
            for (int c = 0; c < 5; ++c) b6[c] = d.eps[c * nv + v];
            break;
        case 2: case 21:
            for (int c = 0; c < 5; ++c) b6[c] = d.edot[c * nv + v];
            break;
        case 3:
            for (int c = 0; c < 6; ++c) b6[c] = d.dgs[c * nv + v];
            break;
        default: break;
        }
        switch (field) {
        case 0: case 1: case 2:
            sym9_from_b(b6, t9);
            for (int q = 0; q < 9; ++q) out[9 * v + q] = t9[q];
            break;
        case 3: {
            sym9_from_b(b6, t9);
            const double a0 = d.dga[v], a1 = d.dga[nv + v], a2 = d.dga[2 * nv + v];
            t9[5] += a0; t9[7] -= a0;
            t9[2] += a1; t9[6] -= a1;
            t9[1] += a2; t9[3] -= a2;
            for (int q = 0; q < 9; ++q) out[9 * v + q] = t9[q];
            break;
        }
        case 4:
            for (int q = 0; q < 9; ++q) out[9 * v + q] = d.tm[q * nv + v];
            break;
        case 5:
            for (int k = 0; k < VOCE_NS; ++k) out[VOCE_NS * v + k] = d.crss[(2 * k) * nv + v];
            break;
        case 6:
            for (int k = 0; k < VOCE_NS; ++k) out[VOCE_NS * v + k] = d.gamdot[k * nv + v];
            break;
        case 7: out[v] = d.gamacum[v]; break;
        case 8: out[v] = d.svm[v]; break;
        case 9: out[v] = d.evm[v]; break;
        case 10:
            for (int k = 0; k < VOCE_NS; ++k) out[VOCE_NS * v + k] = d.gtot[k * nv + v];
            break;
        case 11:
            for (int k = 0; k < VOCE_NS; ++k) out[VOCE_NS * v + k] = d.taux[k * nv + v];
            break;
        case 12: case 13: case 14: out[v] = d.diag[(field - 12) * nv + v]; break;
        case 20: case 21:
            b_to_t6<double>(b6, t6);
            for (int c = 0; c < 6; ++c) out[(long long)c * nv + v] = t6[c];
            break;
        default: break;
        }
    }
}


// ===========================================================================
// batched entry points: one launch per phase covers many RVEs.  Work item w
// of a phase is map[w] = (rve, unit); the unit functions are the ones the
// single-RVE kernels call, so an RVE computes the same numbers alone and in
// a batch.  RVEs are skipped per phase by their macro flags.
// ===========================================================================
enum { MASK_ACTIVE = 0, MASK_CONVERGED = 1, MASK_PRELUDE = 2 };

__device__ __forceinline__ bool unit_on(const RveDesc &d, int mask)
{
    const MacroDev *m = d.macro;
    if (!m->active) return false;
    if (mask == MASK_CONVERGED) return m->converged != 0;
    if (mask == MASK_PRELUDE) return m->pending_prelude != 0;
    return true;
}

// resident blocks per SM the single-precision z passes are compiled for
// (256^3, mixed forms, us per launch: z forward / inverse 461 / 946 at 2,
// 524 / 1239 at 3, 586 / 1319 at 4, 461 / 1098 at 1)
#ifndef VOCE_FFTZ32_BLOCKS
#define VOCE_FFTZ32_BLOCKS 2
#endif
template <typename R>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? VOCE_FFTZ32_BLOCKS : 1)
kb_fft_z_fwd(const RveDesc *descs, const int2 *map, int total)
{
    for (int w = blockIdx.x; w < total; w += gridDim.x) {
        const int2 e = map[w];
        const RveDesc &d = descs[e.x];
        if (!unit_on(d, MASK_ACTIVE)) continue;
        fft_z_fwd_unit<R>(d, d.zrows, e.y);
        __syncthreads();
    }
}

// which: 0 spectrum forward, 1 spectrum inverse, 2 antisymmetric accumulator inverse
// cp.async of a y tile (NL lines of L contiguous coefficients at g) into the
// stream layout; with 256 threads and L dividing 256 a thread keeps its
// coefficient index and steps by whole lines
template <int N1, int N2>
__device__ __forceinline__ void ystream_issue(float2 *A, const float2 *g, int NL)
{
    constexpr int L = N1 * N2, LP = L + N1 + 1;
    if (256 % L == 0 && blockDim.x == 256) {
        constexpr int dl = 256 % L == 0 ? 256 / L : 1;
        const int i = threadIdx.x % L;
        float2 *s = A + (threadIdx.x / L) * LP + i + i / N2;
        const float2 *src = g + threadIdx.x;
        for (int l = threadIdx.x / L; l < NL; l += dl, s += dl * LP, src += 256) cp_async8(s, src);
    } else {
        for (int e = threadIdx.x; e < NL * L; e += blockDim.x) {
            const int l = e / L, i = e - l * L;
            cp_async8(A + l * LP + i + i / N2, g + e);
        }
    }
}

__device__ void fft_y_stream_f32(const RveDesc *descs, const int2 *map, int total, int which, int S)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2 *cur = reinterpret_cast<float2 *>(smem_raw), *nxt = cur + S;
    const int mask = which == 2 ? MASK_CONVERGED : MASK_ACTIVE;
    const int sign = which == 0 ? -1 : +1;
    auto next_on = [&](int w) {
        while (w < total && !unit_on(descs[map[w].x], mask)) w += gridDim.x;
        return w;
    };
    // the unit's RVE, its spectrum (y lines: contiguous) and tile base
    auto tile = [&](int w, const RveDesc *&dp, float2 *&g) {
        const int2 e = map[w];
        dp = &descs[e.x];
        const RveDesc &d = *dp;
        const int xtiles = d.nx / d.yxt;
        const int line = e.y / xtiles, x0 = (e.y % xtiles) * d.yxt;
        g = (float2 *)(which == 2 ? d.aacc : d.spec) + ((long long)line * d.nx + x0) * d.ny;
    };
    auto issue = [&](int w, float2 *A) {
        const RveDesc *dp;
        float2 *g;
        tile(w, dp, g);
        switch (dp->ny) {
        case 16: ystream_issue<4, 4>(A, g, dp->yxt); break;
        case 24: ystream_issue<4, 6>(A, g, dp->yxt); break;
        case 32: ystream_issue<4, 8>(A, g, dp->yxt); break;
        case 48: ystream_issue<6, 8>(A, g, dp->yxt); break;
        case 64: ystream_issue<8, 8>(A, g, dp->yxt); break;
        case 96: ystream_issue<8, 12>(A, g, dp->yxt); break;
        case 128: ystream_issue<8, 16>(A, g, dp->yxt); break;
        case 192: ystream_issue<12, 16>(A, g, dp->yxt); break;
        case 256: ystream_issue<16, 16>(A, g, dp->yxt); break;
        default: break;
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    };
    int w = next_on(blockIdx.x);
    if (w < total) issue(w, cur);
    while (w < total) {
        const int nw = next_on(w + gridDim.x);
        if (nw < total) {
            issue(nw, nxt);
            asm volatile("cp.async.wait_group 1;" ::: "memory");
        } else {
            cp_async_wait_all();
        }
        __syncthreads();
        const RveDesc *dp;
        float2 *g;
        tile(w, dp, g);
        const float2 *tw = (const float2 *)dp->twy;
        const int NL = dp->yxt;
#define VOCE_YSTREAM(L_, N1_) \
    case L_: \
        if (sign < 0) ystream_tile<N1_, L_ / N1_, -1>(cur, NL, g, tw); \
        else ystream_tile<N1_, L_ / N1_, 1>(cur, NL, g, tw); \
        break;
        switch (dp->ny) {
        VOCE_YSTREAM(16, 4)
        VOCE_YSTREAM(24, 4)
        VOCE_YSTREAM(32, 4)
        VOCE_YSTREAM(48, 6)
        VOCE_YSTREAM(64, 8)
        VOCE_YSTREAM(96, 8)
        VOCE_YSTREAM(128, 8)
        VOCE_YSTREAM(192, 12)
        VOCE_YSTREAM(256, 16)
        default: break;
        }
#undef VOCE_YSTREAM
        __syncthreads();
        float2 *t = cur; cur = nxt; nxt = t;
        w = nw;
    }
}

// resident blocks per SM the single-precision y and Green passes are
// compiled for (their register budget)
#ifndef VOCE_FFTY32_BLOCKS
#define VOCE_FFTY32_BLOCKS 2
#endif
#ifndef VOCE_FFTXG32_BLOCKS
#define VOCE_FFTXG32_BLOCKS 2
#endif
template <typename R>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? VOCE_FFTY32_BLOCKS : 1)
kb_fft_y(const RveDesc *descs, const int2 *map, int total, int which, int stream)
{
    if constexpr (sizeof(R) == 4) {
        if (stream > 0) {
            fft_y_stream_f32(descs, map, total, which, stream);
            return;
        }
    }
    for (int w = blockIdx.x; w < total; w += gridDim.x) {
        const int2 e = map[w];
        const RveDesc &d = descs[e.x];
        if (!unit_on(d, which == 2 ? MASK_CONVERGED : MASK_ACTIVE)) continue;
        fft_y_unit<R>(d, which == 2 ? d.aacc : d.spec, which == 0 ? -1 : +1, d.yxt, e.y);
        __syncthreads();
    }
}

// resident blocks per SM the Green pass is compiled for (registers): 3 with
// the FP64 spectrum (measured faster despite some spilling), 2 with FP32
// (256^3 FP32, us per launch: 641 at 2, 1095 at 3, 1227 at 4: the register
// FFT spills below 128 registers)
template <typename R>
__global__ void __launch_bounds__(256, sizeof(R) == 8 ? 3 : VOCE_FFTXG32_BLOCKS)
kb_fft_x_green(const RveDesc *descs, const int2 *map, int total)
{
    for (int w = blockIdx.x; w < total; w += gridDim.x) {
        const int2 e = map[w];
        const RveDesc &d = descs[e.x];
        if (!unit_on(d, MASK_ACTIVE)) continue;
        bool done = false;
        if constexpr (sizeof(R) == 4) {
            if (d.plx.n1 > 0) {
                done = true;
                switch (d.nx) {
                case 16: xg_unit_f32<4, 4>(d, d.xkc, e.y); break;
                case 24: xg_unit_f32<4, 6>(d, d.xkc, e.y); break;
                case 32: xg_unit_f32<4, 8>(d, d.xkc, e.y); break;
                case 48: xg_unit_f32<6, 8>(d, d.xkc, e.y); break;
                case 64: xg_unit_f32<8, 8>(d, d.xkc, e.y); break;
                case 96: xg_unit_f32<8, 12>(d, d.xkc, e.y); break;
                case 128: xg_unit_f32<8, 16>(d, d.xkc, e.y); break;
                case 192: xg_unit_f32<12, 16>(d, d.xkc, e.y); break;
                case 256: xg_unit_f32<16, 16>(d, d.xkc, e.y); break;
                default: done = false; break;
                }
            }
        }
        if (!done) fft_x_green_unit<R>(d, d.xkc, e.y);
        __syncthreads();
    }
}

template <typename R>
__global__ void __launch_bounds__(256) kb_fft_x_aacc(const RveDesc *descs, const int2 *map, int total)
{
    for (int w = blockIdx.x; w < total; w += gridDim.x) {
        const int2 e = map[w];
        const RveDesc &d = descs[e.x];
        if (!unit_on(d, MASK_CONVERGED)) continue;
        fft_x_unit<R>(d, d.aacc, 3, +1, d.xkc3, e.y);
        __syncthreads();
    }
}

// mode 0: spectrum -> displacement gradient; 1: accumulator -> rotl
template <typename R>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? VOCE_FFTZ32_BLOCKS : 1)
kb_fft_z_inv(const RveDesc *descs, const int2 *map, int total, int mode)
{
    for (int w = blockIdx.x; w < total; w += gridDim.x) {
        const int2 e = map[w];
        const RveDesc &d = descs[e.x];
        if (!unit_on(d, mode == 0 ? MASK_ACTIVE : MASK_CONVERGED)) continue;
        if (mode == 0) {
            if constexpr (sizeof(R) == 4) fft_z_inv_dgs_f32(d, d.zirows, e.y);
            else fft_z_inv_unit<R>(d, d.spec, 6, d.zirows, 0, e.y);
        } else {
            fft_z_inv_unit<R>(d, d.aacc, 3, d.zirows3, 1, e.y);
        }
        __syncthreads();
    }
}

// resident blocks of 128 threads per SM the single-precision Newton kernel
// (kb_nr<true>) is compiled for (register budget 65536 / (128 x blocks))
#ifndef VOCE_NR_MIXED_BLOCKS
#define VOCE_NR_MIXED_BLOCKS 3
#endif

// CHORD: the FP64 Newton may take chord steps (VOCE_PREC_MIXED plans; each
// RVE's d.chord decides); the FP64 form's instance is the exact-Jacobian one
// IR: the VOCE_PREC_MIXED_IR form (FP64 residual, float Jacobian)
#ifndef VOCE_NR_IR_BLOCKS
#define VOCE_NR_IR_BLOCKS 3
#endif
template <bool NR32, bool CHORD = false, bool IR = false>
__global__ void __launch_bounds__(128, NR32 ? VOCE_NR_MIXED_BLOCKS : IR ? VOCE_NR_IR_BLOCKS : 1)
kb_nr(const RveDesc *descs, const int2 *map, int total)
{
    for (int w = blockIdx.x; w < total; w += gridDim.x) {
        const int2 e = map[w];
        const RveDesc &d = descs[e.x];
        if (!unit_on(d, MASK_ACTIVE)) continue;
        nr_unit<NR32, CHORD, IR>(d, e.y, d.npart);
    }
}

__global__ void __launch_bounds__(128) kb_incr_end(const RveDesc *descs, const int2 *map, int total)
{
    for (int w = blockIdx.x; w < total; w += gridDim.x) {
        const int2 e = map[w];
        const RveDesc &d = descs[e.x];
        if (!unit_on(d, MASK_CONVERGED)) continue;
        incr_end_unit(d, e.y, d.npart);
    }
}

__global__ void __launch_bounds__(128) kb_prelude(const RveDesc *descs, const int2 *map, int total)
{
    for (int w = blockIdx.x; w < total; w += gridDim.x) {
        const int2 e = map[w];
        const RveDesc &d = descs[e.x];
        if (!unit_on(d, MASK_PRELUDE)) continue;
        prelude_unit(d, e.y, d.npart);
    }
}

// one block per RVE.  With use_cond (a plan of one RVE), the iteration
// finaliser also sets the condition of the graph's WHILE node: continue
// while the RVE has not converged (evolution.c:342).
// The RVE's descriptor and macro state are first copied into shared memory
// by the whole block, so that the finaliser's single thread reads and
// updates them at shared-memory latency instead of in a chain of dependent
// global round trips; the macro state is written back once at the end.  The
// arithmetic is unchanged.
__global__ void __launch_bounds__(256) kb_finalize(const RveDesc *descs, int nrve, int incr_end,
                                                   cudaGraphConditionalHandle cond, int use_cond)
{
    static_assert(sizeof(RveDesc) % 8 == 0 && sizeof(MacroDev) % 8 == 0, "staged as 8-byte words");
    constexpr int kDescWords = (int)(sizeof(RveDesc) / 8), kMacroWords = (int)(sizeof(MacroDev) / 8);
    __shared__ unsigned long long s_desc[kDescWords];
    __shared__ unsigned long long s_macro[kMacroWords];
    for (int r = blockIdx.x; r < nrve; r += gridDim.x) {
        const RveDesc &dg = descs[r];
        if (!unit_on(dg, incr_end ? MASK_CONVERGED : MASK_ACTIVE)) continue;
        unsigned long long *gm = reinterpret_cast<unsigned long long *>(dg.macro);
        const unsigned long long *gd = reinterpret_cast<const unsigned long long *>(&dg);
        for (int i = threadIdx.x; i < kDescWords; i += blockDim.x) s_desc[i] = gd[i];
        for (int i = threadIdx.x; i < kMacroWords; i += blockDim.x) s_macro[i] = gm[i];
        __syncthreads();
        const RveDesc &d = *reinterpret_cast<const RveDesc *>(s_desc);
        MacroDev *m = reinterpret_cast<MacroDev *>(s_macro);
        if (incr_end) finalize_incr_body(d, m, d.npart);
        else finalize_iter_body(d, m, d.npart);
        __syncthreads();
        for (int i = threadIdx.x; i < kMacroWords; i += blockDim.x) gm[i] = s_macro[i];
        if (use_cond && threadIdx.x == 0) cudaGraphSetConditional(cond, m->converged ? 0u : 1u);
        __syncthreads();
    }
}

// loop condition of the batch: continue while any RVE is active and the
// tick budget is not spent
__global__ void kb_cond(const RveDesc *descs, int nrve, int *ticks, const int *max_ticks,
                        int *active_out, cudaGraphConditionalHandle cond, int use_cond)
{
    __shared__ int any;
    if (threadIdx.x == 0) any = 0;
    __syncthreads();
    int a = 0;
    for (int r = threadIdx.x; r < nrve; r += blockDim.x) a += descs[r].macro->active;
    if (a) atomicAdd(&any, a);
    __syncthreads();
    if (threadIdx.x == 0) {
        const int t = *ticks + 1;
        *ticks = t;
        *active_out = any;
        if (use_cond) cudaGraphSetConditional(cond, (any > 0 && t < *max_ticks) ? 1u : 0u);
    }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
template <typename R>
static int pick_div(int n, int limit)
{
    int best = 1;
    for (int k = 1; k <= n; ++k)
        if (n % k == 0 && k <= limit) best = k;
    return best;
}

template <typename R>
void Tiles::choose(const RveDesc &d)
{
    const int budget = (sizeof(R) == 8) ? 2048 : 4096;  // complex elements per buffer
    zrows = pick_div<R>(d.ny, budget / (3 * d.nz));
    yxt = pick_div<R>(d.nx, budget / d.ny);
    xkc = pick_div<R>(d.ny, (budget * 3 / 2) / (6 * d.nx));
    xkc3 = pick_div<R>(d.ny, (budget * 3 / 2) / (3 * d.nx));
    zirows = pick_div<R>(d.ny, budget / (3 * d.nz));
    zirows3 = pick_div<R>(d.ny, budget / (2 * d.nz));
}
template void Tiles::choose<double>(const RveDesc &);
template void Tiles::choose<float>(const RveDesc &);


template <typename R>
static size_t smem_lines(int L, int NL)
{
    return (size_t)2 * L * (size_t)(NL | 1) * sizeof(typename Cx<R>::T);
}

void batch_units(const RveDesc &d, int u[BP_COUNT])
{
    u[BP_NP] = d.npart;
    u[BP_ZF] = d.nx * (d.ny / d.zrows);
    u[BP_Y6] = 6 * d.nzh * (d.nx / d.yxt);
    u[BP_XG] = d.nzh * (d.ny / d.xkc);
    u[BP_ZI] = d.nx * (d.ny / d.zirows);
    u[BP_X3] = d.nzh * (d.ny / d.xkc3);
    u[BP_Y3] = 3 * d.nzh * (d.nx / d.yxt);
    u[BP_Z3] = d.nx * (d.ny / d.zirows3);
}

template <typename R>
static size_t batch_smem_t(const RveDesc &d, int ph)
{
    if (sizeof(R) == 4) {   // the staged single-precision z passes, the register-FFT Green pass
        if (ph == BP_ZF) return sizeof(float2) * (size_t)zf32_fwd_size(d.nz, d.zrows);
        if (ph == BP_ZI) return sizeof(float2) * (size_t)zi32_size(d.nz, d.nzh, d.zirows);
        if (ph == BP_XG && d.plx.n1 > 0) return xg32_smem(d.nx, d.plx.n1, d.xkc);
    }
    switch (ph) {
    case BP_ZF: return smem_lines<R>(d.nz, 3 * d.zrows);
    case BP_Y6: case BP_Y3: return smem_lines<R>(d.ny, d.yxt);
    case BP_XG: return smem_lines<R>(d.nx, 6 * d.xkc);
    case BP_ZI: return smem_lines<R>(d.nz, 3 * d.zirows);
    case BP_X3: return smem_lines<R>(d.nx, 3 * d.xkc3);
    case BP_Z3: return smem_lines<R>(d.nz, 2 * d.zirows3);
    default: return 0;
    }
}

size_t batch_smem(const RveDesc &d, int ph)
{
    return d.mixed ? batch_smem_t<float>(d, ph) : batch_smem_t<double>(d, ph);
}

template <typename R>
static cudaError_t set_batch_smem_t(const BatchPlan &bp)
{
    auto set = [](const void *fn, size_t b) {
        if (b) cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b);
    };
    set((const void *)kb_fft_z_fwd<R>, bp.smem[BP_ZF]);
    set((const void *)kb_fft_y<R>, std::max(bp.smem[BP_Y6], bp.smem[BP_Y3]));
    set((const void *)kb_fft_x_green<R>, bp.smem[BP_XG]);
    set((const void *)kb_fft_x_aacc<R>, bp.smem[BP_X3]);
    set((const void *)kb_fft_z_inv<R>, std::max(bp.smem[BP_ZI], bp.smem[BP_Z3]));
    return cudaGetLastError();
}

cudaError_t set_batch_smem(const BatchPlan &bp)
{
    return bp.mixed ? set_batch_smem_t<float>(bp) : set_batch_smem_t<double>(bp);
}

// dynamic shared memory of kb_nr<true>: the staged float model columns
static const int kNrStageBytes = VOCE_STAGE_FLOATS * VOCE_NR_THREADS * (int)sizeof(float);

// Newton-kernel blocks resident per GPU (SMs x blocks per SM): the grid cap
// of kb_nr and the most units an RVE is split into for it.  The first call
// also raises kb_nr<true>'s dynamic shared-memory limit; it is made when an
// RVE is created, before any launch or stream capture.
int nr_resident_blocks(int kind)
{
    // several host threads may ask at once: each computes the same value
    static std::atomic<int> cached[3];
    std::atomic<int> &c = cached[(kind >= 0 && kind < 3) ? kind : 0];
    if (!c.load()) {
        int dev = 0, sms = 152, per = 2;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (kind == 1) {
            cudaFuncSetAttribute(kb_nr<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kNrStageBytes);
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kb_nr<true>, VOCE_NR_THREADS, kNrStageBytes);
        } else if (kind == 2) {
            cudaFuncSetAttribute(kb_nr<false, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 kNrStageBytes);
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kb_nr<false, false, true>, VOCE_NR_THREADS,
                                                          kNrStageBytes);
        } else {
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kb_nr<false>, VOCE_NR_THREADS, 0);
        }
        c.store(sms * (per > 0 ? per : 1));
    }
    return c.load();
}

static int grid_for(int total, int cap)
{
    return total < cap ? (total > 0 ? total : 1) : cap;
}

template <typename R>
static void plan_prelude_t(const BatchPlan &bp, cudaStream_t s, Prof &pf)
{
    const int NG = 152 * 2;
    pf.begin(K_PRELUDE, s);
    kb_prelude<<<grid_for(bp.total[BP_NP], NG), 128, 0, s>>>(bp.descs, bp.map[BP_NP], bp.total[BP_NP]);
    pf.end(K_PRELUDE, s);
}

template <typename R>
static void plan_iteration_t(const BatchPlan &bp, cudaStream_t s, Prof &pf, cudaGraphConditionalHandle cond,
                             int use_cond)
{
    const int FG = 152 * 4;
    const RveDesc *D = bp.descs;
    pf.begin(K_FFT_Z_FWD, s);
    kb_fft_z_fwd<R><<<grid_for(bp.total[BP_ZF], FG), 256, bp.smem[BP_ZF], s>>>(D, bp.map[BP_ZF], bp.total[BP_ZF]);
    pf.end(K_FFT_Z_FWD, s);
    pf.begin(K_FFT_Y_FWD, s);
    kb_fft_y<R><<<grid_for(bp.total[BP_Y6], FG), 256, bp.smem[BP_Y6], s>>>(D, bp.map[BP_Y6], bp.total[BP_Y6], 0, bp.ystream);
    pf.end(K_FFT_Y_FWD, s);
    pf.begin(K_FFT_X_GREEN, s);
    kb_fft_x_green<R><<<grid_for(bp.total[BP_XG], FG), 256, bp.smem[BP_XG], s>>>(D, bp.map[BP_XG], bp.total[BP_XG]);
    pf.end(K_FFT_X_GREEN, s);
    pf.begin(K_FFT_Y_INV, s);
    kb_fft_y<R><<<grid_for(bp.total[BP_Y6], FG), 256, bp.smem[BP_Y6], s>>>(D, bp.map[BP_Y6], bp.total[BP_Y6], 1, bp.ystream);
    pf.end(K_FFT_Y_INV, s);
    pf.begin(K_FFT_Z_INV, s);
    kb_fft_z_inv<R><<<grid_for(bp.total[BP_ZI], FG), 256, bp.smem[BP_ZI], s>>>(D, bp.map[BP_ZI], bp.total[BP_ZI], 0);
    pf.end(K_FFT_Z_INV, s);
    pf.begin(K_NR, s);
    if (bp.nr32)
        kb_nr<true><<<grid_for(bp.total[BP_NP], nr_resident_blocks(1)), VOCE_NR_THREADS, kNrStageBytes, s>>>(
            D, bp.map[BP_NP], bp.total[BP_NP]);
    else if (bp.ir)
        kb_nr<false, false, true><<<grid_for(bp.total[BP_NP], nr_resident_blocks(2)), VOCE_NR_THREADS,
                                    kNrStageBytes, s>>>(D, bp.map[BP_NP], bp.total[BP_NP]);
    else if (bp.mixed)
        kb_nr<false, true><<<grid_for(bp.total[BP_NP], nr_resident_blocks(0)), VOCE_NR_THREADS, 0, s>>>(
            D, bp.map[BP_NP], bp.total[BP_NP]);
    else
        kb_nr<false><<<grid_for(bp.total[BP_NP], nr_resident_blocks(0)), VOCE_NR_THREADS, 0, s>>>(
            D, bp.map[BP_NP], bp.total[BP_NP]);
    pf.end(K_NR, s);
    pf.begin(K_FIN_ITER, s);
    kb_finalize<<<grid_for(bp.nrve, 152 * 4), 256, 0, s>>>(D, bp.nrve, 0, cond, use_cond);
    pf.end(K_FIN_ITER, s);
}

template <typename R>
static void plan_incr_end_t(const BatchPlan &bp, cudaStream_t s, Prof &pf)
{
    const int FG = 152 * 4, NG = 152 * 2;
    const RveDesc *D = bp.descs;
    pf.begin(K_INC_FFT, s);
    kb_fft_x_aacc<R><<<grid_for(bp.total[BP_X3], FG), 256, bp.smem[BP_X3], s>>>(D, bp.map[BP_X3], bp.total[BP_X3]);
    kb_fft_y<R><<<grid_for(bp.total[BP_Y3], FG), 256, bp.smem[BP_Y3], s>>>(D, bp.map[BP_Y3], bp.total[BP_Y3], 2, bp.ystream);
    kb_fft_z_inv<R><<<grid_for(bp.total[BP_Z3], FG), 256, bp.smem[BP_Z3], s>>>(D, bp.map[BP_Z3], bp.total[BP_Z3], 1);
    pf.end(K_INC_FFT, s, 3);
    pf.begin(K_INCR_END, s);
    kb_incr_end<<<grid_for(bp.total[BP_NP], NG), 128, 0, s>>>(D, bp.map[BP_NP], bp.total[BP_NP]);
    pf.end(K_INCR_END, s);
    pf.begin(K_FIN_INCR, s);
    kb_finalize<<<grid_for(bp.nrve, 152 * 4), 256, 0, s>>>(D, bp.nrve, 1, 0, 0);
    pf.end(K_FIN_INCR, s);
}

cudaError_t launch_plan_prelude(const BatchPlan &bp, cudaStream_t s, Prof &pf)
{
    if (bp.mixed) plan_prelude_t<float>(bp, s, pf);
    else plan_prelude_t<double>(bp, s, pf);
    return cudaGetLastError();
}

cudaError_t launch_plan_iteration(const BatchPlan &bp, cudaStream_t s, Prof &pf,
                                  cudaGraphConditionalHandle cond, int use_cond)
{
    if (bp.mixed) plan_iteration_t<float>(bp, s, pf, cond, use_cond);
    else plan_iteration_t<double>(bp, s, pf, cond, use_cond);
    return cudaGetLastError();
}

cudaError_t launch_plan_incr_end(const BatchPlan &bp, cudaStream_t s, Prof &pf)
{
    if (bp.mixed) plan_incr_end_t<float>(bp, s, pf);
    else plan_incr_end_t<double>(bp, s, pf);
    return cudaGetLastError();
}

template <typename R>
static void plan_phase_t(const BatchPlan &bp, int phase, cudaStream_t s)
{
    const int FG = 152 * 4;
    const RveDesc *D = bp.descs;
    switch (phase) {
    case BP_ZF:
        kb_fft_z_fwd<R><<<grid_for(bp.total[BP_ZF], FG), 256, bp.smem[BP_ZF], s>>>(D, bp.map[BP_ZF], bp.total[BP_ZF]);
        break;
    case BP_Y6:
        kb_fft_y<R><<<grid_for(bp.total[BP_Y6], FG), 256, bp.smem[BP_Y6], s>>>(D, bp.map[BP_Y6], bp.total[BP_Y6], 0, bp.ystream);
        break;
    case BP_XG:
        kb_fft_x_green<R><<<grid_for(bp.total[BP_XG], FG), 256, bp.smem[BP_XG], s>>>(D, bp.map[BP_XG], bp.total[BP_XG]);
        break;
    case BP_ZI:
        kb_fft_z_inv<R><<<grid_for(bp.total[BP_ZI], FG), 256, bp.smem[BP_ZI], s>>>(D, bp.map[BP_ZI], bp.total[BP_ZI], 0);
        break;
    default: break;
    }
}

cudaError_t launch_plan_phase(const BatchPlan &bp, int phase, cudaStream_t s)
{
    if (bp.mixed) plan_phase_t<float>(bp, phase, s);
    else plan_phase_t<double>(bp, phase, s);
    return cudaGetLastError();
}

int tile_candidates(const RveDesc &d, int phase, int *out, int max)
{
    const bool f = d.mixed != 0;
    const int B = f ? 4096 : 2048;
    const size_t cs = f ? sizeof(float2) : sizeof(double2);
    const size_t smem_max = 200 * 1024;
    int n = 0;
    for (int k = -2; k <= 2 && n < max; ++k) {
        const int budget = k < 0 ? (B >> -k) : (B << k);
        int t = 0;
        size_t sm = 0;
        switch (phase) {
        case BP_ZF:
            t = pick_div<double>(d.ny, budget / (3 * d.nz));
            sm = f ? cs * (size_t)zf32_fwd_size(d.nz, t) : 2 * (size_t)d.nz * ((3 * t) | 1) * cs;
            break;
        case BP_Y6: t = pick_div<double>(d.nx, budget / d.ny); sm = 2 * (size_t)d.ny * (t | 1) * cs; break;
        case BP_XG:
            t = pick_div<double>(d.ny, (budget * 3 / 2) / (6 * d.nx));
            sm = (f && d.plx.n1 > 0) ? xg32_smem(d.nx, d.plx.n1, t) : 2 * (size_t)d.nx * ((6 * t) | 1) * cs;
            break;
        case BP_ZI:
            t = pick_div<double>(d.ny, budget / (3 * d.nz));
            sm = f ? cs * (size_t)zi32_size(d.nz, d.nzh, t) : 2 * (size_t)d.nz * ((3 * t) | 1) * cs;
            break;
        default: return 0;
        }
        if (t < 1 || sm > smem_max) continue;
        bool seen = false;
        for (int i = 0; i < n; ++i) seen = seen || out[i] == t;
        if (!seen) out[n++] = t;
    }
    return n;
}

cudaError_t launch_batch_tick(const BatchPlan &bp, cudaStream_t s, cudaGraphConditionalHandle cond)
{
    Prof none;
    launch_plan_prelude(bp, s, none);
    launch_plan_iteration(bp, s, none, 0, 0);
    launch_plan_incr_end(bp, s, none);
    kb_cond<<<1, 256, 0, s>>>(bp.descs, bp.nrve, bp.ticks, bp.max_ticks, bp.active_out, cond, 1);
    return cudaGetLastError();
}

cudaError_t launch_batch_tick_timed(const BatchPlan &bp, cudaStream_t s, Prof &pf)
{
    launch_plan_prelude(bp, s, pf);
    launch_plan_iteration(bp, s, pf, 0, 0);
    launch_plan_incr_end(bp, s, pf);
    kb_cond<<<1, 256, 0, s>>>(bp.descs, bp.nrve, bp.ticks, bp.max_ticks, bp.active_out, 0, 0);
    pf.launches += 1;
    return cudaGetLastError();
}

// Periodic Voronoi labels: each voxel centre ((x+0.5)/nx, ...) of the unit
// cube takes the nearest seed by minimum-image distance, ties to the lowest
// index.  The arithmetic is that of the host generator's numpy form: the
// image by round-half-to-even (rint), the squared distance summed as
// (d0^2 + d1^2) + d2^2 without contraction, strict < over seeds in order.
__global__ void k_voronoi(int nx, int ny, int nz, int ns, const double *__restrict__ seeds,
                          int *__restrict__ label)
{
    extern __shared__ double s_seed[];   // 3 x VORONOI_TILE
    const long long nv = (long long)nx * ny * nz;
    const long long v0 = (long long)blockIdx.x * blockDim.x;
    const long long v = v0 + threadIdx.x;
    double p0 = 0.0, p1 = 0.0, p2 = 0.0;
    if (v < nv) {
        const int z = (int)(v % nz), y = (int)((v / nz) % ny), x = (int)(v / ((long long)ny * nz));
        p0 = ((double)x + 0.5) / (double)nx;
        p1 = ((double)y + 0.5) / (double)ny;
        p2 = ((double)z + 0.5) / (double)nz;
    }
    double best = 1e300;
    int bi = 0;
    for (int t0 = 0; t0 < ns; t0 += VORONOI_TILE) {
        const int tn = min(VORONOI_TILE, ns - t0);
        __syncthreads();
        for (int i = threadIdx.x; i < 3 * tn; i += blockDim.x) s_seed[i] = seeds[3 * t0 + i];
        __syncthreads();
        for (int j = 0; j < tn; ++j) {
            double d0 = __dsub_rn(p0, s_seed[3 * j]);
            double d1 = __dsub_rn(p1, s_seed[3 * j + 1]);
            double d2 = __dsub_rn(p2, s_seed[3 * j + 2]);
            d0 = __dsub_rn(d0, rint(d0));
            d1 = __dsub_rn(d1, rint(d1));
            d2 = __dsub_rn(d2, rint(d2));
            const double dd = __dadd_rn(__dadd_rn(__dmul_rn(d0, d0), __dmul_rn(d1, d1)), __dmul_rn(d2, d2));
            if (dd < best) {
                best = dd;
                bi = t0 + j;
            }
        }
    }
    if (v < nv) label[v] = bi;
}

cudaError_t launch_voronoi(int nx, int ny, int nz, int ns, const double *seeds, int *label, cudaStream_t s)
{
    const long long nv = (long long)nx * ny * nz;
    const int blocks = (int)((nv + 255) / 256);
    k_voronoi<<<blocks, 256, 3 * VORONOI_TILE * sizeof(double), s>>>(nx, ny, nz, ns, seeds, label);
    return cudaGetLastError();
}

// gstore: n and omega of every frequency of the half spectrum (FP64 form),
// with the arithmetic green_apply uses when it computes them
__global__ void k_fill_green(RveDesc d)
{
    const long long ns = d.nspec, plane = (long long)d.nx * d.ny;
    for (long long o = (long long)blockIdx.x * blockDim.x + threadIdx.x; o < ns;
         o += (long long)gridDim.x * blockDim.x) {
        const int iz = (int)(o / plane), ix = (int)((o % plane) / d.ny), iy = (int)(o % d.ny);
        double n[3] = {0.0, 0.0, 0.0}, w[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        if ((ix | iy | iz) != 0) {
            unit_freq(d, ix, iy, iz, n);
            green_omega<double>(d.Kq, n, w);
        }
        for (int q = 0; q < 3; ++q) d.gstore[q * ns + o] = n[q];
        for (int q = 0; q < 6; ++q) d.gstore[(3 + q) * ns + o] = w[q];
    }
}

cudaError_t launch_fill_green(const RveDesc &d, cudaStream_t s)
{
    if (!d.gstore) return cudaSuccess;
    int blocks = (int)((d.nspec + 255) / 256);
    if (blocks > 152 * 8) blocks = 152 * 8;
    k_fill_green<<<blocks, 256, 0, s>>>(d);
    return cudaGetLastError();
}

// sgp32 + sgp_lo = S_g + S0 once S0 is known (mixed form)
__global__ void k_fill_p32(RveDesc d)
{
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < d.nv;
         v += (long long)gridDim.x * blockDim.x) {
        double P[21];
        load_P(d, v, P);
        const bool solid = d.solid[d.phase[v]] != 0;
        for (int q = 0; q < 21; ++q) put_pair(d.sgp32, d.sgp_lo, (long long)q * d.nv + v, solid ? P[q] : 0.0);
        if (d.sgp)
            for (int q = 0; q < 21; ++q) d.sgp[(long long)q * d.nv + v] = solid ? P[q] : 0.0;
    }
}

cudaError_t launch_fill_p32(const RveDesc &d, cudaStream_t s)
{
    int blocks = (int)((d.nv + 255) / 256);
    if (blocks > 152 * 8) blocks = 152 * 8;
    k_fill_p32<<<blocks, 256, 0, s>>>(d);
    return cudaGetLastError();
}

cudaError_t launch_setup(const RveDesc &d, const SetupConst &sc, const double *euler, int npart,
                         cudaStream_t s)
{
    k_setup<<<npart, 128, 0, s>>>(d, sc, euler);
    return cudaGetLastError();
}


// writes n doubles: evicts the L2 between timed steps
__global__ void k_flush(double *buf, long long n)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        buf[i] = (double)i;
}

cudaError_t launch_flush(double *buf, long long n, cudaStream_t s)
{
    k_flush<<<152 * 8, 256, 0, s>>>(buf, n);
    return cudaGetLastError();
}

// rcp_nr on n doubles (a check of the Newton step's reciprocal against 1/x)
__global__ void k_rcp_probe(const double *__restrict__ x, double *__restrict__ out, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = rcp_nr(x[i]);
}

cudaError_t launch_rcp_probe(const double *x, double *out, int n, cudaStream_t s)
{
    if (n > 0) k_rcp_probe<<<(n + 255) / 256, 256, 0, s>>>(x, out, n);
    return cudaGetLastError();
}

__global__ void k_sqrt_probe(const double *__restrict__ x, double *__restrict__ out, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = sqrt_nr(x[i]);
}

cudaError_t launch_sqrt_probe(const double *x, double *out, int n, cudaStream_t s)
{
    if (n > 0) k_sqrt_probe<<<(n + 255) / 256, 256, 0, s>>>(x, out, n);
    return cudaGetLastError();
}

// One block transforms nl lines of length pl.L with the single-precision
// line FFT of the spectrum passes: in and out are [nl][L] complex doubles,
// rounded to float on the way in.
__global__ void __launch_bounds__(256) k_fft_probe(FftPlan1 pl, const float2 *__restrict__ tw,
                                                   const double2 *__restrict__ in, double2 *__restrict__ out,
                                                   int nl, int sign)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2 *a = reinterpret_cast<float2 *>(smem_raw);
    const int L = pl.L, ldl = nl | 1;
    float2 *b = a + L * ldl;
    for (int e = threadIdx.x; e < nl * L; e += blockDim.x) {
        const int l = e / L, i = e - l * L;
        a[i * ldl + l] = make_float2((float)in[e].x, (float)in[e].y);
    }
    __syncthreads();
    const float2 *res = fft_lines<float>(a, b, nl, ldl, pl, tw, sign);
    for (int e = threadIdx.x; e < nl * L; e += blockDim.x) {
        const int l = e / L, i = e - l * L;
        const float2 v = res[i * ldl + l];
        out[e] = make_double2(v.x, v.y);
    }
}

cudaError_t launch_fft_probe(const FftPlan1 &pl, const void *tw, const double *in, double *out, int nl, int sign,
                             cudaStream_t s)
{
    const size_t smem = (size_t)2 * pl.L * (nl | 1) * sizeof(float2);
    cudaError_t e = cudaFuncSetAttribute((const void *)k_fft_probe, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    k_fft_probe<<<1, 256, smem, s>>>(pl, (const float2 *)tw, (const double2 *)in, (double2 *)out, nl, sign);
    return cudaGetLastError();
}

// FP64 FMA throughput: 8 independent FMA chains per thread
__global__ void k_fp64_fma(double *out, int iters, double a, double b)
{
    double x[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = threadIdx.x * 1e-9 + k;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) x[k] = fma(x[k], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += x[k];
    if (s == 12345.678) out[0] = s;   // keeps the chains live; never true
}

double measure_fp64_tflops()
{
    double *out = nullptr;
    if (cudaMalloc(&out, sizeof(double)) != cudaSuccess) return -1.0;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = sms * 8, threads = 256, iters = 8192;
    k_fp64_fma<<<blocks, threads>>>(out, 64, 0.999999, 1e-7);   // warm-up
    cudaEventRecord(e0);
    k_fp64_fma<<<blocks, threads>>>(out, iters, 0.999999, 1e-7);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    const double flops = 2.0 * 8.0 * (double)iters * blocks * threads;
    return ms > 0.f ? flops / (ms * 1e-3) / 1e12 : -1.0;
}

// ---------------------------------------------------------------------------
// Displacement fluctuation: the periodic field u~ whose gradient is the
// fluctuating part of DisGrad, in voxel units of length.  The reference means
// to compute it at evolution.c:532-560 from
//   u^_i(k) = -i sum_j F^_ij(k) g_j(k),   u~ = Re(IFFT(u^)) / N
// but sums tmp_re/tmp_im into one scalar per component over all voxels, then
// stores it at a stale voxel index, and its g = xi/|xi| (init.c:660-676)
// lacks the 1/|xi| an inverse gradient needs.  Here F is DisGrad (its
// fluctuating part is the reference's `fluctuation`, evolution.c:392, up to
// the uniform terms that only reach k = 0), g_j = xi_j/|xi|^2 with the
// reference's frequencies xi, g(0) = 0, and the real part is taken the way
// the Green operator takes it: the spectrum is replaced by its Hermitian part
// (X(k) + conj X(-k))/2, which turns g into (g(k) - g(-k))/2 and cancels the
// terms along a Nyquist coordinate.  The work array holds [9][nzh][nx][ny]
// complex values of the spectrum type: DisGrad's six B-basis symmetric
// components, then its three antisymmetric ones.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void freq_over_sq(const RveDesc &d, int ix, int iy, int iz, double (&q)[3])
{
    const double g0 = kfreq(ix, d.inv_n[0]), g1 = kfreq(iy, d.inv_n[1]), g2 = kfreq(iz, d.inv_n[2]);
    const double s = 1.0 / (g0 * g0 + g1 * g1 + g2 * g2);
    q[0] = g0 * s; q[1] = g1 * s; q[2] = g2 * s;
}

// which 0: the symmetric part into components 0-5; 1: the antisymmetric
// part into 6-8
template <typename R>
__global__ void __launch_bounds__(256) k_disp_z_fwd(RveDesc d, void *work, int which, int total)
{
    typedef typename Cx<R>::T C;
    C *anti = (C *)work + 6 * d.nspec;
    for (int u = blockIdx.x; u < total; u += gridDim.x) {
        if (which == 0) fft_z_fwd_src<R, 6>(d, d.dgs, work, d.zrows, u);
        else fft_z_fwd_src<R, 3>(d, d.dga, anti, d.zirows3, u);
        __syncthreads();
    }
}

template <typename R>
__global__ void __launch_bounds__(256) k_disp_fft_y(RveDesc d, void *work, int sign, int total)
{
    for (int u = blockIdx.x; u < total; u += gridDim.x) {
        fft_y_unit<R>(d, work, sign, d.yxt, u);
        __syncthreads();
    }
}

template <typename R>
__global__ void __launch_bounds__(256) k_disp_fft_x(RveDesc d, void *work, int ncomp, int sign, int kc, int total)
{
    for (int u = blockIdx.x; u < total; u += gridDim.x) {
        fft_x_unit<R>(d, work, ncomp, sign, kc, u);
        __syncthreads();
    }
}

// per frequency: the nine transformed components -> u^ in components 0-2
template <typename R>
__global__ void __launch_bounds__(256) k_disp_spec(RveDesc d, void *work)
{
    typedef typename Cx<R>::T C;
    C *w = (C *)work;
    const long long ns = d.nspec, plane = (long long)d.nx * d.ny;
    for (long long o = (long long)blockIdx.x * blockDim.x + threadIdx.x; o < ns;
         o += (long long)gridDim.x * blockDim.x) {
        const int iz = (int)(o / plane), ix = (int)((o % plane) / d.ny), iy = (int)(o % d.ny);
        double q[3] = {0.0, 0.0, 0.0};
        if ((ix | iy | iz) != 0) {
            double a[3], b[3];
            freq_over_sq(d, ix, iy, iz, a);
            freq_over_sq(d, (d.nx - ix) % d.nx, (d.ny - iy) % d.ny, (d.nz - iz) % d.nz, b);
            for (int m = 0; m < 3; ++m) q[m] = 0.5 * (a[m] - b[m]);
        }
        double br[6], bi[6], Fr[9], Fi[9];
        for (int c = 0; c < 6; ++c) {
            const C e = w[c * ns + o];
            br[c] = (double)e.x;
            bi[c] = (double)e.y;
        }
        sym9_from_b(br, Fr);
        sym9_from_b(bi, Fi);
        // antisymmetric parts (D12-D21)/2, (D02-D20)/2, (D01-D10)/2
        const int ij[3] = {5, 2, 1}, ji[3] = {7, 6, 3};
        for (int c = 0; c < 3; ++c) {
            const C e = w[(6 + c) * ns + o];
            Fr[ij[c]] += (double)e.x; Fr[ji[c]] -= (double)e.x;
            Fi[ij[c]] += (double)e.y; Fi[ji[c]] -= (double)e.y;
        }
        for (int i = 0; i < 3; ++i) {
            double ur = 0.0, ui = 0.0;   // -i (Fr + i Fi) q = Fi q - i Fr q
            for (int j = 0; j < 3; ++j) {
                ur = fma(Fi[3 * i + j], q[j], ur);
                ui = fma(-Fr[3 * i + j], q[j], ui);
            }
            C e;
            e.x = (R)ur;
            e.y = (R)ui;
            w[i * ns + o] = e;
        }
    }
}

template <typename R>
__global__ void __launch_bounds__(256) k_disp_z_inv(RveDesc d, void *work, double *out, int total)
{
    for (int u = blockIdx.x; u < total; u += gridDim.x) {
        fft_z_inv_unit<R>(d, work, 3, d.zirows3, 2, u, out);
        __syncthreads();
    }
}

template <typename R>
static cudaError_t disp_fluct_t(const RveDesc &d, void *work, double *out, cudaStream_t s)
{
    const int FG = 152 * 4;
    const int budget = (sizeof(R) == 8) ? 2048 : 4096;
    const int kc9 = pick_div<R>(d.ny, (budget * 3 / 2) / (9 * d.nx));
    const int xt = d.nx / d.yxt, nzh = d.nzh;
    const size_t sz = std::max(smem_lines<R>(d.nz, 3 * d.zrows), smem_lines<R>(d.nz, 2 * d.zirows3));
    const size_t sy = smem_lines<R>(d.ny, d.yxt);
    const size_t sx = std::max(smem_lines<R>(d.nx, 9 * kc9), smem_lines<R>(d.nx, 3 * d.xkc3));
    const size_t si = smem_lines<R>(d.nz, 2 * d.zirows3);
    cudaFuncSetAttribute(k_disp_z_fwd<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sz);
    cudaFuncSetAttribute(k_disp_fft_y<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sy);
    cudaFuncSetAttribute(k_disp_fft_x<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sx);
    cudaFuncSetAttribute(k_disp_z_inv<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)si);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const int uz6 = d.nx * (d.ny / d.zrows), uz3 = d.nx * (d.ny / d.zirows3);
    k_disp_z_fwd<R><<<grid_for(uz6, FG), 256, smem_lines<R>(d.nz, 3 * d.zrows), s>>>(d, work, 0, uz6);
    k_disp_z_fwd<R><<<grid_for(uz3, FG), 256, smem_lines<R>(d.nz, 2 * d.zirows3), s>>>(d, work, 1, uz3);
    const int uy9 = 9 * nzh * xt, uy3 = 3 * nzh * xt;
    k_disp_fft_y<R><<<grid_for(uy9, FG), 256, sy, s>>>(d, work, -1, uy9);
    const int ux9 = nzh * (d.ny / kc9), ux3 = nzh * (d.ny / d.xkc3);
    k_disp_fft_x<R><<<grid_for(ux9, FG), 256, smem_lines<R>(d.nx, 9 * kc9), s>>>(d, work, 9, -1, kc9, ux9);
    int blocks = (int)((d.nspec + 255) / 256);
    if (blocks > 152 * 8) blocks = 152 * 8;
    k_disp_spec<R><<<blocks, 256, 0, s>>>(d, work);
    k_disp_fft_x<R><<<grid_for(ux3, FG), 256, smem_lines<R>(d.nx, 3 * d.xkc3), s>>>(d, work, 3, +1, d.xkc3, ux3);
    k_disp_fft_y<R><<<grid_for(uy3, FG), 256, sy, s>>>(d, work, +1, uy3);
    k_disp_z_inv<R><<<grid_for(uz3, FG), 256, si, s>>>(d, work, out, uz3);
    return cudaGetLastError();
}

size_t disp_work_bytes(const RveDesc &d)
{
    return (size_t)9 * (size_t)d.nspec * (d.mixed ? sizeof(float2) : sizeof(double2));
}

cudaError_t launch_disp_fluct(const RveDesc &d, void *work, double *out, cudaStream_t s)
{
    return d.mixed ? disp_fluct_t<float>(d, work, out, s) : disp_fluct_t<double>(d, work, out, s);
}

cudaError_t launch_field_out(const RveDesc &d, int field, double *out, cudaStream_t s)
{
    int blocks = (int)((d.nv + 255) / 256);
    if (blocks > 4096) blocks = 4096;
    k_field_out<<<blocks, 256, 0, s>>>(d, field, out);
    return cudaGetLastError();
}

}  // namespace voce
