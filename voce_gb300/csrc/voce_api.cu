// Host side of libvoce_gpu.so: input readers, material setup, RVE lifecycle
// and the C ABI declared in include/voce_gpu.h.
#include "voce_gpu.h"
#include "voce_gpu_diag.h"
#include "voce_batch.h"
#include "voce_io.h"
#include "voce_kernels.h"
#include "voce_internal.h"
#include "voce_trace.h"

#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <algorithm>
#include <cstring>
#include <cstddef>
#include <cstdint>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

using namespace voce;

namespace {

thread_local std::string g_err;

int fail(int code, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

}  // namespace

// error reporting for the other host translation units (voce_internal.h)
int voce::set_error(int code, const char *msg)
{
    g_err = msg;
    return code;
}

namespace {

#define CUDA_TRY_NEG(x)                                                                    \
    do {                                                                                   \
        cudaError_t e_ = (x);                                                              \
        if (e_ != cudaSuccess) return -fail(VOCE_ERR_CUDA, "%s: %s", #x, cudaGetErrorString(e_)); \
    } while (0)

#define CUDA_TRY(x)                                                                        \
    do {                                                                                   \
        cudaError_t e_ = (x);                                                              \
        if (e_ != cudaSuccess)                                                             \
            return fail(e_ == cudaErrorMemoryAllocation ? VOCE_ERR_NOMEM : VOCE_ERR_CUDA,  \
                        "%s: %s", #x, cudaGetErrorString(e_));                             \
    } while (0)

// ---- Lebensohn-Tome basis (kinematics.c:346-364) on the host ------------
double HB[6][3][3];
std::once_flag hb_once;

// filled once per process; RVEs may be created from several host threads
void hb_fill()
{
    std::memset(HB, 0, sizeof(HB));
    HB[1][0][0] = -1. * RSQ6; HB[1][1][1] = -1. * RSQ6; HB[1][2][2] = 2. * RSQ6;
    HB[0][0][0] = -1. * RSQ2; HB[0][1][1] = RSQ2;
    HB[2][1][2] = RSQ2; HB[2][2][1] = RSQ2;
    HB[3][0][2] = RSQ2; HB[3][2][0] = RSQ2;
    HB[4][0][1] = RSQ2; HB[4][1][0] = RSQ2;
    HB[5][0][0] = RSQ3; HB[5][1][1] = RSQ3; HB[5][2][2] = RSQ3;
}

void hb_init() { std::call_once(hb_once, hb_fill); }

// chg_basis opt 2 (3x3 -> nb-vector) and opt 4 (3x3x3x3 -> 6x6), opt 3
void t_to_v(const double t[3][3], double *v, int nb)
{
    for (int i = 0; i < nb; ++i) {
        double s = 0.0;
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) s += t[a][b] * HB[i][a][b];
        v[i] = s;
    }
}

void t4_to_c66(const double *t4, double *c)
{
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) {
            double s = 0.0;
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b)
                    for (int k = 0; k < 3; ++k)
                        for (int l = 0; l < 3; ++l)
                            s += t4[((a * 3 + b) * 3 + k) * 3 + l] * HB[i][a][b] * HB[j][k][l];
            c[i * 6 + j] = s;
        }
}

void c66_to_t4(const double *c, double *t4)
{
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b)
            for (int k = 0; k < 3; ++k)
                for (int l = 0; l < 3; ++l) {
                    double s = 0.0;
                    for (int i = 0; i < 6; ++i)
                        for (int j = 0; j < 6; ++j) s += c[i * 6 + j] * HB[i][a][b] * HB[j][k][l];
                    t4[((a * 3 + b) * 3 + k) * 3 + l] = s;
                }
}

// LU_inv_66: Crout LU with implicit scaling and the reference's TINY pivot
// rule (kinematics.c:282-424).  Returns false on a near-zero row.
bool lu_inv66(double c[6][6])
{
    const int n = 6;
    double vv[6], y[6][6];
    int indx[6], imax = 0;
    for (int i = 0; i < n; ++i) {
        double big = 0.0, t;
        for (int j = 0; j < n; ++j)
            if ((t = std::fabs(c[i][j])) > big) big = t;
        if (std::fabs(big) < 1E-5) return false;
        vv[i] = 1.0 / big;
    }
    for (int j = 0; j < n; ++j) {
        for (int i = 0; i < j; ++i) {
            double s = c[i][j];
            for (int k = 0; k < i; ++k) s -= c[i][k] * c[k][j];
            c[i][j] = s;
        }
        double big = 0.0, dum;
        for (int i = j; i < n; ++i) {
            double s = c[i][j];
            for (int k = 0; k < j; ++k) s -= c[i][k] * c[k][j];
            c[i][j] = s;
            if ((dum = vv[i] * std::fabs(s)) >= big) { big = dum; imax = i; }
        }
        if (j != imax) {
            for (int k = 0; k < n; ++k) std::swap(c[imax][k], c[j][k]);
            vv[imax] = vv[j];
        }
        indx[j] = imax;
        if (std::fabs(c[j][j]) < 1E-5) c[j][j] = 1.0E-20;
        if (j != n - 1) {
            dum = 1.0 / c[j][j];
            for (int i = j + 1; i < n; ++i) c[i][j] *= dum;
        }
    }
    for (int jc = 0; jc < n; ++jc) {
        double b[6] = {0, 0, 0, 0, 0, 0};
        b[jc] = 1.0;
        int ii = -1;
        for (int i = 0; i < n; ++i) {
            int ip = indx[i];
            double s = b[ip];
            b[ip] = b[i];
            if (ii >= 0)
                for (int q = ii; q < i; ++q) s -= c[i][q] * b[q];
            else if (std::fabs(s) > 1E-5) ii = i;
            b[i] = s;
        }
        for (int i = n - 1; i >= 0; --i) {
            double s = b[i];
            for (int q = i + 1; q < n; ++q) s -= c[i][q] * b[q];
            b[i] = s / c[i][i];
        }
        for (int i = 0; i < n; ++i) y[i][jc] = b[i];
    }
    std::memcpy(c, y, sizeof(y));
    return true;
}

bool fft_plan(int L, FftPlan1 &p)
{
    p.L = L;
    p.nst = 0;
    p.n1 = 0;
    int m = L;
    while (m % 4 == 0 && p.nst < VOCE_MAXRAD) { p.rad[p.nst++] = 4; m /= 4; }
    while (m % 2 == 0 && p.nst < VOCE_MAXRAD) { p.rad[p.nst++] = 2; m /= 2; }
    while (m % 3 == 0 && p.nst < VOCE_MAXRAD) { p.rad[p.nst++] = 3; m /= 3; }
    return m == 1 && L >= 2;
}

// Radix schedules of one axis: the stage orders of its radix-4, -2 and -3
// passes the Stockham kernels can run (any order transforms correctly; the
// order changes the strides of each pass and the rounding of the result, at
// the last bit).  out[0] is fft_plan's 4s-2-3s; then 3s first, the lone 2
// first, and 3s-2-4s, each kept when it differs from those before.  Returns
// how many were written (at most max); 0 when L is not of the form 2^a 3^b.
int fft_schedules(int L, FftPlan1 *out, int max)
{
    FftPlan1 base;
    if (max < 1 || !fft_plan(L, base)) return 0;
    int n4 = 0, n2 = 0, n3 = 0;
    for (int k = 0; k < base.nst; ++k) (base.rad[k] == 4 ? n4 : base.rad[k] == 2 ? n2 : n3)++;
    // orders: 0 = 4,2,3   1 = 3,4,2   2 = 2,4,3   3 = 3,2,4
    static const int order[4][3] = {{4, 2, 3}, {3, 4, 2}, {2, 4, 3}, {3, 2, 4}};
    int n = 0;
    for (int o = 0; o < 4 && n < max; ++o) {
        FftPlan1 p;
        p.L = L;
        p.nst = 0;
        p.n1 = 0;
        for (int q = 0; q < 3; ++q) {
            const int r = order[o][q], cnt = r == 4 ? n4 : r == 2 ? n2 : n3;
            for (int k = 0; k < cnt; ++k) p.rad[p.nst++] = r;
        }
        bool seen = false;
        for (int i = 0; i < n && !seen; ++i)
            seen = out[i].nst == p.nst && std::memcmp(out[i].rad, p.rad, sizeof(int) * p.nst) == 0;
        if (!seen) out[n++] = p;
    }
    return n;
}

// Transform candidates of an axis of an RVE: for the single-precision
// spectrum forms, the register FFT first where the length has one
// (reg_fft_split), then the Stockham schedules; for the FP64 form, the
// Stockham schedules only.  Candidate 0 is the default.
int axis_schedules(int L, bool mixed, FftPlan1 *out, int max)
{
    int n = 0;
    if (mixed && max > 0 && reg_fft_split(L) > 0 && fft_plan(L, out[0])) {
        out[0].n1 = reg_fft_split(L);
        n = 1;
    }
    return n + fft_schedules(L, out + n, max - n);
}

}  // namespace

// ===========================================================================
// the RVE object
// ===========================================================================
struct voce_rve {
    int precision = 0;
    RveDesc d{};
    SetupConst sc{};
    Tiles tiles{};
    int npart = 0;
    cudaStream_t stream = nullptr;
    std::vector<void *> dev_allocs;
    int *h_flag = nullptr;  // pinned
    double *d_out = nullptr;
    void *d_dispwork = nullptr;   // spectrum work array of the displacement fluctuation
    double *d_flush = nullptr;
    long long flush_n = 0;
    Prof prof;
    bool use_graph = true;
    struct voce_batch *batch = nullptr;
    // a lone RVE runs as a plan of one, with the same kernels as a batch
    BatchPlan plan;
    RveDesc *plan_desc = nullptr;
    int2 *plan_maps = nullptr;
    bool plan_dirty = true;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    int n_done = 0, n_steps = 0;
    std::vector<int> grain, phase;  // mesh ids, for the .iout records
    voce_namelist nl{};
    std::vector<voce_increment> incr;
    std::vector<std::vector<double>> itlog;
    ~voce_rve()
    {
        if (stream) cudaStreamSynchronize(stream);
        if (graph_exec) cudaGraphExecDestroy(graph_exec);
        if (graph) cudaGraphDestroy(graph);
        if (plan_desc) cudaFree(plan_desc);
        if (plan_maps) cudaFree(plan_maps);
        for (void *p : dev_allocs) cudaFree(p);
        if (d_out) cudaFree(d_out);
        if (d_dispwork) cudaFree(d_dispwork);
        if (d_flush) cudaFree(d_flush);
        if (h_flag) cudaFreeHost(h_flag);
        for (int k = 0; k < 2 * K_COUNT; ++k)
            if (prof.ev[k]) cudaEventDestroy(prof.ev[k]);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace {

template <typename T>
int dalloc(voce_rve *r, T *&p, size_t count)
{
    void *q = nullptr;
    cudaError_t e = cudaMalloc(&q, count * sizeof(T) + 16);
    if (e != cudaSuccess)
        return fail(VOCE_ERR_NOMEM, "cudaMalloc of %zu bytes failed: %s", count * sizeof(T), cudaGetErrorString(e));
    r->dev_allocs.push_back(q);
    p = (T *)q;
    return VOCE_OK;
}

// exp(-2 pi i j / L) for j < L; where the length has a register-FFT split
// L = N1 N2, followed by the twiddle matrix of its first pass,
// [L + k N2 + t] = exp(-2 pi i t k / L) (t < N2, k < N1): a pass-1 task
// (t) reads its N1 twiddles at fixed offsets from one address, and the
// threads of consecutive t read consecutive entries
template <typename C, typename R>
std::vector<C> twiddles(int L)
{
    const int n1 = reg_fft_split(L);
    std::vector<C> t(n1 ? 2 * L : L);
    const long double two_pi = 6.283185307179586476925286766559005768L;
    auto w = [&](long long e, C &c) {
        const long double a = two_pi * (long double)(e % L) / (long double)L;
        c.x = (R)cosl(a);
        c.y = (R)(-sinl(a));
    };
    for (int j = 0; j < L; ++j) w(j, t[j]);
    if (n1)
        for (int q = 0; q < L / n1; ++q)
            for (int k = 0; k < n1; ++k) w((long long)q * k, t[L + k * (L / n1) + q]);
    return t;
}

}  // namespace

extern "C" {

int voce_abi_version(void) { return VOCE_ABI_VERSION; }
const char *voce_last_error(void) { return g_err.c_str(); }

// ---------------------------------------------------------------------------
// readers
// ---------------------------------------------------------------------------

// GetNameList (io.c:54-122): 80-byte lines, '#' and empty lines skipped, a
// line with no first token ends the read, case-sensitive keys, unknown keys
// ignored (so the shipped input's "Hirth" never sets hirth), a repeated key
// keeps its first values, missing values leave the variable unchanged.
int voce_namelist_read(const char *path, voce_namelist *nl)
{
    if (!path || !nl) return fail(VOCE_ERR_ARG, "null argument");
    std::memset(nl, 0, sizeof(*nl));
    struct Var { const char *name; int type; int len; void *ptr; };
    Var vars[] = {
        {"CellDim", 0, 3, nl->CellDim}, {"N_phases", 0, 1, &nl->N_phases},
        {"Type_phases", 0, 2, nl->Type_phases}, {"TimeStep", 1, 1, &nl->TimeStep},
        {"N_steps", 0, 1, &nl->N_steps}, {"Update_Flag", 0, 1, &nl->Update_Flag},
        {"Hard_Flag", 0, 1, &nl->Hard_Flag}, {"Tex_Flag", 0, 1, &nl->Tex_Flag},
        {"IterMax", 0, 1, &nl->IterMax}, {"PrintControl", 0, 2, nl->PrintControl},
        {"Err", 1, 1, &nl->Err}, {"VelGrad_BC_Flag", 0, 6, nl->VelGrad_BC_Flag},
        {"VelGrad_BC", 1, 6, nl->VelGrad_BC}, {"Stress_BC_Flag", 0, 6, nl->Stress_BC_Flag},
        {"Stress_BC", 1, 6, nl->Stress_BC}, {"ElastConst_PhaseI", 1, 4, nl->ElastConst_PhaseI},
        {"ElastConst_PhaseII", 1, 4, nl->ElastConst_PhaseII}, {"Slip_PhaseI", 2, 1, nl->Slip_PhaseI},
        {"Slip_PhaseII", 2, 1, nl->Slip_PhaseII}, {"initial_ms", 2, 1, nl->initial_ms},
        {"self", 1, 2, nl->self}, {"coplane", 1, 2, nl->coplane}, {"cross", 1, 2, nl->cross},
        {"glissile", 1, 2, nl->glissile}, {"hirth", 1, 2, nl->hirth}, {"lomer", 1, 2, nl->lomer},
    };
    const int nvars = (int)(sizeof(vars) / sizeof(vars[0]));
    bool seen[32] = {false};
    FILE *fp = std::fopen(path, "r");
    if (!fp) return fail(VOCE_ERR_IO, "cannot open namelist '%s'", path);
    char buf[80];
    while (true) {
        if (!std::fgets(buf, 80, fp)) break;
        if (std::feof(fp)) break;
        if (buf[0] == '#' || buf[0] == '\n') continue;
        char *save = nullptr;
        char *tok = strtok_r(buf, " \t\n", &save);
        if (!tok) break;
        for (int k = 0; k < nvars; ++k) {
            if (std::strcmp(tok, vars[k].name) != 0) continue;
            if (!seen[k]) {
                seen[k] = true;
                for (int q = 0; q < vars[k].len; ++q) {
                    tok = strtok_r(nullptr, ", \t\n", &save);
                    if (!tok) continue;
                    if (vars[k].type == 0) ((int *)vars[k].ptr)[q] = (int)std::atol(tok);
                    else if (vars[k].type == 1) ((double *)vars[k].ptr)[q] = std::atof(tok);
                    else std::snprintf((char *)vars[k].ptr, 100, "%s", tok);
                }
            }
            break;
        }
    }
    std::fclose(fp);
    return VOCE_OK;
}

// PlasticInit's reader (init.c:65-186): fixed line positions, one mode used
int voce_slip_read(const char *path, voce_slip *out)
{
    if (!path || !out) return fail(VOCE_ERR_ARG, "null argument");
    std::memset(out, 0, sizeof(*out));
    FILE *fp = std::fopen(path, "r");
    if (!fp) return fail(VOCE_ERR_IO, "cannot open .sx '%s'", path);
    char buf[80] = {0};
    auto L = [&]() { if (!std::fgets(buf, 80, fp)) buf[0] = 0; };
    int nmax = 0, nmodes = 0, imode[16] = {0};
    L(); L(); L(); L(); L(); L(); L(); L(); std::sscanf(buf, "%d", &nmax);
    L(); L(); L(); std::sscanf(buf, "%d", &nmodes);
    if (nmodes < 1 || nmodes > 16) { std::fclose(fp); return fail(VOCE_ERR_PARSE, "%s: bad N_modes", path); }
    L(); L();
    for (int i = 0; i < nmodes; ++i) { L(); std::sscanf(buf, "%d", &imode[i]); }
    L();
    int found = 0, mx = 0;
    for (int i = 0; i < nmax; ++i) {
        L();
        std::sscanf(buf, "%*s %*s %d %*s", &mx);
        bool match = false;
        for (int q = 0; q < nmodes; ++q) if (mx == imode[q]) match = true;
        if (!match) { for (int q = 0; q < 24; ++q) L(); continue; }
        ++found;
        double twsh, hs, hl;
        int isect;
        L(); L(); std::sscanf(buf, "%d %lf %lf %lf %d", &out->nsys, &out->nrs, &out->gamd0, &twsh, &isect);
        if (out->nsys < 1 || out->nsys > VOCE_NS) { std::fclose(fp); return fail(VOCE_ERR_UNSUPPORTED, "nsmx %d", out->nsys); }
        L(); L(); std::sscanf(buf, "%lf %lf %lf %lf %lf", &out->tau0f, &out->tau0b, &out->tau1, &out->thet0, &out->thet1);
        L(); L(); std::sscanf(buf, "%lf %lf", &hs, &hl);
        L();
        for (int s = 0; s < out->nsys; ++s) {
            L();
            std::sscanf(buf, "%lf %lf %lf %lf %lf %lf", &out->bn[s][0], &out->bn[s][1], &out->bn[s][2],
                        &out->bb[s][0], &out->bb[s][1], &out->bb[s][2]);
        }
    }
    std::fclose(fp);
    if (!found) return fail(VOCE_ERR_PARSE, "%s: selected mode not found", path);
    return VOCE_OK;
}

// InitMicroStruct's reader (init.c:410-433): one line per voxel
// "phi1 Phi phi2 i j k grain phase", x slowest / z fastest, 1-based.
// voce_mesh_read: voce_parse.cpp

}  // extern "C"

namespace {

int autotune_tiles(voce_rve *r);
void apply_tiles(voce_rve *r, const Tiles &t);
Tiles tiles_of(const RveDesc &d);
FftPlan1 schedule_of(int L, bool mixed, int k);
extern int g_autotune;
extern int g_newton_chord;
extern int g_ir_predictor;

// Device arrays of one RVE, state and scratch, sized from its descriptor;
// the twiddle tables are filled, the rest is left to the caller.
int alloc_device(voce_rve *r)
{
    RveDesc &d = r->d;
    const long long nv = d.nv;
    int rc = VOCE_OK;
#define AL(ptr, n) if ((rc = dalloc(r, ptr, (size_t)(n))) != VOCE_OK) return rc;
    AL(d.sig, 6 * nv); AL(d.sigp, 6 * nv); AL(d.eps, 5 * nv); AL(d.dgs, 6 * nv); AL(d.dga, 3 * nv);
    AL(d.tm, 9 * nv); AL(d.sch, 60 * nv); AL(d.sg, 21 * nv); AL(d.crss, 24 * nv); AL(d.itau, 24 * nv);
    AL(d.gamacum, nv); AL(d.gtot, 12 * nv); AL(d.edot, 5 * nv); AL(d.gamdot, 12 * nv); AL(d.taux, 12 * nv);
    AL(d.svm, nv); AL(d.evm, nv); AL(d.rotl, 3 * nv); AL(d.diag, 3 * nv); AL(d.phase, nv);
    d.sch32 = nullptr;
    d.itau32 = nullptr;
    d.sgp32 = nullptr;
    d.sch_lo = d.itau_lo = d.sgp_lo = nullptr;
    d.sgp = nullptr;
    if (d.ir) AL(d.sgp, 21 * nv);
    if (d.nr32 || d.ir) {
        AL(d.sch32, 60 * nv); AL(d.itau32, 24 * nv); AL(d.sgp32, 21 * nv);
        AL(d.sch_lo, 60 * nv); AL(d.itau_lo, 24 * nv); AL(d.sgp_lo, 21 * nv);
    }
    AL(d.part, (size_t)3 * r->npart * VOCE_NPART);
    AL(d.macro, 1);
    d.incr_cap = 32;   // increments per host read-back
    AL(d.itlog, (size_t)d.incr_cap * VOCE_ITLOG * (d.iter_max > 0 ? d.iter_max : 1));
    AL(d.incr, d.incr_cap);
    const size_t csz = d.mixed ? sizeof(float2) : sizeof(double2);
    char *p;
    d.gstore = nullptr;
    if (!d.mixed) AL(d.gstore, 9 * d.nspec);
    AL(p, 6 * d.nspec * csz); d.spec = p;
    AL(p, 3 * d.nspec * csz); d.aacc = p;
    const int Ls[3] = {d.nx, d.ny, d.nz};
    const void **tws[3] = {&d.twx, &d.twy, &d.twz};
    for (int a = 0; a < 3; ++a) {
        if (d.mixed) {
            auto t = twiddles<float2, float>(Ls[a]);
            AL(p, t.size() * sizeof(float2));
            CUDA_TRY(cudaMemcpy(p, t.data(), t.size() * sizeof(float2), cudaMemcpyHostToDevice));
        } else {
            auto t = twiddles<double2, double>(Ls[a]);
            AL(p, t.size() * sizeof(double2));
            CUDA_TRY(cudaMemcpy(p, t.data(), t.size() * sizeof(double2), cudaMemcpyHostToDevice));
        }
        *tws[a] = p;
    }
#undef AL
    CUDA_TRY(cudaMallocHost(&r->h_flag, 64));
    return VOCE_OK;
}

// The device arrays that carry an RVE's state from one call to the next, in
// snapshot order, with their sizes in bytes: f(&pointer, bytes).
template <class F>
void for_state(RveDesc &d, F &&f)
{
    const size_t nv = (size_t)d.nv, D = sizeof(double), S = sizeof(float);
    f((void **)&d.sig, 6 * nv * D);      f((void **)&d.sigp, 6 * nv * D);
    f((void **)&d.eps, 5 * nv * D);      f((void **)&d.dgs, 6 * nv * D);
    f((void **)&d.dga, 3 * nv * D);      f((void **)&d.tm, 9 * nv * D);
    f((void **)&d.sch, 60 * nv * D);     f((void **)&d.sg, 21 * nv * D);
    f((void **)&d.crss, 24 * nv * D);    f((void **)&d.itau, 24 * nv * D);
    f((void **)&d.gamacum, nv * D);      f((void **)&d.gtot, 12 * nv * D);
    f((void **)&d.edot, 5 * nv * D);     f((void **)&d.gamdot, 12 * nv * D);
    f((void **)&d.taux, 12 * nv * D);    f((void **)&d.svm, nv * D);
    f((void **)&d.evm, nv * D);          f((void **)&d.rotl, 3 * nv * D);
    f((void **)&d.diag, 3 * nv * D);     f((void **)&d.phase, nv * sizeof(int));
    if (d.ir) f((void **)&d.sgp, 21 * nv * D);
    if (d.nr32 || d.ir) {
        f((void **)&d.sch32, 60 * nv * S);
        f((void **)&d.itau32, 24 * nv * S);
        f((void **)&d.sgp32, 21 * nv * S);
        f((void **)&d.sch_lo, 60 * nv * S);
        f((void **)&d.itau_lo, 24 * nv * S);
        f((void **)&d.sgp_lo, 21 * nv * S);
    }
    // the antisymmetric Green update summed over the current increment's
    // iterations, and the macro state
    f((void **)&d.aacc, 3 * (size_t)d.nspec * (d.mixed ? sizeof(float2) : sizeof(double2)));
    f((void **)&d.macro, sizeof(MacroDev));
}

}  // namespace

extern "C" {

long long voce_rve_footprint(const int dims[3], int precision)
{
    const long long nv = (long long)dims[0] * dims[1] * dims[2];
    const long long nspec = (long long)(dims[2] / 2 + 1) * dims[0] * dims[1];
    const long long cplx = precision == VOCE_PREC_FP64 ? 16 : 8;
    // doubles per voxel: sig 6, sigp 6, eps 5, dgs 6, dga 3, tm 9, sch 60,
    // sg 21, crss 24, itau 24, gamacum 1, gtot 12, edot 5, gamdot 12, taux 12,
    // svm 1, evm 1, rotl 3, diag 3  (= 214) + phase (4 bytes)
    // + the FP64 form's stored Green-operator frequencies, 9 doubles each
    // + the mixed_nr32 and mixed_ir forms' float pairs of sch, itau and
    // S_g + S0 (2 x 105 floats), and the mixed_ir form's S_g + S0 in FP64 (21
    // doubles)
    const long long f32 = precision == VOCE_PREC_MIXED_NR32 ? 840 : precision == VOCE_PREC_MIXED_IR ? 840 + 168 : 0;
    return nv * (214 * 8 + 4 + f32) + nspec * 9 * cplx +
           (precision == VOCE_PREC_FP64 ? nspec * 9 * 8 : 0);
}

// ---------------------------------------------------------------------------
// SetupJob (init.c:617-828)
// ---------------------------------------------------------------------------
int voce_rve_create(const voce_namelist *nl, const voce_slip *slip[2], const voce_mesh *mesh,
                    int precision, voce_rve **out)
{
    VOCE_TRACE("voce_rve_create");
    if (!nl || !mesh || !out || !mesh->euler_deg || !mesh->phase) return fail(VOCE_ERR_ARG, "null argument");
    *out = nullptr;
    hb_init();
    const int nx = nl->CellDim[0], ny = nl->CellDim[1], nz = nl->CellDim[2];
    if (mesh->dims[0] != nx || mesh->dims[1] != ny || mesh->dims[2] != nz)
        return fail(VOCE_ERR_ARG, "mesh dims differ from CellDim");
    FftPlan1 plx, ply, plz;
    if (!fft_plan(nx, plx) || !fft_plan(ny, ply) || !fft_plan(nz, plz) || nz % 2)
        return fail(VOCE_ERR_UNSUPPORTED, "grid %dx%dx%d: each edge must be 2^a 3^b >= 2 and nz even", nx, ny, nz);
    if (nl->N_phases < 1 || nl->N_phases > 2) return fail(VOCE_ERR_UNSUPPORTED, "N_phases %d", nl->N_phases);
    int solid_phase = -1;
    for (int p = 0; p < nl->N_phases; ++p)
        if (!nl->Type_phases[p]) {
            if (solid_phase >= 0) return fail(VOCE_ERR_UNSUPPORTED, "more than one crystalline phase");
            solid_phase = p;
        }
    if (solid_phase < 0 || !slip || !slip[solid_phase]) return fail(VOCE_ERR_ARG, "no slip data for the crystal phase");
    const voce_slip &sx = *slip[solid_phase];
    if (sx.nsys < 1 || sx.nsys > VOCE_NS) return fail(VOCE_ERR_UNSUPPORTED, "nsys %d", sx.nsys);
    // boundary conditions (init.c:713-745)
    if (nl->VelGrad_BC_Flag[0] + nl->VelGrad_BC_Flag[1] + nl->VelGrad_BC_Flag[2] == 2)
        return fail(VOCE_ERR_BC, "Cannot enforce only two deviatoric components (VelGrad_BC_Flag)");
    for (int i = 0; i < 6; ++i)
        if ((nl->Stress_BC_Flag[i] * nl->VelGrad_BC_Flag[i] != 0) ||
            ((nl->Stress_BC_Flag[i] + nl->VelGrad_BC_Flag[i]) != 1))
            return fail(VOCE_ERR_BC, "Check boundary conditions on strain rate and stress");
    const long long nv = (long long)nx * ny * nz;
    for (long long v = 0; v < nv; ++v)
        if (mesh->phase[v] < 1 || mesh->phase[v] > nl->N_phases)
            return fail(VOCE_ERR_PARSE, "phase id %d at voxel %lld", mesh->phase[v], v);
    // a non-finite Euler angle would turn the whole field into NaN (the
    // reference propagates it silently); refused before anything reaches
    // the GPU
    for (long long i = 0; i < 3 * nv; ++i)
        if (!std::isfinite(mesh->euler_deg[i]))
            return fail(VOCE_ERR_ARG, "non-finite Euler angle at voxel %lld", i / 3);

    if (precision < VOCE_PREC_FP64 || precision > VOCE_PREC_MIXED_IR)
        return fail(VOCE_ERR_ARG, "unknown precision %d", precision);
    // owned until handed out: every early return (a failed CUDA call
    // included) frees what was made so far
    std::unique_ptr<voce_rve> own(new voce_rve());
    voce_rve *r = own.get();
    r->precision = precision;
    RveDesc &d = r->d;
    SetupConst &sc = r->sc;
    d.nx = nx; d.ny = ny; d.nz = nz; d.nzh = nz / 2 + 1;
    d.nv = nv;
    d.nspec = (long long)d.nzh * nx * ny;
    const int dims3[3] = {nx, ny, nz};
    for (int a = 0; a < 3; ++a) {
        d.inv_n[a] = 1.0 / dims3[a];
        d.inv_nf[a] = (float)(1.0 / dims3[a]);
    }
    d.plx = plx; d.ply = ply; d.plz = plz;
    d.mixed = r->precision != VOCE_PREC_FP64;
    // chord steps only where the spectrum is single precision already: the
    // FP64 form keeps the reference's Newton path, because the strain rate
    // and the error norms are evaluated at the stress before the last Newton
    // update (evolution.c:67,118-126), which moves with the step count
    d.chord = r->precision == VOCE_PREC_MIXED ? g_newton_chord : 0;
    d.nr32 = r->precision == VOCE_PREC_MIXED_NR32;
    d.ir = r->precision == VOCE_PREC_MIXED_IR;
    d.ir_pred = d.ir ? g_ir_predictor : 0;
    for (int p = 0; p < 2; ++p) d.solid[p + 1] = (p < nl->N_phases && !nl->Type_phases[p]) ? 1 : 0;
    d.nsys = sx.nsys;
    d.update_flag = nl->Update_Flag;
    d.hard_flag = nl->Hard_Flag;
    d.iter_max = nl->IterMax;
    d.err_tol = nl->Err;
    d.dt = nl->TimeStep;
    d.dth = (float)d.dt;
    d.dtl = (float)(d.dt - (double)d.dth);
    const int Nxyz = nx * ny * nz;
    d.wgt = 1. / Nxyz;
    d.inv_nv = 1.0 / (double)Nxyz;
    r->n_steps = nl->N_steps;

    // material (ElastStiffnessMatrix init.c:9-49, PlasticInit init.c:51-391)
    const double *ec = solid_phase == 0 ? nl->ElastConst_PhaseI : nl->ElastConst_PhaseII;
    double C4[81] = {0};
    for (int i = 0; i < 3; ++i) C4[((i * 3 + i) * 3 + i) * 3 + i] = ec[0];
    for (int i = 0; i < 3; ++i)
        for (int k = 0; k < 3; ++k)
            if (i != k) {
                C4[((i * 3 + i) * 3 + k) * 3 + k] = ec[1];
                C4[((i * 3 + k) * 3 + i) * 3 + k] = ec[2];
                C4[((i * 3 + k) * 3 + k) * 3 + i] = ec[2];
            }
    t4_to_c66(C4, sc.cxt);
    {
        double s[6][6];
        std::memcpy(s, sc.cxt, sizeof(s));
        if (!lu_inv66(s)) return fail(VOCE_ERR_SINGULAR, "singular crystal stiffness");
        std::memcpy(sc.sxt, s, sizeof(s));
    }
    double tau1 = sx.tau1, thet0 = sx.thet0;
    if (tau1 < 1.E-6) { tau1 = 1.E-6; thet0 = sx.thet1; }  // init.c:141-144
    double nr = sx.nrs;
    d.ipow_n = (nr >= 1.0 && nr <= 256.0 && std::floor(nr) == nr) ? (int)nr : -1;
    for (int s = 0; s < sx.nsys; ++s) {
        d.gam0[s] = sx.gamd0;
        d.nrs[s] = nr;
        d.g0n[s] = sx.gamd0 * nr;
        d.gam0f[s] = (float)sx.gamd0;
        d.nrsf[s] = (float)nr;
        d.gam0l[s] = (float)(sx.gamd0 - (double)d.gam0f[s]);
        d.gam0_uniform = 1;   // one slip mode per phase: one gam0
        d.tau0[s] = sx.tau0f;
        d.tau0b[s] = sx.tau0b;
        d.tau1[s] = tau1;
        d.thet0[s] = thet0;
        d.thet1[s] = sx.thet1;
        double n[3], b[3];
        double nn = std::sqrt(std::pow(sx.bn[s][0], 2.0) + std::pow(sx.bn[s][1], 2.0) + std::pow(sx.bn[s][2], 2.0));
        double nb = std::sqrt(std::pow(sx.bb[s][0], 2.0) + std::pow(sx.bb[s][1], 2.0) + std::pow(sx.bb[s][2], 2.0));
        for (int q = 0; q < 3; ++q) { n[q] = sx.bn[s][q] / nn; b[q] = sx.bb[s][q] / nb; }
        double dot = n[0] * b[0] + n[1] * b[1] + n[2] * b[2];
        if (dot > 1E-3) return fail(VOCE_ERR_PARSE, "slip system %d is not orthogonal", s + 1);
        double a[3][3];
        for (int p = 0; p < 3; ++p)
            for (int q = 0; q < 3; ++q) a[p][q] = (n[p] * b[q] + n[q] * b[p]) / 2.0;
        t_to_v(a, d.schxt + 5 * s, 5);
        for (int q = 0; q < 3; ++q) { d.bn[3 * s + q] = n[q]; d.bb[3 * s + q] = b[q]; }
    }
    {
        // latent hardening pattern of the 12 {111}<110> systems (init.c:283-381)
        static const char tbl[12][13] = {
            "SCCHGLXGGHLG", " SCGXGGHLLHG", "  SLGHGLHGGX", "   SCCHLGXGG",
            "    SCLHGGHL", "     SGGXGLH", "      SCCHGL", "       SCGXG",
            "        SLGH", "         SCC", "          SC", "           S"};
        const int ph = solid_phase;
        for (int p = 0; p < 12; ++p)
            for (int q = p; q < 12; ++q) {
                double v = 0.0;
                switch (tbl[p][q]) {
                case 'S': v = nl->self[ph]; break;
                case 'C': v = nl->coplane[ph]; break;
                case 'X': v = nl->cross[ph]; break;
                case 'G': v = nl->glissile[ph]; break;
                case 'H': v = nl->hirth[ph]; break;
                case 'L': v = nl->lomer[ph]; break;
                }
                d.hard[p * VOCE_NS + q] = v;
                d.hard[q * VOCE_NS + p] = v;
            }
    }
    // boundary conditions: Udot, Scauchy, creep (init.c:716-745)
    const double *vb = nl->VelGrad_BC, *sb = nl->Stress_BC;
    const double U[9] = {vb[0], vb[5], vb[4], vb[5], vb[1], vb[3], vb[4], vb[3], vb[2]};
    const double S[9] = {sb[0], sb[5], sb[4], sb[5], sb[1], sb[3], sb[4], sb[3], sb[2]};
    std::memcpy(d.Udot, U, sizeof(U));
    std::memcpy(d.Scauchy, S, sizeof(S));
    int creep = 0;
    for (int i = 0; i < 6; ++i) creep += nl->Stress_BC_Flag[i];
    d.creep = creep / 6;
    for (int i = 0; i < 6; ++i) { d.vflag[i] = nl->VelGrad_BC_Flag[i]; d.sflag[i] = nl->Stress_BC_Flag[i]; }
    {
        double us[6] = {U[0], U[4], U[8], 0.5 * (U[5] + U[7]), 0.5 * (U[2] + U[6]), 0.5 * (U[1] + U[3])};
        t6_to_b<double>(us, d.u6);
        d.ua[0] = 0.5 * (U[5] - U[7]);
        d.ua[1] = 0.5 * (U[2] - U[6]);
        d.ua[2] = 0.5 * (U[1] - U[3]);
        double ud[6];
        for (int q = 0; q < 6; ++q) ud[q] = us[q] * d.dt;
        t6_to_b<double>(ud, sc.d6);
        double s6[6] = {S[0], S[4], S[8], S[5], S[2], S[1]};
        t6_to_b<double>(s6, sc.sc6);
    }

    // the default tiles must fit in a block's shared memory; they keep to a
    // budget well inside it and fall back to one line per tile when a line
    // is longer, so this refuses a grid exactly when one line does not fit
    // (in FP64, an x edge above 1024 points)
    {
        Tiles t;
        if (d.mixed) t.choose<float>(d);
        else t.choose<double>(d);
        RveDesc dt = d;
        dt.zrows = t.zrows; dt.yxt = t.yxt; dt.xkc = t.xkc;
        dt.xkc3 = t.xkc3; dt.zirows = t.zirows; dt.zirows3 = t.zirows3;
        dt.plx = schedule_of(nx, d.mixed != 0, 0);
        dt.ply = schedule_of(ny, d.mixed != 0, 0);
        dt.plz = schedule_of(nz, d.mixed != 0, 0);
        for (int ph = BP_ZF; ph < BP_COUNT; ++ph)
            if (batch_smem(dt, ph) > 227 * 1024)
                return fail(VOCE_ERR_UNSUPPORTED,
                            "grid %dx%dx%d: a line is too long for the FFT passes' shared memory in this precision",
                            nx, ny, nz);
    }

    // device memory
    CUDA_TRY(cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking));
    // Newton / increment-end work split into 128-thread units: at most one
    // per Newton block the GPU holds at once (at least two per SM).  The
    // per-RVE partial sums follow this split, so it is fixed per grid size
    // and precision.
    const long long sm_count = 152;
    long long nb = (nv + 127) / 128;
    const long long cap = std::max<long long>(sm_count * 2, nr_resident_blocks(nr_kind(r->precision)));
    r->npart = (int)(nb < cap ? nb : cap);
    d.npart = r->npart;
    int rc = alloc_device(r);
    if (rc) return rc;
    double *d_eul = nullptr;
    if ((rc = dalloc(r, d_eul, (size_t)(3 * nv))) != VOCE_OK) return rc;
    CUDA_TRY(cudaMemcpyAsync(d_eul, mesh->euler_deg, sizeof(double) * 3 * nv, cudaMemcpyHostToDevice, r->stream));
    CUDA_TRY(cudaMemcpyAsync(d.phase, mesh->phase, sizeof(int) * nv, cudaMemcpyHostToDevice, r->stream));
    r->nl = *nl;
    r->phase.assign(mesh->phase, mesh->phase + nv);
    if (mesh->grain) r->grain.assign(mesh->grain, mesh->grain + nv);
    else r->grain.assign(nv, 1);
    long long nph1 = 0;
    for (long long v = 0; v < nv; ++v) nph1 += mesh->phase[v] == 1;
    d.wgt_ph1 = (1.0 * (double)nph1) / Nxyz;
    d.wgt_ratio = d.wgt / d.wgt_ph1;
    d.all_ph1 = nph1 == nv ? 1 : 0;

    CUDA_TRY(launch_setup(d, sc, d_eul, r->npart, r->stream));
    std::vector<double> part((size_t)3 * r->npart * VOCE_NPART);
    CUDA_TRY(cudaMemcpyAsync(part.data(), d.part, sizeof(double) * part.size(), cudaMemcpyDeviceToHost, r->stream));
    CUDA_TRY(cudaStreamSynchronize(r->stream));
    // the Euler angles live on as the orientation matrices: their staging
    // array (24 bytes a voxel) goes now, so the RVE holds what
    // voce_rve_footprint counts
    r->dev_allocs.erase(std::find(r->dev_allocs.begin(), r->dev_allocs.end(), (void *)d_eul));
    CUDA_TRY(cudaFree(d_eul));
    d_eul = nullptr;
    // C066 = WGT * sum over voxels of C_gr (init.c:450-456), block partials
    // summed in block order
    double sums[48] = {0};
    for (int pass = 0; pass < 3; ++pass)
        for (int b = 0; b < r->npart; ++b)
            for (int q = 0; q < VOCE_NPART - 1; ++q)
                sums[pass * (VOCE_NPART - 1) + q] += part[((size_t)pass * r->npart + b) * VOCE_NPART + q];
    double C066[6][6], S066[6][6];
    for (int q = 0; q < 36; ++q) C066[q / 6][q % 6] = sums[1 + q] * d.wgt;
    std::memcpy(S066, C066, sizeof(S066));
    if (!lu_inv66(S066)) return fail(VOCE_ERR_SINGULAR, "singular reference stiffness C066");
    std::memcpy(d.S0, S066, sizeof(S066));
    for (int q = 0; q < 36; ++q) d.S0f[q] = (float)d.S0[q];
    if (d.nr32 || d.ir) CUDA_TRY(launch_fill_p32(d, r->stream));
    double C0t[81];
    c66_to_t4(&C066[0][0], C0t);
    c66_to_t4(&S066[0][0], d.S0t);
    // acoustic-tensor coefficients: K_ik = sum_jl C0_ijkl n_j n_l
    {
        const int P[6][2] = {{0, 0}, {1, 1}, {2, 2}, {1, 2}, {0, 2}, {0, 1}};
        for (int a = 0; a < 6; ++a)
            for (int m = 0; m < 6; ++m) {
                const int i = P[a][0], k = P[a][1], j = P[m][0], l = P[m][1];
                double v = C0t[((i * 3 + j) * 3 + k) * 3 + l];
                if (j != l) v += C0t[((i * 3 + l) * 3 + k) * 3 + j];
                d.Kq[a * 6 + m] = v;
                d.Kqf[a * 6 + m] = (float)v;
            }
    }
    CUDA_TRY(launch_fill_green(d, r->stream));
    // macro state (InitFields init.c:494-499, 536; Evolution locals)
    MacroDev m;
    std::memset(&m, 0, sizeof(m));
    for (int q = 0; q < 9; ++q) m.DisGradAvg[q] = U[q] * d.dt;
    {
        double dev[3][3], dvm = 0.0, us6[6];
        double Us[3][3] = {{U[0], U[1], U[2]}, {U[3], U[4], U[5]}, {U[6], U[7], U[8]}};
        t_to_v(Us, us6, 6);
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                double s = 0.0;
                for (int i = 0; i < 5; ++i) s += us6[i] * HB[i][a][b];
                dev[a][b] = s;
            }
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) dvm += std::pow(dev[a][b], 2.0);
        m.d_vm = std::sqrt(2. / 3. * dvm);
        m.e_vm = m.d_vm * d.dt;
    }
    m.istep = 1;
    m.first_iter = 1;
    m.active = 1;
    m.target = 0x7fffffff;
    m.pending_prelude = 1;
    m.Err_e = 2. * d.err_tol;
    m.Err_s = 2. * d.err_tol;
    CUDA_TRY(cudaMemcpyAsync(d.macro, &m, sizeof(m), cudaMemcpyHostToDevice, r->stream));
    if (d.mixed) r->tiles.choose<float>(d);
    else r->tiles.choose<double>(d);
    apply_tiles(r, r->tiles);   // tiles and the default transform of every axis
    CUDA_TRY(cudaStreamSynchronize(r->stream));
    if (g_autotune) {
        rc = autotune_tiles(r);
        if (rc) return rc;
    }
    *out = own.release();
    return VOCE_OK;
}

int voce_rve_create_from_files(const char *namelist_path, int precision, voce_rve **out)
{
    if (!namelist_path || !out) return fail(VOCE_ERR_ARG, "null argument");
    voce_namelist nl;
    int rc = voce_namelist_read(namelist_path, &nl);
    if (rc) return rc;
    std::string dir;
    const char *sl = std::strrchr(namelist_path, '/');
    if (sl) dir.assign(namelist_path, sl - namelist_path + 1);
    auto rel = [&](const char *f) { return (f[0] == '/') ? std::string(f) : dir + f; };
    voce_slip sx[2];
    const voce_slip *sp[2] = {nullptr, nullptr};
    for (int p = 0; p < nl.N_phases && p < 2; ++p) {
        if (nl.Type_phases[p]) continue;
        rc = voce_slip_read(rel(p == 0 ? nl.Slip_PhaseI : nl.Slip_PhaseII).c_str(), &sx[p]);
        if (rc) return rc;
        sp[p] = &sx[p];
    }
    const long long nv = (long long)nl.CellDim[0] * nl.CellDim[1] * nl.CellDim[2];
    if (nv <= 0) return fail(VOCE_ERR_PARSE, "CellDim missing");
    std::vector<double> eul(3 * nv);
    std::vector<int> grain(nv), phase(nv);
    rc = voce_mesh_read(rel(nl.initial_ms).c_str(), nl.CellDim, eul.data(), grain.data(), phase.data());
    if (rc) return rc;
    voce_mesh mesh;
    std::memcpy(mesh.dims, nl.CellDim, sizeof(mesh.dims));
    mesh.euler_deg = eul.data();
    mesh.grain = grain.data();
    mesh.phase = phase.data();
    return voce_rve_create(&nl, sp, &mesh, precision, out);
}

// ---------------------------------------------------------------------------
// Evolution (evolution.c:265-622), n increments at a time
// ---------------------------------------------------------------------------
}  // extern "C"

namespace {

// Record of one finished increment, copied from the device rings.
void collect_increment(voce_rve *r, const IncrDev &rec, const double *log_rows)
{
    voce_increment o;
    std::memset(&o, 0, sizeof(o));
    o.istep = rec.istep; o.iters = rec.iters; o.iter_total = rec.iter_total; o.nr_max = rec.nr_max;
    o.e_vm = rec.e_vm; o.evmp = rec.evmp; o.d_vm = rec.d_vm; o.dvmp = rec.dvmp;
    o.s_vm = rec.s_vm; o.s_vm1 = rec.s_vm1;
    std::memcpy(o.sig_avg, rec.sig_avg, sizeof(o.sig_avg));
    std::memcpy(o.sig_avg1, rec.sig_avg1, sizeof(o.sig_avg1));
    std::memcpy(o.eps_avg, rec.eps_avg, sizeof(o.eps_avg));
    std::memcpy(o.edot_avg, rec.edot_avg, sizeof(o.edot_avg));
    std::memcpy(o.disgrad_avg, rec.disgrad_avg, sizeof(o.disgrad_avg));
    o.err_e = rec.err_e; o.err_s = rec.err_s;
    o.rot_slip_avg = rec.rsl; o.rot_loc_avg = rec.rlc;
    o.nr_iters_total = rec.nr_total;
    r->incr.push_back(o);
    r->itlog.emplace_back(log_rows, log_rows + (size_t)VOCE_ITLOG * rec.iters);
    r->n_done++;
}

// Work lists and descriptor array of a set of RVEs (device memory).
int make_plan(const std::vector<RveDesc> &descs, int precision, RveDesc *&d_descs, int2 *&d_maps,
              BatchPlan &p)
{
    if (d_descs) cudaFree(d_descs);
    if (d_maps) cudaFree(d_maps);
    d_descs = nullptr;
    d_maps = nullptr;
    int *ticks = p.ticks, *maxt = p.max_ticks, *act = p.active_out;
    p = BatchPlan();
    p.ticks = ticks; p.max_ticks = maxt; p.active_out = act;
    p.mixed = precision != VOCE_PREC_FP64;
    p.nr32 = precision == VOCE_PREC_MIXED_NR32;
    p.ir = precision == VOCE_PREC_MIXED_IR;
    p.nrve = (int)descs.size();
    if (descs.empty()) return VOCE_OK;
    std::vector<std::vector<int2>> maps(BP_COUNT);
    for (int i = 0; i < p.nrve; ++i) {
        int u[BP_COUNT];
        batch_units(descs[i], u);
        for (int ph = 0; ph < BP_COUNT; ++ph) {
            for (int k = 0; k < u[ph]; ++k) maps[ph].push_back(make_int2(i, k));
            p.smem[ph] = std::max(p.smem[ph], batch_smem(descs[i], ph));
        }
    }
    if (p.mixed) {   // the streamed y pass: all RVEs on the register FFT along y
        long long S = 0;
        bool all = true;
        for (const RveDesc &d : descs) {
            if (d.ply.n1 <= 0) all = false;
            else S = std::max(S, (long long)d.yxt * (d.ny + d.ply.n1 + 1));
        }
        if (all) {
            p.ystream = (int)((S + 1) & ~1LL);
            const size_t sm = 2 * (size_t)p.ystream * sizeof(float2);
            p.smem[BP_Y6] = std::max(p.smem[BP_Y6], sm);
            p.smem[BP_Y3] = std::max(p.smem[BP_Y3], sm);
        }
    }
    size_t tot = 0;
    for (int ph = 0; ph < BP_COUNT; ++ph) tot += maps[ph].size();
    CUDA_TRY(cudaMalloc(&d_descs, sizeof(RveDesc) * descs.size()));
    CUDA_TRY(cudaMalloc(&d_maps, sizeof(int2) * tot));
    CUDA_TRY(cudaMemcpy(d_descs, descs.data(), sizeof(RveDesc) * descs.size(), cudaMemcpyHostToDevice));
    size_t off = 0;
    for (int ph = 0; ph < BP_COUNT; ++ph) {
        CUDA_TRY(cudaMemcpy(d_maps + off, maps[ph].data(), sizeof(int2) * maps[ph].size(), cudaMemcpyHostToDevice));
        p.map[ph] = d_maps + off;
        p.total[ph] = (int)maps[ph].size();
        off += maps[ph].size();
    }
    p.descs = d_descs;
    CUDA_TRY(set_batch_smem(p));
    return VOCE_OK;
}

int ensure_self_plan(voce_rve *r)
{
    if (!r->plan_dirty) return VOCE_OK;
    std::vector<RveDesc> one(1, r->d);
    int rc = make_plan(one, r->precision, r->plan_desc, r->plan_maps, r->plan);
    if (rc) return rc;
    r->plan_dirty = false;
    return VOCE_OK;
}

// ---- FFT tile tuning --------------------------------------------------------
// The forward-pass FFT phases (z forward, y, x with the Green operator, z
// inverse) are timed with each candidate tile on the RVE itself, before its
// first increment, and the fastest kept.  A tile only changes how many lines
// a block transforms, never a line's arithmetic, so results do not depend on
// it.  The choice is cached per grid shape and spectrum precision for the
// life of the process.  The z-inverse phase updates DisGrad, which is saved
// and put back; the x phase writes the antisymmetric sum, which the first
// iteration of an increment overwrites; the spectrum is scratch.
struct TileKey {
    int nx, ny, nz, mixed;
    bool operator<(const TileKey &o) const
    {
        if (nx != o.nx) return nx < o.nx;
        if (ny != o.ny) return ny < o.ny;
        if (nz != o.nz) return nz < o.nz;
        return mixed < o.mixed;
    }
};
std::mutex g_tile_mu;
std::map<TileKey, Tiles> g_tile_cache;
int g_autotune = 1;
int g_newton_chord = 1;   // chord steps in the FP64 Newton of new VOCE_PREC_MIXED RVEs
int g_ir_predictor = 1;   // single-precision start of the FP64 steps in new VOCE_PREC_MIXED_IR RVEs

constexpr int kMaxSchedules = 5;

// schedule index k of an axis of length L (the default when out of range)
FftPlan1 schedule_of(int L, bool mixed, int k)
{
    FftPlan1 c[kMaxSchedules];
    const int n = axis_schedules(L, mixed, c, kMaxSchedules);
    return c[(k >= 0 && k < n) ? k : 0];
}

// the tiles and schedule indices an RVE descriptor runs (a restored RVE's)
Tiles tiles_of(const RveDesc &d)
{
    Tiles t;
    t.zrows = d.zrows; t.yxt = d.yxt; t.xkc = d.xkc;
    t.xkc3 = d.xkc3; t.zirows = d.zirows; t.zirows3 = d.zirows3;
    const FftPlan1 *pl[3] = {&d.plx, &d.ply, &d.plz};
    int *slot[3] = {&t.sx, &t.sy, &t.sz};
    for (int a = 0; a < 3; ++a) {
        FftPlan1 c[kMaxSchedules];
        const int n = axis_schedules(pl[a]->L, d.mixed, c, kMaxSchedules);
        for (int k = 0; k < n; ++k)
            if (c[k].n1 == pl[a]->n1 && c[k].nst == pl[a]->nst &&
                std::memcmp(c[k].rad, pl[a]->rad, sizeof(int) * c[k].nst) == 0) {
                *slot[a] = k;
                break;
            }
    }
    return t;
}

void apply_tiles(voce_rve *r, const Tiles &t)
{
    r->tiles = t;
    RveDesc &d = r->d;
    d.zrows = t.zrows; d.yxt = t.yxt; d.xkc = t.xkc;
    d.xkc3 = t.xkc3; d.zirows = t.zirows; d.zirows3 = t.zirows3;
    d.plx = schedule_of(d.nx, d.mixed, t.sx);
    d.ply = schedule_of(d.ny, d.mixed, t.sy);
    d.plz = schedule_of(d.nz, d.mixed, t.sz);
    r->plan_dirty = true;
}

// VOCE_TILE_CACHE=<file>: tile choices are read from the file before any
// tuning and each new choice is appended, so that another process on the
// same machine (a profiler's run of the same command, say) uses the same
// tiles.  One line per shape: nx ny nz mixed zrows yxt xkc xkc3 zirows
// zirows3 sx sy sz (the last three: radix schedule indices of x, y, z).
bool g_tile_file_read = false;

void read_tile_file()
{
    g_tile_file_read = true;
    const char *path = std::getenv("VOCE_TILE_CACHE");
    if (!path || !path[0]) return;
    FILE *f = std::fopen(path, "r");
    if (!f) return;
    TileKey k;
    Tiles t;
    while (std::fscanf(f, "%d %d %d %d %d %d %d %d %d %d %d %d %d", &k.nx, &k.ny, &k.nz, &k.mixed, &t.zrows,
                       &t.yxt, &t.xkc, &t.xkc3, &t.zirows, &t.zirows3, &t.sx, &t.sy, &t.sz) == 13) {
        // the FP64 form runs the default radix schedules whatever the file says
        if (!k.mixed) t.sx = t.sy = t.sz = 0;
        g_tile_cache[k] = t;
    }
    std::fclose(f);
}

void append_tile_file(const TileKey &k, const Tiles &t)
{
    const char *path = std::getenv("VOCE_TILE_CACHE");
    if (!path || !path[0]) return;
    FILE *f = std::fopen(path, "a");
    if (!f) return;
    std::fprintf(f, "%d %d %d %d %d %d %d %d %d %d %d %d %d\n", k.nx, k.ny, k.nz, k.mixed, t.zrows, t.yxt, t.xkc,
                 t.xkc3, t.zirows, t.zirows3, t.sx, t.sy, t.sz);
    std::fclose(f);
}

int autotune_tiles(voce_rve *r)
{
    VOCE_TRACE("autotune_tiles");
    RveDesc &d = r->d;
    const TileKey key{d.nx, d.ny, d.nz, d.mixed};
    {
        std::lock_guard<std::mutex> lock(g_tile_mu);
        if (!g_tile_file_read) read_tile_file();
        auto it = g_tile_cache.find(key);
        if (it != g_tile_cache.end()) {
            apply_tiles(r, it->second);
            return VOCE_OK;
        }
    }
    double *saved = nullptr;
    CUDA_TRY(cudaMalloc(&saved, sizeof(double) * 6 * (size_t)d.nv));
    CUDA_TRY(cudaMemcpyAsync(saved, d.dgs, sizeof(double) * 6 * (size_t)d.nv, cudaMemcpyDeviceToDevice, r->stream));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    Tiles best = r->tiles;
    int rc = VOCE_OK;
    // one phase with tiles t: best of two rounds of 10 launches, after one
    // warm-up launch (ms < 0: a CUDA error, recorded in rc)
    auto time_phase = [&](const Tiles &t, int ph) -> float {
        RveDesc dt = d;
        dt.zrows = t.zrows; dt.yxt = t.yxt; dt.xkc = t.xkc; dt.zirows = t.zirows;
        dt.plx = schedule_of(d.nx, d.mixed, t.sx);
        dt.ply = schedule_of(d.ny, d.mixed, t.sy);
        dt.plz = schedule_of(d.nz, d.mixed, t.sz);
        std::vector<RveDesc> one(1, dt);
        RveDesc *pd = nullptr;
        int2 *pm = nullptr;
        BatchPlan bp;
        rc = make_plan(one, r->precision, pd, pm, bp);
        if (rc) return -1.f;
        float ms = 1e30f;
        cudaError_t e = launch_plan_phase(bp, ph, r->stream);
        for (int round = 0; round < 2 && e == cudaSuccess; ++round) {
            float t = 0.f;
            e = cudaEventRecord(e0, r->stream);
            for (int k = 0; k < 10 && e == cudaSuccess; ++k) e = launch_plan_phase(bp, ph, r->stream);
            if (e == cudaSuccess) e = cudaEventRecord(e1, r->stream);
            if (e == cudaSuccess) e = cudaEventSynchronize(e1);
            if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
            if (e == cudaSuccess && t < ms) ms = t;
        }
        cudaFree(pd);
        cudaFree(pm);
        if (e != cudaSuccess) {
            rc = fail(VOCE_ERR_CUDA, "tile tuning: %s", cudaGetErrorString(e));
            return -1.f;
        }
        return ms;
    };
    const int phases[4] = {BP_ZF, BP_Y6, BP_XG, BP_ZI};
    for (int ph : phases) {
        int cand[8];
        const int nc = tile_candidates(d, ph, cand, 8);
        float best_ms = 1e30f;
        int best_t = 0;
        for (int c = 0; c < nc && rc == VOCE_OK; ++c) {
            Tiles t = best;
            switch (ph) {
            case BP_ZF: t.zrows = cand[c]; break;
            case BP_Y6: t.yxt = cand[c]; break;
            case BP_XG: t.xkc = cand[c]; break;
            default: t.zirows = cand[c]; break;
            }
            const float ms = time_phase(t, ph);
            if (rc) break;
            if (ms < best_ms) {
                best_ms = ms;
                best_t = cand[c];
            }
        }
        if (rc) break;
        if (best_t > 0) {
            switch (ph) {
            case BP_ZF: best.zrows = best_t; break;
            case BP_Y6: best.yxt = best_t; break;
            case BP_XG: best.xkc = best_t; break;
            default: best.zirows = best_t; break;
            }
        }
        // the radix schedule of the axis this phase transforms (z with the
        // forward z pass, which the inverse one shares), with the chosen tile.
        // The schedule changes the rounding of the transform, so a timed
        // choice would make results depend on timing noise: the FP64 form
        // keeps the default schedule of every axis (its bits are the same in
        // every process), only the single-precision spectrum forms tune it.
        if (ph == BP_ZI || !d.mixed) continue;
        const int L = ph == BP_ZF ? d.nz : ph == BP_Y6 ? d.ny : d.nx;
        FftPlan1 sc[kMaxSchedules];
        const int ns = axis_schedules(L, true, sc, kMaxSchedules);
        int &slot = ph == BP_ZF ? best.sz : ph == BP_Y6 ? best.sy : best.sx;
        const int start = slot;
        float sched_ms = best_ms;
        for (int k = 0; k < ns && rc == VOCE_OK && ns > 1; ++k) {
            if (k == start) continue;
            Tiles t = best;
            (ph == BP_ZF ? t.sz : ph == BP_Y6 ? t.sy : t.sx) = k;
            const float ms = time_phase(t, ph);
            if (rc) break;
            // another schedule must be clearly faster: the default's order
            // stays unless timing says otherwise
            if (ms < 0.97f * sched_ms) {
                sched_ms = ms;
                slot = k;
            }
        }
        if (rc) break;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaError_t e = cudaMemcpyAsync(d.dgs, saved, sizeof(double) * 6 * (size_t)d.nv, cudaMemcpyDeviceToDevice,
                                    r->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(r->stream);
    cudaFree(saved);
    if (rc) return rc;
    if (e != cudaSuccess) return fail(VOCE_ERR_CUDA, "tile tuning: %s", cudaGetErrorString(e));
    apply_tiles(r, best);
    std::lock_guard<std::mutex> lock(g_tile_mu);
    g_tile_cache[key] = best;
    append_tile_file(key, best);
    return VOCE_OK;
}

// One increment with the host deciding after every iteration (used when
// profiling per kernel, and when the loop bounds are degenerate).
int run_increment_hostloop(voce_rve *r)
{
    RveDesc &d = r->d;
    int rc = ensure_self_plan(r);
    if (rc) return rc;
    CUDA_TRY(launch_plan_prelude(r->plan, r->stream, r->prof));
    int guard = 0;
    // the reference tests the loop condition before the first iteration
    const bool any = d.iter_max > 0 && 2.0 * std::fabs(d.err_tol) > std::fabs(d.err_tol);
    while (any) {
        cudaError_t e = launch_plan_iteration(r->plan, r->stream, r->prof, 0, 0);
        if (e != cudaSuccess) return fail(VOCE_ERR_CUDA, "iteration launch: %s", cudaGetErrorString(e));
        CUDA_TRY(cudaMemcpyAsync(r->h_flag, &d.macro->converged, sizeof(int), cudaMemcpyDeviceToHost, r->stream));
        CUDA_TRY(cudaStreamSynchronize(r->stream));
        r->prof.collect();
        if (*r->h_flag) break;
        if (++guard > d.iter_max + 1) return fail(VOCE_ERR_STATE, "iteration control lost");
    }
    cudaError_t e = launch_plan_incr_end(r->plan, r->stream, r->prof);
    if (e != cudaSuccess) return fail(VOCE_ERR_CUDA, "increment-end launch: %s", cudaGetErrorString(e));
    return VOCE_OK;
}

// The increment as one CUDA graph: prelude, a conditional WHILE node whose
// body is one Green-operator iteration (the finaliser sets the condition),
// then the increment end.  Built on first use; kernel arguments do not
// change between launches, all state lives in device memory.
int build_graph(voce_rve *r)
{
    int rc = ensure_self_plan(r);
    if (rc) return rc;
    Prof none;  // no events inside graphs
    cudaGraph_t g;
    CUDA_TRY(cudaGraphCreate(&g, 0));
    CUDA_TRY(cudaStreamBeginCaptureToGraph(r->stream, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    CUDA_TRY(launch_plan_prelude(r->plan, r->stream, none));
    CUDA_TRY(cudaStreamEndCapture(r->stream, &g));
    size_t nn = 0;
    CUDA_TRY(cudaGraphGetNodes(g, nullptr, &nn));
    std::vector<cudaGraphNode_t> pre(nn);
    CUDA_TRY(cudaGraphGetNodes(g, pre.data(), &nn));
    cudaGraphConditionalHandle h;
    CUDA_TRY(cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t cond;
    CUDA_TRY(cudaGraphAddNode(&cond, g, pre.data(), nullptr, pre.size(), &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    CUDA_TRY(cudaStreamBeginCaptureToGraph(r->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = launch_plan_iteration(r->plan, r->stream, none, h, 1);
    CUDA_TRY(cudaStreamEndCapture(r->stream, &body));
    CUDA_TRY(e);
    CUDA_TRY(cudaStreamBeginCaptureToGraph(r->stream, g, &cond, nullptr, 1, cudaStreamCaptureModeThreadLocal));
    e = launch_plan_incr_end(r->plan, r->stream, none);
    CUDA_TRY(cudaStreamEndCapture(r->stream, &g));
    CUDA_TRY(e);
    CUDA_TRY(cudaGraphInstantiate(&r->graph_exec, g, 0));
    r->graph = g;
    return VOCE_OK;
}

// Copy the records and iteration logs of the increments finished since the
// last read-back from the device rings (capacity incr_cap increments).
int collect_new(voce_rve *r, bool count_graph_launches)
{
    RveDesc &d = r->d;
    MacroDev m;
    CUDA_TRY(cudaMemcpyAsync(&m, d.macro, sizeof(m), cudaMemcpyDeviceToHost, r->stream));
    CUDA_TRY(cudaStreamSynchronize(r->stream));
    const int completed = m.istep - 1;
    const int fresh = completed - r->n_done;
    if (fresh <= 0) return VOCE_OK;
    if (fresh > d.incr_cap) return fail(VOCE_ERR_STATE, "increment ring overflow (%d > %d)", fresh, d.incr_cap);
    std::vector<IncrDev> recs(d.incr_cap);
    std::vector<double> logs((size_t)d.incr_cap * d.iter_max * VOCE_ITLOG);
    CUDA_TRY(cudaMemcpyAsync(recs.data(), d.incr, sizeof(IncrDev) * recs.size(), cudaMemcpyDeviceToHost, r->stream));
    CUDA_TRY(cudaMemcpyAsync(logs.data(), d.itlog, sizeof(double) * logs.size(), cudaMemcpyDeviceToHost, r->stream));
    CUDA_TRY(cudaStreamSynchronize(r->stream));
    CUDA_TRY(cudaGetLastError());
    const int first = r->n_done;
    for (int k = 0; k < fresh; ++k) {
        const int slot = (first + k) % d.incr_cap;
        if (recs[slot].istep != first + k + 1)
            return fail(VOCE_ERR_STATE, "increment record %d missing", first + k + 1);
        // one prelude, 7 launches per iteration, 7 at the increment end
        if (count_graph_launches) r->prof.launches += 1 + 7LL * recs[slot].iters + 7;
        collect_increment(r, recs[slot], logs.data() + (size_t)slot * d.iter_max * VOCE_ITLOG);
    }
    return VOCE_OK;
}

// Grow the record rings to hold `cap` increments (drops the cached graph
// and plan, whose kernel arguments point at the old rings).
int ensure_ring(voce_rve *r, int cap)
{
    RveDesc &d = r->d;
    if (cap <= d.incr_cap) return VOCE_OK;
    int rc = collect_new(r, false);
    if (rc) return rc;
    double *lg = nullptr;
    IncrDev *ic = nullptr;
    if ((rc = dalloc(r, lg, (size_t)cap * VOCE_ITLOG * (d.iter_max > 0 ? d.iter_max : 1)))) return rc;
    if ((rc = dalloc(r, ic, (size_t)cap))) return rc;
    // live slots keep their absolute index modulo the capacity
    std::vector<IncrDev> old(d.incr_cap);
    CUDA_TRY(cudaMemcpy(old.data(), d.incr, sizeof(IncrDev) * old.size(), cudaMemcpyDeviceToHost));
    for (int k = 0; k < d.incr_cap; ++k)
        if (old[k].istep > 0)
            CUDA_TRY(cudaMemcpy(ic + (old[k].istep - 1) % cap, &old[k], sizeof(IncrDev), cudaMemcpyHostToDevice));
    // the increment in progress keeps the log rows of its iterations so far
    // (an RVE taken out of a batch in the middle of an increment)
    if (d.iter_max > 0) {
        MacroDev m;
        CUDA_TRY(cudaMemcpy(&m, d.macro, sizeof(m), cudaMemcpyDeviceToHost));
        if (m.istep >= 1) {
            const size_t rows = (size_t)d.iter_max * VOCE_ITLOG;
            CUDA_TRY(cudaMemcpy(lg + (size_t)((m.istep - 1) % cap) * rows,
                                d.itlog + (size_t)((m.istep - 1) % d.incr_cap) * rows, sizeof(double) * rows,
                                cudaMemcpyDeviceToDevice));
        }
    }
    // the old ring goes (nothing in flight uses it: the RVE's stream was
    // drained by collect_new, and it belongs to no batch)
    for (void *q : {(void *)d.itlog, (void *)d.incr}) {
        auto it = std::find(r->dev_allocs.begin(), r->dev_allocs.end(), q);
        if (it != r->dev_allocs.end()) {
            r->dev_allocs.erase(it);
            CUDA_TRY(cudaFree(q));
        }
    }
    d.itlog = lg;
    d.incr = ic;
    d.incr_cap = cap;
    if (r->graph_exec) { cudaGraphExecDestroy(r->graph_exec); r->graph_exec = nullptr; }
    if (r->graph) { cudaGraphDestroy(r->graph); r->graph = nullptr; }
    r->plan_dirty = true;
    return VOCE_OK;
}

}  // namespace

bool voce::tiles_known(const int dims[3], int precision)
{
    std::lock_guard<std::mutex> lock(g_tile_mu);
    if (!g_autotune) return true;
    if (!g_tile_file_read) read_tile_file();
    return g_tile_cache.count(TileKey{dims[0], dims[1], dims[2], precision != VOCE_PREC_FP64 ? 1 : 0}) != 0;
}

extern "C" {

int voce_rve_run(voce_rve *r, int n)
{
    VOCE_TRACE("voce_rve_run");
    if (!r || n < 0) return fail(VOCE_ERR_ARG, "bad argument");
    if (r->batch) return fail(VOCE_ERR_STATE, "the RVE belongs to a batch; run the batch or remove it");
    RveDesc &d = r->d;
    const bool graph_ok = r->use_graph && !r->prof.on && d.iter_max > 0 && d.err_tol != 0.0;
    if (graph_ok && !r->graph_exec) {
        int rc = build_graph(r);
        if (rc) return rc;
    }
    int done = 0;
    while (done < n) {
        const int chunk = std::min(n - done, d.incr_cap);
        for (int k = 0; k < chunk; ++k) {
            if (graph_ok) {
                CUDA_TRY(cudaGraphLaunch(r->graph_exec, r->stream));
            } else {
                int rc = run_increment_hostloop(r);
                if (rc) return rc;
            }
        }
        int rc = collect_new(r, graph_ok);
        if (rc) return rc;
        done += chunk;
    }
    return VOCE_OK;
}

int voce_rve_increments_done(const voce_rve *r) { return r ? r->n_done : -1; }

int voce_rve_get_increment(const voce_rve *r, int k, voce_increment *out)
{
    if (!r || !out || k < 0 || k >= (int)r->incr.size()) return fail(VOCE_ERR_ARG, "bad increment index");
    *out = r->incr[k];
    return VOCE_OK;
}

int voce_rve_get_iter_log(const voce_rve *r, int k, double *ee, double *es, double *sv, int max)
{
    if (!r || k < 0 || k >= (int)r->itlog.size()) return -fail(VOCE_ERR_ARG, "bad increment index");
    const std::vector<double> &l = r->itlog[k];
    int n = (int)(l.size() / VOCE_ITLOG);
    if (n > max) n = max;
    for (int i = 0; i < n; ++i) {
        if (ee) ee[i] = l[VOCE_ITLOG * i];
        if (es) es[i] = l[VOCE_ITLOG * i + 1];
        if (sv) sv[i] = l[VOCE_ITLOG * i + 2];
    }
    return n;
}

int voce_rve_get_iter_detail(const voce_rve *r, int k, double *rows, int max)
{
    if (!r || k < 0 || k >= (int)r->itlog.size()) return -fail(VOCE_ERR_ARG, "bad increment index");
    const std::vector<double> &l = r->itlog[k];
    int n = (int)(l.size() / VOCE_ITLOG);
    if (n > max) n = max;
    if (rows) std::memcpy(rows, l.data(), sizeof(double) * VOCE_ITLOG * (size_t)n);
    return n;
}

int voce_rve_get_field(voce_rve *r, int field, double *host_out)
{
    VOCE_TRACE("voce_rve_get_field");
    if (!r || !host_out) return fail(VOCE_ERR_ARG, "null argument");
    int per;
    switch (field) {
    case 0: case 1: case 2: case 3: case 4: per = 9; break;
    case 5: case 6: case 10: case 11: per = 12; break;
    case 7: case 8: case 9: case 12: case 13: case 14: per = 1; break;
    case 15: per = 3; break;
    case 20: case 21: per = 6; break;
    default: return fail(VOCE_ERR_ARG, "unknown field %d", field);
    }
    if (!r->d_out) CUDA_TRY(cudaMalloc(&r->d_out, sizeof(double) * 12 * r->d.nv));
    if (field == VOCE_FIELD_DISP_FLUCT) {
        if (!r->d_dispwork) CUDA_TRY(cudaMalloc(&r->d_dispwork, disp_work_bytes(r->d)));
        CUDA_TRY(launch_disp_fluct(r->d, r->d_dispwork, r->d_out, r->stream));
    } else {
        CUDA_TRY(launch_field_out(r->d, field, r->d_out, r->stream));
    }
    CUDA_TRY(cudaMemcpyAsync(host_out, r->d_out, sizeof(double) * per * r->d.nv, cudaMemcpyDeviceToHost, r->stream));
    CUDA_TRY(cudaStreamSynchronize(r->stream));
    return VOCE_OK;
}

}  // extern "C"

// ---- field download without device allocation -----------------------------
// voce_rve_get_field stages a field in a buffer it cudaMallocs on first use.
// Callers that cannot allocate use voce_rve_get_field_noalloc instead, which
// stages in the fixed array below: a server whose HBM budget is committed to
// admitted RVEs when it downloads a finished request (the download comes
// before that request's memory is freed), a host that overlaps downloads with
// other RVEs' increments on other streams (cudaMalloc and cudaFree can
// synchronise the whole device), and hosts that hand all device memory to
// their own pool allocator.  The array is 32 MiB on every GPU that loads this
// library's device code, held until the process exits.
static __device__ __align__(256) double g_field_stage[VOCE_NOALLOC_MAX_DOUBLES];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_stage_mu;
double *g_stage_ptr[kMaxDevices] = {};

// Device address of g_field_stage on device dev, which must be current.  The
// host-side name is only a stand-in for the symbol, so the address is asked
// for once per device and kept.
int stage_address(int dev, double **out)
{
    if (dev < 0 || dev >= kMaxDevices)
        return fail(VOCE_ERR_UNSUPPORTED, "device %d: no staging array above device %d", dev,
                    kMaxDevices - 1);
    std::lock_guard<std::mutex> lock(g_stage_mu);
    if (!g_stage_ptr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_field_stage);
        if (e != cudaSuccess || !p)
            return fail(VOCE_ERR_CUDA, "cudaGetSymbolAddress(g_field_stage) on device %d: %s", dev,
                        cudaGetErrorString(e));
        g_stage_ptr[dev] = static_cast<double *>(p);
    }
    *out = g_stage_ptr[dev];
    return VOCE_OK;
}

int noalloc_download(voce_rve *r, int field, long long n, int dev, double *host_out)
{
    double *stage = nullptr;
    int rc = stage_address(dev, &stage);
    if (rc) return rc;
    // k_field_out writes each of the n doubles read back below, so nothing in
    // the array has to start at zero; what lies past n keeps an earlier call's
    // values and is never read.
    CUDA_TRY(launch_field_out(r->d, field, stage, r->stream));
    CUDA_TRY(cudaMemcpyAsync(host_out, stage, sizeof(double) * n, cudaMemcpyDeviceToHost, r->stream));
    CUDA_TRY(cudaStreamSynchronize(r->stream));
    return VOCE_OK;
}

}  // namespace

extern "C" {

int voce_rve_get_field_noalloc(voce_rve *r, int field, double *host_out)
{
    if (!r || !host_out) return fail(VOCE_ERR_ARG, "null argument");
    int per;
    switch (field) {
    case 0: case 1: case 2: case 3: case 4: per = 9; break;
    case 5: case 6: case 10: case 11: per = 12; break;
    case 7: case 8: case 9: case 12: case 13: case 14: per = 1; break;
    case 20: case 21: per = 6; break;
    case 15:
        return fail(VOCE_ERR_UNSUPPORTED,
                    "field 15 (displacement fluctuation) transforms through a spectrum work array; "
                    "use voce_rve_get_field");
    default: return fail(VOCE_ERR_ARG, "unknown field %d", field);
    }
    const long long n = (long long)per * r->d.nv;
    if (n > VOCE_NOALLOC_MAX_DOUBLES)
        return fail(VOCE_ERR_UNSUPPORTED,
                    "field %d of %lld voxels is %lld doubles, more than the %d doubles of the "
                    "no-allocation staging array; use voce_rve_get_field",
                    field, (long long)r->d.nv, n, VOCE_NOALLOC_MAX_DOUBLES);
    // the RVE's stream names its device; run there and restore the caller's
    int dev = 0, cur = 0;
    CUDA_TRY(cudaStreamGetDevice(r->stream, &dev));
    CUDA_TRY(cudaGetDevice(&cur));
    if (dev != cur) CUDA_TRY(cudaSetDevice(dev));
    int rc = noalloc_download(r, field, n, dev, host_out);
    if (dev != cur) cudaSetDevice(cur);
    return rc;
}

int voce_rve_get_ids(const voce_rve *r, int *grain, int *phase)
{
    if (!r) return fail(VOCE_ERR_ARG, "null argument");
    if (grain) std::memcpy(grain, r->grain.data(), sizeof(int) * r->grain.size());
    if (phase) std::memcpy(phase, r->phase.data(), sizeof(int) * r->phase.size());
    return VOCE_OK;
}

int voce_rve_get_namelist(const voce_rve *r, voce_namelist *out)
{
    if (!r || !out) return fail(VOCE_ERR_ARG, "null argument");
    *out = r->nl;
    return VOCE_OK;
}

}  // extern "C"

// ---- snapshot / restore ----------------------------------------------------
namespace {

struct SnapHead {
    char magic[8];
    uint32_t version, desc_size, macro_size, nl_size, incr_size;
    int32_t precision, npart, n_incr, pad;
    int64_t nv, total;
};
const char kSnapMagic[8] = {'V', 'O', 'C', 'E', 'S', 'N', 'A', 'P'};

// Writes (or, with out == nullptr, only sizes) the snapshot of r.
long long snapshot_write(voce_rve *r, char *out)
{
    RveDesc &d = r->d;
    long long pos = 0;
    auto put = [&](const void *src, size_t n) {
        if (out) std::memcpy(out + pos, src, n);
        pos += (long long)n;
    };
    SnapHead h;
    std::memset(&h, 0, sizeof(h));
    std::memcpy(h.magic, kSnapMagic, 8);
    h.version = 3;
    h.desc_size = sizeof(RveDesc);
    h.macro_size = sizeof(MacroDev);
    h.nl_size = sizeof(voce_namelist);
    h.incr_size = sizeof(voce_increment);
    h.precision = r->precision;
    h.npart = r->npart;
    h.n_incr = (int32_t)r->incr.size();
    h.nv = d.nv;
    put(&h, sizeof(h));
    put(&d, sizeof(RveDesc));
    put(&r->nl, sizeof(voce_namelist));
    put(r->grain.data(), sizeof(int) * r->grain.size());
    put(r->phase.data(), sizeof(int) * r->phase.size());
    for (size_t k = 0; k < r->incr.size(); ++k) {
        put(&r->incr[k], sizeof(voce_increment));
        const int64_t n = (int64_t)r->itlog[k].size();
        put(&n, sizeof(n));
        put(r->itlog[k].data(), sizeof(double) * (size_t)n);
    }
    int rc = VOCE_OK;
    for_state(d, [&](void **p, size_t n) {
        if (out && rc == VOCE_OK) {
            cudaError_t e = cudaMemcpy(out + pos, *p, n, cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) rc = fail(VOCE_ERR_CUDA, "snapshot copy: %s", cudaGetErrorString(e));
        }
        pos += (long long)n;
    });
    // the log rows of the increment in progress (its iterations so far; the
    // records of finished increments are above)
    if (d.iter_max > 0) {
        const size_t rows = (size_t)d.iter_max * VOCE_ITLOG;
        if (out && rc == VOCE_OK) {
            MacroDev m;
            cudaError_t e = cudaMemcpy(&m, d.macro, sizeof(m), cudaMemcpyDeviceToHost);
            if (e == cudaSuccess)
                e = cudaMemcpy(out + pos, d.itlog + (size_t)((m.istep - 1) % d.incr_cap) * rows,
                               sizeof(double) * rows, cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) rc = fail(VOCE_ERR_CUDA, "snapshot copy: %s", cudaGetErrorString(e));
        }
        pos += (long long)(sizeof(double) * rows);
    }
    if (rc) return -rc;
    if (out) {
        h.total = pos;
        std::memcpy(out + offsetof(SnapHead, total), &h.total, sizeof(h.total));
    }
    return pos;
}

// A restored RVE runs the kernels on the descriptor its snapshot carries.
// Everything in it that sizes an array or bounds an index is checked against
// what creation makes for the same grid and form, so that a damaged or
// edited snapshot is refused on the host and never reaches the GPU.  Returns
// what is wrong, or nullptr.
const char *snapshot_desc_problem(const SnapHead &h, const RveDesc &d, const voce_namelist &nl)
{
    if (h.precision < VOCE_PREC_FP64 || h.precision > VOCE_PREC_MIXED_IR) return "unknown precision";
    if (d.mixed != (h.precision != VOCE_PREC_FP64 ? 1 : 0) ||
        d.nr32 != (h.precision == VOCE_PREC_MIXED_NR32 ? 1 : 0) ||
        d.ir != (h.precision == VOCE_PREC_MIXED_IR ? 1 : 0))
        return "precision flags disagree with the precision";
    if (d.chord < 0 || d.chord > 1 || (d.chord && h.precision != VOCE_PREC_MIXED) ||
        d.ir_pred < 0 || d.ir_pred > 1 || (d.ir_pred && !d.ir))
        return "Newton options disagree with the precision";
    FftPlan1 p;
    if (!fft_plan(d.nx, p) || !fft_plan(d.ny, p) || !fft_plan(d.nz, p) || d.nz % 2) return "unsupported grid";
    if (d.nzh != d.nz / 2 + 1 || d.nv != (long long)d.nx * d.ny * d.nz ||
        d.nspec != (long long)d.nzh * d.nx * d.ny || d.nv != h.nv)
        return "grid sizes disagree";
    // each axis runs one of its transform candidates
    const FftPlan1 *pl[3] = {&d.plx, &d.ply, &d.plz};
    const int L[3] = {d.nx, d.ny, d.nz};
    for (int a = 0; a < 3; ++a) {
        FftPlan1 c[kMaxSchedules];
        const int n = axis_schedules(L[a], d.mixed != 0, c, kMaxSchedules);
        bool found = false;
        for (int k = 0; k < n && !found; ++k)
            found = pl[a]->L == L[a] && c[k].n1 == pl[a]->n1 && c[k].nst == pl[a]->nst &&
                    std::memcmp(c[k].rad, pl[a]->rad, sizeof(int) * c[k].nst) == 0;
        if (!found) return "FFT schedule";
    }
    // the tiles: the rule voce_rve_set_tiles applies
    const int dim[6] = {d.ny, d.nx, d.ny, d.ny, d.ny, d.ny};
    const int tl[6] = {d.zrows, d.yxt, d.xkc, d.zirows, d.xkc3, d.zirows3};
    for (int k = 0; k < 6; ++k)
        if (tl[k] < 1 || dim[k] % tl[k] != 0) return "FFT tiles";
    for (int ph = BP_ZF; ph < BP_COUNT; ++ph)
        if (batch_smem(d, ph) > 227 * 1024) return "FFT tiles";
    if (h.npart < 1 || d.npart != h.npart || h.npart > std::max<long long>(1, (d.nv + 127) / 128))
        return "work split";
    if (d.nsys < 1 || d.nsys > VOCE_NS) return "number of slip systems";
    if (d.iter_max < 0 || d.iter_max != nl.IterMax) return "IterMax";
    if (d.ipow_n != -1 && (d.ipow_n < 1 || d.ipow_n > 256)) return "flow exponent";
    return nullptr;
}

// The device state bytes the kernels index by: phase ids (1 or 2) and the
// macro state's increment and iteration counters.
const char *snapshot_state_problem(const RveDesc &d, void **which, const char *bytes, size_t n)
{
    if (which == (void **)&d.phase) {
        for (size_t i = 0; i < n / sizeof(int); ++i) {
            int v;
            std::memcpy(&v, bytes + i * sizeof(int), sizeof(int));
            if (v < 1 || v > 2) return "phase id";
        }
    } else if (which == (void **)&d.macro) {
        MacroDev m;
        std::memcpy(&m, bytes, sizeof(m));
        if (m.istep < 1 || m.iter < 0 || m.iter > d.iter_max) return "increment or iteration counter";
    }
    return nullptr;
}

}  // namespace

extern "C" {

long long voce_rve_snapshot_size(voce_rve *r)
{
    if (!r) return -fail(VOCE_ERR_ARG, "null argument");
    if (!r->batch) {
        CUDA_TRY_NEG(cudaStreamSynchronize(r->stream));
        const int rc = collect_new(r, false);
        if (rc) return -rc;
    }
    return snapshot_write(r, nullptr);
}

int voce_rve_snapshot(voce_rve *r, void *buf, long long size)
{
    VOCE_TRACE("voce_rve_snapshot");
    if (!r || !buf) return fail(VOCE_ERR_ARG, "null argument");
    if (r->batch) return fail(VOCE_ERR_STATE, "the RVE belongs to a batch; remove it first");
    CUDA_TRY(cudaStreamSynchronize(r->stream));
    int rc = collect_new(r, false);
    if (rc) return rc;
    const long long need = snapshot_write(r, nullptr);
    if (size < need) return fail(VOCE_ERR_ARG, "snapshot buffer of %lld bytes, %lld needed", size, need);
    const long long n = snapshot_write(r, static_cast<char *>(buf));
    return n < 0 ? (int)-n : VOCE_OK;
}

int voce_rve_restore(const void *buf, long long size, voce_rve **out)
{
    VOCE_TRACE("voce_rve_restore");
    if (!buf || !out) return fail(VOCE_ERR_ARG, "null argument");
    const char *in = static_cast<const char *>(buf);
    SnapHead h;
    if (size < (long long)sizeof(h)) return fail(VOCE_ERR_PARSE, "snapshot too short");
    std::memcpy(&h, in, sizeof(h));
    if (std::memcmp(h.magic, kSnapMagic, 8) != 0) return fail(VOCE_ERR_PARSE, "not an RVE snapshot");
    if (h.version != 3 || h.desc_size != sizeof(RveDesc) || h.macro_size != sizeof(MacroDev) ||
        h.nl_size != sizeof(voce_namelist) || h.incr_size != sizeof(voce_increment))
        return fail(VOCE_ERR_UNSUPPORTED, "snapshot written by a different build of the library");
    if (h.total != size) return fail(VOCE_ERR_PARSE, "snapshot of %lld bytes, header says %lld", size, (long long)h.total);
    long long pos = sizeof(h);
    auto get = [&](void *dst, size_t n) -> bool {
        if (pos + (long long)n > size) return false;
        std::memcpy(dst, in + pos, n);
        pos += (long long)n;
        return true;
    };
    voce_rve *r = new voce_rve();
    RveDesc &d = r->d;
    bool ok = get(&d, sizeof(RveDesc)) && get(&r->nl, sizeof(voce_namelist));
    if (!ok || d.nv != h.nv || h.npart < 1 || h.n_incr < 0) {
        delete r;
        return fail(VOCE_ERR_PARSE, "snapshot header and descriptor disagree");
    }
    if (const char *bad = snapshot_desc_problem(h, d, r->nl)) {
        delete r;
        return fail(VOCE_ERR_PARSE, "damaged snapshot: %s", bad);
    }
    r->precision = h.precision;
    r->npart = h.npart;
    r->tiles = tiles_of(d);
    r->grain.resize((size_t)d.nv);
    r->phase.resize((size_t)d.nv);
    ok = get(r->grain.data(), sizeof(int) * (size_t)d.nv) && get(r->phase.data(), sizeof(int) * (size_t)d.nv);
    for (int k = 0; ok && k < h.n_incr; ++k) {
        voce_increment rec;
        int64_t n = 0;
        ok = get(&rec, sizeof(rec)) && get(&n, sizeof(n)) && n >= 0 && n < (int64_t)1 << 30;
        if (!ok) break;
        std::vector<double> lg((size_t)n);
        ok = get(lg.data(), sizeof(double) * (size_t)n);
        r->incr.push_back(rec);
        r->itlog.push_back(std::move(lg));
    }
    if (!ok) {
        delete r;
        return fail(VOCE_ERR_PARSE, "truncated snapshot");
    }
    r->n_done = h.n_incr;
    r->n_steps = r->nl.N_steps;
    cudaError_t e = cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete r;
        return fail(VOCE_ERR_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(e));
    }
    int rc = alloc_device(r);
    if (rc) {
        delete r;
        return rc;
    }
    int istep = 1;
    for_state(d, [&](void **p, size_t n) {
        if (rc) return;
        if (pos + (long long)n > size) { rc = fail(VOCE_ERR_PARSE, "truncated snapshot"); return; }
        if (const char *bad = snapshot_state_problem(d, p, in + pos, n)) {
            rc = fail(VOCE_ERR_PARSE, "damaged snapshot: %s", bad);
            return;
        }
        if (p == (void **)&d.macro) {
            MacroDev m;
            std::memcpy(&m, in + pos, sizeof(m));
            istep = m.istep;
        }
        cudaError_t e2 = cudaMemcpy(*p, in + pos, n, cudaMemcpyHostToDevice);
        if (e2 != cudaSuccess) rc = fail(VOCE_ERR_CUDA, "restore copy: %s", cudaGetErrorString(e2));
        pos += (long long)n;
    });
    // the log rows of the increment in progress, into its slot of the new ring
    if (rc == VOCE_OK && d.iter_max > 0) {
        const size_t rows = (size_t)d.iter_max * VOCE_ITLOG;
        if (pos + (long long)(sizeof(double) * rows) > size) {
            rc = fail(VOCE_ERR_PARSE, "truncated snapshot");
        } else {
            cudaError_t e4 = cudaMemcpy(d.itlog + (size_t)((istep - 1) % d.incr_cap) * rows, in + pos,
                                        sizeof(double) * rows, cudaMemcpyHostToDevice);
            if (e4 != cudaSuccess) rc = fail(VOCE_ERR_CUDA, "restore copy: %s", cudaGetErrorString(e4));
            pos += (long long)(sizeof(double) * rows);
        }
    }
    if (rc == VOCE_OK && pos != size) rc = fail(VOCE_ERR_PARSE, "snapshot of %lld bytes, %lld read", size, pos);
    if (rc == VOCE_OK) {
        cudaError_t e3 = launch_fill_green(d, r->stream);
        if (e3 == cudaSuccess) e3 = cudaStreamSynchronize(r->stream);
        if (e3 != cudaSuccess) rc = fail(VOCE_ERR_CUDA, "restore: %s", cudaGetErrorString(e3));
    }
    if (rc) {
        delete r;
        return rc;
    }
    // the device record rings start empty; the next increment writes slot
    // (istep - 1) mod capacity as usual
    *out = r;
    return VOCE_OK;
}

int voce_rve_save(voce_rve *r, const char *path)
{
    if (!r || !path) return fail(VOCE_ERR_ARG, "null argument");
    const long long n = voce_rve_snapshot_size(r);
    if (n < 0) return (int)-n;
    std::vector<char> buf((size_t)n);
    int rc = voce_rve_snapshot(r, buf.data(), n);
    if (rc) return rc;
    FILE *f = std::fopen(path, "wb");
    if (!f) return fail(VOCE_ERR_IO, "cannot open %s", path);
    const bool ok = std::fwrite(buf.data(), 1, buf.size(), f) == buf.size();
    if (std::fclose(f) != 0 || !ok) return fail(VOCE_ERR_IO, "cannot write %s", path);
    return VOCE_OK;
}

int voce_rve_load(const char *path, voce_rve **out)
{
    if (!path || !out) return fail(VOCE_ERR_ARG, "null argument");
    FILE *f = std::fopen(path, "rb");
    if (!f) return fail(VOCE_ERR_IO, "cannot open %s", path);
    std::fseek(f, 0, SEEK_END);
    const long n = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (n <= 0) {
        std::fclose(f);
        return fail(VOCE_ERR_IO, "cannot read %s", path);
    }
    std::vector<char> buf((size_t)n);
    const bool ok = std::fread(buf.data(), 1, buf.size(), f) == buf.size();
    std::fclose(f);
    if (!ok) return fail(VOCE_ERR_IO, "cannot read %s", path);
    return voce_rve_restore(buf.data(), (long long)n, out);
}

int voce_mesh_voronoi(const int dims[3], int n_seeds, const double *seeds_xyz,
                      const double *grain_euler_deg, double *euler_deg, int *grain, int *phase)
{
    if (!dims || !seeds_xyz || !grain_euler_deg || !euler_deg || !grain || !phase)
        return fail(VOCE_ERR_ARG, "null argument");
    if (dims[0] < 1 || dims[1] < 1 || dims[2] < 1 || n_seeds < 1)
        return fail(VOCE_ERR_ARG, "empty grid or no seeds");
    const long long nv = (long long)dims[0] * dims[1] * dims[2];
    if (nv > (1LL << 31) - 1) return fail(VOCE_ERR_UNSUPPORTED, "grid of %lld voxels", nv);
    double *d_seeds = nullptr;
    int *d_label = nullptr;
    cudaStream_t s = nullptr;
    int rc = VOCE_OK;
    std::vector<int> lab((size_t)nv);
    do {
        cudaError_t e;
        if ((e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)) != cudaSuccess ||
            (e = cudaMalloc(&d_seeds, sizeof(double) * 3 * (size_t)n_seeds)) != cudaSuccess ||
            (e = cudaMalloc(&d_label, sizeof(int) * (size_t)nv)) != cudaSuccess ||
            (e = cudaMemcpyAsync(d_seeds, seeds_xyz, sizeof(double) * 3 * (size_t)n_seeds,
                                 cudaMemcpyHostToDevice, s)) != cudaSuccess ||
            (e = launch_voronoi(dims[0], dims[1], dims[2], n_seeds, d_seeds, d_label, s)) != cudaSuccess ||
            (e = cudaMemcpyAsync(lab.data(), d_label, sizeof(int) * (size_t)nv, cudaMemcpyDeviceToHost, s)) !=
                cudaSuccess ||
            (e = cudaStreamSynchronize(s)) != cudaSuccess) {
            rc = fail(e == cudaErrorMemoryAllocation ? VOCE_ERR_NOMEM : VOCE_ERR_CUDA, "voronoi: %s",
                      cudaGetErrorString(e));
        }
    } while (0);
    if (d_seeds) cudaFree(d_seeds);
    if (d_label) cudaFree(d_label);
    if (s) cudaStreamDestroy(s);
    if (rc) return rc;
    for (long long v = 0; v < nv; ++v) {
        const int g = lab[(size_t)v];
        euler_deg[3 * v] = grain_euler_deg[3 * g];
        euler_deg[3 * v + 1] = grain_euler_deg[3 * g + 1];
        euler_deg[3 * v + 2] = grain_euler_deg[3 * g + 2];
        grain[v] = g + 1;
        phase[v] = 1;
    }
    return VOCE_OK;
}

int voce_set_autotune(int on)
{
    g_autotune = on ? 1 : 0;
    return VOCE_OK;
}

int voce_rve_get_tiles(const voce_rve *r, int tiles[6])
{
    if (!r || !tiles) return fail(VOCE_ERR_ARG, "null argument");
    const Tiles &t = r->tiles;
    tiles[0] = t.zrows; tiles[1] = t.yxt; tiles[2] = t.xkc;
    tiles[3] = t.zirows; tiles[4] = t.xkc3; tiles[5] = t.zirows3;
    return VOCE_OK;
}

int voce_set_newton_chord(int on)
{
    g_newton_chord = on ? 1 : 0;
    return VOCE_OK;
}

int voce_set_ir_predictor(int on)
{
    g_ir_predictor = on ? 1 : 0;
    return VOCE_OK;
}

int voce_fft_schedule_count(int L)
{
    FftPlan1 c[4];
    return fft_schedules(L, c, 4);
}

int voce_rve_fft_schedule_count(const voce_rve *r, int axis)
{
    if (!r || axis < 0 || axis > 2) return -fail(VOCE_ERR_ARG, "bad argument");
    const int L = axis == 0 ? r->d.nx : axis == 1 ? r->d.ny : r->d.nz;
    FftPlan1 c[kMaxSchedules];
    return axis_schedules(L, r->d.mixed, c, kMaxSchedules);
}

int voce_rve_get_fft_schedule(const voce_rve *r, int axis, int *radices, int max)
{
    if (!r || axis < 0 || axis > 2) return -fail(VOCE_ERR_ARG, "bad argument");
    const FftPlan1 &p = axis == 0 ? r->d.plx : axis == 1 ? r->d.ply : r->d.plz;
    if (p.n1 > 0) {   // the register FFT: its two passes
        const int rr[2] = {p.n1, p.L / p.n1};
        for (int k = 0; k < 2 && k < max && radices; ++k) radices[k] = rr[k];
        return 2;
    }
    for (int k = 0; k < p.nst && k < max && radices; ++k) radices[k] = p.rad[k];
    return p.nst;
}

int voce_rve_set_fft_schedule(voce_rve *r, int axis, int k)
{
    if (!r || axis < 0 || axis > 2) return fail(VOCE_ERR_ARG, "bad argument");
    if (r->batch) return fail(VOCE_ERR_STATE, "the RVE belongs to a batch");
    const int n = voce_rve_fft_schedule_count(r, axis);
    const int L = axis == 0 ? r->d.nx : axis == 1 ? r->d.ny : r->d.nz;
    if (k < 0 || k >= n) return fail(VOCE_ERR_ARG, "schedule %d of %d for length %d", k, n, L);
    CUDA_TRY(cudaStreamSynchronize(r->stream));
    Tiles t = r->tiles;
    (axis == 0 ? t.sx : axis == 1 ? t.sy : t.sz) = k;
    apply_tiles(r, t);
    if (r->graph_exec) { cudaGraphExecDestroy(r->graph_exec); r->graph_exec = nullptr; }
    if (r->graph) { cudaGraphDestroy(r->graph); r->graph = nullptr; }
    return VOCE_OK;
}

int voce_rve_set_tiles(voce_rve *r, const int tiles[6])
{
    if (!r || !tiles) return fail(VOCE_ERR_ARG, "null argument");
    if (r->batch) return fail(VOCE_ERR_STATE, "the RVE belongs to a batch");
    const RveDesc &d = r->d;
    // each tile divides the dimension it splits, and its phase fits in shared memory
    const int dim[6] = {d.ny, d.nx, d.ny, d.ny, d.ny, d.ny};
    for (int k = 0; k < 6; ++k)
        if (tiles[k] < 1 || dim[k] % tiles[k] != 0) return fail(VOCE_ERR_ARG, "tile %d = %d", k, tiles[k]);
    Tiles t = r->tiles;   // the radix schedules stay
    t.zrows = tiles[0]; t.yxt = tiles[1]; t.xkc = tiles[2];
    t.zirows = tiles[3]; t.xkc3 = tiles[4]; t.zirows3 = tiles[5];
    RveDesc dt = d;
    dt.zrows = t.zrows; dt.yxt = t.yxt; dt.xkc = t.xkc; dt.xkc3 = t.xkc3; dt.zirows = t.zirows; dt.zirows3 = t.zirows3;
    for (int ph = BP_ZF; ph < BP_COUNT; ++ph)
        if (batch_smem(dt, ph) > 227 * 1024) return fail(VOCE_ERR_ARG, "tiles need more shared memory than a block has");
    CUDA_TRY(cudaStreamSynchronize(r->stream));
    apply_tiles(r, t);
    if (r->graph_exec) { cudaGraphExecDestroy(r->graph_exec); r->graph_exec = nullptr; }
    if (r->graph) { cudaGraphDestroy(r->graph); r->graph = nullptr; }
    return VOCE_OK;
}

int voce_rve_destroy(voce_rve *r)
{
    if (r && r->batch) voce_batch_remove(r->batch, r);
    delete r;
    return VOCE_OK;
}

// ---------------------------------------------------------------------------
// measurement and diagnostics (voce_gpu_diag.h)
// ---------------------------------------------------------------------------
int voce_rve_run_timed(voce_rve *r, int n, double *device_ms)
{
    if (!r || !device_ms) return fail(VOCE_ERR_ARG, "null argument");
    cudaEvent_t e0, e1;
    CUDA_TRY(cudaEventCreate(&e0));
    CUDA_TRY(cudaEventCreate(&e1));
    CUDA_TRY(cudaEventRecord(e0, r->stream));
    int rc = voce_rve_run(r, n);
    if (rc == VOCE_OK) {
        CUDA_TRY(cudaEventRecord(e1, r->stream));
        CUDA_TRY(cudaEventSynchronize(e1));
        float ms = 0.f;
        CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
        *device_ms = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
}

int voce_rve_set_graph(voce_rve *r, int on)
{
    if (!r) return fail(VOCE_ERR_ARG, "null argument");
    r->use_graph = on != 0;
    return VOCE_OK;
}

int voce_rve_set_profiling(voce_rve *r, int on)
{
    if (!r) return fail(VOCE_ERR_ARG, "null argument");
    if (on && !r->prof.ev[0])
        for (int k = 0; k < 2 * K_COUNT; ++k) CUDA_TRY(cudaEventCreate(&r->prof.ev[k]));
    r->prof.on = on != 0;
    return VOCE_OK;
}

int voce_rve_get_kernel_time(const voce_rve *r, int kernel, double *ms_total, long long *timed_launches)
{
    if (!r || kernel < 0 || kernel >= K_COUNT) return fail(VOCE_ERR_ARG, "bad kernel id");
    if (ms_total) *ms_total = r->prof.ms[kernel];
    if (timed_launches) *timed_launches = r->prof.n[kernel];
    return VOCE_OK;
}

int voce_rve_reset_kernel_times(voce_rve *r)
{
    if (!r) return fail(VOCE_ERR_ARG, "null argument");
    for (int k = 0; k < K_COUNT; ++k) { r->prof.ms[k] = 0.0; r->prof.n[k] = 0; }
    return VOCE_OK;
}

long long voce_rve_kernel_launches(const voce_rve *r) { return r ? r->prof.launches : -1; }

int voce_rve_flush_l2(voce_rve *r, long long bytes)
{
    if (!r || bytes <= 0) return fail(VOCE_ERR_ARG, "bad argument");
    long long n = bytes / 8;
    if (n > r->flush_n) {
        if (r->d_flush) cudaFree(r->d_flush);
        r->d_flush = nullptr;
        CUDA_TRY(cudaMalloc(&r->d_flush, sizeof(double) * n));
        r->flush_n = n;
    }
    CUDA_TRY(launch_flush(r->d_flush, n, r->stream));
    r->prof.launches += 1;
    CUDA_TRY(cudaStreamSynchronize(r->stream));
    return VOCE_OK;
}

void *voce_host_alloc(long long bytes)
{
    void *p = nullptr;
    if (bytes <= 0 || cudaMallocHost(&p, (size_t)bytes) != cudaSuccess) return nullptr;
    return p;
}

void voce_host_free(void *p)
{
    if (p) cudaFreeHost(p);
}

double voce_measure_fp64_tflops(void) { return measure_fp64_tflops(); }

int voce_device_memory(long long *free_bytes, long long *total_bytes)
{
    size_t f = 0, t = 0;
    CUDA_TRY(cudaMemGetInfo(&f, &t));
    if (free_bytes) *free_bytes = (long long)f;
    if (total_bytes) *total_bytes = (long long)t;
    return VOCE_OK;
}

int voce_diag_rcp(const double *x, double *out, int n)
{
    if (n < 0 || (n > 0 && (!x || !out))) return fail(VOCE_ERR_ARG, "bad argument");
    if (n == 0) return VOCE_OK;
    double *d = nullptr;
    CUDA_TRY(cudaMalloc(&d, sizeof(double) * 2 * (size_t)n));
    cudaError_t e = cudaMemcpy(d, x, sizeof(double) * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = launch_rcp_probe(d, d + n, n, 0);
    if (e == cudaSuccess) e = cudaMemcpy(out, d + n, sizeof(double) * n, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return fail(VOCE_ERR_CUDA, "rcp probe: %s", cudaGetErrorString(e));
    return VOCE_OK;
}

int voce_diag_sqrt(const double *x, double *out, int n)
{
    if (n < 0 || (n > 0 && (!x || !out))) return fail(VOCE_ERR_ARG, "bad argument");
    if (n == 0) return VOCE_OK;
    double *d = nullptr;
    CUDA_TRY(cudaMalloc(&d, sizeof(double) * 2 * (size_t)n));
    cudaError_t e = cudaMemcpy(d, x, sizeof(double) * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = launch_sqrt_probe(d, d + n, n, 0);
    if (e == cudaSuccess) e = cudaMemcpy(out, d + n, sizeof(double) * n, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return fail(VOCE_ERR_CUDA, "sqrt probe: %s", cudaGetErrorString(e));
    return VOCE_OK;
}

int voce_diag_fft(int L, int nlines, int sign, int schedule, const double *in, double *out)
{
    if (nlines < 1 || (sign != 1 && sign != -1) || !in || !out) return fail(VOCE_ERR_ARG, "bad argument");
    FftPlan1 c[kMaxSchedules];
    const int n = axis_schedules(L, true, c, kMaxSchedules);
    if (schedule < 0 || schedule >= n) return fail(VOCE_ERR_ARG, "schedule %d of %d for length %d", schedule, n, L);
    if ((size_t)2 * L * (nlines | 1) * sizeof(float2) > 200 * 1024)
        return fail(VOCE_ERR_ARG, "%d lines of length %d do not fit in shared memory", nlines, L);
    const size_t bytes = sizeof(double) * 2 * (size_t)L * nlines;
    const auto tw = twiddles<float2, float>(L);
    char *buf = nullptr;
    CUDA_TRY(cudaMalloc(&buf, 2 * bytes + tw.size() * sizeof(float2)));
    double *din = reinterpret_cast<double *>(buf), *dout = reinterpret_cast<double *>(buf + bytes);
    void *dtw = buf + 2 * bytes;
    cudaError_t e = cudaMemcpy(din, in, bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dtw, tw.data(), tw.size() * sizeof(float2), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = launch_fft_probe(c[schedule], dtw, din, dout, nlines, sign, 0);
    if (e == cudaSuccess) e = cudaMemcpy(out, dout, bytes, cudaMemcpyDeviceToHost);
    cudaFree(buf);
    if (e != cudaSuccess) return fail(VOCE_ERR_CUDA, "fft probe: %s", cudaGetErrorString(e));
    return VOCE_OK;
}

}  // extern "C"

// ===========================================================================
// batches (voce_batch.h): many RVEs advanced together, one launch per phase
// ===========================================================================
struct voce_batch {
    int precision = 0;
    std::vector<voce_rve *> rves;
    cudaStream_t stream = nullptr;
    RveDesc *d_descs = nullptr;
    int2 *d_maps = nullptr;
    int *d_ctl = nullptr;   // ticks, max_ticks, active_out
    int *h_ctl = nullptr;   // pinned
    BatchPlan plan;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    bool dirty = true;
    bool inflight = false;   // ticks launched (voce_batch_launch) and not yet waited for
    long long ticks_total = 0;
    Prof prof;
    void drop_graph()
    {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        exec = nullptr;
        graph = nullptr;
    }
    void drop_plan()
    {
        drop_graph();
        if (d_descs) cudaFree(d_descs);
        if (d_maps) cudaFree(d_maps);
        d_descs = nullptr;
        d_maps = nullptr;
    }
    ~voce_batch()
    {
        if (stream) cudaStreamSynchronize(stream);
        drop_plan();
        if (d_ctl) cudaFree(d_ctl);
        if (h_ctl) cudaFreeHost(h_ctl);
        for (int k = 0; k < 2 * K_COUNT; ++k)
            if (prof.ev[k]) cudaEventDestroy(prof.ev[k]);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace {

int set_macro_flags(voce_rve *r, int active, int target, int pending)
{
    int v[3] = {active, pending, target};
    MacroDev *m = r->d.macro;
    CUDA_TRY(cudaMemcpyAsync(&m->active, &v[0], sizeof(int), cudaMemcpyHostToDevice, r->stream));
    CUDA_TRY(cudaMemcpyAsync(&m->pending_prelude, &v[1], sizeof(int), cudaMemcpyHostToDevice, r->stream));
    CUDA_TRY(cudaMemcpyAsync(&m->target, &v[2], sizeof(int), cudaMemcpyHostToDevice, r->stream));
    CUDA_TRY(cudaStreamSynchronize(r->stream));
    return VOCE_OK;
}

// descriptor array + per-phase work lists + the tick graph
int build_batch(voce_batch *b)
{
    VOCE_TRACE("build_batch");
    b->drop_plan();
    const int n = (int)b->rves.size();
    BatchPlan &p = b->plan;
    p = BatchPlan();
    p.nrve = n;
    p.mixed = b->precision != VOCE_PREC_FP64;
    p.nr32 = b->precision == VOCE_PREC_MIXED_NR32;
    p.ir = b->precision == VOCE_PREC_MIXED_IR;
    if (n == 0) { b->dirty = false; return VOCE_OK; }
    std::vector<RveDesc> descs(n);
    for (int i = 0; i < n; ++i) descs[i] = b->rves[i]->d;
    p.ticks = b->d_ctl;
    p.max_ticks = b->d_ctl + 1;
    p.active_out = b->d_ctl + 2;
    int rc = make_plan(descs, b->precision, b->d_descs, b->d_maps, p);
    if (rc) return rc;
    // graph: WHILE (any RVE active and ticks < max) { tick }
    cudaGraph_t g;
    CUDA_TRY(cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle h;
    CUDA_TRY(cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t cond;
    CUDA_TRY(cudaGraphAddNode(&cond, g, nullptr, nullptr, 0, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    CUDA_TRY(cudaStreamBeginCaptureToGraph(b->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = launch_batch_tick(p, b->stream, h);
    CUDA_TRY(cudaStreamEndCapture(b->stream, &body));
    CUDA_TRY(e);
    CUDA_TRY(cudaGraphInstantiate(&b->exec, g, 0));
    b->graph = g;
    b->dirty = false;
    return VOCE_OK;
}

}  // namespace

extern "C" {

int voce_batch_create(int precision, voce_batch **out)
{
    if (!out) return fail(VOCE_ERR_ARG, "null argument");
    voce_batch *b = new voce_batch();
    if (precision < VOCE_PREC_FP64 || precision > VOCE_PREC_MIXED_IR) {
        delete b;
        return fail(VOCE_ERR_ARG, "unknown precision %d", precision);
    }
    b->precision = precision;
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_ctl, 4 * sizeof(int));
    if (e == cudaSuccess) e = cudaMallocHost(&b->h_ctl, 4 * sizeof(int));
    if (e != cudaSuccess) {
        delete b;
        return fail(VOCE_ERR_CUDA, "batch setup: %s", cudaGetErrorString(e));
    }
    *out = b;
    return VOCE_OK;
}

int voce_batch_add(voce_batch *b, voce_rve *r, int n_increments)
{
    if (!b || !r || n_increments < 1 || n_increments > (1 << 24)) return fail(VOCE_ERR_ARG, "bad argument");
    if (r->batch) return fail(VOCE_ERR_STATE, "the RVE already belongs to a batch");
    if (r->precision != b->precision) return fail(VOCE_ERR_ARG, "precision differs from the batch's");
    int rc = ensure_ring(r, n_increments + 1);
    if (rc) return rc;
    // at an increment boundary the next prelude is pending; an RVE taken out
    // of a batch in the middle of an increment continues that increment
    // (it counts as the first of the n)
    MacroDev m;
    CUDA_TRY(cudaStreamSynchronize(r->stream));
    CUDA_TRY(cudaMemcpy(&m, r->d.macro, sizeof(m), cudaMemcpyDeviceToHost));
    rc = set_macro_flags(r, 1, r->n_done + n_increments, m.iter != 0 ? 0 : 1);
    if (rc) return rc;
    r->batch = b;
    b->rves.push_back(r);
    b->dirty = true;
    return VOCE_OK;
}

static int batch_finish(voce_batch *b, int *active_left);

int voce_batch_remove(voce_batch *b, voce_rve *r)
{
    if (!b || !r || r->batch != b) return fail(VOCE_ERR_ARG, "the RVE is not in this batch");
    if (b->inflight) {
        int rc = batch_finish(b, nullptr);
        if (rc) return rc;
    }
    MacroDev m;
    CUDA_TRY(cudaStreamSynchronize(b->stream));
    CUDA_TRY(cudaMemcpy(&m, r->d.macro, sizeof(m), cudaMemcpyDeviceToHost));
    int rc = collect_new(r, false);
    if (rc) return rc;
    // between increments the next increment's prelude has not run yet; in
    // the middle of one it has, and the increment goes on where it stopped
    rc = set_macro_flags(r, 1, 0x7fffffff, m.iter != 0 ? 0 : 1);
    if (rc) return rc;
    b->rves.erase(std::find(b->rves.begin(), b->rves.end(), r));
    r->batch = nullptr;
    b->dirty = true;
    return VOCE_OK;
}

int voce_batch_size(const voce_batch *b) { return b ? (int)b->rves.size() : -1; }

// Enqueue up to max_ticks ticks on the batch stream and return: the graph
// (or, with profiling, the host-driven ticks, which wait for themselves)
// and the copy of the tick counters back to pinned host memory.
static int batch_launch(voce_batch *b, int max_ticks)
{
    VOCE_TRACE("voce_batch_launch");
    for (voce_rve *r : b->rves) CUDA_TRY(cudaStreamSynchronize(r->stream));
    if (b->dirty) {
        int rc = build_batch(b);
        if (rc) return rc;
    }
    if (b->rves.empty()) {
        b->h_ctl[0] = 0;
        b->h_ctl[2] = 0;
        b->inflight = true;
        return VOCE_OK;
    }
    b->h_ctl[0] = 0;
    b->h_ctl[1] = max_ticks;
    b->h_ctl[2] = 0;
    CUDA_TRY(cudaMemcpyAsync(b->d_ctl, b->h_ctl, 3 * sizeof(int), cudaMemcpyHostToDevice, b->stream));
    if (b->prof.on) {
        // host-driven ticks with every launch timed; stops where the graph's
        // WHILE condition would
        for (int t = 0; t < max_ticks; ++t) {
            CUDA_TRY(launch_batch_tick_timed(b->plan, b->stream, b->prof));
            CUDA_TRY(cudaMemcpyAsync(b->h_ctl, b->d_ctl, 3 * sizeof(int), cudaMemcpyDeviceToHost, b->stream));
            CUDA_TRY(cudaStreamSynchronize(b->stream));
            b->prof.collect();
            if (b->h_ctl[2] == 0) break;
        }
    } else {
        CUDA_TRY(cudaGraphLaunch(b->exec, b->stream));
        CUDA_TRY(cudaMemcpyAsync(b->h_ctl, b->d_ctl, 3 * sizeof(int), cudaMemcpyDeviceToHost, b->stream));
    }
    b->inflight = true;
    return VOCE_OK;
}

// Wait for the launched ticks and take in the increment records they made.
static int batch_finish(voce_batch *b, int *active_left)
{
    VOCE_TRACE("voce_batch_wait");
    if (!b->inflight) {
        if (active_left) *active_left = b->rves.empty() ? 0 : b->h_ctl[2];
        return VOCE_OK;
    }
    b->inflight = false;
    CUDA_TRY(cudaStreamSynchronize(b->stream));
    CUDA_TRY(cudaGetLastError());
    b->ticks_total += b->h_ctl[0];
    for (voce_rve *r : b->rves) {
        // RVEs added after the launch have no new records yet
        int rc = collect_new(r, false);
        if (rc) return rc;
        // launches of a tick are counted per batch, not per RVE
    }
    if (active_left) *active_left = b->h_ctl[2];
    return VOCE_OK;
}

int voce_batch_launch(voce_batch *b, int max_ticks)
{
    if (!b || max_ticks < 1) return fail(VOCE_ERR_ARG, "bad argument");
    if (b->inflight) {
        int rc = batch_finish(b, nullptr);
        if (rc) return rc;
    }
    return batch_launch(b, max_ticks);
}

int voce_batch_wait(voce_batch *b, int *active_left)
{
    if (!b) return fail(VOCE_ERR_ARG, "null argument");
    return batch_finish(b, active_left);
}

int voce_batch_run(voce_batch *b, int max_ticks, int *active_left)
{
    int rc = voce_batch_launch(b, max_ticks);
    if (rc) return rc;
    return batch_finish(b, active_left);
}

long long voce_batch_ticks(const voce_batch *b) { return b ? b->ticks_total : -1; }

int voce_batch_set_profiling(voce_batch *b, int on)
{
    if (!b) return fail(VOCE_ERR_ARG, "null argument");
    if (on && !b->prof.ev[0])
        for (int k = 0; k < 2 * K_COUNT; ++k) CUDA_TRY(cudaEventCreate(&b->prof.ev[k]));
    b->prof.on = on != 0;
    return VOCE_OK;
}

int voce_batch_get_kernel_time(const voce_batch *b, int k, double *ms, long long *launches)
{
    if (!b || k < 0 || k >= K_COUNT) return fail(VOCE_ERR_ARG, "bad argument");
    if (ms) *ms = b->prof.ms[k];
    if (launches) *launches = b->prof.n[k];
    return VOCE_OK;
}

int voce_batch_reset_kernel_times(voce_batch *b)
{
    if (!b) return fail(VOCE_ERR_ARG, "null argument");
    for (int k = 0; k < K_COUNT; ++k) {
        b->prof.ms[k] = 0.0;
        b->prof.n[k] = 0;
    }
    return VOCE_OK;
}

int voce_batch_destroy(voce_batch *b)
{
    if (!b) return VOCE_OK;
    if (b->inflight) batch_finish(b, nullptr);
    if (b->stream) cudaStreamSynchronize(b->stream);
    for (voce_rve *r : b->rves) {
        collect_new(r, false);
        MacroDev m;
        const bool mid = cudaMemcpy(&m, r->d.macro, sizeof(m), cudaMemcpyDeviceToHost) == cudaSuccess &&
                         m.iter != 0;
        set_macro_flags(r, 1, 0x7fffffff, mid ? 0 : 1);
        r->batch = nullptr;
    }
    delete b;
    return VOCE_OK;
}

}  // extern "C"
