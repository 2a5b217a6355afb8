// Host-side declarations of the kernel launchers (voce_kernels.cu).
#pragma once
#include "voce_dev.cuh"

namespace voce {

// Constants used only by the setup and increment-end kernels.
struct SetupConst {
    double cxt[36], sxt[36];  // crystal stiffness / compliance, 6-vector basis
    double d6[6];             // B-basis sym(DisGradAvg) at t=0 (init.c:495-499)
    double sc6[6];            // B-basis Scauchy (creep start stress, init.c:523-525)
};

// FFT tile sizes (lines per block) for one grid, and the radix schedule of
// each axis (an index into fft_schedules' candidates of that axis' length)
struct Tiles {
    int zrows, yxt, xkc, xkc3, zirows, zirows3;
    int sx = 0, sy = 0, sz = 0;
    template <typename R> void choose(const RveDesc &d);
};

// Per-kernel timing: when `on`, an event pair brackets every launch of the
// listed kernels; the host reads them after the stream synchronises.
enum KernelId {
    K_FFT_Z_FWD = 0, K_FFT_Y_FWD, K_FFT_X_GREEN, K_FFT_Y_INV, K_FFT_Z_INV, K_NR, K_FIN_ITER,
    K_PRELUDE, K_INC_FFT, K_INCR_END, K_FIN_INCR, K_COUNT
};
struct Prof {
    bool on = false;
    cudaEvent_t ev[2 * K_COUNT] = {};
    bool pending[K_COUNT] = {};
    double ms[K_COUNT] = {};
    long long n[K_COUNT] = {};
    long long launches = 0;   // kernels issued, counted whether or not timing is on
    void begin(int k, cudaStream_t s) { if (on) cudaEventRecord(ev[2 * k], s); }
    void end(int k, cudaStream_t s, int count = 1)
    {
        launches += count;
        if (on) { cudaEventRecord(ev[2 * k + 1], s); pending[k] = true; }
    }
    void collect()   // after a stream synchronisation
    {
        for (int k = 0; k < K_COUNT; ++k)
            if (pending[k]) {
                float t = 0.f;
                cudaEventElapsedTime(&t, ev[2 * k], ev[2 * k + 1]);
                ms[k] += t;
                n[k] += 1;
                pending[k] = false;
            }
    }
};


// Work lists of one batch (device memory): per phase, (rve, unit) pairs.
enum BatchPhase {
    BP_NP = 0,   // Newton / increment-end / prelude units (npart per RVE)
    BP_ZF, BP_Y6, BP_XG, BP_ZI, BP_X3, BP_Y3, BP_Z3, BP_COUNT
};
struct BatchPlan {
    const RveDesc *descs = nullptr;   // device array [nrve]
    int nrve = 0;
    const int2 *map[BP_COUNT] = {};
    int total[BP_COUNT] = {};
    size_t smem[BP_COUNT] = {};       // dynamic shared memory of the FFT phases
    int *ticks = nullptr, *max_ticks = nullptr, *active_out = nullptr;
    bool mixed = false;   // float spectrum
    bool nr32 = false;    // float Newton iterations (kb_nr<true>)
    bool ir = false;      // FP64-residual Newton with a float Jacobian
    int ystream = 0;      // > 0: every RVE runs the register FFT along y; the y
                          // pass streams its units through two tile buffers of
                          // this many complex floats
};
// units of one RVE in each phase
void batch_units(const RveDesc &d, int units[BP_COUNT]);
size_t batch_smem(const RveDesc &d, int phase);
cudaError_t set_batch_smem(const BatchPlan &bp);
// one forward-pass FFT phase (BP_ZF, BP_Y6 forward, BP_XG, BP_ZI) alone, for
// tile tuning
cudaError_t launch_plan_phase(const BatchPlan &bp, int phase, cudaStream_t s);
// tile sizes worth trying for that phase of d (distinct, fitting in shared
// memory); returns how many were written to out
int tile_candidates(const RveDesc &d, int phase, int *out, int max);
// one tick: prelude (pending), one Green iteration of every active RVE, the
// increment end of every RVE that converged, the loop condition
cudaError_t launch_batch_tick(const BatchPlan &bp, cudaStream_t s, cudaGraphConditionalHandle cond);
// the same tick outside a graph, every launch bracketed by pf's events
cudaError_t launch_batch_tick_timed(const BatchPlan &bp, cudaStream_t s, Prof &pf);
// The phases of a plan (a lone RVE runs as a plan of one, with the same
// kernels as any batch): prelude; one Green iteration, whose finaliser sets
// the WHILE condition when use_cond; the increment end.
cudaError_t launch_plan_prelude(const BatchPlan &bp, cudaStream_t s, Prof &pf);
cudaError_t launch_plan_iteration(const BatchPlan &bp, cudaStream_t s, Prof &pf,
                                  cudaGraphConditionalHandle cond, int use_cond);
cudaError_t launch_plan_incr_end(const BatchPlan &bp, cudaStream_t s, Prof &pf);
cudaError_t launch_flush(double *buf, long long n, cudaStream_t s);
// periodic Voronoi labels of an nx x ny x nz grid (synthetic microstructures)
#define VORONOI_TILE 1024
cudaError_t launch_voronoi(int nx, int ny, int nz, int ns, const double *seeds, int *label, cudaStream_t s);
// the FP64 form's stored Green-operator frequencies, once Kq is set in d
cudaError_t launch_fill_green(const RveDesc &d, cudaStream_t s);
// the mixed form's float (S_g + S0), once S0 is set in d
cudaError_t launch_fill_p32(const RveDesc &d, cudaStream_t s);
// Newton-kernel instance of a precision form: 0 FP64 Newton (FP64 and
// mixed forms), 1 FP32 Newton (mixed_nr32), 2 FP64 residual with an FP32
// Jacobian (mixed_ir)
inline int nr_kind(int precision) { return precision == 2 ? 1 : precision == 3 ? 2 : 0; }
// kb_nr blocks resident on the current GPU (SMs x blocks per SM) for an
// instance of nr_kind
int nr_resident_blocks(int kind);
double measure_fp64_tflops();
// out[i] = rcp_nr(x[i]) for i < n (device arrays)
cudaError_t launch_rcp_probe(const double *x, double *out, int n, cudaStream_t s);
cudaError_t launch_sqrt_probe(const double *x, double *out, int n, cudaStream_t s);
// nl lines of length pl.L through the single-precision line FFT (one block;
// 2 L (nl | 1) complex floats of shared memory): in, out [nl][L] complex
// doubles on the device, tw the length's float twiddles
cudaError_t launch_fft_probe(const FftPlan1 &pl, const void *tw, const double *in, double *out, int nl, int sign,
                             cudaStream_t s);
cudaError_t launch_setup(const RveDesc &d, const SetupConst &sc, const double *euler, int npart,
                         cudaStream_t s);
cudaError_t launch_field_out(const RveDesc &d, int field, double *out, cudaStream_t s);
// displacement fluctuation of d's DisGrad into out[3 * v + i], through a work
// array of disp_work_bytes(d) (its contents on entry do not matter)
size_t disp_work_bytes(const RveDesc &d);
cudaError_t launch_disp_fluct(const RveDesc &d, void *work, double *out, cudaStream_t s);

}  // namespace voce
