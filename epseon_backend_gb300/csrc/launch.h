// launch.h -- host-side launchers of the libepseon_cuda kernels (one per
// translation unit), called by the orchestration in epscu.cu.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "common.cuh"

namespace epscu {

struct DevBatch {
    int32_t n;                 // potentials
    PotMeta* meta;             // [n]
    const double* V64;         // concatenated potentials
    double* W64;               // a V (FP64)
    double* Msuf;              // suffix minima of V on i0..i1
    double* Mpre;              // prefix minima of V on i0..i1 (fast method), or nullptr
    float* Bmin;               // minima of W over 32-point blocks (index offf / 32 + block; fast method)
    float2* Wf2;               // a V as (hi, lo) floats, tile-aligned per potential
    int32_t* counts;           // [n * n_trial]
    float* gam;                // [n * n_trial] the scan's matching function f_k gamma_k at the counted trial
                               // energies (fast method: the refinement's first energy), or nullptr
    LevelWork* levels;         // [max_levels]
    int32_t* fallback_list;    // [max_levels] slots handed to the bisection fallback
    int2* units;               // [max_units] (first slot, count) per warp work unit
    int32_t max_units;
    int32_t* twist_list;       // [max_twist] slots for the twist-index search
    double* twist_scratch;     // [max_twist * twist_stride] sampled outward ratios
    int32_t max_twist, twist_stride;
    int32_t max_levels;        // capacity of levels (n * level_capacity)
    int32_t level_capacity;    // slots per potential
    Header* hdr;
    int32_t* order;            // [n] potentials by decreasing cost
    int2* scan_win;            // [n * ceil(n_trial / kScanWinBlock)] scan windows, or nullptr (full grid)
    int32_t* long_list;        // [max_levels] slots with long windows (CTA-per-level passes), or nullptr
    int32_t* mid_list;         // [max_levels] slots with middle windows (warp-per-level passes), or nullptr
    int32_t* bis_list;         // [n * n_trial] trial indices of the bisection scan's current round, or
                               // nullptr (every trial energy scanned)
    int32_t* bis_n;            // [n] entries of bis_list per potential
    int2* bis_items;           // [max_bis_items] (potential, first entry) chunks of a bisection round
    int32_t max_bis_items;
    double* psi;               // compact wavefunctions or nullptr
    int64_t psi_capacity;
    volatile int32_t* cancel;  // host-mapped cancel flag (device pointer) or nullptr
    int32_t n_trial;
    int32_t min_level, max_level;
    int32_t max_N;             // longest grid of the batch
    int32_t long_window;       // window length above which a level takes the CTA passes
    int32_t mid_window;        // window length above which a level takes the warp passes (< 0: none)
    int32_t wait_polls;        // polls of a bounded wait on a staged scan tile (0: kWaitPolls)
    int32_t max_iter;          // cap on FP32 refinement passes (0: 48; fallback passes: twice it)
    double tol;
};

constexpr int kWaitPolls = 1 << 22;       // default bound of the TMA scan's mbarrier waits
// persistent grid of the lane-per-level kernels (refine32, newton_df,
// norm_df): threads per CTA and CTAs per SM launched (together 512 threads at
// up to 128 registers, the whole register file)
constexpr int kLaneThreads = 128;
constexpr int kLaneCtasPerSm = 4;
constexpr int kRefineMaxIter = 48;        // default cap on a level's FP32 refinement passes
__device__ __forceinline__ int refine_cap(const DevBatch& b) { return b.max_iter > 0 ? b.max_iter : kRefineMaxIter; }
// double-float fallback passes (bisection from the widened scan bracket)
__device__ __forceinline__ int fallback_cap(const DevBatch& b) { return 2 * refine_cap(b); }

// Warp-level work queue of the per-level kernels: units of up to 32
// consecutive level slots of one potential, longest grids first.  Lane 0
// takes the next unit and broadcasts it; false when the queue is drained.
// (Measured slower on the mixed batch: units of levels sorted by window
// length across potentials, and a lane-level state machine that hands each
// lane a new level as soon as it finishes -- its divergent bookkeeping costs
// more than the idle lanes it saves.)
__device__ __forceinline__ bool next_unit(const DevBatch& b, int qid, int2& unit) {
    int u = 0;
    if ((threadIdx.x & 31) == 0) u = atomicAdd(&b.hdr->queue[qid], 1);
    u = __shfl_sync(0xffffffffu, u, 0);
    if (u >= b.hdr->n_units || u >= b.max_units) return false;
    unit = b.units[u];
    return true;
}


// prepare.cu
void launch_prepare(const DevBatch& b, cudaStream_t s);
void launch_level_setup(const DevBatch& b, cudaStream_t s);
void launch_window(const DevBatch& b, int sm_count, cudaStream_t s);
void launch_scan_window(const DevBatch& b, int sm_count, cudaStream_t s);
void launch_tabulate(int32_t n, const int32_t* kind, const double* params, const int64_t* offsets,
                     const int32_t* N, const double* r_min, const double* r_max, int32_t n_knots,
                     double* knot_scratch, double* V, cudaStream_t s);

void launch_tabulate_adjoint(int32_t n, const int32_t* kind, const double* params, const int64_t* offsets,
                             const int32_t* N, const double* r_min, const double* r_max, int32_t n_knots,
                             double* knot_scratch, const double* gV, double* gP, cudaStream_t s);

// scan.cu
void launch_scan64(const DevBatch& b, cudaStream_t s);
struct ScanShape {
    int threads;      // threads per CTA (energies per CTA = threads)
    int tile;         // floats2 per TMA stage
    int stages;
    int ctas_per_sm;  // persistent grid = sm_count * ctas_per_sm
};
void launch_scan32(const DevBatch& b, const ScanShape& shape, int sm_count, cudaStream_t s, int stride = 1);
void launch_bisect_scan(const DevBatch& b, const ScanShape& shape, int sm_count, cudaStream_t s);
int64_t bisect_max_items(int n, int n_trial);  // capacity of DevBatch::bis_items
int scan32_max_tile();
void scan32_set_attributes();

// levels.cu
void launch_bisect64(const DevBatch& b, int sm_count, cudaStream_t s);
void launch_refine32(const DevBatch& b, int sm_count, cudaStream_t s);
void launch_norm64(const DevBatch& b, int use_k, int sm_count, cudaStream_t s);
void launch_write64(const DevBatch& b, int sm_count, cudaStream_t s);
void launch_gather(const DevBatch& b, int32_t* n_total, int32_t* n_out, double* energy, int32_t* nodes,
                   int32_t* status, double* err_est, int apply_dE, cudaStream_t s);

// polish.cu (fast method: compensated-FP32 recurrence, FP64 matching and norm)
void launch_newton_df(const DevBatch& b, int sm_count, cudaStream_t s);
void launch_norm_df(const DevBatch& b, int sm_count, cudaStream_t s);
void launch_write_df(const DevBatch& b, int sm_count, cudaStream_t s);
void launch_scale_psi(const DevBatch& b, int sm_count, cudaStream_t s);
void launch_zero_psi(const DevBatch& b, int sm_count, cudaStream_t s);
void launch_twist64(const DevBatch& b, int sm_count, cudaStream_t s);

// longwin.cu
void launch_refine_long(const DevBatch& b, int sm_count, cudaStream_t s);
void launch_fallback_long(const DevBatch& b, int sm_count, cudaStream_t s);
void launch_norm_long(const DevBatch& b, int sm_count, cudaStream_t s);
void launch_write_long(const DevBatch& b, int sm_count, cudaStream_t s);
void launch_twist_long(const DevBatch& b, int sm_count, cudaStream_t s);
void launch_norm_fallback(const DevBatch& b, int sm_count, cudaStream_t s);
void launch_refine_mid(const DevBatch& b, int sm_count, cudaStream_t s);
void launch_norm_mid(const DevBatch& b, int sm_count, cudaStream_t s);

// adjoint.cu
// points per CTA of the adjoint (one thread each)
constexpr int kAdjointPoints = 256;
void launch_adjoint(const DevBatch& b, const double* dL_dE, double* dL_dV, const int64_t* offsets_dev,
                    const int32_t* tiles_dev, int32_t n_tiles, cudaStream_t s);

void launch_adjoint_explicit(int32_t n, int32_t cap, int32_t max_N, const int64_t* offsets, const int32_t* N,
                             const double* h, const int32_t* n_out, const int64_t* psi_off, const double* psi,
                             const double* gE, double* gV, cudaStream_t s);

// epscu.cu: the calling thread's message for epscu_last_error()
void set_last_error(const std::string& msg);

// peaks.cu
void measure_fma_peaks(int sm_count, double* fp32_tflops, double* fp64_tflops);

}  // namespace epscu
