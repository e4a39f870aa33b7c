// polish.cu -- final passes of the fast method in compensated FP32.
//
// The double-float lane passes (lanedf.cuh) cost ~110 FP32 instructions per
// grid point and no FP64 instruction, against ~16 FP64 instructions (~1000
// FP32-issue equivalents on GB300) for the same pass in native FP64.
//
//  newton_df : Cooley corrections from the FP32 energy (one or two passes) in
//              an FP64 count bracket; levels that do not settle go to the
//              CTA-per-level Newton of longwin.cu (the fallback), which also
//              takes their norm and write passes.
//  norm_df   : sums, node count, peak of |psi| and the constants of the
//              write; with psi requested its final pass also stores the
//              unnormalised psi-hat in the level's row as tagged float pairs
//              (dfpass.cuh), and
//  scale_psi : turns them into the normalised doubles (one HBM pass over the
//              windows, no FP64 instruction per point).
//  (the twist-index search for the levels norm_df flags is twist_long in
//  longwin.cu, one CTA per level)
//  write_df  : recomputes psi from the stored constants (the adjoint's
//              recompute path).
//
// (Measured on GB300: one persistent kernel running refine32, newton_df and
// norm_df back to back per unit was slower, 36.8 against 31.4 ms a step on
// the 2048-potential batch.  Each stage's duration is the serial march of the
// same longest units, so fusing saves no tail; it holds the SMs for the whole
// lane branch and shuts out the CTA branch that runs beside it.)
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "common.cuh"
#include "dfloat.cuh"
#include "dfpass.cuh"
#include "launch.h"
#include "lane32.cuh"
#include "lanedf.cuh"

namespace epscu {

namespace {

constexpr int kThreads = 128;

__global__ void __launch_bounds__(kLaneThreads, kLaneCtasPerSm) newton_df_kernel(DevBatch b) {
    for (int2 unit; next_unit(b, kQNewtonDF, unit);) {
        if ((int)(threadIdx.x & 31) >= unit.y) continue;
        newton_df_level(b, unit.x + (threadIdx.x & 31));
    }
}

__global__ void __launch_bounds__(kLaneThreads, kLaneCtasPerSm) norm_df_kernel(DevBatch b) {
    for (int2 unit; next_unit(b, kQNormDF, unit);) {
        if ((int)(threadIdx.x & 31) >= unit.y) continue;
        norm_df_level(b, unit.x + (threadIdx.x & 31));
    }
}

__global__ void __launch_bounds__(kThreads, 4) write_df_kernel(DevBatch b) {
    if (!b.psi || b.hdr->error) return;
    const int lane = threadIdx.x & 31;
    for (int2 unit; next_unit(b, kQWriteDF, unit);) {
        // zeros outside each level's window (the whole row of a level without a
        // result), stored by the whole warp with coalesced stores
        for (int u = 0; u < unit.y; ++u) {
            const LevelWork wu = b.levels[unit.x + u];
            if (is_long(wu)) continue;  // written by write_long
            const int N = b.meta[wu.p].N;
            double* row = b.psi + b.meta[wu.p].psi_off + (int64_t)(wu.v - b.min_level) * N;
            const bool none = no_result(wu);
            const int a = none ? N : wu.j0;
            for (int i = lane; i < a; i += 32) row[i] = 0.0;
            if (!none)
                for (int i = wu.j1 + 1 + lane; i < N; i += 32) row[i] = 0.0;
        }
        if (lane >= unit.y) continue;
        const int slot = unit.x + lane;
        const LevelWork w = b.levels[slot];
        if (no_result(w) || is_long(w) || (w.status & EPSCU_STATUS_FALLBACK)) continue;
        const PotMeta m = b.meta[w.p];
        double* out = b.psi + m.psi_off + (int64_t)(w.v - b.min_level) * m.N;
        const float2* Wf = b.Wf2 + m.offf;
        const dfl aE = energy_df(m, w.E);
        SideDF<2> st;
        side_df<2>(Wf, aE, w.j0, w.k, +1, st, out, w.norm_k_out, w.ex_out);
        side_df<2>(Wf, aE, w.j1, w.k, -1, st, out, w.norm_k_in, w.ex_in);
        out[w.k] = w.ck;
    }
}

// Zeros of the psi rows outside each level's window (the whole row of a
// level that has no result yet), run beside the compute-bound refinement
// kernels.  The windows are final once the window kernel has run; their
// points are written by the norm passes and scale_psi, so every point of a
// row is written once by one of the two (the window is ~a fifth of the row
// on the mixed batch).  One warp per level, coalesced stores.
__global__ void __launch_bounds__(256) zero_psi_kernel(DevBatch b) {
    if (!b.psi || b.hdr->error) return;
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int n_warps = (gridDim.x * blockDim.x) >> 5;
    const int total = b.hdr->total_levels;
    unsigned long long zeroed = 0;
    for (int slot = warp; slot < total; slot += n_warps) {
        const LevelWork w = b.levels[slot];
        const PotMeta m = b.meta[w.p];
        const int N = m.N;
        double* row = b.psi + m.psi_off + (int64_t)(w.v - b.min_level) * N;
        const bool none = no_result(w);
        const int a = none ? N : w.j0, c = none ? N : w.j1 + 1;
        for (int i = lane; i < a; i += 32) row[i] = 0.0;
        for (int i = c + lane; i < N; i += 32) row[i] = 0.0;
        zeroed += (unsigned long long)(a + (N - c));
    }
    if (lane == 0 && zeroed) atomicAdd(&b.hdr->psi_zero_points, zeroed);
}

// The write-back of the fused norm/write: each row holds the unnormalised
// psi-hat of the level's final norm pass (norm_df, norm_long or twist_long)
// on [j0, k) and (k, j1] as scaled float pairs; scale it by the
// side constants (norm_k 2^-ex) and set psi_k = ck.  The rest of the row was
// zeroed by zero_psi; the window of a level left without a result is zeroed
// here.  One warp per level, coalesced: HBM-bound (8 B read + 8 B written per
// window point).
__global__ void __launch_bounds__(256) scale_psi_kernel(DevBatch b) {
    if (!b.psi || b.hdr->error) return;
    __shared__ int s_slot;
    const int total = b.hdr->total_levels;
    unsigned long long converted = 0;
    // levels from a device queue, one CTA each: the windows range from a few
    // hundred to ~6.5e4 points, and a warp per level handed out round-robin
    // left the SMs busy only ~40% of the kernel (ncu)
    for (;;) {
        if (threadIdx.x == 0) s_slot = atomicAdd(&b.hdr->queue[kQScalePsi], 1);
        __syncthreads();
        const int slot = s_slot;
        __syncthreads();  // every thread has read s_slot
        if (slot >= total) break;
        const LevelWork w = b.levels[slot];
        const PotMeta m = b.meta[w.p];
        double* row = b.psi + m.psi_off + (int64_t)(w.v - b.min_level) * m.N;
        if (no_result(w)) {
            for (int i = w.j0 + (int)threadIdx.x; i <= w.j1; i += blockDim.x) row[i] = 0.0;
            continue;
        }
        if (threadIdx.x == 0) converted += (unsigned long long)(w.j1 - w.j0 + 1);
        // the side constants norm_k 2^-ex as m 2^e, m in [0.5, 1) a
        // double-float: per point the pair times m in double-float and the
        // double assembled with integer operations, scaled by 2^(64 r + e)
        // in its exponent bits (no FP64 instruction per point)
        int e_out, e_in;
        const dfl M_out = df_from_double(frexp(w.norm_k_out, &e_out));
        const dfl M_in = df_from_double(frexp(w.norm_k_in, &e_in));
        e_out -= w.ex_out;
        e_in -= w.ex_in;
        const float2* pair = reinterpret_cast<const float2*>(row);
        auto convert = [&](int i, float2 raw) {
            int r;
            const dfl v = load_psi_pair(raw, r);
            const bool outward = i < w.k;
            const dfl p = df_mul(v, outward ? M_out : M_in);
            return i == w.k ? w.ck : df_pair_to_double_scaled(p.h, p.l, 64 * r + (outward ? e_out : e_in));
        };
        // four points per thread per step (four loads in flight), the CTA's
        // 256 threads coalesced over the window
        constexpr int kS = 256;
        int i = w.j0 + (int)threadIdx.x;
        for (; i + 3 * kS <= w.j1; i += 4 * kS) {
            const float2 r0 = pair[i], r1 = pair[i + kS], r2 = pair[i + 2 * kS], r3 = pair[i + 3 * kS];
            row[i] = convert(i, r0);
            row[i + kS] = convert(i + kS, r1);
            row[i + 2 * kS] = convert(i + 2 * kS, r2);
            row[i + 3 * kS] = convert(i + 3 * kS, r3);
        }
        for (; i <= w.j1; i += kS) row[i] = convert(i, pair[i]);
    }
    if (threadIdx.x == 0 && converted) atomicAdd(&b.hdr->psi_window_points, converted);
}

}  // namespace

void launch_zero_psi(const DevBatch& b, int sm_count, cudaStream_t s) {
    zero_psi_kernel<<<sm_count * 8, 256, 0, s>>>(b);
}

void launch_scale_psi(const DevBatch& b, int sm_count, cudaStream_t s) {
    scale_psi_kernel<<<sm_count * 8, 256, 0, s>>>(b);
}

void launch_newton_df(const DevBatch& b, int sm_count, cudaStream_t s) {
    newton_df_kernel<<<sm_count * kLaneCtasPerSm, kLaneThreads, 0, s>>>(b);
}
void launch_norm_df(const DevBatch& b, int sm_count, cudaStream_t s) {
    norm_df_kernel<<<sm_count * kLaneCtasPerSm, kLaneThreads, 0, s>>>(b);
}
void launch_write_df(const DevBatch& b, int sm_count, cudaStream_t s) {
    write_df_kernel<<<sm_count * 8, kThreads, 0, s>>>(b);
}

}  // namespace epscu
