// dfpass.cuh -- pieces shared by the double-float passes of the fast method
// (polish.cu: one lane per level; longwin.cu: one CTA per long level).
#pragma once

#include <math.h>

#include "common.cuh"
#include "dfloat.cuh"
#include "launch.h"

namespace epscu {

// Windows longer than a threshold take the CTA-per-level passes of
// longwin.cu (parallel prefix over chunks) instead of one lane per level.  A
// lane marching a long window is the tail of the per-level kernels: its
// latency, not the throughput, sets their duration; the CTA passes cost ~3x
// the point-updates in double-float but cut the latency ~80x.  So the
// threshold falls with the number of levels (fewer lanes to keep the GPU
// busy): 8192 points at >= ~9e4 levels (the 2048-potential mixed batch),
// proportionally less below, never under 1024.  Measured on GB300 with the
// long levels on their own stream beside the lane kernels and FP32 passes on
// the CTA path: the 2048-potential batch (93k levels) is fastest at 8192, the
// 256-potential bump batch (14k levels) at 2048, the 64-Morse batch (3.4k
// levels) at 1024-1536.  With the fallback levels and the psi zeroing on the
// long levels' stream the 2048-potential batch measured 28.6 / 27.4 / 27.2 /
// 27.3 ms a step at 6144 / 8192 / 10240 / 12288 points (flat from 8192 up).
// DevBatch::long_window > 0 overrides it.
constexpr int kLongWindow = 8192;
constexpr int kLongWindowLevels = 60000;
constexpr int kMinLongWindow = 1024;
// windows above this many points (and up to the long-window threshold) can
// run their double-float passes one warp per level, after the lane FP32
// refinement (DevBatch::mid_window > 0).  Off by default: on the
// 2048-potential batch the warp passes (three marches of a chunked pass per
// point) cost as much as the lane passes they replace (9 against 10 ms), and
// the step was not shorter at thresholds of 1024 or 4096 points.
constexpr int kMidWindow = -1;

__host__ __device__ __forceinline__ int default_long_window(int total_levels) {
    int w = kMinLongWindow;
    while (w < kLongWindow && (long long)w * kLongWindowLevels < (long long)kLongWindow * total_levels) w <<= 1;
    return w;
}

// the level runs its double-float passes on a group of warps (CTA or warp
// per level), not on a lane
__device__ __forceinline__ bool is_long(const LevelWork& w) {
    return (w.status & (EPSCU_STATUS_LONG | EPSCU_STATUS_MID)) != 0;
}

// match points stay inside the level's window, off its two end points
__device__ __forceinline__ int clamp_k(const LevelWork& w, int k) { return max(w.j0 + 1, min(k, w.j1 - 1)); }

__device__ __forceinline__ dfl energy_df(const PotMeta& m, double E) {
    return df_from_double(__dmul_rn(m.a, E));
}

struct PassDF {
    double dE, gamma, sum;
    double pk_out, pk_in;
    int ex_out, ex_in;
    int nodes, count;
    int peak_i, peak_log2;
};

// Write the normalisation constants of pass r (match point k) into w.
__device__ __forceinline__ void finalize_df(const PotMeta& m, LevelWork& w, const PassDF& r, int k) {
    double ck = 1.0 / sqrt(m.h * r.sum);
    if (r.pk_out < 0.0) ck = -ck;  // psi > 0 next to the inner wall
    w.k = k;
    w.ck = ck;
    w.norm_k_out = ck / r.pk_out;
    w.norm_k_in = ck / r.pk_in;
    w.ex_out = r.ex_out;
    w.ex_in = r.ex_in;
    w.dE = r.dE;
    w.nodes = r.nodes;
    w.status &= ~EPSCU_STATUS_NOTFOUND;
    if (!isfinite(r.dE) || !isfinite(ck)) w.status |= EPSCU_STATUS_NONFINITE;
    if (r.nodes != w.v && !(m.status & EPSCU_STATUS_UNDER)) w.status |= EPSCU_STATUS_NOTFOUND;
}

// a converged level whose final pass disagrees (node count, or a Cooley
// correction far above the energy's accuracy) was matched at a poor point
__device__ __forceinline__ bool suspicious(const PotMeta& m, const LevelWork& w, int nodes, double dE) {
    return (nodes != w.v && !(m.status & EPSCU_STATUS_UNDER)) || !(fabs(dE) <= 1e-11 * fmax(1.0, fabs(w.E)));
}

// psi is only as accurate as the energy it is computed at (error ~ |E - E_v|
// over the gap to the next level, 1e-5 Eh near dissociation): a norm pass
// whose Cooley correction is above this is redone once at E + dE
__device__ __forceinline__ bool redo_norm(const LevelWork& w, const PassDF& r) {
    return r.nodes == w.v && isfinite(r.dE) && fabs(r.dE) > 1e-13 * fmax(1.0, fabs(w.E)) && fabs(r.dE) < 1e-8;
}

// The norm passes store psi-hat = (h + l) 2^X in the 8 bytes of each window
// point of the level's row as a tagged float pair for scale_psi: X = 64 r + x
// with x in [-32, 31], the pair (h 2^x, l 2^x) in floats, and r in the five
// low bits of the second float (which only cost l bits 2^-43 below h).  X can
// reach hundreds (a window edge deep in a steep wall lies far below the peak);
// |X| is clamped to the tag's range of about +-1000, beyond any value that
// survives the normalisation.
struct PsiTag {
    float sc;  // 2^x
    int r;     // the tag
};

__device__ __forceinline__ PsiTag psi_tag(int X) {
    X = max(-1000, min(X, 990));
    const int r = (X + 32) >> 6;  // floor((X + 32) / 64): x = X - 64 r in [-32, 31]
    return {fpow2(X - 64 * r), r};
}

__device__ __forceinline__ void store_psi_pair(double* __restrict__ row, int i, dfl psi, PsiTag t) {
    const float l = __fmul_rn(psi.l, t.sc);
    const uint32_t lt = (__float_as_uint(l) & ~31u) | ((uint32_t)t.r & 31u);
    reinterpret_cast<float2*>(row)[i] = make_float2(__fmul_rn(psi.h, t.sc), __uint_as_float(lt));
}

// the stored pair back: (h, l) and the tag r (psi-hat = (h + l) 2^(64 r))
__device__ __forceinline__ dfl load_psi_pair(float2 v, int& r) {
    const uint32_t lt = __float_as_uint(v.y);
    r = ((int)(lt << 27)) >> 27;  // sign-extended five bits
    return {v.x, __uint_as_float(lt & ~31u)};
}

// the level's psi row for the fused norm/write, or nullptr (no psi requested,
// or the psi buffer overflowed: the level setup raised the capacity error)
__device__ __forceinline__ double* psi_row(const DevBatch& b, const PotMeta& m, const LevelWork& w) {
    if (!b.psi || b.hdr->error) return nullptr;
    return b.psi + m.psi_off + (int64_t)(w.v - b.min_level) * m.N;
}

__device__ __forceinline__ bool no_result(const LevelWork& w) {
    return (w.status & (EPSCU_STATUS_NOTFOUND | EPSCU_STATUS_CANCELLED | EPSCU_STATUS_NONFINITE)) != 0;
}

}  // namespace epscu
