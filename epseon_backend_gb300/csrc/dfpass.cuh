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
// proportionally less below, never under 2048.  Measured on GB300 with the
// long levels on their own stream beside the lane kernels: the 2048-potential
// batch (93k levels) is fastest at 8192-12288, the 256-potential bump batch
// (14k levels) at 4096, the 64-Morse batch (3.4k levels) at 2048.
// DevBatch::long_window > 0 overrides it.
constexpr int kLongWindow = 8192;
constexpr int kLongWindowLevels = 45000;
constexpr int kMinLongWindow = 2048;

__host__ __device__ __forceinline__ int default_long_window(int total_levels) {
    int w = kMinLongWindow;
    while (w < kLongWindow && (long long)w * kLongWindowLevels < (long long)kLongWindow * total_levels) w <<= 1;
    return w;
}

__device__ __forceinline__ bool is_long(const LevelWork& w) { return (w.status & EPSCU_STATUS_LONG) != 0; }

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
