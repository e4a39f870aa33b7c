// common.cuh -- device-side data layout and arithmetic shared by the solver
// kernels of libepseon_cuda (sm_103a).
//
// The discrete problem is the one the FP64 oracle restates (Numerov on a
// uniform grid with E-independent Dirichlet cut-offs, twisted Sturm counts):
//   a = mu h^2 / 6,  T_i = aE - W_i with W_i = a V_i,  f_i = 1 + T_i,
//   g_i = 2 - 10 T_i,  projective step (A, B) <- (g A - f B, f A).
// Every FP64 expression on the count/bisection path is written with explicit
// __dadd_rn/__dmul_rn/__fma_rn so that nvcc cannot contract it differently
// from the oracle's explicit fma() calls.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "epscu.h"

// status bits kept per potential / level (public values from epscu.h)
#define EPSCU_STATUS_MAXITER EPSCU_LEVEL_MAXITER
#define EPSCU_STATUS_NONFINITE EPSCU_LEVEL_NONFINITE
#define EPSCU_STATUS_UNDER EPSCU_LEVEL_UNDER_RESOLVED
#define EPSCU_STATUS_CANCELLED EPSCU_LEVEL_CANCELLED
#define EPSCU_STATUS_NOTFOUND EPSCU_LEVEL_NOT_FOUND
#define EPSCU_STATUS_BAD EPSCU_LEVEL_BAD_INPUT

namespace epscu {

constexpr int kRenorm = 32;  // renormalise the projective state every kRenorm steps

// Per-potential constants, written by the prepare kernel.
struct PotMeta {
    double r_min, r_max, mu, e_cap;  // inputs
    double h, a, e_lo, delta;        // derived (same formulas as the oracle)
    int64_t off;                     // first element in V64 / W64 / Msuf
    int64_t offf;                    // first element in Wf2 (tile aligned)
    int64_t psi_off;                 // first element of this potential's psi rows
    int32_t N, i0, i1, k_scan;
    int32_t n_bisect, n_trial;
    int32_t n_total, n_out;
    int32_t level_base, status;
    int32_t pad0, pad1;
};

// One level slot of the refinement stages.
struct LevelWork {
    double lo, hi;      // bracket (count(lo) <= v < count(hi))
    double lo0, hi0;    // the scan bracket
    double E;           // current energy
    double dE;          // last correction (error estimate)
    double norm_k_out;  // write-pass constants: psi scale on the outward side
    double norm_k_in;   //   and on the inward side
    double ck;          // psi at the match index
    int32_t ex_out, ex_in;  // binary exponents of the two side constants
    int32_t p, v;
    int32_t nodes, status;
    int32_t k;          // match index used by the write pass
    int32_t iters;
    int32_t j0, j1;     // grid window of the level's passes ([i0, i1] unless narrowed
                        // by the decay window of the fast method)
    int32_t n_in_bracket;  // levels the scan counted inside the scan bracket
    int32_t pad1;
};

// Global counters and flags of one solve (device memory).
struct Header {
    int32_t total_levels;
    int32_t queue_scan;
    int32_t queue_refine;
    int32_t queue_polish;
    int32_t error;          // first device-side error code (0 = none)
    int32_t fallbacks;      // levels that needed the bisection fallback
    int32_t n_units;        // warp work units (<= 32 levels of one potential)
    int32_t n_twist;        // levels handed to the twist-index search
    int32_t queue[16];      // work-queue heads of the per-level kernels
    int32_t n_long;         // levels whose window takes the CTA-per-level passes
    int32_t n_mid;          // levels whose window takes the warp-per-level passes
    int32_t pad_mid;
    int32_t bis_items_n;    // bisection round: (potential, chunk) items listed
    int32_t bis_items_q;    //   and the work-queue head over them
    int32_t n_redo;         // norm passes redone at E + dE
    unsigned long long scan_updates;    // point-updates the windowed FP32 scan performed
    unsigned long long refine_updates;  // point-updates of the FP32 refinement passes
    unsigned long long df_updates;      // point-updates of the double-float passes
    long long psi_total;                // psi doubles of the batch (level setup)
    unsigned long long refine_max_updates;  // largest per-level point-updates of refine32
    unsigned long long df_max_updates;      // largest per-level point-updates of newton_df / norm_df
    int32_t refine_max_iters;               // most refine32 passes of one level
    int32_t pad_hdr;
    unsigned long long long32_updates;      // refine_long (long list): FP32 pass point-updates
    unsigned long long longdf_updates;      //   and double-float pass point-updates
    unsigned long long psi_zero_points;     // psi points zeroed by zero_psi (outside the windows)
    unsigned long long psi_window_points;   // window points scale_psi converted
};

// queue ids of the per-level kernels
enum { kQRefine32 = 0, kQNewtonDF, kQNormDF, kQWriteDF, kQBisect64, kQNorm64, kQWrite64, kQLongRefine, kQFallback,
       kQNormLong, kQTwistLong, kQMidRefine, kQNormMid, kQScalePsi, kQNormFallback };

// internal level flags (not reported: gather keeps the public bits only)
// the Newton stage handed the level to the fallback: its refinement, norm pass
// and (recompute) write run one CTA per level over the fallback list, and its
// norm constants are the group passes' (the lane kernels skip it)
#define EPSCU_STATUS_FALLBACK 0x10000
// the level's passes run one CTA per level (longwin.cu)
#define EPSCU_STATUS_LONG 0x20000
// the level's double-float passes run one warp per level (the middle tier, longwin.cu)
#define EPSCU_STATUS_MID 0x40000
#define EPSCU_STATUS_PUBLIC 0xffff
// spacing of the samples of the twist-index search
constexpr int kTwistSample = 64;

// ---------------------------------------------------------------- FP64 helpers

// One divide-free projective Numerov step (identical to the oracle's
// numerov_step): state (A, B) ~ s (u_i, u_{i-1}) -> s f_i (u_{i+1}, u_i).
__device__ __forceinline__ void step64(double aE, double w, double& A, double& B) {
    const double T = __dsub_rn(aE, w);
    const double f = __dadd_rn(1.0, T);
    const double g = __fma_rn(-10.0, T, 2.0);
    const double An = __fma_rn(g, A, -__dmul_rn(f, B));
    B = __dmul_rn(f, A);
    A = An;
}

// frexp-style exponent of |m| (m = f 2^e, f in [0.5, 1)) for finite normal m.
__device__ __forceinline__ int exp_of(double m) {
    const int hi = __double2hiint(m);
    return ((hi >> 20) & 0x7ff) - 1022;
}

// Exact power of two 2^e for |e| < 1000.
__device__ __forceinline__ double pow2(int e) { return __hiloint2double((1023 + e) << 20, 0); }

// Rescale (x, y) by the power of two that brings max(|x|,|y|) into [0.5, 1);
// returns the exponent removed (0 when the pair is zero or not finite).
__device__ __forceinline__ int renorm_pair(double& x, double& y) {
    const double m = fmax(fabs(x), fabs(y));
    if (!(m > 0.0) || !isfinite(m)) return 0;
    const int e = exp_of(m);
    if (e > 1000 || e < -1000) return 0;
    const double s = pow2(-e);
    x *= s;
    y *= s;
    return e;
}

// E_j = E_lo + (j+1) delta (two roundings, as in the oracle).
__device__ __forceinline__ double trial_energy(const PotMeta& m, int j) {
    return __dadd_rn(m.e_lo, __dmul_rn((double)(j + 1), m.delta));
}

// Largest i in [i0, i1] with V_i <= E, by binary search on the suffix minima
// Msuf_i = min(V_i .. V_{i1}); k_scan when there is none.  Equals the
// oracle's linear search.
__device__ __forceinline__ int match_index(const PotMeta& m, const double* __restrict__ Msuf, double E) {
    const double* M = Msuf + m.off;
    if (!(M[m.i0] <= E)) return m.k_scan;
    int lo = m.i0, hi = m.i1;  // invariant: M[lo] <= E
    while (lo < hi) {
        const int mid = lo + (hi - lo + 1) / 2;
        if (M[mid] <= E) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// bisection scan: the throughput scan on every kBisectCoarse-th trial
// energy, then counts inside the coarse cells whose end counts differ
constexpr int kBisectCoarse = 16;
// parts a cell with two or more levels is cut into per round (a power of two
// dividing kBisectCoarse; equal to it: one round, a count at every trial
// energy of the cell)
constexpr int kBisectSplit = 16;
// parts a coarse cell that holds exactly one level is cut into (a power of
// two dividing kBisectCoarse; 1: no count inside, the level's bracket is the
// whole cell, which isolates it already)
constexpr int kBisectSingle = 4;
// batches of at least this many potentials take the bisection scan (smaller
// ones have too few CTAs per round to cover its latency; measured on GB300)
constexpr int kBisectMinPotentials = 512;

// e-folds of decay at the ends of the fast method's windows: e^-36 = 2.3e-16,
// psi at the cut is below FP64 resolution relative to its value at the
// turning point (dense eigen-decompositions of the discrete problem keep
// every level to 1e-12 and every eigenvector to 1e-10 in L2 down to 26)
constexpr float kWindowDecay = 36.0f;
// trial energies per entry of the scan's window table
constexpr int kScanWinBlock = 128;

// Twisted Sturm count at E with twist index k (identical arithmetic to the
// oracle's eo_count).
__device__ __forceinline__ int count64(const PotMeta& m, const double* __restrict__ W, double E, int k) {
    const double aE = __dmul_rn(m.a, E);
    int nodes = 0;
    double A = 1.0, B = 0.0;
    int s = 0;
    for (int i = m.i0; i < k; ++i) {
        const double Ap = A;
        step64(aE, __ldg(W + i), A, B);
        nodes += (A < 0.0) != (Ap < 0.0);
        if (++s == kRenorm) {
            s = 0;
            renorm_pair(A, B);
        }
    }
    double C = 1.0, D = 0.0;
    s = 0;
    for (int i = m.i1; i > k; --i) {
        const double Cp = C;
        step64(aE, __ldg(W + i), C, D);
        nodes += (C < 0.0) != (Cp < 0.0);
        if (++s == kRenorm) {
            s = 0;
            renorm_pair(C, D);
        }
    }
    const double Tk = __dsub_rn(aE, __ldg(W + k));
    const double fk = __dadd_rn(1.0, Tk);
    const double gk = __fma_rn(-10.0, Tk, 2.0);
    const double AC = __dmul_rn(A, C);
    const double num = __fma_rn(gk, AC, -__dmul_rn(fk, __fma_rn(B, C, __dmul_rn(D, A))));
    nodes += (num < 0.0) != (AC < 0.0);
    return nodes;
}

// 1/f for f in [0.4, 4]: FP32 reciprocal refined by two FP64 Newton steps
// (relative error at the FP64 rounding level).
__device__ __forceinline__ double recip64(double f) {
    double r = (double)__frcp_rn((float)f);
    r = __fma_rn(r, __fma_rn(-f, r, 1.0), r);
    r = __fma_rn(r, __fma_rn(-f, r, 1.0), r);
    return r;
}

}  // namespace epscu
