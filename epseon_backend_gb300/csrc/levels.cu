// levels.cu -- per-level refinement, normalisation and write-back.
//
// Every kernel here is persistent (grid = SMs x resident CTAs) and walks the
// level slots written by the bracket kernel; the number of slots is read from
// device memory, so the whole solve can be captured in one CUDA graph.
//
//  bisect64 : plain method, FP64 bisection on the twisted Sturm count with the
//             match index k(E) (outer classical turning point), n_bisect halvings
//             of the scan bracket -- identical arithmetic to the oracle.
//  refine32 : fast method, safeguarded Cooley-Newton iteration in the FP32
//             difference form (count + matching residual + norm per pass).
//  norm64   : FP64 Cooley pass that also fixes the normalisation constants
//             (sum psi^2 h = 1, psi > 0 next to the inner wall) and the node
//             count reported for the level.
//  write64  : recomputes the FP64 recurrence and writes psi.
//  gather   : level slots -> the caller's [potential x capacity] layout; the
//             fast method reports E + dE of the last FP64 pass, the plain
//             method the bisection midpoint itself.
//
// Scale handling: the divide-free state after step i is s_{i+1} (u_{i+1}, u_i)
// with s_{i+1} = f_{i0} ... f_i, so psi_i = u_i / f_i = A_i / s_{i+1}.  Sums
// of psi^2 use S_{i+1} = f_i^2 S_i + A_i^2 (no division); the write pass
// carries q_i = 1 / s_i with a refined reciprocal of f_i.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "common.cuh"
#include "dfpass.cuh"
#include "launch.h"
#include "lane32.cuh"

namespace epscu {

namespace {

constexpr int kLevelThreads = 128;

// match points stay off the two boundary points (both sides non-empty)
__device__ __forceinline__ int clamp_inner(const PotMeta& m, int k) { return max(m.i0 + 1, min(k, m.i1 - 1)); }

// ------------------------------------------------------------------ FP64 pass

struct Side64 {
    double A, B, S, q;  // state, psi^2 sum, 1/s (TRACK only)
    int eA, eQ;         // exponents removed from A/B and from q
    int nodes;
    int peak_L, peak_i;  // TRACK: largest log2 |psi-hat| seen at a renormalisation point, and where
};

template <bool TRACK, bool WRITE>
__device__ __forceinline__ void side64(const double* __restrict__ W, double aE, int from, int to, int dir, Side64& st,
                                       double* __restrict__ out, double L, int Xk) {
    st.A = 1.0;
    st.B = 0.0;
    st.S = 0.0;
    st.q = 1.0;
    st.eA = 0;
    st.eQ = 0;
    st.nodes = 0;
    st.peak_L = -1 << 30;
    st.peak_i = from;
    int s = 0;
    double F = 0.0;
    if (WRITE) F = L * ldexp(1.0, min(1000, max(-1100, -Xk)));
    for (int i = from; i != to; i += dir) {
        const double T = __dsub_rn(aE, __ldg(W + i));
        const double f = __dadd_rn(1.0, T);
        if (TRACK) {
            const double qn = st.q * recip64(f);
            if (WRITE) out[i] = st.A * qn * F;
            st.q = qn;
        }
        if (!WRITE) st.S = __fma_rn(f * f, st.S, st.A * st.A);
        const double g = __fma_rn(-10.0, T, 2.0);
        const double An = __fma_rn(g, st.A, -__dmul_rn(f, st.B));
        st.B = __dmul_rn(f, st.A);
        st.nodes += (An < 0.0) != (st.A < 0.0);
        st.A = An;
        if (++s == kRenorm) {
            s = 0;
            const int e = renorm_pair(st.A, st.B);
            st.eA += e;
            if (!WRITE && e) st.S *= pow2(-2 * e);
            if (TRACK) {
                const int eq = exp_of(st.q);
                st.q *= pow2(-eq);
                st.eQ += eq;
                if (!WRITE) {
                    const double mag = fabs(st.A * st.q);
                    if (mag > 0.0) {
                        const int L = exp_of(mag) + st.eA + st.eQ;
                        if (L > st.peak_L) {
                            st.peak_L = L;
                            st.peak_i = i;
                        }
                    }
                }
            }
            if (WRITE) F = L * ldexp(1.0, min(1000, max(-1100, st.eA + st.eQ - Xk)));
        }
    }
}

struct Pass64 {
    double dE, gamma, sum;
    double pk_out, pk_in;  // psi-hat at k from each side (TRACK)
    int ex_out, ex_in;
    int nodes;
    int peak_i;       // TRACK: where |psi| peaks (sampled every kRenorm points)
    int peak_log2;    // TRACK: log2 of that peak over |psi| at k
};

template <bool TRACK>
__device__ Pass64 cooley64(const PotMeta& m, const double* __restrict__ W, double E, int k) {
    const double aE = __dmul_rn(m.a, E);
    Side64 o, in;
    side64<TRACK, false>(W, aE, m.i0, k, +1, o, nullptr, 0.0, 0);
    side64<TRACK, false>(W, aE, m.i1, k, -1, in, nullptr, 0.0, 0);
    const double Tk = __dsub_rn(aE, __ldg(W + k));
    const double fk = __dadd_rn(1.0, Tk);
    const double gk = __fma_rn(-10.0, Tk, 2.0);
    Pass64 r;
    const double fk2 = fk * fk;
    r.sum = fk2 * (o.S / (o.A * o.A) + in.S / (in.A * in.A)) + 1.0;
    r.gamma = gk / fk - o.B / o.A - in.B / in.A;
    r.dE = r.gamma * fk2 / (12.0 * m.a * r.sum);
    r.nodes = o.nodes + in.nodes;
    if (TRACK) {
        const double rk = recip64(fk);
        r.pk_out = o.A * o.q * rk;
        r.pk_in = in.A * in.q * rk;
        r.ex_out = o.eA + o.eQ;
        r.ex_in = in.eA + in.eQ;
        const int Lo = (r.pk_out != 0.0 ? exp_of(fabs(r.pk_out)) : -1000) + r.ex_out;
        const int Li = (r.pk_in != 0.0 ? exp_of(fabs(r.pk_in)) : -1000) + r.ex_in;
        const int po = o.peak_L - Lo, pi = in.peak_L - Li;
        r.peak_log2 = max(po, pi);
        r.peak_i = po >= pi ? o.peak_i : in.peak_i;
    } else {
        r.pk_out = r.pk_in = 0.0;
        r.ex_out = r.ex_in = 0;
        r.peak_log2 = 0;
        r.peak_i = k;
    }
    return r;
}

// ----------------------------------------------------------------- kernels

__global__ void __launch_bounds__(kLevelThreads) bisect64_kernel(DevBatch b) {
    for (int2 unit; next_unit(b, kQBisect64, unit);) {
        if ((int)(threadIdx.x & 31) >= unit.y) continue;
        const int slot = unit.x + (threadIdx.x & 31);
        LevelWork w = b.levels[slot];
        if (w.status & EPSCU_STATUS_NOTFOUND) continue;
        if (cancelled(b)) {
            b.levels[slot].status = w.status | EPSCU_STATUS_CANCELLED;
            continue;
        }
        const PotMeta m = b.meta[w.p];
        const double* W = b.W64 + m.off;
        double lo = w.lo, hi = w.hi;
        for (int it = 0; it < m.n_bisect; ++it) {
            const double mid = __dmul_rn(0.5, __dadd_rn(lo, hi));
            if (count64(m, W, mid, match_index(m, b.Msuf, mid)) > w.v) hi = mid;
            else lo = mid;
        }
        w.lo = lo;
        w.hi = hi;
        w.E = __dmul_rn(0.5, __dadd_rn(lo, hi));
        w.iters = m.n_bisect;
        b.levels[slot] = w;
    }
}

__global__ void __launch_bounds__(kLaneThreads, kLaneCtasPerSm) refine32_kernel(DevBatch b) {
    for (int2 unit; next_unit(b, kQRefine32, unit);) {
        if ((int)(threadIdx.x & 31) >= unit.y) continue;
        refine32_level(b, unit.x + (threadIdx.x & 31));
    }
}

// Write the normalisation constants of pass r (match point k) into w.
__device__ __forceinline__ void finalize64(const PotMeta& m, LevelWork& w, const Pass64& r, int k) {
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

// use_k: keep the match point chosen by the FP32 refinement (fast method);
// otherwise the outer turning point, moved to the peak of |psi| of the solution
// stitched there (as the oracle's match point).
__global__ void __launch_bounds__(kLevelThreads) norm64_kernel(DevBatch b, int use_k) {
    for (int2 unit; next_unit(b, kQNorm64, unit);) {
        if ((int)(threadIdx.x & 31) >= unit.y) continue;
        const int slot = unit.x + (threadIdx.x & 31);
        LevelWork w = b.levels[slot];
        if (w.status & (EPSCU_STATUS_NOTFOUND | EPSCU_STATUS_CANCELLED)) continue;
        const PotMeta m = b.meta[w.p];
        int k = use_k ? w.k : clamp_inner(m, match_index(m, b.Msuf, w.E));
        Pass64 r = cooley64<true>(m, b.W64 + m.off, w.E, k);
        if (!use_k && r.peak_log2 >= 1) {
            k = clamp_inner(m, r.peak_i);
            r = cooley64<true>(m, b.W64 + m.off, w.E, k);
        }
        finalize64(m, w, r, k);
        // a poor match point shows as a wrong node count or as a Cooley
        // correction far above the accuracy of the bisected energy
        const bool bad = (r.nodes != w.v && !(m.status & EPSCU_STATUS_UNDER)) ||
                         !(fabs(r.dE) <= 1e-11 * fmax(1.0, fabs(w.E)));
        if (bad && b.twist_list) {
            const int q = atomicAdd(&b.hdr->n_twist, 1);
            if (q < b.max_twist) b.twist_list[q] = slot;
        }
        b.levels[slot] = w;
    }
}

// Twist-index search of the plain method (FP64): sampled outward ratios
// u_{k-1}/u_k, inward ratios v_{k+1}/v_k, match point argmin |gamma_k|.
__global__ void __launch_bounds__(64) twist64_kernel(DevBatch b) {
    const int n = min(b.hdr->n_twist, b.max_twist);
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        const int slot = b.twist_list[q];
        LevelWork w = b.levels[slot];
        const PotMeta m = b.meta[w.p];
        const double* W = b.W64 + m.off;
        double* rho = b.twist_scratch + (int64_t)q * b.twist_stride;
        const double aE = __dmul_rn(m.a, w.E);
        double A = 1.0, B = 0.0;
        int s = 0;
        for (int i = m.i0; i < m.i1; ++i) {
            const int j = (i - m.i0) / kTwistSample;
            if ((i - m.i0) % kTwistSample == 0 && j < b.twist_stride) rho[j] = B / A;
            step64(aE, __ldg(W + i), A, B);
            if (++s == kRenorm) {
                s = 0;
                renorm_pair(A, B);
            }
        }
        double C = 1.0, D = 0.0, best = INFINITY;
        int kbest = w.k;
        s = 0;
        for (int i = m.i1; i > m.i0; --i) {
            if ((i - m.i0) % kTwistSample == 0 && i <= m.i1 - 1) {
                const int j = (i - m.i0) / kTwistSample;
                if (j < b.twist_stride) {
                    const double T = __dsub_rn(aE, __ldg(W + i));
                    const double gam = (2.0 - 10.0 * T) / (1.0 + T) - rho[j] - D / C;
                    if (fabs(gam) < best) {
                        best = fabs(gam);
                        kbest = i;
                    }
                }
            }
            step64(aE, __ldg(W + i), C, D);
            if (++s == kRenorm) {
                s = 0;
                renorm_pair(C, D);
            }
        }
        const int k = clamp_inner(m, kbest);
        const Pass64 r = cooley64<true>(m, W, w.E, k);
        finalize64(m, w, r, k);
        b.levels[slot] = w;
    }
}

__global__ void __launch_bounds__(kLevelThreads) write64_kernel(DevBatch b) {
    if (!b.psi || b.hdr->error) return;
    for (int2 unit; next_unit(b, kQWrite64, unit);) {
        if ((int)(threadIdx.x & 31) >= unit.y) continue;
        const int slot = unit.x + (threadIdx.x & 31);
        const LevelWork w = b.levels[slot];
        const PotMeta m = b.meta[w.p];
        double* out = b.psi + m.psi_off + (int64_t)(w.v - b.min_level) * m.N;
        for (int i = 0; i < m.i0; ++i) out[i] = 0.0;
        for (int i = m.i1 + 1; i < m.N; ++i) out[i] = 0.0;
        if (w.status & (EPSCU_STATUS_NOTFOUND | EPSCU_STATUS_CANCELLED | EPSCU_STATUS_NONFINITE)) {
            for (int i = m.i0; i <= m.i1; ++i) out[i] = 0.0;
            continue;
        }
        const double* W = b.W64 + m.off;
        const double aE = __dmul_rn(m.a, w.E);
        Side64 st;
        side64<true, true>(W, aE, m.i0, w.k, +1, st, out, w.norm_k_out, w.ex_out);
        side64<true, true>(W, aE, m.i1, w.k, -1, st, out, w.norm_k_in, w.ex_in);
        out[w.k] = w.ck;
    }
}

__global__ void gather_kernel(DevBatch b, int32_t* n_total, int32_t* n_out, double* energy, int32_t* nodes,
                              int32_t* status, double* err_est, int apply_dE) {
    const int p = blockIdx.x;
    const PotMeta m = b.meta[p];
    if (threadIdx.x == 0) {
        n_total[p] = m.n_total;
        n_out[p] = m.n_out;
    }
    for (int s = threadIdx.x; s < b.level_capacity; s += blockDim.x) {
        const int64_t o = (int64_t)p * b.level_capacity + s;
        if (s < m.n_out) {
            const LevelWork w = b.levels[m.level_base + s];
            energy[o] = (apply_dE && fabs(w.dE) <= 1e-9) ? w.E + w.dE : w.E;
            nodes[o] = w.nodes;
            status[o] = (w.status & EPSCU_STATUS_PUBLIC) | (m.status & EPSCU_STATUS_UNDER);
            if (err_est) err_est[o] = fabs(w.dE);
        } else {
            energy[o] = NAN;
            nodes[o] = -1;
            status[o] = EPSCU_STATUS_NOTFOUND | (m.status & (EPSCU_STATUS_BAD | EPSCU_STATUS_NONFINITE));
            if (err_est) err_est[o] = NAN;
        }
    }
}

int persistent_grid(int sm_count, int per_sm) { return sm_count * per_sm; }

}  // namespace

void launch_bisect64(const DevBatch& b, int sm_count, cudaStream_t s) {
    bisect64_kernel<<<persistent_grid(sm_count, 8), kLevelThreads, 0, s>>>(b);
}
void launch_refine32(const DevBatch& b, int sm_count, cudaStream_t s) {
    refine32_kernel<<<persistent_grid(sm_count, kLaneCtasPerSm), kLaneThreads, 0, s>>>(b);
}
void launch_norm64(const DevBatch& b, int use_k, int sm_count, cudaStream_t s) {
    norm64_kernel<<<persistent_grid(sm_count, 8), kLevelThreads, 0, s>>>(b, use_k);
}
void launch_twist64(const DevBatch& b, int sm_count, cudaStream_t s) {
    twist64_kernel<<<sm_count, 64, 0, s>>>(b);
}
void launch_write64(const DevBatch& b, int sm_count, cudaStream_t s) {
    write64_kernel<<<persistent_grid(sm_count, 8), kLevelThreads, 0, s>>>(b);
}
void launch_gather(const DevBatch& b, int32_t* n_total, int32_t* n_out, double* energy, int32_t* nodes,
                   int32_t* status, double* err_est, int apply_dE, cudaStream_t s) {
    gather_kernel<<<b.n, 128, 0, s>>>(b, n_total, n_out, energy, nodes, status, err_est, apply_dE);
}

}  // namespace epscu
