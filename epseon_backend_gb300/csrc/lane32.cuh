// lane32.cuh -- the FP32 lane pass of the fast method and the per-level
// refinement built on it (one lane per level), shared by refine32_kernel
// (levels.cu) and the fused lane kernel (polish.cu).
#pragma once

#include <math.h>
#include <stdint.h>

#include "common.cuh"
#include "dfpass.cuh"
#include "launch.h"

namespace epscu {

namespace {

__device__ __forceinline__ bool cancelled(const DevBatch& b) { return b.cancel && *b.cancel; }

// move the match point to the peak of |psi| when the sampled peak is at least
// 2^kPeakLog2 (in binary exponent) above |psi_k|
constexpr int kPeakLog2 = 2;

// FP32 Cooley pass in the difference form; returns dE (FP64), count, nodes,
// sum psi~^2 and where |psi| peaks (sampled every 16 points, u = f s psi used
// as the proxy: the scale s barely moves against exponential growth).
struct Pass32 {
    double dE, sum;
    int count, nodes;
    int peak_i, peak_log2;
};

// One side's FP32 state: u ~ A 2^ecum, D ~ u_i - u_{i-dir}, S = sum of A_j^2
// weighted by the f^2 of the later points (the Cooley denominator), node
// count and the peak of |A| seen at the renormalisations.
struct Side32 {
    float A, D, S;
    int ecum, nodes, Lpk, ipk;
};

__device__ __forceinline__ void step32s(Side32& s, float aEh, float aEl, float2 w) {
    const float T = (aEh - w.x) + (aEl - w.y);
    const float f = 1.0f + T;
    s.S = fmaf(f * f, s.S, s.A * s.A);
    const float X = fmaf(-12.0f, s.A, s.D);
    s.D = fmaf(T, X, s.D);
    const float An = s.A + fmaf(T, s.A, s.D);
    s.nodes += (__float_as_uint(An) ^ __float_as_uint(s.A)) >> 31;
    s.A = An;
}

// renormalise (exact powers of two) and sample the peak at point i
__device__ __forceinline__ void renorm32s(Side32& s, int i) {
    const float mm = fmaxf(fabsf(s.A), fabsf(s.D));
    const int e = ((__float_as_int(mm) >> 23) & 0xff) - 126;
    if (mm > 0.0f && e > -60 && e < 60) {
        const float sc = __int_as_float((127 - e) << 23);
        s.A *= sc;
        s.D *= sc;
        s.S *= sc * sc;
        s.ecum += e;
    }
    const int L = s.ecum + ((__float_as_int(fabsf(s.A)) >> 23) & 0xff);
    if (s.A != 0.0f && L > s.Lpk) {
        s.Lpk = L;
        s.ipk = i;
    }
}

// steps base.. of one side alone (points from + dir * step, nsteps in all),
// in 8-step chunks renormalised at their ends; grid values do not depend on
// the state, so two chunks are kept in flight (register double buffer)
__device__ __forceinline__ void side32_rest(Side32& s, const float2* __restrict__ Wf, float aEh, float aEl, int from,
                                            int dir, int base, int nsteps) {
    auto load8 = [&](float2* w8, int b0) {
#pragma unroll
        for (int u = 0; u < 8; ++u) w8[u] = __ldg(Wf + from + dir * min(b0 + u, nsteps - 1));
    };
    auto run8 = [&](const float2* w8, int b0) {
#pragma unroll
        for (int u = 0; u < 8; ++u)
            if (b0 + u < nsteps) step32s(s, aEh, aEl, w8[u]);
        renorm32s(s, from + dir * min(b0 + 7, nsteps - 1));
    };
    float2 wa[8], wb[8];
    if (base < nsteps) load8(wa, base);
    for (int b0 = base; b0 < nsteps; b0 += 16) {
        if (b0 + 8 < nsteps) load8(wb, b0 + 8);
        run8(wa, b0);
        if (b0 + 8 >= nsteps) break;
        if (b0 + 16 < nsteps) load8(wa, b0 + 16);
        run8(wb, b0 + 8);
    }
}

__device__ __forceinline__ Pass32 cooley32(const PotMeta& m, const float2* __restrict__ Wf, const double* __restrict__ W64,
                                           double E, int k, int j0, int j1) {
    const double aE = __dmul_rn(m.a, E);
    const float aEh = __double2float_rn(aE);
    const float aEl = __double2float_rn(aE - (double)aEh);
    // outward from j0 (u_{j0} = 1, u_{j0-1} = 0) and inward from j1, both to k
    Side32 o{1.0f, 1.0f, 0.0f, 0, 0, -(1 << 30), j0};
    Side32 in{1.0f, 1.0f, 0.0f, 0, 0, -(1 << 30), j1};
    const int no = k - j0, ni = j1 - k;
    // the two sides are independent recurrences: their common full chunks run
    // interleaved (two dependency chains per lane), the rest of the longer
    // side alone; the arithmetic of each side is unchanged
    const int nb = min(no, ni) & ~7;
    int base = 0;
    for (; base < nb; base += 8) {
        float2 wo[8], wi[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            wo[u] = __ldg(Wf + j0 + base + u);
            wi[u] = __ldg(Wf + j1 - base - u);
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            step32s(o, aEh, aEl, wo[u]);
            step32s(in, aEh, aEl, wi[u]);
        }
        renorm32s(o, j0 + base + 7);
        renorm32s(in, j1 - base - 7);
    }
    side32_rest(o, Wf, aEh, aEl, j0, +1, base, no);
    side32_rest(in, Wf, aEh, aEl, j1, -1, base, ni);
    const int nodes = o.nodes + in.nodes;
    const float Ao = o.A, Do = o.D, So = o.S, Ai = in.A, Di = in.D, Si = in.S;
    const int Lk[2] = {o.ecum + (o.A != 0.0f ? ((__float_as_int(fabsf(o.A)) >> 23) & 0xff) : -1000),
                       in.ecum + (in.A != 0.0f ? ((__float_as_int(fabsf(in.A)) >> 23) & 0xff) : -1000)};
    const int Lpk[2] = {o.Lpk, in.Lpk}, ipk[2] = {o.ipk, in.ipk};
    const double Tk = aE - W64[k];
    const double fk = 1.0 + Tk;
    const double uA = Ao, vC = Ai;
    // gamma_k = -12 T_k / f_k + D_o / u_k + D_i / v_k   (no cancellation)
    const double gamma = -12.0 * Tk / fk + (double)Do / uA + (double)Di / vC;
    const double fk2 = fk * fk;
    Pass32 r;
    r.sum = fk2 * ((double)So / (uA * uA) + (double)Si / (vC * vC)) + 1.0;
    r.dE = gamma * fk2 / (12.0 * m.a * r.sum);
    r.nodes = nodes;
    r.count = nodes + (gamma < 0.0 ? 1 : 0);
    const int po = Lpk[0] - Lk[0], pi = Lpk[1] - Lk[1];
    r.peak_log2 = max(po, pi);
    r.peak_i = po >= pi ? ipk[0] : ipk[1];
    return r;
}

// Safeguarded Cooley-Newton in FP32.  The match point follows the peak of
// |psi| (re-estimated from every pass: matching where the eigenvector is
// largest keeps the correction quadratic; at a turning point where psi is small
// it converges to a spurious point).  Every pass updates the count bracket.  A
// small Newton step is accepted outright when the scan bracket held this level
// alone and the pass saw its node count; otherwise it is confirmed by a count
// on the far side of the predicted root, or the level continues by bisection.
constexpr double kTol32 = 2e-9;
// a Newton step accepted outright (the level alone in its scan bracket, its
// node count seen): the energy after it is within ~1e-4 of the step (the
// relative error of the FP32 sum) plus the step's square over the curvature.
// (Measured on the 2048-potential batch: 2e-8 takes no fewer passes, the
// quadratic steps jump past it; 5e-8 and above leave more norm passes to
// redo, +0.6 and +2.6 ms a step.)
constexpr double kAccept32 = 2e-9;

// The FP32 refinement of the level in slot `slot` (one lane); false when the
// level takes no lane refinement (no bracket, a long window, or cancelled).
__device__ __forceinline__ bool refine32_level(const DevBatch& b, int slot) {
    LevelWork w = b.levels[slot];
    // long windows: refine_long (middle windows take their FP32 passes here)
    if (w.status & (EPSCU_STATUS_NOTFOUND | EPSCU_STATUS_LONG)) return false;
    if (cancelled(b)) {
        b.levels[slot].status = w.status | EPSCU_STATUS_CANCELLED;
        return false;
    }
    const PotMeta m = b.meta[w.p];
    const float2* Wf = b.Wf2 + m.offf;
    const double* W64 = b.W64 + m.off;
    double lo = w.lo, hi = w.hi, E = w.E;
    // the level's window (decay window of its bracket)
    auto clamp_w = [&](int kk) { return max(w.j0 + 1, min(kk, w.j1 - 1)); };
    int k = clamp_w(match_index(m, b.Msuf, E));
    bool bisect = false, confirming = false, done = false;
    double E_star = E, sum = 1.0;
    int it = 0;
    int k_sum = k;  // match point of `sum` (sum psi~^2 is normalised by psi at k)
    // the Newton stage divides by sum psi~^2 at the final match point: when
    // the deciding pass moved the match point, one more pass at E_star
    // recomputes the sum there (a stale sum is off by (psi_k_old/psi_k)^2
    // and slows Newton to a crawl)
    bool final_pass = false;
    for (const int cap = refine_cap(b); it < cap || final_pass; ++it) {
        const Pass32 r = cooley32(m, Wf, W64, E, k, w.j0, w.j1);
        sum = r.sum;
        k_sum = k;
        if (final_pass) break;
        if (r.count > w.v) hi = E;
        else lo = E;
        const bool moved = r.peak_log2 >= kPeakLog2;
        if (moved) k = clamp_w(r.peak_i);
        if (confirming) {
            confirming = false;
            if (hi - lo <= 3.0 * kTol32 + 1e-15 && E_star >= lo && E_star <= hi) done = true;
            else bisect = true;  // the predicted root was not confirmed
        }
        if (!done && hi - lo <= 2.0 * kTol32) {
            E_star = 0.5 * (lo + hi);
            done = true;
        }
        if (done) {
            if (k == k_sum) break;
            final_pass = true;
            E = E_star;
            continue;
        }
        double En;
        if (!bisect && !moved) {
            En = E + r.dE;
            if (!(En > lo && En < hi) || !isfinite(En)) {
                En = 0.5 * (lo + hi);
            } else if (fabs(r.dE) <= kAccept32 && w.n_in_bracket == 1 && r.nodes == w.v) {
                // the scan bracket holds this level alone and the pass sees
                // its node count: the root is the level (the double-float
                // Newton re-checks the count)
                E_star = En;
                done = true;
                break;
            } else if (fabs(r.dE) <= kTol32) {
                E_star = En;
                En = En + (r.dE >= 0.0 ? kTol32 : -kTol32);
                if (En <= lo || En >= hi) En = 0.5 * (E_star + (r.dE >= 0.0 ? hi : lo));
                confirming = true;
            }
        } else {
            En = 0.5 * (lo + hi);  // bisection (also after moving the match point)
        }
        E = En;
    }
    if (!done) {
        w.status |= EPSCU_STATUS_MAXITER;
        E_star = 0.5 * (lo + hi);
    }
    w.lo = lo;
    w.hi = hi;
    w.E = E_star;
    w.k = k;
    w.norm_k_in = sum;  // sum psi~^2 at the match point k, the Newton denominator of newton_df
    w.iters = it;
    const unsigned long long upd = (unsigned long long)(it + 1) * (unsigned long long)(w.j1 - w.j0);
    atomicAdd(&b.hdr->refine_updates, upd);
    atomicMax(&b.hdr->refine_max_updates, upd);
    atomicMax(&b.hdr->refine_max_iters, it + 1);
    b.levels[slot] = w;
    return true;
}

}  // namespace

}  // namespace epscu
