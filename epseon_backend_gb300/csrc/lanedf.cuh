// lanedf.cuh -- the double-float lane passes of the fast method (one lane
// per level) and the per-level Newton and norm stages built on them, shared
// by newton_df_kernel / norm_df_kernel and the fused lane kernel (polish.cu).
//
// The recurrence of the last passes runs in double-float arithmetic (~48-bit
// significands, see dfloat.cuh) in the Blatt difference form
//     D' = D + T (D - 12 A),   A' = A + (T A + D')
// with T = aE - W carried as a double-float pair; FP64 is used only for the
// matching-point difference gamma_k, the Newton step and the rare spill of
// the norm integral (sum psi^2 in double-float, dfloat.cuh SqSum).
#pragma once

#include <math.h>
#include <stdint.h>

#include "common.cuh"
#include "dfloat.cuh"
#include "dfpass.cuh"
#include "launch.h"

namespace epscu {

namespace {

// MODE 0: state only (Newton)   MODE 1: + sums, psi-hat, peak   MODE 2: + write
// MODE 3: MODE 1 + psi-hat written unnormalised (absolute scale, FP64)
//
// One side of a pass: the double-float state marched one point at a time
// (step) and renormalised every 8 points (renorm).
template <int MODE>
struct SideDF {
    dfl A, D, q;      // state ~ s (u_i, u_i - u_{i-1}); q = 1/s (MODE >= 1)
    int eA, eQ;       // exponents removed from (A, D) and from q
    int nodes;
    SqSum ss;         // MODE 1/3: sum of psi-hat^2 in the current scale
    double S;         // MODE 1/3: that sum at the end of the side (FP64)
    PsiTag tag;       // MODE 3: scale and tag of the stored pair (X = eA + eQ)
    int peak_L, peak_i;
    dfl F;            // MODE 2: psi scale constant in the current scale
    double L;         // MODE 2: the side's norm constant
    int Xk;           //   and its exponent

    __device__ __forceinline__ void init(int from, double L_, int Xk_) {
        A = {1.0f, 0.0f};
        D = {1.0f, 0.0f};  // u_from = 1, u_{from-dir} = 0
        q = {1.0f, 0.0f};
        eA = eQ = 0;
        nodes = 0;
        ss.init();
        S = 0.0;
        peak_L = -(1 << 30);
        peak_i = from;
        tag = psi_tag(0);
        L = L_;
        Xk = Xk_;
        F = {0.0f, 0.0f};
        if (MODE == 2) F = df_from_double(L * pow2(min(1000, max(-1000, -Xk))));
    }

    // the step at point i (grid value w)
    __device__ __forceinline__ void step(dfl aE, float2 w, double* __restrict__ out, int i) {
        dfl T = two_sum(aE.h, -w.x);
        T = fast_two_sum(T.h, __fadd_rn(T.l, __fsub_rn(aE.l, w.y)));
        if (MODE >= 1) {
            const dfl f = df_add({1.0f, 0.0f}, T);
            const dfl qn = df_mul(q, df_recip(f));
            const dfl psi = df_mul(A, qn);  // psi-hat_i = A_i / s_{i+1}
            if (MODE == 1 || MODE == 3) {
                const float p = __fmul_rn(psi.h, psi.h);
                const float e = __fmaf_rn(psi.h, psi.h, -p);
                ss.add({p, __fmaf_rn(2.0f * psi.h, psi.l, e)});
                if (MODE == 3) store_psi_pair(out, i, psi, tag);  // absolute scale
            } else {
                const dfl v = df_mul(psi, F);
                out[i] = f2d(v.h) + f2d(v.l);
            }
            q = qn;
        }
        const dfl X = df_add(D, df_mulf(A, -12.0f));
        D = df_add(D, df_mul(T, X));
        const dfl An = df_add(A, df_add(df_mul(T, A), D));
        nodes += (__float_as_uint(An.h) ^ __float_as_uint(A.h)) >> 31;
        A = An;
    }

    // renormalise (exact powers of two) after the step at point i
    __device__ __forceinline__ void renorm(int i) {
        const float mm = fmaxf(fabsf(A.h), fabsf(D.h));
        int e = 0, eq = 0;
        if (mm > 0.0f && mm < INFINITY) {
            e = max(-120, min(120, fexp(mm)));
            const float sc = fpow2(-e);
            A = df_scale(A, sc);
            D = df_scale(D, sc);
            eA += e;
        }
        if (MODE >= 1) {
            eq = max(-120, min(120, fexp(q.h)));
            q = df_scale(q, fpow2(-eq));
            eQ += eq;
            if (MODE == 1 || MODE == 3) {
                ss.rescale(-2 * (e + eq));
                if (MODE == 3) tag = psi_tag(eA + eQ);
                const float mag = fabsf(__fmul_rn(A.h, q.h));
                if (mag > 0.0f) {
                    const int Lm = fexp(mag) + eA + eQ;
                    if (Lm > peak_L) {
                        peak_L = Lm;
                        peak_i = i;
                    }
                }
            } else if (e + eq != 0) {
                F = df_from_double(L * pow2(min(1000, max(-1000, eA + eQ - Xk))));
            }
        }
    }
};

// steps base..nsteps-1 of a side alone (point from + dir * step), 8-step
// chunks renormalised at their ends; one chunk in flight (the double-float
// body is long enough to hide the load behind the other resident warps)
template <int MODE>
__device__ __forceinline__ void side_df_rest(SideDF<MODE>& st, const float2* __restrict__ Wf, dfl aE, int from,
                                             int dir, int base, int nsteps, double* __restrict__ out) {
    for (int b0 = base; b0 < nsteps; b0 += 8) {
        float2 w8[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) w8[u] = __ldg(Wf + from + dir * min(b0 + u, nsteps - 1));
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            if (b0 + u >= nsteps) break;
            st.step(aE, w8[u], out, from + dir * (b0 + u));
        }
        st.renorm(from + dir * min(b0 + 7, nsteps - 1));
    }
}

// one side on its own (the write pass)
template <int MODE>
__device__ __forceinline__ void side_df(const float2* __restrict__ Wf, dfl aE, int from, int to, int dir,
                                        SideDF<MODE>& st, double* __restrict__ out, double L, int Xk) {
    st.init(from, L, Xk);
    side_df_rest(st, Wf, aE, from, dir, 0, (to - from) * dir, out);
    if (MODE == 1 || MODE == 3) st.S = st.ss.value();
}

// one pass at E with match point k over the level's window [w.j0, w.j1];
// MODE 0: gamma/count only, MODE 1: + sums, MODE 3: + unnormalised psi-hat
// into row (the level's psi row).  PAIRED: the outward and inward sides are
// independent recurrences, so their common full chunks can run interleaved
// (two dependency chains per lane) and the rest of the longer side alone; the
// arithmetic of each side is unchanged.  (Measured on GB300: slower for both
// the state-only Newton pass and the norm pass, whose doubled loop bodies
// cost more than the second chain gains; the FP32 lane pass, with a far
// shorter step, does gain from it.)
template <int MODE, bool PAIRED>
__device__ PassDF pass_df(const PotMeta& m, const LevelWork& w, const float2* __restrict__ Wf,
                          const double* __restrict__ W64, double E, int k, double sum_fallback,
                          double* __restrict__ row = nullptr) {
    const dfl aE = energy_df(m, E);
    SideDF<MODE> o, in;
    o.init(w.j0, 0.0, 0);
    in.init(w.j1, 0.0, 0);
    const int no = k - w.j0, ni = w.j1 - k;
    const int nb = PAIRED ? (min(no, ni) & ~7) : 0;
    int base = 0;
    for (; base < nb; base += 8) {
        float2 wo[8], wi[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            wo[u] = __ldg(Wf + w.j0 + base + u);
            wi[u] = __ldg(Wf + w.j1 - base - u);
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            o.step(aE, wo[u], row, w.j0 + base + u);
            in.step(aE, wi[u], row, w.j1 - base - u);
        }
        o.renorm(w.j0 + base + 7);
        in.renorm(w.j1 - base - 7);
    }
    side_df_rest(o, Wf, aE, w.j0, +1, base, no, row);
    side_df_rest(in, Wf, aE, w.j1, -1, base, ni, row);
    if (MODE == 1 || MODE == 3) {
        o.S = o.ss.value();
        in.S = in.ss.value();
    }
    const double Tk = __dsub_rn(__dmul_rn(m.a, E), __ldg(W64 + k));
    const double fk = 1.0 + Tk;
    const double Ao = df_to_double(o.A), Do = df_to_double(o.D);
    const double Ai = df_to_double(in.A), Di = df_to_double(in.D);
    PassDF r;
    // gamma_k = -12 T_k / f_k + D_o / u_k + D_i / v_k in FP64 (no cancellation)
    r.gamma = -12.0 * Tk / fk + Do / Ao + Di / Ai;
    r.nodes = o.nodes + in.nodes;
    r.count = r.nodes + (r.gamma < 0.0 ? 1 : 0);
    r.peak_i = k;
    r.peak_log2 = 0;
    r.pk_out = r.pk_in = 0.0;
    r.ex_out = r.ex_in = 0;
    if (MODE == 1 || MODE == 3) {
        // psi-hat at k from each side: A_k q_k / f_k
        const double rfk = 1.0 / fk;
        r.pk_out = Ao * df_to_double(o.q) * rfk;
        r.pk_in = Ai * df_to_double(in.q) * rfk;
        r.ex_out = o.eA + o.eQ;
        r.ex_in = in.eA + in.eQ;
        r.sum = o.S / (r.pk_out * r.pk_out) + in.S / (r.pk_in * r.pk_in) + 1.0;
        const int Lo = (r.pk_out != 0.0 ? exp_of(fabs(r.pk_out)) : -1000) + r.ex_out;
        const int Li = (r.pk_in != 0.0 ? exp_of(fabs(r.pk_in)) : -1000) + r.ex_in;
        const int po = o.peak_L - Lo, pi = in.peak_L - Li;
        r.peak_log2 = max(po, pi);
        r.peak_i = po >= pi ? o.peak_i : in.peak_i;
    } else {
        r.sum = sum_fallback;
    }
    r.dE = r.gamma * fk * fk / (12.0 * m.a * r.sum);
    return r;
}

// Cooley corrections of the level in slot `slot` from its FP32 energy (one
// or two state-only passes) in an FP64 count bracket.  False when the level
// takes no lane Newton (no bracket, cancelled, a group level) or did not
// settle: such a level is handed to the bisection fallback (fallback_list).
__device__ __forceinline__ bool newton_df_level(const DevBatch& b, int slot) {
    LevelWork w = b.levels[slot];
    if ((w.status & (EPSCU_STATUS_NOTFOUND | EPSCU_STATUS_CANCELLED)) || is_long(w)) return false;
    const PotMeta m = b.meta[w.p];
    const float2* Wf = b.Wf2 + m.offf;
    const double* W = b.W64 + m.off;
    double E = w.E;
    double lo = w.lo - 1e-8, hi = w.hi + 1e-8;
    bool ok = false;
    int n_pass = 0;
    for (int it = 0; it < 4 && !ok; ++it) {
        const PassDF r = pass_df<0, false>(m, w, Wf, W, E, w.k, w.norm_k_in);
        ++n_pass;
        if (r.count > w.v) hi = fmin(hi, E);
        else lo = fmax(lo, E);
        const double En = E + r.dE;
        if (!isfinite(En) || !(En >= lo && En <= hi) || r.nodes != w.v) break;
        // the step divides by the FP32 pass's sum psi~^2 (relative error up
        // to ~1e-4 on long windows), so it leaves ~1e-4 |dE|: one step is
        // enough from within 1e-10, and the norm pass corrects the rest.
        // (A pass with its own sum costs ~1.5x: measured slower overall.)
        ok = fabs(r.dE) <= (it == 0 ? 1e-10 : 1e-12 * fmax(1.0, fabs(E)));
        E = En;
    }
    if (!ok) {
        // hand the level to the bisection fallback kernel (so this warp
        // does not stall on it)
        w.status |= EPSCU_STATUS_FALLBACK;
        const int q = atomicAdd(&b.hdr->fallbacks, 1);
        if (q < b.max_levels) b.fallback_list[q] = slot;
    } else {
        w.E = E;
    }
    {
        const unsigned long long upd = (unsigned long long)n_pass * (unsigned long long)(w.j1 - w.j0);
        atomicAdd(&b.hdr->df_updates, upd);
        atomicMax(&b.hdr->df_max_updates, upd);
    }
    b.levels[slot] = w;
    return ok;
}

// The norm pass of the level in slot `slot` and its match-point candidates:
// sums, node count, peak of |psi| and the constants of the write; with psi
// requested every pass also stores the unnormalised psi-hat in the level's
// row.  False when the level takes no lane norm (a group level, or one the
// fallback refined: norm_long normalises it over the fallback list).
__device__ __forceinline__ bool norm_df_level(const DevBatch& b, int slot) {
    LevelWork w = b.levels[slot];
    if ((w.status & (EPSCU_STATUS_NOTFOUND | EPSCU_STATUS_CANCELLED | EPSCU_STATUS_FALLBACK)) || is_long(w))
        return false;
    const PotMeta m = b.meta[w.p];
    const float2* Wf = b.Wf2 + m.offf;
    const double* W = b.W64 + m.off;
    // with psi requested every pass also stores its unnormalised psi-hat
    // in the level's row; scale_psi applies the constants afterwards
    double* row = psi_row(b, m, w);
    int n_pass = 0;
    auto pass = [&](int kk) {
        ++n_pass;
        return row ? pass_df<3, false>(m, w, Wf, W, w.E, kk, 1.0, row) : pass_df<1, false>(m, w, Wf, W, w.E, kk, 1.0);
    };
    // match point candidates: the FP32 one, the peak of |psi| seen by this
    // pass, the outer turning point and its peak; the first whose
    // stitched solution has v nodes wins
    int k = w.k;
    PassDF r = pass(k);
    if (r.peak_log2 >= 2) {
        k = clamp_k(w, r.peak_i);
        r = pass(k);
    }
    int k_row = k;  // the pass whose psi-hat the row holds
    if (r.nodes != w.v) {
        const int kt = clamp_k(w, match_index(m, b.Msuf, w.E));
        PassDF r2 = pass(kt);
        int k2 = kt;
        if (r2.nodes != w.v && r2.peak_log2 >= 1) {
            k2 = clamp_k(w, r2.peak_i);
            r2 = pass(k2);
        }
        k_row = k2;
        if (r2.nodes == w.v) {
            r = r2;
            k = k2;
        }
    }
    if (redo_norm(w, r)) {
        atomicAdd(&b.hdr->n_redo, 1);
        w.E += r.dE;
        r = pass(k);
    } else if (row && k_row != k) {
        r = pass(k);
    }
    finalize_df(m, w, r, k);
    {
        const unsigned long long upd = (unsigned long long)n_pass * (unsigned long long)(w.j1 - w.j0);
        atomicAdd(&b.hdr->df_updates, upd);
        atomicMax(&b.hdr->df_max_updates, upd);
    }
    if (suspicious(m, w, r.nodes, r.dE) && b.twist_list) {
        const int q = atomicAdd(&b.hdr->n_twist, 1);
        if (q < b.max_twist) b.twist_list[q] = slot;
    }
    b.levels[slot] = w;
    return true;
}

}  // namespace

}  // namespace epscu
