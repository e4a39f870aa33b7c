// longwin.cu -- the fast method's per-level passes for long windows.
//
// A level whose window holds more than kLongWindow points (a long grid: the
// 2^20-point Morse has windows of 10^5 - 4.7 10^5 points) cannot be marched
// by one lane: a pass would cost ~10^6 dependent steps of latency while most
// of the GPU idles.  Such a level takes one CTA of kLongThreads threads
// instead.  Each side of a pass (outward from j0 to the match point k, inward
// from j1 to k) is split into one contiguous chunk per thread and the
// double-float difference-form recurrence
//     D' = D + T (D - 12 A),   A' = A + (T A + D')
// runs in three phases:
//   1. every thread marches the two unit states (A, D) = (1, 0) and (0, 1)
//      through its chunk: the step is linear in (A, D), so these are the
//      columns of the chunk's 2x2 transfer matrix (with the product of 1/f
//      over the chunk for the passes that need psi);
//   2. a parallel prefix scan of the transfer matrices -- Hillis-Steele over
//      the 32 lanes of each warp with shuffles, then over the warps through
//      shared memory -- gives the exact starting state and scale of every
//      chunk;
//   3. every thread re-runs its chunk from that state: node counts, the sum
//      of psi^2, the peak of |psi| or the psi write, reduced over the CTA.
// A pass costs about three serial marches of point-updates, spread over
// kLongThreads threads.  The matrices span exponential growth, so every
// product is renormalised by a power of two with the exponent carried in an
// int; the physical solution is the growing one on both sides (each side runs
// from a forbidden region towards the match point at the peak of |psi|), so a
// product applied to the starting state loses nothing to the discarded
// subdominant solution.
//
// Kernels (one CTA per long level, levels taken from a device queue over the
// long list the window kernel fills; the lane-per-level kernels skip these
// levels):
//   refine_long : from the scan bracket, FP32 passes (the same three phases
//                 in FP32, long_side32) to 2e-9, then double-float
//                 state-only Newton to 1e-12 (replaces refine32 + newton_df);
//                 run again over the levels newton_df could not settle (the
//                 fallback: any window length, full double-float passes from
//                 the scan bracket widened by one trial spacing);
//   norm_long   : the norm pass and its match-point candidates (as norm_df),
//                 storing psi-hat as tagged float pairs for scale_psi;
//   twist_long  : the twist-index search for the levels the norm passes flag;
//   write_long  : psi from the final constants (the adjoint's recompute path).
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "common.cuh"
#include "dfloat.cuh"
#include "dfpass.cuh"
#include "launch.h"

namespace epscu {

namespace {

constexpr int kLongThreads = 256;
constexpr int kLongWarps = kLongThreads / 32;

// [[a, b], [c, d]] 2^e acting on the column (A, D)
struct Mat2 {
    dfl a, b, c, d;
    int e;
};

// v 2^e
struct Scal {
    dfl v;
    int e;
};

__device__ __forceinline__ Mat2 mat_identity() {
    return {{1.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}, {1.0f, 0.0f}, 0};
}

__device__ __forceinline__ void mat_norm(Mat2& m) {
    const float mm = fmaxf(fmaxf(fabsf(m.a.h), fabsf(m.b.h)), fmaxf(fabsf(m.c.h), fabsf(m.d.h)));
    if (mm > 0.0f && mm < INFINITY) {
        const int e = max(-120, min(120, fexp(mm)));
        const float sc = fpow2(-e);
        m.a = df_scale(m.a, sc);
        m.b = df_scale(m.b, sc);
        m.c = df_scale(m.c, sc);
        m.d = df_scale(m.d, sc);
        m.e += e;
    }
}

// x y (x applied after y)
__device__ __forceinline__ Mat2 mat_mul(const Mat2& x, const Mat2& y) {
    Mat2 r;
    r.a = df_add(df_mul(x.a, y.a), df_mul(x.b, y.c));
    r.b = df_add(df_mul(x.a, y.b), df_mul(x.b, y.d));
    r.c = df_add(df_mul(x.c, y.a), df_mul(x.d, y.c));
    r.d = df_add(df_mul(x.c, y.b), df_mul(x.d, y.d));
    r.e = x.e + y.e;
    mat_norm(r);
    return r;
}

__device__ __forceinline__ void scal_norm(Scal& s) {
    const float mm = fabsf(s.v.h);
    if (mm > 0.0f && mm < INFINITY) {
        const int e = max(-120, min(120, fexp(mm)));
        s.v = df_scale(s.v, fpow2(-e));
        s.e += e;
    }
}

__device__ __forceinline__ Scal scal_mul(const Scal& x, const Scal& y) {
    Scal r{df_mul(x.v, y.v), x.e + y.e};
    scal_norm(r);
    return r;
}

__device__ __forceinline__ dfl shfl_up_df(dfl v, int o) {
    return {__shfl_up_sync(0xffffffffu, v.h, o), __shfl_up_sync(0xffffffffu, v.l, o)};
}

__device__ __forceinline__ Mat2 shfl_up_mat(const Mat2& m, int o) {
    return {shfl_up_df(m.a, o), shfl_up_df(m.b, o), shfl_up_df(m.c, o), shfl_up_df(m.d, o),
            __shfl_up_sync(0xffffffffu, m.e, o)};
}

__device__ __forceinline__ Scal shfl_up_scal(const Scal& s, int o) {
    return {shfl_up_df(s.v, o), __shfl_up_sync(0xffffffffu, s.e, o)};
}

// T = aE - W as a double-float (the same operations as the lane passes)
__device__ __forceinline__ dfl t_of(dfl aE, float2 w) {
    const dfl T = two_sum(aE.h, -w.x);
    return fast_two_sum(T.h, __fadd_rn(T.l, __fsub_rn(aE.l, w.y)));
}

__device__ __forceinline__ void df_step(dfl T, dfl& A, dfl& D) {
    const dfl X = df_add(D, df_mulf(A, -12.0f));
    D = df_add(D, df_mul(T, X));
    A = df_add(A, df_add(df_mul(T, A), D));
}

struct LongShared {
    Mat2 wtot[kLongWarps], wpre[kLongWarps];
    Scal qtot[kLongWarps], qpre[kLongWarps];
    int nodes[kLongWarps];
    double S[kLongWarps];
    int pk_L[kLongWarps], pk_s[kLongWarps];
    // the side's final state (written by the thread holding the last chunk)
    dfl A, D, q;
    int eA, eQ;
};

// One side of a pass over steps 0..nsteps-1 (point from + dir * step), the
// CTA-parallel twin of side_df<MODE>: the same outputs in the same scales
// (state and psi-hat at the end with their exponents, S relative to the
// final scale, peak in absolute log2).  Called by every thread of the CTA.
template <int MODE>
struct LongSide {
    dfl A, D, q;
    int eA, eQ;
    int nodes;
    double S;
    int peak_L, peak_i;
};

// The twist-index search (MODE 4: outward sweep storing the sampled ratios,
// MODE 5: inward sweep forming |gamma_k| at the same samples) reuses the
// state-only chunked march; this is its scratch and result.
struct TwistIO {
    double* rho;        // sampled outward ratios (one every kTwistSample points from j0)
    const double* W;    // a V (FP64) of the potential
    double aEd;         // a E in FP64
    int j0, j1, stride;
    double best;        // MODE 5 result: min |gamma_k| over the samples
    int k;              //   and its point
};

template <int MODE>
__device__ LongSide<MODE> long_side(const float2* __restrict__ Wf, dfl aE, int from, int to, int dir,
                                    double* __restrict__ out, double L, int Xk, LongShared& sh,
                                    TwistIO* tw = nullptr) {
    // MODE 0: state, 1: + sums/peak, 2: + psi write, 3: MODE 1 + unnormalised
    // psi-hat written in the absolute scale, 4/5: twist sweeps (state)
    constexpr bool kPsi = MODE == 1 || MODE == 2 || MODE == 3;
    constexpr bool kSums = MODE == 1 || MODE == 3;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nsteps = (to - from) * dir;
    LongSide<MODE> res;
    if (nsteps <= 0) {
        res.A = {1.0f, 0.0f};
        res.D = {1.0f, 0.0f};
        res.q = {1.0f, 0.0f};
        res.eA = res.eQ = 0;
        res.nodes = 0;
        res.S = 0.0;
        res.peak_L = -(1 << 30);
        res.peak_i = from;
        return res;
    }
    const int len = (nsteps + kLongThreads - 1) / kLongThreads;
    const int s0 = min(tid * len, nsteps), s1 = min(s0 + len, nsteps);

    // ---- phase 1: this chunk's transfer matrix (and product of 1/f)
    Mat2 M;
    Scal P{{1.0f, 0.0f}, 0};
    {
        dfl A1 = {1.0f, 0.0f}, D1 = {0.0f, 0.0f}, A2 = {0.0f, 0.0f}, D2 = {1.0f, 0.0f};
        int e = 0;
        for (int st = s0; st < s1; ++st) {
            const dfl T = t_of(aE, __ldg(Wf + from + dir * st));
            if (kPsi) P.v = df_mul(P.v, df_recip(df_add({1.0f, 0.0f}, T)));
            df_step(T, A1, D1);
            df_step(T, A2, D2);
            if (((st - s0) & 7) == 7) {
                const float mm = fmaxf(fmaxf(fabsf(A1.h), fabsf(D1.h)), fmaxf(fabsf(A2.h), fabsf(D2.h)));
                if (mm > 0.0f && mm < INFINITY) {
                    const int ee = max(-120, min(120, fexp(mm)));
                    const float sc = fpow2(-ee);
                    A1 = df_scale(A1, sc);
                    D1 = df_scale(D1, sc);
                    A2 = df_scale(A2, sc);
                    D2 = df_scale(D2, sc);
                    e += ee;
                }
                if (kPsi) scal_norm(P);
            }
        }
        M = {A1, A2, D1, D2, e};
        mat_norm(M);
        if (kPsi) scal_norm(P);
    }

    // ---- phase 2: exclusive prefix of the transfer matrices (later chunks on the left)
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const Mat2 y = shfl_up_mat(M, o);
        const Scal py = shfl_up_scal(P, o);
        if (lane >= o) {
            M = mat_mul(M, y);
            if (kPsi) P = scal_mul(P, py);
        }
    }
    if (lane == 31) {
        sh.wtot[warp] = M;
        sh.qtot[warp] = P;
    }
    __syncthreads();
    if (tid == 0) {
        Mat2 acc = mat_identity();
        Scal qa{{1.0f, 0.0f}, 0};
        for (int w = 0; w < kLongWarps; ++w) {
            sh.wpre[w] = acc;
            sh.qpre[w] = qa;
            acc = mat_mul(sh.wtot[w], acc);
            if (kPsi) qa = scal_mul(sh.qtot[w], qa);
        }
    }
    __syncthreads();
    Mat2 Mx = shfl_up_mat(M, 1);
    Scal Px = shfl_up_scal(P, 1);
    if (lane == 0) {
        Mx = sh.wpre[warp];
        Px = sh.qpre[warp];
    } else {
        Mx = mat_mul(Mx, sh.wpre[warp]);
        if (kPsi) Px = scal_mul(Px, sh.qpre[warp]);
    }

    // ---- phase 3: this chunk from its starting state (A, D) = Mx (1, 1)
    dfl A = df_add(Mx.a, Mx.b), D = df_add(Mx.c, Mx.d);
    int eA = Mx.e;
    {
        const float mm = fmaxf(fabsf(A.h), fabsf(D.h));
        if (mm > 0.0f && mm < INFINITY) {
            const int e = max(-120, min(120, fexp(mm)));
            const float sc = fpow2(-e);
            A = df_scale(A, sc);
            D = df_scale(D, sc);
            eA += e;
        }
    }
    dfl q = Px.v;
    int eQ = Px.e;
    PsiTag tag = psi_tag(MODE == 3 ? eA + eQ : 0);  // the stored pairs' scale and tag
    int nodes = 0;
    double S = 0.0;
    SqSum ss;
    ss.init();
    int peak_L = -(1 << 30), peak_s = 0x7fffffff;
    dfl F = {0.0f, 0.0f};
    if (MODE == 2) F = df_from_double(L * pow2(min(1000, max(-1000, eA + eQ - Xk))));
    double g_best = INFINITY;  // MODE 5
    int g_k = 0x7fffffff;
    for (int st = s0; st < s1; ++st) {
        const int i = from + dir * st;
        const dfl T = t_of(aE, __ldg(Wf + i));
        if (MODE == 4 || MODE == 5) {
            // twist search samples, before the step at i: outward, D/A of the
            // outward state; inward, gamma_i = -12 T_i / f_i + (D/A)_out +
            // (D/A)_in (the lane twist search's formula)
            const int rel = i - tw->j0;
            if (rel % kTwistSample == 0 && rel / kTwistSample < tw->stride) {
                const double ratio = df_to_double(D) / df_to_double(A);
                if (MODE == 4) {
                    tw->rho[rel / kTwistSample] = ratio;
                } else if (i <= tw->j1 - 1) {
                    const double Ti = tw->aEd - __ldg(tw->W + i);
                    const double gam = fabs(-12.0 * Ti / (1.0 + Ti) + tw->rho[rel / kTwistSample] + ratio);
                    if (gam < g_best || (gam == g_best && i < g_k)) {
                        g_best = gam;
                        g_k = i;
                    }
                }
            }
        }
        if (kPsi) {
            const dfl f = df_add({1.0f, 0.0f}, T);
            const dfl qn = df_mul(q, df_recip(f));
            const dfl psi = df_mul(A, qn);
            if (kSums) {
                const float p = __fmul_rn(psi.h, psi.h);
                const float e = __fmaf_rn(psi.h, psi.h, -p);
                ss.add({p, __fmaf_rn(2.0f * psi.h, psi.l, e)});
                if (MODE == 3 && out) store_psi_pair(out, i, psi, tag);  // absolute scale (as side_df)
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
        if (((st - s0) & 7) == 7 || st == s1 - 1) {
            const float mm = fmaxf(fabsf(A.h), fabsf(D.h));
            int e = 0, eq = 0;
            if (mm > 0.0f && mm < INFINITY) {
                e = max(-120, min(120, fexp(mm)));
                const float sc = fpow2(-e);
                A = df_scale(A, sc);
                D = df_scale(D, sc);
                eA += e;
            }
            if (kPsi) {
                eq = max(-120, min(120, fexp(q.h)));
                q = df_scale(q, fpow2(-eq));
                eQ += eq;
                if (kSums) {
                    ss.rescale(-2 * (e + eq));
                    if (MODE == 3) tag = psi_tag(eA + eQ);
                    const float mag = fabsf(__fmul_rn(A.h, q.h));
                    if (mag > 0.0f) {
                        const int Lm = fexp(mag) + eA + eQ;
                        if (Lm > peak_L) {
                            peak_L = Lm;
                            peak_s = st;
                        }
                    }
                } else if (e + eq != 0) {
                    F = df_from_double(L * pow2(min(1000, max(-1000, eA + eQ - Xk))));
                }
            }
        }
    }

    if (kSums) S = ss.value();

    // ---- reductions over the CTA
    const int t_last = (nsteps - 1) / len;
    if (tid == t_last) {
        sh.A = A;
        sh.D = D;
        sh.q = q;
        sh.eA = eA;
        sh.eQ = eQ;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) nodes += __shfl_xor_sync(0xffffffffu, nodes, o);
    if (kSums) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const int L2 = __shfl_xor_sync(0xffffffffu, peak_L, o);
            const int s2 = __shfl_xor_sync(0xffffffffu, peak_s, o);
            if (L2 > peak_L || (L2 == peak_L && s2 < peak_s)) {
                peak_L = L2;
                peak_s = s2;
            }
        }
    }
    if (MODE == 5) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double g2 = __shfl_xor_sync(0xffffffffu, g_best, o);
            const int k2 = __shfl_xor_sync(0xffffffffu, g_k, o);
            if (g2 < g_best || (g2 == g_best && k2 < g_k)) {
                g_best = g2;
                g_k = k2;
            }
        }
        if (lane == 0) {
            sh.S[warp] = g_best;
            sh.pk_s[warp] = g_k;
        }
    }
    if (lane == 0) {
        sh.nodes[warp] = nodes;
        if (MODE != 5) sh.pk_s[warp] = peak_s;
        sh.pk_L[warp] = peak_L;
    }
    __syncthreads();
    res.A = sh.A;
    res.D = sh.D;
    res.q = sh.q;
    res.eA = sh.eA;
    res.eQ = sh.eQ;
    if (kSums) {
        // this chunk's sum in the side's final scale
        const int d = 2 * (eA + eQ - (res.eA + res.eQ));
        double term = (s1 > s0 && d > -1000) ? S * pow2(min(d, 1000)) : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) term += __shfl_xor_sync(0xffffffffu, term, o);
        if (lane == 0) sh.S[warp] = term;
    }
    __syncthreads();
    int nsum = 0;
    double Ssum = 0.0;
    int pL = -(1 << 30), ps = 0x7fffffff;
    for (int w = 0; w < kLongWarps; ++w) {
        nsum += sh.nodes[w];
        if (kSums) {
            Ssum += sh.S[w];
            if (sh.pk_L[w] > pL || (sh.pk_L[w] == pL && sh.pk_s[w] < ps)) {
                pL = sh.pk_L[w];
                ps = sh.pk_s[w];
            }
        }
    }
    res.nodes = nsum;
    res.S = Ssum;
    res.peak_L = pL;
    res.peak_i = ps == 0x7fffffff ? from : from + dir * ps;
    if (MODE == 5) {
        double gb = INFINITY;
        int gk = 0x7fffffff;
        for (int w = 0; w < kLongWarps; ++w)
            if (sh.S[w] < gb || (sh.S[w] == gb && sh.pk_s[w] < gk)) {
                gb = sh.S[w];
                gk = sh.pk_s[w];
            }
        tw->best = gb;
        tw->k = gk;
    }
    __syncthreads();  // the shared scratch is reused by the next call
    return res;
}

// One pass at E with match point k (the CTA twin of pass_df<MODE>, MODE 0/1).
// MODE 3 also stores the unnormalised psi-hat of the window in row (if not null).
template <int MODE>
__device__ PassDF long_pass(const PotMeta& m, const LevelWork& w, const float2* __restrict__ Wf,
                            const double* __restrict__ W64, double E, int k, double sum_fallback, LongShared& sh,
                            double* __restrict__ row = nullptr) {
    const dfl aE = energy_df(m, E);
    const LongSide<MODE> o = long_side<MODE>(Wf, aE, w.j0, k, +1, row, 0.0, 0, sh);
    const LongSide<MODE> in = long_side<MODE>(Wf, aE, w.j1, k, -1, row, 0.0, 0, sh);
    const double Tk = __dsub_rn(__dmul_rn(m.a, E), __ldg(W64 + k));
    const double fk = 1.0 + Tk;
    const double Ao = df_to_double(o.A), Do = df_to_double(o.D);
    const double Ai = df_to_double(in.A), Di = df_to_double(in.D);
    PassDF r;
    r.gamma = -12.0 * Tk / fk + Do / Ao + Di / Ai;
    r.nodes = o.nodes + in.nodes;
    r.count = r.nodes + (r.gamma < 0.0 ? 1 : 0);
    r.peak_i = k;
    r.peak_log2 = 0;
    r.pk_out = r.pk_in = 0.0;
    r.ex_out = r.ex_in = 0;
    if (MODE == 1 || MODE == 3) {
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

// ------------------------------------------------------------------ FP32 passes
// The CTA-parallel twin of the lane kernel's FP32 Cooley pass (refine32): the
// same FP32 recurrence and sums, chunked and scanned as above.  It takes a
// long level from its scan bracket to ~1e-9 at ~1/7 of a double-float pass's
// cost; the double-float passes then only finish the last digits.

// [[a, b], [c, d]] 2^e in FP32
struct Mat2f {
    float a, b, c, d;
    int e;
};

struct Scalf {
    float v;
    int e;
};

__device__ __forceinline__ void matf_norm(Mat2f& m) {
    const float mm = fmaxf(fmaxf(fabsf(m.a), fabsf(m.b)), fmaxf(fabsf(m.c), fabsf(m.d)));
    if (mm > 0.0f && mm < INFINITY) {
        const int e = max(-120, min(120, fexp(mm)));
        const float sc = fpow2(-e);
        m.a *= sc;
        m.b *= sc;
        m.c *= sc;
        m.d *= sc;
        m.e += e;
    }
}

// x y (x applied after y)
__device__ __forceinline__ Mat2f matf_mul(const Mat2f& x, const Mat2f& y) {
    Mat2f r;
    r.a = fmaf(x.a, y.a, x.b * y.c);
    r.b = fmaf(x.a, y.b, x.b * y.d);
    r.c = fmaf(x.c, y.a, x.d * y.c);
    r.d = fmaf(x.c, y.b, x.d * y.d);
    r.e = x.e + y.e;
    matf_norm(r);
    return r;
}

__device__ __forceinline__ void scalf_norm(Scalf& s) {
    const float mm = fabsf(s.v);
    if (mm > 0.0f && mm < INFINITY) {
        const int e = max(-120, min(120, fexp(mm)));
        s.v *= fpow2(-e);
        s.e += e;
    }
}

__device__ __forceinline__ Scalf scalf_mul(const Scalf& x, const Scalf& y) {
    Scalf r{x.v * y.v, x.e + y.e};
    scalf_norm(r);
    return r;
}

__device__ __forceinline__ Mat2f shfl_up_matf(const Mat2f& m, int o) {
    return {__shfl_up_sync(0xffffffffu, m.a, o), __shfl_up_sync(0xffffffffu, m.b, o),
            __shfl_up_sync(0xffffffffu, m.c, o), __shfl_up_sync(0xffffffffu, m.d, o),
            __shfl_up_sync(0xffffffffu, m.e, o)};
}

__device__ __forceinline__ Scalf shfl_up_scalf(const Scalf& s, int o) {
    return {__shfl_up_sync(0xffffffffu, s.v, o), __shfl_up_sync(0xffffffffu, s.e, o)};
}

struct LongShared32 {
    Mat2f wtot[kLongWarps], wpre[kLongWarps];
    Scalf ftot[kLongWarps], fpre[kLongWarps];
    Scalf fall;  // product of f^2 over the side
    int nodes[kLongWarps];
    double S[kLongWarps];
    int pk_L[kLongWarps], pk_s[kLongWarps];
    float A, D;  // the side's final state (thread holding the last chunk)
    int eA;
};

struct LongSide32 {
    float A, D;
    int eA;      // the final state is (A, D) 2^eA
    int nodes;
    double S;    // sum_j A_j^2 prod_{l>j} f_l^2 over the side, in units of 2^(2 eA)
    int peak_L;  // log2 of the largest |A_j| seen at the renormalisations
    int peak_i;
};

// One side in FP32 over steps 0..nsteps-1 (point from + dir * step): the
// state, the node count, the sum S and the peak of |A| exactly as the lane
// pass accumulates them (S' = f^2 S + A^2 before each step), chunked: phase 1
// gives each chunk's transfer matrix and product F of f^2, phase 2 scans
// them, phase 3 re-runs the chunk from its exact start state; a chunk's S is
// carried to the side's end by the product of F over the later chunks.
__device__ LongSide32 long_side32(const float2* __restrict__ Wf, float aEh, float aEl, int from, int to, int dir,
                                  LongShared32& sh) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nsteps = (to - from) * dir;
    LongSide32 res;
    if (nsteps <= 0) {
        res.A = 1.0f;
        res.D = 1.0f;
        res.eA = 0;
        res.nodes = 0;
        res.S = 0.0;
        res.peak_L = -(1 << 30);
        res.peak_i = from;
        return res;
    }
    const int len = (nsteps + kLongThreads - 1) / kLongThreads;
    const int s0 = min(tid * len, nsteps), s1 = min(s0 + len, nsteps);

    // ---- phase 1: transfer matrix and product of f^2 of this chunk
    Mat2f M;
    Scalf F{1.0f, 0};
    {
        float A1 = 1.0f, D1 = 0.0f, A2 = 0.0f, D2 = 1.0f;
        int e = 0;
        for (int st = s0; st < s1; ++st) {
            const float2 w = __ldg(Wf + from + dir * st);
            const float T = (aEh - w.x) + (aEl - w.y);
            const float f = 1.0f + T;
            F.v *= f * f;
            float X = fmaf(-12.0f, A1, D1);
            D1 = fmaf(T, X, D1);
            A1 = A1 + fmaf(T, A1, D1);
            X = fmaf(-12.0f, A2, D2);
            D2 = fmaf(T, X, D2);
            A2 = A2 + fmaf(T, A2, D2);
            if (((st - s0) & 7) == 7) {
                const float mm = fmaxf(fmaxf(fabsf(A1), fabsf(D1)), fmaxf(fabsf(A2), fabsf(D2)));
                if (mm > 0.0f && mm < INFINITY) {
                    const int ee = max(-120, min(120, fexp(mm)));
                    const float sc = fpow2(-ee);
                    A1 *= sc;
                    D1 *= sc;
                    A2 *= sc;
                    D2 *= sc;
                    e += ee;
                }
                scalf_norm(F);
            }
        }
        M = {A1, A2, D1, D2, e};
        matf_norm(M);
        scalf_norm(F);
    }

    // ---- phase 2: exclusive prefix of the matrices, inclusive prefix of F
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const Mat2f y = shfl_up_matf(M, o);
        const Scalf fy = shfl_up_scalf(F, o);
        if (lane >= o) {
            M = matf_mul(M, y);
            F = scalf_mul(F, fy);
        }
    }
    if (lane == 31) {
        sh.wtot[warp] = M;
        sh.ftot[warp] = F;
    }
    __syncthreads();
    if (tid == 0) {
        Mat2f acc = {1.0f, 0.0f, 0.0f, 1.0f, 0};
        Scalf fa{1.0f, 0};
        for (int w = 0; w < kLongWarps; ++w) {
            sh.wpre[w] = acc;
            sh.fpre[w] = fa;
            acc = matf_mul(sh.wtot[w], acc);
            fa = scalf_mul(sh.ftot[w], fa);
        }
        sh.fall = fa;
    }
    __syncthreads();
    Mat2f Mx = shfl_up_matf(M, 1);
    if (lane == 0) Mx = sh.wpre[warp];
    else Mx = matf_mul(Mx, sh.wpre[warp]);
    const Scalf Fin = scalf_mul(F, sh.fpre[warp]);  // f^2 over chunks 0..tid

    // ---- phase 3: this chunk from its start state (A, D) = Mx (1, 1)
    float A = Mx.a + Mx.b, D = Mx.c + Mx.d;
    int eA = Mx.e;
    {
        const float mm = fmaxf(fabsf(A), fabsf(D));
        if (mm > 0.0f && mm < INFINITY) {
            const int e = max(-120, min(120, fexp(mm)));
            const float sc = fpow2(-e);
            A *= sc;
            D *= sc;
            eA += e;
        }
    }
    float S = 0.0f;  // in units of 2^(2 eA)
    int nodes = 0;
    int peak_L = -(1 << 30), peak_s = 0x7fffffff;
    for (int st = s0; st < s1; ++st) {
        const float2 w = __ldg(Wf + from + dir * st);
        const float T = (aEh - w.x) + (aEl - w.y);
        const float f = 1.0f + T;
        S = fmaf(f * f, S, A * A);
        const float X = fmaf(-12.0f, A, D);
        D = fmaf(T, X, D);
        const float An = A + fmaf(T, A, D);
        nodes += (__float_as_uint(An) ^ __float_as_uint(A)) >> 31;
        A = An;
        if (((st - s0) & 7) == 7 || st == s1 - 1) {
            const float mm = fmaxf(fabsf(A), fabsf(D));
            if (mm > 0.0f && mm < INFINITY) {
                const int e = max(-60, min(60, fexp(mm)));
                const float sc = fpow2(-e);
                A *= sc;
                D *= sc;
                S *= sc * sc;
                eA += e;
            }
            if (A != 0.0f) {
                const int L = eA + fexp(fabsf(A));
                if (L > peak_L) {
                    peak_L = L;
                    peak_s = st;
                }
            }
        }
    }

    // ---- reductions over the CTA
    const int t_last = (nsteps - 1) / len;
    if (tid == t_last) {
        sh.A = A;
        sh.D = D;
        sh.eA = eA;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        nodes += __shfl_xor_sync(0xffffffffu, nodes, o);
        const int L2 = __shfl_xor_sync(0xffffffffu, peak_L, o);
        const int s2 = __shfl_xor_sync(0xffffffffu, peak_s, o);
        if (L2 > peak_L || (L2 == peak_L && s2 < peak_s)) {
            peak_L = L2;
            peak_s = s2;
        }
    }
    if (lane == 0) {
        sh.nodes[warp] = nodes;
        sh.pk_L[warp] = peak_L;
        sh.pk_s[warp] = peak_s;
    }
    __syncthreads();
    res.A = sh.A;
    res.D = sh.D;
    res.eA = sh.eA;
    {
        // this chunk's S carried to the side's end (times f^2 over the later
        // chunks = F_all / F_in) in units of 2^(2 eA_final)
        double term = 0.0;
        if (s1 > s0 && S != 0.0f) {
            const int d = 2 * (eA - res.eA) + sh.fall.e - Fin.e;
            if (d > -1000) term = (double)S * ((double)sh.fall.v / (double)Fin.v) * pow2(min(d, 1000));
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) term += __shfl_xor_sync(0xffffffffu, term, o);
        if (lane == 0) sh.S[warp] = term;
    }
    __syncthreads();
    int nsum = 0;
    double Ssum = 0.0;
    int pL = -(1 << 30), ps = 0x7fffffff;
    for (int w = 0; w < kLongWarps; ++w) {
        nsum += sh.nodes[w];
        Ssum += sh.S[w];
        if (sh.pk_L[w] > pL || (sh.pk_L[w] == pL && sh.pk_s[w] < ps)) {
            pL = sh.pk_L[w];
            ps = sh.pk_s[w];
        }
    }
    res.nodes = nsum;
    res.S = Ssum;
    res.peak_L = pL;
    res.peak_i = ps == 0x7fffffff ? from : from + dir * ps;
    __syncthreads();  // the shared scratch is reused by the next call
    return res;
}

// One FP32 pass at E with match point k (the CTA twin of the lane pass):
// Cooley correction, count, sum and the peak of |psi| relative to psi_k.
__device__ PassDF long_pass32(const PotMeta& m, const LevelWork& w, const float2* __restrict__ Wf,
                              const double* __restrict__ W64, double E, int k, LongShared32& sh) {
    const double aE = __dmul_rn(m.a, E);
    const float aEh = __double2float_rn(aE);
    const float aEl = __double2float_rn(aE - (double)aEh);
    const LongSide32 o = long_side32(Wf, aEh, aEl, w.j0, k, +1, sh);
    const LongSide32 in = long_side32(Wf, aEh, aEl, w.j1, k, -1, sh);
    const double Tk = aE - __ldg(W64 + k);
    const double fk = 1.0 + Tk;
    const double uA = o.A, vC = in.A;
    PassDF r;
    // gamma_k = -12 T_k / f_k + D_o / u_k + D_i / v_k   (no cancellation)
    r.gamma = -12.0 * Tk / fk + (double)o.D / uA + (double)in.D / vC;
    const double fk2 = fk * fk;
    r.sum = fk2 * (o.S / (uA * uA) + in.S / (vC * vC)) + 1.0;
    r.dE = r.gamma * fk2 / (12.0 * m.a * r.sum);
    r.nodes = o.nodes + in.nodes;
    r.count = r.nodes + (r.gamma < 0.0 ? 1 : 0);
    const int Lo = o.eA + (o.A != 0.0f ? fexp(fabsf(o.A)) : -1000);
    const int Li = in.eA + (in.A != 0.0f ? fexp(fabsf(in.A)) : -1000);
    const int po = o.peak_L - Lo, pi = in.peak_L - Li;
    r.peak_log2 = max(po, pi);
    r.peak_i = po >= pi ? o.peak_i : in.peak_i;
    r.pk_out = r.pk_in = 0.0;
    r.ex_out = r.ex_in = 0;
    return r;
}

__device__ __forceinline__ bool cancelled(const DevBatch& b) { return b.cancel && *b.cancel; }

// Long levels from their scan bracket, in three stages:
//   1. FP32 passes (long_pass32): safeguarded Cooley-Newton to |dE| <= 2e-9
//      with the count bracket, the match point moved to the peak of |psi|;
//   2. double-float state-only passes with the FP32 sum as the Newton
//      denominator (as newton_df): usually one step, accepted from within
//      1e-8 (the chunked FP32 sum is accurate to ~1e-6);
//   3. if stage 2 does not settle (the FP32 counts are off near a trial
//      energy, or the pass sees another node count): safeguarded
//      Cooley-Newton in double-float with full sums from the scan bracket
//      widened by one trial spacing.  Every pass updates the count bracket;
//      Newton steps are taken only while the pass sees the level's own node
//      count (so a neighbouring level cannot attract the iteration) and stay
//      inside the bracket, bisection otherwise.  After the match point moves
//      to the peak of |psi| the pass is redone at the same E.
// fallback = 0: the long list (stages 1-3); 1: the levels newton_df handed
// over (stage 3 only).
constexpr double kTol32Long = 2e-9;

__global__ void __launch_bounds__(kLongThreads) refine_long_kernel(DevBatch b, int fallback) {
    __shared__ LongShared sh;
    __shared__ LongShared32 sh32;
    const int n = fallback ? min(b.hdr->fallbacks, b.max_levels) : min(b.hdr->n_long, b.max_levels);
    const int32_t* list = fallback ? b.fallback_list : b.long_list;
    __shared__ int s_q;
    // levels from a device queue (a CTA takes the next as it finishes one)
    for (;;) {
        if (threadIdx.x == 0) s_q = atomicAdd(&b.hdr->queue[fallback ? kQFallback : kQLongRefine], 1);
        __syncthreads();
        const int q = s_q;
        __syncthreads();  // every thread has read s_q
        if (q >= n) break;
        const int slot = list[q];
        LevelWork w = b.levels[slot];
        if (w.status & EPSCU_STATUS_NOTFOUND) continue;
        if (cancelled(b)) {
            if (threadIdx.x == 0) b.levels[slot].status = w.status | EPSCU_STATUS_CANCELLED;
            continue;
        }
        const PotMeta m = b.meta[w.p];
        const float2* Wf = b.Wf2 + m.offf;
        const double* W = b.W64 + m.off;
        double lo = w.lo, hi = w.hi, E = w.E, sum = 1.0;
        int k = clamp_k(w, match_index(m, b.Msuf, E));
        bool done = false;
        int n_pass = 0, n_pass32 = 0;
        if (!fallback) {
            // ---- stage 1: FP32
            bool moved_last = false, ok32 = false;
            for (int it = 0, cap = refine_cap(b); it < cap; ++it) {
                const PassDF r = long_pass32(m, w, Wf, W, E, k, sh32);
                ++n_pass32;
                sum = r.sum;
                if (r.count > w.v) hi = E;
                else lo = E;
                if (r.peak_log2 >= 2 && !moved_last) {
                    k = clamp_k(w, r.peak_i);
                    moved_last = true;
                    continue;  // the same energy at the new match point
                }
                moved_last = false;
                const double En = E + r.dE;
                const bool near = r.nodes == w.v || (m.status & EPSCU_STATUS_UNDER);
                if (near && isfinite(En) && En > lo && En < hi) {
                    E = En;
                    if (fabs(r.dE) <= kTol32Long) {
                        ok32 = true;
                        break;
                    }
                } else {
                    E = 0.5 * (lo + hi);
                }
                if (hi - lo <= 2.0 * kTol32Long) {
                    E = 0.5 * (lo + hi);
                    ok32 = true;
                    break;
                }
            }
            // ---- stage 2: double-float state-only Newton (FP32 sum)
            if (ok32) {
                double lo2 = lo - 1e-8, hi2 = hi + 1e-8;
                for (int it = 0; it < 4 && !done; ++it) {
                    const PassDF r = long_pass<0>(m, w, Wf, W, E, k, sum, sh);
                    ++n_pass;
                    if (r.count > w.v) hi2 = fmin(hi2, E);
                    else lo2 = fmax(lo2, E);
                    const double En = E + r.dE;
                    if (!isfinite(En) || !(En >= lo2 && En <= hi2) || r.nodes != w.v) break;
                    // the FP32 sum of the CTA pass is accurate to ~1e-6 (chunk
                    // sums of a few hundred terms, added in FP64), so one step
                    // from within 1e-8 leaves ~1e-14: the first pass settles
                    done = fabs(r.dE) <= (it == 0 ? 1e-8 * fmax(1.0, fabs(E)) : 1e-12 * fmax(1.0, fabs(E)));
                    E = En;
                }
                if (done) {
                    lo = lo2;
                    hi = hi2;
                }
            }
        }
        if (!done) {
            // ---- stage 3: the FP32 bracket may be off by its count errors:
            // restart from the scan bracket widened by one trial spacing
            lo = fmax(m.e_lo, w.lo0 - m.delta);
            hi = fmin(m.e_cap, w.hi0 + m.delta);
            if (!(E > lo && E < hi)) E = 0.5 * (lo + hi);
            bool moved_last = false;
            for (int it = 0, cap = fallback_cap(b); it < cap; ++it) {
                const PassDF r = long_pass<1>(m, w, Wf, W, E, k, 1.0, sh);
                ++n_pass;
                sum = r.sum;
                if (r.count > w.v) hi = E;
                else lo = E;
                if (r.peak_log2 >= 2 && !moved_last) {
                    k = clamp_k(w, r.peak_i);
                    moved_last = true;
                    continue;  // the same energy at the new match point
                }
                moved_last = false;
                const double tol = 1e-12 * fmax(1.0, fabs(E));
                const double En = E + r.dE;
                const bool near = r.nodes == w.v || (m.status & EPSCU_STATUS_UNDER);
                if (near && isfinite(En) && En > lo && En < hi) {
                    E = En;
                    if (fabs(r.dE) <= tol) {
                        done = true;
                        break;
                    }
                } else {
                    E = 0.5 * (lo + hi);
                }
                if (hi - lo <= tol) {
                    E = 0.5 * (lo + hi);
                    done = true;
                    break;
                }
            }
        }
        if (threadIdx.x == 0) {
            if (!done) w.status |= EPSCU_STATUS_MAXITER;
            w.status &= ~EPSCU_STATUS_FALLBACK;
            w.lo = lo;
            w.hi = hi;
            w.E = E;
            w.k = k;
            w.norm_k_in = sum;
            w.iters = n_pass32 + n_pass;
            const unsigned long long pts = (unsigned long long)(w.j1 - w.j0);
            atomicAdd(&b.hdr->refine_updates, (unsigned long long)n_pass32 * pts);
            atomicAdd(&b.hdr->df_updates, (unsigned long long)n_pass * pts);
            if (!fallback) {
                atomicAdd(&b.hdr->long32_updates, (unsigned long long)n_pass32 * pts);
                atomicAdd(&b.hdr->longdf_updates, (unsigned long long)n_pass * pts);
            }
            b.levels[slot] = w;
        }
        __syncthreads();
    }
}

// The norm pass of a long level and its match-point candidates (as norm_df).
// With psi requested every pass also stores its unnormalised psi-hat in the
// level's row (MODE 3) and the last pass is the one kept; scale_psi applies
// the constants afterwards.
__global__ void __launch_bounds__(kLongThreads) norm_long_kernel(DevBatch b) {
    __shared__ LongShared sh;
    const int n = min(b.hdr->n_long, b.max_levels);
    __shared__ int s_q;
    // levels from a device queue (a CTA takes the next as it finishes one)
    for (;;) {
        if (threadIdx.x == 0) s_q = atomicAdd(&b.hdr->queue[kQNormLong], 1);
        __syncthreads();
        const int q = s_q;
        __syncthreads();  // every thread has read s_q
        if (q >= n) break;
        const int slot = b.long_list[q];
        LevelWork w = b.levels[slot];
        if (w.status & (EPSCU_STATUS_NOTFOUND | EPSCU_STATUS_CANCELLED)) continue;
        const PotMeta m = b.meta[w.p];
        const float2* Wf = b.Wf2 + m.offf;
        const double* W = b.W64 + m.off;
        double* row = psi_row(b, m, w);
        auto pass = [&](int kk) { return long_pass<3>(m, w, Wf, W, w.E, kk, 1.0, sh, row); };
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
            if (threadIdx.x == 0) atomicAdd(&b.hdr->n_redo, 1);
            w.E += r.dE;
            r = pass(k);
        } else if (row && k_row != k) {
            r = pass(k);
        }
        finalize_df(m, w, r, k);
        if (threadIdx.x == 0) {
            if (suspicious(m, w, r.nodes, r.dE) && b.twist_list) {
                const int t = atomicAdd(&b.hdr->n_twist, 1);
                if (t < b.max_twist) b.twist_list[t] = slot;
            }
            b.levels[slot] = w;
        }
        __syncthreads();
    }
}

// Twist-index search for the levels the norm passes flagged (any window
// length): a chunked outward sweep stores D/A every kTwistSample points, a
// chunked inward sweep forms |gamma_k| at the same points, the match point
// becomes argmin |gamma_k| (Dhillon and Parlett's twisted-factorisation
// rule), then Newton and the norm pass run there; with psi requested the
// final pass stores the unnormalised psi-hat in the level's row (scale_psi
// applies the constants).  The level joins the long list, so the adjoint's
// recompute path (write_long) writes its psi.
__global__ void __launch_bounds__(kLongThreads) twist_long_kernel(DevBatch b) {
    __shared__ LongShared sh;
    const int n = min(b.hdr->n_twist, b.max_twist);
    __shared__ int s_q;
    // levels from a device queue (a CTA takes the next as it finishes one)
    for (;;) {
        if (threadIdx.x == 0) s_q = atomicAdd(&b.hdr->queue[kQTwistLong], 1);
        __syncthreads();
        const int q = s_q;
        __syncthreads();  // every thread has read s_q
        if (q >= n) break;
        const int slot = b.twist_list[q];
        LevelWork w = b.levels[slot];
        const PotMeta m = b.meta[w.p];
        const float2* Wf = b.Wf2 + m.offf;
        const double* W = b.W64 + m.off;
        const dfl aE = energy_df(m, w.E);
        TwistIO tw;
        tw.rho = b.twist_scratch + (int64_t)q * b.twist_stride;
        tw.W = W;
        tw.aEd = __dmul_rn(m.a, w.E);
        tw.j0 = w.j0;
        tw.j1 = w.j1;
        tw.stride = b.twist_stride;
        tw.best = INFINITY;
        tw.k = w.k;
        long_side<4>(Wf, aE, w.j0, w.j1, +1, nullptr, 0.0, 0, sh, &tw);
        long_side<5>(Wf, aE, w.j1, w.j0, -1, nullptr, 0.0, 0, sh, &tw);
        const int k = clamp_k(w, tw.k == 0x7fffffff ? w.k : tw.k);
        double* row = psi_row(b, m, w);
        auto pass = [&](double e) { return long_pass<3>(m, w, Wf, W, e, k, 1.0, sh, row); };
        double E1 = w.E;
        PassDF r = pass(E1);
        for (int it = 0; it < 8; ++it) {
            if (r.nodes != w.v || !isfinite(r.dE) || !(fabs(r.dE) < 1e-7)) break;
            if (fabs(r.dE) <= 1e-13 * fmax(1.0, fabs(E1))) break;
            E1 += r.dE;
            r = pass(E1);
        }
        w.E = E1;
        finalize_df(m, w, r, k);
        if (threadIdx.x == 0) {
            if (!(w.status & EPSCU_STATUS_LONG) && b.long_list) {
                const int t = atomicAdd(&b.hdr->n_long, 1);
                if (t < b.max_levels) {
                    b.long_list[t] = slot;
                    w.status |= EPSCU_STATUS_LONG;
                }
            }
            b.levels[slot] = w;
        }
        __syncthreads();
    }
}

// psi of the long levels in FP64 from the final constants (window points and
// psi_k; the rest of each row is zero): the adjoint's recompute path.
__global__ void __launch_bounds__(kLongThreads) write_long_kernel(DevBatch b) {
    __shared__ LongShared sh;
    if (!b.psi || b.hdr->error) return;
    const int n = min(b.hdr->n_long, b.max_levels);
    for (int q = blockIdx.x; q < n; q += gridDim.x) {
        const int slot = b.long_list[q];
        const LevelWork w = b.levels[slot];
        const PotMeta m = b.meta[w.p];
        double* out = b.psi + m.psi_off + (int64_t)(w.v - b.min_level) * m.N;
        // the rows were zeroed by zero_psi: only the window is written
        if (no_result(w)) continue;
        const float2* Wf = b.Wf2 + m.offf;
        const dfl aE = energy_df(m, w.E);
        long_side<2>(Wf, aE, w.j0, w.k, +1, out, w.norm_k_out, w.ex_out, sh);
        long_side<2>(Wf, aE, w.j1, w.k, -1, out, w.norm_k_in, w.ex_in, sh);
        if (threadIdx.x == 0) out[w.k] = w.ck;
    }
}

}  // namespace

void launch_refine_long(const DevBatch& b, int sm_count, cudaStream_t s) {
    if (!b.long_list) return;
    refine_long_kernel<<<sm_count * 2, kLongThreads, 0, s>>>(b, 0);
}
void launch_fallback_long(const DevBatch& b, int sm_count, cudaStream_t s) {
    if (!b.fallback_list) return;
    refine_long_kernel<<<sm_count * 2, kLongThreads, 0, s>>>(b, 1);
}
void launch_norm_long(const DevBatch& b, int sm_count, cudaStream_t s) {
    if (!b.long_list) return;
    norm_long_kernel<<<sm_count * 2, kLongThreads, 0, s>>>(b);
}
void launch_twist_long(const DevBatch& b, int sm_count, cudaStream_t s) {
    if (!b.twist_list || !b.long_list) return;
    twist_long_kernel<<<sm_count * 2, kLongThreads, 0, s>>>(b);
}
void launch_write_long(const DevBatch& b, int sm_count, cudaStream_t s) {
    if (!b.long_list) return;
    write_long_kernel<<<sm_count * 2, kLongThreads, 0, s>>>(b);
}

}  // namespace epscu
