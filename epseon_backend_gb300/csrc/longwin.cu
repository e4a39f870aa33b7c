// longwin.cu -- the fast method's per-level passes on groups of warps.
//
// A level whose window is long (a long grid: the 2^20-point Morse has windows
// of 10^5 - 4.7 10^5 points; on the mixed batch every window above a few
// thousand points) cannot be marched by one lane: a pass would cost ~10^4 -
// 10^6 dependent steps of latency while most of the GPU idles.  Such a level
// takes a group of NW warps instead: the whole CTA (NW = 8) for the longest
// windows, or one warp (NW = 1) for the middle tier.  Each side of a pass
// (outward from j0 to the match point k, inward from j1 to k) is split into
// one contiguous chunk per thread of the group and the double-float
// difference-form recurrence
//     D' = D + T (D - 12 A),   A' = A + (T A + D')
// runs in three phases:
//   1. every thread marches the two unit states (A, D) = (1, 0) and (0, 1)
//      through its chunk: the step is linear in (A, D), so these are the
//      columns of the chunk's 2x2 transfer matrix (with the product of 1/f
//      over the chunk for the passes that need psi);
//   2. a parallel prefix scan of the transfer matrices -- Hillis-Steele over
//      the 32 lanes of each warp with shuffles, then over the group's warps
//      through shared memory -- gives the exact starting state and scale of
//      every chunk;
//   3. every thread re-runs its chunk from that state: node counts, the sum
//      of psi^2, the peak of |psi| or the psi write, reduced over the group.
// A pass costs about three serial marches of point-updates, spread over the
// group.  The matrices span exponential growth, so every product is
// renormalised by a power of two with the exponent carried in an int; the
// physical solution is the growing one on both sides (each side runs from a
// forbidden region towards the match point at the peak of |psi|), so a
// product applied to the starting state loses nothing to the discarded
// subdominant solution.
//
// FP64 runs once per pass, in the group's thread 0 (the leader): the sums are
// reduced over the warps in FP32 (FP32 passes) or double-float (double-float
// passes) with their binary exponents aligned, and the leader forms the
// side's sum in FP64, the matching function gamma_k, the psi^2 sum and the
// Cooley step, and hands the pass's result to the group through shared
// memory.  (Every thread doing that FP64 work kept the FP64 pipe, 1/62 of the
// FP32 rate on GB300, busy for a large part of a pass on windows of a few
// thousand points per CTA.)
//
// Kernels (one group per level, levels taken from a device queue over a list
// the window kernel fills; the lane-per-level kernels skip these levels):
//   refine_long : from the scan bracket, FP32 passes (the same three phases
//                 in FP32, long_side32) to a Newton step of 3e-8, then double-float
//                 state-only Newton to 1e-12 (replaces refine32 + newton_df);
//                 run again over the levels newton_df could not settle (the
//                 fallback: any window length, full double-float passes from
//                 the scan bracket widened by one trial spacing), and over
//                 the middle list from the lane FP32 refinement's result;
//   norm_long   : the norm pass and its match-point candidates (as norm_df),
//                 storing psi-hat as tagged float pairs for scale_psi; run
//                 over the long list and over the fallback list;
//   twist_long  : the twist-index search for the levels the norm passes flag;
//   write_long  : psi from the final constants (the adjoint's recompute path;
//                 the long, middle and fallback lists).
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "common.cuh"
#include "dfloat.cuh"
#include "dfpass.cuh"
#include "launch.h"

namespace epscu {

namespace {

// CTA shape of the group passes: threads per CTA and the persistent grid's
// CTAs per SM
constexpr int kLongThreads = 256;
constexpr int kLongWarps = kLongThreads / 32;
constexpr int kLongCtasPerSm = 2;

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

// ---------------------------------------------------------------- groups
// A level's passes run on a group of NW warps (NW = 8: the whole CTA of
// kLongThreads; NW = 1: one warp, kLongThreads / 32 groups per CTA).  The
// group's thread 0 is its leader.
template <int NW>
struct Grp {
    static constexpr int kThreads = 32 * NW;
    // thread in the group, lane, warp in the group, group in the CTA (read
    // from threadIdx each time: nothing held in registers)
    __device__ __forceinline__ int t() const { return (int)(threadIdx.x % kThreads); }
    __device__ __forceinline__ int lane() const { return (int)(threadIdx.x & 31); }
    __device__ __forceinline__ int warp() const { return (int)((threadIdx.x % kThreads) >> 5); }
    __device__ __forceinline__ int g() const { return (int)(threadIdx.x / kThreads); }
    __device__ __forceinline__ bool leader() const { return t() == 0; }
};

template <int NW>
__device__ __forceinline__ void gsync() {
    static_assert(NW == 1 || NW == kLongWarps, "a group is one warp or the whole CTA");
    if constexpr (NW == 1) __syncwarp();
    else __syncthreads();
}

// the leader's value to the whole group (slot: the group's shared word)
template <int NW>
__device__ __forceinline__ int grp_bcast(const Grp<NW>& G, int v, int& slot) {
    if constexpr (NW == 1) {
        return __shfl_sync(0xffffffffu, v, 0);
    } else {
        if (G.leader()) slot = v;
        __syncthreads();
        const int r = slot;
        __syncthreads();  // every thread has read the slot
        return r;
    }
}

// the next entry of a device queue for the group
template <int NW>
__device__ __forceinline__ int grp_next(const Grp<NW>& G, int* queue, int& slot) {
    int q = 0;
    if (G.leader()) q = atomicAdd(queue, 1);
    return grp_bcast<NW>(G, q, slot);
}

// A non-negative sum (h + l) 2^e in double-float, and its warp-wide total:
// each lane's value aligned to the largest exponent of the warp (exact
// power-of-two scalings), then added with shuffles.  Lane 0's result is the
// one used (the butterfly's order is fixed, so it is reproducible).
struct DfE {
    dfl v;
    int e;
};

__device__ __forceinline__ DfE warp_sum_dfe(DfE x) {
    const bool has = x.v.h > 0.0f;
    int em = has ? x.e : -(1 << 30);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) em = max(em, __shfl_xor_sync(0xffffffffu, em, o));
    dfl v = {0.0f, 0.0f};
    if (has) {
        const int d = x.e - em;
        if (d > -120) v = df_scale(x.v, fpow2(d));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v = df_add(v, {__shfl_xor_sync(0xffffffffu, v.h, o), __shfl_xor_sync(0xffffffffu, v.l, o)});
    return {v, em};
}

// The same for FP32 sums v 2^e.
struct FE {
    float v;
    int e;
};

__device__ __forceinline__ FE warp_sum_fe(FE x) {
    const bool has = x.v > 0.0f;
    int em = has ? x.e : -(1 << 30);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) em = max(em, __shfl_xor_sync(0xffffffffu, em, o));
    float v = 0.0f;
    if (has) {
        const int d = x.e - em;
        if (d > -120) v = x.v * fpow2(d);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return {v, em};
}

// a thread's SqSum (in units of 2^e0) as a DfE; the FP64 spill is rare
__device__ __forceinline__ DfE sqsum_dfe(const SqSum& ss, int e0) {
    if (ss.x == 0.0) return {ss.d, e0};
    const double v = ss.value();
    if (!(v > 0.0) || !isfinite(v)) return {{0.0f, 0.0f}, e0};
    const int ex = exp_of(v);
    return {df_from_double(v * pow2(-ex)), e0 + ex};
}

// (h + l) 2^e in FP64 (the leader's combine)
__device__ __forceinline__ double dfe_to_double(DfE x) {
    if (!(x.v.h > 0.0f)) return 0.0;
    return (f2d(x.v.h) + f2d(x.v.l)) * pow2(max(-1000, min(1000, x.e)));
}

// ------------------------------------------------------- double-float sides
template <int NW>
struct SharedDF {
    Mat2 wtot[NW], wpre[NW];
    Scal qtot[NW], qpre[NW];
    int nodes[NW];
    DfE s[NW];  // warp partial sums of psi-hat^2, absolute exponents
    int pk_L[NW], pk_s[NW];
    double gb[NW];  // MODE 5: warp minima of |gamma| and their points
    int gk[NW];
    // the side's final state (written by the thread holding the last chunk)
    dfl A, D, q;
    int eA, eQ;
    // the leader's broadcasts: the pass energy and the pass result
    dfl aE;
    PassDF res;
    int word;  // grp_bcast / grp_next slot
};

// One side of a pass over steps 0..nsteps-1 (point from + dir * step), the
// group-parallel twin of side_df<MODE>: the same outputs in the same scales
// (state and psi-hat at the end with their exponents, S relative to the
// final scale, peak in absolute log2), valid in the leader.  Called by every
// thread of the group.
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
// state-only chunked march; this is its scratch and result (the result is
// handed to every thread of the group).
struct TwistIO {
    double* rho;        // sampled outward ratios (one every kTwistSample points from j0)
    const double* W;    // a V (FP64) of the potential
    double aEd;         // a E in FP64
    int j0, j1, stride;
    double best;        // MODE 5 result: min |gamma_k| over the samples
    int k;              //   and its point
};

template <int NW, int MODE>
__device__ LongSide<MODE> long_side(const Grp<NW>& G, const float2* __restrict__ Wf, dfl aE, int from, int to,
                                    int dir, double* __restrict__ out, double L, int Xk, SharedDF<NW>& sh,
                                    TwistIO* tw = nullptr) {
    // MODE 0: state, 1: + sums/peak, 2: + psi write, 3: MODE 1 + unnormalised
    // psi-hat written in the absolute scale, 4/5: twist sweeps (state)
    constexpr bool kPsi = MODE == 1 || MODE == 2 || MODE == 3;
    constexpr bool kSums = MODE == 1 || MODE == 3;
    constexpr int kT = Grp<NW>::kThreads;
    const int tid = G.t(), lane = G.lane(), warp = G.warp();
    const int nsteps = (to - from) * dir;
    LongSide<MODE> res;
    if (nsteps <= 0) {  // uniform over the group: no barrier is skipped by part of it
        res.A = {1.0f, 0.0f};
        res.D = {1.0f, 0.0f};
        res.q = {1.0f, 0.0f};
        res.eA = res.eQ = 0;
        res.nodes = 0;
        res.S = 0.0;
        res.peak_L = -(1 << 30);
        res.peak_i = from;
        if (MODE == 5) {
            tw->best = INFINITY;
            tw->k = 0x7fffffff;
        }
        return res;
    }
    const int len = (nsteps + kT - 1) / kT;
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
    Mat2 Mx = shfl_up_mat(M, 1);
    Scal Px = shfl_up_scal(P, 1);
    if constexpr (NW > 1) {
        if (lane == 31) {
            sh.wtot[warp] = M;
            sh.qtot[warp] = P;
        }
        gsync<NW>();
        if (tid == 0) {
            Mat2 acc = mat_identity();
            Scal qa{{1.0f, 0.0f}, 0};
            for (int w = 0; w < NW; ++w) {
                sh.wpre[w] = acc;
                sh.qpre[w] = qa;
                acc = mat_mul(sh.wtot[w], acc);
                if (kPsi) qa = scal_mul(sh.qtot[w], qa);
            }
        }
        gsync<NW>();
        if (lane == 0) {
            Mx = sh.wpre[warp];
            Px = sh.qpre[warp];
        } else {
            Mx = mat_mul(Mx, sh.wpre[warp]);
            if (kPsi) Px = scal_mul(Px, sh.qpre[warp]);
        }
    } else if (lane == 0) {
        Mx = mat_identity();
        Px = {{1.0f, 0.0f}, 0};
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

    // ---- reductions: over each warp with shuffles, over the warps by the leader
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
    DfE sw{{0.0f, 0.0f}, 0};
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
        // this chunk's sum in the absolute scale 2^(2 (eA + eQ))
        sw = warp_sum_dfe(s1 > s0 ? sqsum_dfe(ss, 2 * (eA + eQ)) : DfE{{0.0f, 0.0f}, 0});
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
    }
    if (lane == 0) {
        sh.nodes[warp] = nodes;
        sh.pk_L[warp] = peak_L;
        sh.pk_s[warp] = peak_s;
        if (kSums) sh.s[warp] = sw;
        if (MODE == 5) {
            sh.gb[warp] = g_best;
            sh.gk[warp] = g_k;
        }
    }
    gsync<NW>();
    if (G.leader()) {
        res.A = sh.A;
        res.D = sh.D;
        res.q = sh.q;
        res.eA = sh.eA;
        res.eQ = sh.eQ;
        int nsum = 0;
        double Ssum = 0.0;
        int pL = -(1 << 30), ps = 0x7fffffff;
        for (int w = 0; w < NW; ++w) {
            nsum += sh.nodes[w];
            if (kSums) {
                // the warp's sum in the side's final scale
                DfE x = sh.s[w];
                x.e -= 2 * (res.eA + res.eQ);
                Ssum += dfe_to_double(x);
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
    }
    if (MODE == 5) {
        // every thread of the group takes the search's result
        double gb = INFINITY;
        int gk = 0x7fffffff;
        for (int w = 0; w < NW; ++w)
            if (sh.gb[w] < gb || (sh.gb[w] == gb && sh.gk[w] < gk)) {
                gb = sh.gb[w];
                gk = sh.gk[w];
            }
        tw->best = gb;
        tw->k = gk;
    }
    // (no barrier here: the next writes of these fields come after the next
    // call's phase-2 barriers, which the leader reaches only after its reads)
    return res;
}

// One pass at E with match point k (the group twin of pass_df<MODE>): the
// leader turns the two sides into the Cooley correction, the count, the sum
// and the peak, and hands the result to the group.  MODE 3 also stores the
// unnormalised psi-hat of the window in row (if not null).
template <int NW, int MODE>
__device__ __forceinline__ PassDF long_pass(const Grp<NW>& G, const PotMeta& m, const LevelWork& w,
                                            const float2* __restrict__ Wf, const double* __restrict__ W64, double E,
                                            int k, double sum_fallback, SharedDF<NW>& sh,
                                            double* __restrict__ row = nullptr) {
    if (G.leader()) sh.aE = energy_df(m, E);
    gsync<NW>();
    const dfl aE = sh.aE;
    const LongSide<MODE> o = long_side<NW, MODE>(G, Wf, aE, w.j0, k, +1, row, 0.0, 0, sh);
    const LongSide<MODE> in = long_side<NW, MODE>(G, Wf, aE, w.j1, k, -1, row, 0.0, 0, sh);
    if (G.leader()) {
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
        sh.res = r;
    }
    gsync<NW>();
    return sh.res;
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

template <int NW>
struct Shared32 {
    Mat2f wtot[NW], wpre[NW];
    Scalf ftot[NW], fpre[NW];
    Scalf fall;  // product of f^2 over the side
    int nodes[NW];
    FE s[NW];  // warp partial sums, absolute exponents
    int pk_L[NW], pk_s[NW];
    float A, D;  // the side's final state (thread holding the last chunk)
    int eA;
    // the leader's broadcasts: a E as a float pair and the pass result
    float aEh, aEl;
    PassDF res;
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
// carried to the side's end by the product of F over the later chunks.  The
// result is valid in the leader.
template <int NW>
__device__ LongSide32 long_side32(const Grp<NW>& G, const float2* __restrict__ Wf, float aEh, float aEl, int from,
                                  int to, int dir, Shared32<NW>& sh) {
    constexpr int kT = Grp<NW>::kThreads;
    const int tid = G.t(), lane = G.lane(), warp = G.warp();
    const int nsteps = (to - from) * dir;
    LongSide32 res;
    if (nsteps <= 0) {  // uniform over the group
        res.A = 1.0f;
        res.D = 1.0f;
        res.eA = 0;
        res.nodes = 0;
        res.S = 0.0;
        res.peak_L = -(1 << 30);
        res.peak_i = from;
        return res;
    }
    const int len = (nsteps + kT - 1) / kT;
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
    Mat2f Mx = shfl_up_matf(M, 1);
    Scalf Fin = F;  // f^2 over the chunks up to this thread's
    Scalf Fall;     // f^2 over the side
    if constexpr (NW > 1) {
        if (lane == 31) {
            sh.wtot[warp] = M;
            sh.ftot[warp] = F;
        }
        gsync<NW>();
        if (tid == 0) {
            Mat2f acc = {1.0f, 0.0f, 0.0f, 1.0f, 0};
            Scalf fa{1.0f, 0};
            for (int w = 0; w < NW; ++w) {
                sh.wpre[w] = acc;
                sh.fpre[w] = fa;
                acc = matf_mul(sh.wtot[w], acc);
                fa = scalf_mul(sh.ftot[w], fa);
            }
            sh.fall = fa;
        }
        gsync<NW>();
        if (lane == 0) Mx = sh.wpre[warp];
        else Mx = matf_mul(Mx, sh.wpre[warp]);
        Fin = scalf_mul(F, sh.fpre[warp]);
        Fall = sh.fall;
    } else {
        if (lane == 0) Mx = {1.0f, 0.0f, 0.0f, 1.0f, 0};
        Fall = {__shfl_sync(0xffffffffu, F.v, 31), __shfl_sync(0xffffffffu, F.e, 31)};
    }

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

    // ---- reductions
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
    // this chunk's S carried to the side's end (times f^2 over the later
    // chunks = F_all / F_in), in the absolute scale: S (Fall.v / Fin.v)
    // 2^(2 eA + Fall.e - Fin.e)
    FE x{0.0f, 0};
    if (s1 > s0 && S != 0.0f && Fin.v != 0.0f) x = {S * __fdividef(Fall.v, Fin.v), 2 * eA + Fall.e - Fin.e};
    const FE sw = warp_sum_fe(x);
    if (lane == 0) {
        sh.nodes[warp] = nodes;
        sh.pk_L[warp] = peak_L;
        sh.pk_s[warp] = peak_s;
        sh.s[warp] = sw;
    }
    gsync<NW>();
    if (G.leader()) {
        res.A = sh.A;
        res.D = sh.D;
        res.eA = sh.eA;
        int nsum = 0;
        double Ssum = 0.0;
        int pL = -(1 << 30), ps = 0x7fffffff;
        for (int w = 0; w < NW; ++w) {
            nsum += sh.nodes[w];
            const FE s = sh.s[w];
            if (s.v > 0.0f) Ssum += (double)s.v * pow2(max(-1000, min(1000, s.e - 2 * res.eA)));
            if (sh.pk_L[w] > pL || (sh.pk_L[w] == pL && sh.pk_s[w] < ps)) {
                pL = sh.pk_L[w];
                ps = sh.pk_s[w];
            }
        }
        res.nodes = nsum;
        res.S = Ssum;
        res.peak_L = pL;
        res.peak_i = ps == 0x7fffffff ? from : from + dir * ps;
    }
    return res;
}

// One FP32 pass at E with match point k (the group twin of the lane pass):
// Cooley correction, count, sum and the peak of |psi| relative to psi_k,
// formed by the leader and handed to the group.
template <int NW>
__device__ __forceinline__ PassDF long_pass32(const Grp<NW>& G, const PotMeta& m, const LevelWork& w,
                                              const float2* __restrict__ Wf, const double* __restrict__ W64,
                                              double E, int k, Shared32<NW>& sh) {
    if (G.leader()) {
        const double aE = __dmul_rn(m.a, E);
        const float aEh = __double2float_rn(aE);
        sh.aEh = aEh;
        sh.aEl = __double2float_rn(aE - (double)aEh);
    }
    gsync<NW>();
    const float aEh = sh.aEh, aEl = sh.aEl;
    const LongSide32 o = long_side32<NW>(G, Wf, aEh, aEl, w.j0, k, +1, sh);
    const LongSide32 in = long_side32<NW>(G, Wf, aEh, aEl, w.j1, k, -1, sh);
    if (G.leader()) {
        const double aE = __dmul_rn(m.a, E);
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
        sh.res = r;
    }
    gsync<NW>();
    return sh.res;
}

// the host-mapped cancel flag, read by the leader and handed to the group
// (threads that read it separately could see it change between their reads
// and part at the next barrier)
template <int NW>
__device__ __forceinline__ bool grp_cancelled(const Grp<NW>& G, const DevBatch& b, int& slot) {
    return grp_bcast<NW>(G, G.leader() && b.cancel && *b.cancel ? 1 : 0, slot) != 0;
}

// Levels on groups of warps, in up to three stages:
//   1. FP32 passes (long_pass32): safeguarded Cooley-Newton with the count
//      bracket, the match point moved to the peak of |psi|, until a Newton
//      step of at most kTol32Long is taken (the energy after it is then far
//      inside stage 2's first-pass acceptance);
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
// mode 0: the long list (stages 1-3); 1: the levels newton_df handed over
// (stage 3 only); 2: the middle list, whose FP32 refinement the lane kernel
// refine32 did (stage 2 from its energy, bracket, match point and sum, with
// newton_df's acceptance rule, then stage 3 if it does not settle).  Every
// thread of a group runs the same control flow on the leader's pass results
// (the group's passes are collective).
// (Measured on the 2048-potential batch, refine_long / step: 2e-9 7.8 /
// 30.0 ms, 1e-8 7.4 / 29.8, 3e-8 7.4 / 29.6, 1e-7 7.0 / 29.6 with more
// double-float passes after it.)
constexpr double kTol32Long = 3e-8;

template <int NW>
__global__ void __launch_bounds__(kLongThreads, kLongCtasPerSm) refine_long_kernel(DevBatch b, int mode, const int32_t* list,
                                                                   const int32_t* list_len, int qid) {
    constexpr int kG = kLongThreads / (32 * NW);
    __shared__ SharedDF<NW> shd[kG];
    __shared__ Shared32<NW> sh32s[kG];
    const Grp<NW> G;
    SharedDF<NW>& sh = shd[G.g()];
    Shared32<NW>& sh32 = sh32s[G.g()];
    const int n = min(*list_len, b.max_levels);  // filled on the device earlier in the solve
    // levels from a device queue (a group takes the next as it finishes one)
    for (;;) {
        const int q = grp_next<NW>(G, &b.hdr->queue[qid], sh.word);
        if (q >= n) break;
        const int slot = list[q];
        LevelWork w = b.levels[slot];
        if (w.status & EPSCU_STATUS_NOTFOUND) continue;
        if (grp_cancelled<NW>(G, b, sh.word)) {
            if (G.leader()) b.levels[slot].status = w.status | EPSCU_STATUS_CANCELLED;
            continue;
        }
        const PotMeta m = b.meta[w.p];
        const float2* Wf = b.Wf2 + m.offf;
        const double* W = b.W64 + m.off;
        double lo = w.lo, hi = w.hi, E = w.E, sum = 1.0;
        int k = mode == 2 ? w.k : grp_bcast<NW>(G, G.leader() ? clamp_k(w, match_index(m, b.Msuf, E)) : 0, sh.word);
        bool done = false;
        int n_pass = 0, n_pass32 = 0;
        if (mode == 2) {
            // ---- stage 2 from the lane FP32 refinement (as newton_df): its sum
            // psi~^2 is accurate to ~1e-4 on long windows, so one step is
            // accepted from within 1e-10 and the norm pass corrects the rest
            sum = w.norm_k_in;
            double lo2 = w.lo - 1e-8, hi2 = w.hi + 1e-8;
            for (int it = 0; it < 4 && !done; ++it) {
                const PassDF r = long_pass<NW, 0>(G, m, w, Wf, W, E, k, sum, sh);
                ++n_pass;
                if (r.count > w.v) hi2 = fmin(hi2, E);
                else lo2 = fmax(lo2, E);
                const double En = E + r.dE;
                if (!isfinite(En) || !(En >= lo2 && En <= hi2) || r.nodes != w.v) break;
                done = fabs(r.dE) <= (it == 0 ? 1e-10 : 1e-12 * fmax(1.0, fabs(E)));
                E = En;
            }
            if (done) {
                lo = lo2;
                hi = hi2;
            }
        }
        if (mode == 0) {
            // ---- stage 1: FP32
            bool moved_last = false, ok32 = false;
            for (int it = 0, cap = refine_cap(b); it < cap; ++it) {
                const PassDF r = long_pass32<NW>(G, m, w, Wf, W, E, k, sh32);
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
                    const PassDF r = long_pass<NW, 0>(G, m, w, Wf, W, E, k, sum, sh);
                    ++n_pass;
                    if (r.count > w.v) hi2 = fmin(hi2, E);
                    else lo2 = fmax(lo2, E);
                    const double En = E + r.dE;
                    if (!isfinite(En) || !(En >= lo2 && En <= hi2) || r.nodes != w.v) break;
                    // the FP32 sum of the group pass is accurate to ~1e-6 (chunk
                    // sums of a few hundred terms), so one step from within 1e-8
                    // leaves ~1e-14: the first pass settles
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
                const PassDF r = long_pass<NW, 1>(G, m, w, Wf, W, E, k, 1.0, sh);
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
        if (G.leader()) {
            if (!done) w.status |= EPSCU_STATUS_MAXITER;
            w.lo = lo;
            w.hi = hi;
            w.E = E;
            w.k = k;
            w.norm_k_in = sum;
            w.iters = n_pass32 + n_pass;
            const unsigned long long pts = (unsigned long long)(w.j1 - w.j0);
            atomicAdd(&b.hdr->refine_updates, (unsigned long long)n_pass32 * pts);
            atomicAdd(&b.hdr->df_updates, (unsigned long long)n_pass * pts);
            if (mode == 0 && NW == kLongWarps) {
                atomicAdd(&b.hdr->long32_updates, (unsigned long long)n_pass32 * pts);
                atomicAdd(&b.hdr->longdf_updates, (unsigned long long)n_pass * pts);
            }
            b.levels[slot] = w;
        }
    }
}

// The norm pass of a group level and its match-point candidates (as
// norm_df).  With psi requested every pass also stores its unnormalised
// psi-hat in the level's row (MODE 3) and the last pass is the one kept;
// scale_psi applies the constants afterwards.
template <int NW>
__global__ void __launch_bounds__(kLongThreads, kLongCtasPerSm) norm_long_kernel(DevBatch b, const int32_t* list,
                                                                 const int32_t* list_len, int qid) {
    constexpr int kG = kLongThreads / (32 * NW);
    __shared__ SharedDF<NW> shd[kG];
    const Grp<NW> G;
    SharedDF<NW>& sh = shd[G.g()];
    const int n = min(*list_len, b.max_levels);
    for (;;) {
        const int q = grp_next<NW>(G, &b.hdr->queue[qid], sh.word);
        if (q >= n) break;
        const int slot = list[q];
        LevelWork w = b.levels[slot];
        if (w.status & (EPSCU_STATUS_NOTFOUND | EPSCU_STATUS_CANCELLED)) continue;
        const PotMeta m = b.meta[w.p];
        const float2* Wf = b.Wf2 + m.offf;
        const double* W = b.W64 + m.off;
        double* row = psi_row(b, m, w);
        auto pass = [&](int kk) { return long_pass<NW, 3>(G, m, w, Wf, W, w.E, kk, 1.0, sh, row); };
        int k = w.k;
        PassDF r = pass(k);
        if (r.peak_log2 >= 2) {
            k = clamp_k(w, r.peak_i);
            r = pass(k);
        }
        int k_row = k;  // the pass whose psi-hat the row holds
        if (r.nodes != w.v) {
            const int kt = grp_bcast<NW>(G, G.leader() ? clamp_k(w, match_index(m, b.Msuf, w.E)) : 0, sh.word);
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
            if (G.leader()) atomicAdd(&b.hdr->n_redo, 1);
            w.E += r.dE;
            r = pass(k);
        } else if (row && k_row != k) {
            r = pass(k);
        }
        if (G.leader()) {
            finalize_df(m, w, r, k);
            if (suspicious(m, w, r.nodes, r.dE) && b.twist_list) {
                const int t = atomicAdd(&b.hdr->n_twist, 1);
                if (t < b.max_twist) b.twist_list[t] = slot;
            }
            b.levels[slot] = w;
        }
    }
}

// Twist-index search for the levels the norm passes flagged (any window
// length): a chunked outward sweep stores D/A every kTwistSample points, a
// chunked inward sweep forms |gamma_k| at the same points, the match point
// becomes argmin |gamma_k| (Dhillon and Parlett's twisted-factorisation
// rule), then Newton and the norm pass run there; with psi requested the
// final pass stores the unnormalised psi-hat in the level's row (scale_psi
// applies the constants).  The level joins the long list, so the adjoint's
// recompute path (write_long) writes its psi.  One CTA per level.
__global__ void __launch_bounds__(kLongThreads, kLongCtasPerSm) twist_long_kernel(DevBatch b) {
    __shared__ SharedDF<kLongWarps> sh;
    const Grp<kLongWarps> G;
    const int n = min(b.hdr->n_twist, b.max_twist);
    for (;;) {
        const int q = grp_next<kLongWarps>(G, &b.hdr->queue[kQTwistLong], sh.word);
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
        long_side<kLongWarps, 4>(G, Wf, aE, w.j0, w.j1, +1, nullptr, 0.0, 0, sh, &tw);
        long_side<kLongWarps, 5>(G, Wf, aE, w.j1, w.j0, -1, nullptr, 0.0, 0, sh, &tw);
        const int k = clamp_k(w, tw.k == 0x7fffffff ? w.k : tw.k);
        double* row = psi_row(b, m, w);
        auto pass = [&](double e) { return long_pass<kLongWarps, 3>(G, m, w, Wf, W, e, k, 1.0, sh, row); };
        double E1 = w.E;
        PassDF r = pass(E1);
        for (int it = 0; it < 8; ++it) {
            if (r.nodes != w.v || !isfinite(r.dE) || !(fabs(r.dE) < 1e-7)) break;
            if (fabs(r.dE) <= 1e-13 * fmax(1.0, fabs(E1))) break;
            E1 += r.dE;
            r = pass(E1);
        }
        w.E = E1;
        if (G.leader()) {
            finalize_df(m, w, r, k);
            if (!(w.status & EPSCU_STATUS_LONG) && b.long_list) {
                const int t = atomicAdd(&b.hdr->n_long, 1);
                if (t < b.max_levels) {
                    b.long_list[t] = slot;
                    w.status |= EPSCU_STATUS_LONG;
                }
            }
            b.levels[slot] = w;
        }
    }
}

// psi of the listed levels in FP64 from the final constants (window points
// and psi_k; the rest of each row is zero): the adjoint's recompute path.
// One CTA per level.
__global__ void __launch_bounds__(kLongThreads, kLongCtasPerSm) write_long_kernel(DevBatch b, const int32_t* list,
                                                                  const int32_t* list_len) {
    __shared__ SharedDF<kLongWarps> sh;
    const Grp<kLongWarps> G;
    if (!b.psi || b.hdr->error) return;
    const int n = min(*list_len, b.max_levels);
    for (int q = blockIdx.x; q < n; q += gridDim.x) {
        const int slot = list[q];
        const LevelWork w = b.levels[slot];
        const PotMeta m = b.meta[w.p];
        double* out = b.psi + m.psi_off + (int64_t)(w.v - b.min_level) * m.N;
        // the rows were zeroed by zero_psi: only the window is written
        if (no_result(w)) continue;
        const float2* Wf = b.Wf2 + m.offf;
        const dfl aE = energy_df(m, w.E);
        long_side<kLongWarps, 2>(G, Wf, aE, w.j0, w.k, +1, out, w.norm_k_out, w.ex_out, sh);
        long_side<kLongWarps, 2>(G, Wf, aE, w.j1, w.k, -1, out, w.norm_k_in, w.ex_in, sh);
        if (threadIdx.x == 0) out[w.k] = w.ck;
        __syncthreads();  // the shared scratch is reused by the next level
    }
}

}  // namespace

void launch_refine_long(const DevBatch& b, int sm_count, cudaStream_t s) {
    if (!b.long_list) return;
    refine_long_kernel<kLongWarps>
        <<<sm_count * kLongCtasPerSm, kLongThreads, 0, s>>>(b, 0, b.long_list, &b.hdr->n_long, kQLongRefine);
}
void launch_fallback_long(const DevBatch& b, int sm_count, cudaStream_t s) {
    if (!b.fallback_list) return;
    refine_long_kernel<kLongWarps>
        <<<sm_count * kLongCtasPerSm, kLongThreads, 0, s>>>(b, 1, b.fallback_list, &b.hdr->fallbacks, kQFallback);
}
void launch_norm_long(const DevBatch& b, int sm_count, cudaStream_t s) {
    if (!b.long_list) return;
    norm_long_kernel<kLongWarps><<<sm_count * kLongCtasPerSm, kLongThreads, 0, s>>>(b, b.long_list, &b.hdr->n_long, kQNormLong);
}
void launch_norm_fallback(const DevBatch& b, int sm_count, cudaStream_t s) {
    if (!b.fallback_list) return;
    norm_long_kernel<kLongWarps>
        <<<sm_count * kLongCtasPerSm, kLongThreads, 0, s>>>(b, b.fallback_list, &b.hdr->fallbacks, kQNormFallback);
}
void launch_twist_long(const DevBatch& b, int sm_count, cudaStream_t s) {
    if (!b.twist_list || !b.long_list) return;
    twist_long_kernel<<<sm_count * kLongCtasPerSm, kLongThreads, 0, s>>>(b);
}
void launch_write_long(const DevBatch& b, int sm_count, cudaStream_t s) {
    // the group levels of both tiers (the recompute path: one CTA per level)
    if (b.long_list) write_long_kernel<<<sm_count * kLongCtasPerSm, kLongThreads, 0, s>>>(b, b.long_list, &b.hdr->n_long);
    if (b.mid_list) write_long_kernel<<<sm_count * kLongCtasPerSm, kLongThreads, 0, s>>>(b, b.mid_list, &b.hdr->n_mid);
    if (b.fallback_list)
        write_long_kernel<<<sm_count * kLongCtasPerSm, kLongThreads, 0, s>>>(b, b.fallback_list, &b.hdr->fallbacks);
}
// the middle tier is in use (its list can be non-empty): the same threshold
// as the window kernel's
static bool mid_tier_on(const DevBatch& b) {
    return b.mid_list && (b.mid_window != 0 ? b.mid_window : kMidWindow) > 0;
}
void launch_refine_mid(const DevBatch& b, int sm_count, cudaStream_t s) {
    if (!mid_tier_on(b)) return;
    refine_long_kernel<1><<<sm_count * kLongCtasPerSm, kLongThreads, 0, s>>>(b, 2, b.mid_list, &b.hdr->n_mid, kQMidRefine);
}
void launch_norm_mid(const DevBatch& b, int sm_count, cudaStream_t s) {
    if (!mid_tier_on(b)) return;
    norm_long_kernel<1><<<sm_count * kLongCtasPerSm, kLongThreads, 0, s>>>(b, b.mid_list, &b.hdr->n_mid, kQNormMid);
}

}  // namespace epscu
