// dfloat.cuh -- compensated FP32 ("double-float") arithmetic for the polish
// passes of the fast method.
//
// A value is an unevaluated sum h + l of two floats with |l| <= ulp(h)/2,
// about 48 significant bits.  The error-free transformations are Knuth's
// TwoSum, Dekker's FastTwoSum and the FMA-based TwoProduct; every operation is
// written with explicit round-to-nearest intrinsics so the compiler can
// neither contract nor reassociate them.  On GB300 one double-float operation
// costs 3-11 FP32 instructions, a fraction of one FP64 instruction's issue
// cost (FP64 runs at 1/62 of the FP32 rate).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace epscu {

struct dfl {
    float h, l;
};

__device__ __forceinline__ dfl two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}

// requires |a| >= |b| (or a == 0)
__device__ __forceinline__ dfl fast_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float e = __fsub_rn(b, __fsub_rn(s, a));
    return {s, e};
}

__device__ __forceinline__ dfl df_add(dfl a, dfl b) {
    const dfl s = two_sum(a.h, b.h);
    const float e = __fadd_rn(s.l, __fadd_rn(a.l, b.l));
    return fast_two_sum(s.h, e);
}

__device__ __forceinline__ dfl df_mul(dfl a, dfl b) {
    const float p = __fmul_rn(a.h, b.h);
    float e = __fmaf_rn(a.h, b.h, -p);
    e = __fmaf_rn(a.h, b.l, e);
    e = __fmaf_rn(a.l, b.h, e);
    return fast_two_sum(p, e);
}

__device__ __forceinline__ dfl df_mulf(dfl a, float b) {
    const float p = __fmul_rn(a.h, b);
    float e = __fmaf_rn(a.h, b, -p);
    e = __fmaf_rn(a.l, b, e);
    return fast_two_sum(p, e);
}

// exact scaling by a power of two
__device__ __forceinline__ dfl df_scale(dfl a, float p2) { return {__fmul_rn(a.h, p2), __fmul_rn(a.l, p2)}; }

// 1/a: FP32 reciprocal refined by one Newton step carried in double-float
__device__ __forceinline__ dfl df_recip(dfl a) {
    const float r = __frcp_rn(a.h);
    float e = __fmaf_rn(-a.h, r, 1.0f);
    e = __fmaf_rn(-a.l, r, e);
    return fast_two_sum(r, __fmul_rn(r, e));
}

// exact float -> double through the bit pattern (integer pipe); zero,
// subnormal and non-finite inputs take the hardware conversion
__device__ __forceinline__ double f2d(float x) {
    const uint32_t u = __float_as_uint(x);
    const uint32_t ex = (u >> 23) & 0xffu;
    if (ex == 0u || ex == 0xffu) return (double)x;
    const uint32_t man = u & 0x7fffffu;
    const uint32_t hi = (u & 0x80000000u) | ((ex + 896u) << 20) | (man >> 3);
    return __hiloint2double((int)hi, (int)(man << 29));
}

__device__ __forceinline__ double df_to_double(dfl a) { return f2d(a.h) + f2d(a.l); }

// binary exponent e of |x| = m 2^e, m in [0.5, 1), for finite nonzero x
__device__ __forceinline__ int fexp(float x) { return (int)((__float_as_uint(x) >> 23) & 0xffu) - 126; }

// 2^e as a float, |e| <= 125
__device__ __forceinline__ float fpow2(int e) { return __int_as_float((127 + e) << 23); }

// exact x 2^X as a double, built from the bit pattern (integer pipe, no FP64
// instruction) while the result stays a normal double; |X| < 900
__device__ __forceinline__ double f2d_pow2(float x, int X) {
    const uint32_t u = __float_as_uint(x);
    const uint32_t ex = (u >> 23) & 0xffu;
    if (ex == 0u || ex == 0xffu) return (double)x * __hiloint2double((1023 + X) << 20, 0);
    const uint32_t man = u & 0x7fffffu;
    const uint32_t hi = (u & 0x80000000u) | ((ex + 896u + (uint32_t)X) << 20) | (man >> 3);
    return __hiloint2double((int)hi, (int)(man << 29));
}

// Sum of squares in double-float with an FP64 spill.  The sum is d + x 2^pend
// in the current scale; add() takes terms, rescale(s) multiplies the whole sum
// by 2^s (the renormalisation of the state), value() returns it in FP64.  The
// double-float part d absorbs the rescalings with two exact FP32 multiplies;
// x is touched only when d would leave the float range, so a pass issues
// almost no FP64 instruction (one costs ~62 FP32 issue slots on GB300).
struct SqSum {
    dfl d;
    double x;
    int pend;

    __device__ __forceinline__ void init() {
        d = {0.0f, 0.0f};
        x = 0.0;
        pend = 0;
    }
    __device__ __forceinline__ void add(dfl v) { d = df_add(d, v); }
    __device__ __forceinline__ void rescale(int s) {
        if (s == 0) return;
        if (x != 0.0) {
            pend += s;
            if (pend < -1000) {  // the spilled part fell below any contribution
                x = 0.0;
                pend = 0;
            }
        }
        if (d.h == 0.0f) return;
        const int ex = fexp(d.h) + s;
        if (s > -120 && s < 120 && ex > -100 && ex < 100) {
            d = df_scale(d, fpow2(s));
            return;
        }
        const double dd = f2d(d.h) + f2d(d.l);  // d 2^s = dd 2^s
        if (x == 0.0) {
            x = dd;
            pend = s;
        } else {
            const int r = s - pend;
            if (r > 1000) {
                x = dd;  // the old spill is negligible against d
                pend = s;
            } else if (r > -1000) {
                x += dd * __hiloint2double((1023 + r) << 20, 0);
            }
        }
        d = {0.0f, 0.0f};
    }
    __device__ __forceinline__ double value() const {
        const double xs = x == 0.0 ? 0.0 : x * __hiloint2double((1023 + max(-1000, min(1000, pend))) << 20, 0);
        return xs + (f2d(d.h) + f2d(d.l));
    }
};

__device__ __forceinline__ dfl df_from_double(double x) {
    const float h = __double2float_rn(x);
    const float l = __double2float_rn(x - (double)h);
    return {h, l};
}


}  // namespace epscu
