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

// The double of a double-float pair h + l (|l| <= ulp(h)/2, as every
// operation above leaves it) within one unit in its last place, built with
// integer operations only: h's significand at the top of the 53 bits, l's
// added or subtracted below it (its bits past the 53rd are dropped).  Zero,
// subnormal or non-finite h, and pairs that are not normalised, take two
// exact conversions and one FP64 add instead.
__device__ __forceinline__ double df_pair_to_double(float h, float l) {
    const uint32_t uh = __float_as_uint(h), ul = __float_as_uint(l);
    const uint32_t eh = (uh >> 23) & 0xffu, el = (ul >> 23) & 0xffu;
    if (eh == 0u || eh == 0xffu || el == 0xffu) return f2d(h) + f2d(l);
    uint64_t M = (uint64_t)((uh & 0x7fffffu) | 0x800000u) << 29;  // bits 52..29
    if (el != 0u) {  // (a subnormal l lies below the 53 bits)
        const int d = (int)eh - (int)el;
        if (d < 24) return f2d(h) + f2d(l);
        const uint64_t ml = (uint64_t)((ul & 0x7fffffu) | 0x800000u);
        const int sh = 29 - d;  // <= 5: l's significand stays below bit 29
        const uint64_t add = sh >= 0 ? (ml << sh) : (-sh < 64 ? (ml >> -sh) : 0ull);
        M = ((uh ^ ul) >> 31) ? M - add : M + add;
    }
    uint32_t e = eh + 896u;  // biased double exponent of bit 52
    if (!(M >> 52)) {        // a subtraction from a power of two: one bit down
        M <<= 1;
        --e;
    }
    return __longlong_as_double((long long)(((uint64_t)(uh >> 31) << 63) | ((uint64_t)e << 52) |
                                            (M & 0xfffffffffffffull)));
}

// df_pair_to_double(h, l) * 2^e2, the exponent added in the bits while the
// result stays a normal double (ldexp otherwise)
__device__ __forceinline__ double df_pair_to_double_scaled(float h, float l, int e2) {
    const double d = df_pair_to_double(h, l);
    const long long u = __double_as_longlong(d);
    const int ex = (int)((u >> 52) & 0x7ff);
    if (ex == 0) return d;  // zero (a subnormal pair product: below any psi value)
    const int en = ex + e2;
    if (en >= 1 && en <= 2046) return __longlong_as_double(u + ((long long)e2 << 52));
    return ldexp(d, e2);
}

// A double as a double-float pair (h + l, ~48 significant bits) through its
// bit pattern on the integer pipe: h keeps the top 24 significand bits, l the
// next 29 (converted once).  No FP64 instruction.  Zero, subnormal and very
// small or large |x| (outside 2^+-100) give a zero pair: the callers square
// and weight values whose useful range is far inside that.
__device__ __forceinline__ dfl df_split_double_bits(double x) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(x);
    const uint32_t hi = (uint32_t)(u >> 32), lo = (uint32_t)u;
    const int e = (int)((hi >> 20) & 0x7ffu) - 1023;
    if (e < -100 || e > 100) return {0.0f, 0.0f};
    const uint32_t sgn = hi & 0x80000000u;
    const uint32_t top23 = ((hi & 0xfffffu) << 3) | (lo >> 29);
    const float h = __uint_as_float(sgn | ((uint32_t)(e + 127) << 23) | top23);
    // the remaining 29 bits are worth (lo & (2^29 - 1)) 2^(e - 52)
    float l = __uint2float_rn(lo & 0x1fffffffu) * 2.220446049250313e-16f;  // 2^-52 (a normal float)
    l = __fmul_rn(l, __int_as_float((127 + e) << 23));                    // 2^e, |e| <= 100
    return {h, sgn ? -l : l};
}

__device__ __forceinline__ dfl df_from_double(double x) {
    const float h = __double2float_rn(x);
    const float l = __double2float_rn(x - (double)h);
    return {h, l};
}


}  // namespace epscu
