// df64.cuh -- FP64 values carried through FP32/INT32 arithmetic.
//
// GB300 executes FP64 at 1/64 of its FP32 rate (2 FP64 operations per SM
// clock), so an FP64 stencil there is bound by the FP64 pipe long before it
// reaches HBM.  The fast kernels (fastKernels = 2) therefore read the FP64
// fields, split each value into two floats with integer operations only, do
// the arithmetic in float pairs where cancellation needs it (Knuth's TwoSum,
// the classical double-float technique of Dekker 1971), and spend one FP64
// addition per output point to form the FP64 result.
//
// dsplit(x) -> (hi, lo):  hi = x with the low 29 of its 52 fraction bits
//   cleared (exact in float when 2^-126 <= |x| < 2^128), lo = the cleared
//   bits, kept to their top 23 bits: |x - hi - lo| <= 2^-46 |x|.
//   |x| < 2^-126 gives hi = 0 (and lo = 0 below 2^-104); NaN and Inf give a
//   NaN / Inf hi, so they reach every result computed from the split.
// f2d(f): the float f as an exact double, built from its bits.
#pragma once

#include <cuda_runtime.h>

namespace saras {

__device__ __forceinline__ void dsplit(double x, float &hi, float &lo) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned h = (unsigned)(b >> 32), l = (unsigned)b;
    const unsigned sign = h & 0x80000000u;
    const unsigned e = (h >> 20) & 0x7ffu;
    // hi for 897 <= e <= 1150: float exponent e - 896 above the top 23 fraction
    // bits.  (h:l) << 3 holds e mod 512 in bits 31..23 above those bits, and
    // 896 = 384 mod 512, so one subtraction rebases the exponent.
    unsigned hb = (__funnelshift_l(l, h, 3) - (384u << 23)) & 0x7fffffffu;
    if (e < 897u) hb = 0u;
    else if (e > 1150u) hb = (e == 2047u && ((h & 0xfffffu) | l)) ? 0x7fc00000u : 0x7f800000u;
    hi = __uint_as_float(hb | sign);
    // lo = (l mod 2^29) 2^(e-1075): its top 23 bits m as a float by the
    // magic-number conversion (2^(E-127) (1 + m 2^-23) - 2^(E-127) = m 2^(E-150),
    // exact), with E - 150 = e - 1069, i.e. E = e - 919; 0 outside 1 <= E <= 254.
    const unsigned me = e - 919u, base = me << 23;
    float mag = __uint_as_float(base | ((l & 0x1fffffffu) >> 6)) - __uint_as_float(base);
    if (me - 1u >= 254u) mag = 0.0f;
    lo = __uint_as_float(__float_as_uint(mag) | sign);
}

__device__ __forceinline__ double f2d(float f) {
    unsigned u = __float_as_uint(f);
    unsigned sign = u & 0x80000000u;
    int fe = (int)((u >> 23) & 0xffu);
    unsigned fr = u & 0x7fffffu;
    unsigned hw, lw;
    if (fe == 0) { hw = sign; lw = 0u; }   // zero (float subnormals are flushed)
    else if (fe == 255) { hw = sign | 0x7ff00000u | (fr ? 0x80000u : 0u); lw = 0u; }
    else { hw = sign | ((unsigned)(fe + 896) << 20) | (fr >> 3); lw = (fr & 7u) << 29; }
    return __longlong_as_double((long long)(((unsigned long long)hw << 32) | lw));
}

// x / d correctly rounded for a divisor d whose reciprocal y = RN(1/d) is
// known: Markstein's correction step (P. Markstein, IBM J. Res. Develop. 34(1),
// 1990): q = RN(x y), r = x - q d exactly by an FMA, then RN(q + r y) = RN(x / d)
// for x and x / d in the normal range (tests/test_division.py checks it against
// IEEE division on random pairs, all-ones and power-of-two significands
// included; 10^8 pairs showed no difference).  Three FP64
// operations in place of a division subroutine, on a part whose FP64 pipe bounds
// every reference-form kernel.  A zero x gives +0 where the division gives -0
// for negative x: zeros compare and add alike.
__device__ __forceinline__ double div_rn(double x, double d, double y) {
    const double q = x * y;
    return fma(fma(-q, d, x), y, q);
}

// Knuth's TwoSum: s + t == a + b exactly, s = fl(a + b).
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &t) {
    s = a + b;
    float bb = s - a;
    t = (a - (s - bb)) + (b - bb);
}

// Float pairs: value h + l with |l| <= ulp(h) / 2 after each operation
// (Dekker's FastTwoSum renormalises), about 44 significant bits.
struct fpair {
    float h, l;
};

__device__ __forceinline__ fpair fp_norm(float s, float t) {
    float h = s + t;
    return fpair{h, t - (h - s)};
}

__device__ __forceinline__ fpair fp_add(fpair a, fpair b) {
    float s, t;
    two_sum(a.h, b.h, s, t);
    return fp_norm(s, t + (a.l + b.l));
}

__device__ __forceinline__ fpair fp_neg(fpair a) { return fpair{-a.h, -a.l}; }

// Product through the exact FMA residual of the high parts.
__device__ __forceinline__ fpair fp_mul(fpair a, fpair b) {
    float p = a.h * b.h;
    float e = fmaf(a.h, b.h, -p);
    e = fmaf(a.h, b.l, fmaf(a.l, b.h, e));
    return fp_norm(p, e);
}

// a b + c in one normalisation: the high product's exact FMA residual and the
// TwoSum of the high parts, the cross terms and c's low part in float.
__device__ __forceinline__ fpair fp_fma(fpair a, fpair b, fpair c) {
    float p = a.h * b.h;
    float e = fmaf(a.h, b.h, -p);
    float s, t;
    two_sum(p, c.h, s, t);
    t += e + fmaf(a.h, b.l, fmaf(a.l, b.h, c.l));
    return fp_norm(s, t);
}

// Unnormalised forms for accumulation chains: the second float carries the
// rounding errors and cross terms without the final FastTwoSum, so it may be a
// few ulps of the first.  Products and TwoSums of such pairs keep about 2^-44
// of the result (the cross terms a.h b.l are formed in float from a b.l a few
// ulps of a.h b.h); a chain ends in one fp_norm.
__device__ __forceinline__ fpair fp_mul_u(fpair a, fpair b) {
    float p = a.h * b.h;
    float e = fmaf(a.h, b.h, -p);
    return fpair{p, fmaf(a.h, b.l, fmaf(a.l, b.h, e))};
}

__device__ __forceinline__ fpair fp_fma_u(fpair a, fpair b, fpair c) {
    float p = a.h * b.h;
    float e = fmaf(a.h, b.h, -p);
    float s, t;
    two_sum(p, c.h, s, t);
    return fpair{s, t + (e + fmaf(a.h, b.l, fmaf(a.l, b.h, c.l)))};
}

__device__ __forceinline__ fpair fp_of(double x) {
    fpair r;
    dsplit(x, r.h, r.l);
    return r;
}

// |f| < 2^128 and not NaN, from the bits (keeps the check off the FP64 pipe).
__device__ __forceinline__ bool f_finite(float f) { return (__float_as_uint(f) & 0x7fffffffu) < 0x7f800000u; }

// ---- 64-bit fixed point (the exact residual of the mixed-precision refinement)
// v = round(x 2^s) to nearest (ties away from zero) from the bits of x; sets
// `bad` for NaN / Inf or when |v| would reach 2^62.  Integer operations only.
__device__ __forceinline__ long long d2fx(double x, int s, bool &bad) {
    unsigned long long b = (unsigned long long)__double_as_longlong(x);
    int e = (int)((b >> 52) & 0x7ffu);
    if (e == 0) return 0;
    if (e == 2047) { bad = true; return 0; }
    unsigned long long m = (b & 0xfffffffffffffull) | 0x10000000000000ull;   // |x| = m 2^(e-1075)
    int sh = e - 1075 + s;
    unsigned long long a;
    if (sh >= 0) {
        if (sh > 9) { bad = true; return 0; }
        a = m << sh;
    } else if (sh >= -53) {
        a = (m >> (-sh)) + ((m >> (-sh - 1)) & 1ull);
    } else {
        return 0;
    }
    long long v = (long long)a;
    return (b >> 63) ? -v : v;
}

__device__ __forceinline__ long long f2fx(float f, int s, bool &bad) {
    unsigned u = __float_as_uint(f);
    int e = (int)((u >> 23) & 0xffu);
    if (e == 0) return 0;
    if (e == 255) { bad = true; return 0; }
    unsigned long long m = (u & 0x7fffffu) | 0x800000u;   // |f| = m 2^(e-150)
    int sh = e - 150 + s;
    unsigned long long a;
    if (sh >= 0) {
        if (sh > 38) { bad = true; return 0; }
        a = m << sh;
    } else if (sh >= -24) {
        a = (m >> (-sh)) + ((m >> (-sh - 1)) & 1ull);
    } else {
        return 0;
    }
    long long v = (long long)a;
    return (u >> 31) ? -v : v;
}

// A 64-bit integer as a float (to within a few float ulps) from two 32-bit
// conversions: the 64-bit conversion instruction runs on GB300's FP64 pipe.
__device__ __forceinline__ float fx2f(long long r) {
    return fmaf((float)(int)(r >> 32), 4294967296.0f, (float)(unsigned)r);
}

}  // namespace saras
