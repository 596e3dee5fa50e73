// df64.cuh -- double-float arithmetic: a value is the unevaluated sum hi + lo of two
// FP32 numbers with |lo| <= ulp(hi)/2, a 48-bit significand with the FP32 exponent range.
//
// The 48 bits hold for |x| >= 2^-74, where a non-zero lo is an FP32 normal number; below,
// lo may flush to zero (absolute error < 2^-126); |x| must stay below 2^128.
//
// Why on GB300: its FP64 pipe issues 1/64 of the FP32 rate, so a reconstruction that is
// bound by FP64 instruction issue runs several times faster on FP32 pairs, where an add
// costs ~11 and a multiply ~6 FP32 instructions.  The building blocks are the classical
// error-free transformations: Knuth's TwoSum, Dekker's FastTwoSum and the FMA-based
// TwoProduct (exact a*b = p + e); the operations follow the double-double algorithms of
// Dekker (1971) and Hida, Li & Bailey's QD library report (2001), "sloppy" addition
// (error ~2^-48 (|x| + |y|)).  Every FP32 operation goes through an _rn intrinsic, which the
// compiler never contracts into an FMA or reorders: the transformations rely on the
// rounding of each individual operation.
#pragma once

#include <cuda_runtime.h>

namespace hype {

struct __align__(8) df64 {
    float hi, lo;
};

// x rounded to a 24-bit significand, as FP32 (f) and as FP64 (fd), on the bit pattern:
// adding half a unit of the 24th bit and clearing the 29 bits below rounds to nearest
// (ties away from zero) and carries into the exponent where needed; values outside the
// FP32 normal range take the F2F conversion
__device__ __forceinline__ float df_round24(double x, double& fd) {
    const unsigned long long r = ((unsigned long long)__double_as_longlong(x) + 0x10000000ull) & ~0x1FFFFFFFull;
    const unsigned hi = (unsigned)(r >> 32);
    const unsigned ex = (hi >> 20) & 0x7FFu;
    if (ex - 897u <= 253u) {
        fd = __longlong_as_double((long long)r);
        return __uint_as_float((hi & 0x80000000u) | ((ex - 896u) << 23) | ((unsigned)(r >> 29) & 0x7FFFFFu));
    }
    if ((r & 0x7FFFFFFFFFFFFFFFull) == 0ull) {
        fd = __longlong_as_double((long long)r);
        return __uint_as_float(hi & 0x80000000u);
    }
    const float f = __double2float_rn(x);
    fd = (double)f;
    return f;
}

// split of an FP64 value: hi = x rounded to 24 bits, lo = (x - hi, exact in FP64) rounded
// likewise; one FP64 subtraction, the rest on the integer pipe
__device__ __forceinline__ df64 df_from_double(double x) {
    double hd, ld;
    const float h = df_round24(x, hd);
    return df64{h, df_round24(x - hd, ld)};
}

// FP32 -> FP64 conversion by assembling the bits on the integer pipe (GB300 runs the F2F
// conversion on its narrow FP64 pipe), without branches: sign, exponent rebased from 127
// to 1023 (255, infinity or NaN, to 2047), the 23 significand bits shifted into the top of
// the 52.  Exact for normal numbers, zeros and infinities, NaN stays NaN; FP32 subnormals
// (below 1.2e-38) become zeros of their sign.
__device__ __forceinline__ double df_f2d(float x) {
    const unsigned b = __float_as_uint(x);
    const unsigned ex = (b >> 23) & 0xFFu;
    const unsigned exd = ex == 0u ? 0u : ex == 255u ? 0x7FFu : ex + 896u;
    const unsigned man = ex == 0u ? 0u : b & 0x7FFFFFu;
    return __hiloint2double((int)((b & 0x80000000u) | (exd << 20) | (man >> 3)), (int)(man << 29));
}

// hi + lo in FP64: exact unless lo lies more than 29 bits below hi's last bit, and then
// rounded once
__device__ __forceinline__ double df_to_double(df64 a) { return df_f2d(a.hi) + df_f2d(a.lo); }

// a compile-time constant c as a pair (folded by the compiler for literal arguments)
__host__ __device__ constexpr df64 dfc(double c) {
    return df64{(float)c, (float)(c - (double)(float)c)};
}

__device__ __forceinline__ df64 df_fast_two_sum(float a, float b) {  // |a| >= |b| or a == 0
    const float s = __fadd_rn(a, b);
    return df64{s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ df64 df_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bp = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bp)), __fsub_rn(b, bp));
    return df64{s, e};
}

__device__ __forceinline__ df64 operator+(df64 x, df64 y) {
    const df64 s = df_two_sum(x.hi, y.hi);
    return df_fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(x.lo, y.lo)));
}

__device__ __forceinline__ df64 operator-(df64 x) { return df64{-x.hi, -x.lo}; }

__device__ __forceinline__ df64 operator-(df64 x, df64 y) {
    const df64 s = df_two_sum(x.hi, -y.hi);
    return df_fast_two_sum(s.hi, __fadd_rn(s.lo, __fsub_rn(x.lo, y.lo)));
}

// Products are left unnormalised (p + e with |e| up to ~2^-22 |p| instead of ulp(p)/2):
// every operation below takes such inputs at full accuracy, and the next addition
// normalises again.
__device__ __forceinline__ df64 operator*(df64 x, df64 y) {
    const float p = __fmul_rn(x.hi, y.hi);
    float e = __fmaf_rn(x.hi, y.hi, -p);
    e = __fmaf_rn(x.hi, y.lo, e);
    e = __fmaf_rn(x.lo, y.hi, e);
    return df64{p, e};
}

// times an FP32 number
__device__ __forceinline__ df64 df_mul(df64 x, float c) {
    const float p = __fmul_rn(x.hi, c);
    return df64{p, __fmaf_rn(x.lo, c, __fmaf_rn(x.hi, c, -p))};
}

// times a power of two (exact)
__device__ __forceinline__ df64 df_scale(df64 x, float two_pow) { return df64{__fmul_rn(x.hi, two_pow), __fmul_rn(x.lo, two_pow)}; }

__device__ __forceinline__ df64 df_sqr(df64 x) {
    const float p = __fmul_rn(x.hi, x.hi);
    float e = __fmaf_rn(x.hi, x.hi, -p);
    return df64{p, __fmaf_rn(__fadd_rn(x.hi, x.hi), x.lo, e)};
}

// x / y: q1 = x.hi / y.hi from the approximate FP32 reciprocal (rcp.approx, ~1 ulp) after
// one Newton step, the remainder x - q1 y in double-float, and its quotient as the
// correction (~2^-47 relative accuracy); y.hi must be a nonzero normal number with
// |y.hi| < 2^126 (the FP32 reciprocal of larger values flushes to zero)
__device__ __forceinline__ df64 df_div(df64 x, df64 y) {
    float ry;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(ry) : "f"(y.hi));
    ry = __fmaf_rn(ry, __fmaf_rn(-y.hi, ry, 1.0f), ry);
    const float q1 = __fmul_rn(x.hi, ry);
    const df64 r = x - df_mul(y, q1);
    return df_fast_two_sum(q1, __fmul_rn(r.hi, ry));
}

// sqrt(x) for x > 0: the FP32 root s and one Heron correction (x - s^2) / (2 s), with s^2
// formed exactly by TwoProduct; x <= 0 (or not finite in hi) gives the FP32 root alone
__device__ __forceinline__ df64 df_sqrt(df64 x) {
    const float s = __fsqrt_rn(x.hi);
    if (!(x.hi > 0.0f) || !(s < 3.0e38f)) return df64{s, 0.0f};
    const float p = __fmul_rn(s, s);
    const float e = __fmaf_rn(s, s, -p);
    const df64 r = x - df64{p, e};
    return df_fast_two_sum(s, __fdiv_rn(r.hi, __fadd_rn(s, s)));
}

__device__ __forceinline__ df64 df_abs(df64 x) { return x.hi < 0.0f ? df64{-x.hi, -x.lo} : x; }

// (normalised operands: results of + or -)
__device__ __forceinline__ bool df_lt(df64 a, df64 b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ df64 df_min(df64 a, df64 b) { return df_lt(b, a) ? b : a; }

}  // namespace hype
