// Float-float ("double-FP32") arithmetic for the momentum kernels.
//
// GB300 issues FP64 at 1/64 of the FP32 rate, so a stencil that spends tens of
// FP64 operations per cell is bound by the FP64 pipe long before HBM.  A value
// here is an unevaluated sum x = hi + lo of two FP32 numbers with
// |lo| <= ulp(hi)/2 (a 48-bit significand, relative precision about 2^-47),
// and every operation is built from error-free transformations on the FP32
// pipe:
//   * TwoSum (Knuth, TAOCP vol. 2, 1969): s + e == a + b exactly, 6 additions;
//   * FastTwoSum (Dekker, Numer. Math. 18, 1971): the same for |a| >= |b|, 3;
//   * TwoProduct with a fused multiply-add (the FMA form of Dekker's product,
//     e.g. Ogita, Rump & Oishi, SIAM J. Sci. Comput. 26, 2005): p + e == a*b
//     exactly, 2 operations.
// Addition is Dekker's add2 (TwoSum of the high parts, the low parts added,
// FastTwoSum renormalisation): its error is a few units of 2^-48 (|x| + |y|).
// Multiplication is Dekker's mul2 with FMAs: a few units of 2^-48 |x y| (up to about
// 9 units when both operands come straight from ff_split, whose low part may reach one ulp of the
// high part).
// Conversions from and to FP64 are integer bit operations (no FP64 instruction):
// the high part takes the top 24 significand bits, the low part the next 23.
// Values must lie in the normal FP32 range: |x| < 2^-126 becomes 0 (an absolute
// error below 1.2e-38), |x| >= 2^128 becomes inf; NaN and inf pass through.  The
// low part of |x| < 2^-104 is dropped (relative error below 2^-23 there).
//
// The functions are __host__ __device__ so that a host build can check them
// against FP64 (tests/host/ff_check.cu).  They use the round-to-nearest FP32
// intrinsics on the device, which the compiler never contracts into FMAs (an
// error-free transformation needs every operation rounded on its own); the
// host build is compiled with contraction off.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>

namespace ia {

struct ff {
    float hi, lo;
};

#ifdef __CUDA_ARCH__
__device__ __forceinline__ float ff_add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float ff_sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float ff_mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float ff_fma_rn(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ uint32_t ff_fbits(float v) { return (uint32_t)__float_as_uint(v); }
__device__ __forceinline__ float ff_bitsf(uint32_t b) { return __uint_as_float(b); }
__device__ __forceinline__ uint64_t ff_dbits(double v) { return (uint64_t)__double_as_longlong(v); }
__device__ __forceinline__ double ff_bitsd(uint64_t b) { return __longlong_as_double((long long)b); }
#else
inline float ff_add_rn(float a, float b) { return a + b; }
inline float ff_sub_rn(float a, float b) { return a - b; }
inline float ff_mul_rn(float a, float b) { return a * b; }
inline float ff_fma_rn(float a, float b, float c) { return std::fmaf(a, b, c); }
inline uint32_t ff_fbits(float v) { uint32_t b; __builtin_memcpy(&b, &v, 4); return b; }
inline float ff_bitsf(uint32_t b) { float v; __builtin_memcpy(&v, &b, 4); return v; }
inline uint64_t ff_dbits(double v) { uint64_t b; __builtin_memcpy(&b, &v, 8); return b; }
inline double ff_bitsd(uint64_t b) { double v; __builtin_memcpy(&v, &b, 8); return v; }
#endif

#define FF_HD __host__ __device__ __forceinline__

// ---------------------------------------------------------------- error-free transformations
FF_HD ff two_sum(float a, float b) {
    const float s = ff_add_rn(a, b);
    const float bb = ff_sub_rn(s, a);
    const float e = ff_add_rn(ff_sub_rn(a, ff_sub_rn(s, bb)), ff_sub_rn(b, bb));
    return {s, e};
}
FF_HD ff fast_two_sum(float a, float b) {   // |a| >= |b| (or a == 0)
    const float s = ff_add_rn(a, b);
    return {s, ff_sub_rn(b, ff_sub_rn(s, a))};
}
FF_HD ff two_prod(float a, float b) {
    const float p = ff_mul_rn(a, b);
    return {p, ff_fma_rn(a, b, -p)};
}

// ---------------------------------------------------------------- arithmetic
FF_HD ff ff_from(float a) { return {a, 0.0f}; }
FF_HD ff operator-(ff x) { return {-x.hi, -x.lo}; }
FF_HD ff ff_add(ff x, ff y) {
    const ff s = two_sum(x.hi, y.hi);
    return fast_two_sum(s.hi, ff_add_rn(s.lo, ff_add_rn(x.lo, y.lo)));
}
FF_HD ff ff_sub(ff x, ff y) { return ff_add(x, -y); }
FF_HD ff ff_mul(ff x, ff y) {
    const ff p = two_prod(x.hi, y.hi);
    float e = ff_fma_rn(x.hi, y.lo, p.lo);
    e = ff_fma_rn(x.lo, y.hi, e);
    return fast_two_sum(p.hi, e);
}
FF_HD ff ff_mulf(ff x, float b) {   // by an FP32 number (exact small integers, powers of two, ...)
    const ff p = two_prod(x.hi, b);
    return fast_two_sum(p.hi, ff_fma_rn(x.lo, b, p.lo));
}
// x / y: an FP32 quotient, then one correction from the float-float remainder (Dekker's div2)
FF_HD ff ff_div(ff x, ff y) {
    const float q1 = x.hi / y.hi;
    const ff r = ff_sub(x, ff_mulf(y, q1));
    return fast_two_sum(q1, r.hi / y.hi);
}
FF_HD ff ff_scale2(ff x, float p2) { return {ff_mul_rn(x.hi, p2), ff_mul_rn(x.lo, p2)}; }   // p2 a power of two
FF_HD ff ff_fma(ff a, ff b, ff c) { return ff_add(ff_mul(a, b), c); }                         // a*b + c
FF_HD ff operator+(ff x, ff y) { return ff_add(x, y); }
FF_HD ff operator-(ff x, ff y) { return ff_sub(x, y); }
FF_HD ff operator*(ff x, ff y) { return ff_mul(x, y); }

// ---------------------------------------------------------------- order (normalised pairs)
FF_HD bool ff_lt(ff x, ff y) { return x.hi < y.hi || (x.hi == y.hi && x.lo < y.lo); }
FF_HD bool ff_gt(ff x, ff y) { return ff_lt(y, x); }
FF_HD bool ff_pos(ff x) { return x.hi > 0.0f; }   // x > 0 (the high part carries the sign)
FF_HD bool ff_neg(ff x) { return x.hi < 0.0f; }
FF_HD bool ff_zero(ff x) { return x.hi == 0.0f; }
FF_HD ff ff_abs(ff x) { return x.hi < 0.0f ? -x : x; }
FF_HD ff ff_min(ff a, ff b) { return ff_lt(b, a) ? b : a; }
FF_HD ff ff_max(ff a, ff b) { return ff_lt(a, b) ? b : a; }
FF_HD ff ff_median3(ff a, ff b, ff c) { return ff_max(ff_min(a, b), ff_min(ff_max(a, b), c)); }

// ---------------------------------------------------------------- FP64 conversions (integer only)
// x -> (hi, lo): hi = the top 24 significand bits (truncated), lo = the next 23 (truncated), both
// with x's sign, so hi + lo differs from x by less than 2^-46 |x| and |lo| < ulp(hi).
FF_HD ff ff_split(double x) {
    const uint64_t b = ff_dbits(x);
    const uint32_t h32 = uint32_t(b >> 32), l32 = uint32_t(b);
    const uint32_t sgn = h32 & 0x80000000u;
    const int e = int((h32 >> 20) & 0x7FFu);
    const uint32_t m23 = ((h32 & 0xFFFFFu) << 3) | (l32 >> 29);
    float hi, lo = 0.0f;
    if (e >= 897 && e <= 1150) {
        hi = ff_bitsf(sgn | (uint32_t(e - 896) << 23) | m23);
        if (e >= 920) {
            // the low 29 significand bits are worth low29 * 2^(e-1075); with m = low29 >> 6 that is
            // m * 2^(e-1069) = (2^E (1 + m/2^23)) - 2^E for the FP32 exponent E = e - 1046 (biased
            // e - 919): one exact FP32 subtraction
            const uint32_t eb = sgn | (uint32_t(e - 919) << 23);
            lo = ff_sub_rn(ff_bitsf(eb | ((l32 & 0x1FFFFFFFu) >> 6)), ff_bitsf(eb));
        }
    } else if (e > 1150) {
        const bool nan = e == 2047 && ((h32 & 0xFFFFFu) | l32);
        hi = ff_bitsf(sgn | 0x7F800000u | (nan ? 0x400000u : 0u));
    } else {
        hi = ff_bitsf(sgn);   // ±0
    }
    return {hi, lo};
}
// FP32 -> FP64 bit pattern (exact; FP32 subnormals become ±0, inf and NaN pass through)
FF_HD double ff_widen(float v) {
    const uint32_t u = ff_fbits(v);
    const uint32_t sgn = u & 0x80000000u;
    const uint32_t e = (u >> 23) & 0xFFu, m = u & 0x7FFFFFu;
    uint32_t h32 = sgn, l32 = 0;
    if (e == 0xFFu) {
        h32 |= 0x7FF00000u | (m ? 0x80000u : 0u);
    } else if (e != 0u) {
        h32 |= ((e + 896u) << 20) | (m >> 3);
        l32 = m << 29;
    }
    return ff_bitsd((uint64_t(h32) << 32) | l32);
}
// hi + lo rounded to FP64 (one FP64 addition of the two exact widenings)
FF_HD double ff_join(ff x) { return ff_widen(x.hi) + ff_widen(x.lo); }

// the conversion instruction, out of line on the device: inlined, the compiler if-converts the rare
// branch into every call and the conversion (an FP64-pipe instruction) issues for every value
#ifdef __CUDA_ARCH__
static __device__ __noinline__ float ff_f32_cvt(double v) { return __double2float_rn(v); }
#else
inline float ff_f32_cvt(double v) { return (float)v; }
#endif
// FP64 -> FP32 rounded to nearest even (= float(v), bit for bit) with integer operations where the
// result is a normal FP32 number or a zero, so that no conversion issues on the FP64 pipe; any other
// value (the FP32 subnormal range, overflow to inf, inf, NaN) takes the conversion.
FF_HD float f32_rn(double v) {
    const uint64_t b = ff_dbits(v);
    const uint32_t h32 = uint32_t(b >> 32), l32 = uint32_t(b);
    const int e = int((h32 >> 20) & 0x7FFu);
    if (e >= 897 && e <= 1150) {
        // FP32 exponent e - 896 in [1, 254]; the top 23 significand bits kept, the other 29 rounded
        // away (a carry out of the significand moves into the exponent, up to inf, as rounding does)
        uint32_t f = (uint32_t(e - 896) << 23) | ((h32 & 0xFFFFFu) << 3) | (l32 >> 29);
        const uint32_t rem = l32 & 0x1FFFFFFFu;
        f += (rem > 0x10000000u || (rem == 0x10000000u && (f & 1u))) ? 1u : 0u;
        return ff_bitsf((h32 & 0x80000000u) | f);
    }
    if ((b << 1) == 0) return ff_bitsf(h32 & 0x80000000u);
    return ff_f32_cvt(v);
}

}  // namespace ia
