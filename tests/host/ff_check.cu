// Host check of the float-float arithmetic (interfaceadvection.jl_gb300/csrc/ff.cuh) that the
// momentum kernels use: the same source, compiled for the host with FMA contraction off, against
// exact (long double) results.  Bounds checked, with u = 2^-48:
//   split/join:  |join(split(x)) - x| <= 2 u' |x|, u' = 2^-46 (truncation of 6 + 23 bits)
//   add:         |join(x + y) - (x + y)| <= 8 u (|x| + |y|)
//   mul:         |join(x * y) - x y|     <= 16 u |x y|
//   mulf:        |join(x * b) - x b|     <= 16 u |x b|
//   div:         |join(x / y) - x/y|     <= 16 u |x/y|
// (split inputs carry |lo| up to one ulp of hi, so the dropped lo·lo term and the roundings of the
// FMA chain reach about 9 u in a product)
//   widen:       exact for every normal FP32 number
//   f32_rn:      float(v) bit for bit (round to nearest even)
//   order:       ff_lt agrees with the order of the values unless they are within 8 u of each other
// plus an absolute 2^-140 on every result: below about 2^-100 the low part of a pair reaches the FP32
// subnormal range and the relative bound no longer holds (operands here span 2^-60 .. 2^60, so products
// go down to 2^-120); and the special values (signed zeros, inf, NaN, values below the FP32 normal range).
// Exit status 0 on success.
#include <cmath>
#include <cstdint>
#include <cfloat>
#include <cstdio>
#include <random>

#include "../../interfaceadvection.jl_gb300/csrc/ff.cuh"

using namespace ia;
typedef long double LD;

static int bad = 0;
static void fail(const char* what, double a, double b, double got, double want) {
    if (bad < 20) std::printf("FAIL %s: a=%.17g b=%.17g got=%.17g want=%.17g\n", what, a, b, got, want);
    ++bad;
}

static LD val(ff x) { return (LD)x.hi + (LD)x.lo; }

int main() {
    const double u = std::ldexp(1.0, -48), us = std::ldexp(1.0, -46), tiny = std::ldexp(1.0, -140);
    std::mt19937_64 rng(12345);
    std::uniform_real_distribution<double> mant(1.0, 2.0);
    std::uniform_int_distribution<int> ex(-60, 60), sg(0, 1);
    auto rnd = [&]() { return (sg(rng) ? -1.0 : 1.0) * std::ldexp(mant(rng), ex(rng)); };
    for (int it = 0; it < 2000000; ++it) {
        const double a = rnd(), b = (it % 7 == 0) ? -a * (1.0 + std::ldexp(mant(rng), -30)) : rnd();
        const ff A = ff_split(a), B = ff_split(b);
        if (std::fabs((double)(val(A) - (LD)a)) > us * std::fabs(a)) fail("split", a, 0, (double)val(A), a);
        if (!(std::fabs(A.lo) <= std::fabs(A.hi) * std::ldexp(1.0, -23))) fail("split lo", a, 0, A.lo, A.hi);
        const double j = ff_join(A);
        if (std::fabs(j - (double)val(A)) > std::ldexp(1.0, -53) * std::fabs(j)) fail("join", a, 0, j, (double)val(A));
        const LD xa = val(A), xb = val(B);
        const ff s = ff_add(A, B);
        if ((double)std::fabs(val(s) - (xa + xb)) > 8 * u * (double)(std::fabs(xa) + std::fabs(xb)) + tiny)
            fail("add", a, b, (double)val(s), (double)(xa + xb));
        const ff p = ff_mul(A, B);
        if ((double)std::fabs(val(p) - xa * xb) > 16 * u * (double)std::fabs(xa * xb) + tiny) fail("mul", a, b, (double)val(p), (double)(xa * xb));
        const float fb = (float)b;
        const ff q = ff_mulf(A, fb);
        if ((double)std::fabs(val(q) - xa * (LD)fb) > 16 * u * (double)std::fabs(xa * (LD)fb) + tiny)
            fail("mulf", a, fb, (double)val(q), (double)(xa * (LD)fb));
        const ff dq = ff_div(A, B);
        if ((double)std::fabs(val(dq) - xa / xb) > 16 * u * (double)std::fabs(xa / xb) + tiny)
            fail("div", a, b, (double)val(dq), (double)(xa / xb));
        const bool lt = ff_lt(s, p), want = val(s) < val(p);
        if (lt != want && std::fabs((double)(val(s) - val(p))) > 8 * u * (double)std::fabs(val(p))) fail("lt", a, b, lt, want);
        const ff mx = ff_max(A, B), mn = ff_min(A, B);
        if (val(mx) != std::max(xa, xb) || val(mn) != std::min(xa, xb)) fail("minmax", a, b, (double)val(mx), (double)std::max(xa, xb));
    }
    // widen is exact for random normal FP32 bit patterns
    std::uniform_int_distribution<uint32_t> bits(0, 0xFFFFFFFFu);
    for (int it = 0; it < 1000000; ++it) {
        const uint32_t w = bits(rng);
        const uint32_t e = (w >> 23) & 0xFF;
        if (e == 0 || e == 0xFF) continue;
        const float f = ff_bitsf(w);
        if (ff_widen(f) != (double)f) fail("widen", f, 0, ff_widen(f), (double)f);
    }
    // special values
    const double z = ff_join(ff_split(0.0)), nz = ff_join(ff_split(-0.0));
    if (z != 0.0 || nz != 0.0) fail("zero", 0, 0, z, nz);
    if (ff_split(-0.0).hi != 0.0f || !std::signbit(ff_split(-0.0).hi)) fail("-0 hi", 0, 0, ff_split(-0.0).hi, -0.0);
    if (!std::isnan(ff_join(ff_split(NAN)))) fail("nan", 0, 0, ff_join(ff_split(NAN)), NAN);
    if (ff_join(ff_split(INFINITY)) != INFINITY || ff_join(ff_split(-INFINITY)) != -INFINITY) fail("inf", 0, 0, 0, 0);
    if (ff_join(ff_split(1e300)) != INFINITY) fail("overflow", 1e300, 0, ff_join(ff_split(1e300)), INFINITY);
    if (ff_join(ff_split(1e-300)) != 0.0) fail("underflow", 1e-300, 0, ff_join(ff_split(1e-300)), 0);
    for (double x : {1.0, -1.0, 0.5, 1024.0, 3.0, 0.1, -1e-3, 1.0 / 6.0, 123456.789})
        if (std::fabs(ff_join(ff_split(x)) - x) > us * std::fabs(x)) fail("fixed", x, 0, ff_join(ff_split(x)), x);
    if (!ff_pos(ff_split(1e-20)) || ff_pos(ff_split(-0.0)) || ff_pos(ff_split(0.0)) || !ff_neg(ff_split(-2.0)))
        fail("sign", 0, 0, 0, 0);
    // f32_rn is float(v) bit for bit: random patterns over every exponent and around the FP32 range,
    // exact ties (both parities), carries into the exponent, the largest finite values and zeros
    auto same = [](float x, float y) { return ff_fbits(x) == ff_fbits(y) || (std::isnan(x) && std::isnan(y)); };
    std::uniform_int_distribution<uint64_t> b64(0, ~0ull);
    std::uniform_int_distribution<int> enear(880, 1160);
    for (int it = 0; it < 4000000; ++it) {
        uint64_t w = b64(rng);
        if (it & 1) w = (w & 0x800FFFFFFFFFFFFFull) | (uint64_t(enear(rng)) << 52);
        if ((it & 7) == 2) w = (w & ~0x1FFFFFFFull) | 0x10000000ull;   // a tie
        if ((it & 7) == 4) w |= 0x000FFFFFE0000000ull;                   // top 23 bits all ones
        const double v = ff_bitsd(w);
        if (!same(f32_rn(v), (float)v)) fail("f32_rn", v, 0, f32_rn(v), (float)v);
    }
    for (double v : {0.0, -0.0, 1.0, -1.0, 1e-3, 1000.0, (double)FLT_MAX, -(double)FLT_MAX,
                     std::nextafter((double)FLT_MAX, INFINITY), 3.4028235677973366e38, 3.4028235677973362e38,
                     (double)FLT_MIN, std::nextafter((double)FLT_MIN, 0.0), 1e-45, 1e-300, 1e300, (double)INFINITY,
                     -(double)INFINITY, (double)NAN})
        if (!same(f32_rn(v), (float)v)) fail("f32_rn fixed", v, 0, f32_rn(v), (float)v);
    std::printf(bad ? "FAIL %d\n" : "ok\n", bad);
    return bad != 0;
}
