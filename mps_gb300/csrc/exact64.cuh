// Correctly rounded FP64 square root and division computed on the integer
// and FP32 pipes.
//
// GB300 issues FP64 at 1/64 of its FP32 rate, and an FP64 square root or
// division is a sequence of about ten FP64 operations (measured on the whole
// GPU: 52 G/s each, against 67 TFLOP/s of FP32 FMA).  The neighbour sweeps
// need the correctly rounded results, not approximations: distances and
// weights are compared bit for bit with the reference implementation.  These
// routines return exactly the IEEE 754 round-to-nearest-even result from
//   1. an FP32 first approximation: the hardware reciprocal square root or
//      reciprocal (any with relative error below 2^-12; the hardware's are
//      2 ulp) refined by one Newton step in FP32 FMAs, which leaves a relative
//      error below 2^-22 that rests on IEEE FP32 rounding alone,
//   2. two Newton-Raphson corrections whose residuals are computed exactly in
//      64-bit integer arithmetic (modulo 2^64 where the true value is known to
//      be small), so that the only error left after the second one is the
//      FP32 rounding of a small correction: within 0.52 units in the last
//      place of the exact result, and
//   3. a rounding test on the exact integer remainder, which moves the result
//      by at most one unit: Tuckerman's test for the square root
//      (S = RN(sqrt N) iff -S < N - S^2 <= S), |R| < d/2 for the quotient
//      (a quotient of two 53-bit significands is never a midpoint).
// No conversion instruction is used (the 64-bit ones run on the FP64 pipe):
// integers of magnitude below 2^22 cross to FP32 and back through the FP32
// adder (the 1.5 * 2^23 exponent trick), larger ones are shifted down first.
// Only positive normal inputs with a normal result take this path; zero,
// subnormals, infinities, NaN and negative square-root arguments return false
// and the caller uses the FP64 instruction sequence.
//
// Error budget of step 2 with the step-1 error eta <= 2^-22 (each range
// below still holds for eta up to 2^-20):
// square root - D = m2 - 16 s0^2 = (N - S0^2) / 2^52 is exact, |D| <= 2^33
// (D >> 13 fits the 2^22 conversion range up to 2^35); the first correction
// c1 = D 2^23 / s0 (<= 2^32) is formed from D >> 13 and rounded to a
// multiple of 2^12: off by <= 2^12.8, plus the exact Newton step's overshoot
// eta^2 S / 2 <= 2^8; e = 2^23 D - s0 c1 is exact (|e| <= 2^37.8; e >> 17
// fits up to 2^39), N - S1^2 = 2^29 e - c1^2 is evaluated in FP32 within
// 2^46.2 (2^-6.8 units after the division by 2 S1 >= 2^53), and 1 / (2 S1) is
// taken as 2^-29 / s0 (1 - c1 / S0) within a relative 2^-22 on a correction
// <= 2^12.9 (2^-9 units).
// Division - q0 = fa / fb cut to 24 bits has relative error <= 2^-21.3;
// D = (ma 2^sh - mb Q0) / 2^28 is exact modulo 2^64 (|D| <= 2^56.7; D >> 36
// fits up to 2^58); the exact Newton step of a quotient has no quadratic
// term, so c1 = D 2^28 / mb (formed from D >> 36, rounded to a multiple of
// 2^12) is off by <= 2^12.8 only; T = (ma 2^sh - mb Q1) / 2^12 is exact modulo
// 2^64 (|T| <= 2^53.8; T >> 33 fits up to 2^55), and c2 = T 2^12 / mb from
// T >> 33 is within 0.01 units.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define MPS_X64_FN __host__ __device__ __forceinline__
#else
#define MPS_X64_FN inline
#endif

namespace mpsg {
namespace x64 {

constexpr uint64_t kMant = (1ull << 52) - 1;
constexpr uint64_t kHidden = 1ull << 52;

MPS_X64_FN uint64_t bits_of(double x) {
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t u;
    std::memcpy(&u, &x, sizeof u);
    return u;
#endif
}

MPS_X64_FN double double_of(uint64_t u) {
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)u);
#else
    double x;
    std::memcpy(&x, &u, sizeof x);
    return x;
#endif
}

MPS_X64_FN float f_of(uint32_t u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float f;
    std::memcpy(&f, &u, sizeof f);
    return f;
#endif
}

MPS_X64_FN uint32_t u_of(float f) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(f);
#else
    uint32_t u;
    std::memcpy(&u, &f, sizeof u);
    return u;
#endif
}

// Conversions without the conversion instructions (the 64-bit ones run on
// the FP64 pipe): |v| < 2^22 between int32 and FP32 through the FP32 adder
// and the exponent 1.5 * 2^23, and a float in [2^23, 2^26) (an integer) to
// uint64 from its bit fields.
MPS_X64_FN float i2f_small(int32_t v) { return f_of(0x4B400000u + (uint32_t)v) - 12582912.0f; }
MPS_X64_FN int32_t f2i_small(float x) { return (int32_t)(u_of(x + 12582912.0f) - 0x4B400000u); }
MPS_X64_FN uint64_t u_of_big(float f) {
    const uint32_t u = u_of(f);
    return (uint64_t)((u & 0x7FFFFFu) | 0x800000u) << ((u >> 23) - 150u);
}

MPS_X64_FN int clz64(uint64_t v) {
#ifdef __CUDA_ARCH__
    return __clzll((long long)v);
#else
    return __builtin_clzll(v);
#endif
}

// q - 1 for 1 <= q < 2^53, which is exact (a multiple of q's unit in the last
// place, below q); false for any other q.
MPS_X64_FN bool sub_one(double q, double& out) {
    const uint64_t Q = bits_of(q);
    const uint32_t E = (uint32_t)(Q >> 52);  // the sign bit included
    if (E - 1023u > 52u) return false;
    const uint64_t D = ((Q & kMant) | kHidden) - (1ull << (1075u - E));
    if (D == 0) {
        out = 0.0;
        return true;
    }
    const int lz = clz64(D) - 11;
    out = double_of(((uint64_t)(E - (uint32_t)lz - 1u) << 52) + (D << lz));
    return true;
}

// x rounded to FP32 (nearest, ties to even) for zero and for x in the FP32
// normal range; false for the rest (subnormal or overflowing results, inf,
// NaN).
MPS_X64_FN bool to_f32(double x, float& out) {
    const uint64_t X = bits_of(x);
    const uint32_t E = (uint32_t)(X >> 52) & 0x7ffu;
    const uint32_t sign = (uint32_t)(X >> 32) & 0x80000000u;
    if (E - 897u > 253u) {
        if ((X << 1) != 0) return false;
        out = f_of(sign);
        return true;
    }
    const uint64_t m = X & kMant;
    const uint32_t top = (uint32_t)(m >> 29);
    const uint32_t rem = (uint32_t)m & 0x1FFFFFFFu;
    const uint32_t up = (rem > 0x10000000u || (rem == 0x10000000u && (top & 1u))) ? 1u : 0u;
    out = f_of(sign | ((((E - 896u) << 23) | top) + up));
    return true;
}

// v < cut for a cut > 0 and a v that is >= 0 or NaN (a squared distance or a
// distance): the order of such doubles is the order of their bit patterns.
MPS_X64_FN bool lt_cut(double v, double cut) { return (int64_t)bits_of(v) < (int64_t)bits_of(cut); }

// One Newton step on FP32 approximations of 1/sqrt(x) and 1/x: relative
// error below 2^-12 in, below 2^-22.5 out.
MPS_X64_FN float refine_rsqrt(float x, float y) {
    return fmaf(0.5f * y, fmaf(-(x * y), y, 1.0f), y);
}
MPS_X64_FN float refine_rcp(float x, float y) { return fmaf(y, fmaf(-x, y, 1.0f), y); }

// sqrt(x) for a positive normal x, correctly rounded (see the file comment).
// Ap supplies the raw FP32 approximations Ap::rsqrt(f) ~ 1/sqrt(f) and
// Ap::rcp(f) ~ 1/f (relative error below 2^-12).
template <class Ap>
MPS_X64_FN bool sqrt_rn(double x, double& out) {
    const uint64_t X = bits_of(x);
    const uint32_t E = (uint32_t)(X >> 52);  // the sign bit included
    if (E - 1u >= 2046u) return false;       // zero, subnormal, infinite, NaN or negative
    const uint64_t m = (X & kMant) | kHidden;
    const int t = (int)E - 1075;  // x = m 2^t
    const int odd = t & 1;
    const uint64_t m2 = m << odd;    // [2^52, 2^54); x = m2 2^(t - odd)
    const int half = (t - odd) / 2;  // exact: t - odd is even
    // S = RN(sqrt(N)), N = m2 2^52 in [2^104, 2^106): S in [2^52, 2^53) and
    // sqrt(x) = S 2^(half - 26).  mf: m2 / 2^22 cut to 24 bits, in [2^30, 2^32).
    const float mf = f_of(((uint32_t)(157 + odd) << 23) | (uint32_t)((X >> 29) & 0x7FFFFFu));
    const float s512 = mf * refine_rsqrt(mf, Ap::rsqrt(mf)) * 512.0f;  // ~ sqrt(N) / 2^28
    const uint64_t s0 = u_of_big(s512);               // S0 = s0 2^28, s0 in [2^24, 2^25]
    const int64_t D = (int64_t)(m2 - 16u * s0 * s0);  // (N - S0^2) / 2^52, exact
    const float inv_s0 = refine_rcp(s512, Ap::rcp(s512));
    // c1 = D 2^23 / s0 = k 2^12 (D taken to 2^13: |D| < 2^35)
    const int32_t k = f2i_small(i2f_small((int32_t)(D >> 13)) * (inv_s0 * 16777216.0f));
    const int64_t c1 = (int64_t)k * 4096;
    const int64_t e = (int64_t)(((uint64_t)D << 23) - (uint64_t)((int64_t)s0 * c1));  // exact
    // N - S1^2 = 2^29 e - c1^2 for S1 = S0 + c1 (e taken to 2^17), and
    // 1 / (2 S1) = 2^-29 / s0 / (1 + c1 / S0) ~ 2^-29 / s0 (1 - c1 / S0)
    const float c1f = i2f_small(k) * 4096.0f;
    const float r1 = i2f_small((int32_t)(e >> 17)) * 70368744177664.0f - c1f * c1f;
    const float inv2s1 = inv_s0 * 1.862645149230957e-9f * (1.0f - c1f * inv_s0 * 3.725290298461914e-9f);
    const int64_t c2 = f2i_small(r1 * inv2s1);
    uint64_t S = (s0 << 28) + (uint64_t)(c1 + c2);
    // Tuckerman's test on the exact remainder (|N - S^2| < 2^56: mod 2^64 is exact)
    const int64_t R = (int64_t)((m2 << 52) - S * S);
    if (R > (int64_t)S)
        S++;
    else if (R <= -(int64_t)S)
        S--;
    out = double_of(((uint64_t)(half + 1048) << 52) + S);  // biased exponent half - 26 + 1075
    return true;
}

// a / b for normal a, b whose quotient is normal, correctly rounded.
template <class Ap>
MPS_X64_FN bool div_rn(double a, double b, double& out) {
    const uint64_t A = bits_of(a), B = bits_of(b);
    const uint32_t Ea = (uint32_t)(A >> 52) & 0x7ffu, Eb = (uint32_t)(B >> 52) & 0x7ffu;
    if (Ea - 1u >= 2046u || Eb - 1u >= 2046u) return false;
    const uint64_t ma = (A & kMant) | kHidden, mb = (B & kMant) | kHidden;
    const int lt = ma < mb ? 1 : 0;
    const int sh = 52 + lt;
    // a / b = Q* 2^eq with Q* = ma 2^sh / mb in [2^52, 2^53)
    const int be = (int)Ea - (int)Eb - sh + 1075;  // biased exponent of the result
    if (be < 1 || be > 2046) return false;
    // the significands cut to 24 bits, in [1, 2)
    const float fa = f_of(0x3F800000u | (uint32_t)((A >> 29) & 0x7FFFFFu));
    const float fb = f_of(0x3F800000u | (uint32_t)((B >> 29) & 0x7FFFFFu));
    const float ib = refine_rcp(fb, Ap::rcp(fb));  // ~ 2^52 / mb
    const uint64_t q0 = u_of_big(fa * ib * (lt ? 33554432.0f : 16777216.0f));  // Q0 = q0 2^28
    // (A' - mb Q0) / 2^28 with A' = ma 2^sh: exact modulo 2^64, |D| < 2^58
    const int64_t D = (int64_t)((ma << (sh - 28)) - mb * q0);
    // c1 = D 2^28 / mb = k 2^12 (D taken to 2^36)
    const int32_t k = f2i_small(i2f_small((int32_t)(D >> 36)) * ib);
    // T = R1 / 2^12 = 2^16 D - mb k with R1 = A' - mb (Q0 + c1): exact modulo
    // 2^64, |T| < 2^55
    const int64_t T = (int64_t)(((uint64_t)D << 16) - mb * (uint64_t)(int64_t)k);
    // c2 = R1 / mb = T 2^12 / mb (T taken to 2^33)
    const int64_t c2 = f2i_small(i2f_small((int32_t)(T >> 33)) * (ib * 0.0078125f));
    uint64_t Q = (q0 << 28) + (uint64_t)((int64_t)k * 4096 + c2);
    // |A' - mb Q| < mb / 2 <=> Q = RN(Q*); the remainder is exact modulo 2^64
    const int64_t R = (int64_t)((ma << sh) - mb * Q);
    if (2 * R >= (int64_t)mb)
        Q++;
    else if (2 * R <= -(int64_t)mb)
        Q--;
    out = double_of(((A ^ B) & (1ull << 63)) | (((uint64_t)(be - 1) << 52) + Q));
    return true;
}

}  // namespace x64
}  // namespace mpsg
