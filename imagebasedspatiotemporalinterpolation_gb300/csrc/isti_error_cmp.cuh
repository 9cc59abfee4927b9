// Reprojection errors kept squared, compared exactly as their square roots.
//
// computeReprojError (src/renderer.cu:204-215) returns length(e) = RN(sqrt(e.x^2 + e.y^2)),
// and every later use of that value is a comparison: against EPS_1 (:343-344), between the
// two directions (:369) and between cameras (:442).  The square root is monotonic, so the
// kernel stores the squared sum s and compares bit patterns as integers (non-negative
// floats order like their bits), taking square roots only where their rounding decides:
//  - RN(sqrt(s)) < eps  <=>  s < T(eps), T the first float whose root rounds to eps or above
//    (err_threshold; a square root never falls on a rounding midpoint, so the set is a
//    prefix of the floats);
//  - RN(sqrt(a)) < RN(sqrt(b)) is false for a >= b and true when b is 3 or more floats
//    above a (checked for every finite a); for 1 or 2 floats apart both roots are taken.
// Stored patterns (sign bit clear, bit 31 is free for the caller):
//   finite s          its bits
//   ERR_UNSEARCHED    the error FLT_MAX of a direction that was not searched
//   ERR_INF           s = +inf (above FLT_MAX, as the reference's inf is)
//   0x7fc00000 and up NaN: every comparison false
// err_pack / err_eps / err_below / err_less select between these squared patterns and the
// rounded roots.
// Host-compilable, so the comparisons are tested against square roots on the CPU.
#pragma once

#include <stdint.h>
#include <string.h>

#include <bit>

#ifdef __CUDACC__
#define ISTI_EC __host__ __device__ __forceinline__
#else
#include <math.h>
#define ISTI_EC inline
#endif

namespace isti
{
constexpr uint32_t ERR_UNSEARCHED = 0x7f800000u;
constexpr uint32_t ERR_INF = 0x7f800001u;

ISTI_EC uint32_t err_bits(float f)
{
#ifdef __CUDA_ARCH__
    return __float_as_uint(f);
#else
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
#endif
}

ISTI_EC float err_float(uint32_t u)
{
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float f;
    memcpy(&f, &u, 4);
    return f;
#endif
}

ISTI_EC float err_sqrt(float x)
{
#if defined(__CUDA_ARCH__) && defined(ISTI_FASTMATH) && ISTI_FASTMATH
    return sqrtf(x); // the reference's length() under -use_fast_math
#elif defined(__CUDA_ARCH__)
    return __fsqrt_rn(x);
#else
    return sqrtf(x);
#endif
}

// Stored pattern of a squared sum s (>= +0, +inf or NaN).
ISTI_EC uint32_t err_store(float s)
{
    const uint32_t q = err_bits(s) & 0x7fffffffu;
    return q == ERR_UNSEARCHED ? ERR_INF : q;
}

// The first float T with RN(sqrt(T)) >= eps, for a positive normal eps: T is the first float
// above m^2, m the midpoint between eps and the float below it (m^2 has at most 50
// significant bits, so the double product is exact, and is no float).
constexpr uint32_t err_threshold(float eps)
{
    const float below = std::bit_cast<float>(std::bit_cast<uint32_t>(eps) - 1u);
    const double m = (double(eps) + double(below)) * 0.5;
    const double m2 = m * m;
    const float f = float(m2);
    return std::bit_cast<uint32_t>(f) + (double(f) < m2 ? 1u : 0u);
}

// error(q) < eps, with t = err_threshold(eps)
ISTI_EC bool err_lt_eps(uint32_t q, uint32_t t) { return q < t; }

// error(qa) < error(qb) for stored patterns
ISTI_EC bool err_lt(uint32_t qa, uint32_t qb)
{
    if (qa >= qb || qb > ERR_INF)
        return false;
    if (qb - qa >= 3u || qb >= ERR_UNSEARCHED)
        return true;
    return err_sqrt(err_float(qa)) < err_sqrt(err_float(qb));
}

// Selected by SQ: the squared patterns above (true), or the reference's own values (false):
// the bits of the rounded root RN(sqrt(s)) (sign bit cleared), FLT_MAX for a direction that
// was not searched, compared as floats.
template <bool SQ>
constexpr uint32_t ERR_UNSEARCHED_OF = SQ ? ERR_UNSEARCHED : 0x7f7fffffu;

template <bool SQ>
ISTI_EC uint32_t err_pack(float s)
{
    if constexpr (SQ)
        return err_store(s);
    else
        return err_bits(err_sqrt(s)) & 0x7fffffffu;
}

// the second argument of err_below: error < eps <=> err_below(q, err_eps(eps))
template <bool SQ>
constexpr uint32_t err_eps(float eps)
{
    return SQ ? err_threshold(eps) : std::bit_cast<uint32_t>(eps);
}

template <bool SQ>
ISTI_EC bool err_below(uint32_t q, uint32_t t)
{
    if constexpr (SQ)
        return err_lt_eps(q, t);
    else
        return err_float(q) < err_float(t);
}

template <bool SQ>
ISTI_EC bool err_less(uint32_t qa, uint32_t qb)
{
    if constexpr (SQ)
        return err_lt(qa, qb);
    else
        return err_float(qa) < err_float(qb);
}
} // namespace isti
