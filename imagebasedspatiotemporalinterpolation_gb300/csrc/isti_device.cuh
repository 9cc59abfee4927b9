// Device-side arithmetic of the interpolation path.
//
// Every function restates one helper of the reference renderer in the same
// floating-point operation order.  Two arithmetic modes, one per translation unit:
//
//  * IEEE (ISTI_FASTMATH = 0, isti_render.cu): compiled with -fmad=false, and the
//    x-helpers below are the correctly rounded intrinsics, so each result is
//    bit-identical to the host oracle's (and to the reference's code run on the CPU);
//  * reference GPU semantics (ISTI_FASTMATH = 1, isti_render_fm.cu): compiled with
//    the reference's -use_fast_math (CMakeLists.txt:36), the x-helpers are the plain
//    operators, and every expression keeps the reference's tree, so the compiler
//    contracts, divides and takes roots the way it does for the reference's own GPU
//    build.  The exactness shortcuts of the IEEE mode (w / w = 1, quotients decided
//    by an approximation, squared errors, to_8bit without the division) do not hold
//    under those semantics and are replaced by the reference's direct expressions.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#ifndef ISTI_FASTMATH
#define ISTI_FASTMATH 0
#endif

namespace isti
{
// src/renderer.cu:16-28
constexpr float EPS_1_FULL_RES = 0.002f;
constexpr float EPS_1_LOW_RES = EPS_1_FULL_RES * 4.0f;
constexpr float EPS_2_FULL_RES = 0.001f;
constexpr float EPS_2_LOW_RES = 0.004f;
constexpr float EPS_3 = 0.01f;
constexpr unsigned long long SPLAT_EMPTY = 0xfefefefefefefefeull; // cudaMemset(..., 0xfe) of every byte
constexpr uint32_t SOFTSHADOW_BITS = 2u;
constexpr uint32_t SOFTSHADOW_VAL_MASK = 3u;
constexpr bool FAST_MATH = ISTI_FASTMATH != 0;

// one rounding per operation (IEEE) or the plain operator (reference GPU semantics)
__device__ __forceinline__ float xadd(float a, float b)
{
    if constexpr (FAST_MATH)
        return a + b;
    else
        return __fadd_rn(a, b);
}
__device__ __forceinline__ float xsub(float a, float b)
{
    if constexpr (FAST_MATH)
        return a - b;
    else
        return __fsub_rn(a, b);
}
__device__ __forceinline__ float xmul(float a, float b)
{
    if constexpr (FAST_MATH)
        return a * b;
    else
        return __fmul_rn(a, b);
}
__device__ __forceinline__ float xdiv(float a, float b)
{
    if constexpr (FAST_MATH)
        return a / b;
    else
        return __fdiv_rn(a, b);
}
__device__ __forceinline__ float xsqrt(float a)
{
    if constexpr (FAST_MATH)
        return sqrtf(a);
    else
        return __fsqrt_rn(a);
}

struct KeyInfo
{
    float depth;
    uint32_t sx, sy; // source pixel
};

// encodeSplattingKey / decodeSplattingKey, src/renderer.cu:65-74
__device__ __forceinline__ unsigned long long encode_key(float depth, uint32_t x, uint32_t y)
{
    return ((unsigned long long)__float_as_uint(depth) << 32) | (unsigned long long)((x << 16) | y);
}

__device__ __forceinline__ KeyInfo decode_key(unsigned long long key)
{
    KeyInfo k;
    k.depth = __uint_as_float((uint32_t)(key >> 32));
    k.sx = ((uint32_t)key) >> 16;
    k.sy = (uint32_t)(key & 0xFFFFull);
    return k;
}

// pixel2CS, include/util/helper_common.h:66-69: 2 * (p + 0.5) / res - 1
__device__ __forceinline__ float2 pixel2cs(uint32_t px, uint32_t py, uint32_t w, uint32_t h)
{
    float ax = (float)px + 0.5f, ay = (float)py + 0.5f;
    ax = 2.0f * ax;
    ay = 2.0f * ay;
    ax = xdiv(ax, (float)w);
    ay = xdiv(ay, (float)h);
    return make_float2(ax - 1.0f, ay - 1.0f);
}

// CS2pixel, include/util/helper_common.h:71-75: floor((cs + 1) * res * 0.5)
// (float -> int conversion truncates and saturates, NaN -> 0)
__device__ __forceinline__ int2 cs2pixel(float cx, float cy, uint32_t w, uint32_t h)
{
    float ax = cx + 1.0f, ay = cy + 1.0f;
    ax = ax * (float)w;
    ay = ay * (float)h;
    ax = ax * 0.5f;
    ay = ay * 0.5f;
    return make_int2(__float2int_rz(floorf(ax)), __float2int_rz(floorf(ay)));
}

// inRange, include/util/helper_common.h:8-11 (a negative coordinate wraps to >= 2^31 > w)
__device__ __forceinline__ bool in_range(int2 p, uint32_t w, uint32_t h)
{
    return (uint32_t)p.x < w && (uint32_t)p.y < h;
}

// -lim < RN(n / d) < lim, IEEE-exact.  __fdividef is within 2 ulp for
// 2^-126 <= |d| <= 2^126 (CUDA programming guide, intrinsic functions); the
// exact division is only carried out outside that range or when the
// approximate quotient lies within 1e-4 (relative) of the bounds.
__device__ __forceinline__ bool quotient_inside(float n, float d, float lim)
{
    if constexpr (FAST_MATH)
    {
        const float q = n / d;
        return q > -lim && q < lim;
    }
    const float ad = fabsf(d);
    if (ad >= 0x1p-126f && ad <= 0x1p126f)
    {
        const float q = fabsf(__fdividef(n, d));
        if (q < lim * 0.9999f)
            return true;
        if (q > lim * 1.0001f)
            return false;
    }
    const float e = xdiv(n, d);
    return e > -lim && e < lim;
}

// glm-subset mat4 * vec4: (m0*x + m1*y) + (m2*z + m3*w), column-major m
__device__ __forceinline__ float4 matvec(const float *m, float4 v)
{
    float4 r;
    r.x = xadd(xadd(xmul(m[0], v.x), xmul(m[4], v.y)), xadd(xmul(m[8], v.z), xmul(m[12], v.w)));
    r.y = xadd(xadd(xmul(m[1], v.x), xmul(m[5], v.y)), xadd(xmul(m[9], v.z), xmul(m[13], v.w)));
    r.z = xadd(xadd(xmul(m[2], v.x), xmul(m[6], v.y)), xadd(xmul(m[10], v.z), xmul(m[14], v.w)));
    r.w = xadd(xadd(xmul(m[3], v.x), xmul(m[7], v.y)), xadd(xmul(m[11], v.z), xmul(m[15], v.w)));
    return r;
}

// w / w without a division: exactly 1 for finite non-zero w, NaN otherwise
__device__ __forceinline__ float self_ratio(float w)
{
    return (isfinite(w) && w != 0.0f) ? 1.0f : __int_as_float(0x7fffffff);
}

// CS2WS / WS2CS, include/util/helper_common.h:77-87: (M v) / (M v).w
__device__ __forceinline__ float4 project(const float *m, float4 v)
{
    const float4 p = matvec(m, v);
    return make_float4(xdiv(p.x, p.w), xdiv(p.y, p.w), xdiv(p.z, p.w), FAST_MATH ? xdiv(p.w, p.w) : self_ratio(p.w));
}

__device__ __forceinline__ float z_to_depth(float z) { return xmul(xadd(z, 1.0f), 0.5f); } // :89-91
__device__ __forceinline__ float depth_to_z(float d) { return xsub(xmul(d, 2.0f), 1.0f); } // :93-95

// lerp_color, include/util/helper_common.h:22-25: (a + t * (b - a)) / 255
__device__ __forceinline__ float lerp_ch(uint32_t a, uint32_t b, float t)
{
    const float fa = (float)a, fb = (float)b;
    return xdiv(xadd(fa, xmul(t, xsub(fb, fa))), 255.f);
}

// to_8bit, include/util/helper_common.h:27-30: min(255, max(0, int(f * 255)))
__device__ __forceinline__ uint32_t to_8bit(float f)
{
    const int v = __float2int_rz(xmul(f, 255.f));
    return (uint32_t)min(255, max(0, v));
}

// to_8bit(v / 255) for v = a + t * (b - a).  The round trip RN(RN(v / 255) * 255)
// stays within 256 * 2^-23 = 2^-15 of v for 0 <= v < 256 and returns every integer
// 0..255 unchanged, so its truncation is floor(v) unless v lies within 2^-12 of an
// integer without being one; only that case (and v outside [0, 256), NaN) takes
// the division.
__device__ __forceinline__ uint32_t to_8bit_255ths(float v)
{
    if constexpr (FAST_MATH)
        return to_8bit(v / 255.f);
    const float fl = floorf(v);
    const float fr = xsub(v, fl);
    if (v >= 0.0f && v < 256.0f && (fr == 0.0f || (fr > 0x1p-12f && fr < 1.0f - 0x1p-12f)))
        return (uint32_t)fl;
    return to_8bit(xdiv(v, 255.f));
}

// color_to_uchar4(lerp_color(a, b, t)), packed RGBA8 in a uint32 (R in bits 0-7)
__device__ __forceinline__ uint32_t lerp_color_u8(uint32_t a, uint32_t b, float t)
{
    uint32_t r = 0;
#pragma unroll
    for (int c = 0; c < 4; c++)
    {
        const float fa = (float)((a >> (8 * c)) & 255u), fb = (float)((b >> (8 * c)) & 255u);
        r |= to_8bit_255ths(xadd(fa, xmul(t, xsub(fb, fa)))) << (8 * c);
    }
    return r;
}

// sqrtf(s) < e; IEEE-exact mode: the square root is only taken within 0.01 % of e^2
__device__ __forceinline__ bool sqrt_less(float s, float e)
{
    if constexpr (FAST_MATH)
        return sqrtf(s) < e;
    const float e2 = e * e;
    if (s < e2 * 0.9999f)
        return true;
    if (s > e2 * 1.0001f)
        return false;
    return xsqrt(s) < e;
}

// float -> unsigned char of make_uchar4(float, ...): truncation, saturation, NaN -> 0
__device__ __forceinline__ uint32_t cvt_u8(float f)
{
    return (uint32_t)min(255u, __float2uint_rz(f));
}
} // namespace isti
