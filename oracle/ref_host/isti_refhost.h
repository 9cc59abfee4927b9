// Host emulation of the CUDA device built-ins that the reference's
// src/renderer.cu uses, so that file can be compiled by g++ and executed on
// the CPU as a test oracle.  Force-included (g++ -include) ahead of the
// reference sources; compiled with -D__host__= -D__device__= -D__global__=.
//
// Test infrastructure only: nothing in the product links or loads this.
//
// Emulated semantics (CUDA programming guide / PTX ISA):
//  * tex2D<T>(tex, x, y): point filtering, unnormalised coordinates, border
//    address mode -> texel (floor x, floor y), zero outside the image
//    (the reference creates every texture that way, src/util/image_buffer.cu:54-58,227-249).
//  * surf2Dwrite / surf2Dread: byte x offset, element y, in range.
//  * atomicMin(u64) / atomicAdd(f32): read-modify-write on one host thread.
//  * __float2uint_rn/_rd/_ru: round (nearest-even / down / up) then saturate
//    to [0, 2^32-1]; NaN -> 0 (PTX cvt.rni/rmi/rpi.u32.f32).
//  * kernel launch: blocks in row-major order, threads in row-major order
//    inside a block, one at a time.  Every kernel on the path is per-thread
//    independent except for the order-independent 64-bit atomicMin.
#pragma once

#include <cuda_runtime.h>

#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <functional>
#include <iomanip>
#include <iostream>
#include <memory>
#include <optional>
#include <sstream>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

inline uint3 threadIdx;
inline uint3 blockIdx;
inline dim3 blockDim;
inline dim3 gridDim;

namespace isti_refhost
{
struct Image
{
    void *ptr;
    unsigned w, h;
    size_t elem;
};

// Registry of host "device images"; handle = index + 1 (0 is never issued).
const Image &image(unsigned long long handle);
unsigned long long register_image(void *ptr, unsigned w, unsigned h, size_t elem);

template <class K>
struct Launcher
{
    dim3 grid, block;
    K kernel;
    template <class... A>
    void operator()(A... args) const
    {
        gridDim = grid;
        blockDim = block;
        for (unsigned bz = 0; bz < grid.z; bz++)
            for (unsigned by = 0; by < grid.y; by++)
                for (unsigned bx = 0; bx < grid.x; bx++)
                    for (unsigned tz = 0; tz < block.z; tz++)
                        for (unsigned ty = 0; ty < block.y; ty++)
                            for (unsigned tx = 0; tx < block.x; tx++)
                            {
                                blockIdx = make_uint3(bx, by, bz);
                                threadIdx = make_uint3(tx, ty, tz);
                                kernel(args...);
                            }
    }
};

template <class K>
Launcher<K> launch(dim3 grid, dim3 block, K kernel)
{
    return Launcher<K>{grid, block, kernel};
}
} // namespace isti_refhost

template <class T>
inline T tex2D(cudaTextureObject_t tex, float x, float y)
{
    const isti_refhost::Image &im = isti_refhost::image(tex);
    const float fx = std::floor(x), fy = std::floor(y);
    if (!(fx >= 0.0f && fx < (float)im.w && fy >= 0.0f && fy < (float)im.h))
        return T{};
    return static_cast<const T *>(im.ptr)[(size_t)fy * im.w + (size_t)fx];
}

template <class T>
inline T surf2Dread(cudaSurfaceObject_t surf, int x_bytes, int y)
{
    const isti_refhost::Image &im = isti_refhost::image(surf);
    const size_t x = (size_t)x_bytes / sizeof(T);
    if (x_bytes < 0 || y < 0 || x >= im.w || (unsigned)y >= im.h)
        throw std::runtime_error("surf2Dread out of range");
    return static_cast<const T *>(im.ptr)[(size_t)y * im.w + x];
}

template <class T>
inline void surf2Dwrite(T val, cudaSurfaceObject_t surf, int x_bytes, int y)
{
    const isti_refhost::Image &im = isti_refhost::image(surf);
    const size_t x = (size_t)x_bytes / sizeof(T);
    if (x_bytes < 0 || y < 0 || x >= im.w || (unsigned)y >= im.h)
        throw std::runtime_error("surf2Dwrite out of range");
    static_cast<T *>(im.ptr)[(size_t)y * im.w + x] = val;
}

inline unsigned long long atomicMin(unsigned long long *address, unsigned long long val)
{
    const unsigned long long old = *address;
    if (val < old)
        *address = val;
    return old;
}

inline float atomicAdd(float *address, float val)
{
    const float old = *address;
    *address = old + val;
    return old;
}

namespace isti_refhost
{
inline unsigned int saturate_u32(double r)
{
    if (std::isnan(r) || r <= 0.0)
        return 0u;
    if (r >= 4294967295.0)
        return 4294967295u;
    return (unsigned int)r;
}
} // namespace isti_refhost

inline unsigned int __float2uint_rn(float x) { return isti_refhost::saturate_u32(std::nearbyint((double)x)); }
inline unsigned int __float2uint_rd(float x) { return isti_refhost::saturate_u32(std::floor((double)x)); }
inline unsigned int __float2uint_ru(float x) { return isti_refhost::saturate_u32(std::ceil((double)x)); }
