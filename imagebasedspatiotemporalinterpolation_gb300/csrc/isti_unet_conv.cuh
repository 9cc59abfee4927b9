// Implicit-GEMM convolutions of the learned flow initialiser on the tcgen05 tensor core.
//
// Activations are NHWC bf16 (channels innermost, a multiple of 16); weights are kept as
// f32 masters [cout][tap][cin] (tap = 3 * (dy + 1) + (dx + 1) for 3x3, 0 for 1x1) and
// packed to bf16 operand images by pack_kernel.
//
// conv_kernel (forward, and the data gradient with packed transposed weights): one CTA of
// 128 threads computes a tile of 16 x 8 output pixels (M = 128) x all output channels
// (N = cout <= 256) into TMEM.  The K loop runs over (tap, chunk of ck input channels)
// stages through a ring in shared memory:
//   warp 0, one thread: per stage, ck / 8 TMA boxes {8 channels, 16 x, 8 y} of the input at
//     the tap's offset (zero fill outside the image = the convolution's zero padding) and
//     one bulk copy of the stage's packed weights, completion on full[s];
//   warp 1, one thread: waits full[s], issues ck / 16 tcgen05.mma (K = 16 each) and commits
//     to empty[s], which frees the stage for the producer; after the last stage, commits
//     to `done`;
//   all four warps (epilogue): wait `done`, read their 32 TMEM lanes (= tile rows) with
//     tcgen05.ld, add the bias, apply ReLU and/or the gradient mask (x > 0 of a saved
//     activation), convert to bf16 and store the pixel's channels.
// Every mbarrier wait is bounded; on timeout the status word is set, the loops stop, the
// producer waits (bounded) for the copies it issued, and TMEM is freed before returning.
//
// wgrad_kernel (weight gradient): D[co][ci] of one tap = sum over pixels of
// dY[p][co] * X[p + offset(tap)][ci], with M = 128 (cout padded; the padding boxes are
// never loaded and stay zero), N = cin, K = pixels: both operands are MN-major (the
// channel runs along the 16-byte row), again as TMA boxes of 8 channels x 128 pixels; for
// them the descriptor's LBO steps along K and its SBO along M/N (checked against torch).
// A CTA covers one tap and a range of pixel tiles and writes its partial sums; a second
// kernel adds the partials in a fixed order (deterministic).
#pragma once

#include "isti_tc.cuh"

#include <cuda_bf16.h>
#include <stdint.h>

namespace isti_unet
{
using namespace isti_tc;

constexpr int CONV_THREADS = 128;
constexpr int TILE_W = 16, TILE_H = 8, TILE_M = TILE_W * TILE_H;
constexpr uint32_t BOX_BYTES = TILE_M * 16; // one TMA box: 8 channels x 128 pixels

__host__ __device__ constexpr uint32_t tmem_cols(int n)
{
    uint32_t c = 32;
    while (c < (uint32_t)n)
        c <<= 1;
    return c;
}

struct ConvParams
{
    const __nv_bfloat16 *wpack; // packed weights: per stage ck x cout, K-major core matrices [ck/8][cout/8][8][8]
    const float *bias;          // cout, or null
    const __nv_bfloat16 *mask;  // NHWC, cout channels: output *= (mask > 0); or null
    __nv_bfloat16 *out;         // NHWC, cout channels
    int32_t *status;
    int w, h, b;
    int cin, cout, ck;          // ck: input channels per stage (16 or 32)
    int tiles_x, tiles_y;
    int relu;
    int stages;                 // depth of the shared-memory ring
};

__host__ __device__ constexpr uint32_t conv_stage_bytes(int ck, int cout) { return (uint32_t)ck * 256u + (uint32_t)ck * cout * 2u; }

// bf16 > 0 (positive, non-zero, not NaN)
__device__ __forceinline__ bool bf16_positive(uint16_t b) { return (b & 0x8000u) == 0 && (b & 0x7fffu) != 0 && (b & 0x7fffu) <= 0x7f80u; }

template <int TAPS>
__global__ void __launch_bounds__(CONV_THREADS) conv_kernel(const __grid_constant__ ConvParams p, const __grid_constant__ CUtensorMap xmap)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    const int S = p.stages;
    const uint32_t a_bytes = (uint32_t)p.ck * 256u, b_bytes = (uint32_t)p.ck * p.cout * 2u, stage_bytes = a_bytes + b_bytes;
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + (size_t)S * stage_bytes);
    uint64_t *empty = full + S;
    uint64_t *done = empty + S;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(done + 1);
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;

    int t = blockIdx.x;
    const int tx = t % p.tiles_x;
    t /= p.tiles_x;
    const int ty = t % p.tiles_y;
    const int bi = t / p.tiles_y;
    const int x0 = tx * TILE_W, y0 = ty * TILE_H;
    const uint32_t ncols = tmem_cols(p.cout);

    if (threadIdx.x == 0)
    {
        for (int s = 0; s < S; s++)
        {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(done, 1);
        fence_barrier_init();
    }
    if (warp == 0)
        tmem_alloc(tmem_slot, ncols);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    const int chunks = p.cin / p.ck, iters = TAPS * chunks;
    if (warp == 0 && lane == 0)
    {
        int issued = 0;
        for (int it = 0; it < iters; it++)
        {
            const int s = it % S, r = it / S;
            if (r > 0 && !mbar_wait(&empty[s], (uint32_t)((r - 1) & 1), p.status))
                break;
            uint8_t *st = smem + (size_t)s * stage_bytes;
            mbar_expect_tx(&full[s], stage_bytes);
            const int tap = it / chunks, c = it % chunks;
            const int dy = TAPS == 9 ? tap / 3 - 1 : 0, dx = TAPS == 9 ? tap % 3 - 1 : 0;
            for (int j = 0; j < p.ck / 8; j++)
                tma_load_4d(st + j * BOX_BYTES, &xmap, c * p.ck + 8 * j, x0 + dx, y0 + dy, bi, &full[s]);
            bulk_load(st + a_bytes, p.wpack + (size_t)it * p.ck * p.cout, b_bytes, &full[s]);
            issued = it + 1;
        }
        for (int it = issued > S ? issued - S : 0; it < issued; it++) // copies still landing
            if (!mbar_wait(&full[it % S], (uint32_t)((it / S) & 1), p.status))
                break;
    }
    else if (warp == 1 && lane == 0)
    {
        const uint32_t idesc = idesc_bf16(TILE_M, (uint32_t)p.cout, 0, 0);
        const uint32_t lbo_b = (uint32_t)(p.cout / 8) * 128u;
        for (int it = 0; it < iters; it++)
        {
            const int s = it % S, r = it / S;
            if (!mbar_wait(&full[s], (uint32_t)(r & 1), p.status))
                break;
            tc_fence_after();
            const uint32_t a0 = smem_u32(smem + (size_t)s * stage_bytes), b0 = a0 + a_bytes;
            for (int k = 0; k < p.ck / 16; k++)
                mma_bf16(tmem, smem_desc(a0 + k * 2 * BOX_BYTES, BOX_BYTES, 128), smem_desc(b0 + k * 2 * lbo_b, lbo_b, 128), idesc,
                         it > 0 || k > 0);
            mma_commit(&empty[s]);
        }
        mma_commit(done);
    }
    __syncwarp();

    const bool ok = mbar_wait(done, 0, p.status);
    tc_fence_after();
    if (ok)
    {
        const int m = warp * 32 + lane; // TMEM lane = tile row
        const int px = x0 + (m % TILE_W), py = y0 + (m / TILE_W);
        const bool inb = px < p.w && py < p.h;
        const size_t pix = ((size_t)bi * p.h + (inb ? py : 0)) * p.w + (inb ? px : 0);
        for (int c0 = 0; c0 < p.cout; c0 += 16)
        {
            uint32_t r[16];
            tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, r);
            tmem_ld_wait();
            if (!inb)
                continue;
            float v[16];
#pragma unroll
            for (int i = 0; i < 16; i++)
            {
                v[i] = __uint_as_float(r[i]);
                if (p.bias)
                    v[i] += __ldg(p.bias + c0 + i);
                if (p.relu)
                    v[i] = fmaxf(v[i], 0.0f);
            }
            if (p.mask)
            {
                const uint4 *mk = reinterpret_cast<const uint4 *>(p.mask + pix * p.cout + c0);
                const uint4 m0 = __ldg(mk), m1 = __ldg(mk + 1);
                const uint32_t mw[8] = {m0.x, m0.y, m0.z, m0.w, m1.x, m1.y, m1.z, m1.w};
#pragma unroll
                for (int i = 0; i < 16; i++)
                    if (!bf16_positive((uint16_t)(mw[i / 2] >> (16 * (i % 2)))))
                        v[i] = 0.0f;
            }
            uint32_t o[8];
#pragma unroll
            for (int i = 0; i < 8; i++)
            {
                const __nv_bfloat162 h = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
                o[i] = *reinterpret_cast<const uint32_t *>(&h);
            }
            uint4 *dst = reinterpret_cast<uint4 *>(p.out + pix * p.cout + c0);
            dst[0] = make_uint4(o[0], o[1], o[2], o[3]);
            dst[1] = make_uint4(o[4], o[5], o[6], o[7]);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0)
        tmem_dealloc(tmem, ncols);
}

struct WgradParams
{
    float *partial; // [splits][cout][TAPS][cin]
    int32_t *status;
    int w, h, b;
    int cin, cout;
    int tiles_x, tiles_y, n_tiles, tiles_per_split;
    int stages;
};

__host__ __device__ constexpr uint32_t wgrad_a_bytes() { return 16u * BOX_BYTES; } // M = 128 output channels
__host__ __device__ constexpr uint32_t wgrad_stage_bytes(int cin) { return wgrad_a_bytes() + (uint32_t)(cin / 8) * BOX_BYTES; }

template <int TAPS>
__global__ void __launch_bounds__(CONV_THREADS) wgrad_kernel(const __grid_constant__ WgradParams p, const __grid_constant__ CUtensorMap dymap,
                                                             const __grid_constant__ CUtensorMap xmap)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    const int S = p.stages;
    const uint32_t a_bytes = wgrad_a_bytes(), stage_bytes = wgrad_stage_bytes(p.cin);
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + (size_t)S * stage_bytes);
    uint64_t *empty = full + S;
    uint64_t *done = empty + S;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(done + 1);
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const int tap = blockIdx.y, split = blockIdx.x;
    const int dy = TAPS == 9 ? tap / 3 - 1 : 0, dx = TAPS == 9 ? tap % 3 - 1 : 0;
    const int t_begin = split * p.tiles_per_split;
    const int t_end = min(p.n_tiles, t_begin + p.tiles_per_split);
    const uint32_t ncols = tmem_cols(p.cin);

    // the output-channel boxes beyond cout are never loaded: zero once, for every stage
    for (uint32_t i = threadIdx.x * 16u; i < (uint32_t)S * stage_bytes; i += CONV_THREADS * 16u)
        *reinterpret_cast<uint4 *>(smem + i) = make_uint4(0, 0, 0, 0);
    fence_proxy_async();
    if (threadIdx.x == 0)
    {
        for (int s = 0; s < S; s++)
        {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(done, 1);
        fence_barrier_init();
    }
    if (warp == 0)
        tmem_alloc(tmem_slot, ncols);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const int iters = t_end > t_begin ? t_end - t_begin : 0;
    const uint32_t tx_bytes = (uint32_t)(p.cout / 8 + p.cin / 8) * BOX_BYTES;

    if (warp == 0 && lane == 0)
    {
        int issued = 0;
        for (int it = 0; it < iters; it++)
        {
            const int s = it % S, r = it / S;
            if (r > 0 && !mbar_wait(&empty[s], (uint32_t)((r - 1) & 1), p.status))
                break;
            int t = t_begin + it;
            const int tx = t % p.tiles_x;
            t /= p.tiles_x;
            const int ty = t % p.tiles_y;
            const int bi = t / p.tiles_y;
            uint8_t *st = smem + (size_t)s * stage_bytes;
            mbar_expect_tx(&full[s], tx_bytes);
            for (int j = 0; j < p.cout / 8; j++)
                tma_load_4d(st + j * BOX_BYTES, &dymap, 8 * j, tx * TILE_W, ty * TILE_H, bi, &full[s]);
            for (int j = 0; j < p.cin / 8; j++)
                tma_load_4d(st + a_bytes + j * BOX_BYTES, &xmap, 8 * j, tx * TILE_W + dx, ty * TILE_H + dy, bi, &full[s]);
            issued = it + 1;
        }
        for (int it = issued > S ? issued - S : 0; it < issued; it++)
            if (!mbar_wait(&full[it % S], (uint32_t)((it / S) & 1), p.status))
                break;
    }
    else if (warp == 1 && lane == 0)
    {
        const uint32_t idesc = idesc_bf16(TILE_M, (uint32_t)p.cin, 1, 1);
        // MN-major operands: LBO = distance between core matrices adjacent in K (the next 8
        // pixels, 128 bytes on), SBO = between core matrices adjacent in M/N (the next 8
        // channels, the next box)
        const uint32_t lbo = 128u, sbo = BOX_BYTES;
        for (int it = 0; it < iters; it++)
        {
            const int s = it % S, r = it / S;
            if (!mbar_wait(&full[s], (uint32_t)(r & 1), p.status))
                break;
            tc_fence_after();
            const uint32_t a0 = smem_u32(smem + (size_t)s * stage_bytes), b0 = a0 + a_bytes;
            // K = 16 pixels per MMA: two 8-pixel core-matrix groups, 256 bytes on
            for (int k = 0; k < TILE_M / 16; k++)
                mma_bf16(tmem, smem_desc(a0 + k * 256, lbo, sbo), smem_desc(b0 + k * 256, lbo, sbo), idesc, it > 0 || k > 0);
            mma_commit(&empty[s]);
        }
        mma_commit(done);
    }
    __syncwarp();

    const bool ok = mbar_wait(done, 0, p.status);
    tc_fence_after();
    const int co = warp * 32 + lane;
    if (ok)
        for (int c0 = 0; c0 < p.cin; c0 += 16)
        {
            uint32_t r[16];
            tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, r);
            tmem_ld_wait();
            if (co >= p.cout)
                continue;
            float4 *dst = reinterpret_cast<float4 *>(p.partial + (((size_t)split * p.cout + co) * TAPS + tap) * p.cin + c0);
#pragma unroll
            for (int i = 0; i < 4; i++)
                dst[i] = iters > 0 ? make_float4(__uint_as_float(r[4 * i]), __uint_as_float(r[4 * i + 1]), __uint_as_float(r[4 * i + 2]),
                                                 __uint_as_float(r[4 * i + 3]))
                                   : make_float4(0.f, 0.f, 0.f, 0.f);
        }
    tc_fence_before();
    __syncthreads();
    if (warp == 0)
        tmem_dealloc(tmem, ncols);
}

// dW (+)= sum over splits of the partials, in split order.
__global__ void wgrad_reduce_kernel(const float *partial, int splits, size_t n, float *dw, int accumulate)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    float s = accumulate ? dw[i] : 0.0f;
    for (int k = 0; k < splits; k++)
        s += partial[(size_t)k * n + i];
    dw[i] = s;
}

// Packs f32 weights [cout][taps][cin] into the bf16 operand image of conv_kernel:
// per stage (tap, chunk of ck input channels) a K-major block [ck/8][cout/8][8 rows = out
// channel][8 = in channel].  transpose != 0 packs the data-gradient convolution instead:
// its inputs are the forward's outputs and its taps mirrored (dX = conv(dY, W^T flipped)).
__global__ void pack_kernel(const float *w, int taps, int cin, int cout, int transpose, __nv_bfloat16 *wpack)
{
    const int n = taps * cin * cout;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const int co = i / (taps * cin), tap = (i / cin) % taps, ci = i % cin;
    // the packed convolution's (input channel, tap, output channel)
    const int pin = transpose ? co : ci, pout = transpose ? ci : co, ptap = transpose ? taps - 1 - tap : tap;
    const int pcin = transpose ? cout : cin, pcout = transpose ? cin : cout;
    const int ck = pcin % 32 == 0 ? 32 : 16;
    const int stage = ptap * (pcin / ck) + pin / ck;
    const int kin = pin % ck;
    const size_t off = (size_t)stage * ck * pcout + (((size_t)(kin / 8) * (pcout / 8) + pout / 8) * 8 + pout % 8) * 8 + kin % 8;
    wpack[off] = __float2bfloat16_rn(w[i]);
}
} // namespace isti_unet
