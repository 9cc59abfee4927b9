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
#include <cuda_fp16.h>
#include <stdint.h>

namespace isti_unet
{
using namespace isti_tc;

constexpr int CONV_THREADS = 128; // weight-gradient kernel: warp 0 producer, warp 1 MMA, all four epilogue
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
    int tiles_x, tiles_y, n_tiles;
    int relu;
    int stages;                 // depth of the shared-memory ring
    int chunked_map;            // 1: one 5-D box per stage (channel chunks outermost); 0: ck / 8 4-D boxes
    // 1x1 output head fused into the epilogue (row_conv_kernel, inference): when head_w is
    // set, each pixel's bf16 outputs feed HEAD outputs = head_b + head_w . out (f32, fused
    // multiply-adds in channel order) written to head_flow (f32) and/or head_flow16 (f16),
    // and `out` is not written
    const float *head_w;        // [HEAD][cout]
    const float *head_b;        // [HEAD]
    float *head_flow;           // [pixel][HEAD], or null
    __half *head_flow16;        // [pixel][HEAD], or null
};

constexpr int CONV_HEAD = 4; // outputs of a fused head

__host__ __device__ constexpr uint32_t conv_stage_bytes(int ck, int cout) { return (uint32_t)ck * 256u + (uint32_t)ck * cout * 2u; }

// bf16 > 0 (positive, non-zero, not NaN)
__device__ __forceinline__ bool bf16_positive(uint16_t b) { return (b & 0x8000u) == 0 && (b & 0x7fffu) != 0 && (b & 0x7fffu) <= 0x7f80u; }

// 5-D tiled TMA load (c_lo, x, y, c_hi, n): the channel chunks of a box land one after another
__device__ __forceinline__ void tma_load_5d(void *dst, const CUtensorMap *map, int c0, int c1, int c2, int c3, int c4, uint64_t *bar)
{
    asm volatile("cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(
                     smem_u32(dst)),
                 "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(smem_u32(bar))
                 : "memory");
}

constexpr int PCONV_THREADS = 192; // warp 0: TMA producer, warp 1: MMA issuer, warps 2-5: epilogue

// Persistent convolution: each CTA works through tiles blockIdx.x, blockIdx.x + gridDim.x, ...
// The producer runs ahead through the ring across tiles; the MMA issuer accumulates tile i into
// TMEM buffer i % 2 while the epilogue warps drain buffer (i - 1) % 2 (acc_full / acc_empty
// barriers), so stores overlap the next tile's loads and MMAs.
template <int TAPS>
__global__ void __launch_bounds__(PCONV_THREADS, 1) conv_kernel(const __grid_constant__ ConvParams p, const __grid_constant__ CUtensorMap xmap)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    const int S = p.stages;
    const uint32_t a_bytes = (uint32_t)p.ck * 256u, b_bytes = (uint32_t)p.ck * p.cout * 2u, stage_bytes = a_bytes + b_bytes;
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + (size_t)S * stage_bytes);
    uint64_t *empty = full + S;
    uint64_t *acc_full = empty + S;
    uint64_t *acc_empty = acc_full + 2;
    uint64_t *mma_done = acc_empty + 2;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(mma_done + 1);
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const uint32_t acc_cols = tmem_cols(p.cout), ncols = 2 * acc_cols;

    if (threadIdx.x == 0)
    {
        for (int s = 0; s < S; s++)
        {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; b++)
        {
            mbar_init(&acc_full[b], 1);
            mbar_init(&acc_empty[b], 4); // one arrival per epilogue warp
        }
        mbar_init(mma_done, 1);
        fence_barrier_init();
    }
    if (warp == 0)
        tmem_alloc(tmem_slot, ncols);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const int chunks = p.cin / p.ck, iters = TAPS * chunks;
    if (threadIdx.x == 0)
        griddep_launch_dependents(); // the next layer may set up while this one runs

    if (warp == 0 && lane == 0)
    {
        griddep_wait(); // the previous layer's output is complete (every load below is later)
        fence_proxy_async_global();
        uint32_t g = 0;
        bool stop = false;
        for (int t = blockIdx.x; t < p.n_tiles && !stop; t += gridDim.x)
        {
            int tt = t;
            const int tx = tt % p.tiles_x;
            tt /= p.tiles_x;
            const int ty = tt % p.tiles_y;
            const int bi = tt / p.tiles_y;
            const int x0 = tx * TILE_W, y0 = ty * TILE_H;
            for (int it = 0; it < iters; it++, g++)
            {
                const uint32_t s = g % (uint32_t)S, r = g / (uint32_t)S;
                if (r > 0 && !mbar_wait(&empty[s], (r - 1) & 1u, p.status))
                {
                    stop = true;
                    break;
                }
                uint8_t *st = smem + (size_t)s * stage_bytes;
                mbar_expect_tx(&full[s], stage_bytes);
                const int tap = it / chunks, c = it % chunks;
                const int dy = TAPS == 9 ? tap / 3 - 1 : 0, dx = TAPS == 9 ? tap % 3 - 1 : 0;
                if (p.chunked_map)
                    tma_load_5d(st, &xmap, 0, x0 + dx, y0 + dy, c * (p.ck / 8), bi, &full[s]);
                else
                    for (int j = 0; j < p.ck / 8; j++)
                        tma_load_4d(st + j * BOX_BYTES, &xmap, c * p.ck + 8 * j, x0 + dx, y0 + dy, bi, &full[s]);
                bulk_load(st + a_bytes, p.wpack + (size_t)it * p.ck * p.cout, b_bytes, &full[s]);
            }
        }
        for (uint32_t q = g > (uint32_t)S ? g - (uint32_t)S : 0u; q < g; q++) // copies still landing
            if (!mbar_wait(&full[q % (uint32_t)S], (q / (uint32_t)S) & 1u, p.status))
                break;
    }
    else if (warp == 1 && lane == 0)
    {
        const uint32_t idesc = idesc_bf16(TILE_M, (uint32_t)p.cout, 0, 0);
        const uint32_t lbo_b = (uint32_t)(p.cout / 8) * 128u;
        uint32_t g = 0;
        int i = 0;
        bool stop = false;
        for (int t = blockIdx.x; t < p.n_tiles && !stop; t += gridDim.x, i++)
        {
            const int buf = i & 1;
            if (i >= 2 && !mbar_wait(&acc_empty[buf], (uint32_t)(((i >> 1) - 1) & 1), p.status))
                break;
            tc_fence_after();
            const uint32_t d = tmem + (uint32_t)buf * acc_cols;
            for (int it = 0; it < iters; it++, g++)
            {
                const uint32_t s = g % (uint32_t)S, r = g / (uint32_t)S;
                if (!mbar_wait(&full[s], r & 1u, p.status))
                {
                    stop = true;
                    break;
                }
                tc_fence_after();
                const uint32_t a0 = smem_u32(smem + (size_t)s * stage_bytes), b0 = a0 + a_bytes;
                for (int k = 0; k < p.ck / 16; k++)
                    mma_bf16(d, smem_desc(a0 + k * 2 * BOX_BYTES, BOX_BYTES, 128), smem_desc(b0 + k * 2 * lbo_b, lbo_b, 128), idesc,
                             it > 0 || k > 0);
                mma_commit(&empty[s]);
            }
            if (!stop)
                mma_commit(&acc_full[buf]);
        }
        mma_commit(mma_done);
    }
    else if (warp >= 2)
    {
        const int q = warp % 4; // the TMEM lane quadrant this warp may read
        const int m = q * 32 + lane;
        int i = 0;
        for (int t = blockIdx.x; t < p.n_tiles; t += gridDim.x, i++)
        {
            const int buf = i & 1;
            if (!mbar_wait(&acc_full[buf], (uint32_t)((i >> 1) & 1), p.status))
                break;
            tc_fence_after();
            int tt = t;
            const int tx = tt % p.tiles_x;
            tt /= p.tiles_x;
            const int ty = tt % p.tiles_y;
            const int bi = tt / p.tiles_y;
            const int px = tx * TILE_W + (m % TILE_W), py = ty * TILE_H + (m / TILE_W);
            const bool inb = px < p.w && py < p.h;
            const size_t pix = ((size_t)bi * p.h + (inb ? py : 0)) * p.w + (inb ? px : 0);
            for (int c0 = 0; c0 < p.cout; c0 += 16)
            {
                uint32_t r[16];
                tmem_ld16(tmem + (uint32_t)buf * acc_cols + ((uint32_t)(q * 32) << 16) + (uint32_t)c0, r);
                tmem_ld_wait();
                if (!inb)
                    continue;
                float v[16];
#pragma unroll
                for (int j = 0; j < 16; j++)
                {
                    v[j] = __uint_as_float(r[j]);
                    if (p.bias)
                        v[j] += __ldg(p.bias + c0 + j);
                    if (p.relu)
                        v[j] = fmaxf(v[j], 0.0f);
                }
                if (p.mask)
                {
                    const uint4 *mk = reinterpret_cast<const uint4 *>(p.mask + pix * p.cout + c0);
                    const uint4 m0 = __ldg(mk), m1 = __ldg(mk + 1);
                    const uint32_t mw[8] = {m0.x, m0.y, m0.z, m0.w, m1.x, m1.y, m1.z, m1.w};
#pragma unroll
                    for (int j = 0; j < 16; j++)
                        if (!bf16_positive((uint16_t)(mw[j / 2] >> (16 * (j % 2)))))
                            v[j] = 0.0f;
                }
                uint32_t o[8];
#pragma unroll
                for (int j = 0; j < 8; j++)
                {
                    const __nv_bfloat162 h2 = __floats2bfloat162_rn(v[2 * j], v[2 * j + 1]);
                    o[j] = *reinterpret_cast<const uint32_t *>(&h2);
                }
                uint4 *dst = reinterpret_cast<uint4 *>(p.out + pix * p.cout + c0);
                dst[0] = make_uint4(o[0], o[1], o[2], o[3]);
                dst[1] = make_uint4(o[4], o[5], o[6], o[7]);
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0)
                mbar_arrive(&acc_empty[buf]);
        }
    }
    __syncwarp();
    if (warp == 0)
    {
        if (lane == 0)
            mbar_wait(mma_done, 0, p.status); // no MMA may still write TMEM when it is freed
        __syncwarp();
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0)
    {
        tc_fence_after();
        tmem_dealloc(tmem, ncols);
    }
}

// ---- row-tile 3x3 convolution for the wide, thin layers ----
//
// A unit is 128 consecutive output pixels of one row (M = 128).  Per chunk of ck input
// channels one TMA copy (5-D map, box {8, 130 x, 3 y, ck / 8 chunks, 1}) lands the unit's
// halo -- 3 input rows of 130 pixels, chunk-major -- and the 9 taps are 9 descriptor start
// offsets into it ((dy + 1) rows and (dx + 1) pixels on, 16 bytes per pixel and chunk), so
// every input pixel is fetched for 3 units instead of 9 taps.  The weights of all taps and
// chunks stay in shared memory for the CTA's lifetime (one bulk copy).  Roles and the
// double-buffered TMEM accumulators are those of conv_kernel.
constexpr int ROW_M = 128, ROW_HALO = ROW_M + 2;
__host__ __device__ constexpr uint32_t row_chunk_bytes() { return 3u * ROW_HALO * 16u; }          // one 8-channel chunk
__host__ __device__ constexpr uint32_t row_stage_bytes(int ck) { return ((uint32_t)(ck / 8) * row_chunk_bytes() + 1023u) / 1024u * 1024u; }

template <int UNUSED = 0>
__global__ void __launch_bounds__(PCONV_THREADS, 1) row_conv_kernel(const __grid_constant__ ConvParams p, const __grid_constant__ CUtensorMap xmap)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    const int S = p.stages;
    const int chunks = p.cin / p.ck;
    const uint32_t w_bytes = 9u * (uint32_t)p.cin * p.cout * 2u; // every tap and chunk, packed
    const uint32_t w_region = (w_bytes + 1023u) / 1024u * 1024u;
    const uint32_t a_bytes = (uint32_t)(p.ck / 8) * row_chunk_bytes(), stage_bytes = row_stage_bytes(p.ck);
    uint8_t *wsm = smem;
    uint8_t *ring = smem + w_region;
    uint64_t *full = reinterpret_cast<uint64_t *>(ring + (size_t)S * stage_bytes);
    uint64_t *empty = full + S;
    uint64_t *acc_full = empty + S;
    uint64_t *acc_empty = acc_full + 2;
    uint64_t *mma_done = acc_empty + 2;
    uint64_t *wbar = mma_done + 1;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(wbar + 1);
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const uint32_t acc_cols = tmem_cols(p.cout), ncols = 2 * acc_cols;
    const int segs = (p.w + ROW_M - 1) / ROW_M;
    const int n_units = p.b * p.h * segs;

    if (threadIdx.x == 0)
    {
        for (int s = 0; s < S; s++)
        {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; b++)
        {
            mbar_init(&acc_full[b], 1);
            mbar_init(&acc_empty[b], 4);
        }
        mbar_init(mma_done, 1);
        mbar_init(wbar, 1);
        fence_barrier_init();
    }
    if (warp == 0)
        tmem_alloc(tmem_slot, ncols);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (threadIdx.x == 0)
        griddep_launch_dependents(); // the next layer may set up while this one runs
    if (warp == 0 && lane == 0)
    {
        mbar_expect_tx(wbar, w_bytes);
        for (uint32_t o = 0; o < w_bytes; o += 32768u) // pieces of at most 32 KiB (weights: no previous kernel writes them)
            bulk_load(wsm + o, reinterpret_cast<const uint8_t *>(p.wpack) + o, min(32768u, w_bytes - o), wbar);
        griddep_wait(); // the previous layer's output is complete (every activation load below is later)
        fence_proxy_async_global();
        uint32_t g = 0;
        bool stop = false;
        for (int u = blockIdx.x; u < n_units && !stop; u += gridDim.x)
        {
            const int seg = u % segs, row = (u / segs) % p.h, bi = u / (segs * p.h);
            for (int c = 0; c < chunks; c++, g++)
            {
                const uint32_t s = g % (uint32_t)S, r = g / (uint32_t)S;
                if (r > 0 && !mbar_wait(&empty[s], (r - 1) & 1u, p.status))
                {
                    stop = true;
                    break;
                }
                mbar_expect_tx(&full[s], a_bytes);
                tma_load_5d(ring + (size_t)s * stage_bytes, &xmap, 0, seg * ROW_M - 1, row - 1, c * (p.ck / 8), bi, &full[s]);
            }
        }
        for (uint32_t q = g > (uint32_t)S ? g - (uint32_t)S : 0u; q < g; q++)
            if (!mbar_wait(&full[q % (uint32_t)S], (q / (uint32_t)S) & 1u, p.status))
                break;
        mbar_wait(wbar, 0, p.status);
    }
    else if (warp == 1 && lane == 0)
    {
        const uint32_t idesc = idesc_bf16(ROW_M, (uint32_t)p.cout, 0, 0);
        const uint32_t lbo_b = (uint32_t)(p.cout / 8) * 128u;
        const uint32_t wbase = smem_u32(wsm);
        uint32_t g = 0;
        int i = 0;
        bool stop = !mbar_wait(wbar, 0, p.status);
        for (int u = blockIdx.x; u < n_units && !stop; u += gridDim.x, i++)
        {
            const int buf = i & 1;
            if (i >= 2 && !mbar_wait(&acc_empty[buf], (uint32_t)(((i >> 1) - 1) & 1), p.status))
                break;
            tc_fence_after();
            const uint32_t d = tmem + (uint32_t)buf * acc_cols;
            for (int c = 0; c < chunks; c++, g++)
            {
                const uint32_t s = g % (uint32_t)S, r = g / (uint32_t)S;
                if (!mbar_wait(&full[s], r & 1u, p.status))
                {
                    stop = true;
                    break;
                }
                tc_fence_after();
                const uint32_t a0 = smem_u32(ring + (size_t)s * stage_bytes);
                for (int tap = 0; tap < 9; tap++)
                {
                    const uint32_t shift = (uint32_t)((tap / 3) * ROW_HALO + (tap % 3)) * 16u;
                    const uint32_t b0 = wbase + (uint32_t)(tap * chunks + c) * (uint32_t)p.ck * p.cout * 2u;
                    for (int k = 0; k < p.ck / 16; k++)
                        mma_bf16(d, smem_desc(a0 + (uint32_t)(2 * k) * row_chunk_bytes() + shift, row_chunk_bytes(), 128),
                                 smem_desc(b0 + k * 2 * lbo_b, lbo_b, 128), idesc, c > 0 || tap > 0 || k > 0);
                }
                mma_commit(&empty[s]);
            }
            if (!stop)
                mma_commit(&acc_full[buf]);
        }
        mma_commit(mma_done);
    }
    else if (warp >= 2)
    {
        const int q = warp % 4;
        const int m = q * 32 + lane;
        int i = 0;
        for (int u = blockIdx.x; u < n_units; u += gridDim.x, i++)
        {
            const int buf = i & 1;
            if (!mbar_wait(&acc_full[buf], (uint32_t)((i >> 1) & 1), p.status))
                break;
            tc_fence_after();
            const int seg = u % segs, row = (u / segs) % p.h, bi = u / (segs * p.h);
            const int px = seg * ROW_M + m;
            const bool inb = px < p.w;
            const size_t pix = ((size_t)bi * p.h + row) * p.w + (inb ? px : 0);
            float hacc[CONV_HEAD];
            if (p.head_w)
#pragma unroll
                for (int q = 0; q < CONV_HEAD; q++)
                    hacc[q] = __ldg(p.head_b + q);
            for (int c0 = 0; c0 < p.cout; c0 += 16)
            {
                uint32_t r[16];
                tmem_ld16(tmem + (uint32_t)buf * acc_cols + ((uint32_t)(q * 32) << 16) + (uint32_t)c0, r);
                tmem_ld_wait();
                if (!inb)
                    continue;
                float v[16];
#pragma unroll
                for (int j = 0; j < 16; j++)
                {
                    v[j] = __uint_as_float(r[j]);
                    if (p.bias)
                        v[j] += __ldg(p.bias + c0 + j);
                    if (p.relu)
                        v[j] = fmaxf(v[j], 0.0f);
                }
                if (p.mask)
                {
                    const uint4 *mk = reinterpret_cast<const uint4 *>(p.mask + pix * p.cout + c0);
                    const uint4 m0 = __ldg(mk), m1 = __ldg(mk + 1);
                    const uint32_t mw[8] = {m0.x, m0.y, m0.z, m0.w, m1.x, m1.y, m1.z, m1.w};
#pragma unroll
                    for (int j = 0; j < 16; j++)
                        if (!bf16_positive((uint16_t)(mw[j / 2] >> (16 * (j % 2)))))
                            v[j] = 0.0f;
                }
                uint32_t o[8];
#pragma unroll
                for (int j = 0; j < 8; j++)
                {
                    const __nv_bfloat162 h2 = __floats2bfloat162_rn(v[2 * j], v[2 * j + 1]);
                    o[j] = *reinterpret_cast<const uint32_t *>(&h2);
                }
                if (p.head_w)
                {
#pragma unroll
                    for (int j = 0; j < 8; j++)
                    {
                        const float2 f = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(&o[j]));
#pragma unroll
                        for (int q = 0; q < CONV_HEAD; q++)
                        {
                            hacc[q] = fmaf(__ldg(p.head_w + q * p.cout + c0 + 2 * j), f.x, hacc[q]);
                            hacc[q] = fmaf(__ldg(p.head_w + q * p.cout + c0 + 2 * j + 1), f.y, hacc[q]);
                        }
                    }
                    continue;
                }
                uint4 *dst = reinterpret_cast<uint4 *>(p.out + pix * p.cout + c0);
                dst[0] = make_uint4(o[0], o[1], o[2], o[3]);
                dst[1] = make_uint4(o[4], o[5], o[6], o[7]);
            }
            if (p.head_w && inb)
            {
                if (p.head_flow)
                    *reinterpret_cast<float4 *>(p.head_flow + pix * CONV_HEAD) = make_float4(hacc[0], hacc[1], hacc[2], hacc[3]);
                if (p.head_flow16)
                {
                    const __half2 h0 = __floats2half2_rn(hacc[0], hacc[1]), h1 = __floats2half2_rn(hacc[2], hacc[3]);
                    *reinterpret_cast<uint2 *>(p.head_flow16 + pix * CONV_HEAD) =
                        make_uint2(*reinterpret_cast<const uint32_t *>(&h0), *reinterpret_cast<const uint32_t *>(&h1));
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0)
                mbar_arrive(&acc_empty[buf]);
        }
    }
    __syncwarp();
    if (warp == 0)
    {
        if (lane == 0)
            mbar_wait(mma_done, 0, p.status);
        __syncwarp();
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0)
    {
        tc_fence_after();
        tmem_dealloc(tmem, ncols);
    }
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
