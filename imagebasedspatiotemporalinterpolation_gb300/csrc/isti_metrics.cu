// PSNR and SSIM of RGBA8 image pairs (include/isti_metrics.h): the metrics of
// the reference's evaluation script (scripts/eval.py:66-132,
// scripts/loss_utils.py:17-57), as two kernels.
//
// quality_tile_kernel: one block per 32x16 output tile.  For each colour
// channel the tile plus a 5-pixel halo of both images is staged in shared
// memory as floats in [0, 1] (zero outside the image: the reference's zero
// padding), the five moments x, y, x^2, y^2, xy are filtered horizontally
// into shared memory and then vertically per output pixel, and the SSIM
// value is accumulated; the squared error is accumulated exactly in
// integers.  Each block writes its two partial sums.
// quality_final_kernel: one block adds the partial sums in a fixed order.
#include "isti_metrics.h"
#include "host/isti_error.hpp"

#include <cuda_runtime.h>

#include <cmath>
#include <string>

namespace
{
constexpr int TW = 32, TH = 16, R = 5, WIN = 2 * R + 1;
constexpr int SW = TW + 2 * R, SH = TH + 2 * R;
constexpr int THREADS = 256; // 32 x 8: each thread owns one column and two rows of the tile

struct Gauss
{
    float g[WIN];
};

__global__ void __launch_bounds__(THREADS) quality_tile_kernel(const uint32_t *__restrict__ a, const uint32_t *__restrict__ b,
                                                               int w, int h, double *__restrict__ partials, const Gauss gw)
{
    __shared__ float xs[SH][SW], ys[SH][SW];
    __shared__ float hm[5][SH][TW]; // horizontally filtered x, y, x^2, y^2, xy
    const int tid = threadIdx.y * 32 + threadIdx.x;
    const int x0 = blockIdx.x * TW, y0 = blockIdx.y * TH;
    double ssim_sum = 0.0;
    unsigned long long sq_sum = 0;

    for (int c = 0; c < 3; c++)
    {
        const int shift = 8 * c;
        for (int i = tid; i < SH * SW; i += THREADS)
        {
            const int yy = i / SW, xx = i % SW;
            const int gx = x0 + xx - R, gy = y0 + yy - R;
            float va = 0.0f, vb = 0.0f;
            if (gx >= 0 && gx < w && gy >= 0 && gy < h)
            {
                const size_t idx = (size_t)gy * w + gx;
                va = __fdiv_rn((float)((__ldg(a + idx) >> shift) & 255u), 255.0f);
                vb = __fdiv_rn((float)((__ldg(b + idx) >> shift) & 255u), 255.0f);
            }
            xs[yy][xx] = va;
            ys[yy][xx] = vb;
        }
        __syncthreads();
        for (int i = tid; i < SH * TW; i += THREADS)
        {
            const int row = i / TW, col = i % TW;
            float s1 = 0.f, s2 = 0.f, s11 = 0.f, s22 = 0.f, s12 = 0.f;
#pragma unroll
            for (int k = 0; k < WIN; k++)
            {
                const float g = gw.g[k], x = xs[row][col + k], y = ys[row][col + k];
                s1 = fmaf(g, x, s1);
                s2 = fmaf(g, y, s2);
                s11 = fmaf(g, x * x, s11);
                s22 = fmaf(g, y * y, s22);
                s12 = fmaf(g, x * y, s12);
            }
            hm[0][row][col] = s1;
            hm[1][row][col] = s2;
            hm[2][row][col] = s11;
            hm[3][row][col] = s22;
            hm[4][row][col] = s12;
        }
        __syncthreads();
        const int tx = threadIdx.x;
#pragma unroll
        for (int r = 0; r < 2; r++)
        {
            const int oy = threadIdx.y * 2 + r;
            const int gx = x0 + tx, gy = y0 + oy;
            if (gx >= w || gy >= h)
                continue;
            float m1 = 0.f, m2 = 0.f, e11 = 0.f, e22 = 0.f, e12 = 0.f;
#pragma unroll
            for (int k = 0; k < WIN; k++)
            {
                const float g = gw.g[k];
                m1 = fmaf(g, hm[0][oy + k][tx], m1);
                m2 = fmaf(g, hm[1][oy + k][tx], m2);
                e11 = fmaf(g, hm[2][oy + k][tx], e11);
                e22 = fmaf(g, hm[3][oy + k][tx], e22);
                e12 = fmaf(g, hm[4][oy + k][tx], e12);
            }
            constexpr float C1 = 0.01f * 0.01f, C2 = 0.03f * 0.03f;
            const float m1s = m1 * m1, m2s = m2 * m2, m12 = m1 * m2;
            const float v1 = e11 - m1s, v2 = e22 - m2s, v12 = e12 - m12;
            const float num = (2.0f * m12 + C1) * (2.0f * v12 + C2);
            const float den = (m1s + m2s + C1) * (v1 + v2 + C2);
            ssim_sum += (double)__fdiv_rn(num, den);
            const size_t idx = (size_t)gy * w + gx;
            const int d = (int)((__ldg(a + idx) >> shift) & 255u) - (int)((__ldg(b + idx) >> shift) & 255u);
            sq_sum += (unsigned long long)(d * d);
        }
        __syncthreads();
    }

    // block reduction (warp shuffles, then one value per warp)
    for (int o = 16; o > 0; o >>= 1)
    {
        ssim_sum += __shfl_down_sync(0xffffffffu, ssim_sum, o);
        sq_sum += __shfl_down_sync(0xffffffffu, sq_sum, o);
    }
    __shared__ double ws[THREADS / 32];
    __shared__ unsigned long long wq[THREADS / 32];
    if ((tid & 31) == 0)
    {
        ws[tid >> 5] = ssim_sum;
        wq[tid >> 5] = sq_sum;
    }
    __syncthreads();
    if (tid == 0)
    {
        double s = 0.0;
        unsigned long long q = 0;
        for (int k = 0; k < THREADS / 32; k++)
        {
            s += ws[k];
            q += wq[k];
        }
        const size_t blk = (size_t)blockIdx.y * gridDim.x + blockIdx.x;
        partials[2 * blk] = s;
        partials[2 * blk + 1] = (double)q; // exact: at most 3 * 512 * 65025 per block
    }
}

__global__ void __launch_bounds__(THREADS) quality_final_kernel(const double *__restrict__ partials, size_t n_blocks,
                                                                double n_values, isti_quality *out)
{
    __shared__ double ss[THREADS], sq[THREADS];
    double s = 0.0, q = 0.0;
    for (size_t i = threadIdx.x; i < n_blocks; i += THREADS) // fixed assignment and order: deterministic
    {
        s += partials[2 * i];
        q += partials[2 * i + 1];
    }
    ss[threadIdx.x] = s;
    sq[threadIdx.x] = q;
    __syncthreads();
    for (int o = THREADS / 2; o > 0; o >>= 1)
    {
        if ((int)threadIdx.x < o)
        {
            ss[threadIdx.x] += ss[threadIdx.x + o];
            sq[threadIdx.x] += sq[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0)
    {
        const double mse = sq[0] / (n_values * 65025.0);
        out->mse = mse;
        out->psnr = mse > 0.0 ? -10.0 * log10(mse) : INFINITY;
        out->ssim = ss[0] / n_values;
    }
}

Gauss make_gauss()
{
    // loss_utils.gaussian(11, 1.5): float32 of exp(-(x - 5)^2 / (2 sigma^2)), divided by its float32 sum
    Gauss g;
    float sum = 0.0f;
    for (int k = 0; k < WIN; k++)
    {
        g.g[k] = (float)std::exp(-double((k - R) * (k - R)) / (2.0 * 1.5 * 1.5));
        sum += g.g[k];
    }
    for (float &v : g.g)
        v = v / sum;
    return g;
}

size_t n_tiles(int32_t w, int32_t h) { return (size_t)((w + TW - 1) / TW) * (size_t)((h + TH - 1) / TH); }
} // namespace

extern "C" {

size_t isti_quality_scratch_bytes(int32_t width, int32_t height)
{
    if (width <= 0 || height <= 0)
        return 0;
    return n_tiles(width, height) * 2 * sizeof(double);
}

isti_status isti_quality_rgba8(const void *a, const void *b, int32_t width, int32_t height, void *scratch,
                               isti_quality *out, void *stream)
{
    if (!a || !b || !scratch || !out || width <= 0 || height <= 0 || width > 65535 || height > 65535)
        return isti::set_error(ISTI_ERR_INVALID_ARG, "isti_quality_rgba8: bad argument");
    if (((uintptr_t)a | (uintptr_t)b) & 3u)
        return isti::set_error(ISTI_ERR_INVALID_ARG, "isti_quality_rgba8: images must be 4-byte aligned");
    if (((uintptr_t)scratch | (uintptr_t)out) & 7u)
        return isti::set_error(ISTI_ERR_INVALID_ARG, "isti_quality_rgba8: scratch and out must be 8-byte aligned");
    static const Gauss gw = make_gauss();
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const dim3 grid((width + TW - 1) / TW, (height + TH - 1) / TH);
    quality_tile_kernel<<<grid, dim3(32, 8), 0, s>>>(static_cast<const uint32_t *>(a), static_cast<const uint32_t *>(b),
                                                    width, height, static_cast<double *>(scratch), gw);
    quality_final_kernel<<<1, THREADS, 0, s>>>(static_cast<const double *>(scratch), n_tiles(width, height),
                                               3.0 * (double)width * (double)height, out);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return isti::set_error(ISTI_ERR_CUDA, std::string("isti_quality_rgba8: ") + cudaGetErrorString(e));
    return ISTI_OK;
}

} // extern "C"
