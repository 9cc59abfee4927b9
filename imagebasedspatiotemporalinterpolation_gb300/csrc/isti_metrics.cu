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

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

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

// ---------------------------------------------------------------- LDR-FLIP
//
// scripts/flip_loss.py (the published LDR-FLIP, Andersson et al. 2020).  Every 2-D
// kernel of the reference is a sum of products f(x) g(y): the contrast-sensitivity
// filters are (sums of) normalised Gaussians, the edge / point detectors a derivative
// of a Gaussian in x times a Gaussian in y, normalised per sign of the x factor.  So
// each is applied as a horizontal then a vertical 1-D pass, all taps padded to a
// common radius R (the reference pads every filter by the largest radius, replicating
// the border).

constexpr int FR_MAX = ISTI_FLIP_MAX_RADIUS;
constexpr int FTAPS = 2 * FR_MAX + 1;
constexpr int FTW = 32, FTH = 16;

struct FlipFilters
{
    int r;                     // common radius of every 1-D filter
    float csf_a[FTAPS];        // achromatic CSF, 1-D factor
    float csf_rg[FTAPS];       // red-green CSF
    float csf_by1[FTAPS];      // blue-yellow CSF = by1(x) by1(y) + by2(x) by2(y)
    float csf_by2[FTAPS];
    float gauss[FTAPS];        // feature detectors: normalised Gaussian factor
    float edge[FTAPS];         // d/dx factor of the edge detector
    float point[FTAPS];        // d2/dx2 factor of the point detector
    float cmax;                // maximum HyAB^qc (green vs blue), redistribute_errors
};

constexpr float FLIP_QC = 0.7f, FLIP_QF = 0.5f, FLIP_PC = 0.4f, FLIP_PT = 0.95f, FLIP_EPS = 1e-15f;

// linear RGB -> XYZ (D65), the reference's rational constants rounded to float
__constant__ float L2X[3][3] = {{(float)(10135552.0 / 24577794.0), (float)(8788810.0 / 24577794.0), (float)(4435075.0 / 24577794.0)},
                             {(float)(2613072.0 / 12288897.0), (float)(8788810.0 / 12288897.0), (float)(887015.0 / 12288897.0)},
                             {(float)(1425312.0 / 73733382.0), (float)(8788810.0 / 73733382.0), (float)(70074185.0 / 73733382.0)}};

__device__ __forceinline__ float3 lin_to_xyz_scaled(float r, float g, float b)
{
    // XYZ divided by the D65 white (the reference's inv_reference_illuminant)
    return make_float3((L2X[0][0] * r + L2X[0][1] * g + L2X[0][2] * b) * 1.052156925f, L2X[1][0] * r + L2X[1][1] * g + L2X[1][2] * b,
                       (L2X[2][0] * r + L2X[2][1] * g + L2X[2][2] * b) * 0.918357670f);
}

// sRGB byte -> YCxCz (color_space_transform 'srgb2ycxcz'): Y, Cx, Cz
__device__ __forceinline__ float3 srgb8_to_ycxcz(uint32_t p)
{
    float c[3];
#pragma unroll
    for (int k = 0; k < 3; k++)
    {
        const float v = (float)((p >> (8 * k)) & 255u) / 255.0f;
        c[k] = v > 0.04045f ? powf((fmaxf(v, 0.04045f) + 0.055f) / 1.055f, 2.4f) : v / 12.92f;
    }
    const float3 xyz = lin_to_xyz_scaled(c[0], c[1], c[2]);
    return make_float3(116.0f * xyz.y - 16.0f, 500.0f * (xyz.x - xyz.y), 200.0f * (xyz.y - xyz.z));
}

// filtered YCxCz -> linear RGB clamped to the unit cube -> L*a*b* -> Hunt-adjusted
__device__ __forceinline__ float3 ycxcz_to_hunt_lab(float Y, float Cx, float Cz)
{
    const float yy = (Y + 16.0f) / 116.0f;
    const float X = (yy + Cx / 500.0f) * 0.950428545f, Yv = yy, Z = (yy - Cz / 200.0f) * 1.088900371f;
    float rgb[3] = {3.241003275f * X - 1.537398934f * Yv - 0.498615861f * Z, -0.969224334f * X + 1.875930071f * Yv + 0.041554224f * Z,
                    0.055639423f * X - 0.204011202f * Yv + 1.057148933f * Z};
#pragma unroll
    for (int k = 0; k < 3; k++)
        rgb[k] = fminf(fmaxf(rgb[k], 0.0f), 1.0f);
    const float3 s = lin_to_xyz_scaled(rgb[0], rgb[1], rgb[2]);
    float xyz[3] = {s.x, s.y, s.z};
    constexpr float d3 = (6.0f / 29.0f) * (6.0f / 29.0f) * (6.0f / 29.0f);
    constexpr float factor = 1.0f / (3.0f * (6.0f / 29.0f) * (6.0f / 29.0f));
#pragma unroll
    for (int k = 0; k < 3; k++)
        xyz[k] = xyz[k] > d3 ? powf(fmaxf(xyz[k], d3), 1.0f / 3.0f) : factor * xyz[k] + 4.0f / 29.0f;
    const float L = 116.0f * xyz[1] - 16.0f;
    const float a = 500.0f * (xyz[0] - xyz[1]), b = 200.0f * (xyz[1] - xyz[2]);
    return make_float3(L, 0.01f * L * a, 0.01f * L * b);
}

// One block per 32x16 output tile; both images in turn: stage Y, Cx, Cz and the
// normalised Y of the tile plus an R-pixel replicate-padded halo, filter rows
// (7 outputs), then columns per output pixel; then combine per pixel.
__global__ void __launch_bounds__(THREADS) flip_tile_kernel(const uint32_t *__restrict__ test, const uint32_t *__restrict__ ref, int w,
                                                            int h, const __grid_constant__ FlipFilters f, double *__restrict__ partials,
                                                            float *__restrict__ map)
{
    extern __shared__ float fsm[];
    const int R = f.r, SW = FTW + 2 * R, SH = FTH + 2 * R;
    float *pin = fsm;                     // [4][SH][SW]: Y, Cx, Cz, (Y + 16) / 116
    float *hor = fsm + 4 * SH * SW;       // [7][SH][FTW]
    const int tid = threadIdx.y * 32 + threadIdx.x;
    const int x0 = blockIdx.x * FTW, y0 = blockIdx.y * FTH;
    const int tx = threadIdx.x;
    float Lab[2][2][3], en[2][2], pn[2][2]; // [image][row]

#pragma unroll
    for (int im = 0; im < 2; im++)
    {
        const uint32_t *src = im == 0 ? ref : test;
        for (int i = tid; i < SH * SW; i += THREADS)
        {
            const int yy = i / SW, xx = i % SW;
            const int gx = min(max(x0 + xx - R, 0), w - 1), gy = min(max(y0 + yy - R, 0), h - 1);
            const float3 c = srgb8_to_ycxcz(__ldg(src + (size_t)gy * w + gx));
            pin[i] = c.x;
            pin[SH * SW + i] = c.y;
            pin[2 * SH * SW + i] = c.z;
            pin[3 * SH * SW + i] = (c.x + 16.0f) / 116.0f;
        }
        __syncthreads();
        for (int i = tid; i < SH * FTW; i += THREADS)
        {
            const int row = i / FTW, col = i % FTW;
            const float *rY = pin + row * SW + col, *rX = rY + SH * SW, *rZ = rY + 2 * SH * SW, *rN = rY + 3 * SH * SW;
            float a = 0.f, rg = 0.f, by1 = 0.f, by2 = 0.f, g = 0.f, e = 0.f, p = 0.f;
            for (int k = 0; k <= 2 * R; k++)
            {
                const int t = FR_MAX - R + k;
                a = fmaf(f.csf_a[t], rY[k], a);
                rg = fmaf(f.csf_rg[t], rX[k], rg);
                by1 = fmaf(f.csf_by1[t], rZ[k], by1);
                by2 = fmaf(f.csf_by2[t], rZ[k], by2);
                g = fmaf(f.gauss[t], rN[k], g);
                e = fmaf(f.edge[t], rN[k], e);
                p = fmaf(f.point[t], rN[k], p);
            }
            float *o = hor + row * FTW + col;
            o[0] = a;
            o[SH * FTW] = rg;
            o[2 * SH * FTW] = by1;
            o[3 * SH * FTW] = by2;
            o[4 * SH * FTW] = g;
            o[5 * SH * FTW] = e;
            o[6 * SH * FTW] = p;
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < 2; r++)
        {
            const int oy = threadIdx.y * 2 + r;
            const float *c = hor + oy * FTW + tx;
            float a = 0.f, rg = 0.f, by = 0.f, ex = 0.f, ey = 0.f, px = 0.f, py = 0.f;
            for (int k = 0; k <= 2 * R; k++)
            {
                const int t = FR_MAX - R + k;
                const float *ck = c + k * FTW;
                a = fmaf(f.csf_a[t], ck[0], a);
                rg = fmaf(f.csf_rg[t], ck[SH * FTW], rg);
                by = fmaf(f.csf_by1[t], ck[2 * SH * FTW], by);
                by = fmaf(f.csf_by2[t], ck[3 * SH * FTW], by);
                ex = fmaf(f.gauss[t], ck[5 * SH * FTW], ex);
                ey = fmaf(f.edge[t], ck[4 * SH * FTW], ey);
                px = fmaf(f.gauss[t], ck[6 * SH * FTW], px);
                py = fmaf(f.point[t], ck[4 * SH * FTW], py);
            }
            const float3 lab = ycxcz_to_hunt_lab(a, rg, by);
            Lab[im][r][0] = lab.x;
            Lab[im][r][1] = lab.y;
            Lab[im][r][2] = lab.z;
            en[im][r] = sqrtf(ex * ex + ey * ey);
            pn[im][r] = sqrtf(px * px + py * py);
        }
        __syncthreads(); // the staging buffers are reused by the next image
    }

    double sum = 0.0;
    const float pccmax = FLIP_PC * f.cmax;
#pragma unroll
    for (int r = 0; r < 2; r++)
    {
        const int gx = x0 + tx, gy = y0 + threadIdx.y * 2 + r;
        if (gx >= w || gy >= h)
            continue;
        // color pipeline: HyAB(reference, test) of the Hunt-adjusted colours
        const float dL = Lab[0][r][0] - Lab[1][r][0], da = Lab[0][r][1] - Lab[1][r][1], db = Lab[0][r][2] - Lab[1][r][2];
        const float hy = sqrtf(fmaxf(dL * dL, FLIP_EPS)) + sqrtf(da * da + db * db);
        const float power = powf(hy, FLIP_QC);
        const float dec = power < pccmax ? (FLIP_PT / pccmax) * power
                                         : FLIP_PT + ((power - pccmax) / (f.cmax - pccmax)) * (1.0f - FLIP_PT);
        // feature pipeline
        float def = fmaxf(fabsf(en[0][r] - en[1][r]), fabsf(pn[1][r] - pn[0][r]));
        def = fmaxf(def, FLIP_EPS);
        def = powf(0.70710678f * def, FLIP_QF);
        const float v = powf(dec, 1.0f - def);
        sum += (double)v;
        if (map)
            map[(size_t)gy * w + gx] = v;
    }
    for (int o = 16; o > 0; o >>= 1)
        sum += __shfl_down_sync(0xffffffffu, sum, o);
    __shared__ double ws[THREADS / 32];
    if ((tid & 31) == 0)
        ws[tid >> 5] = sum;
    __syncthreads();
    if (tid == 0)
    {
        double s = 0.0;
        for (int k = 0; k < THREADS / 32; k++)
            s += ws[k];
        partials[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = s;
    }
}

__global__ void __launch_bounds__(THREADS) flip_final_kernel(const double *__restrict__ partials, size_t n_blocks, double n_px,
                                                             double *out)
{
    __shared__ double ss[THREADS];
    double s = 0.0;
    for (size_t i = threadIdx.x; i < n_blocks; i += THREADS)
        s += partials[i];
    ss[threadIdx.x] = s;
    __syncthreads();
    for (int o = THREADS / 2; o > 0; o >>= 1)
    {
        if ((int)threadIdx.x < o)
            ss[threadIdx.x] += ss[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        *out = ss[0] / n_px;
}

// The reference's filter definitions (generate_spatial_filter, feature_detection) as
// 1-D factors, in double, centred at FR_MAX.  Returns false when a filter's radius
// exceeds FR_MAX.
bool make_flip_filters(double ppd, FlipFilters &f)
{
    std::memset(&f, 0, sizeof f);
    const double pi = 3.14159265358979323846;
    const int rc = (int)std::ceil(3.0 * std::sqrt(0.04 / (2.0 * pi * pi)) * ppd); // max CSF scale parameter 0.04
    const double sd = 0.5 * 0.082 * ppd;
    const int rf = (int)std::ceil(3.0 * sd);
    if (rc > FR_MAX || rf > FR_MAX || rc < 0 || rf < 0)
        return false;
    f.r = std::max(rc, rf);
    const double dx = 1.0 / ppd;
    auto gauss_1d = [&](double b, std::vector<double> &e) {
        e.assign(FTAPS, 0.0);
        double s = 0.0;
        for (int x = -rc; x <= rc; x++)
            s += (e[FR_MAX + x] = std::exp(-pi * pi * (x * dx) * (x * dx) / b));
        return s;
    };
    std::vector<double> ea, erg, e1, e2;
    const double sa = gauss_1d(0.0047, ea), srg = gauss_1d(0.0053, erg), s1 = gauss_1d(0.04, e1), s2 = gauss_1d(0.025, e2);
    // BY: 34.1 sqrt(pi / 0.04) e1(x) e1(y) + 13.5 sqrt(pi / 0.025) e2(x) e2(y), normalised to sum 1
    const double w1 = 34.1 * std::sqrt(pi / 0.04), w2 = 13.5 * std::sqrt(pi / 0.025);
    const double norm = w1 * s1 * s1 + w2 * s2 * s2;
    for (int t = 0; t < FTAPS; t++)
    {
        f.csf_a[t] = (float)(ea[t] / sa);
        f.csf_rg[t] = (float)(erg[t] / srg);
        f.csf_by1[t] = (float)(e1[t] * std::sqrt(w1 / norm));
        f.csf_by2[t] = (float)(e2[t] * std::sqrt(w2 / norm));
    }
    std::vector<double> g(FTAPS, 0.0), de(FTAPS, 0.0), dp(FTAPS, 0.0);
    double gs = 0.0, pos_e = 0.0, neg_e = 0.0, pos_p = 0.0, neg_p = 0.0;
    for (int x = -rf; x <= rf; x++)
    {
        const double e = std::exp(-(double)(x * x) / (2.0 * sd * sd));
        g[FR_MAX + x] = e;
        gs += e;
        de[FR_MAX + x] = -x * e;
        dp[FR_MAX + x] = ((double)(x * x) / (sd * sd) - 1.0) * e;
        (de[FR_MAX + x] < 0 ? neg_e : pos_e) += std::fabs(de[FR_MAX + x]);
        (dp[FR_MAX + x] < 0 ? neg_p : pos_p) += std::fabs(dp[FR_MAX + x]);
    }
    for (int t = 0; t < FTAPS; t++)
    {
        f.gauss[t] = (float)(g[t] / gs);
        f.edge[t] = (float)(de[t] / (de[t] < 0 ? neg_e : pos_e));
        f.point[t] = (float)(dp[t] / (dp[t] < 0 ? neg_p : pos_p));
    }
    // cmax = HyAB(hunt(lab(green)), hunt(lab(blue)))^qc
    auto hunt_lab = [&](double r, double gg, double b, double out[3]) {
        static const double M[3][3] = {{10135552.0 / 24577794, 8788810.0 / 24577794, 4435075.0 / 24577794},
                                       {2613072.0 / 12288897, 8788810.0 / 12288897, 887015.0 / 12288897},
                                       {1425312.0 / 73733382, 8788810.0 / 73733382, 70074185.0 / 73733382}};
        static const double inv_illum[3] = {1.052156925, 1.0, 0.918357670};
        double v[3];
        for (int k = 0; k < 3; k++)
        {
            const double c = (M[k][0] * r + M[k][1] * gg + M[k][2] * b) * inv_illum[k];
            const double d = 6.0 / 29.0;
            v[k] = c > d * d * d ? std::cbrt(c) : c / (3 * d * d) + 4.0 / 29.0;
        }
        const double L = 116 * v[1] - 16;
        out[0] = L;
        out[1] = 0.01 * L * 500 * (v[0] - v[1]);
        out[2] = 0.01 * L * 200 * (v[1] - v[2]);
    };
    double gl[3], bl[3];
    hunt_lab(0, 1, 0, gl);
    hunt_lab(0, 0, 1, bl);
    const double hy = std::sqrt(std::max((gl[0] - bl[0]) * (gl[0] - bl[0]), 1e-15)) +
                      std::sqrt((gl[1] - bl[1]) * (gl[1] - bl[1]) + (gl[2] - bl[2]) * (gl[2] - bl[2]));
    f.cmax = (float)std::pow(hy, 0.7);
    return true;
}

size_t flip_tiles(int32_t w, int32_t h) { return (size_t)((w + FTW - 1) / FTW) * (size_t)((h + FTH - 1) / FTH); }

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

size_t isti_flip_scratch_bytes(int32_t width, int32_t height)
{
    if (width <= 0 || height <= 0)
        return 0;
    return flip_tiles(width, height) * sizeof(double);
}

isti_status isti_flip_rgba8(const void *test, const void *reference, int32_t width, int32_t height, float pixels_per_degree,
                            void *scratch, double *out_mean, float *out_map, void *stream)
{
    if (!test || !reference || !scratch || !out_mean || width <= 0 || height <= 0 || width > 65535 || height > 65535 ||
        !(pixels_per_degree > 0.0f))
        return isti::set_error(ISTI_ERR_INVALID_ARG, "isti_flip_rgba8: bad argument");
    if (((uintptr_t)test | (uintptr_t)reference | (uintptr_t)out_map) & 3u || ((uintptr_t)scratch | (uintptr_t)out_mean) & 7u)
        return isti::set_error(ISTI_ERR_INVALID_ARG, "isti_flip_rgba8: misaligned pointer");
    FlipFilters f;
    if (!make_flip_filters((double)pixels_per_degree, f))
        return isti::set_error(ISTI_ERR_INVALID_ARG, "isti_flip_rgba8: pixels_per_degree too large for the filter radius limit");
    const int R = f.r;
    const size_t smem = (size_t)(4 * (FTH + 2 * R) * (FTW + 2 * R) + 7 * (FTH + 2 * R) * FTW) * sizeof(float);
    static std::once_flag attr_once;
    static cudaError_t attr_err = cudaSuccess;
    std::call_once(attr_once, [] {
        const size_t max_smem = (size_t)(4 * (FTH + 2 * FR_MAX) * (FTW + 2 * FR_MAX) + 7 * (FTH + 2 * FR_MAX) * FTW) * sizeof(float);
        attr_err = cudaFuncSetAttribute(flip_tile_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem);
    });
    if (attr_err != cudaSuccess)
        return isti::set_error(ISTI_ERR_CUDA, std::string("isti_flip_rgba8: ") + cudaGetErrorString(attr_err));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const dim3 grid((width + FTW - 1) / FTW, (height + FTH - 1) / FTH);
    flip_tile_kernel<<<grid, dim3(32, 8), smem, s>>>(static_cast<const uint32_t *>(test), static_cast<const uint32_t *>(reference), width,
                                                     height, f, static_cast<double *>(scratch), out_map);
    flip_final_kernel<<<1, THREADS, 0, s>>>(static_cast<const double *>(scratch), flip_tiles(width, height),
                                            (double)width * (double)height, out_mean);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return isti::set_error(ISTI_ERR_CUDA, std::string("isti_flip_rgba8: ") + cudaGetErrorString(e));
    return ISTI_OK;
}

} // extern "C"
