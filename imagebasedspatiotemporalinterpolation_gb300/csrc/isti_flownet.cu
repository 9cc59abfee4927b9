// The learned flow initialiser network: layers, forward pass, training backward pass and
// Adam, over the tcgen05 convolution operators (isti_unet.cu) and the CUDA-core kernels
// below (pooling, upsampling skips, gradient masks, the 1x1 output head, loss, bias
// gradients, optimiser).  C ABI: include/isti_unet.h.
//
// Architecture (H, W: the quarter-resolution input size, multiples of 8):
//   x0  [H,W,16]  inputs (isti_flownet_input_channels)
//   e1 = relu(conv3x3 16->32)(x0)          q1 = avgpool2(e1)   [H/2]
//   e2 = relu(conv3x3 32->64)(q1)          q2 = avgpool2(e2)   [H/4]
//   e3 = relu(conv3x3 64->96)(q2)          q3 = avgpool2(e3)   [H/8]
//   e4 = relu(conv3x3 96->128)(q3)
//   s3 = up2(conv1x1 128->96 (e4)) + e3    d3 = relu(conv3x3 96->96)(s3)
//   s2 = up2(conv1x1 96->64 (d3)) + e2     d2 = relu(conv3x3 64->64)(s2)
//   s1 = up2(conv1x1 64->32 (d2)) + e1     d1 = relu(conv3x3 32->32)(s1)
//   flow = conv1x1 32->4 (d1)              [H,W,4] f32
// 10 tensor-core layers + the head: 339,268 parameters.
#include "isti_tc.cuh"
#include "isti_unet.h"
#include "isti_unet_ops.h"
#include "host/isti_error.hpp"

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <vector>

namespace
{
using bf16 = __nv_bfloat16;

struct LayerDef
{
    int taps, cin, cout, relu;
};

constexpr int N_CONV = 10;
constexpr LayerDef LAYERS[N_CONV] = {
    {9, 16, 32, 1},   // 0 e1
    {9, 32, 64, 1},   // 1 e2
    {9, 64, 96, 1},   // 2 e3
    {9, 96, 128, 1},  // 3 e4
    {1, 128, 96, 0},  // 4 p3
    {9, 96, 96, 1},   // 5 d3
    {1, 96, 64, 0},   // 6 p2
    {9, 64, 64, 1},   // 7 d2
    {1, 64, 32, 0},   // 8 p1
    {9, 32, 32, 1},   // 9 d1
};
constexpr int HEAD_CIN = 32, HEAD_COUT = 4;
constexpr int IN_CH = 16;

isti_status cuda_fail(cudaError_t e, const char *what) { return isti::set_error(ISTI_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e)); }

// ---- elementwise kernels on NHWC bf16, 8 channels (16 bytes) per thread ----

__device__ __forceinline__ void unpack8(uint4 u, float (&f)[8])
{
    const uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
    for (int i = 0; i < 4; i++)
    {
        const __nv_bfloat162 h = *reinterpret_cast<const __nv_bfloat162 *>(&w[i]);
        const float2 v = __bfloat1622float2(h);
        f[2 * i] = v.x;
        f[2 * i + 1] = v.y;
    }
}

__device__ __forceinline__ uint4 pack8(const float (&f)[8])
{
    uint32_t w[4];
#pragma unroll
    for (int i = 0; i < 4; i++)
    {
        const __nv_bfloat162 h = __floats2bfloat162_rn(f[2 * i], f[2 * i + 1]);
        w[i] = *reinterpret_cast<const uint32_t *>(&h);
    }
    return make_uint4(w[0], w[1], w[2], w[3]);
}

// y[n, h/2, w/2] = mean of the 2x2 block of x[n, h, w]
__global__ void pool_kernel(const bf16 *x, int n, int h, int w, int c, bf16 *y)
{
    isti_tc::griddep_launch_dependents();
    isti_tc::griddep_wait();
    const int cg = c / 8, ho = h / 2, wo = w / 2;
    const size_t total = (size_t)n * ho * wo * cg;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x)
    {
        const int g = (int)(i % cg);
        size_t pix = i / cg;
        const int xo = (int)(pix % wo);
        pix /= wo;
        const int yo = (int)(pix % ho);
        const int b = (int)(pix / ho);
        float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int dy = 0; dy < 2; dy++)
            for (int dx = 0; dx < 2; dx++)
            {
                float f[8];
                unpack8(*reinterpret_cast<const uint4 *>(x + ((((size_t)b * h + 2 * yo + dy) * w + 2 * xo + dx) * c + 8 * g)), f);
#pragma unroll
                for (int k = 0; k < 8; k++)
                    acc[k] += f[k];
            }
#pragma unroll
        for (int k = 0; k < 8; k++)
            acc[k] *= 0.25f;
        *reinterpret_cast<uint4 *>(y + (((size_t)b * ho + yo) * wo + xo) * c + 8 * g) = pack8(acc);
    }
}

// s[n, h, w] = a[n, h/2, w/2] (nearest upsampling) + b[n, h, w]
__global__ void upadd_kernel(const bf16 *a, const bf16 *b, int n, int h, int w, int c, bf16 *s)
{
    isti_tc::griddep_launch_dependents();
    isti_tc::griddep_wait();
    const int cg = c / 8;
    const size_t total = (size_t)n * h * w * cg;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x)
    {
        const int g = (int)(i % cg);
        size_t pix = i / cg;
        const int x = (int)(pix % w);
        pix /= w;
        const int y = (int)(pix % h);
        const int bi = (int)(pix / h);
        float fa[8], fb[8];
        unpack8(*reinterpret_cast<const uint4 *>(a + (((size_t)bi * (h / 2) + y / 2) * (w / 2) + x / 2) * c + 8 * g), fa);
        unpack8(*reinterpret_cast<const uint4 *>(b + i * 8), fb);
#pragma unroll
        for (int k = 0; k < 8; k++)
            fa[k] += fb[k];
        *reinterpret_cast<uint4 *>(s + i * 8) = pack8(fa);
    }
}

// r[n, h/2, w/2] = sum of the 2x2 block of g[n, h, w] (gradient of nearest upsampling)
__global__ void downsum_kernel(const bf16 *g, int n, int h, int w, int c, bf16 *r)
{
    const int cg = c / 8, ho = h / 2, wo = w / 2;
    const size_t total = (size_t)n * ho * wo * cg;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x)
    {
        const int gi = (int)(i % cg);
        size_t pix = i / cg;
        const int xo = (int)(pix % wo);
        pix /= wo;
        const int yo = (int)(pix % ho);
        const int b = (int)(pix / ho);
        float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int dy = 0; dy < 2; dy++)
            for (int dx = 0; dx < 2; dx++)
            {
                float f[8];
                unpack8(*reinterpret_cast<const uint4 *>(g + ((((size_t)b * h + 2 * yo + dy) * w + 2 * xo + dx) * c + 8 * gi)), f);
#pragma unroll
                for (int k = 0; k < 8; k++)
                    acc[k] += f[k];
            }
        *reinterpret_cast<uint4 *>(r + (((size_t)b * ho + yo) * wo + xo) * c + 8 * gi) = pack8(acc);
    }
}

// ge[n, h, w] = (gskip[n, h, w] + gq[n, h/2, w/2] / 4) * (act > 0): the gradient of an encoder
// activation that feeds both a skip connection and the 2x2 average pool, through its ReLU
__global__ void poolback_kernel(const bf16 *gskip, const bf16 *gq, const bf16 *act, int n, int h, int w, int c, bf16 *ge)
{
    const int cg = c / 8;
    const size_t total = (size_t)n * h * w * cg;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x)
    {
        const int g = (int)(i % cg);
        size_t pix = i / cg;
        const int x = (int)(pix % w);
        pix /= w;
        const int y = (int)(pix % h);
        const int bi = (int)(pix / h);
        float fs[8], fq[8], fa[8];
        unpack8(*reinterpret_cast<const uint4 *>(gskip + i * 8), fs);
        unpack8(*reinterpret_cast<const uint4 *>(gq + (((size_t)bi * (h / 2) + y / 2) * (w / 2) + x / 2) * c + 8 * g), fq);
        unpack8(*reinterpret_cast<const uint4 *>(act + i * 8), fa);
#pragma unroll
        for (int k = 0; k < 8; k++)
            fs[k] = fa[k] > 0.0f ? fs[k] + 0.25f * fq[k] : 0.0f;
        *reinterpret_cast<uint4 *>(ge + i * 8) = pack8(fs);
    }
}

// Per-block partial sums over pixels of every channel: partial[block][c].  blockDim = 256,
// c <= 256: the first (256 / c) * c threads take a channel each.
__global__ void colsum_partial_kernel(const bf16 *g, size_t npix, int c, float *partial)
{
    __shared__ float red[256];
    const int ch = threadIdx.x % c, lane_pix = threadIdx.x / c, ppb = 256 / c;
    float acc = 0.0f;
    if (lane_pix < ppb)
        for (size_t p = (size_t)blockIdx.x * ppb + lane_pix; p < npix; p += (size_t)gridDim.x * ppb)
            acc += __bfloat162float(g[p * c + ch]);
    red[threadIdx.x] = acc;
    __syncthreads();
    if (threadIdx.x < c)
    {
        float s = 0.0f;
        for (int k = 0; k < ppb; k++)
            s += red[k * c + threadIdx.x];
        partial[(size_t)blockIdx.x * c + threadIdx.x] = s;
    }
}

// out[i] = sum over blocks of partial[block][i] (fixed order)
__global__ void sum_partials_kernel(const float *partial, int blocks, int n, float *out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    float s = 0.0f;
    for (int b = 0; b < blocks; b++)
        s += partial[(size_t)b * n + i];
    out[i] = s;
}

// flow[p][0..3] = hb + hw . d1[p]  (the 1x1 output head, f32); optionally also f16
__global__ void head_kernel(const bf16 *d1, size_t npix, const float *hw, const float *hb, float *flow, __half *flow16)
{
    __shared__ float sw[HEAD_COUT * HEAD_CIN + HEAD_COUT];
    for (int i = threadIdx.x; i < HEAD_COUT * HEAD_CIN; i += blockDim.x)
        sw[i] = hw[i];
    if (threadIdx.x < HEAD_COUT)
        sw[HEAD_COUT * HEAD_CIN + threadIdx.x] = hb[threadIdx.x];
    isti_tc::griddep_launch_dependents();
    isti_tc::griddep_wait(); // the weights above are no previous kernel's output; d1 is
    __syncthreads();
    for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += (size_t)gridDim.x * blockDim.x)
    {
        float f[HEAD_CIN];
        const uint4 *src = reinterpret_cast<const uint4 *>(d1 + p * HEAD_CIN);
#pragma unroll
        for (int q = 0; q < HEAD_CIN / 8; q++)
        {
            float t[8];
            unpack8(src[q], t); // plain load: written by the previous kernel, which may still run at launch
#pragma unroll
            for (int k = 0; k < 8; k++)
                f[8 * q + k] = t[k];
        }
        float o[HEAD_COUT];
#pragma unroll
        for (int j = 0; j < HEAD_COUT; j++)
        {
            float a = sw[HEAD_COUT * HEAD_CIN + j];
#pragma unroll
            for (int k = 0; k < HEAD_CIN; k++)
                a = fmaf(sw[j * HEAD_CIN + k], f[k], a); // fused multiply-adds in channel order, as the fused head
            o[j] = a;
        }
        if (flow)
            *reinterpret_cast<float4 *>(flow + p * 4) = make_float4(o[0], o[1], o[2], o[3]);
        if (flow16)
        {
            __half2 a = __floats2half2_rn(o[0], o[1]), b = __floats2half2_rn(o[2], o[3]);
            uint2 u;
            u.x = *reinterpret_cast<uint32_t *>(&a);
            u.y = *reinterpret_cast<uint32_t *>(&b);
            *reinterpret_cast<uint2 *>(flow16 + p * 4) = u;
        }
    }
}

// Loss and head backward.  Loss = sum over labelled entries of huber(flow - label) / npix
// (label NaN = not labelled; huber with delta 1: 0.5 d^2 for |d| < 1, |d| - 0.5 beyond).
// Writes the gradient of the head's input through d1's ReLU (bf16), and per-block partials
// of the loss [block][1] and of the head's weight/bias gradients [block][4 * 32 + 4].
constexpr int HEAD_GRADS = HEAD_COUT * HEAD_CIN + HEAD_COUT;
__global__ void head_back_kernel(const bf16 *d1, size_t npix, const float *hw, const float *hb, const float *label, float inv_norm, bf16 *g_d1,
                                 float *loss_partial, float *hgrad_partial)
{
    __shared__ float sw[HEAD_GRADS];
    __shared__ float acc[HEAD_GRADS + 1];
    for (int i = threadIdx.x; i < HEAD_COUT * HEAD_CIN; i += blockDim.x)
        sw[i] = hw[i];
    if (threadIdx.x < HEAD_COUT)
        sw[HEAD_COUT * HEAD_CIN + threadIdx.x] = hb[threadIdx.x];
    for (int i = threadIdx.x; i < HEAD_GRADS + 1; i += blockDim.x)
        acc[i] = 0.0f;
    __syncthreads();
    float my_loss = 0.0f;
    float my_g[HEAD_GRADS];
#pragma unroll
    for (int i = 0; i < HEAD_GRADS; i++)
        my_g[i] = 0.0f;
    for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += (size_t)gridDim.x * blockDim.x)
    {
        float f[HEAD_CIN];
        const uint4 *src = reinterpret_cast<const uint4 *>(d1 + p * HEAD_CIN);
#pragma unroll
        for (int q = 0; q < HEAD_CIN / 8; q++)
        {
            float t[8];
            unpack8(__ldg(src + q), t);
#pragma unroll
            for (int k = 0; k < 8; k++)
                f[8 * q + k] = t[k];
        }
        float go[HEAD_COUT];
#pragma unroll
        for (int j = 0; j < HEAD_COUT; j++)
        {
            float a = sw[HEAD_COUT * HEAD_CIN + j];
#pragma unroll
            for (int k = 0; k < HEAD_CIN; k++)
                a = fmaf(sw[j * HEAD_CIN + k], f[k], a); // fused multiply-adds in channel order, as the fused head
            const float l = __ldg(label + p * 4 + j);
            go[j] = 0.0f;
            if (!isnan(l))
            {
                const float d = a - l, ad = fabsf(d);
                my_loss += (ad < 1.0f ? 0.5f * d * d : ad - 0.5f) * inv_norm;
                go[j] = fminf(1.0f, fmaxf(-1.0f, d)) * inv_norm;
            }
        }
        float gi[HEAD_CIN];
#pragma unroll
        for (int k = 0; k < HEAD_CIN; k++)
        {
            float s = 0.0f;
#pragma unroll
            for (int j = 0; j < HEAD_COUT; j++)
                s += sw[j * HEAD_CIN + k] * go[j];
            gi[k] = f[k] > 0.0f ? s : 0.0f;
        }
#pragma unroll
        for (int j = 0; j < HEAD_COUT; j++)
        {
#pragma unroll
            for (int k = 0; k < HEAD_CIN; k++)
                my_g[j * HEAD_CIN + k] += go[j] * f[k];
            my_g[HEAD_COUT * HEAD_CIN + j] += go[j];
        }
        uint4 *dst = reinterpret_cast<uint4 *>(g_d1 + p * HEAD_CIN);
#pragma unroll
        for (int q = 0; q < HEAD_CIN / 8; q++)
        {
            float t[8];
#pragma unroll
            for (int k = 0; k < 8; k++)
                t[k] = gi[8 * q + k];
            dst[q] = pack8(t);
        }
    }
    // block reduction: warp shuffles, then one shared-memory add per warp and value
#pragma unroll
    for (int i = 0; i < HEAD_GRADS; i++)
    {
        float v = my_g[i];
        for (int o = 16; o > 0; o >>= 1)
            v += __shfl_xor_sync(0xffffffffu, v, o);
        my_g[i] = v;
    }
    for (int o = 16; o > 0; o >>= 1)
        my_loss += __shfl_xor_sync(0xffffffffu, my_loss, o);
    const int warps = blockDim.x / 32;
    for (int wv = 0; wv < warps; wv++) // fixed warp order: deterministic
    {
        if ((int)threadIdx.x / 32 == wv && threadIdx.x % 32 == 0)
        {
            for (int i = 0; i < HEAD_GRADS; i++)
                acc[i] += my_g[i];
            acc[HEAD_GRADS] += my_loss;
        }
        __syncthreads();
    }
    for (int i = threadIdx.x; i < HEAD_GRADS; i += blockDim.x)
        hgrad_partial[(size_t)blockIdx.x * HEAD_GRADS + i] = acc[i];
    if (threadIdx.x == 0)
        loss_partial[blockIdx.x] = acc[HEAD_GRADS];
}

// Adam on f32 parameters (bias-corrected; beta1 0.9, beta2 0.999, eps 1e-8)
__global__ void adam_kernel(float *w, const float *g, float *m, float *v, size_t n, float lr, float c1, float c2)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const float gi = g[i];
    const float mi = 0.9f * m[i] + 0.1f * gi, vi = 0.999f * v[i] + 0.001f * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + 1e-8f);
}

unsigned grid_for(size_t work) { return (unsigned)std::max<size_t>(1, std::min<size_t>((work + 255) / 256, 152 * 8)); }

constexpr int REDUCE_BLOCKS = 256;
} // namespace

struct isti_flownet
{
    int device = 0;
    // parameters: f32 [w_0 b_0 w_1 b_1 ... w_9 b_9 head_w head_b], grads and Adam moments alike
    size_t n_params = 0;
    size_t w_off[N_CONV + 1] = {}, b_off[N_CONV + 1] = {};
    float *params = nullptr, *grads = nullptr, *adam_m = nullptr, *adam_v = nullptr;
    int adam_step = 0;
    // packed bf16 operand images (forward and data-gradient) per layer
    size_t pk_off[N_CONV] = {}, pkt_off[N_CONV] = {};
    bf16 *packs = nullptr;
    int32_t *status = nullptr;
    float *loss = nullptr;     // device scalar of the last training step
    // activation / gradient arena for the current shape
    int n = 0, h = 0, w = 0;
    void *arena = nullptr;
    size_t arena_bytes = 0;
};

namespace
{
// activations and gradients of one shape, carved from the arena
struct Buffers
{
    bf16 *e1, *q1, *e2, *q2, *e3, *q3, *e4, *p3, *s3, *d3, *p2, *s2, *d2, *p1, *s1, *d1;
    bf16 *g_d1, *g_s1, *g_p1, *g_d2, *g_s2, *g_p2, *g_d3, *g_s3, *g_p3, *g_e4, *g_q3, *g_e3, *g_q2, *g_e2, *g_q1, *g_e1;
    float *flow, *partial, *wscratch;
    size_t wscratch_bytes;
};

size_t align256(size_t v) { return (v + 255) / 256 * 256; }

// Lays out (or, with base == nullptr, measures) the buffers of an n x h x w input.
size_t layout(Buffers &b, char *base, int n, int h, int w)
{
    size_t off = 0;
    auto take = [&](size_t bytes) {
        char *p = base ? base + off : nullptr;
        off += align256(bytes);
        return p;
    };
    const size_t p1 = (size_t)n * h * w, p2 = p1 / 4, p3 = p1 / 16, p4 = p1 / 64;
    auto t = [&](size_t pix, int c) { return reinterpret_cast<bf16 *>(take(pix * c * 2)); };
    b.e1 = t(p1, 32), b.q1 = t(p2, 32), b.e2 = t(p2, 64), b.q2 = t(p3, 64), b.e3 = t(p3, 96), b.q3 = t(p4, 96), b.e4 = t(p4, 128);
    b.p3 = t(p4, 96), b.s3 = t(p3, 96), b.d3 = t(p3, 96), b.p2 = t(p3, 64), b.s2 = t(p2, 64), b.d2 = t(p2, 64), b.p1 = t(p2, 32);
    b.s1 = t(p1, 32), b.d1 = t(p1, 32);
    b.g_d1 = t(p1, 32), b.g_s1 = t(p1, 32), b.g_p1 = t(p2, 32), b.g_d2 = t(p2, 64), b.g_s2 = t(p2, 64), b.g_p2 = t(p3, 64);
    b.g_d3 = t(p3, 96), b.g_s3 = t(p3, 96), b.g_p3 = t(p4, 96), b.g_e4 = t(p4, 128), b.g_q3 = t(p4, 96), b.g_e3 = t(p3, 96);
    b.g_q2 = t(p3, 64), b.g_e2 = t(p2, 64), b.g_q1 = t(p2, 32), b.g_e1 = t(p1, 32);
    b.flow = reinterpret_cast<float *>(take(p1 * 4 * sizeof(float)));
    b.partial = reinterpret_cast<float *>(take((size_t)REDUCE_BLOCKS * (HEAD_GRADS + 128) * sizeof(float)));
    size_t ws = 0;
    const int hs[N_CONV] = {h, h / 2, h / 4, h / 8, h / 8, h / 4, h / 4, h / 2, h / 2, h};
    const int wsz[N_CONV] = {w, w / 2, w / 4, w / 8, w / 8, w / 4, w / 4, w / 2, w / 2, w};
    for (int l = 0; l < N_CONV; l++)
        ws = std::max(ws, isti_unet::wgrad_scratch(LAYERS[l].taps, n, hs[l], wsz[l], LAYERS[l].cin, LAYERS[l].cout));
    b.wscratch_bytes = ws;
    b.wscratch = reinterpret_cast<float *>(take(ws));
    return off;
}

isti_status ensure_arena(isti_flownet *net, int n, int h, int w, Buffers &b)
{
    Buffers tmp{};
    const size_t need = layout(tmp, nullptr, n, h, w);
    if (need > net->arena_bytes)
    {
        if (net->arena)
            cudaFree(net->arena);
        net->arena = nullptr;
        net->arena_bytes = 0;
        const cudaError_t e = cudaMalloc(&net->arena, need);
        if (e != cudaSuccess)
            return e == cudaErrorMemoryAllocation ? isti::set_error(ISTI_ERR_OOM, "flownet: activation arena") : cuda_fail(e, "cudaMalloc");
        net->arena_bytes = need;
    }
    net->n = n;
    net->h = h;
    net->w = w;
    layout(b, static_cast<char *>(net->arena), n, h, w);
    return ISTI_OK;
}

isti_status repack(isti_flownet *net, cudaStream_t s)
{
    for (int l = 0; l < N_CONV; l++)
    {
        const LayerDef &d = LAYERS[l];
        isti_status st = isti_unet::pack_launch(d.taps, net->params + net->w_off[l], d.cin, d.cout, 0, net->packs + net->pk_off[l], s);
        if (st == ISTI_OK && l > 0) // the first layer's data gradient is never needed
            st = isti_unet::pack_launch(d.taps, net->params + net->w_off[l], d.cin, d.cout, 1, net->packs + net->pkt_off[l], s);
        if (st != ISTI_OK)
            return st;
    }
    return ISTI_OK;
}

isti_status conv(isti_flownet *net, int l, const bf16 *x, int n, int h, int w, const bf16 *mask, bf16 *out, cudaStream_t s, bool pdl = false,
                 const isti_unet::ConvHead *head = nullptr, bool *head_fused = nullptr)
{
    const LayerDef &d = LAYERS[l];
    return isti_unet::conv_launch(d.taps, x, n, h, w, d.cin, net->packs + net->pk_off[l], net->params + net->b_off[l], mask, d.relu, out, d.cout,
                                  net->status, s, pdl, head, head_fused);
}

// data gradient of layer l: g_in = conv(g_out, W^T flipped), masked by (mask > 0) when given
isti_status dgrad(isti_flownet *net, int l, const bf16 *g_out, int n, int h, int w, const bf16 *mask, bf16 *g_in, cudaStream_t s)
{
    const LayerDef &d = LAYERS[l];
    return isti_unet::conv_launch(d.taps, g_out, n, h, w, d.cout, net->packs + net->pkt_off[l], nullptr, mask, 0, g_in, d.cin, net->status, s);
}

isti_status wgrad(isti_flownet *net, int l, const bf16 *g_out, const bf16 *x, int n, int h, int w, Buffers &b, cudaStream_t s)
{
    const LayerDef &d = LAYERS[l];
    isti_status st = isti_unet::wgrad_launch(d.taps, g_out, x, n, h, w, d.cin, d.cout, net->grads + net->w_off[l], 0, b.wscratch,
                                             b.wscratch_bytes, net->status, s);
    if (st != ISTI_OK)
        return st;
    // bias gradient: column sums of g_out
    const size_t npix = (size_t)n * h * w;
    colsum_partial_kernel<<<REDUCE_BLOCKS, 256, 0, s>>>(g_out, npix, d.cout, b.partial);
    sum_partials_kernel<<<(d.cout + 127) / 128, 128, 0, s>>>(b.partial, REDUCE_BLOCKS, d.cout, net->grads + net->b_off[l]);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? ISTI_OK : cuda_fail(e, "bias gradient");
}

#define ISTI_TRY(x)                                                                                                                             \
    do                                                                                                                                          \
    {                                                                                                                                           \
        const isti_status st_ = (x);                                                                                                            \
        if (st_ != ISTI_OK)                                                                                                                     \
            return st_;                                                                                                                         \
    } while (0)

// pdl: every launch after the first is a programmatic dependent of the one before (each
// kernel sets up while its predecessor finishes; inference only)
isti_status forward(isti_flownet *net, const bf16 *x0, int n, int h, int w, Buffers &b, float *flow, __half *flow16, cudaStream_t s,
                    bool pdl = false)
{
    using isti_unet::launch_kernel;
    const int h2 = h / 2, w2 = w / 2, h4 = h / 4, w4 = w / 4, h8 = h / 8, w8 = w / 8;
    const dim3 blk(256);
    cudaError_t e = cudaSuccess;
    auto ok = [&](cudaError_t x) {
        if (e == cudaSuccess)
            e = x;
        return e == cudaSuccess;
    };
    ISTI_TRY(conv(net, 0, x0, n, h, w, nullptr, b.e1, s, pdl));
    ok(launch_kernel(pool_kernel, dim3(grid_for((size_t)n * h2 * w2 * 4)), blk, 0, s, pdl, (const bf16 *)b.e1, n, h, w, 32, b.q1));
    ISTI_TRY(conv(net, 1, b.q1, n, h2, w2, nullptr, b.e2, s, pdl));
    ok(launch_kernel(pool_kernel, dim3(grid_for((size_t)n * h4 * w4 * 8)), blk, 0, s, pdl, (const bf16 *)b.e2, n, h2, w2, 64, b.q2));
    ISTI_TRY(conv(net, 2, b.q2, n, h4, w4, nullptr, b.e3, s, pdl));
    ok(launch_kernel(pool_kernel, dim3(grid_for((size_t)n * h8 * w8 * 12)), blk, 0, s, pdl, (const bf16 *)b.e3, n, h4, w4, 96, b.q3));
    ISTI_TRY(conv(net, 3, b.q3, n, h8, w8, nullptr, b.e4, s, pdl));
    ISTI_TRY(conv(net, 4, b.e4, n, h8, w8, nullptr, b.p3, s, pdl));
    ok(launch_kernel(upadd_kernel, dim3(grid_for((size_t)n * h4 * w4 * 12)), blk, 0, s, pdl, (const bf16 *)b.p3, (const bf16 *)b.e3, n, h4, w4,
                     96, b.s3));
    ISTI_TRY(conv(net, 5, b.s3, n, h4, w4, nullptr, b.d3, s, pdl));
    ISTI_TRY(conv(net, 6, b.d3, n, h4, w4, nullptr, b.p2, s, pdl));
    ok(launch_kernel(upadd_kernel, dim3(grid_for((size_t)n * h2 * w2 * 8)), blk, 0, s, pdl, (const bf16 *)b.p2, (const bf16 *)b.e2, n, h2, w2,
                     64, b.s2));
    ISTI_TRY(conv(net, 7, b.s2, n, h2, w2, nullptr, b.d2, s, pdl));
    ISTI_TRY(conv(net, 8, b.d2, n, h2, w2, nullptr, b.p1, s, pdl));
    ok(launch_kernel(upadd_kernel, dim3(grid_for((size_t)n * h * w * 4)), blk, 0, s, pdl, (const bf16 *)b.p1, (const bf16 *)b.e1, n, h, w, 32,
                     b.s1));
    // inference: the 1x1 head in d1's epilogue where the row-tile kernel runs d1 (d1 itself is
    // then not stored), else its own kernel
    const isti_unet::ConvHead head{net->params + net->w_off[N_CONV], net->params + net->b_off[N_CONV], flow, flow16};
    bool fused = false;
    ISTI_TRY(conv(net, 9, b.s1, n, h, w, nullptr, b.d1, s, pdl, pdl && (flow || flow16) ? &head : nullptr, &fused));
    if ((flow || flow16) && !fused)
        ok(launch_kernel(head_kernel, dim3(grid_for((size_t)n * h * w)), blk, 0, s, pdl, (const bf16 *)b.d1, (size_t)n * h * w,
                         (const float *)(net->params + net->w_off[N_CONV]), (const float *)(net->params + net->b_off[N_CONV]), flow, flow16));
    if (e == cudaSuccess)
        e = cudaGetLastError();
    return e == cudaSuccess ? ISTI_OK : cuda_fail(e, "flownet forward");
}

isti_status backward(isti_flownet *net, const bf16 *x0, const float *label, int n, int h, int w, Buffers &b, cudaStream_t s)
{
    const int h2 = h / 2, w2 = w / 2, h4 = h / 4, w4 = w / 4, h8 = h / 8, w8 = w / 8;
    const size_t npix = (size_t)n * h * w;
    head_back_kernel<<<REDUCE_BLOCKS, 256, 0, s>>>(b.d1, npix, net->params + net->w_off[N_CONV], net->params + net->b_off[N_CONV], label,
                                                  1.0f / (float)npix, b.g_d1, b.partial, b.partial + REDUCE_BLOCKS);
    sum_partials_kernel<<<1, 32, 0, s>>>(b.partial, REDUCE_BLOCKS, 1, net->loss);
    sum_partials_kernel<<<1, 256, 0, s>>>(b.partial + REDUCE_BLOCKS, REDUCE_BLOCKS, HEAD_GRADS, net->grads + net->w_off[N_CONV]);
    // level 1 decoder
    ISTI_TRY(wgrad(net, 9, b.g_d1, b.s1, n, h, w, b, s));
    ISTI_TRY(dgrad(net, 9, b.g_d1, n, h, w, nullptr, b.g_s1, s));
    downsum_kernel<<<grid_for((size_t)n * h2 * w2 * 4), 256, 0, s>>>(b.g_s1, n, h, w, 32, b.g_p1);
    ISTI_TRY(wgrad(net, 8, b.g_p1, b.d2, n, h2, w2, b, s));
    ISTI_TRY(dgrad(net, 8, b.g_p1, n, h2, w2, b.d2, b.g_d2, s));
    // level 2 decoder
    ISTI_TRY(wgrad(net, 7, b.g_d2, b.s2, n, h2, w2, b, s));
    ISTI_TRY(dgrad(net, 7, b.g_d2, n, h2, w2, nullptr, b.g_s2, s));
    downsum_kernel<<<grid_for((size_t)n * h4 * w4 * 8), 256, 0, s>>>(b.g_s2, n, h2, w2, 64, b.g_p2);
    ISTI_TRY(wgrad(net, 6, b.g_p2, b.d3, n, h4, w4, b, s));
    ISTI_TRY(dgrad(net, 6, b.g_p2, n, h4, w4, b.d3, b.g_d3, s));
    // level 3 decoder
    ISTI_TRY(wgrad(net, 5, b.g_d3, b.s3, n, h4, w4, b, s));
    ISTI_TRY(dgrad(net, 5, b.g_d3, n, h4, w4, nullptr, b.g_s3, s));
    downsum_kernel<<<grid_for((size_t)n * h8 * w8 * 12), 256, 0, s>>>(b.g_s3, n, h4, w4, 96, b.g_p3);
    ISTI_TRY(wgrad(net, 4, b.g_p3, b.e4, n, h8, w8, b, s));
    ISTI_TRY(dgrad(net, 4, b.g_p3, n, h8, w8, b.e4, b.g_e4, s));
    // bottleneck and encoder
    ISTI_TRY(wgrad(net, 3, b.g_e4, b.q3, n, h8, w8, b, s));
    ISTI_TRY(dgrad(net, 3, b.g_e4, n, h8, w8, nullptr, b.g_q3, s));
    poolback_kernel<<<grid_for((size_t)n * h4 * w4 * 12), 256, 0, s>>>(b.g_s3, b.g_q3, b.e3, n, h4, w4, 96, b.g_e3);
    ISTI_TRY(wgrad(net, 2, b.g_e3, b.q2, n, h4, w4, b, s));
    ISTI_TRY(dgrad(net, 2, b.g_e3, n, h4, w4, nullptr, b.g_q2, s));
    poolback_kernel<<<grid_for((size_t)n * h2 * w2 * 8), 256, 0, s>>>(b.g_s2, b.g_q2, b.e2, n, h2, w2, 64, b.g_e2);
    ISTI_TRY(wgrad(net, 1, b.g_e2, b.q1, n, h2, w2, b, s));
    ISTI_TRY(dgrad(net, 1, b.g_e2, n, h2, w2, nullptr, b.g_q1, s));
    poolback_kernel<<<grid_for((size_t)n * h * w * 4), 256, 0, s>>>(b.g_s1, b.g_q1, b.e1, n, h, w, 32, b.g_e1);
    ISTI_TRY(wgrad(net, 0, b.g_e1, x0, n, h, w, b, s));
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? ISTI_OK : cuda_fail(e, "flownet backward");
}

isti_status check_shape(const void *x, int n, int h, int w)
{
    if (!x || n < 1 || h < 8 || w < 16 || h % 8 || w % 8)
        return isti::set_error(ISTI_ERR_INVALID_ARG, "flownet: input must be n x h x w x 16 with h, w multiples of 8 (w >= 16)");
    return ISTI_OK;
}
} // namespace

extern "C" {

int32_t isti_flownet_input_channels(void) { return IN_CH; }
int32_t isti_flownet_output_channels(void) { return HEAD_COUT; }
int32_t isti_flownet_num_layers(void) { return N_CONV + 1; }

isti_status isti_flownet_layer(int32_t index, int32_t *taps, int32_t *cin, int32_t *cout, int32_t *relu)
{
    if (index < 0 || index > N_CONV)
        return isti::set_error(ISTI_ERR_INVALID_ARG, "flownet: layer index out of range");
    const LayerDef d = index < N_CONV ? LAYERS[index] : LayerDef{1, HEAD_CIN, HEAD_COUT, 0};
    if (taps)
        *taps = d.taps;
    if (cin)
        *cin = d.cin;
    if (cout)
        *cout = d.cout;
    if (relu)
        *relu = d.relu;
    return ISTI_OK;
}

isti_status isti_flownet_create(isti_flownet **out, uint64_t seed)
{
    if (!out)
        return isti::set_error(ISTI_ERR_INVALID_ARG, "out is NULL");
    isti_flownet *net = new (std::nothrow) isti_flownet();
    if (!net)
        return isti::set_error(ISTI_ERR_OOM, "host allocation failed");
    cudaGetDevice(&net->device);
    size_t off = 0, pk = 0;
    for (int l = 0; l <= N_CONV; l++)
    {
        const LayerDef d = l < N_CONV ? LAYERS[l] : LayerDef{1, HEAD_CIN, HEAD_COUT, 0};
        net->w_off[l] = off;
        off += (size_t)d.taps * d.cin * d.cout;
        net->b_off[l] = off;
        off += (size_t)d.cout;
        off = (off + 3) / 4 * 4; // 16-byte aligned tensors
        if (l < N_CONV)
        {
            net->pk_off[l] = pk;
            pk += (size_t)d.taps * d.cin * d.cout;
            net->pkt_off[l] = pk;
            pk += (size_t)d.taps * d.cin * d.cout;
        }
    }
    net->n_params = off;
    // He-normal weights, zero biases (host PRNG: reproducible for a seed)
    std::vector<float> host(off, 0.0f);
    std::mt19937_64 rng(seed);
    for (int l = 0; l <= N_CONV; l++)
    {
        const LayerDef d = l < N_CONV ? LAYERS[l] : LayerDef{1, HEAD_CIN, HEAD_COUT, 0};
        const float sd = l < N_CONV ? std::sqrt(2.0f / (float)(d.taps * d.cin)) : 0.01f;
        std::normal_distribution<float> nd(0.0f, sd);
        for (size_t i = 0; i < (size_t)d.taps * d.cin * d.cout; i++)
            host[net->w_off[l] + i] = nd(rng);
    }
    cudaError_t e = cudaMalloc(&net->params, off * sizeof(float) * 4);
    if (e == cudaSuccess)
        e = cudaMalloc(&net->packs, pk * sizeof(bf16));
    if (e == cudaSuccess)
        e = cudaMalloc(&net->status, 256);
    if (e != cudaSuccess)
    {
        isti_flownet_destroy(net);
        return isti::set_error(ISTI_ERR_OOM, "flownet: parameter allocation");
    }
    net->grads = net->params + off;
    net->adam_m = net->grads + off;
    net->adam_v = net->adam_m + off;
    net->loss = reinterpret_cast<float *>(net->status + 32);
    cudaMemset(net->params, 0, off * sizeof(float) * 4);
    cudaMemset(net->status, 0, 256);
    cudaMemcpy(net->params, host.data(), off * sizeof(float), cudaMemcpyHostToDevice);
    isti_status st = repack(net, nullptr);
    if (st == ISTI_OK)
    {
        e = cudaDeviceSynchronize();
        if (e != cudaSuccess)
            st = cuda_fail(e, "flownet init");
    }
    if (st != ISTI_OK)
    {
        isti_flownet_destroy(net);
        return st;
    }
    *out = net;
    return ISTI_OK;
}

isti_status isti_flownet_destroy(isti_flownet *net)
{
    if (!net)
        return ISTI_OK;
    cudaFree(net->params);
    cudaFree(net->packs);
    cudaFree(net->status);
    cudaFree(net->arena);
    delete net;
    return ISTI_OK;
}

isti_status isti_flownet_tensors(isti_flownet *net, float **params, float **grads, size_t *count)
{
    if (!net)
        return isti::set_error(ISTI_ERR_INVALID_ARG, "flownet is NULL");
    if (params)
        *params = net->params;
    if (grads)
        *grads = net->grads;
    if (count)
        *count = net->n_params;
    return ISTI_OK;
}

isti_status isti_flownet_param_offsets(const isti_flownet *net, int32_t layer, size_t *w_off, size_t *b_off)
{
    if (!net || layer < 0 || layer > N_CONV)
        return isti::set_error(ISTI_ERR_INVALID_ARG, "flownet: bad layer");
    if (w_off)
        *w_off = net->w_off[layer];
    if (b_off)
        *b_off = net->b_off[layer];
    return ISTI_OK;
}

isti_status isti_flownet_sync_params(isti_flownet *net, void *stream)
{
    if (!net)
        return isti::set_error(ISTI_ERR_INVALID_ARG, "flownet is NULL");
    return repack(net, static_cast<cudaStream_t>(stream));
}

isti_status isti_flownet_forward(isti_flownet *net, const void *x, int32_t n, int32_t h, int32_t w, float *flow, void *flow_f16, void *stream)
{
    if (!net)
        return isti::set_error(ISTI_ERR_INVALID_ARG, "flownet is NULL");
    ISTI_TRY(check_shape(x, n, h, w));
    Buffers b{};
    ISTI_TRY(ensure_arena(net, n, h, w, b));
    return forward(net, static_cast<const bf16 *>(x), n, h, w, b, flow, static_cast<__half *>(flow_f16), static_cast<cudaStream_t>(stream),
                   true);
}

isti_status isti_flownet_backward(isti_flownet *net, const void *x, const float *label, int32_t n, int32_t h, int32_t w, void *stream)
{
    if (!net || !label)
        return isti::set_error(ISTI_ERR_INVALID_ARG, "NULL argument");
    ISTI_TRY(check_shape(x, n, h, w));
    Buffers b{};
    ISTI_TRY(ensure_arena(net, n, h, w, b));
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    ISTI_TRY(forward(net, static_cast<const bf16 *>(x), n, h, w, b, nullptr, nullptr, s));
    return backward(net, static_cast<const bf16 *>(x), label, n, h, w, b, s);
}

isti_status isti_flownet_adam(isti_flownet *net, float lr, void *stream)
{
    if (!net)
        return isti::set_error(ISTI_ERR_INVALID_ARG, "flownet is NULL");
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    net->adam_step++;
    const float c1 = 1.0f - std::pow(0.9f, (float)net->adam_step), c2 = 1.0f - std::pow(0.999f, (float)net->adam_step);
    adam_kernel<<<(unsigned)((net->n_params + 255) / 256), 256, 0, s>>>(net->params, net->grads, net->adam_m, net->adam_v, net->n_params, lr, c1,
                                                                        c2);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return cuda_fail(e, "flownet adam");
    return repack(net, s);
}

isti_status isti_flownet_loss(isti_flownet *net, float **loss_device)
{
    if (!net || !loss_device)
        return isti::set_error(ISTI_ERR_INVALID_ARG, "NULL argument");
    *loss_device = net->loss;
    return ISTI_OK;
}

isti_status isti_flownet_device_status(isti_flownet *net, int32_t *status)
{
    if (!net || !status)
        return isti::set_error(ISTI_ERR_INVALID_ARG, "NULL argument");
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess)
        e = cudaMemcpy(status, net->status, sizeof(int32_t), cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? ISTI_OK : cuda_fail(e, "flownet status");
}

} // extern "C"
