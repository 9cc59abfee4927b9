// Host side of the learned flow initialiser: tensor maps and launches of the tcgen05
// convolution kernels (isti_unet_conv.cuh) and the C ABI of include/isti_unet.h.
#include "isti_unet.h"
#include "isti_unet_conv.cuh"
#include "isti_unet_ops.h"
#include "host/isti_error.hpp"

#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <string>
#include <vector>

namespace
{
using namespace isti_unet;

isti_status cuda_fail(cudaError_t e, const char *what) { return isti::set_error(ISTI_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e)); }

using EncodeTiledFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *, const cuuint64_t *,
                                   const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                   CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_tiled()
{
    static EncodeTiledFn fn = [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            return (EncodeTiledFn) nullptr;
        return reinterpret_cast<EncodeTiledFn>(f);
    }();
    return fn;
}

// 4-D map over an NHWC bf16 tensor: dims (c, w, h, n), box {8 channels, 16 x, 8 y, 1}.
isti_status nhwc_map(CUtensorMap &m, const void *base, int n, int h, int w, int c)
{
    EncodeTiledFn enc = encode_tiled();
    if (!enc)
        return isti::set_error(ISTI_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled unavailable");
    if (((uintptr_t)base & 15u) || c % 8)
        return isti::set_error(ISTI_ERR_INVALID_ARG, "NHWC tensor: base 16-byte aligned, channels a multiple of 8");
    const cuuint64_t dims[4] = {(cuuint64_t)c, (cuuint64_t)w, (cuuint64_t)h, (cuuint64_t)n};
    const cuuint64_t strides[3] = {(cuuint64_t)c * 2u, (cuuint64_t)w * c * 2u, (cuuint64_t)h * w * c * 2u};
    const cuuint32_t box[4] = {8, (cuuint32_t)TILE_W, (cuuint32_t)TILE_H, 1};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    if (enc(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void *>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return isti::set_error(ISTI_ERR_INVALID_ARG, "cuTensorMapEncodeTiled rejected an NHWC tensor");
    return ISTI_OK;
}

// 5-D map over an NHWC bf16 tensor with the channels split as (8, c / 8) and the chunk index
// outermost: dims (c_lo, w, h, c_hi, n), box {8, 16 x, 8 y, ck / 8 chunks, 1}, so one copy lands
// a stage's channel chunks one after another (the layout of ck / 8 separate 4-D boxes).
// Returns false when the driver does not accept the strides.
bool nhwc_chunked_map(CUtensorMap &m, const void *base, int n, int h, int w, int c, int ck)
{
    EncodeTiledFn enc = encode_tiled();
    if (!enc || ((uintptr_t)base & 15u) || c % 8 || ck % 8)
        return false;
    const cuuint64_t dims[5] = {8, (cuuint64_t)w, (cuuint64_t)h, (cuuint64_t)(c / 8), (cuuint64_t)n};
    const cuuint64_t strides[4] = {(cuuint64_t)c * 2u, (cuuint64_t)w * c * 2u, 16u, (cuuint64_t)h * w * c * 2u};
    const cuuint32_t box[5] = {8, (cuuint32_t)TILE_W, (cuuint32_t)TILE_H, (cuuint32_t)(ck / 8), 1};
    const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
    return enc(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<void *>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// 5-D map for row_conv_kernel: box {8, 130 x, 3 y, ck / 8 chunks, 1} (a 128-pixel row segment
// with its halo).
bool nhwc_row_map(CUtensorMap &m, const void *base, int n, int h, int w, int c, int ck)
{
    EncodeTiledFn enc = encode_tiled();
    if (!enc || ((uintptr_t)base & 15u) || c % 8 || ck % 8)
        return false;
    const cuuint64_t dims[5] = {8, (cuuint64_t)w, (cuuint64_t)h, (cuuint64_t)(c / 8), (cuuint64_t)n};
    const cuuint64_t strides[4] = {(cuuint64_t)c * 2u, (cuuint64_t)w * c * 2u, 16u, (cuuint64_t)h * w * c * 2u};
    const cuuint32_t box[5] = {8, (cuuint32_t)ROW_HALO, 3, (cuuint32_t)(ck / 8), 1};
    const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
    return enc(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<void *>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

int sm_count()
{
    static int n[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess)
        return 152;
    if (!n[dev & 63])
    {
        int v = 0;
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        n[dev & 63] = v > 0 ? v : 152;
    }
    return n[dev & 63];
}

// A kernel's dynamic shared-memory limit, raised once per kernel and device to the largest
// size asked (keyed by the kernel's address: instances of one template share a type).
template <class K>
cudaError_t smem_limit(K kernel, size_t bytes)
{
    struct Entry
    {
        const void *fn;
        int dev;
        size_t bytes;
    };
    static std::mutex mu;
    static std::vector<Entry> set;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || bytes <= 48 * 1024)
        return e;
    std::lock_guard<std::mutex> lock(mu);
    const void *fn = reinterpret_cast<const void *>(kernel);
    for (Entry &x : set)
        if (x.fn == fn && x.dev == dev)
        {
            if (bytes > x.bytes)
            {
                e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
                if (e == cudaSuccess)
                    x.bytes = bytes;
            }
            return e;
        }
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess)
        set.push_back({fn, dev, bytes});
    return e;
}

constexpr size_t SMEM_BUDGET = 200 * 1024;
int32_t *g_null_status = nullptr; // device word for callers that pass no status

isti_status status_word(int32_t *&status)
{
    if (status)
        return ISTI_OK;
    static std::mutex mu;
    std::lock_guard<std::mutex> lock(mu);
    if (!g_null_status)
    {
        cudaError_t e = cudaMalloc(&g_null_status, 256);
        if (e != cudaSuccess)
            return cuda_fail(e, "cudaMalloc(status word)");
        cudaMemset(g_null_status, 0, 256);
    }
    status = g_null_status;
    return ISTI_OK;
}
} // namespace

namespace isti_unet
{
// Launch of conv_kernel<taps> (shared with the network code in isti_flownet.cu).
isti_status conv_launch(int taps, const void *x, int n, int h, int w, int cin, const void *wpack, const float *bias, const void *mask, int relu,
                        void *out, int cout, int32_t *status, cudaStream_t stream, bool pdl, const ConvHead *head, bool *head_fused)
{
    if (head_fused)
        *head_fused = false;
    if (head && (!head->w || !head->b || (!head->flow && !head->flow16) || ((uintptr_t)head->flow & 15u) || ((uintptr_t)head->flow16 & 7u)))
        return isti::set_error(ISTI_ERR_INVALID_ARG, "isti_unet_conv: fused head needs weights, bias and an aligned output");
    if ((taps != 9 && taps != 1) || n < 1 || h < 1 || w < 1 || cin % 16 || cout % 16 || cout < 16 || cout > 256 || !x || !wpack || !out)
        return isti::set_error(ISTI_ERR_INVALID_ARG, "isti_unet_conv: bad shape or NULL buffer");
    if (((uintptr_t)out & 15u) || ((uintptr_t)mask & 15u) || ((uintptr_t)wpack & 15u))
        return isti::set_error(ISTI_ERR_INVALID_ARG, "isti_unet_conv: buffers must be 16-byte aligned");
    isti_status st = status_word(status);
    if (st != ISTI_OK)
        return st;
    ConvParams p{};
    p.wpack = static_cast<const __nv_bfloat16 *>(wpack);
    p.bias = bias;
    p.mask = static_cast<const __nv_bfloat16 *>(mask);
    p.out = static_cast<__nv_bfloat16 *>(out);
    p.status = status;
    p.w = w;
    p.h = h;
    p.b = n;
    p.cin = cin;
    p.cout = cout;
    p.ck = cin % 32 == 0 ? 32 : 16;
    p.tiles_x = (w + TILE_W - 1) / TILE_W;
    p.tiles_y = (h + TILE_H - 1) / TILE_H;
    p.n_tiles = n * p.tiles_x * p.tiles_y;
    p.relu = relu;
    CUtensorMap xmap;
    // wide, thin 3x3 layers: row-tile kernel with a loaded-once halo and resident weights
    const uint32_t w_bytes = 9u * (uint32_t)cin * cout * 2u;
    if (taps == 9 && w >= ROW_M && w_bytes <= 96u * 1024u && nhwc_row_map(xmap, x, n, h, w, cin, p.ck))
    {
        const size_t w_region = (w_bytes + 1023) / 1024 * 1024, sb = row_stage_bytes(p.ck), tail = 16 * 8 + 16;
        int per_sm = 2;
        size_t stages = w_region + 2 * sb + 2 * 16 + tail <= 100 * 1024 ? (100 * 1024 - w_region - tail) / (sb + 16) : 0;
        if (stages < 2)
        {
            per_sm = 1;
            stages = (SMEM_BUDGET - w_region - tail) / (sb + 16);
        }
        p.stages = (int)std::min<size_t>(8, stages);
        if (p.stages >= 2)
        {
            if (head)
            {
                p.head_w = head->w;
                p.head_b = head->b;
                p.head_flow = head->flow;
                p.head_flow16 = static_cast<__half *>(head->flow16);
            }
            const size_t smem = w_region + (size_t)p.stages * sb + (2 * p.stages + 6) * 8 + 16;
            const int units = n * h * ((w + ROW_M - 1) / ROW_M);
            const int grid = std::min(units, sm_count() * per_sm);
            cudaError_t e = smem_limit(row_conv_kernel<0>, smem);
            if (e == cudaSuccess)
                e = launch_kernel(row_conv_kernel<0>, dim3((unsigned)grid), dim3(PCONV_THREADS), smem, stream, pdl, p, xmap);
            if (e == cudaSuccess && head && head_fused)
                *head_fused = true;
            return e == cudaSuccess ? ISTI_OK : cuda_fail(e, "isti_unet_conv launch");
        }
    }
    p.chunked_map = nhwc_chunked_map(xmap, x, n, h, w, cin, p.ck) ? 1 : 0;
    if (!p.chunked_map && (st = nhwc_map(xmap, x, n, h, w, cin)) != ISTI_OK)
        return st;
    // ring: about 100 KB, so that two CTAs share an SM; the ring runs across tiles
    const uint32_t sb = conv_stage_bytes(p.ck, cout);
    p.stages = (int)std::min<size_t>(16, std::max<size_t>(2, (100 * 1024) / sb));
    const size_t smem = (size_t)p.stages * sb + (2 * p.stages + 5) * 8 + 16;
    if (smem > SMEM_BUDGET)
        return isti::set_error(ISTI_ERR_INVALID_ARG, "isti_unet_conv: stage does not fit in shared memory");
    const uint32_t ncols = 2 * tmem_cols(cout);
    const int per_sm = std::max(1, std::min(2, (int)(512 / ncols)));
    const int grid = std::min(p.n_tiles, sm_count() * per_sm);
    cudaError_t e;
    if (taps == 9)
    {
        e = smem_limit(conv_kernel<9>, smem);
        if (e == cudaSuccess)
            e = launch_kernel(conv_kernel<9>, dim3((unsigned)grid), dim3(PCONV_THREADS), smem, stream, pdl, p, xmap);
    }
    else
    {
        e = smem_limit(conv_kernel<1>, smem);
        if (e == cudaSuccess)
            e = launch_kernel(conv_kernel<1>, dim3((unsigned)grid), dim3(PCONV_THREADS), smem, stream, pdl, p, xmap);
    }
    if (e == cudaSuccess)
        e = cudaGetLastError();
    return e == cudaSuccess ? ISTI_OK : cuda_fail(e, "isti_unet_conv launch");
}

int wgrad_splits(int taps, int n_tiles)
{
    // about four CTAs per SM over all taps, at least 8 pixel tiles each
    const int want = std::max(1, (152 * 4) / taps);
    return std::max(1, std::min(want, (n_tiles + 7) / 8));
}

size_t wgrad_scratch(int taps, int n, int h, int w, int cin, int cout)
{
    const int n_tiles = n * ((w + TILE_W - 1) / TILE_W) * ((h + TILE_H - 1) / TILE_H);
    return (size_t)wgrad_splits(taps, n_tiles) * cout * taps * cin * sizeof(float);
}

isti_status wgrad_launch(int taps, const void *dy, const void *x, int n, int h, int w, int cin, int cout, float *dw, int accumulate, void *scratch,
                         size_t scratch_bytes, int32_t *status, cudaStream_t stream)
{
    if ((taps != 9 && taps != 1) || n < 1 || h < 1 || w < 1 || cin % 16 || cout % 16 || cin < 16 || cin > 256 || cout > 128 || !dy || !x ||
        !dw || !scratch)
        return isti::set_error(ISTI_ERR_INVALID_ARG, "isti_unet_wgrad: bad shape or NULL buffer");
    if (scratch_bytes < wgrad_scratch(taps, n, h, w, cin, cout))
        return isti::set_error(ISTI_ERR_INVALID_ARG, "isti_unet_wgrad: scratch too small");
    isti_status st = status_word(status);
    if (st != ISTI_OK)
        return st;
    CUtensorMap dymap, xmap;
    if ((st = nhwc_map(dymap, dy, n, h, w, cout)) != ISTI_OK || (st = nhwc_map(xmap, x, n, h, w, cin)) != ISTI_OK)
        return st;
    WgradParams p{};
    p.partial = static_cast<float *>(scratch);
    p.status = status;
    p.w = w;
    p.h = h;
    p.b = n;
    p.cin = cin;
    p.cout = cout;
    p.tiles_x = (w + TILE_W - 1) / TILE_W;
    p.tiles_y = (h + TILE_H - 1) / TILE_H;
    p.n_tiles = n * p.tiles_x * p.tiles_y;
    const int splits = wgrad_splits(taps, p.n_tiles);
    p.tiles_per_split = (p.n_tiles + splits - 1) / splits;
    const uint32_t sb = wgrad_stage_bytes(cin);
    p.stages = (int)std::max<size_t>(2, std::min<size_t>(4, (160 * 1024) / sb));
    const size_t smem = (size_t)p.stages * sb + (2 * p.stages + 1) * 8 + 16;
    if (smem > SMEM_BUDGET)
        return isti::set_error(ISTI_ERR_INVALID_ARG, "isti_unet_wgrad: stage does not fit in shared memory");
    const dim3 grid((unsigned)splits, (unsigned)taps);
    cudaError_t e;
    if (taps == 9)
    {
        e = smem_limit(wgrad_kernel<9>, smem);
        if (e == cudaSuccess)
            wgrad_kernel<9><<<grid, CONV_THREADS, smem, stream>>>(p, dymap, xmap);
    }
    else
    {
        e = smem_limit(wgrad_kernel<1>, smem);
        if (e == cudaSuccess)
            wgrad_kernel<1><<<grid, CONV_THREADS, smem, stream>>>(p, dymap, xmap);
    }
    if (e == cudaSuccess)
    {
        const size_t nw = (size_t)cout * taps * cin;
        wgrad_reduce_kernel<<<(unsigned)((nw + 255) / 256), 256, 0, stream>>>(p.partial, splits, nw, dw, accumulate);
        e = cudaGetLastError();
    }
    return e == cudaSuccess ? ISTI_OK : cuda_fail(e, "isti_unet_wgrad launch");
}

isti_status pack_launch(int taps, const float *w, int cin, int cout, int transpose, void *wpack, cudaStream_t stream)
{
    if ((taps != 9 && taps != 1) || cin % 16 || cout % 16 || !w || !wpack)
        return isti::set_error(ISTI_ERR_INVALID_ARG, "isti_unet_pack: bad shape or NULL buffer");
    const int n = taps * cin * cout;
    pack_kernel<<<(n + 255) / 256, 256, 0, stream>>>(w, taps, cin, cout, transpose, static_cast<__nv_bfloat16 *>(wpack));
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? ISTI_OK : cuda_fail(e, "isti_unet_pack launch");
}
} // namespace isti_unet

extern "C" {

size_t isti_unet_packed_bytes(int32_t taps, int32_t cin, int32_t cout) { return (size_t)taps * cin * cout * 2u; }

isti_status isti_unet_pack(int32_t taps, const float *w, int32_t cin, int32_t cout, int32_t transpose, void *wpack, void *stream)
{
    return isti_unet::pack_launch(taps, w, cin, cout, transpose, wpack, static_cast<cudaStream_t>(stream));
}

isti_status isti_unet_conv(int32_t taps, const void *x, int32_t n, int32_t h, int32_t w, int32_t cin, const void *wpack, const float *bias,
                           const void *mask, int32_t relu, void *out, int32_t cout, int32_t *status, void *stream)
{
    return isti_unet::conv_launch(taps, x, n, h, w, cin, wpack, bias, mask, relu, out, cout, status, static_cast<cudaStream_t>(stream));
}

size_t isti_unet_wgrad_scratch_bytes(int32_t taps, int32_t n, int32_t h, int32_t w, int32_t cin, int32_t cout)
{
    return isti_unet::wgrad_scratch(taps, n, h, w, cin, cout);
}

isti_status isti_unet_wgrad(int32_t taps, const void *dy, const void *x, int32_t n, int32_t h, int32_t w, int32_t cin, int32_t cout,
                            float *dw, int32_t accumulate, void *scratch, size_t scratch_bytes, int32_t *status, void *stream)
{
    return isti_unet::wgrad_launch(taps, dy, x, n, h, w, cin, cout, dw, accumulate, scratch, scratch_bytes, status,
                                   static_cast<cudaStream_t>(stream));
}

} // extern "C"
