// Device code of the interpolation path: init, splat and bidirectional
// reprojection kernels (reference: src/renderer.cu of
// DerThomy/ImageBasedSpatioTemporalInterpolation).  Included by isti_render.cu,
// which holds the host side and the C ABI.
//
// A launch sequence renders a batch of 1..ISTI_MAX_BATCH_FRAMES client frames of
// one keyframe pair:
//  1. init:  every 64-bit splat key <- 0xfefe...fe (the reference's
//            cudaMemset(0xfe), src/renderer.cu:632-638), pixel->clip tables,
//            device status word <- 0;
//  2. splat: blockIdx.z = source view; per source pixel the keyframe part
//            (world positions, flow to the other keyframe, visibility in the main
//            view) once, then per frame the client-camera projection, flow store
//            and 64-bit atomicMin;
//  3. reprojection: a block covers 2 rows x 32 output pixels with one warp per
//            source view (view = threadIdx.y).  The block's splat-key tiles (every
//            view, a group of frames) are fetched into shared memory by TMA
//            (cp.async.bulk.tensor, one elected thread, mbarrier completion).
//            Phase 1: each thread runs window initialisation + iterative search +
//            reprojection error for its view and both rows, frame by frame.
//            Phase 2: the (frame, row) tasks are spread over the warps; each
//            chooses the direction per camera and the winning camera and computes
//            the colour (second chance, soft shadows) only for the result that is
//            written.  The reference colours every camera's result
//            (src/renderer.cu:378-396,436); only the written one is observable and
//            colour never feeds a choice, so the output is identical.  Phase 3
//            writes chained outputs.
#pragma once

#include "isti.h"
#include "isti_device.cuh"
#include "isti_error_cmp.cuh"

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstddef>

#include <utility>

namespace isti
{
constexpr int MAX_VIEWS = 2 + 2 * ISTI_MAX_AUX_CAMS;
constexpr int MAX_FRAMES = ISTI_MAX_BATCH_FRAMES;
constexpr int ROWS = 2; // output rows searched together by one reprojection thread
// Registers per reprojection thread (the kernel's register cap, a template argument).
// The kernel waits on dependent gathers, so resident warps matter more than registers:
// at 48 (no spills) a 6-view block of 192 threads fits 7 times into the register file
// (5 times at its natural 62), at 40 (a few spilled words) 8 times.  Measured at 1080p,
// 3 frames: for the 3x3 window 40 is faster with 4 or more views (4 views 0.441 -> 0.425
// ms, 6 views 0.590 -> 0.564 ms) and 48 with 2 (0.240 -> 0.239 ms, 56: 0.252); the 7x7
// window (mode 1) spills more and runs best at 56 (6 views: 40 1.203, 48 1.164, 56 1.153 ms).
constexpr int REPROJ_REGS = 48;
constexpr int REPROJ_REGS_MANY_VIEWS = 40;
constexpr int REPROJ_MANY_VIEWS = 4;
constexpr int REPROJ_REGS_WIDE_WINDOW = 56;

struct DevView
{
    const uint32_t *color; // RGBA8 packed, R in bits 0-7
    const float *z;
    const void *motion;
    const uint32_t *sha, *shb, *shi;
    unsigned long long *splat; // frame 0; frame k at + k * FrameParams::key_stride
    // The client-camera flow of each source pixel (full_motion_cam, src/renderer.cu:117), split
    // by use: (x, y), read at every search step, and the depth the reprojection derives from
    // its z, z_to_depth(z + dz) (src/renderer.cu:339), read once after the search.
    float2 *cam_xy;            // frame 0; frame k at + k * FrameParams::cam_stride
    float *cam_depth;          // frame 0; frame k at + k * FrameParams::depth_stride
    uint8_t *vis;              // visible_in_main per source pixel (the flow's w), shared by the frames
    float4 *full_ff;
    float *lut;                // pixel2CS tables: x at [0, w), y at [w, w + h)
    uint32_t w, h;
    uint32_t sx, sy;           // output pixels per view pixel (aux_idx = idx / s, src/renderer.cu:433)
    int32_t motion_fmt;
    int32_t forward;
    int32_t priority;
    float err_sx, err_sy;      // res / min(res.x, res.y), computeReprojError scale (src/renderer.cu:213)
    float inv_vp[16];          // this view's inverse viewproj
    float vp_to[16];           // the other keyframe's viewproj (same camera)
    float vp_main[16];         // main camera viewproj at this keyframe (visible_in_main test)
    float vp_self[16];         // this view's viewproj (timewarp)
};

// Per-frame settings (RenderInfo / AdditionalRenderInfo, include/renderer.h:18-35)
struct FrameCfg
{
    float alpha;
    int32_t fpa, sfpa, no_shadows;
};

// The views come last: a copy of the first params_prefix(n) bytes holds every field a
// launch over n views reads (the persistent kernel stages that much in shared memory, in
// 16-byte words).
struct alignas(16) FrameParams
{
    float cam_vp[MAX_FRAMES][16];
    float cam_ivp[MAX_FRAMES][16]; // client inverse viewproj (timewarp rays)
    double *tw_rows;               // timewarp: per-row sums of the forward keyframe's z
    float *tw_mean;                // timewarp: mean z (the reference's ImageBuffer::average)
    uint32_t *out[MAX_FRAMES];
    FrameCfg f[MAX_FRAMES];
    size_t key_stride; // elements between frames in the key block
    size_t cam_stride;   // float2 elements between frames in the cam-flow (x, y) block
    size_t depth_stride; // float elements between frames in the cam-flow depth block
    ulonglong2 *keys;  // the whole key block (16-byte units) for the init kernel
    size_t key_units;
    int32_t *status;   // device status word: 0 ok, ISTI_ERR_TIMEOUT after a bounded wait gave up
    uint32_t out_w, out_h;
    int32_t n_views, n_aux, n_frames, linear, chain;
    int32_t use_tma;          // key tiles fetched by TMA (every view's row pitch a multiple of 16 bytes)
    int32_t row_pairs;        // pairs of output rows per reprojection block
    // Failure-detection test hook: the reprojection block with this linear index
    // (blockIdx.y * gridDim.x + blockIdx.x) announces its tile bytes but issues no copy,
    // so its bounded wait runs out after `wait_limit` polls; -1 = none.  0 = default limit.
    // The host derives the index from an output pixel (withhold_x, withhold_y; -1 = none).
    int32_t withhold_block;
    uint32_t wait_limit;
    int32_t withhold_x, withhold_y;
    DevView v[MAX_VIEWS];
};

__host__ __device__ constexpr size_t params_prefix(int n_views)
{
    return (offsetof(FrameParams, v) + (size_t)n_views * sizeof(DevView) + 15) & ~(size_t)15;
}

// One 3-D tensor map per source view over its splat keys: (x, y, frame), u64 elements.
struct KeyMaps
{
    CUtensorMap m[MAX_VIEWS];
};

// ---- TMA / mbarrier (PTX) ----

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.b32 %0, 1, 0, p;\n}"
                 : "=r"(ok)
                 : "r"(smem_u32(bar)), "r"(parity)
                 : "memory");
    return ok != 0;
}

// The part of mbar_wait_bounded after its first limit ran out, out of line so that the
// common path keeps no registers for it: the status word is set and the wait is retried
// once more with the same limit (the copies may still be landing).
__device__ __noinline__ bool mbar_wait_late(unsigned long long *bar, uint32_t parity, int32_t *status, uint32_t lim)
{
    atomicExch(status, (int32_t)ISTI_ERR_TIMEOUT);
    for (uint32_t i = 0; i < lim; i++)
        if (mbar_try_wait(bar, parity))
            return true;
    return false;
}

// Waits for phase `parity` of the barrier with an iteration limit (0: the default of 2^22
// polls, seconds at most).  Returns false when the wait and its retry (mbar_wait_late) gave
// up: the tiles are then not to be read.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long *bar, uint32_t parity, int32_t *status, uint32_t limit)
{
    const uint32_t lim = limit ? limit : (1u << 22);
    for (uint32_t i = 0; i < lim; i++)
        if (mbar_try_wait(bar, parity))
            return true;
    return mbar_wait_late(bar, parity, status, lim);
}

// 3-D tiled bulk copy global -> shared, completion counted on `bar`.  x * 8 bytes must be a
// multiple of 16 (x even); x and y may be negative or past the end (zero fill).
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int x, int y, int z, unsigned long long *bar)
{
    asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
                     smem_u32(dst)),
                 "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
                 : "memory");
}

// ---- border-addressed loads: zero outside the image (cudaAddressModeBorder) ----

__device__ __forceinline__ float ld_f(const float *img, uint32_t x, uint32_t y, uint32_t w, uint32_t h)
{
    return (x < w && y < h) ? __ldg(img + (y * w + x)) : 0.0f;
}
__device__ __forceinline__ float4 ld_f4(const float4 *img, uint32_t x, uint32_t y, uint32_t w, uint32_t h)
{
    return (x < w && y < h) ? __ldg(img + (y * w + x)) : make_float4(0.f, 0.f, 0.f, 0.f);
}
__device__ __forceinline__ uint32_t ld_c(const uint32_t *img, uint32_t x, uint32_t y, uint32_t w, uint32_t h)
{
    return (x < w && y < h) ? __ldg(img + (y * w + x)) : 0u;
}

__device__ __forceinline__ float4 load_motion(const DevView &v, uint32_t idx)
{
    if (v.motion_fmt == ISTI_MOTION_F32X4)
        return __ldg(static_cast<const float4 *>(v.motion) + idx);
    if (v.motion_fmt == ISTI_MOTION_F16X3)
    {
        const __half *m = static_cast<const __half *>(v.motion) + 3 * (size_t)idx;
        return make_float4(__half2float(m[0]), __half2float(m[1]), __half2float(m[2]), 0.0f);
    }
    return make_float4(0.f, 0.f, 0.f, 0.f);
}

// pixel2CS of pixel (x, y) of view v from its tables; direct formula outside the image
template <class V>
__device__ __forceinline__ float2 view_pixel2cs(const V &v, uint32_t x, uint32_t y)
{
    if (x < v.w && y < v.h)
        return make_float2(__ldg(v.lut + x), __ldg(v.lut + v.w + y));
    return pixel2cs(x, y, v.w, v.h);
}

// ---- key initialisation (cudaMemset 0xfe, src/renderer.cu:632-638) + pixel->clip tables ----

// Thread t of `stride` threads: keys t, t + stride, ... and table entry t of every view
// (and, when asked, the status word).
__device__ __forceinline__ void init_part(const FrameParams &p, size_t t, size_t stride, bool reset_status = true)
{
    const ulonglong2 empty = make_ulonglong2(SPLAT_EMPTY, SPLAT_EMPTY);
    for (size_t i = t; i < p.key_units; i += stride)
        p.keys[i] = empty;
    if (t == 0 && reset_status)
        *p.status = 0;
    if (t < 65536)
        for (int k = 0; k < p.n_views; k++)
        {
            const DevView &v = p.v[k];
            if (t < v.w)
                v.lut[t] = pixel2cs((uint32_t)t, 0, v.w, 1).x;
            if (t < v.h)
                v.lut[v.w + t] = pixel2cs(0, (uint32_t)t, 1, v.h).y;
        }
}

__global__ void __launch_bounds__(256) init_kernel(const __grid_constant__ FrameParams p)
{
    init_part(p, (size_t)blockIdx.x * blockDim.x + threadIdx.x, (size_t)gridDim.x * blockDim.x);
}

// ---- computeFlowFields_sortedSplatting_kernel, src/renderer.cu:76-146 ----

// 8 blocks of 256 threads per SM (32 registers, a few spilled words): 64 resident warps
// instead of 56 at the natural 36 registers, 3-8 % faster (1080p, 3 frames, 2-6 views).
// One source pixel (x, y) of view `view`: the keyframe part, then every frame's client part.
__device__ __forceinline__ void splat_pixel(const FrameParams &p, int view, uint32_t x, uint32_t y)
{
    const DevView &v = p.v[view];
    if (x >= v.w || y >= v.h)
        return;
    const uint32_t idx = y * v.w + x;

    // keyframe part, independent of the client camera
    const float z_from = __ldg(v.z + idx);
    const float4 om = load_motion(v, idx);
    const float pcx = __ldg(v.lut + x), pcy = __ldg(v.lut + v.w + y); // pixel2CS(idx2D, resolution)
    const float4 cs_from = make_float4(pcx, pcy, z_from, 1.0f);
    const float4 ws_from = project(v.inv_vp, cs_from);
    const float4 moved = make_float4(xadd(pcx, om.x), xadd(pcy, om.y), xadd(z_from, om.z), 1.0f);
    const float4 ws_to = project(v.inv_vp, moved);

    // visible_in_main: WS2CS(posWS_from, viewproj_mat_from_main) inside +-(1 - 1e-3), src/renderer.cu:104-107
    const float4 cm = matvec(v.vp_main, ws_from);
    const float lim = 1.0f - 1e-3f;
    const bool visible = quotient_inside(cm.x, cm.w, lim) && quotient_inside(cm.y, cm.w, lim) && quotient_inside(cm.z, cm.w, lim);
    const float vis = visible ? 1.0f : 0.0f;

    const float4 cs_to = project(v.vp_to, ws_to);
    const float fmx = xsub(cs_to.x, cs_from.x), fmy = xsub(cs_to.y, cs_from.y), fmz = xsub(cs_to.z, cs_from.z);
    v.full_ff[idx] = make_float4(fmx, fmy, fmz, vis);
    v.vis[idx] = visible ? 1u : 0u;
    const float4 d_ws = make_float4(xsub(ws_to.x, ws_from.x), xsub(ws_to.y, ws_from.y), xsub(ws_to.z, ws_from.z),
                                    xsub(ws_to.w, ws_from.w));

    // client-camera part, per frame.  Unrolled over the batch limit, so the client matrix
    // p.cam_vp[k] is read as constant operands rather than by indexed loads (1080p, 3
    // frames, 6 views: 0.287 -> 0.270 ms; a switch on the view index for the same effect on
    // the view's matrices spills at 32 registers and was slower, 0.280 ms).
#pragma unroll
    for (int k = 0; k < MAX_FRAMES; k++)
    {
        if (k >= p.n_frames)
            break;
        const float wg = v.forward ? p.f[k].alpha : xsub(1.0f, p.f[k].alpha);
        unsigned long long *keys = v.splat + k * p.key_stride;
        float2 *cam = v.cam_xy + k * p.cam_stride;
        float *cdep = v.cam_depth + k * p.depth_stride;
        if (!p.linear)
        {
            const float4 scaled = make_float4(xadd(ws_from.x, xmul(wg, d_ws.x)), xadd(ws_from.y, xmul(wg, d_ws.y)),
                                              xadd(ws_from.z, xmul(wg, d_ws.z)), xadd(ws_from.w, xmul(wg, d_ws.w)));
            const float4 pc = project(p.cam_vp[k], scaled);
            cam[idx] = make_float2(xsub(pc.x, cs_from.x), xsub(pc.y, cs_from.y));
            // the reprojection's depth at this source pixel: its z plus the flow's dz, rounded
            // as the reference rounds them (the stored dz, then the sum)
            cdep[idx] = z_to_depth(xadd(z_from, xsub(pc.z, cs_from.z)));
            const float depth_cam = z_to_depth(pc.z);
            const int2 pix = cs2pixel(pc.x, pc.y, v.w, v.h);
            if (in_range(pix, v.w, v.h) && !(depth_cam < 0.0f))
                atomicMin(keys + ((uint32_t)pix.y * v.w + (uint32_t)pix.x), encode_key(depth_cam, x, y));
        }
        else
        {
            cam[idx] = make_float2(xmul(fmx, wg), xmul(fmy, wg));
            // the reference stores the product (the flow's dz) before the search adds it to z:
            // rounded on its own (never contracted into the addition), in either arithmetic
            cdep[idx] = z_to_depth(xadd(z_from, __fmul_rn(fmz, wg)));
            atomicMin(keys + idx, encode_key(z_to_depth(z_from), x, y));
        }
    }
}

__global__ void __launch_bounds__(256, 8) splat_kernel(const __grid_constant__ FrameParams p)
{
    splat_pixel(p, blockIdx.z, blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y * blockDim.y + threadIdx.y);
}

// ---- colour: colorFromShadow / secondChanceAndBlend_kernel, src/renderer.cu:217-327 ----

// The colour inputs of one source pixel of one view: colour and, when soft shadows apply,
// shadow info, then the shadow colours A/B where the levels need them, and the pixel's
// shadow levels (min / max over the shadow sub-frames and the initial level) computed
// once for every level index asked for.  Reads outside the view are zero (border
// addressing).
struct PixelShade
{
    uint32_t color, sha, shb;
    uint32_t bf;          // 24-bit level field (shadowInfo RGB, src/renderer.cu:241-242)
    int32_t init, mn, mx; // initial level, min and max over the sfpa sub-frames
    bool levels;          // colour B present and a non-zero level field
};

template <class V>
__device__ __forceinline__ PixelShade load_shade(const V &v, uint32_t px, uint32_t py, bool shadows, int32_t sfpa)
{
    PixelShade s;
    const bool in = px < v.w && py < v.h;
    const uint32_t idx = py * v.w + px;
    s.color = in ? __ldg(v.color + idx) : 0u;
    s.sha = s.shb = 0u;
    const uint32_t si = (shadows && in) ? __ldg(v.shi + idx) : 0u;
    s.bf = ((si & 255u) << 16) | (((si >> 8) & 255u) << 8) | ((si >> 16) & 255u);
    s.levels = shadows && v.shb != nullptr && s.bf != 0;
    s.init = (int32_t)(s.bf & SOFTSHADOW_VAL_MASK);
    s.mn = (int32_t)SOFTSHADOW_VAL_MASK;
    s.mx = 0;
    if (s.levels)
    {
        for (int32_t i = 0; i < sfpa; i++)
        {
            const int32_t lv = (int32_t)((s.bf >> (SOFTSHADOW_BITS * (uint32_t)i)) & SOFTSHADOW_VAL_MASK);
            s.mn = min(s.mn, lv);
            s.mx = max(s.mx, lv);
        }
        // colour A / B are read only where a level differs from the initial one
        // (colorFromShadow uses the pixel's own colour otherwise)
        if (s.mn != s.init)
            s.sha = __ldg(v.sha + idx);
        if (s.mx != s.init)
            s.shb = __ldg(v.shb + idx);
    }
    return s;
}

// colorFromShadow (level-index form), src/renderer.cu:217-268
__device__ __forceinline__ uint32_t color_from_shadow_idx(uint32_t sidx, int32_t sfpa, const PixelShade &s)
{
    if (sidx < (uint32_t)sfpa && sidx > 0 && s.levels)
    {
        const int32_t my_val = (int32_t)((s.bf >> (SOFTSHADOW_BITS * sidx)) & SOFTSHADOW_VAL_MASK);
        const float t = xdiv((float)(my_val - s.mn), (float)(s.mx - s.mn));
        const uint32_t cmin = s.mn == s.init ? s.color : s.sha;
        const uint32_t cmax = s.mx == s.init ? s.color : s.shb;
        // (float)(1.0 - (double)t): t is k / d with d in {1, 2, 3} (or NaN), for which the
        // double difference is exact, so one float subtraction rounds identically.
        const float omt = xsub(1.0f, t);
        uint32_t r = 255u << 24;
#pragma unroll
        for (int c = 0; c < 3; c++)
        {
            const float a = (float)((cmin >> (8 * c)) & 255u), b = (float)((cmax >> (8 * c)) & 255u);
            r |= cvt_u8(xadd(xmul(a, omt), xmul(b, t))) << (8 * c);
        }
        return r;
    }
    return s.color;
}

struct ShadowFrames
{
    uint32_t frame_idx, sfx, sfy;
    float sft;
};

// frame_idx / shadow sub-frames, src/renderer.cu:359-364
__device__ __forceinline__ ShadowFrames shadow_frames(const FrameCfg &c)
{
    ShadowFrames sf;
    const float fa = xmul((float)c.fpa, c.alpha);
    const float sa = xmul((float)c.sfpa, c.alpha);
    sf.frame_idx = __float2uint_rn(fa);
    sf.sfx = __float2uint_rd(xadd(sa, 1e-9f));
    sf.sfy = __float2uint_ru(xsub(sa, 1e-9f));
    sf.sft = xsub(sa, (float)sf.sfx);
    return sf;
}

// Whether colorFromShadow blends shadow levels for view v (src/renderer.cu:277).
template <class V>
__device__ __forceinline__ bool shadows_on(const ShadowFrames &sf, const FrameCfg &c, const V &v)
{
    return !(c.no_shadows || sf.sfx >= (uint32_t)c.sfpa || sf.sfy == 0 || v.sha == nullptr);
}

// colorFromShadow (two sub-frame form), src/renderer.cu:270-295, on loaded inputs
template <class V>
__device__ __forceinline__ uint32_t color_from_shadow(const ShadowFrames &sf, const FrameCfg &c, const V &v, bool on,
                                                      const PixelShade &s)
{
    if (!on)
        return s.color;
    const int32_t sfpa = c.sfpa;
    const uint32_t vx = (uint32_t)(v.forward ? (int32_t)sf.sfx : sfpa - (int32_t)sf.sfx);
    const uint32_t vy = (uint32_t)(v.forward ? (int32_t)sf.sfy : sfpa - (int32_t)sf.sfy);
    // single-index cases: vx when vx == vy or vy is out of range, else vy when vx is; one
    // code path for every lane (forward and backward views differ within a warp)
    const bool only_x = vx == vy || vy >= (uint32_t)sfpa;
    const bool single = only_x || vx >= (uint32_t)sfpa;
    const uint32_t a = color_from_shadow_idx(only_x || !single ? vx : vy, sfpa, s);
    if (single)
        return a;
    const uint32_t b = color_from_shadow_idx(vy, sfpa, s);
    return lerp_color_u8(a, b, sf.sft);
}

// secondChanceAndBlend_kernel<EPS_2>, src/renderer.cu:297-327.  Two rounds of loads: the
// source pixel's flow, z and colour inputs together, then at the projected pixel in the
// other keyframe its z, flow and colour inputs together (the colour is used only when the
// round trip is consistent).
template <class V>
__device__ uint32_t second_chance(float weight, const ShadowFrames &sf, const FrameCfg &c, uint32_t sx, uint32_t sy, const V &from,
                                  const V &to, float eps2)
{
    const bool on_from = shadows_on(sf, c, from);
    const float4 m_ft = ld_f4(from.full_ff, sx, sy, from.w, from.h);
    const float sz = ld_f(from.z, sx, sy, from.w, from.h);
    const PixelShade s_from = load_shade(from, sx, sy, on_from, c.sfpa);
    const float2 spcs = view_pixel2cs(from, sx, sy);
    const float pcx = xadd(spcs.x, m_ft.x), pcy = xadd(spcs.y, m_ft.y), pcz = xadd(sz, m_ft.z);
    const int2 pp = cs2pixel(pcx, pcy, to.w, to.h);

    uint32_t out = color_from_shadow(sf, c, from, on_from, s_from);
    if (sf.frame_idx >= (uint32_t)c.fpa)
        return out;
    if (in_range(pp, to.w, to.h))
    {
        const bool on_to = shadows_on(sf, c, to);
        const uint32_t pi = (uint32_t)pp.y * to.w + (uint32_t)pp.x;
        const float az = __ldg(to.z + pi);
        const float4 m_tf = __ldg(to.full_ff + pi);
        const PixelShade s_to = load_shade(to, (uint32_t)pp.x, (uint32_t)pp.y, on_to, c.sfpa);
        const float dx = xsub(m_ft.x, -m_tf.x), dy = xsub(m_ft.y, -m_tf.y), dz = xsub(m_ft.z, -m_tf.z);
        if (sqrt_less(xadd(xadd(xmul(dx, dx), xmul(dy, dy)), xmul(dz, dz)), EPS_3) &&
            fabsf(xsub(az, pcz)) < eps2)
            out = lerp_color_u8(color_from_shadow(sf, c, to, on_to, s_to), out, weight);
    }
    return out;
}

// ---- bidirectional reprojection, src/renderer.cu:148-465 ----

// One direction of one camera for one output pixel: window init + search + error.
// 12 bytes in shared memory.  The error is stored as a pattern of isti_error_cmp.cuh:
// squared (SQ, no square root per searched direction) or its rounded root; bit 31 carries
// visible_in_main.
struct DirRes
{
    uint32_t error_vis; // err_pack<SQ>(squared error), ERR_UNSEARCHED_OF<SQ> when not searched; bit 31 = visible_in_main
    float depth;        // searched depth, else the window-initialisation depth
    uint32_t src;       // source pixel, x << 16 | y
};

// Squared errors save the square root, but the freer schedule spills at 40 registers, where
// the roots are faster (1080p, 3 frames, 6 views: 0.537 ms roots, 0.548 squared; 2 views at
// 48 registers 0.238 -> 0.222 ms squared; 7x7 window at 56, 6 views 1.116 -> 1.092 ms).
template <int REGS>
constexpr bool SQUARED_ERRORS = !FAST_MATH && REGS != REPROJ_REGS_MANY_VIEWS;

template <bool SQ>
constexpr uint32_t ERR_EPS_1_FULL_RES = err_eps<SQ>(EPS_1_FULL_RES); // error < EPS_1 <=> pattern < this
template <bool SQ>
constexpr uint32_t ERR_EPS_1_LOW_RES = err_eps<SQ>(EPS_1_LOW_RES);

template <bool SQ>
__device__ __forceinline__ uint32_t pack_error_vis(float error2, bool vis)
{
    return err_pack<SQ>(error2) | (vis ? 0x80000000u : 0u);
}
__device__ __forceinline__ uint32_t dir_error(const DirRes &d) { return d.error_vis & 0x7fffffffu; }
__device__ __forceinline__ bool dir_vis(const DirRes &d) { return (d.error_vis >> 31) != 0u; }

// Result of bidirectionalReprojection for one camera (src/renderer.cu:366-397), without its colour.
struct CamRes
{
    bool valid;
    bool vis;
    bool blend;      // always-valid 50/50 blend of both directions
    int32_t priority;
    uint32_t error;  // squared error bits; indeterminate in the reference for the blend, 0 here
    float depth;
    int32_t dir;     // 0 forward keyframe, 1 backward keyframe
    uint32_t src;
};

// Shared-memory key tile of one view and frame: rows iy0 - SW .. iy0 + ROWS - 1 + SW and
// W columns from x = (tx0 - SW) rounded down to even (the TMA start-coordinate rule for
// 8-byte elements), covering the 32 + 2 * SW columns the window reads.
template <int SW>
struct Tile
{
    static constexpr int W = SW == 1 ? 36 : 40;
    static constexpr int H = ROWS + 2 * SW;
    static constexpr int ELEMS = W * H;
    static constexpr int BYTES = ELEMS * 8; // a multiple of 128: TMA destinations stay 128-byte aligned
};

__device__ __forceinline__ int tile_x0(uint32_t tx0, int sw) { return ((int)tx0 - sw) & ~1; }

// A reprojection block works through units = (frame, pair of output rows): n_frames x
// row_pairs of them.  Bytes at the start of its shared memory: the key tiles of one unit
// (every view) in phase 1, then (the tiles are dead by then) the chained colours and flags
// of phases 2-3.  A multiple of 128, so the results that follow stay aligned.
template <int SW>
__host__ __device__ constexpr size_t reproj_tile_region(int n_views, int n_units)
{
    const size_t tiles = (size_t)n_views * Tile<SW>::BYTES;
    const size_t chain = (size_t)n_units * ROWS * 32 * sizeof(uint32_t) * 2;
    return tiles > chain ? tiles : chain;
}

template <bool SQ>
__device__ __forceinline__ CamRes cam_result(const DirRes &f, const DirRes &b, const DevView &vf, const DevView &vb, uint32_t eps1, float eps2,
                                             bool always_valid)
{
    CamRes r;
    r.valid = false;
    r.vis = false;
    r.blend = false;
    r.priority = 0;
    r.error = 0u;
    r.depth = 0.0f;
    r.dir = 0;
    r.src = 0;
    const uint32_t fe = dir_error(f), be = dir_error(b);
    const bool fvis = dir_vis(f), bvis = dir_vis(b);
    const bool fok = err_below<SQ>(fe, eps1), bok = err_below<SQ>(be, eps1);
    if (fok || bok)
    {
        const bool both = fok && bok;
        const bool similar = fabsf(xsub(depth_to_z(f.depth), depth_to_z(b.depth))) < eps2;
        const bool choose_fwd = (both && !similar && f.depth < b.depth) || ((!both || similar) && err_less<SQ>(fe, be));
        r.valid = true;
        if (choose_fwd)
        {
            r.vis = fvis || (both && similar && bvis);
            r.priority = vf.priority;
            r.error = fe;
            r.depth = f.depth;
            r.dir = 0;
            r.src = f.src;
        }
        else
        {
            r.vis = bvis || (both && similar && fvis);
            r.priority = vb.priority;
            r.error = be;
            r.depth = b.depth;
            r.dir = 1;
            r.src = b.src;
        }
    }
    else if (always_valid)
    {
        r.valid = true;
        r.blend = true;
    }
    return r;
}

// Chooses among the cameras of one output pixel and returns the colour to
// write (false: keep the previous output), src/renderer.cu:400-465.
// res points at the [n_views][32] results of this pixel's row and frame.
template <bool MAV, bool SQ>
__device__ __forceinline__ bool resolve_pixel(const DirRes *res, int lane, const FrameParams &p, const FrameCfg &c, uint32_t &color)
{
    const CamRes m = cam_result<SQ>(res[lane], res[32 + lane], p.v[0], p.v[1], ERR_EPS_1_FULL_RES<SQ>, EPS_2_FULL_RES, MAV);
    CamRes best;
    best.valid = false;
    best.vis = false;
    best.priority = 0;
    best.error = 0u;
    best.depth = 0.0f;
    int best_cam = 0;
    const int n_cams = p.n_views / 2;
    for (int cam = 1; cam < n_cams; cam++)
    {
        const CamRes r = cam_result<SQ>(res[(2 * cam) * 32 + lane], res[(2 * cam + 1) * 32 + lane], p.v[2 * cam], p.v[2 * cam + 1],
                                        ERR_EPS_1_LOW_RES<SQ>, EPS_2_LOW_RES, false);
        bool take = !best.valid;
        if (best.valid && r.valid)
        {
            const bool similar = fabsf(xsub(depth_to_z(best.depth), depth_to_z(r.depth))) < EPS_2_LOW_RES;
            take = (!similar && r.depth < best.depth) || (similar && r.priority >= best.priority && err_less<SQ>(r.error, best.error));
        }
        if (take)
        {
            best = r;
            best_cam = cam;
        }
    }
    int cam = -1;
    CamRes fin = m;
    if (m.valid)
        cam = 0;
    if (best.valid)
    {
        bool choose_aux = !m.valid;
        if (m.valid && !best.vis)
        {
            const bool similar = fabsf(xsub(depth_to_z(best.depth), depth_to_z(m.depth))) < EPS_2_LOW_RES;
            choose_aux = !similar && best.depth < m.depth;
        }
        if (choose_aux)
        {
            cam = best_cam;
            fin = best;
        }
    }
    if (cam < 0)
        return false; // temporal hole filling: keep the previous output (src/renderer.cu:416-419,462-463)

    const ShadowFrames sf = shadow_frames(c);
    const float eps2 = cam == 0 ? EPS_2_FULL_RES : EPS_2_LOW_RES;
    const float oma = xsub(1.0f, c.alpha);
    if (MAV && fin.blend)
    {
        const DevView &vf = p.v[2 * cam], &vb = p.v[2 * cam + 1];
        const DirRes &f = res[lane], &b = res[32 + lane];
        const uint32_t cf = second_chance(oma, sf, c, f.src >> 16, f.src & 0xFFFFu, vf, vb, eps2);
        const uint32_t cb = second_chance(c.alpha, sf, c, b.src >> 16, b.src & 0xFFFFu, vb, vf, eps2);
        color = lerp_color_u8(cf, cb, 0.5f);
        return true;
    }
    // one call for either direction (the lanes of a warp choose different ones): from = the
    // chosen keyframe's view, to = the other one, weight 1 - t from the earlier keyframe
    const int dir = fin.dir;
    const DevView &from = p.v[2 * cam + dir], &to = p.v[2 * cam + 1 - dir];
    color = second_chance(dir == 0 ? oma : c.alpha, sf, c, fin.src >> 16, fin.src & 0xFFFFu, from, to, eps2);
    return true;
}

// Upper bound for the window comparison, from the depth bits l of the current lowest key.
// The reference replaces the lowest entry by a candidate c with c > 0 when
//   !isfinite(l) || l < 0 || c < l            (src/renderer.cu:167)
// For c > 0 (bits in [1, 0x7f800000], +inf included) this is c_bits < bound(l_bits):
//   l = +-inf, NaN, or negative non-zero  -> always true  -> bound 0xffffffff;
//   l = -0.0                              -> always false -> bound 0;
//   l in [+0, +max finite]                -> c < l, monotonic in the bits -> bound l_bits.
__device__ __forceinline__ uint32_t key_bound(uint32_t l)
{
    return l == 0x80000000u ? 0u : (l >= 0x7f800000u ? 0xffffffffu : l);
}

// initializeSearchFromSplatting<SW> on a shared-memory tile, src/renderer.cu:148-175, same
// scan order.  Tile row `row` holds the view row of this pixel; keys outside the view read
// as 0 (depth +0.0), which the window never selects, exactly like the reference's skipped
// out-of-range neighbours.  Returns the selected raw key.
template <int SW>
__device__ __forceinline__ unsigned long long window_key(const unsigned long long *tile, int row, int col)
{
    using T = Tile<SW>;
    unsigned long long best = tile[row * T::W + col];
    uint32_t bound = key_bound((uint32_t)(best >> 32));
#pragma unroll
    for (int yo = -SW; yo <= SW; yo++)
#pragma unroll
        for (int xo = -SW; xo <= SW; xo++)
        {
            const unsigned long long c = tile[(row + yo) * T::W + col + xo];
            const uint32_t cb = (uint32_t)(c >> 32);
            if (cb - 1u < 0x7f800000u && cb < bound) // c > 0 && (the reference's replacement test)
            {
                best = c;
                bound = key_bound(cb);
            }
        }
    return best;
}

// bidirectionalReprojection_kernel<SW, SI, MAIN_ALWAYS_VALID>, src/renderer.cu:400-465
// block = (32, n_views): 32 output columns x (2 * row_pairs) output rows, one warp per source
// view.  The block works through units (frame k, row pair): phase 1 runs one unit at a time
// on every warp; phases 2-3 spread the units' rows over the warps.  More row pairs per block
// (for single frames) keep every warp busy in phase 2.
// One reprojection block (bx, by) of frame batch p, executed by a block of (32, n_views)
// threads: the body of reproj_kernel, also run as a work unit of batch_kernel.  `maps`: the
// views' key-tile tensor maps; `bar`: the block's TMA completion barrier, initialised once per
// thread block; `round`: TMA rounds that barrier has completed so far (its phase carries over
// from unit to unit); `aborted`: a shared word, 0 when the block starts, that a thread whose
// wait for the key tiles gave up sets to 1; `block_id`: the index the test hook
// `withhold_block` refers to, compiled in only where HOOK is set.  Every thread returns
// together (early exits are block-uniform or come after the last barrier).
template <int SW, int SI, bool MAV, int REGS, bool HOOK = false>
__device__ __forceinline__ void reproj_block(const FrameParams &p, const CUtensorMap *maps, uint32_t bx, uint32_t by, uint32_t block_id,
                                             unsigned char *smem, unsigned long long &bar, int &round, volatile uint32_t &aborted)
{
    using T = Tile<SW>;
    const int nv = p.n_views, nf = p.n_frames, np = p.row_pairs, nu = nf * np;
    // [key tiles, phase 1 | chained colours and flags, phases 2-3 (same bytes)][results][barrier]
    unsigned long long *tiles = reinterpret_cast<unsigned long long *>(smem);                 // [nv][H][W]
    uint32_t *cols = reinterpret_cast<uint32_t *>(smem);                                      // [nu][ROWS][32]
    uint32_t *valid = cols + nu * ROWS * 32;                                                 // [nu][ROWS][32]
    DirRes *res = reinterpret_cast<DirRes *>(smem + reproj_tile_region<SW>(nv, nu));         // [nu][ROWS][nv][32]

    const int lane = threadIdx.x, vw = threadIdx.y;
    const uint32_t x0 = bx * 32, x = x0 + lane, yb = by * (ROWS * np);
    const bool xok = x < p.out_w;
    const bool leader = lane == 0 && vw == 0;
    const int round0 = round;
    {
        const DevView &v = p.v[vw];
        const uint32_t ix = v.sx == 1 ? x : x / v.sx, tx0 = v.sx == 1 ? x0 : x0 / v.sx;
        const bool fwd = (vw & 1) == 0;
        const int xs = tile_x0(tx0, SW);
        const int col = (int)ix - xs;
        // pixel2CS of the output pixels in the main view (the search target) and in this view (the error)
        const DevView &v0 = p.v[0];
        const uint32_t xc = min(x, p.out_w - 1);
        const float qx = __ldg(v0.lut + xc);
        const float pcx = __ldg(v.lut + min(ix, v.w - 1));
        const uint32_t vwid = v.w, vhei = v.h;
#pragma unroll 1
        for (int rp = 0; rp < np; rp++)
        {
            const uint32_t y0 = yb + (uint32_t)rp * ROWS; // the row pair's first output row
            const uint32_t iy0 = v.sy == 1 ? y0 : y0 / v.sy, iy1 = v.sy == 1 ? y0 + 1 : (y0 + 1) / v.sy;
            const bool rok[ROWS] = {xok && y0 < p.out_h, xok && y0 + 1 < p.out_h};
            const int wrow[ROWS] = {SW, (int)(iy1 - iy0) + SW}; // tile row of each output row's window centre
            const uint32_t y0c = min(y0, p.out_h - 1), y1c = min(y0 + 1, p.out_h - 1);
            const float qy[ROWS] = {__ldg(v0.lut + v0.w + y0c), __ldg(v0.lut + v0.w + y1c)};
            const float pcy[ROWS] = {__ldg(v.lut + v.w + min(iy0, vhei - 1)), __ldg(v.lut + v.w + min(iy1, vhei - 1))};
#pragma unroll 1
        for (int k = 0; k < nf; k++, round++)
        {
            const int u = k * np + rp;
            if (round > round0)
                __syncthreads(); // every warp is done with the previous unit's tiles
            bool arrived = true;
            if (p.use_tma)
            {
                // Once a wait of this block has given up (marked before the barrier above), the
                // leader issues no more rounds: its arrival on a barrier whose phase did not
                // complete would overrun the barrier's count.  The other waits then run out too
                // (bounded), and the block writes nothing.
                if (leader && aborted == 0u)
                {
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    mbar_expect_tx(&bar, (uint32_t)(nv * T::BYTES));
                    if (!HOOK || p.withhold_block != (int32_t)block_id)
                        for (int w = 0; w < nv; w++)
                        {
                            const DevView &vv = p.v[w];
                            const uint32_t wx0 = vv.sx == 1 ? x0 : x0 / vv.sx, wy0 = vv.sy == 1 ? y0 : y0 / vv.sy;
                            tma_load_3d(tiles + (size_t)w * T::ELEMS, &maps[w], tile_x0(wx0, SW), (int)wy0 - SW, k, &bar);
                        }
                }
                // a thread whose copies did not arrive reads none of the tiles and marks the block,
                // which then leaves after the barrier that ends phase 1, writing nothing (the
                // mark is written before that barrier and read after it, by every thread)
                arrived = mbar_wait_bounded(&bar, (uint32_t)(round & 1), p.status, p.wait_limit);
                if (!arrived)
                    aborted = 1u;
            }
            else
            {
                const unsigned long long *keys = v.splat + k * p.key_stride;
                unsigned long long *tg = tiles + (size_t)vw * T::ELEMS;
#pragma unroll
                for (int r = 0; r < T::H; r++)
                {
                    const uint32_t gy = iy0 - SW + r;
                    const bool row_ok = gy < vhei;
                    for (int c = lane; c < T::W; c += 32)
                    {
                        const uint32_t gx = (uint32_t)(xs + c);
                        tg[r * T::W + c] = (row_ok && gx < vwid) ? __ldg(keys + (gy * vwid + gx)) : 0ull;
                    }
                }
                __syncwarp();
            }
            if (arrived)
            {
                const unsigned long long *tg = tiles + (size_t)vw * T::ELEMS;
                const float2 *cam = v.cam_xy + k * p.cam_stride;
                const float *cdep = v.cam_depth + k * p.depth_stride;
                const bool search_ok = !fwd || p.f[k].alpha < 1.0f;
                bool s[ROWS];
                uint32_t ax[ROWS], ay[ROWS];
                float d_init[ROWS];
#pragma unroll
                for (int r = 0; r < ROWS; r++)
                {
                    const unsigned long long lo = window_key<SW>(tg, wrow[r], col);
                    d_init[r] = __uint_as_float((uint32_t)(lo >> 32));
                    ax[r] = ((uint32_t)lo) >> 16;
                    ay[r] = (uint32_t)lo & 0xFFFFu;
                    s[r] = rok[r] && search_ok && d_init[r] > 0.0f;
                    // a selected key with positive depth is a splat of an in-range source pixel;
                    // the clamp keeps every gather inside the view even if a tile were stale
                    if (s[r])
                    {
                        ax[r] = min(ax[r], vwid - 1u);
                        ay[r] = min(ay[r], vhei - 1u);
                    }
                    // the depth read after the search is mostly at or next to the start (a
                    // splatted source pixel, in range): fetch its line into L1 during the search
                    // (3x3 window, 6 views: 0.537 -> 0.533 ms; no gain for the 7x7 window)
                    if (SW == 1 && s[r])
                        asm volatile("prefetch.global.L1 [%0];" ::"l"(cdep + (ay[r] * vwid + ax[r])));
                }
                // iterativeSearch<SI>, src/renderer.cu:177-202, both rows interleaved.  The start is a
                // splatted source pixel and every accepted step is in range: no border handling needed.
#pragma unroll
                for (int i = 0; i < SI; i++)
                {
                    float2 m[ROWS];
#pragma unroll
                    for (int r = 0; r < ROWS; r++)
                        m[r] = s[r] ? __ldg(cam + (ay[r] * vwid + ax[r])) : make_float2(0.f, 0.f);
#pragma unroll
                    for (int r = 0; r < ROWS; r++)
                    {
                        const int2 t = cs2pixel(xsub(qx, m[r].x), xsub(qy[r], m[r].y), vwid, vhei);
                        if (s[r] && in_range(t, vwid, vhei))
                        {
                            ax[r] = (uint32_t)t.x;
                            ay[r] = (uint32_t)t.y;
                        }
                    }
                }
                // final flow, depth and computeReprojError, src/renderer.cu:338-341, 204-215
                float2 m[ROWS];
                float dz[ROWS], fx[ROWS], fy[ROWS];
                bool vs[ROWS];
#pragma unroll
                for (int r = 0; r < ROWS; r++)
                {
                    m[r] = make_float2(0.f, 0.f);
                    dz[r] = fx[r] = fy[r] = 0.f;
                    vs[r] = false;
                    if (s[r])
                    {
                        const uint32_t si = ay[r] * vwid + ax[r];
                        m[r] = __ldg(cam + si);
                        dz[r] = __ldg(cdep + si);
                        vs[r] = __ldg(v.vis + si) != 0;
                        fx[r] = __ldg(v.lut + ax[r]);
                        fy[r] = __ldg(v.lut + vwid + ay[r]);
                    }
                }
#pragma unroll
                for (int r = 0; r < ROWS; r++)
                {
                    DirRes d;
                    d.error_vis = ERR_UNSEARCHED_OF<SQUARED_ERRORS<REGS>>;
                    d.depth = d_init[r];
                    if (s[r])
                    {
                        d.depth = dz[r];
                        // the scale res / min(res) (src/renderer.cu:213): the host's IEEE quotient, or
                        // under the reference's GPU semantics its device division
                        const float esx = FAST_MATH ? xdiv((float)vwid, (float)min(vwid, vhei)) : v.err_sx;
                        const float esy = FAST_MATH ? xdiv((float)vhei, (float)min(vwid, vhei)) : v.err_sy;
                        const float ex = xmul(xsub(xadd(fx[r], m[r].x), pcx), esx);
                        const float ey = xmul(xsub(xadd(fy[r], m[r].y), pcy[r]), esy);
                        d.error_vis = pack_error_vis<SQUARED_ERRORS<REGS>>(xadd(xmul(ex, ex), xmul(ey, ey)), vs[r]);
                    }
                    d.src = (ax[r] << 16) | ay[r];
                    res[((u * ROWS + r) * nv + vw) * 32 + lane] = d;
                }
            }
        }
        }
    }
    __syncthreads();
    if (aborted)
        return;

    // phase 2: (unit, row) tasks over the warps
#pragma unroll 1
    for (int t = vw; t < nu * ROWS; t += nv)
    {
        const int u = t / ROWS, r = t % ROWS;
        // u = k * np + rp; np is 1..3 (the host's choice), so no general division
        const int k = np == 1 ? u : (np == 2 ? (u >> 1) : (np == 3 ? u / 3 : u / np));
        const uint32_t y = yb + (uint32_t)(u - k * np) * ROWS + r;
        uint32_t color = 0;
        const bool ok = xok && y < p.out_h && resolve_pixel<MAV, SQUARED_ERRORS<REGS>>(res + t * nv * 32, lane, p, p.f[k], color);
        if (!p.chain)
        {
            if (ok)
                p.out[k][y * p.out_w + x] = color;
        }
        else
        {
            cols[t * 32 + lane] = color;
            valid[t * 32 + lane] = ok ? 1u : 0u;
        }
    }
    if (!p.chain)
        return;
    __syncthreads();
    // phase 3: one persistent buffer per row, starting as out[0], copied to out[k] after frame k
    if (vw >= np * ROWS)
        return;
    const uint32_t y = yb + vw; // row vw of the block: row vw % ROWS of row pair vw / ROWS
    if (!xok || y >= p.out_h)
        return;
    uint32_t run = 0;
    for (int k = 0; k < nf; k++)
    {
        uint32_t *o = p.out[k] + (y * p.out_w + x);
        const int t = (k * np + vw / ROWS) * ROWS + vw % ROWS;
        if (k == 0)
            run = *o;
        if (valid[t * 32 + lane])
        {
            run = cols[t * 32 + lane];
            *o = run;
        }
        else if (k > 0)
            *o = run;
    }
}

// bidirectionalReprojection_kernel<SW, SI, MAIN_ALWAYS_VALID>, src/renderer.cu:400-465
// block = (32, n_views): 32 output columns x (2 * row_pairs) output rows, one warp per source
// view (reproj_block).
// HOOK: built with the failure-detection test hook (FrameParams::withhold_block); the
// launch uses that instance only when the hook is armed.
template <int SW, int SI, bool MAV, int REGS, bool HOOK = false>
__global__ void __maxnreg__(REGS) reproj_kernel(const __grid_constant__ FrameParams p, const __grid_constant__ KeyMaps km)
{
    // dynamic shared memory only (no static __shared__ in front of it): the key tiles start at
    // the 1 KiB-aligned window base, so every TMA destination is 128-byte aligned
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned long long &bar = *reinterpret_cast<unsigned long long *>(
        smem + reproj_tile_region<SW>(p.n_views, p.n_frames * p.row_pairs) +
        (size_t)p.n_frames * p.row_pairs * ROWS * p.n_views * 32 * sizeof(DirRes)); // TMA completion barrier
    volatile uint32_t &aborted = *reinterpret_cast<volatile uint32_t *>(&bar + 1);
    if (threadIdx.x == 0 && threadIdx.y == 0)
    {
        if (p.use_tma)
            mbar_init(&bar, 1);
        aborted = 0u;
    }
    __syncthreads();
    int round = 0;
    reproj_block<SW, SI, MAV, REGS, HOOK>(p, km.m, blockIdx.x, blockIdx.y, blockIdx.y * gridDim.x + blockIdx.x, smem, bar, round, aborted);
}

// ---- timewarp (mode 4), src/renderer.cu:467-522, 615-629 ----
//
// Mean NDC z of the forward keyframe (ImageBuffer::average, src/util/image_buffer.cu:80-100).
// The reference accumulates with a float atomicAdd in an unspecified order; here every row is
// summed left to right in double (one thread per row), the rows top to bottom in double, and
// the total is rounded to float and divided by the pixel count in float like the reference's
// final division.  The C oracle uses the same order.

__global__ void __launch_bounds__(128) timewarp_rowsum_kernel(const __grid_constant__ FrameParams p)
{
    const DevView &v = p.v[0];
    const uint32_t y = blockIdx.x * blockDim.x + threadIdx.x;
    if (y >= v.h)
        return;
    double acc = 0.0;
    for (uint32_t x = 0; x < v.w; x++)
        acc = __dadd_rn(acc, (double)__ldg(v.z + (y * v.w + x)));
    p.tw_rows[y] = acc;
}

__global__ void timewarp_mean_kernel(const __grid_constant__ FrameParams p)
{
    if (threadIdx.x != 0 || blockIdx.x != 0)
        return;
    const DevView &v = p.v[0];
    double acc = 0.0;
    for (uint32_t y = 0; y < v.h; y++)
        acc = __dadd_rn(acc, p.tw_rows[y]);
    *p.tw_mean = xdiv(__double2float_rn(acc), (float)(v.w * v.h));
    *p.status = 0;
}

__device__ __forceinline__ float dot3(float ax, float ay, float az, float bx, float by, float bz)
{
    return xadd(xadd(xmul(ax, bx), xmul(ay, by)), xmul(az, bz));
}

// timewarp_kernel body for one pixel and client camera; false: the ray is parallel to the plane (no write)
__device__ __forceinline__ bool timewarp_pixel(const float *cam_ivp, const DevView &to, const DevView &aux, bool has_aux, float depth_to,
                                               uint32_t x, uint32_t y, uint32_t out_w, uint32_t out_h, uint32_t &color)
{
    const float2 pcs = pixel2cs(x, y, out_w, out_h);
    const float4 nws = project(cam_ivp, make_float4(pcs.x, pcs.y, 0.0f, 1.0f));
    const float4 fws = project(cam_ivp, make_float4(pcs.x, pcs.y, 1.0f, 1.0f));
    // ray_dir = normalize(vec3(farWS - nearWS)), glm-subset normalize: v * (1 / sqrt(dot(v, v)))
    float dx = xsub(fws.x, nws.x), dy = xsub(fws.y, nws.y), dz = xsub(fws.z, nws.z);
    const float sd = xdiv(1.0f, xsqrt(dot3(dx, dy, dz, dx, dy, dz)));
    dx = xmul(dx, sd);
    dy = xmul(dy, sd);
    dz = xmul(dz, sd);
    // plane through inv_viewproj_mat_to[3] facing the centre of the keyframe at depth_to
    const float4 cws = project(to.inv_vp, make_float4(0.0f, 0.0f, depth_to, 1.0f));
    const float cpx = to.inv_vp[12], cpy = to.inv_vp[13], cpz = to.inv_vp[14], cpw = to.inv_vp[15];
    float nx = xsub(cws.x, cpx), ny = xsub(cws.y, cpy), nz = xsub(cws.z, cpz);
    const float nw = xsub(cws.w, cpw);
    const float sn = xdiv(1.0f, xsqrt(xadd(dot3(nx, ny, nz, nx, ny, nz), xmul(nw, nw)))); // 4-component normalize
    nx = xmul(nx, sn);
    ny = xmul(ny, sn);
    nz = xmul(nz, sn);
    const float denom = dot3(dx, dy, dz, nx, ny, nz);
    if (fabsf(denom) < 1e-6f)
        return false;
    const float t = xdiv(dot3(xsub(cpx, nws.x), xsub(cpy, nws.y), xsub(cpz, nws.z), nx, ny, nz), denom);
    const float4 hit = make_float4(xadd(nws.x, xmul(t, dx)), xadd(nws.y, xmul(t, dy)), xadd(nws.z, xmul(t, dz)), 1.0f);
    const float4 pc = project(to.vp_self, hit); // WS2CS(intersection, viewproj_mat_to)
    int2 pix = cs2pixel(pc.x, pc.y, to.w, to.h);
    const DevView *src = &to;
    if (!in_range(pix, to.w, to.h) && has_aux)
    {
        const float4 pa = project(aux.vp_self, hit);
        pix = cs2pixel(pa.x, pa.y, aux.w, aux.h);
        src = &aux;
    }
    pix.x = min(max(pix.x, 0), (int)src->w - 1);
    pix.y = min(max(pix.y, 0), (int)src->h - 1);
    color = __ldg(src->color + ((uint32_t)pix.y * src->w + (uint32_t)pix.x));
    return true;
}

// One thread per output pixel, looping over the frames of the batch (chained like the reprojection).
__global__ void __launch_bounds__(256) timewarp_kernel(const __grid_constant__ FrameParams p)
{
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= p.out_w || y >= p.out_h)
        return;
    const bool has_aux = p.n_aux > 0;
    const float depth_to = *p.tw_mean;
    uint32_t run = 0;
    for (int k = 0; k < p.n_frames; k++)
    {
        uint32_t color = 0;
        const bool ok = timewarp_pixel(p.cam_ivp[k], p.v[0], p.v[has_aux ? 2 : 0], has_aux, depth_to, x, y, p.out_w, p.out_h, color);
        uint32_t *o = p.out[k] + (y * p.out_w + x);
        if (!p.chain)
        {
            if (ok)
                *o = color;
            continue;
        }
        if (k == 0)
            run = *o;
        if (ok)
        {
            run = color;
            *o = run;
        }
        else if (k > 0)
            *o = run;
    }
}

// Unity depth (reversed, [0,1]) to NDC z in place: convertDepthToZ_kernel
// (src/file_reader.cu:17-37) with the reader's settings, d <- 1 - d, then
// d <- 2 d - 1 (2 d is exact, so the two roundings are those of the
// reference).  VEC: four pixels per thread with 16-byte accesses (z 16-byte
// aligned), the last n % 4 pixels one per thread.
__device__ __forceinline__ float unity_depth_to_z(float d) { return xsub(xmul(2.0f, xsub(1.0f, d)), 1.0f); }

template <bool VEC>
__global__ void depth_to_z_kernel(float *__restrict__ z, size_t n)
{
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    if (!VEC)
    {
        for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
            z[i] = unity_depth_to_z(z[i]);
        return;
    }
    const size_t n4 = n / 4;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += stride)
    {
        float4 v = reinterpret_cast<float4 *>(z)[i];
        v.x = unity_depth_to_z(v.x);
        v.y = unity_depth_to_z(v.y);
        v.z = unity_depth_to_z(v.z);
        v.w = unity_depth_to_z(v.w);
        reinterpret_cast<float4 *>(z)[i] = v;
    }
    const size_t tail = n4 * 4 + (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tail < n)
        z[tail] = unity_depth_to_z(z[tail]);
}

// Packed RGB8 -> RGBA8 with alpha 255.  VEC (src 4-byte and dst 16-byte aligned): a thread
// turns 3 source words (4 pixels, byte 0 = R of the first) into one 16-byte store.
template <bool VEC>
__global__ void rgb8_to_rgba8_kernel(uint32_t *__restrict__ dst, const uint8_t *__restrict__ src, size_t n)
{
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t groups = 0;
    if constexpr (VEC)
    {
        groups = n / 4;
        const uint32_t *s32 = reinterpret_cast<const uint32_t *>(src);
        for (size_t g = t; g < groups; g += stride)
        {
            const uint32_t w0 = __ldg(s32 + 3 * g), w1 = __ldg(s32 + 3 * g + 1), w2 = __ldg(s32 + 3 * g + 2);
            uint4 o;
            o.x = (w0 & 0xffffffu) | 0xff000000u;
            o.y = (w0 >> 24) | ((w1 & 0xffffu) << 8) | 0xff000000u;
            o.z = (w1 >> 16) | ((w2 & 0xffu) << 16) | 0xff000000u;
            o.w = (w2 >> 8) | 0xff000000u;
            reinterpret_cast<uint4 *>(dst)[g] = o;
        }
    }
    for (size_t i = groups * 4 + t; i < n; i += stride)
        dst[i] = (uint32_t)__ldg(src + 3 * i) | (uint32_t)__ldg(src + 3 * i + 1) << 8 | (uint32_t)__ldg(src + 3 * i + 2) << 16 | 0xff000000u;
}

// Sparse shadow entries -> the three RGBA8 shadow images (zeroed before): one thread per
// entry {pixel index, info RGB, A RGB, B RGB, pad} (16 bytes).
__global__ void unpack_shadows_kernel(uint32_t *__restrict__ info, uint32_t *__restrict__ a, uint32_t *__restrict__ b, size_t n_pixels,
                                      const uint4 *__restrict__ entries, size_t n_entries)
{
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n_entries; e += stride)
    {
        const uint4 v = __ldg(entries + e);
        if (v.x >= n_pixels)
            continue;
        // bytes 4..15: info R G B, A R G B, B R G B, pad (little-endian words y, z, w)
        info[v.x] = (v.y & 0xffffffu) | 0xff000000u;
        a[v.x] = (v.y >> 24) | ((v.z & 0xffffu) << 8) | 0xff000000u;
        b[v.x] = (v.z >> 16) | ((v.w & 0xffu) << 16) | 0xff000000u;
    }
}

// The pixels of sparse shadow entries <- 0 in the three shadow images.
__global__ void clear_shadows_kernel(uint32_t *__restrict__ info, uint32_t *__restrict__ a, uint32_t *__restrict__ b, size_t n_pixels,
                                     const uint4 *__restrict__ entries, size_t n_entries)
{
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n_entries; e += stride)
    {
        const uint32_t i = __ldg(&entries[e].x);
        if (i < n_pixels)
            info[i] = a[i] = b[i] = 0u;
    }
}

// Dynamic shared memory of one reprojection block of `n_units` units.
template <int SW>
constexpr size_t reproj_smem(int n_views, int n_units)
{
    return reproj_tile_region<SW>(n_views, n_units) + (size_t)n_units * ROWS * n_views * 32 * sizeof(DirRes) + 16; // + mbarrier, abort word
}
} // namespace isti
