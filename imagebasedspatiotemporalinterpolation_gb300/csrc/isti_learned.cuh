// Device code of the learned-initialisation render path (no counterpart in the
// reference, whose search always starts from splatting, src/renderer.cu:148-202).
// Included by isti_render.cu after isti_kernels.cuh (IEEE arithmetic).
//
// Per keyframe pair (main camera only):
//   keyframe_kernel   per source pixel of both keyframes, the part of the splat kernel
//                     that does not depend on the client camera: world position ws_from,
//                     its motion ws_to - ws_from, the flow to the other keyframe with the
//                     visibility flag (full_ff, as the plain path stores it), and the
//                     pixel->clip tables.
// Per client frame (batched over the frames of one call):
//   input_kernel      the network input at quarter resolution: inverse-depth and motion
//                     of both keyframes, t, and the client-camera flow of both keyframes'
//                     pixels, sampled at the centre (4q + 2) of each 4x4 block;
//   (the U-Net, isti_flownet.cu: per quarter-resolution pixel, the offset of the
//    converged source pixel in each keyframe)
//   learned_kernel    per output pixel and keyframe: start at x + 4 * offset, run the
//                     iterative search (src/renderer.cu:177-202) for the learned number of
//                     iterations with the client-camera flow computed on the fly from
//                     ws_from / ws_to, then the error, direction choice and colour of the
//                     plain path.  A block is one 32 x 8 tile: when any of its pixels is
//                     left without a converged direction (error >= EPS_1 in both
//                     keyframes) and its sources are not on the far plane (sky, which the
//                     plain method does not resolve either), the block writes nothing and
//                     marks the tile for the plain method;
//   fallback_*        the plain method for the marked tiles only: their keys reset to the
//                     empty value, every source pixel splatted whose target falls in a
//                     marked tile, then window initialisation + the plain iteration count
//                     + colour, exactly as the plain path computes them.  Every fallback
//                     kernel returns at once when no tile was marked.
#pragma once

#include "isti_kernels.cuh"

#include <cuda_bf16.h>

namespace isti
{
constexpr int LT_W = 32, LT_H = 8; // learned / fallback tile (one block)

struct LearnedParams
{
    FrameParams fp;             // views 0 (fwd) and 1 (bwd), frames, outputs, client matrices
    float4 *ws[2];              // per source pixel: ws_from (x, y, z, w)
    float4 *dws[2];             // per source pixel: ws_to - ws_from
    const __half *guess;        // [frame][hq][wq][4] source offsets (fwd dx, dy, bwd dx, dy), quarter pixels; null = none
    __nv_bfloat16 *net_in;      // [frame][hq][wq][16] network input
    int32_t hq, wq;             // network grid (multiples of 8, covering ceil(h / 4) x ceil(w / 4))
    int32_t learned_iters;
    int32_t tiles_x, tiles_y;
    uint32_t *tile_flags;       // [frame][tiles_y][tiles_x]: 1 = the plain method renders this tile
    int32_t *fallback_count;    // marked tiles (all frames)
    uint32_t *tile_list;        // the marked tiles' flag indices, fallback_count of them (any order)
    uint8_t *valid;             // [frame][h][w]: 1 where the frame wrote a pixel (chained outputs only)
    uint32_t *cell_bits;        // [frame][cells_y][cell_words]: FB_CELL-pixel square cells near a marked tile (fallback splat)
    int32_t cells_y, cell_words;
};

constexpr int FB_CELL = 8; // pixels per side of a fallback-splat rejection cell

// client-camera position of source pixel (sx, sy) of view v for frame k: the splat kernel's
// per-frame arithmetic (src/renderer.cu:110-116) on the stored keyframe part
__device__ __forceinline__ float4 learned_project(const LearnedParams &p, int v, int k, uint32_t sx, uint32_t sy)
{
    const DevView &dv = p.fp.v[v];
    const uint32_t i = sy * dv.w + sx;
    const float4 a = __ldg(p.ws[v] + i), d = __ldg(p.dws[v] + i);
    const float wg = dv.forward ? p.fp.f[k].alpha : xsub(1.0f, p.fp.f[k].alpha);
    const float4 scaled = make_float4(xadd(a.x, xmul(wg, d.x)), xadd(a.y, xmul(wg, d.y)), xadd(a.z, xmul(wg, d.z)), xadd(a.w, xmul(wg, d.w)));
    return project(p.fp.cam_vp[k], scaled);
}

// client-camera flow (xyz) of that pixel (full_motion_cam, src/renderer.cu:117), and its z in w
__device__ __forceinline__ float4 learned_camflow(const LearnedParams &p, int v, int k, uint32_t sx, uint32_t sy)
{
    const DevView &dv = p.fp.v[v];
    const float4 pc = learned_project(p, v, k, sx, sy);
    const float z = __ldg(dv.z + (sy * dv.w + sx));
    return make_float4(xsub(pc.x, __ldg(dv.lut + sx)), xsub(pc.y, __ldg(dv.lut + dv.w + sy)), xsub(pc.z, z), z);
}

// ---- per keyframe pair ----

__global__ void __launch_bounds__(256) keyframe_kernel(const __grid_constant__ LearnedParams p)
{
    const int v = blockIdx.z;
    const DevView &dv = p.fp.v[v];
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    const uint32_t t = threadIdx.y * blockDim.x + threadIdx.x;
    if (blockIdx.x == 0 && blockIdx.y == 0) // pixel->clip tables, as init_kernel writes them
        for (uint32_t j = t; j < dv.w + dv.h; j += blockDim.x * blockDim.y)
            dv.lut[j] = j < dv.w ? pixel2cs(j, 0, dv.w, 1).x : pixel2cs(0, j - dv.w, 1, dv.h).y;
    if (x >= dv.w || y >= dv.h)
        return;
    const uint32_t idx = y * dv.w + x;
    const float z_from = __ldg(dv.z + idx);
    const float4 om = load_motion(dv, idx);
    const float2 pcs = pixel2cs(x, y, dv.w, dv.h);
    const float4 cs_from = make_float4(pcs.x, pcs.y, z_from, 1.0f);
    const float4 ws_from = project(dv.inv_vp, cs_from);
    const float4 moved = make_float4(xadd(pcs.x, om.x), xadd(pcs.y, om.y), xadd(z_from, om.z), 1.0f);
    const float4 ws_to = project(dv.inv_vp, moved);
    const float4 cm = matvec(dv.vp_main, ws_from);
    const float lim = 1.0f - 1e-3f;
    const bool visible = quotient_inside(cm.x, cm.w, lim) && quotient_inside(cm.y, cm.w, lim) && quotient_inside(cm.z, cm.w, lim);
    const float4 cs_to = project(dv.vp_to, ws_to);
    dv.full_ff[idx] = make_float4(xsub(cs_to.x, cs_from.x), xsub(cs_to.y, cs_from.y), xsub(cs_to.z, cs_from.z), visible ? 1.0f : 0.0f);
    p.ws[v][idx] = ws_from;
    p.dws[v][idx] = make_float4(xsub(ws_to.x, ws_from.x), xsub(ws_to.y, ws_from.y), xsub(ws_to.z, ws_from.z), xsub(ws_to.w, ws_from.w));
}

// ---- per frame: the network input ----

__device__ __forceinline__ uint32_t bf16x2(float a, float b)
{
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t *>(&h);
}

__global__ void __launch_bounds__(256) input_kernel(const __grid_constant__ LearnedParams p)
{
    const int k = blockIdx.z;
    const int qx = blockIdx.x * blockDim.x + threadIdx.x, qy = blockIdx.y * blockDim.y + threadIdx.y;
    if (qx >= p.wq || qy >= p.hq)
        return;
    const DevView &a = p.fp.v[0], &b = p.fp.v[1];
    const uint32_t x = (uint32_t)(4 * qx + 2), y = (uint32_t)(4 * qy + 2);
    float f[16];
#pragma unroll
    for (int c = 0; c < 16; c++)
        f[c] = 0.0f;
    if (x < a.w && y < a.h)
    {
        const float sx = 0.125f * (float)a.w, sy = 0.125f * (float)a.h; // NDC -> quarter pixels
        const uint32_t i = y * a.w + x;
        const float za = __ldg(a.z + i), zb = __ldg(b.z + i);
        f[0] = 10.0f * (1.0f - za); // ~ 2 near / depth: inverse depth
        f[1] = 10.0f * (1.0f - zb);
        const float4 ma = load_motion(a, i), mb = load_motion(b, i);
        f[2] = ma.x * sx;
        f[3] = ma.y * sy;
        f[4] = 100.0f * ma.z;
        f[5] = mb.x * sx;
        f[6] = mb.y * sy;
        f[7] = 100.0f * mb.z;
        f[8] = p.fp.f[k].alpha;
        const float4 ca = learned_camflow(p, 0, k, x, y), cb = learned_camflow(p, 1, k, x, y);
        f[9] = isfinite(ca.x) ? ca.x * sx : 0.0f;
        f[10] = isfinite(ca.y) ? ca.y * sy : 0.0f;
        f[11] = isfinite(cb.x) ? cb.x * sx : 0.0f;
        f[12] = isfinite(cb.y) ? cb.y * sy : 0.0f;
    }
    uint4 *dst = reinterpret_cast<uint4 *>(p.net_in + (((size_t)k * p.hq + qy) * p.wq + qx) * 16);
    dst[0] = make_uint4(bf16x2(f[0], f[1]), bf16x2(f[2], f[3]), bf16x2(f[4], f[5]), bf16x2(f[6], f[7]));
    dst[1] = make_uint4(bf16x2(f[8], f[9]), bf16x2(f[10], f[11]), bf16x2(f[12], f[13]), bf16x2(f[14], f[15]));
}

// ---- per frame: learned search ----

// One direction's search from `start` with on-the-fly client flow: `iters` fixed-point steps
// (src/renderer.cu:177-202), then depth, error and visibility (src/renderer.cu:338-341).
template <bool SQ>
__device__ __forceinline__ DirRes learned_dir(const LearnedParams &p, int v, int k, uint32_t sx, uint32_t sy, int iters, float qx, float qy,
                                               float pcx, float pcy, float esx, float esy)
{
    const DevView &dv = p.fp.v[v];
    for (int i = 0; i < iters; i++)
    {
        const float4 m = learned_camflow(p, v, k, sx, sy);
        const int2 t = cs2pixel(xsub(qx, m.x), xsub(qy, m.y), dv.w, dv.h);
        if (in_range(t, dv.w, dv.h))
        {
            sx = (uint32_t)t.x;
            sy = (uint32_t)t.y;
        }
    }
    const float4 m = learned_camflow(p, v, k, sx, sy);
    const float vis = __ldg(dv.full_ff + (sy * dv.w + sx)).w;
    DirRes d;
    d.depth = z_to_depth(xadd(m.w, m.z));
    const float ex = xmul(xsub(xadd(__ldg(dv.lut + sx), m.x), pcx), esx);
    const float ey = xmul(xsub(xadd(__ldg(dv.lut + dv.w + sy), m.y), pcy), esy);
    d.error_vis = pack_error_vis<SQ>(xadd(xmul(ex, ex), xmul(ey, ey)), vis > 0.0f);
    d.src = (sx << 16) | sy;
    return d;
}

// Direction choice and colour of a main-camera-only pixel (resolve_pixel without aux cameras).
template <bool SQ>
__device__ __forceinline__ bool learned_resolve(const LearnedParams &p, int k, const DirRes &f, const DirRes &b, uint32_t &color)
{
    const CamRes m = cam_result<SQ>(f, b, p.fp.v[0], p.fp.v[1], ERR_EPS_1_FULL_RES<SQ>, EPS_2_FULL_RES, false);
    if (!m.valid)
        return false;
    const FrameCfg &c = p.fp.f[k];
    const ShadowFrames sf = shadow_frames(c);
    const DevView &from = p.fp.v[m.dir], &to = p.fp.v[1 - m.dir];
    color = second_chance(m.dir == 0 ? xsub(1.0f, c.alpha) : c.alpha, sf, c, m.src >> 16, m.src & 0xFFFFu, from, to, EPS_2_FULL_RES);
    return true;
}

constexpr bool LEARNED_SQ = true; // squared errors (as the plain path's 2-view launch)

// Next search position from an approximate client-camera flow (contracted multiply-adds, fast
// division): the intermediate steps of the learned search only choose the next pixel; the
// final step, whose error, depth and colour are kept, is exact.
__device__ __forceinline__ void learned_step_approx(const LearnedParams &p, int v, int k, float qx, float qy, uint32_t &sx, uint32_t &sy)
{
    const DevView &dv = p.fp.v[v];
    const uint32_t i = sy * dv.w + sx;
    const float4 a = __ldg(p.ws[v] + i), d = __ldg(p.dws[v] + i);
    const float wg = dv.forward ? p.fp.f[k].alpha : 1.0f - p.fp.f[k].alpha;
    const float *m = p.fp.cam_vp[k];
    const float x = fmaf(wg, d.x, a.x), y = fmaf(wg, d.y, a.y), z = fmaf(wg, d.z, a.z), w = fmaf(wg, d.w, a.w);
    const float cx = fmaf(m[0], x, fmaf(m[4], y, fmaf(m[8], z, m[12] * w)));
    const float cy = fmaf(m[1], x, fmaf(m[5], y, fmaf(m[9], z, m[13] * w)));
    const float cw = fmaf(m[3], x, fmaf(m[7], y, fmaf(m[11], z, m[15] * w)));
    const float mx = __fdividef(cx, cw) - __ldg(dv.lut + sx), my = __fdividef(cy, cw) - __ldg(dv.lut + dv.w + sy);
    const int2 t = cs2pixel(qx - mx, qy - my, dv.w, dv.h);
    if (in_range(t, dv.w, dv.h))
    {
        sx = (uint32_t)t.x;
        sy = (uint32_t)t.y;
    }
}

// One thread per output pixel handles every frame of the call (a pixel's sources for the
// frames lie close together: the keyframe data stay in L1), both keyframes interleaved.
// 6 blocks of 256 threads per SM (40 registers, no spills) instead of 5 at the natural 48:
// the kernel waits on dependent gathers, so resident warps count
__global__ void __launch_bounds__(LT_W *LT_H, 6) learned_kernel(const __grid_constant__ LearnedParams p)
{
    const uint32_t x = blockIdx.x * LT_W + threadIdx.x, y = blockIdx.y * LT_H + threadIdx.y;
    const bool inb = x < p.fp.out_w && y < p.fp.out_h;
    const DevView &a = p.fp.v[0], &b = p.fp.v[1];
    const float qx = inb ? __ldg(a.lut + x) : 0.0f, qy = inb ? __ldg(a.lut + a.w + y) : 0.0f; // pixel2CS of the output pixel
    const uint32_t qxi = min(x / 4, (uint32_t)p.wq - 1), qyi = min(y / 4, (uint32_t)p.hq - 1);
    for (int k = 0; k < p.fp.n_frames; k++)
    {
        bool fail = false, ok = false;
        uint32_t color = 0;
        if (inb)
        {
            float g[4] = {0.f, 0.f, 0.f, 0.f};
            if (p.guess)
            {
                const uint2 gg = *reinterpret_cast<const uint2 *>(p.guess + (((size_t)k * p.hq + qyi) * p.wq + qxi) * 4);
                const float2 g0 = __half22float2(*reinterpret_cast<const __half2 *>(&gg.x));
                const float2 g1 = __half22float2(*reinterpret_cast<const __half2 *>(&gg.y));
                g[0] = g0.x, g[1] = g0.y, g[2] = g1.x, g[3] = g1.y;
            }
            const bool search[2] = {p.fp.f[k].alpha < 1.0f, true}; // src/renderer.cu:336
            uint32_t sx[2], sy[2];
#pragma unroll
            for (int v = 0; v < 2; v++)
            {
                const DevView &dv = p.fp.v[v];
                float fx = (float)x + 4.0f * g[2 * v], fy = (float)y + 4.0f * g[2 * v + 1];
                fx = isfinite(fx) ? fminf(fmaxf(fx, 0.0f), (float)(dv.w - 1)) : (float)x;
                fy = isfinite(fy) ? fminf(fmaxf(fy, 0.0f), (float)(dv.h - 1)) : (float)y;
                sx[v] = (uint32_t)__float2int_rn(fx);
                sy[v] = (uint32_t)__float2int_rn(fy);
            }
            for (int it = 0; it < p.learned_iters; it++)
            {
#pragma unroll
                for (int v = 0; v < 2; v++)
                    if (search[v])
                        learned_step_approx(p, v, k, qx, qy, sx[v], sy[v]);
            }
            DirRes d[2];
#pragma unroll
            for (int v = 0; v < 2; v++)
            {
                d[v].error_vis = ERR_UNSEARCHED_OF<LEARNED_SQ>;
                d[v].depth = 0.0f;
                d[v].src = (sx[v] << 16) | sy[v];
                if (search[v])
                    d[v] = learned_dir<LEARNED_SQ>(p, v, k, sx[v], sy[v], 0, qx, qy, qx, qy, a.err_sx, a.err_sy);
            }
            const bool conv0 = err_below<LEARNED_SQ>(dir_error(d[0]), ERR_EPS_1_FULL_RES<LEARNED_SQ>);
            const bool conv1 = err_below<LEARNED_SQ>(dir_error(d[1]), ERR_EPS_1_FULL_RES<LEARNED_SQ>);
            if (!conv0 && !conv1)
            {
                // sources on the far plane (z = 1: sky) in both keyframes are left to the temporal
                // hole filling, as the plain method mostly leaves them
                const float z0 = __ldg(a.z + (sy[0] * a.w + sx[0]));
                const float z1 = __ldg(b.z + (sy[1] * b.w + sx[1]));
                fail = !(z0 >= 1.0f && z1 >= 1.0f);
            }
            else
                ok = learned_resolve<LEARNED_SQ>(p, k, d[0], d[1], color);
        }
        if (p.learned_iters < 0)
            fail = true; // every tile to the plain method (checks the fallback against the plain path)
        const uint32_t flag_idx = ((uint32_t)k * p.tiles_y + blockIdx.y) * p.tiles_x + blockIdx.x;
        if (__syncthreads_or(fail ? 1 : 0))
        {
            if (threadIdx.x == 0 && threadIdx.y == 0)
            {
                p.tile_flags[flag_idx] = 1u;
                p.tile_list[atomicAdd(p.fallback_count, 1)] = flag_idx;
            }
            continue;
        }
        if (threadIdx.x == 0 && threadIdx.y == 0)
            p.tile_flags[flag_idx] = 0u;
        if (ok)
            p.fp.out[k][y * p.fp.out_w + x] = color;
        if (p.fp.chain && inb)
            p.valid[((size_t)k * p.fp.out_h + y) * p.fp.out_w + x] = ok ? 1 : 0;
    }
}

// ---- fallback: the plain method for the marked tiles ----
//
// The window initialisation of a marked tile's edge pixels reads keys one pixel outside the
// tile, so the fallback keeps exact keys for the marked tiles and a ring of FB_RING pixels
// around each: both are reset to the empty value and receive every source pixel that splats
// into them.  Keys elsewhere are never read.
constexpr int FB_RING = 1;

// Whether a marked tile of frame k lies within m pixels (either axis) of pixel (x, y), which
// may lie outside the image (the box is clipped to it).
__device__ __forceinline__ bool marked_within(const LearnedParams &p, int k, int x, int y, int m)
{
    const int x0 = max(0, x - m), x1 = min((int)p.fp.out_w - 1, x + m);
    const int y0 = max(0, y - m), y1 = min((int)p.fp.out_h - 1, y + m);
    if (x0 > x1 || y0 > y1)
        return false;
    for (int ty = y0 / LT_H; ty <= y1 / LT_H; ty++)
        for (int tx = x0 / LT_W; tx <= x1 / LT_W; tx++)
            if (__ldg(p.tile_flags + ((size_t)k * p.tiles_y + ty) * p.tiles_x + tx) != 0u)
                return true;
    return false;
}

// The frame and first pixel of a marked tile from its flag index.
__device__ __forceinline__ void tile_origin(const LearnedParams &p, uint32_t flag_idx, int &k, int &x0, int &y0)
{
    const uint32_t per_frame = (uint32_t)(p.tiles_x * p.tiles_y);
    k = (int)(flag_idx / per_frame);
    const uint32_t t = flag_idx % per_frame;
    x0 = (int)(t % (uint32_t)p.tiles_x) * LT_W;
    y0 = (int)(t / (uint32_t)p.tiles_x) * LT_H;
}

// This thread's pixel of a marked tile.
__device__ __forceinline__ void tile_of(const LearnedParams &p, uint32_t flag_idx, int &k, uint32_t &x, uint32_t &y)
{
    int x0, y0;
    tile_origin(p, flag_idx, k, x0, y0);
    x = (uint32_t)x0 + threadIdx.x;
    y = (uint32_t)y0 + threadIdx.y;
}

// Margin of the fallback splat's approximate rejection: the ring plus 2 pixels for the
// approximate projection's error (orders of magnitude below that).
constexpr int FB_MARGIN = FB_RING + 2;

// keys of every marked tile and its ring <- the empty value (both views), and the rejection
// cells within FB_MARGIN pixels of the tile marked.  A small grid walks the list of marked
// tiles (blocks of LT_W x LT_H threads, one tile per iteration); rings and cells shared with a
// neighbour are written twice with the same value.
__global__ void __launch_bounds__(LT_W *LT_H) fallback_init_kernel(const __grid_constant__ LearnedParams p)
{
    constexpr int RW = LT_W + 2 * FB_RING, RH = LT_H + 2 * FB_RING;
    const int n = *p.fallback_count;
    const int cells_x = ((int)p.fp.out_w + FB_CELL - 1) / FB_CELL;
    for (int i = blockIdx.x; i < n; i += gridDim.x)
    {
        int k, x0, y0;
        tile_origin(p, __ldg(p.tile_list + i), k, x0, y0);
        const int t = threadIdx.y * LT_W + threadIdx.x;
        {
            // cells overlapping [x0 - FB_MARGIN, x0 + LT_W + FB_MARGIN) x [y0 - FB_MARGIN, y0 + LT_H + FB_MARGIN)
            const int cx0 = max(0, (x0 - FB_MARGIN) / FB_CELL), cx1 = min(cells_x - 1, (x0 + LT_W + FB_MARGIN - 1) / FB_CELL);
            const int cy0 = max(0, (y0 - FB_MARGIN) / FB_CELL), cy1 = min(p.cells_y - 1, (y0 + LT_H + FB_MARGIN - 1) / FB_CELL);
            const int ncx = cx1 - cx0 + 1;
            if (t < ncx * (cy1 - cy0 + 1))
            {
                const int cx = cx0 + t % ncx, cy = cy0 + t / ncx;
                atomicOr(p.cell_bits + ((size_t)k * p.cells_y + cy) * p.cell_words + cx / 32, 1u << (cx % 32));
            }
        }
        for (int j = t; j < RW * RH; j += LT_W * LT_H)
        {
            const int x = x0 - FB_RING + j % RW, y = y0 - FB_RING + j / RW;
            if (x < 0 || y < 0 || x >= (int)p.fp.out_w || y >= (int)p.fp.out_h)
                continue;
            for (int v = 0; v < 2; v++)
                p.fp.v[v].splat[k * p.fp.key_stride + (uint32_t)y * p.fp.v[v].w + (uint32_t)x] = SPLAT_EMPTY;
        }
    }
}

// Every source pixel whose client-camera target lies in a marked tile or its ring: atomicMin
// of its key (computeFlowFields_sortedSplatting_kernel, src/renderer.cu:110-145).  One thread
// per source pixel and view handles every frame (the keyframe part is read once).  An
// approximate projection (contracted multiply-adds, fast division) first rejects targets
// farther than 2 pixels beyond every tile's ring -- its error is orders of magnitude below
// that margin; a w near zero or a non-finite value is never rejected -- and only candidates
// take the exact projection of the plain path.
__global__ void __launch_bounds__(256) fallback_splat_kernel(const __grid_constant__ LearnedParams p)
{
    if (*p.fallback_count == 0)
        return;
    const int v = blockIdx.z;
    const DevView &dv = p.fp.v[v];
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= dv.w || y >= dv.h)
        return;
    const uint32_t i = y * dv.w + x;
    const float4 a = __ldg(p.ws[v] + i), d = __ldg(p.dws[v] + i);
    for (int k = 0; k < p.fp.n_frames; k++)
    {
        const float *m = p.fp.cam_vp[k];
        const float wg = dv.forward ? p.fp.f[k].alpha : xsub(1.0f, p.fp.f[k].alpha);
        // approximate target pixel
        const float sx = fmaf(wg, d.x, a.x), sy = fmaf(wg, d.y, a.y), sz = fmaf(wg, d.z, a.z), sw = fmaf(wg, d.w, a.w);
        const float qx = fmaf(m[0], sx, fmaf(m[4], sy, fmaf(m[8], sz, m[12] * sw)));
        const float qy = fmaf(m[1], sx, fmaf(m[5], sy, fmaf(m[9], sz, m[13] * sw)));
        const float qw = fmaf(m[3], sx, fmaf(m[7], sy, fmaf(m[11], sz, m[15] * sw)));
        bool candidate = true;
        if (isfinite(qx) && isfinite(qy) && fabsf(qw) > 1e-6f)
        {
            const float fx = (__fdividef(qx, qw) + 1.0f) * (float)dv.w * 0.5f, fy = (__fdividef(qy, qw) + 1.0f) * (float)dv.h * 0.5f;
            if (isfinite(fx) && isfinite(fy))
            {
                // a marked tile within FB_MARGIN pixels of (ix, iy) (the box clipped to the image) is
                // within FB_MARGIN of the nearest pixel of the image too, whose cell is then marked:
                // the cell test keeps every candidate the box test would keep
                const int ix = (int)floorf(fminf(fmaxf(fx, -1e6f), 1e6f)), iy = (int)floorf(fminf(fmaxf(fy, -1e6f), 1e6f));
                if (ix < -FB_MARGIN || iy < -FB_MARGIN || ix >= (int)dv.w + FB_MARGIN || iy >= (int)dv.h + FB_MARGIN)
                    candidate = false;
                else
                {
                    const int cx = min(max(ix, 0), (int)dv.w - 1) / FB_CELL, cy = min(max(iy, 0), (int)dv.h - 1) / FB_CELL;
                    candidate = (__ldg(p.cell_bits + ((size_t)k * p.cells_y + cy) * p.cell_words + cx / 32) >> (cx % 32)) & 1u;
                }
            }
        }
        if (!candidate)
            continue;
        const float4 pc = learned_project(p, v, k, x, y);
        const float depth_cam = z_to_depth(pc.z);
        const int2 pix = cs2pixel(pc.x, pc.y, dv.w, dv.h);
        if (!in_range(pix, dv.w, dv.h) || depth_cam < 0.0f || !marked_within(p, k, pix.x, pix.y, FB_RING))
            continue;
        atomicMin(dv.splat + k * p.fp.key_stride + ((uint32_t)pix.y * dv.w + (uint32_t)pix.x), encode_key(depth_cam, x, y));
    }
}

// window initialisation on global keys (initializeSearchFromSplatting<1>, src/renderer.cu:148-175)
__device__ __forceinline__ unsigned long long window_key_global(const unsigned long long *keys, uint32_t w, uint32_t h, uint32_t x, uint32_t y)
{
    unsigned long long best = keys[y * w + x];
    uint32_t bound = key_bound((uint32_t)(best >> 32));
    for (int yo = -1; yo <= 1; yo++)
        for (int xo = -1; xo <= 1; xo++)
        {
            const uint32_t xx = x + xo, yy = y + yo;
            if (xx >= w || yy >= h)
                continue;
            const unsigned long long c = keys[yy * w + xx];
            const uint32_t cb = (uint32_t)(c >> 32);
            if (cb - 1u < 0x7f800000u && cb < bound)
            {
                best = c;
                bound = key_bound(cb);
            }
        }
    return best;
}

__global__ void __launch_bounds__(LT_W *LT_H) fallback_reproj_kernel(const __grid_constant__ LearnedParams p)
{
    const int n = *p.fallback_count;
    const DevView &a = p.fp.v[0];
    for (int i = blockIdx.x; i < n; i += gridDim.x)
    {
        int k;
        uint32_t x, y;
        tile_of(p, __ldg(p.tile_list + i), k, x, y);
        if (x >= p.fp.out_w || y >= p.fp.out_h)
            continue;
        const float qx = __ldg(a.lut + x), qy = __ldg(a.lut + a.w + y);
        DirRes d[2];
#pragma unroll
        for (int v = 0; v < 2; v++)
        {
            const DevView &dv = p.fp.v[v];
            const unsigned long long lo = window_key_global(dv.splat + k * p.fp.key_stride, dv.w, dv.h, x, y);
            d[v].depth = __uint_as_float((uint32_t)(lo >> 32));
            d[v].src = (uint32_t)lo;
            d[v].error_vis = ERR_UNSEARCHED_OF<LEARNED_SQ>;
            const bool search_ok = v == 1 || p.fp.f[k].alpha < 1.0f;
            if (search_ok && d[v].depth > 0.0f)
                d[v] = learned_dir<LEARNED_SQ>(p, v, k, min(((uint32_t)lo) >> 16, dv.w - 1u), min((uint32_t)lo & 0xFFFFu, dv.h - 1u), 3, qx, qy,
                                               qx, qy, dv.err_sx, dv.err_sy);
        }
        uint32_t color = 0;
        const bool ok = learned_resolve<LEARNED_SQ>(p, k, d[0], d[1], color);
        if (ok)
            p.fp.out[k][y * p.fp.out_w + x] = color;
        if (p.fp.chain)
            p.valid[((size_t)k * p.fp.out_h + y) * p.fp.out_w + x] = ok ? 1 : 0;
    }
}

// Chained outputs (isti_render_batch's chain_outputs semantics): one persistent buffer per
// pixel that starts as out[0]'s content, takes each frame's written value and is copied to
// out[k] after frame k.
__global__ void __launch_bounds__(256) learned_chain_kernel(const __grid_constant__ LearnedParams p)
{
    const size_t n = (size_t)p.fp.out_w * p.fp.out_h;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    {
        uint32_t run = p.fp.out[0][i];
        for (int k = 1; k < p.fp.n_frames; k++)
        {
            if (p.valid[(size_t)k * n + i])
                run = p.fp.out[k][i];
            else
                p.fp.out[k][i] = run;
        }
    }
}

// ---- training labels from a plain render ----

// Per quarter-resolution pixel q of frame k of the last plain render (keys and client flow
// as that render stored them): at the full-resolution pixel 4q + 2, the plain method's
// window initialisation and 3-iteration search per keyframe (src/renderer.cu:148-215); the
// label is the converged source's offset (source - pixel) / 4 in quarter pixels, NaN when
// the direction was not searched or did not converge (error >= EPS_1).
__global__ void __launch_bounds__(256) label_kernel(const __grid_constant__ FrameParams p, int k, int hq, int wq, float *labels)
{
    const int qx = blockIdx.x * blockDim.x + threadIdx.x, qy = blockIdx.y * blockDim.y + threadIdx.y;
    if (qx >= wq || qy >= hq)
        return;
    const uint32_t x = (uint32_t)(4 * qx + 2), y = (uint32_t)(4 * qy + 2);
    float out[4] = {__int_as_float(0x7fc00000), __int_as_float(0x7fc00000), __int_as_float(0x7fc00000), __int_as_float(0x7fc00000)};
    if (x < p.out_w && y < p.out_h)
    {
        const DevView &a = p.v[0];
        const float qxc = __ldg(a.lut + x), qyc = __ldg(a.lut + a.w + y);
        for (int v = 0; v < 2; v++)
        {
            const DevView &dv = p.v[v];
            if (v == 0 && !(p.f[k].alpha < 1.0f))
                continue;
            const unsigned long long lo = window_key_global(dv.splat + k * p.key_stride, dv.w, dv.h, x, y);
            if (!(__uint_as_float((uint32_t)(lo >> 32)) > 0.0f))
                continue;
            uint32_t sx = min(((uint32_t)lo) >> 16, dv.w - 1u), sy = min((uint32_t)lo & 0xFFFFu, dv.h - 1u);
            const float2 *cam = dv.cam_xy + k * p.cam_stride;
            for (int i = 0; i < 3; i++)
            {
                const float2 m = __ldg(cam + (sy * dv.w + sx));
                const int2 t = cs2pixel(xsub(qxc, m.x), xsub(qyc, m.y), dv.w, dv.h);
                if (in_range(t, dv.w, dv.h))
                {
                    sx = (uint32_t)t.x;
                    sy = (uint32_t)t.y;
                }
            }
            const float2 m = __ldg(cam + (sy * dv.w + sx));
            const float ex = xmul(xsub(xadd(__ldg(dv.lut + sx), m.x), qxc), dv.err_sx);
            const float ey = xmul(xsub(xadd(__ldg(dv.lut + dv.w + sy), m.y), qyc), dv.err_sy);
            if (err_below<true>(err_pack<true>(xadd(xmul(ex, ex), xmul(ey, ey))), ERR_EPS_1_FULL_RES<true>))
            {
                out[2 * v] = 0.25f * ((float)sx - (float)x);
                out[2 * v + 1] = 0.25f * ((float)sy - (float)y);
            }
        }
    }
    *reinterpret_cast<float4 *>(labels + (((size_t)qy * wq) + qx) * 4) = make_float4(out[0], out[1], out[2], out[3]);
}
} // namespace isti
