// Launch helpers of the interpolation kernels (isti_kernels.cuh): tensor maps for the
// TMA-staged key tiles, the reprojection launch shapes (fixed rule and autotuner
// candidates), and the launch sequences of a batch.  Included by each translation unit
// that compiles the kernels (one per arithmetic mode, isti_device.cuh), inside that
// unit's kernel namespace.
#pragma once

#include "isti_kernels.cuh"

#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <vector>

namespace isti
{
// Enqueues the timewarp of one batch (src/renderer.cu:615-629): mean z of the forward
// keyframe (two kernels), then one kernel over the output pixels.
cudaError_t launch_timewarp(isti::FrameParams &p, char *base, cudaStream_t stream, cudaEvent_t after_mean, cudaEvent_t after_nothing)
{
    p.tw_rows = reinterpret_cast<double *>(base);
    p.tw_mean = reinterpret_cast<float *>(base + ((size_t)p.v[0].h * sizeof(double) + 255) / 256 * 256);
    isti::timewarp_rowsum_kernel<<<(p.v[0].h + 127) / 128, 128, 0, stream>>>(p);
    isti::timewarp_mean_kernel<<<1, 32, 0, stream>>>(p);
    if (after_mean)
        cudaEventRecord(after_mean, stream);
    if (after_nothing)
        cudaEventRecord(after_nothing, stream); // no splat stage in this mode
    isti::timewarp_kernel<<<dim3((p.out_w + 31) / 32, (p.out_h + 7) / 8), dim3(32, 8), 0, stream>>>(p);
    return cudaGetLastError();
}

// ---- tensor maps for the TMA-staged key tiles ----

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

// One 3-D map (x, y, frame) per view over its keys; false when a view cannot be
// described (row pitch not a multiple of 16 bytes, image smaller than a tile) or
// the driver has no tensor-map support: the kernel then loads tiles with plain loads.
template <int SW>
bool make_key_maps(const isti::FrameParams &p, isti::KeyMaps &km)
{
    using T = isti::Tile<SW>;
    EncodeTiledFn enc = encode_tiled();
    if (!enc)
        return false;
    for (int k = 0; k < p.n_views; k++)
    {
        const isti::DevView &v = p.v[k];
        if ((v.w * 8u) % 16u != 0 || v.w < (uint32_t)T::W || v.h < (uint32_t)T::H)
            return false;
        const cuuint64_t dims[3] = {v.w, v.h, (cuuint64_t)p.n_frames};
        const cuuint64_t strides[2] = {(cuuint64_t)v.w * 8u, (cuuint64_t)p.key_stride * 8u};
        const cuuint32_t box[3] = {(cuuint32_t)T::W, (cuuint32_t)T::H, 1};
        const cuuint32_t estr[3] = {1, 1, 1};
        if (enc(&km.m[k], CU_TENSOR_MAP_DATA_TYPE_UINT64, 3, v.splat, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return false;
    }
    return true;
}

// A reprojection launch shape: register cap and output row pairs per block (0: the fixed rule).
struct ReprojChoice
{
    int regs = 0;
    int row_pairs = 0;
    int plain_tiles = 0; // 1: key tiles by plain loads even where a TMA copy is possible
};

// Per-SM limits of the current device that bound resident blocks (cached per device).
struct SmLimits
{
    int regs = 65536, smem = 233472, threads = 2048, blocks = 32, reserved = 1024;
};

SmLimits sm_limits()
{
    static std::mutex mu;
    static SmLimits cache[64];
    static bool have[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess)
        return SmLimits{};
    std::lock_guard<std::mutex> lock(mu);
    if (!have[dev & 63])
    {
        SmLimits l;
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxRegistersPerMultiprocessor, dev) == cudaSuccess && v > 0)
            l.regs = v;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) == cudaSuccess && v > 0)
            l.smem = v;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxThreadsPerMultiProcessor, dev) == cudaSuccess && v > 0)
            l.threads = v;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxBlocksPerMultiprocessor, dev) == cudaSuccess && v > 0)
            l.blocks = v;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrReservedSharedMemoryPerBlock, dev) == cudaSuccess && v >= 0)
            l.reserved = v;
        cache[dev & 63] = l;
        have[dev & 63] = true;
    }
    return cache[dev & 63];
}

// Resident reprojection blocks per SM at a register cap (registers are allocated per warp in
// units of 256), for blocks of `warps` warps and `smem` bytes of dynamic shared memory.
int resident_blocks(int regs, int warps, size_t smem)
{
    const SmLimits l = sm_limits();
    const int per_warp = (regs * 32 + 255) / 256 * 256;
    int b = std::min(l.blocks, l.threads / (32 * warps));
    b = std::min(b, l.regs / (per_warp * warps));
    return std::min(b, (int)((size_t)l.smem / (smem + (size_t)l.reserved)));
}

// The fixed rule's output row pairs per block: enough (frame, row) tasks for every warp in
// phase 2 (a single frame of 6 views: 3 row pairs).
int rule_row_pairs(int n_views, int n_frames) { return std::max(1, std::min(3, n_views / (isti::ROWS * n_frames))); }

// The fixed rule's register cap: 56 for the 7x7 window, 48 with fewer than 4 views; with 4 or
// more views 40 (more resident warps), unless 48 costs no resident blocks because the block's
// shared memory limits them anyway -- many frames per call (1080p, 6 frames: 6 views 1.254 ->
// 1.158 ms, 4 views 0.865 -> 0.785 ms).
int rule_regs(int sw, int n_views, int n_frames, int row_pairs)
{
    if (sw != 1)
        return isti::REPROJ_REGS_WIDE_WINDOW;
    if (n_views < isti::REPROJ_MANY_VIEWS)
        return isti::REPROJ_REGS;
    const size_t smem = isti::reproj_smem<1>(n_views, n_frames * row_pairs);
    return resident_blocks(isti::REPROJ_REGS, n_views, smem) >= resident_blocks(isti::REPROJ_REGS_MANY_VIEWS, n_views, smem)
               ? isti::REPROJ_REGS
               : isti::REPROJ_REGS_MANY_VIEWS;
}

// The rule's launch for a frame batch (register cap and row pairs; TMA key tiles).
ReprojChoice rule_choice(int sw, const isti::FrameParams &p)
{
    const int rp = rule_row_pairs(p.n_views, p.n_frames);
    return ReprojChoice{rule_regs(sw, p.n_views, p.n_frames, rp), rp, 0};
}

template <int SW, int SI, bool MAV, int REGS>
cudaError_t launch_reproj_regs(isti::FrameParams &p, cudaStream_t stream, int row_pairs, bool plain_tiles)
{
    // One unit's key tiles per TMA round: the least shared memory per block, so the most
    // resident blocks and the largest L1 (1080p, 6 views, 3 frames, 8 blocks per SM: one
    // frame per round 0.569 ms, two 0.581 ms; at 7 blocks two frames 0.590, three 0.594).
    // Row pairs per block: enough (frame, row) tasks for every warp in phase 2 when there
    // are fewer frames than views need (a single frame of 6 views: 3 row pairs).
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return e;
    p.row_pairs = row_pairs > 0 ? std::min(row_pairs, 3) : rule_row_pairs(p.n_views, p.n_frames);
    // Chained outputs of several frames: phase 3 gives each row of a block its own warp, so a
    // block has at most as many rows as there are views.  A single frame's chained output is
    // its unchained output (the persistent buffer is out[0] itself), so that launch runs unchained.
    if (p.chain && p.n_frames > 1)
        p.row_pairs = std::min(p.row_pairs, std::max(1, p.n_views / isti::ROWS));
    static thread_local isti::KeyMaps km; // 2 KiB, passed by value as a kernel parameter
    // the maps depend only on the key buffers' addresses and shapes: encode them again only
    // when those changed (a renderer reuses its arena from call to call)
    struct MapsKey
    {
        const void *splat[isti::MAX_VIEWS];
        uint32_t w[isti::MAX_VIEWS], h[isti::MAX_VIEWS];
        size_t key_stride;
        int n_views, n_frames;
        bool operator==(const MapsKey &) const = default;
    };
    static thread_local MapsKey last{};
    static thread_local int last_tma = -1; // -1: nothing cached
    MapsKey key{};
    for (int k = 0; k < p.n_views; k++)
    {
        key.splat[k] = p.v[k].splat;
        key.w[k] = p.v[k].w;
        key.h[k] = p.v[k].h;
    }
    key.key_stride = p.key_stride;
    key.n_views = p.n_views;
    key.n_frames = p.n_frames;
    if (last_tma < 0 || !(key == last))
    {
        last_tma = make_key_maps<SW>(p, km) ? 1 : 0;
        last = key;
    }
    p.use_tma = (!plain_tiles && last_tma == 1) ? 1 : 0;
    const size_t smem = isti::reproj_smem<SW>(p.n_views, p.n_frames * p.row_pairs);
    const uint32_t block_rows = (uint32_t)(isti::ROWS * p.row_pairs);
    const dim3 gr((p.out_w + 31) / 32, (p.out_h + block_rows - 1) / block_rows);
    p.withhold_block = -1;
    if (p.withhold_x >= 0 && p.withhold_y >= 0 && (uint32_t)p.withhold_x < p.out_w && (uint32_t)p.withhold_y < p.out_h)
        p.withhold_block = (int32_t)(((uint32_t)p.withhold_y / block_rows) * gr.x + (uint32_t)p.withhold_x / 32u);
    const bool hook = p.withhold_block >= 0 && p.use_tma;
    auto kernel = hook ? isti::reproj_kernel<SW, SI, MAV, REGS, true> : isti::reproj_kernel<SW, SI, MAV, REGS, false>;
    // raise the kernel's dynamic shared-memory limit once to the largest size requested, so
    // that calls inside a CUDA graph capture make no attribute calls after a first uncaptured
    // call of the same shape
    static std::mutex attr_mutex;
    static int attr_set[2][64] = {}; // per kernel instance and device
    if (smem > 48 * 1024)
    {
        std::lock_guard<std::mutex> lock(attr_mutex);
        int &cur = attr_set[hook ? 1 : 0][dev & 63];
        if ((int)smem > cur)
        {
            e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess)
                return e;
            cur = (int)smem;
        }
    }
    const int32_t chain = p.chain;
    if (p.n_frames == 1)
        p.chain = 0;
    kernel<<<gr, dim3(32, p.n_views), smem, stream>>>(p, km);
    p.chain = chain;
    return cudaGetLastError();
}

template <int SW, int SI, bool MAV>
cudaError_t launch_reproj(isti::FrameParams &p, cudaStream_t stream, ReprojChoice c)
{
    const int rp = c.row_pairs > 0 ? std::min(c.row_pairs, 3) : rule_row_pairs(p.n_views, p.n_frames);
    const int regs = c.regs > 0 ? c.regs : rule_regs(SW, p.n_views, p.n_frames, rp);
    if constexpr (SW == 1)
    {
        if (regs == isti::REPROJ_REGS_MANY_VIEWS)
            return launch_reproj_regs<SW, SI, MAV, isti::REPROJ_REGS_MANY_VIEWS>(p, stream, rp, c.plain_tiles != 0);
        return launch_reproj_regs<SW, SI, MAV, isti::REPROJ_REGS>(p, stream, rp, c.plain_tiles != 0);
    }
    else
        return launch_reproj_regs<SW, SI, MAV, isti::REPROJ_REGS_WIDE_WINDOW>(p, stream, rp, c.plain_tiles != 0);
}

// window size of the reprojection of a render mode (src/renderer.cu:676-693)
int mode_window(int mode) { return mode == ISTI_MODE_BACKWARD_BIDIRECTIONAL ? 3 : 1; }

// register caps a mode's reprojection is built with (the autotuner's candidates)
std::vector<int> mode_regs(int mode)
{
    if (mode_window(mode) == 1)
        return {isti::REPROJ_REGS_MANY_VIEWS, isti::REPROJ_REGS};
    return {isti::REPROJ_REGS_WIDE_WINDOW};
}

cudaError_t launch_reproj_mode(isti::FrameParams &p, int mode, cudaStream_t stream, ReprojChoice c)
{
    switch (mode)
    {
    case ISTI_MODE_OURS:
    case ISTI_MODE_BACKWARD_UNIDIRECTIONAL:
        return launch_reproj<1, 3, false>(p, stream, c);
    case ISTI_MODE_SPLATTING:
        return launch_reproj<1, 0, false>(p, stream, c);
    case ISTI_MODE_BACKWARD_BIDIRECTIONAL:
        return launch_reproj<3, 5, true>(p, stream, c);
    }
    return cudaGetLastError();
}

// Enqueues the three kernels of one batch; events (optional) are recorded after init and splat.
cudaError_t launch_batch(isti::FrameParams &p, int mode, cudaStream_t stream, cudaEvent_t after_init, cudaEvent_t after_splat,
                         ReprojChoice choice)
{
    uint32_t max_w = 0, max_h = 0;
    for (int k = 0; k < p.n_views; k++)
    {
        max_w = p.v[k].w > max_w ? p.v[k].w : max_w;
        max_h = p.v[k].h > max_h ? p.v[k].h : max_h;
    }
    // init: about 8 x 16-byte stores per thread, at least enough threads for the tables (<= 65535 entries)
    size_t init_blocks = (p.key_units + 8 * 256 - 1) / (8 * 256);
    if (init_blocks < 256)
        init_blocks = 256;
    if (init_blocks > 152 * 64)
        init_blocks = 152 * 64;
    isti::init_kernel<<<(unsigned)init_blocks, 256, 0, stream>>>(p);
    if (after_init)
        cudaEventRecord(after_init, stream);
    const dim3 gs((max_w + 31) / 32, (max_h + 7) / 8, p.n_views);
    isti::splat_kernel<<<gs, dim3(32, 8), 0, stream>>>(p);
    if (after_splat)
        cudaEventRecord(after_splat, stream);
    return launch_reproj_mode(p, mode, stream, choice);
}

} // namespace isti
