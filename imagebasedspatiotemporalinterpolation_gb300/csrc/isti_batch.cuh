// One persistent launch for the frames of many keyframe pairs (isti_render_pairs; no
// counterpart in the reference, which renders frame by frame, src/main.cu:152-190).
//
// The work of every pair -- key initialisation, splatting, reprojection (isti_kernels.cuh) --
// is cut into units: init units (64 KiB of keys each, plus the pixel->clip tables), splat
// units (32 x 16 source pixels of one view, every frame) and reprojection units (one
// reprojection block, reproj_block).  One cooperative launch keeps every CTA resident; each
// CTA takes tickets from one atomic queue until it runs dry.  The queue is
// software-pipelined over the pairs,
//     I0 S0 I1 S1 R0 I2 S2 R1 ... R(n-1)
// so that a reprojection unit of pair p, which must wait for every splat unit of p, comes
// after independent work.  Each pair has two completion counters (init units done, splat
// units done); a splat unit waits for its pair's init count, a reprojection unit for its
// splat count, with an iteration limit: a wait that gives up sets ISTI_ERR_TIMEOUT in the
// status word and the unit is skipped.  Because tickets are handed out in order and every CTA
// is resident, the units a wait depends on are always held by running CTAs.  Each pair has
// its own keys, flows and outputs, so units of different pairs never touch the same data.
#pragma once

#include "isti_kernels.cuh"

namespace isti
{
constexpr uint32_t BATCH_INIT_UNIT_KEYS = 4096; // 16-byte key units per init unit (64 KiB)
constexpr int BATCH_SPLAT_ROWS = 16;            // source rows per splat unit (32 columns)

struct BatchPair
{
    const FrameParams *fp;     // device copy of the pair's kernel parameters
    const CUtensorMap *maps;   // device copy of its key-tile tensor maps (n_views of them)
    uint32_t init_units, splat_units, reproj_units;
    uint32_t reproj_gx;        // reprojection blocks per block row
    uint32_t splat_gx, splat_gy; // splat units per view: columns of 32, rows of BATCH_SPLAT_ROWS
};

struct BatchSeg
{
    uint32_t pair, phase, first; // phase 0 init, 1 splat, 2 reprojection; first ticket of the segment
};

struct BatchParams
{
    const BatchPair *pairs;
    const BatchSeg *segs;
    int32_t n_segs;
    uint32_t total;            // tickets
    uint32_t *ticket;          // the queue (starts at 0)
    uint32_t *done;            // [pair][2]: init units done, splat units done (start at 0)
    int32_t *status;
    uint32_t spin_limit;
    uint32_t region_bytes;     // reprojection shared memory of the largest pair; the barrier follows
};

__device__ __forceinline__ uint32_t ld_acquire(const uint32_t *p)
{
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

template <int SW, int SI, bool MAV, int REGS>
__global__ void __maxnreg__(REGS) batch_kernel(const __grid_constant__ BatchParams bp)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned long long &bar = *reinterpret_cast<unsigned long long *>(smem + bp.region_bytes);
    uint32_t *ctrl = reinterpret_cast<uint32_t *>(smem + bp.region_bytes + 8); // [ticket, dependency satisfied, status]
    const uint32_t tid = threadIdx.y * blockDim.x + threadIdx.x, nthreads = blockDim.x * blockDim.y;
    if (tid == 0)
        mbar_init(&bar, 1);
    __syncthreads();
    int round = 0; // TMA rounds of this block's barrier (its phase carries across units)
    for (;;)
    {
        if (tid == 0)
        {
            ctrl[0] = atomicAdd(bp.ticket, 1u);
            ctrl[2] = (uint32_t)*(volatile int32_t *)bp.status;
        }
        __syncthreads();
        const uint32_t t = ctrl[0];
        if (t >= bp.total)
            break;
        // once a wait has given up (status word set) the remaining units only count themselves
        // done: the failed block's TMA barrier is out of step, and the call's outputs are void
        const bool failed = ctrl[2] != 0;
        int si = 0;
        while (si + 1 < bp.n_segs && bp.segs[si + 1].first <= t)
            si++;
        const BatchSeg sg = bp.segs[si];
        const BatchPair &bpair = bp.pairs[sg.pair];
        const FrameParams &p = *bpair.fp;
        const uint32_t u = t - sg.first;
        bool run = !failed;
        if (run && sg.phase > 0)
        {
            if (tid == 0)
            {
                const uint32_t need = sg.phase == 1 ? bpair.init_units : bpair.splat_units;
                const uint32_t *cnt = bp.done + 2 * sg.pair + (sg.phase - 1);
                uint32_t ok = 0;
                for (uint32_t i = 0; i < bp.spin_limit; i++)
                {
                    if (ld_acquire(cnt) >= need)
                    {
                        ok = 1;
                        break;
                    }
                    __nanosleep(128);
                }
                if (!ok)
                    atomicExch(bp.status, (int32_t)ISTI_ERR_TIMEOUT);
                __threadfence();
                asm volatile("fence.proxy.async.global;" ::: "memory"); // key tiles are read by TMA
                ctrl[1] = ok;
            }
            __syncthreads();
            run = ctrl[1] != 0;
        }
        if (run)
        {
            if (sg.phase == 0)
                init_part(p, (size_t)u * nthreads + tid, (size_t)bpair.init_units * nthreads, false); // the call's status word is reset by the host
            else if (sg.phase == 1)
            {
                const uint32_t per_view = bpair.splat_gx * bpair.splat_gy;
                const int view = (int)(u / per_view);
                const uint32_t r = u % per_view;
                const uint32_t x = (r % bpair.splat_gx) * 32 + threadIdx.x;
                const uint32_t y0 = (r / bpair.splat_gx) * BATCH_SPLAT_ROWS;
                for (uint32_t yy = threadIdx.y; yy < BATCH_SPLAT_ROWS; yy += blockDim.y)
                    splat_pixel(p, view, x, y0 + yy);
            }
            else
            {
                const uint32_t bx = u % bpair.reproj_gx, by = u / bpair.reproj_gx;
                reproj_block<SW, SI, MAV, REGS>(p, bpair.maps, bx, by, u, smem, bar, round);
            }
        }
        __threadfence();
        __syncthreads();
        if (tid == 0 && sg.phase < 2)
            atomicAdd(bp.done + 2 * sg.pair + sg.phase, 1u);
    }
}
} // namespace isti
