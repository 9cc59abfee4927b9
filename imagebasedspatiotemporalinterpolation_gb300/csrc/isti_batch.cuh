// One persistent launch for the frames of many keyframe pairs (isti_render_pairs; no
// counterpart in the reference, which renders frame by frame, src/main.cu:152-190).
//
// The work of every pair -- key initialisation, splatting, reprojection (isti_kernels.cuh) --
// is cut into units: init units (256 KiB of keys each by default, plus the pixel->clip
// tables), splat units (32 x 32 source pixels of one view by default, every frame) and
// reprojection units (one
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
// Unit sizes when the caller sets none (isti_renderer_set_pair_units).  Measured on the
// 96-frame mixed batch (16 pairs x 3 t x 2 eyes, uncaptured calls): 8 rows / 64 KiB 16.68 ms,
// 16 / 64 KiB 15.65, 32 / 256 KiB 15.15, 64 / 1024 KiB 15.73.
constexpr uint32_t BATCH_INIT_UNIT_KEYS = 16384; // 16-byte key units per init unit (256 KiB)
constexpr uint32_t BATCH_SPLAT_ROWS = 32;        // source rows per splat unit (32 columns)

struct BatchPair
{
    const FrameParams *fp;     // device copy of the pair's kernel parameters
    const CUtensorMap *maps;   // device copy of its key-tile tensor maps (n_views of them)
    uint32_t init_units, splat_units, reproj_units;
    uint32_t splat_need;       // splat units a reprojection unit waits for (splat_units; more under a test hook)
    uint32_t reproj_gx;        // reprojection blocks per block row
    uint32_t splat_gx, splat_gy; // splat units per view: columns of 32, rows of BatchParams::splat_rows
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
    uint32_t param_bytes;      // params_prefix(n_views): the staged part of a pair's FrameParams
    uint32_t splat_rows;       // source rows per splat unit
};

// Shared memory of a batch_kernel block: [the current pair's FrameParams prefix, padded to
// batch_param_space][reprojection region][TMA barrier][control words][the current BatchPair].
// The parameters sit at offset 0, so their fields are read at constant shared addresses.
constexpr size_t BATCH_CTRL_BYTES = 8 + 32 + 48; // barrier, 8 control words, the current BatchPair
__host__ __device__ constexpr size_t batch_param_space(size_t param_bytes) { return (param_bytes + 1023) & ~(size_t)1023; }
static_assert(sizeof(FrameParams) % 16 == 0, "FrameParams is staged in 16-byte words");
static_assert(sizeof(BatchPair) <= 48, "BatchPair is staged in 48 bytes");

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
    // the pair's kernel parameters, copied from global memory whenever the block moves to
    // another pair: read from shared memory like the per-call kernels read their constant bank
    uint4 *staged = reinterpret_cast<uint4 *>(smem);
    const FrameParams &p = *reinterpret_cast<const FrameParams *>(smem);
    unsigned char *region = smem + batch_param_space(bp.param_bytes);
    unsigned long long &bar = *reinterpret_cast<unsigned long long *>(region + bp.region_bytes);
    // [0, 1] ticket of the current / next unit and [2, 3] the status word seen for it (both
    // alternating: the entry for the next unit is written before the barrier that ends this
    // one, while some threads may not have read this unit's entry yet), [4] dependency met,
    // [5] a reprojection unit's wait for its key tiles gave up (reproj_block's `aborted`)
    uint32_t *ctrl = reinterpret_cast<uint32_t *>(region + bp.region_bytes + 8);
    BatchPair &bpair = *reinterpret_cast<BatchPair *>(region + bp.region_bytes + 8 + 32);
    const uint32_t tid = threadIdx.y * blockDim.x + threadIdx.x, nthreads = blockDim.x * blockDim.y;
    if (tid == 0)
    {
        mbar_init(&bar, 1);
        ctrl[0] = atomicAdd(bp.ticket, 1u);
        ctrl[2] = 0u;
        ctrl[5] = 0u;
    }
    __syncthreads();
    int round = 0;        // TMA rounds of this block's barrier (its phase carries across units)
    uint32_t slot = 0;    // ctrl word holding the current ticket
    // the segment of the current ticket; a block's tickets only grow, so the search resumes
    // where the previous unit's ended
    int si = -1;
    uint32_t seg_first = 0, seg_end = 0, seg_pair = 0xffffffffu, seg_phase = 0;
    uint32_t met_pair = 0xffffffffu, met_phase = 0; // the last dependency found satisfied
    for (;;)
    {
        const uint32_t t = ctrl[slot];
        if (t >= bp.total)
            break;
        // the next ticket and the status word are fetched while this unit runs, by the block's
        // last thread (not the TMA leader, tid 0, whose fences would wait for the atomic); it
        // waits for them only when it publishes them after the unit
        const bool helper = tid == nthreads - 1;
        uint32_t next_t = 0;
        int32_t status_seen = 0;
        if (helper)
        {
            next_t = atomicAdd(bp.ticket, 1u);
            status_seen = *(volatile int32_t *)bp.status;
        }
        // once a wait has given up (status word set) the remaining units only count themselves
        // done: the failed block's TMA barrier is out of step, and the call's outputs are void
        const bool failed = ctrl[2 + slot] != 0;
        const uint32_t old_pair = seg_pair;
        while (t >= seg_end)
        {
            si++;
            const BatchSeg sg = bp.segs[si];
            seg_first = sg.first;
            seg_pair = sg.pair;
            seg_phase = sg.phase;
            seg_end = si + 1 < bp.n_segs ? bp.segs[si + 1].first : bp.total;
        }
        if (seg_pair != old_pair) // block-uniform; every thread is past the previous unit (barrier below)
        {
            const uint4 *src = reinterpret_cast<const uint4 *>(bp.pairs[seg_pair].fp);
            for (uint32_t i = tid; i < bp.param_bytes / 16; i += nthreads)
                staged[i] = src[i];
            if (tid == 0)
                bpair = bp.pairs[seg_pair];
            __syncthreads();
        }
        const uint32_t u = t - seg_first;
        bool run = !failed;
        if (run && seg_phase > 0 && !(met_pair == seg_pair && met_phase == seg_phase))
        {
            if (tid == 0)
            {
                const uint32_t need = seg_phase == 1 ? bpair.init_units : bpair.splat_need;
                const uint32_t *cnt = bp.done + 2 * seg_pair + (seg_phase - 1);
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
                ctrl[4] = ok;
            }
            __syncthreads();
            run = ctrl[4] != 0;
            if (run)
            {
                met_pair = seg_pair;
                met_phase = seg_phase;
            }
        }
        if (run)
        {
            if (seg_phase == 0)
                init_part(p, (size_t)u * nthreads + tid, (size_t)bpair.init_units * nthreads, false); // the call's status word is reset by the host
            else if (seg_phase == 1)
            {
                const uint32_t per_view = bpair.splat_gx * bpair.splat_gy;
                const int view = (int)(u / per_view);
                const uint32_t r = u % per_view;
                const uint32_t x = (r % bpair.splat_gx) * 32 + threadIdx.x;
                const uint32_t y0 = (r / bpair.splat_gx) * bp.splat_rows;
                for (uint32_t yy = threadIdx.y; yy < bp.splat_rows; yy += blockDim.y)
                    splat_pixel(p, view, x, y0 + yy);
            }
            else
            {
                const uint32_t bx = u % bpair.reproj_gx, by = u / bpair.reproj_gx;
                reproj_block<SW, SI, MAV, REGS>(p, bpair.maps, bx, by, u, region, bar, round, *reinterpret_cast<volatile uint32_t *>(ctrl + 5));
            }
        }
        if (helper)
        {
            ctrl[slot ^ 1u] = next_t; // every thread read both entries before the previous barrier
            ctrl[2 + (slot ^ 1u)] = (uint32_t)status_seen;
        }
        __syncthreads();
        // the unit's writes (every thread's, ordered by the barrier) are published by one
        // release: a fence and the counter increment, as a grid-wide barrier does; a
        // reprojection unit's outputs are read by no other unit
        if (helper && seg_phase < 2)
        {
            __threadfence();
            atomicAdd(bp.done + 2 * seg_pair + seg_phase, 1u);
        }
        slot ^= 1u;
    }
}
} // namespace isti
