// Blackwell (sm_103a) primitives for the U-Net kernels, as inline PTX: mbarriers with
// bounded waits, TMA tensor and bulk copies, and the 5th-generation tensor core
// (tcgen05: TMEM allocation, MMA with shared-memory descriptors, commit, TMEM loads).
//
// Operand layout used throughout (the canonical no-swizzle layout of the tcgen05
// shared-memory descriptor): a "core matrix" is 8 rows of 16 contiguous bytes
// (8 bf16 values), 128 bytes in all.  For a K-major operand a row is one M (or N)
// index and its 16 bytes are 8 consecutive K values; the descriptor's leading byte
// offset (LBO) is the distance between core matrices adjacent in K and the stride byte
// offset (SBO) between core matrices adjacent in M/N.  For an MN-major operand a row is
// one K index holding 8 consecutive M (or N) values, and again LBO is the distance
// between core matrices adjacent in K, SBO between those adjacent in M/N.  An NHWC bf16 activation tile
// fetched by TMA as boxes of {8 channels, 16 x, 8 y} lands exactly in this form: 128
// pixels x 16 bytes per box, 8 consecutive pixels per core matrix.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace isti_tc
{
constexpr uint32_t WAIT_LIMIT = 1u << 22; // mbarrier polls before a wait gives up (seconds at most)
constexpr int32_t ERR_TIMEOUT = 4;        // ISTI_ERR_TIMEOUT

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_barrier_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// Programmatic dependent launch (PTX griddepcontrol).  A kernel launched with
// cudaLaunchAttributeProgrammaticStreamSerialization may start while the previous kernel of
// its stream is still running, once every block of that kernel has called
// griddep_launch_dependents() (or exited).  griddep_wait() returns when the previous kernel
// has completed and its writes are visible; for a launch without the attribute it returns at
// once.  A kernel touches nothing the previous one writes or reads before its wait.
__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void griddep_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
// after griddep_wait, before TMA reads of what the previous kernel wrote (generic -> async proxy)
__device__ __forceinline__ void fence_proxy_async_global() { asm volatile("fence.proxy.async.global;" ::: "memory"); }

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.b32 %0, 1, 0, p;\n}"
                 : "=r"(ok)
                 : "r"(smem_u32(bar)), "r"(parity)
                 : "memory");
    return ok != 0;
}

// Waits for the phase with parity `parity` to complete, at most WAIT_LIMIT polls.  On
// timeout the status word is set and false returned: the caller stops its loop.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, int32_t *status)
{
    for (uint32_t i = 0; i < WAIT_LIMIT; i++)
        if (mbar_try_wait(bar, parity))
            return true;
    atomicExch(status, ERR_TIMEOUT);
    return false;
}

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 4-D tiled TMA load (c, x, y, n) of a tensor map into shared memory; completion on `bar`.
// c * 2 bytes must be a multiple of 16 (c a multiple of 8 for bf16); x and y may be
// negative or past the end (zero fill).
__device__ __forceinline__ void tma_load_4d(void *dst, const CUtensorMap *map, int c, int x, int y, int n, uint64_t *bar)
{
    asm volatile("cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(
                     smem_u32(dst)),
                 "l"(map), "r"(c), "r"(x), "r"(y), "r"(n), "r"(smem_u32(bar))
                 : "memory");
}

// Untiled bulk copy global -> shared (both 16-byte aligned, size a multiple of 16).
__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// ---- tcgen05 ----

// Allocates `ncols` TMEM columns (a power of two, 32..512); whole warp.  The address lands
// in shared memory at *dst.
__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(ncols) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor, no swizzle: start address, LBO, SBO (bytes, multiples of
// 16), the fixed version bits 46-48 = 0b001.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: bf16 A and B, f32 accumulator, M x N, operand
// majorness (0 K-major, 1 MN-major).
__host__ __device__ constexpr uint32_t idesc_bf16(uint32_t m, uint32_t n, uint32_t a_mn_major, uint32_t b_mn_major)
{
    return (1u << 4)            // D format: f32
           | (1u << 7)          // A format: bf16
           | (1u << 10)         // B format: bf16
           | (a_mn_major << 15) // A major
           | (b_mn_major << 16) // B major
           | ((n >> 3) << 17)   // N >> 3
           | ((m >> 4) << 24);  // M >> 4
}

// D[tmem] (+)= A[smem] * B[smem]^T, issued by one thread.
__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, bool accumulate)
{
    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem_d),
                 "l"(adesc), "l"(bdesc), "r"(idesc), "r"((uint32_t)accumulate)
                 : "memory");
}

// Arrives on `bar` once every MMA issued so far by this thread has completed.
__device__ __forceinline__ void mma_commit(uint64_t *bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// 32 lanes x 16 columns of 32-bit TMEM words: thread i of the warp gets lane (base lane + i),
// columns col .. col + 15.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16])
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
                   "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr));
}

__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
} // namespace isti_tc
