// The interpolation kernels under the reference's own GPU arithmetic.
//
// The reference renderer is built with -use_fast_math (CMakeLists.txt:36): its
// divisions and square roots are the fast approximations, denormals are flushed and
// the compiler contracts multiplies and adds into FMAs where its expression trees
// allow.  This translation unit compiles the same kernels as isti_render.cu with the
// same flag and ISTI_FASTMATH = 1 (isti_device.cuh), in the namespace isti_fm, so a
// renderer set to ISTI_ARITH_REFERENCE_GPU (include/isti.h) reproduces the reference
// GPU build's results.  The host side (isti_render.cu) fills the same kernel
// parameters for both modes and launches through the entry points below.
#define ISTI_FASTMATH 1
#define isti isti_fm
#include "isti_kernels.cuh"
#include "isti_launch.cuh"
#undef isti

#include "isti_arith.h"

size_t isti_fm_params_size() { return sizeof(isti_fm::FrameParams); }

cudaError_t isti_fm_launch_batch(void *params, int mode, cudaStream_t stream, cudaEvent_t after_init, cudaEvent_t after_splat, int regs,
                                 int row_pairs, int plain_tiles)
{
    return isti_fm::launch_batch(*static_cast<isti_fm::FrameParams *>(params), mode, stream, after_init, after_splat,
                                 isti_fm::ReprojChoice{regs, row_pairs, plain_tiles});
}

cudaError_t isti_fm_launch_reproj_mode(void *params, int mode, cudaStream_t stream, int regs, int row_pairs, int plain_tiles)
{
    return isti_fm::launch_reproj_mode(*static_cast<isti_fm::FrameParams *>(params), mode, stream,
                                       isti_fm::ReprojChoice{regs, row_pairs, plain_tiles});
}

cudaError_t isti_fm_launch_timewarp(void *params, char *base, cudaStream_t stream, cudaEvent_t after_mean, cudaEvent_t after_nothing)
{
    return isti_fm::launch_timewarp(*static_cast<isti_fm::FrameParams *>(params), base, stream, after_mean, after_nothing);
}
