// Launch entry points of the kernels compiled under the reference's GPU arithmetic
// (isti_render_fm.cu, -use_fast_math).  `params` points at the kernel parameters as
// isti_render.cu fills them (isti::FrameParams); both translation units compile the
// same structure definition, and isti_fm_params_size() lets the caller check that.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

size_t isti_fm_params_size();
cudaError_t isti_fm_launch_batch(void *params, int mode, cudaStream_t stream, cudaEvent_t after_init, cudaEvent_t after_splat, int regs,
                                 int row_pairs, int plain_tiles);
cudaError_t isti_fm_launch_reproj_mode(void *params, int mode, cudaStream_t stream, int regs, int row_pairs, int plain_tiles);
cudaError_t isti_fm_launch_timewarp(void *params, char *base, cudaStream_t stream, cudaEvent_t after_mean, cudaEvent_t after_nothing);
