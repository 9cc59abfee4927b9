// Launches of the tcgen05 convolution operators (isti_unet.cu), shared with the
// network code (isti_flownet.cu).
#pragma once

#include "isti.h"

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace isti_unet
{
isti_status conv_launch(int taps, const void *x, int n, int h, int w, int cin, const void *wpack, const float *bias, const void *mask, int relu,
                        void *out, int cout, int32_t *status, cudaStream_t stream);
isti_status wgrad_launch(int taps, const void *dy, const void *x, int n, int h, int w, int cin, int cout, float *dw, int accumulate, void *scratch,
                         size_t scratch_bytes, int32_t *status, cudaStream_t stream);
isti_status pack_launch(int taps, const float *w, int cin, int cout, int transpose, void *wpack, cudaStream_t stream);
size_t wgrad_scratch(int taps, int n, int h, int w, int cin, int cout);
} // namespace isti_unet
