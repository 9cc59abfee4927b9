// Launches of the tcgen05 convolution operators (isti_unet.cu), shared with the
// network code (isti_flownet.cu).
#pragma once

#include "isti.h"

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <utility>

namespace isti_unet
{
// A 1x1 head of 4 outputs (f32 weights [4][cout] and bias) to fuse into a convolution's
// epilogue: its outputs go to flow (f32) and/or flow16 (f16), [pixel][4].
struct ConvHead
{
    const float *w, *b;
    float *flow;
    void *flow16;
};

// pdl: launch as a programmatic dependent of the previous kernel in `stream` (it prepares
// while that kernel finishes; see griddep_wait in isti_tc.cuh).  head: fuse that head into
// the epilogue where the row-tile kernel runs the layer (then `out` is not written and
// *head_fused is set); otherwise the layer runs as usual and *head_fused is cleared.
isti_status conv_launch(int taps, const void *x, int n, int h, int w, int cin, const void *wpack, const float *bias, const void *mask, int relu,
                        void *out, int cout, int32_t *status, cudaStream_t stream, bool pdl = false, const ConvHead *head = nullptr,
                        bool *head_fused = nullptr);

// <<<grid, block, smem, stream>>> with, when `pdl`, the programmatic-dependent-launch
// attribute; the kernel must call griddep_wait before it touches the previous kernel's data
template <typename... K, typename... A>
cudaError_t launch_kernel(void (*kernel)(K...), dim3 grid, dim3 block, size_t smem, cudaStream_t stream, bool pdl, A &&...args)
{
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = pdl ? attr : nullptr;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<A>(args)...);
}
isti_status wgrad_launch(int taps, const void *dy, const void *x, int n, int h, int w, int cin, int cout, float *dw, int accumulate, void *scratch,
                         size_t scratch_bytes, int32_t *status, cudaStream_t stream);
isti_status pack_launch(int taps, const float *w, int cin, int cout, int transpose, void *wpack, cudaStream_t stream);
size_t wgrad_scratch(int taps, int n, int h, int w, int cin, int cout);
} // namespace isti_unet
