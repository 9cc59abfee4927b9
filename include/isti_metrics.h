/*
 * isti_metrics — image quality of interpolated frames on the GPU.
 *
 * Replaces the per-image metrics of the reference's offline evaluation
 * (scripts/eval.py:66-132), which loads both PNGs as RGB float in [0, 1]
 * (alpha dropped, eval.py:55-57) and computes
 *   PSNR = -10 log10(MSE)                         (eval.py:68, F.mse_loss)
 *   SSIM = mean of the SSIM map, 11x11 Gaussian window, sigma 1.5, zero
 *          padding, C1 = 0.01^2, C2 = 0.03^2, per channel (scripts/loss_utils.py:17-57)
 * for each frame against its ground truth.  FLIP (scripts/flip_loss.py) is not
 * provided.
 *
 * One fused kernel reads both RGBA8 images once: per 32x16 tile it stages the
 * tile and its 5-pixel halo in shared memory, filters the five SSIM moments
 * separably and accumulates the squared error exactly in integers; a second
 * one-block kernel adds the per-tile partial sums in a fixed order, so the
 * result is deterministic.  Both run on `stream`; the result is written to
 * device memory and nothing blocks the host.
 *
 * Numerics: the squared error is summed exactly (integers), MSE = sum /
 * (3 * width * height * 255^2) in double; SSIM per pixel in float32 like the
 * reference, summed in double.  Agreement with eval.py is within 1e-5 (SSIM)
 * and 1e-4 dB (PSNR); the reference's own torch results depend on its
 * convolution algorithm at the 1e-7 level.
 */
#ifndef ISTI_METRICS_H
#define ISTI_METRICS_H

#include "isti.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct isti_quality
{
    double mse;  /* mean squared error of RGB in [0, 1] */
    double psnr; /* dB; +inf for identical images */
    double ssim;
} isti_quality;

/* Device scratch the metric kernels need for an image of this size. */
size_t isti_quality_scratch_bytes(int32_t width, int32_t height);

/* a, b: device RGBA8 images of width*height pixels (4-byte aligned, dense
 * rows); scratch: isti_quality_scratch_bytes(width, height) device bytes;
 * out: device pointer to one isti_quality. */
isti_status isti_quality_rgba8(const void *a, const void *b, int32_t width, int32_t height, void *scratch,
                               isti_quality *out, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* ISTI_METRICS_H */
