/*
 * isti_train — training data of the learned flow initialiser (no counterpart in the
 * reference): a GPU ray-cast of the procedural scene and the labels/inputs the
 * network is trained on.  See include/isti_unet.h for the network and the learned
 * render path.
 */
#ifndef ISTI_TRAIN_H
#define ISTI_TRAIN_H

#include <stddef.h>
#include <stdint.h>

#include "isti.h"

#ifdef __cplusplus
extern "C" {
#endif

/* One sphere of the procedural scene: centre (cx, r, cz) at time 0, radius r,
 * horizontal velocity (vx, vz) in m/s. */
typedef struct isti_gpu_sphere
{
    float cx, cz, r, vx, vz;
} isti_gpu_sphere;

/* Ray-casts one camera at time t0 (ground plane y = 0 plus up to 512 spheres; spheres in
 * device memory): z (width*height f32, NDC z, 1 = sky) and the object motion of every
 * visible sphere point over motion_dt seconds (negative: backwards) as an NDC delta
 * under this camera's viewproj (f16 xyz per pixel; 0 for the ground and the sky) --
 * the renderer's input conventions.  Matrices column-major f64 (host). */
isti_status isti_scene_raycast(const isti_gpu_sphere *spheres, int32_t n_spheres, uint32_t width, uint32_t height, const double *viewproj,
                               const double *inv_viewproj, double t0, double motion_dt, float *z, void *motion_f16x3, void *stream);

/* Quarter-resolution grid of the network for a width x height render (each side
 * ceil(side / 4) rounded up to a multiple of 8). */
isti_status isti_learned_grid(uint32_t width, uint32_t height, int32_t *grid_w, int32_t *grid_h);

/* The network input of n_frames client frames of one keyframe pair (main camera only):
 * net_input = n_frames x grid_h x grid_w x 16 bf16 (device), as isti_render_learned
 * builds it. */
isti_status isti_learned_input(isti_renderer *r, int32_t n_frames, const isti_render_info *infos, const isti_frame_data *frame,
                               void *net_input, void *stream);

/* Training labels from the last plain render of r (isti_render / isti_render_batch,
 * main camera only, modes 0/2/3): for frame `frame_index`, grid_h x grid_w x 4 f32 --
 * per quarter-resolution pixel the converged source offset (fwd dx, dy, bwd dx, dy) in
 * quarter pixels, NaN where that direction did not converge. */
isti_status isti_learned_labels(isti_renderer *r, int32_t frame_index, float *labels, void *stream);

#ifdef __cplusplus
}
#endif
#endif
