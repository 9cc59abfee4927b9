// GPU ray-cast of the procedural scene, for training data of the learned initialiser
// (input generator, not part of the interpolation path).  The same scene as
// isti_scene.c -- ground plane y = 0, spheres resting on it moving with constant
// horizontal velocity -- but only the buffers the search needs: NDC z and the object
// motion towards the other keyframe (f16 xyz).  Ray-sphere tests in f32 (the spheres in
// shared memory), the final projections in f64 as the host generator does them.
#include "isti_train.h"
#include "host/isti_error.hpp"

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <string>

namespace
{
constexpr int MAX_SPHERES = 512;

struct CamDev
{
    double vp[16], ivp[16];
    uint32_t w, h;
    double t0, motion_dt;
    int32_t n;
};

__device__ __forceinline__ void xform_d(const double *m, const double v[4], double r[4])
{
    for (int i = 0; i < 4; i++)
        r[i] = m[i] * v[0] + m[4 + i] * v[1] + m[8 + i] * v[2] + m[12 + i] * v[3];
}

__global__ void __launch_bounds__(256) raycast_kernel(const isti_gpu_sphere *spheres, const __grid_constant__ CamDev c, float *z_out, __half *m_out)
{
    __shared__ float sp[MAX_SPHERES][5];
    const int t = threadIdx.y * blockDim.x + threadIdx.x;
    for (int i = t; i < c.n; i += blockDim.x * blockDim.y)
    {
        const isti_gpu_sphere s = spheres[i];
        sp[i][0] = s.cx + s.vx * (float)c.t0;
        sp[i][1] = s.cz + s.vz * (float)c.t0;
        sp[i][2] = s.r;
        sp[i][3] = s.vx;
        sp[i][4] = s.vz;
    }
    __syncthreads();
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= c.w || y >= c.h)
        return;
    const float pcx = 2.0f * ((float)x + 0.5f) / (float)c.w - 1.0f;
    const float pcy = 2.0f * ((float)y + 0.5f) / (float)c.h - 1.0f;
    const double pn[4] = {pcx, pcy, -1.0, 1.0}, pf[4] = {pcx, pcy, 1.0, 1.0};
    double wn[4], wf[4];
    xform_d(c.ivp, pn, wn);
    xform_d(c.ivp, pf, wf);
    const double ox = wn[0] / wn[3], oy = wn[1] / wn[3], oz = wn[2] / wn[3];
    double dx = wf[0] / wf[3] - ox, dy = wf[1] / wf[3] - oy, dz = wf[2] / wf[3] - oz;
    const double tmax = sqrt(dx * dx + dy * dy + dz * dz);
    dx /= tmax, dy /= tmax, dz /= tmax;
    const float fox = (float)ox, foy = (float)oy, foz = (float)oz, fdx = (float)dx, fdy = (float)dy, fdz = (float)dz;
    float best = (float)tmax;
    int id = -2;
    if (fdy < -1e-12f)
    {
        const float tg = -foy / fdy;
        if (tg > 0.0f && tg < best)
        {
            best = tg;
            id = -1;
        }
    }
    for (int i = 0; i < c.n; i++)
    {
        const float cx = fox - sp[i][0], cy = foy - sp[i][2], cz = foz - sp[i][1];
        const float b = cx * fdx + cy * fdy + cz * fdz;
        const float cc = cx * cx + cy * cy + cz * cz - sp[i][2] * sp[i][2];
        const float disc = b * b - cc;
        if (disc <= 0.0f)
            continue;
        const float sq = sqrtf(disc);
        float th = -b - sq;
        if (th <= 1e-5f)
            th = -b + sq;
        if (th > 1e-5f && th < best)
        {
            best = th;
            id = i;
        }
    }
    const size_t i = (size_t)y * c.w + x;
    if (id == -2)
    {
        z_out[i] = 1.0f;
        m_out[3 * i] = m_out[3 * i + 1] = m_out[3 * i + 2] = __float2half(0.0f);
        return;
    }
    const double px = ox + dx * best, py = oy + dy * best, pz = oz + dz * best;
    const double p4[4] = {px, py, pz, 1.0};
    double q[4];
    xform_d(c.vp, p4, q);
    const float zf = (float)(q[2] / q[3]);
    z_out[i] = zf;
    if (id < 0)
    {
        m_out[3 * i] = m_out[3 * i + 1] = m_out[3 * i + 2] = __float2half(0.0f);
        return;
    }
    const double pm[4] = {px + (double)sp[id][3] * c.motion_dt, py, pz + (double)sp[id][4] * c.motion_dt, 1.0};
    xform_d(c.vp, pm, q);
    m_out[3 * i] = __float2half((float)(q[0] / q[3] - (double)pcx));
    m_out[3 * i + 1] = __float2half((float)(q[1] / q[3] - (double)pcy));
    m_out[3 * i + 2] = __float2half((float)(q[2] / q[3] - (double)zf));
}
} // namespace

extern "C" isti_status isti_scene_raycast(const isti_gpu_sphere *spheres, int32_t n_spheres, uint32_t width, uint32_t height, const double *viewproj,
                                          const double *inv_viewproj, double t0, double motion_dt, float *z, void *motion_f16x3, void *stream)
{
    if (!spheres || n_spheres < 0 || n_spheres > MAX_SPHERES || width == 0 || height == 0 || !viewproj || !inv_viewproj || !z || !motion_f16x3)
        return isti::set_error(ISTI_ERR_INVALID_ARG, "isti_scene_raycast: bad argument");
    CamDev c{};
    for (int k = 0; k < 16; k++)
    {
        c.vp[k] = viewproj[k];
        c.ivp[k] = inv_viewproj[k];
    }
    c.w = width;
    c.h = height;
    c.t0 = t0;
    c.motion_dt = motion_dt;
    c.n = n_spheres;
    raycast_kernel<<<dim3((width + 31) / 32, (height + 7) / 8), dim3(32, 8), 0, static_cast<cudaStream_t>(stream)>>>(
        spheres, c, z, static_cast<__half *>(motion_f16x3));
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? ISTI_OK : isti::set_error(ISTI_ERR_CUDA, std::string("isti_scene_raycast: ") + cudaGetErrorString(e));
}
