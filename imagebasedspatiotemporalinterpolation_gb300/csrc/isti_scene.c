/*
 * Seeded procedural scene for synthetic keyframes (input generator; stands in
 * for the reference's Unity-recorded dataset, which is not available).
 *
 * Scene: ground plane y = 0 (checkerboard albedo) plus spheres resting on it
 * (centre y = radius) moving with constant horizontal velocity, one
 * directional light with Lambertian shading, sky beyond the far plane.
 * Soft shadows: a sphere light of angular radius light_radius_deg; each
 * occluding sphere removes the part of the light disc it covers, estimated
 * from the angular separation of the two discs.
 *
 * Output buffers follow the conventions of the reference renderer's input
 * (the loader's post-conversion state, src/file_reader.cu:16-36,218-229):
 *  - color: RGBA8, sRGB-encoded, A = 255;
 *  - z: NDC z in [-1, 1] of the hit point under this camera's viewproj
 *    (sky: 1.0, the far plane);
 *  - motion_fwd / motion_bwd: f32x3 NDC delta from (pixel centre, z) to the
 *    projection, with this camera's viewproj, of the same surface point
 *    moved by +dt / -dt (object motion only; zero for static geometry);
 *  - shadow_{a,b,info}_{fwd,bwd}: per shadow sub-frame j = 0..sfpa-1 at time
 *    t0 +/- j*dt/sfpa, the 2-bit shadow level (0 lit .. 3 dark) of the moving
 *    surface point, packed at bits 2j..2j+1 of a 24-bit field stored in RGB
 *    (R = bits 16-23).  The field is 0 where the level never changes.
 *    shadow_a / shadow_b are the shaded colours at the lowest / highest level.
 *
 * Generator only: it is not part of the interpolation path.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct isti_sphere
{
    double cx, cz, r;        /* centre (cx, r, cz) at time 0 */
    double vx, vz;           /* velocity, m/s */
    double albedo[3];
} isti_sphere;

typedef struct isti_scene_desc
{
    int32_t n_spheres;
    const isti_sphere *spheres;
    double light_dir[3];     /* unit vector towards the light */
    double light_radius_deg; /* angular radius of the light disc */
} isti_scene_desc;

typedef struct isti_scene_cam
{
    uint32_t width, height;
    double viewproj[16];     /* column-major */
    double inv_viewproj[16];
    double t0;               /* keyframe time, seconds */
    double dt;               /* keyframe interval, seconds */
    int32_t sfpa;            /* shadow sub-frames per keyframe interval (<= 12) */
} isti_scene_cam;

typedef struct isti_scene_out
{
    uint8_t *color;
    float *z;
    float *motion_fwd;       /* f32x3 per pixel, or NULL */
    float *motion_bwd;
    uint8_t *shadow_a_fwd, *shadow_b_fwd, *shadow_info_fwd; /* RGBA8 or NULL */
    uint8_t *shadow_a_bwd, *shadow_b_bwd, *shadow_info_bwd;
} isti_scene_out;

typedef struct { double x, y, z; } d3;

static d3 v3(double x, double y, double z) { d3 r = {x, y, z}; return r; }
static d3 add(d3 a, d3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static d3 sub(d3 a, d3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static d3 mul(d3 a, double s) { return v3(a.x * s, a.y * s, a.z * s); }
static double dot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static d3 nrm(d3 a) { return mul(a, 1.0 / sqrt(dot(a, a))); }

static void xform(const double *m, const double v[4], double r[4])
{
    for (int i = 0; i < 4; i++)
        r[i] = m[i] * v[0] + m[4 + i] * v[1] + m[8 + i] * v[2] + m[12 + i] * v[3];
}

static d3 sphere_centre(const isti_sphere *s, double t) { return v3(s->cx + s->vx * t, s->r, s->cz + s->vz * t); }

/* nearest hit: returns object id (>= 0 sphere, -1 ground, -2 none) */
static int trace(const isti_scene_desc *sc, d3 o, d3 d, double t, double tmax, double *thit)
{
    int id = -2;
    double best = tmax;
    if (d.y < -1e-12)
    {
        const double tg = -o.y / d.y;
        if (tg > 0.0 && tg < best)
        {
            best = tg;
            id = -1;
        }
    }
    for (int i = 0; i < sc->n_spheres; i++)
    {
        const isti_sphere *s = &sc->spheres[i];
        const d3 oc = sub(o, sphere_centre(s, t));
        const double b = dot(oc, d);
        const double c = dot(oc, oc) - s->r * s->r;
        const double disc = b * b - c;
        if (disc <= 0.0)
            continue;
        const double sq = sqrt(disc);
        double th = -b - sq;
        if (th <= 1e-6)
            th = -b + sq;
        if (th > 1e-6 && th < best)
        {
            best = th;
            id = i;
        }
    }
    *thit = best;
    return id;
}

/* fraction of the light disc visible from p at time t (1 = fully lit) */
static double light_visibility(const isti_scene_desc *sc, d3 p, int self, double t)
{
    const d3 L = v3(sc->light_dir[0], sc->light_dir[1], sc->light_dir[2]);
    const double theta = sc->light_radius_deg * (3.14159265358979323846 / 180.0);
    const double sin_theta = sin(theta);
    double vis = 1.0;
    for (int i = 0; i < sc->n_spheres; i++)
    {
        if (i == self)
            continue;
        const isti_sphere *s = &sc->spheres[i];
        const d3 dc = sub(sphere_centre(s, t), p);
        const double proj = dot(dc, L);
        if (proj <= 0.0)
            continue;
        const double d2 = dot(dc, dc);
        /* sin(angle to L) > r/dist + sin(theta) implies the discs are apart */
        const double perp2 = d2 - proj * proj;
        const double reach = s->r + sqrt(d2) * sin_theta;
        if (perp2 > reach * reach)
            continue;
        const double dist = sqrt(d2);
        if (dist <= s->r)
            continue;
        const double beta = asin(s->r / dist);
        double ca = dot(dc, L) / dist;
        ca = ca > 1.0 ? 1.0 : ca;
        const double alpha = acos(ca);
        /* covered fraction: 1 when the light disc lies inside the occluder's,
         * 0 when the discs are apart, linear in between */
        double cover = (beta + theta - alpha) / (2.0 * theta);
        cover = cover < 0.0 ? 0.0 : (cover > 1.0 ? 1.0 : cover);
        vis *= 1.0 - cover;
        if (vis <= 0.0)
            return 0.0;
    }
    return vis;
}

static uint8_t srgb8(double c)
{
    c = c < 0.0 ? 0.0 : (c > 1.0 ? 1.0 : c);
    const double s = c <= 0.0031308 ? 12.92 * c : 1.055 * pow(c, 1.0 / 2.4) - 0.055;
    return (uint8_t)lround(s * 255.0);
}

static void shade(const isti_scene_desc *sc, int id, d3 p, d3 n, d3 dir, double vis, uint8_t rgba[4])
{
    double alb[3];
    if (id == -2)
    {
        const double up = dir.y < 0.0 ? 0.0 : dir.y;
        rgba[0] = srgb8(0.35 + 0.2 * up);
        rgba[1] = srgb8(0.5 + 0.25 * up);
        rgba[2] = srgb8(0.75 + 0.2 * up);
        rgba[3] = 255;
        return;
    }
    if (id == -1)
    {
        const int chk = ((int)floor(p.x) + (int)floor(p.z)) & 1;
        alb[0] = alb[1] = alb[2] = chk ? 0.6 : 0.3;
    }
    else
        memcpy(alb, sc->spheres[id].albedo, sizeof alb);
    const d3 L = v3(sc->light_dir[0], sc->light_dir[1], sc->light_dir[2]);
    double ndl = dot(n, L);
    ndl = ndl < 0.0 ? 0.0 : ndl;
    const double k = 0.2 + 0.8 * ndl * vis;
    for (int c = 0; c < 3; c++)
        rgba[c] = srgb8(alb[c] * k);
    rgba[3] = 255;
}

static int shadow_level(double vis)
{
    int l = (int)floor((1.0 - vis) * 4.0);
    return l < 0 ? 0 : (l > 3 ? 3 : l);
}

static double level_vis(int level) { return 1.0 - level / 3.0; }

static void shadow_fields(const isti_scene_desc *sc, const isti_scene_cam *cam, int id, d3 p, d3 n, d3 dir, double sign,
                          uint8_t *a, uint8_t *b, uint8_t *info)
{
    if (!a && !b && !info)
        return;
    uint32_t field = 0;
    int lo = 3, hi = 0, first = -1, changes = 0;
    for (int j = 0; j < cam->sfpa; j++)
    {
        const double tj = cam->t0 + sign * j * cam->dt / cam->sfpa;
        d3 pj = p;
        if (id >= 0)
            pj = add(p, mul(v3(sc->spheres[id].vx, 0.0, sc->spheres[id].vz), tj - cam->t0));
        const int lv = id == -2 ? 0 : shadow_level(light_visibility(sc, pj, id, tj));
        if (first < 0)
            first = lv;
        if (lv != first)
            changes = 1;
        lo = lv < lo ? lv : lo;
        hi = lv > hi ? lv : hi;
        field |= (uint32_t)lv << (2 * j);
    }
    if (!changes)
        field = 0;
    if (info)
    {
        info[0] = (uint8_t)(field >> 16);
        info[1] = (uint8_t)(field >> 8);
        info[2] = (uint8_t)field;
        info[3] = 255;
    }
    if (a)
        shade(sc, id, p, n, dir, level_vis(lo), a);
    if (b)
        shade(sc, id, p, n, dir, level_vis(hi), b);
}

static void pixel_ndc(const double *vp, d3 p, double out[3])
{
    const double v[4] = {p.x, p.y, p.z, 1.0};
    double r[4];
    xform(vp, v, r);
    out[0] = r[0] / r[3];
    out[1] = r[1] / r[3];
    out[2] = r[2] / r[3];
}

/* Renders one camera at one keyframe time.  Returns 0. */
int isti_scene_render(const isti_scene_desc *sc, const isti_scene_cam *cam, const isti_scene_out *out)
{
    const uint32_t W = cam->width, H = cam->height;
#pragma omp parallel for schedule(dynamic, 4)
    for (int32_t y = 0; y < (int32_t)H; y++)
    {
        for (uint32_t x = 0; x < W; x++)
        {
            const size_t i = (size_t)y * W + x;
            /* pixel centre in clip space, same mapping as the renderer's pixel2CS */
            const float pcx = 2.0f * ((float)x + 0.5f) / (float)W - 1.0f;
            const float pcy = 2.0f * ((float)y + 0.5f) / (float)H - 1.0f;
            const double pn[4] = {pcx, pcy, -1.0, 1.0}, pf[4] = {pcx, pcy, 1.0, 1.0};
            double wn[4], wf[4];
            xform(cam->inv_viewproj, pn, wn);
            xform(cam->inv_viewproj, pf, wf);
            const d3 o = v3(wn[0] / wn[3], wn[1] / wn[3], wn[2] / wn[3]);
            const d3 f = v3(wf[0] / wf[3], wf[1] / wf[3], wf[2] / wf[3]);
            const d3 dfull = sub(f, o);
            const double tmax = sqrt(dot(dfull, dfull));
            const d3 d = mul(dfull, 1.0 / tmax);
            double th;
            const int id = trace(sc, o, d, cam->t0, tmax, &th);
            d3 p = add(o, mul(d, th));
            d3 n = v3(0.0, 1.0, 0.0);
            if (id >= 0)
                n = nrm(sub(p, sphere_centre(&sc->spheres[id], cam->t0)));
            double ndc[3] = {pcx, pcy, 1.0};
            if (id != -2)
                pixel_ndc(cam->viewproj, p, ndc);
            const float zf = id == -2 ? 1.0f : (float)ndc[2];
            if (out->z)
                out->z[i] = zf;
            const double vis = id == -2 ? 1.0 : light_visibility(sc, p, id, cam->t0);
            if (out->color)
                shade(sc, id, p, n, d, vis, out->color + 4 * i);
            for (int dirn = 0; dirn < 2; dirn++)
            {
                float *m = dirn == 0 ? out->motion_fwd : out->motion_bwd;
                if (!m)
                    continue;
                m += 3 * i;
                if (id < 0)
                {
                    m[0] = m[1] = m[2] = 0.0f;
                    continue;
                }
                const double s = dirn == 0 ? cam->dt : -cam->dt;
                const d3 pm = add(p, mul(v3(sc->spheres[id].vx, 0.0, sc->spheres[id].vz), s));
                double q[3];
                pixel_ndc(cam->viewproj, pm, q);
                m[0] = (float)(q[0] - (double)pcx);
                m[1] = (float)(q[1] - (double)pcy);
                m[2] = (float)(q[2] - (double)zf);
            }
            if (cam->sfpa > 0)
            {
                shadow_fields(sc, cam, id, p, n, d, +1.0, out->shadow_a_fwd ? out->shadow_a_fwd + 4 * i : NULL,
                              out->shadow_b_fwd ? out->shadow_b_fwd + 4 * i : NULL,
                              out->shadow_info_fwd ? out->shadow_info_fwd + 4 * i : NULL);
                shadow_fields(sc, cam, id, p, n, d, -1.0, out->shadow_a_bwd ? out->shadow_a_bwd + 4 * i : NULL,
                              out->shadow_b_bwd ? out->shadow_b_bwd + 4 * i : NULL,
                              out->shadow_info_bwd ? out->shadow_info_bwd + 4 * i : NULL);
            }
        }
    }
    return 0;
}
