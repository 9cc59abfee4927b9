// Minimal glm-compatible vector/matrix subset for compiling the reference's
// renderer.cu on the host (test-only oracle harness).
//
// The reference pulls glm from an empty git submodule (dependencies/glm,
// .gitmodules:1-3), so the genuine library is not available.  This header is
// written from the linear-algebra definitions, not from glm's sources, and it
// fixes the floating-point operation order that the whole project uses:
//
//   mat4 * vec4 : r[i] = (m[0][i]*v.x + m[1][i]*v.y) + (m[2][i]*v.z + m[3][i]*v.w)
//   dot(vec3)   : (a.x*b.x + a.y*b.y) + a.z*b.z
//   dot(vec4)   : ((a.x*b.x + a.y*b.y) + a.z*b.z) + a.w*b.w
//   normalize   : v * (1 / sqrt(dot(v, v)))
//   vec / s     : each component divided by s
//
// Matrices are column-major, m[c] is column c, as in GLSL/glm.  The CUDA
// kernels and the C oracle restate exactly this order; agreement with the
// genuine glm build of the reference is not pinned.
#pragma once

#include <cmath>

// Device-callable where nvcc compiles the reference for the GPU (as genuine glm
// does under CUDA); plain host functions for the host build.
#ifdef __CUDACC__
#define ISTI_GLM_HD __host__ __device__
#else
#define ISTI_GLM_HD
#endif

namespace glm
{
struct vec4;

struct vec3
{
    float x, y, z;
    ISTI_GLM_HD vec3() : x(0.f), y(0.f), z(0.f) {}
    ISTI_GLM_HD explicit vec3(float s) : x(s), y(s), z(s) {}
    ISTI_GLM_HD vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    ISTI_GLM_HD vec3(const vec4 &v);  // implicit narrowing copy of xyz, as glm allows
    ISTI_GLM_HD float &operator[](int i) { return (&x)[i]; }
    ISTI_GLM_HD const float &operator[](int i) const { return (&x)[i]; }
};

struct vec4
{
    float x, y, z, w;
    ISTI_GLM_HD vec4() : x(0.f), y(0.f), z(0.f), w(0.f) {}
    ISTI_GLM_HD explicit vec4(float s) : x(s), y(s), z(s), w(s) {}
    ISTI_GLM_HD vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    ISTI_GLM_HD vec4(const vec3 &v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
    ISTI_GLM_HD float &operator[](int i) { return (&x)[i]; }
    ISTI_GLM_HD const float &operator[](int i) const { return (&x)[i]; }
};

ISTI_GLM_HD inline vec3::vec3(const vec4 &v) : x(v.x), y(v.y), z(v.z) {}

ISTI_GLM_HD inline vec4 operator+(const vec4 &a, const vec4 &b) { return vec4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
ISTI_GLM_HD inline vec4 operator-(const vec4 &a, const vec4 &b) { return vec4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
ISTI_GLM_HD inline vec4 operator-(const vec4 &a) { return vec4(-a.x, -a.y, -a.z, -a.w); }
ISTI_GLM_HD inline vec4 operator*(const vec4 &a, float s) { return vec4(a.x * s, a.y * s, a.z * s, a.w * s); }
ISTI_GLM_HD inline vec4 operator*(float s, const vec4 &a) { return vec4(s * a.x, s * a.y, s * a.z, s * a.w); }
ISTI_GLM_HD inline vec4 operator*(const vec4 &a, const vec4 &b) { return vec4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
ISTI_GLM_HD inline vec4 operator/(const vec4 &a, float s) { return vec4(a.x / s, a.y / s, a.z / s, a.w / s); }

ISTI_GLM_HD inline vec3 operator+(const vec3 &a, const vec3 &b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
ISTI_GLM_HD inline vec3 operator-(const vec3 &a, const vec3 &b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
ISTI_GLM_HD inline vec3 operator-(const vec3 &a) { return vec3(-a.x, -a.y, -a.z); }
ISTI_GLM_HD inline vec3 operator*(const vec3 &a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
ISTI_GLM_HD inline vec3 operator*(float s, const vec3 &a) { return vec3(s * a.x, s * a.y, s * a.z); }
ISTI_GLM_HD inline vec3 operator/(const vec3 &a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }

ISTI_GLM_HD inline float dot(const vec3 &a, const vec3 &b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
ISTI_GLM_HD inline float dot(const vec4 &a, const vec4 &b) { return ((a.x * b.x + a.y * b.y) + a.z * b.z) + a.w * b.w; }
ISTI_GLM_HD inline vec3 normalize(const vec3 &v) { return v * (1.0f / sqrtf(dot(v, v))); }
ISTI_GLM_HD inline vec4 normalize(const vec4 &v) { return v * (1.0f / sqrtf(dot(v, v))); }

struct mat4
{
    vec4 value[4];
    ISTI_GLM_HD mat4() : value{vec4(1.f, 0.f, 0.f, 0.f), vec4(0.f, 1.f, 0.f, 0.f), vec4(0.f, 0.f, 1.f, 0.f), vec4(0.f, 0.f, 0.f, 1.f)} {}
    ISTI_GLM_HD explicit mat4(float s) : value{vec4(s, 0.f, 0.f, 0.f), vec4(0.f, s, 0.f, 0.f), vec4(0.f, 0.f, s, 0.f), vec4(0.f, 0.f, 0.f, s)} {}
    ISTI_GLM_HD mat4(const vec4 &c0, const vec4 &c1, const vec4 &c2, const vec4 &c3) : value{c0, c1, c2, c3} {}
    // 16 scalars, column by column
    ISTI_GLM_HD mat4(float x0, float y0, float z0, float w0, float x1, float y1, float z1, float w1,
         float x2, float y2, float z2, float w2, float x3, float y3, float z3, float w3)
        : value{vec4(x0, y0, z0, w0), vec4(x1, y1, z1, w1), vec4(x2, y2, z2, w2), vec4(x3, y3, z3, w3)} {}
    ISTI_GLM_HD vec4 &operator[](int c) { return value[c]; }
    ISTI_GLM_HD const vec4 &operator[](int c) const { return value[c]; }
};

ISTI_GLM_HD inline vec4 operator*(const mat4 &m, const vec4 &v)
{
    const vec4 a = m[0] * v.x + m[1] * v.y;
    const vec4 b = m[2] * v.z + m[3] * v.w;
    return a + b;
}

ISTI_GLM_HD inline mat4 operator*(const mat4 &a, const mat4 &b)
{
    return mat4(a * b[0], a * b[1], a * b[2], a * b[3]);
}

// General 4x4 inverse by cofactors, accumulated in double (host use only:
// the renderer consumes matrices its caller already inverted).
inline mat4 inverse(const mat4 &m)
{
    double a[16], inv[16];
    for (int c = 0; c < 4; c++)
        for (int r = 0; r < 4; r++)
            a[c * 4 + r] = m[c][r];
    inv[0] = a[5] * a[10] * a[15] - a[5] * a[11] * a[14] - a[9] * a[6] * a[15] + a[9] * a[7] * a[14] + a[13] * a[6] * a[11] - a[13] * a[7] * a[10];
    inv[4] = -a[4] * a[10] * a[15] + a[4] * a[11] * a[14] + a[8] * a[6] * a[15] - a[8] * a[7] * a[14] - a[12] * a[6] * a[11] + a[12] * a[7] * a[10];
    inv[8] = a[4] * a[9] * a[15] - a[4] * a[11] * a[13] - a[8] * a[5] * a[15] + a[8] * a[7] * a[13] + a[12] * a[5] * a[11] - a[12] * a[7] * a[9];
    inv[12] = -a[4] * a[9] * a[14] + a[4] * a[10] * a[13] + a[8] * a[5] * a[14] - a[8] * a[6] * a[13] - a[12] * a[5] * a[10] + a[12] * a[6] * a[9];
    inv[1] = -a[1] * a[10] * a[15] + a[1] * a[11] * a[14] + a[9] * a[2] * a[15] - a[9] * a[3] * a[14] - a[13] * a[2] * a[11] + a[13] * a[3] * a[10];
    inv[5] = a[0] * a[10] * a[15] - a[0] * a[11] * a[14] - a[8] * a[2] * a[15] + a[8] * a[3] * a[14] + a[12] * a[2] * a[11] - a[12] * a[3] * a[10];
    inv[9] = -a[0] * a[9] * a[15] + a[0] * a[11] * a[13] + a[8] * a[1] * a[15] - a[8] * a[3] * a[13] - a[12] * a[1] * a[11] + a[12] * a[3] * a[9];
    inv[13] = a[0] * a[9] * a[14] - a[0] * a[10] * a[13] - a[8] * a[1] * a[14] + a[8] * a[2] * a[13] + a[12] * a[1] * a[10] - a[12] * a[2] * a[9];
    inv[2] = a[1] * a[6] * a[15] - a[1] * a[7] * a[14] - a[5] * a[2] * a[15] + a[5] * a[3] * a[14] + a[13] * a[2] * a[7] - a[13] * a[3] * a[6];
    inv[6] = -a[0] * a[6] * a[15] + a[0] * a[7] * a[14] + a[4] * a[2] * a[15] - a[4] * a[3] * a[14] - a[12] * a[2] * a[7] + a[12] * a[3] * a[6];
    inv[10] = a[0] * a[5] * a[15] - a[0] * a[7] * a[13] - a[4] * a[1] * a[15] + a[4] * a[3] * a[13] + a[12] * a[1] * a[7] - a[12] * a[3] * a[5];
    inv[14] = -a[0] * a[5] * a[14] + a[0] * a[6] * a[13] + a[4] * a[1] * a[14] - a[4] * a[2] * a[13] - a[12] * a[1] * a[6] + a[12] * a[2] * a[5];
    inv[3] = -a[1] * a[6] * a[11] + a[1] * a[7] * a[10] + a[5] * a[2] * a[11] - a[5] * a[3] * a[10] - a[9] * a[2] * a[7] + a[9] * a[3] * a[6];
    inv[7] = a[0] * a[6] * a[11] - a[0] * a[7] * a[10] - a[4] * a[2] * a[11] + a[4] * a[3] * a[10] + a[8] * a[2] * a[7] - a[8] * a[3] * a[6];
    inv[11] = -a[0] * a[5] * a[11] + a[0] * a[7] * a[9] + a[4] * a[1] * a[11] - a[4] * a[3] * a[9] - a[8] * a[1] * a[7] + a[8] * a[3] * a[5];
    inv[15] = a[0] * a[5] * a[10] - a[0] * a[6] * a[9] - a[4] * a[1] * a[10] + a[4] * a[2] * a[9] + a[8] * a[1] * a[6] - a[8] * a[2] * a[5];
    const double det = a[0] * inv[0] + a[1] * inv[4] + a[2] * inv[8] + a[3] * inv[12];
    mat4 r;
    for (int c = 0; c < 4; c++)
        for (int rr = 0; rr < 4; rr++)
            r[c][rr] = (float)(inv[c * 4 + rr] / det);
    return r;
}
} // namespace glm
