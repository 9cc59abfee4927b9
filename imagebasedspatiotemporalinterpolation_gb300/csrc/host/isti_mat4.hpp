// 4x4 float matrices for the host side of the frame loop: the glm operations
// the reference's caller applies to camera matrices before a frame is
// rendered (src/main.cu:26-28,158-161,176; src/file_reader.cu:138-143,218-229).
//
// glm is an empty submodule in the reference (.gitmodules), so these are
// restatements of glm's published algorithms (g-truc/glm 0.9.9 / 1.0,
// scalar code path, float arithmetic, every operation rounded on its own):
//   mul          operator*(mat4, mat4): column j = ((A0*B[j][0] + A1*B[j][1]) + A2*B[j][2]) + A3*B[j][3]
//   inverse      glm::inverse (compute_inverse<4,4>): 2x2 cofactors, adjugate,
//                determinant from the first row, one reciprocal
//   interpolate  gtx/matrix_interpolation: the rotation part is interpolated
//                in axis-angle form, the translation linearly
// Agreement with a particular glm release is not pinned (the reference does
// not record its glm commit).  Layout: column-major, element (row r, column
// c) at m[c * 4 + r], as glm and isti_render_info.
#pragma once

#include <cmath>
#include <cstring>
#include <limits>

namespace isti::host
{
struct mat4
{
    float m[16];
    float &operator()(int c, int r) { return m[c * 4 + r]; }
    float operator()(int c, int r) const { return m[c * 4 + r]; }

    static mat4 identity()
    {
        mat4 o{};
        o(0, 0) = o(1, 1) = o(2, 2) = o(3, 3) = 1.0f;
        return o;
    }
    // glm's column-wise constructor: 16 values, column after column
    static mat4 columns(const float (&v)[16])
    {
        mat4 o;
        std::memcpy(o.m, v, sizeof(o.m));
        return o;
    }
};

inline mat4 mul(const mat4 &a, const mat4 &b)
{
    mat4 o;
    for (int j = 0; j < 4; j++)
        for (int r = 0; r < 4; r++)
        {
            float s = a(0, r) * b(j, 0);
            s = s + a(1, r) * b(j, 1);
            s = s + a(2, r) * b(j, 2);
            s = s + a(3, r) * b(j, 3);
            o(j, r) = s;
        }
    return o;
}

inline mat4 transpose(const mat4 &a)
{
    mat4 o;
    for (int c = 0; c < 4; c++)
        for (int r = 0; r < 4; r++)
            o(c, r) = a(r, c);
    return o;
}

inline mat4 inverse(const mat4 &a)
{
    // 2x2 minors of columns 2,3 / 1,3 / 1,2 (rows paired as in glm's Coef00..Coef23)
    auto minor = [&](int c0, int c1, int r0, int r1) { return a(c0, r0) * a(c1, r1) - a(c1, r0) * a(c0, r1); };
    const float c00 = minor(2, 3, 2, 3), c02 = minor(1, 3, 2, 3), c03 = minor(1, 2, 2, 3);
    const float c04 = minor(2, 3, 1, 3), c06 = minor(1, 3, 1, 3), c07 = minor(1, 2, 1, 3);
    const float c08 = minor(2, 3, 1, 2), c10 = minor(1, 3, 1, 2), c11 = minor(1, 2, 1, 2);
    const float c12 = minor(2, 3, 0, 3), c14 = minor(1, 3, 0, 3), c15 = minor(1, 2, 0, 3);
    const float c16 = minor(2, 3, 0, 2), c18 = minor(1, 3, 0, 2), c19 = minor(1, 2, 0, 2);
    const float c20 = minor(2, 3, 0, 1), c22 = minor(1, 3, 0, 1), c23 = minor(1, 2, 0, 1);
    const float f0[4] = {c00, c00, c02, c03}, f1[4] = {c04, c04, c06, c07}, f2[4] = {c08, c08, c10, c11};
    const float f3[4] = {c12, c12, c14, c15}, f4[4] = {c16, c16, c18, c19}, f5[4] = {c20, c20, c22, c23};
    float v0[4], v1[4], v2[4], v3[4]; // rows 0..3 of columns (1, 0, 0, 0)
    for (int k = 0; k < 4; k++)
    {
        const int col = k == 0 ? 1 : 0;
        v0[k] = a(col, 0);
        v1[k] = a(col, 1);
        v2[k] = a(col, 2);
        v3[k] = a(col, 3);
    }
    mat4 inv;
    for (int k = 0; k < 4; k++)
    {
        const float sa = (k & 1) ? -1.0f : 1.0f; // columns 0 and 2
        const float sb = -sa;                    // columns 1 and 3
        inv(0, k) = ((v1[k] * f0[k] - v2[k] * f1[k]) + v3[k] * f2[k]) * sa;
        inv(1, k) = ((v0[k] * f0[k] - v2[k] * f3[k]) + v3[k] * f4[k]) * sb;
        inv(2, k) = ((v0[k] * f1[k] - v1[k] * f3[k]) + v3[k] * f5[k]) * sa;
        inv(3, k) = ((v0[k] * f2[k] - v1[k] * f4[k]) + v2[k] * f5[k]) * sb;
    }
    // determinant: first column of a against the first row of the adjugate
    float d[4];
    for (int r = 0; r < 4; r++)
        d[r] = a(0, r) * inv(r, 0);
    const float det = (d[0] + d[1]) + (d[2] + d[3]);
    const float one_over = 1.0f / det;
    for (float &x : inv.m)
        x = x * one_over;
    return inv;
}

struct vec3
{
    float x, y, z;
};

inline vec3 normalize(vec3 v)
{
    const float dot = (v.x * v.x + v.y * v.y) + v.z * v.z;
    const float inv_len = 1.0f / std::sqrt(dot);
    return {v.x * inv_len, v.y * inv_len, v.z * inv_len};
}

// glm::axisAngle of the rotation part of `m`.
inline void axis_angle(const mat4 &m, vec3 &axis, float &angle)
{
    const float eps = std::numeric_limits<float>::epsilon() * 1e2f;
    const bool near_symmetric = std::fabs(m(1, 0) - m(0, 1)) < eps && std::fabs(m(2, 0) - m(0, 2)) < eps &&
                                std::fabs(m(2, 1) - m(1, 2)) < eps;
    if (near_symmetric)
    {
        const bool near_identity = std::fabs(m(1, 0) + m(0, 1)) < eps && std::fabs(m(2, 0) + m(0, 2)) < eps &&
                                   std::fabs(m(2, 1) + m(1, 2)) < eps &&
                                   std::fabs(((m(0, 0) + m(1, 1)) + m(2, 2)) - 3.0f) < eps;
        if (near_identity)
        {
            angle = 0.0f;
            axis = {1.0f, 0.0f, 0.0f};
            return;
        }
        angle = 3.14159265358979323846264338327950288f;
        const float xx = (m(0, 0) + 1.0f) * 0.5f, yy = (m(1, 1) + 1.0f) * 0.5f, zz = (m(2, 2) + 1.0f) * 0.5f;
        const float xy = (m(1, 0) + m(0, 1)) * 0.25f, xz = (m(2, 0) + m(0, 2)) * 0.25f, yz = (m(2, 1) + m(1, 2)) * 0.25f;
        if (xx > yy && xx > zz)
        {
            if (xx < eps)
                axis = {0.0f, 0.7071f, 0.7071f};
            else
            {
                axis.x = std::sqrt(xx);
                axis.y = xy / axis.x;
                axis.z = xz / axis.x;
            }
        }
        else if (yy > zz)
        {
            if (yy < eps)
                axis = {0.7071f, 0.0f, 0.7071f};
            else
            {
                axis.y = std::sqrt(yy);
                axis.x = xy / axis.y;
                axis.z = yz / axis.y;
            }
        }
        else
        {
            if (zz < eps)
                axis = {0.7071f, 0.7071f, 0.0f};
            else
            {
                axis.z = std::sqrt(zz);
                axis.x = xz / axis.z;
                axis.y = yz / axis.z;
            }
        }
        return;
    }
    const float cos_angle = (((m(0, 0) + m(1, 1)) + m(2, 2)) - 1.0f) * 0.5f;
    if (cos_angle >= 1.0f)
        angle = 0.0f;
    else if (cos_angle <= -1.0f)
        angle = 3.14159265358979323846264338327950288f;
    else
        angle = std::acos(cos_angle);
    axis = normalize({m(1, 2) - m(2, 1), m(2, 0) - m(0, 2), m(0, 1) - m(1, 0)});
}

// glm::axisAngleMatrix: rotation by `angle` about `axis` (normalised first).
inline mat4 axis_angle_matrix(vec3 axis, float angle)
{
    const float c = std::cos(angle), s = std::sin(angle), t = 1.0f - c;
    const vec3 n = normalize(axis);
    const float v[16] = {t * n.x * n.x + c,       t * n.x * n.y + n.z * s, t * n.x * n.z - n.y * s, 0.0f,
                         t * n.x * n.y - n.z * s, t * n.y * n.y + c,       t * n.y * n.z + n.x * s, 0.0f,
                         t * n.x * n.z + n.y * s, t * n.y * n.z - n.x * s, t * n.z * n.z + c,       0.0f,
                         0.0f,                    0.0f,                    0.0f,                    1.0f};
    return mat4::columns(v);
}

// glm::interpolate (gtx/matrix_interpolation), used by the reference as the
// client view between two keyframe views (src/main.cu:26-28).
inline mat4 interpolate(const mat4 &m1, const mat4 &m2, float delta)
{
    mat4 rot1 = mat4::identity(); // extractMatrixRotation
    for (int c = 0; c < 3; c++)
        for (int r = 0; r < 3; r++)
            rot1(c, r) = m1(c, r);
    const mat4 delta_rot = mul(m2, transpose(rot1));
    vec3 axis;
    float angle;
    axis_angle(delta_rot, axis, angle);
    mat4 out = mul(axis_angle_matrix(axis, angle * delta), rot1);
    for (int r = 0; r < 3; r++)
        out(3, r) = m1(3, r) + delta * (m2(3, r) - m1(3, r));
    return out;
}

// FrameFileReader::normalizeProjMat (src/file_reader.cu:218-229) with the
// reader's constants (include/file_reader.h:60-67): Unity's GPU projection
// (reversed z, [0,1] depth, y flipped) back to the OpenGL convention.
inline mat4 normalize_proj(const mat4 &proj)
{
    const float reverse_z[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, -1, 0, 0, 0, 1, 1};
    const float depth_01_to_11[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 2, 0, 0, 0, -1, 1};
    const float unity_2022_3[16] = {1, 0, 0, 0, 0, -1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    mat4 p = mul(mat4::columns(reverse_z), proj);
    p = mul(mat4::columns(depth_01_to_11), p);
    return mul(mat4::columns(unity_2022_3), p);
}
} // namespace isti::host
