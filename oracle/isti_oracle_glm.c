/*
 * ORACLE (test infrastructure only): the glm matrix operations of the
 * reference's frame loop, restated in plain C for the CPU checker.
 *
 * glm is an empty submodule in the reference (.gitmodules:1-3), so these follow
 * glm's published algorithms (g-truc/glm 1.0, scalar path, float arithmetic):
 *   operator*(mat4, mat4)      (glm/detail/type_mat4x4.inl)
 *   inverse                    (glm/detail/func_matrix.inl, compute_inverse<4,4>)
 *   interpolate, axisAngle, axisAngleMatrix, extractMatrixRotation
 *                              (glm/gtx/matrix_interpolation.inl)
 * and FrameFileReader::normalizeProjMat (src/file_reader.cu:218-229) with the
 * constants of include/file_reader.h:60-67.  Used by src/main.cu:26-28,158-176
 * and src/file_reader.cu:138-143.  Agreement with a glm release is not pinned:
 * the reference does not record its glm commit.  Compiled with
 * -ffp-contract=off; matrices column-major, m[c*4 + r].
 */
#include <float.h>
#include <math.h>
#include <string.h>

#define AT(m, c, r) ((m)[(c) * 4 + (r)])

void oracle_mat4_mul(const float *a, const float *b, float *out)
{
    float o[16];
    for (int j = 0; j < 4; j++)
        for (int r = 0; r < 4; r++)
        {
            float acc = AT(a, 0, r) * AT(b, j, 0);
            acc += AT(a, 1, r) * AT(b, j, 1);
            acc += AT(a, 2, r) * AT(b, j, 2);
            acc += AT(a, 3, r) * AT(b, j, 3);
            AT(o, j, r) = acc;
        }
    memcpy(out, o, sizeof(o));
}

void oracle_mat4_inverse(const float *m, float *out)
{
    /* glm's Coef00..Coef23 */
    const float coef00 = AT(m, 2, 2) * AT(m, 3, 3) - AT(m, 3, 2) * AT(m, 2, 3);
    const float coef02 = AT(m, 1, 2) * AT(m, 3, 3) - AT(m, 3, 2) * AT(m, 1, 3);
    const float coef03 = AT(m, 1, 2) * AT(m, 2, 3) - AT(m, 2, 2) * AT(m, 1, 3);
    const float coef04 = AT(m, 2, 1) * AT(m, 3, 3) - AT(m, 3, 1) * AT(m, 2, 3);
    const float coef06 = AT(m, 1, 1) * AT(m, 3, 3) - AT(m, 3, 1) * AT(m, 1, 3);
    const float coef07 = AT(m, 1, 1) * AT(m, 2, 3) - AT(m, 2, 1) * AT(m, 1, 3);
    const float coef08 = AT(m, 2, 1) * AT(m, 3, 2) - AT(m, 3, 1) * AT(m, 2, 2);
    const float coef10 = AT(m, 1, 1) * AT(m, 3, 2) - AT(m, 3, 1) * AT(m, 1, 2);
    const float coef11 = AT(m, 1, 1) * AT(m, 2, 2) - AT(m, 2, 1) * AT(m, 1, 2);
    const float coef12 = AT(m, 2, 0) * AT(m, 3, 3) - AT(m, 3, 0) * AT(m, 2, 3);
    const float coef14 = AT(m, 1, 0) * AT(m, 3, 3) - AT(m, 3, 0) * AT(m, 1, 3);
    const float coef15 = AT(m, 1, 0) * AT(m, 2, 3) - AT(m, 2, 0) * AT(m, 1, 3);
    const float coef16 = AT(m, 2, 0) * AT(m, 3, 2) - AT(m, 3, 0) * AT(m, 2, 2);
    const float coef18 = AT(m, 1, 0) * AT(m, 3, 2) - AT(m, 3, 0) * AT(m, 1, 2);
    const float coef19 = AT(m, 1, 0) * AT(m, 2, 2) - AT(m, 2, 0) * AT(m, 1, 2);
    const float coef20 = AT(m, 2, 0) * AT(m, 3, 1) - AT(m, 3, 0) * AT(m, 2, 1);
    const float coef22 = AT(m, 1, 0) * AT(m, 3, 1) - AT(m, 3, 0) * AT(m, 1, 1);
    const float coef23 = AT(m, 1, 0) * AT(m, 2, 1) - AT(m, 2, 0) * AT(m, 1, 1);

    const float fac0[4] = {coef00, coef00, coef02, coef03};
    const float fac1[4] = {coef04, coef04, coef06, coef07};
    const float fac2[4] = {coef08, coef08, coef10, coef11};
    const float fac3[4] = {coef12, coef12, coef14, coef15};
    const float fac4[4] = {coef16, coef16, coef18, coef19};
    const float fac5[4] = {coef20, coef20, coef22, coef23};
    const float vec0[4] = {AT(m, 1, 0), AT(m, 0, 0), AT(m, 0, 0), AT(m, 0, 0)};
    const float vec1[4] = {AT(m, 1, 1), AT(m, 0, 1), AT(m, 0, 1), AT(m, 0, 1)};
    const float vec2[4] = {AT(m, 1, 2), AT(m, 0, 2), AT(m, 0, 2), AT(m, 0, 2)};
    const float vec3[4] = {AT(m, 1, 3), AT(m, 0, 3), AT(m, 0, 3), AT(m, 0, 3)};
    const float sign_a[4] = {+1.0f, -1.0f, +1.0f, -1.0f};
    const float sign_b[4] = {-1.0f, +1.0f, -1.0f, +1.0f};

    float inv[16];
    for (int i = 0; i < 4; i++)
    {
        AT(inv, 0, i) = (vec1[i] * fac0[i] - vec2[i] * fac1[i] + vec3[i] * fac2[i]) * sign_a[i];
        AT(inv, 1, i) = (vec0[i] * fac0[i] - vec2[i] * fac3[i] + vec3[i] * fac4[i]) * sign_b[i];
        AT(inv, 2, i) = (vec0[i] * fac1[i] - vec1[i] * fac3[i] + vec3[i] * fac5[i]) * sign_a[i];
        AT(inv, 3, i) = (vec0[i] * fac2[i] - vec1[i] * fac4[i] + vec2[i] * fac5[i]) * sign_b[i];
    }
    const float dot0 = AT(m, 0, 0) * AT(inv, 0, 0);
    const float dot1 = AT(m, 0, 1) * AT(inv, 1, 0);
    const float dot2 = AT(m, 0, 2) * AT(inv, 2, 0);
    const float dot3 = AT(m, 0, 3) * AT(inv, 3, 0);
    const float det = (dot0 + dot1) + (dot2 + dot3);
    const float one_over_det = 1.0f / det;
    for (int k = 0; k < 16; k++)
        out[k] = inv[k] * one_over_det;
}

static void normalize3(const float *v, float *o)
{
    const float d = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    const float s = 1.0f / sqrtf(d);
    o[0] = v[0] * s;
    o[1] = v[1] * s;
    o[2] = v[2] * s;
}

static void axis_angle(const float *m, float *axis, float *angle)
{
    const float eps = FLT_EPSILON * 100.0f;
    const float pi = 3.14159265358979323846f;
    if (fabsf(AT(m, 1, 0) - AT(m, 0, 1)) < eps && fabsf(AT(m, 2, 0) - AT(m, 0, 2)) < eps &&
        fabsf(AT(m, 2, 1) - AT(m, 1, 2)) < eps)
    {
        if (fabsf(AT(m, 1, 0) + AT(m, 0, 1)) < eps && fabsf(AT(m, 2, 0) + AT(m, 0, 2)) < eps &&
            fabsf(AT(m, 2, 1) + AT(m, 1, 2)) < eps && fabsf(AT(m, 0, 0) + AT(m, 1, 1) + AT(m, 2, 2) - 3.0f) < eps)
        {
            *angle = 0.0f;
            axis[0] = 1.0f;
            axis[1] = 0.0f;
            axis[2] = 0.0f;
            return;
        }
        *angle = pi;
        const float xx = (AT(m, 0, 0) + 1.0f) * 0.5f;
        const float yy = (AT(m, 1, 1) + 1.0f) * 0.5f;
        const float zz = (AT(m, 2, 2) + 1.0f) * 0.5f;
        const float xy = (AT(m, 1, 0) + AT(m, 0, 1)) * 0.25f;
        const float xz = (AT(m, 2, 0) + AT(m, 0, 2)) * 0.25f;
        const float yz = (AT(m, 2, 1) + AT(m, 1, 2)) * 0.25f;
        if (xx > yy && xx > zz)
        {
            if (xx < eps)
            {
                axis[0] = 0.0f;
                axis[1] = 0.7071f;
                axis[2] = 0.7071f;
            }
            else
            {
                axis[0] = sqrtf(xx);
                axis[1] = xy / axis[0];
                axis[2] = xz / axis[0];
            }
        }
        else if (yy > zz)
        {
            if (yy < eps)
            {
                axis[0] = 0.7071f;
                axis[1] = 0.0f;
                axis[2] = 0.7071f;
            }
            else
            {
                axis[1] = sqrtf(yy);
                axis[0] = xy / axis[1];
                axis[2] = yz / axis[1];
            }
        }
        else
        {
            if (zz < eps)
            {
                axis[0] = 0.7071f;
                axis[1] = 0.7071f;
                axis[2] = 0.0f;
            }
            else
            {
                axis[2] = sqrtf(zz);
                axis[0] = xz / axis[2];
                axis[1] = yz / axis[2];
            }
        }
        return;
    }
    const float c = (AT(m, 0, 0) + AT(m, 1, 1) + AT(m, 2, 2) - 1.0f) * 0.5f;
    if (c >= 1.0f)
        *angle = 0.0f;
    else if (c <= -1.0f)
        *angle = pi;
    else
        *angle = acosf(c);
    const float v[3] = {AT(m, 1, 2) - AT(m, 2, 1), AT(m, 2, 0) - AT(m, 0, 2), AT(m, 0, 1) - AT(m, 1, 0)};
    normalize3(v, axis);
}

void oracle_mat4_interpolate(const float *m1, const float *m2, float delta, float *out)
{
    float rot[16] = {0}, rot_t[16], dlt[16];
    for (int c = 0; c < 3; c++)
        for (int r = 0; r < 3; r++)
            AT(rot, c, r) = AT(m1, c, r);
    AT(rot, 3, 3) = 1.0f;
    for (int c = 0; c < 4; c++)
        for (int r = 0; r < 4; r++)
            AT(rot_t, c, r) = AT(rot, r, c);
    oracle_mat4_mul(m2, rot_t, dlt);
    float axis[3], angle;
    axis_angle(dlt, axis, &angle);
    const float a = angle * delta;
    const float co = cosf(a), si = sinf(a), t = 1.0f - co;
    float n[3];
    normalize3(axis, n);
    float rm[16] = {0};
    AT(rm, 0, 0) = t * n[0] * n[0] + co;
    AT(rm, 0, 1) = t * n[0] * n[1] + n[2] * si;
    AT(rm, 0, 2) = t * n[0] * n[2] - n[1] * si;
    AT(rm, 1, 0) = t * n[0] * n[1] - n[2] * si;
    AT(rm, 1, 1) = t * n[1] * n[1] + co;
    AT(rm, 1, 2) = t * n[1] * n[2] + n[0] * si;
    AT(rm, 2, 0) = t * n[0] * n[2] + n[1] * si;
    AT(rm, 2, 1) = t * n[1] * n[2] - n[0] * si;
    AT(rm, 2, 2) = t * n[2] * n[2] + co;
    AT(rm, 3, 3) = 1.0f;
    oracle_mat4_mul(rm, rot, out);
    for (int r = 0; r < 3; r++)
        AT(out, 3, r) = AT(m1, 3, r) + delta * (AT(m2, 3, r) - AT(m1, 3, r));
}

void oracle_normalize_proj(const float *proj, float *out)
{
    /* include/file_reader.h:64-66, column by column */
    static const float reverse_z[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, -1, 0, 0, 0, 1, 1};
    static const float depth_01_to_11[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 2, 0, 0, 0, -1, 1};
    static const float unity_2022_3[16] = {1, 0, 0, 0, 0, -1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    float a[16], b[16];
    oracle_mat4_mul(reverse_z, proj, a);
    oracle_mat4_mul(depth_01_to_11, a, b);
    oracle_mat4_mul(unity_2022_3, b, out);
}
