/*
 * FP64 vector / quaternion / matrix helpers of the oracle port — TEST INFRASTRUCTURE ONLY.
 *
 * Every helper keeps the exact association and operand order of the reference's math so that,
 * compiled with -ffp-contract=off, the port reproduces the reference bit for bit:
 *   vec3 ops       include/gm.h:611-790 (gm_vec3_*), normalize returns 0 for the zero vector (:664)
 *   mat3 / mat4    include/gm.h:380-470 (gm_mat3_inverse, gm_mat3_multiply, gm_mat4_multiply_vec4 ...)
 *   quaternions    src/quaternion.cpp:3-273
 */
#ifndef RP_ORACLE_MATH_H
#define RP_ORACLE_MATH_H
#include <math.h>

typedef struct { double x, y, z; } v3;
typedef struct { double x, y, z, w; } qt;
typedef struct { double d[3][3]; } m3;
typedef struct { double d[4][4]; } m4;

static inline v3 V3(double x, double y, double z) { v3 r; r.x = x; r.y = y; r.z = z; return r; }
static inline v3 v_add(v3 a, v3 b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 v_sub(v3 a, v3 b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 v_scale(double s, v3 v) { return V3(s * v.x, s * v.y, s * v.z); }
static inline double v_dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline v3 v_cross(v3 a, v3 b) {
    return V3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline double v_len(v3 v) { return sqrt(v.x * v.x + v.y * v.y + v.z * v.z); }
static inline v3 v_norm(v3 v) {
    if (!(v.x != 0.0 || v.y != 0.0 || v.z != 0.0)) return V3(0.0, 0.0, 0.0);
    double l = v_len(v);
    return V3(v.x / l, v.y / l, v.z / l);
}
static inline v3 v_inv(v3 v) { return v_sub(V3(0.0, 0.0, 0.0), v); }
static inline int v_eq(v3 a, v3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }

static inline qt Q(double x, double y, double z, double w) { qt q; q.x = x; q.y = y; q.z = z; q.w = w; return q; }
static inline qt q_mul(qt a, qt b) {
    qt r;
    r.w = a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z;
    r.x = a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y;
    r.y = a.w * b.y + a.y * b.w + a.z * b.x - a.x * b.z;
    r.z = a.w * b.z + a.z * b.w + a.x * b.y - a.y * b.x;
    return r;
}
static inline qt q_normalize(qt q) {
    double l = sqrt(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w);
    return Q(q.x / l, q.y / l, q.z / l, q.w / l);
}
static inline qt q_inverse(qt q) { return Q(-q.x, -q.y, -q.z, q.w); }
static inline v3 q_rotate(qt q, v3 v) {
    double ix = q.w * v.x + q.y * v.z - q.z * v.y;
    double iy = q.w * v.y + q.z * v.x - q.x * v.z;
    double iz = q.w * v.z + q.x * v.y - q.y * v.x;
    double iw = -q.x * v.x - q.y * v.y - q.z * v.z;
    return V3((ix * q.w) + (iw * -q.x) + (iy * -q.z) - (iz * -q.y),
              (iy * q.w) + (iw * -q.y) + (iz * -q.x) - (ix * -q.z),
              (iz * q.w) + (iw * -q.z) + (ix * -q.y) - (iy * -q.x));
}
static inline m3 q_mat3(qt q) {
    m3 r;
    r.d[0][0] = 1.0 - 2.0 * q.y * q.y - 2.0 * q.z * q.z;
    r.d[1][0] = 2.0 * q.x * q.y + 2.0 * q.w * q.z;
    r.d[2][0] = 2.0 * q.x * q.z - 2.0 * q.w * q.y;
    r.d[0][1] = 2.0 * q.x * q.y - 2.0 * q.w * q.z;
    r.d[1][1] = 1.0 - (2.0 * q.x * q.x) - (2.0 * q.z * q.z);
    r.d[2][1] = 2.0 * q.y * q.z + 2.0 * q.w * q.x;
    r.d[0][2] = 2.0 * q.x * q.z + 2.0 * q.w * q.y;
    r.d[1][2] = 2.0 * q.y * q.z - 2.0 * q.w * q.x;
    r.d[2][2] = 1.0 - (2.0 * q.x * q.x) - (2.0 * q.y * q.y);
    return r;
}
static inline m4 q_mat4(qt q) {
    m4 r;
    m3 a = q_mat3(q);
    for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j) r.d[i][j] = a.d[i][j];
        r.d[3][i] = 0.0;
        r.d[i][3] = 0.0;
    }
    r.d[3][3] = 1.0;
    return r;
}
/* quaternion_get_right / up / forward and their *_inverted forms (src/quaternion.cpp:33-78) */
static inline v3 q_axis(qt q, int axis) {
    switch (axis) {
    case 0: return V3(1.0 - 2.0 * q.y * q.y - 2.0 * q.z * q.z, 2.0 * q.x * q.y - 2.0 * -q.w * q.z,
                      2.0 * q.x * q.z + 2.0 * -q.w * q.y);
    case 1: return V3(1.0 - 2.0 * q.y * q.y - 2.0 * q.z * q.z, 2.0 * q.x * q.y - 2.0 * q.w * q.z,
                      2.0 * q.x * q.z + 2.0 * q.w * q.y);
    case 2: return V3(2.0 * q.x * q.y + 2.0 * -q.w * q.z, 1.0 - (2.0 * q.x * q.x) - (2.0 * q.z * q.z),
                      2.0 * q.y * q.z - 2.0 * -q.w * q.x);
    case 3: return V3(2.0 * q.x * q.y + 2.0 * q.w * q.z, 1.0 - (2.0 * q.x * q.x) - (2.0 * q.z * q.z),
                      2.0 * q.y * q.z - 2.0 * q.w * q.x);
    case 4: return V3(2.0 * q.x * q.z - 2.0 * -q.w * q.y, 2.0 * q.y * q.z + 2.0 * -q.w * q.x,
                      1.0 - (2.0 * q.x * q.x) - (2.0 * q.y * q.y));
    default: return V3(2.0 * q.x * q.z - 2.0 * q.w * q.y, 2.0 * q.y * q.z + 2.0 * q.w * q.x,
                       1.0 - (2.0 * q.x * q.x) - (2.0 * q.y * q.y));
    }
}
static inline qt q_from_axis_angle(v3 axis, double angle) {
    if (v_len(axis) != 0.0) axis = v_norm(axis);
    double s = sin(angle / 2.0);
    return Q(axis.x * s, axis.y * s, axis.z * s, cos(angle / 2.0));
}

static inline m3 m3_mul(m3 a, m3 b) {
    m3 r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            r.d[i][j] = a.d[i][0] * b.d[0][j] + a.d[i][1] * b.d[1][j] + a.d[i][2] * b.d[2][j];
    return r;
}
static inline m3 m3_transpose(m3 a) {
    m3 r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r.d[i][j] = a.d[j][i];
    return r;
}
static inline v3 m3_mulv(m3 m, v3 v) {
    return V3(m.d[0][0] * v.x + m.d[0][1] * v.y + m.d[0][2] * v.z,
              m.d[1][0] * v.x + m.d[1][1] * v.y + m.d[1][2] * v.z,
              m.d[2][0] * v.x + m.d[2][1] * v.y + m.d[2][2] * v.z);
}
static inline int m3_inverse(m3 m, m3* out) {
    double det = m.d[0][0] * (m.d[1][1] * m.d[2][2] - m.d[2][1] * m.d[1][2]) -
                 m.d[0][1] * (m.d[1][0] * m.d[2][2] - m.d[1][2] * m.d[2][0]) +
                 m.d[0][2] * (m.d[1][0] * m.d[2][1] - m.d[1][1] * m.d[2][0]);
    if (det == 0.0) return 0;
    double inv = 1 / det;
    out->d[0][0] = (m.d[1][1] * m.d[2][2] - m.d[2][1] * m.d[1][2]) * inv;
    out->d[0][1] = (m.d[0][2] * m.d[2][1] - m.d[0][1] * m.d[2][2]) * inv;
    out->d[0][2] = (m.d[0][1] * m.d[1][2] - m.d[0][2] * m.d[1][1]) * inv;
    out->d[1][0] = (m.d[1][2] * m.d[2][0] - m.d[1][0] * m.d[2][2]) * inv;
    out->d[1][1] = (m.d[0][0] * m.d[2][2] - m.d[0][2] * m.d[2][0]) * inv;
    out->d[1][2] = (m.d[1][0] * m.d[0][2] - m.d[0][0] * m.d[1][2]) * inv;
    out->d[2][0] = (m.d[1][0] * m.d[2][1] - m.d[2][0] * m.d[1][1]) * inv;
    out->d[2][1] = (m.d[2][0] * m.d[0][1] - m.d[0][0] * m.d[2][1]) * inv;
    out->d[2][2] = (m.d[0][0] * m.d[1][1] - m.d[1][0] * m.d[0][1]) * inv;
    return 1;
}
static inline m4 m4_mul(m4 a, m4 b) {
    m4 r;
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
            r.d[i][j] = a.d[i][0] * b.d[0][j] + a.d[i][1] * b.d[1][j] + a.d[i][2] * b.d[2][j] + a.d[i][3] * b.d[3][j];
    return r;
}
/* util_get_model_matrix_no_scale (src/util.cpp:60-74): translation * rotation */
static inline m4 model_matrix_no_scale(qt q, v3 t) {
    m4 tr;
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) tr.d[i][j] = (i == j) ? 1.0 : 0.0;
    tr.d[0][3] = t.x;
    tr.d[1][3] = t.y;
    tr.d[2][3] = t.z;
    return m4_mul(tr, q_mat4(q));
}
/* gm_mat4_multiply_vec4 of (p,1) followed by the divide by w (src/physics/collider.cpp:414-422) */
static inline v3 m4_transform_point(m4 m, v3 p) {
    double x = p.x * m.d[0][0] + p.y * m.d[0][1] + p.z * m.d[0][2] + 1.0 * m.d[0][3];
    double y = p.x * m.d[1][0] + p.y * m.d[1][1] + p.z * m.d[1][2] + 1.0 * m.d[1][3];
    double z = p.x * m.d[2][0] + p.y * m.d[2][1] + p.z * m.d[2][2] + 1.0 * m.d[2][3];
    double w = p.x * m.d[3][0] + p.y * m.d[3][1] + p.z * m.d[3][2] + 1.0 * m.d[3][3];
    double s = 1.0 / w;
    return V3(s * x, s * y, s * z);
}
/* gm_mat4_multiply_vec3(m, v, false) */
static inline v3 m4_transform_dir(m4 m, v3 v) {
    return V3(m.d[0][0] * v.x + m.d[0][1] * v.y + m.d[0][2] * v.z,
              m.d[1][0] * v.x + m.d[1][1] * v.y + m.d[1][2] * v.z,
              m.d[2][0] * v.x + m.d[2][1] * v.y + m.d[2][2] * v.z);
}
#endif
