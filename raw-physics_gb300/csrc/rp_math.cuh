// Device math for the XPBD step, templated on the scalar type.
//
// Every helper keeps the association and operand order of raw-physics' own math
// (include/gm.h:380-790, src/quaternion.cpp:3-273) so that the all-FP64 build of the step, compiled
// without FMA contraction, reproduces the reference's FP64 results bit for bit. The FP32 build uses
// the same formulas with contraction allowed.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define RP_HD __host__ __device__ __forceinline__

namespace rp {

// The reference's "zero length" threshold 1e-50 (pbd_base_constraints.cpp:23, pbd.cpp:304). It
// underflows FP32, where "c <= 1e-50" is "c == 0".
template <typename T> struct Tiny;
template <> struct Tiny<double> { static constexpr double v = 1e-50; };
template <> struct Tiny<float> { static constexpr float v = 0.0f; };

template <typename T> struct V3 { T x, y, z; };
template <typename T> struct Qt { T x, y, z, w; };
template <typename T> struct M3 { T d[3][3]; };

template <typename T> RP_HD V3<T> v3(T x, T y, T z) { V3<T> r; r.x = x; r.y = y; r.z = z; return r; }
template <typename T, typename U> RP_HD V3<T> v3cast(const V3<U>& a) { return v3<T>((T)a.x, (T)a.y, (T)a.z); }
template <typename T> RP_HD V3<T> vadd(V3<T> a, V3<T> b) { return v3<T>(a.x + b.x, a.y + b.y, a.z + b.z); }
template <typename T> RP_HD V3<T> vsub(V3<T> a, V3<T> b) { return v3<T>(a.x - b.x, a.y - b.y, a.z - b.z); }
template <typename T> RP_HD V3<T> vscale(T s, V3<T> v) { return v3<T>(s * v.x, s * v.y, s * v.z); }
template <typename T> RP_HD T vdot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <typename T> RP_HD V3<T> vcross(V3<T> a, V3<T> b) {
    return v3<T>(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
template <typename T> RP_HD T vlen(V3<T> v) { return sqrt(v.x * v.x + v.y * v.y + v.z * v.z); }
template <typename T> RP_HD V3<T> vnorm(V3<T> v) {
    if (!(v.x != (T)0 || v.y != (T)0 || v.z != (T)0)) return v3<T>(0, 0, 0);
    T l = vlen(v);
    return v3<T>(v.x / l, v.y / l, v.z / l);
}
template <typename T> RP_HD V3<T> vinv(V3<T> v) { return vsub(v3<T>(0, 0, 0), v); }
#ifdef __CUDACC__
// FP64 unit vector without FP64 square root or division (GB300 issues FP64 at 1/64 of the FP32
// rate): an FP32 reciprocal-square-root seed refined by two Newton-Raphson steps,
// r <- r (3 - d r^2) / 2, which reach full FP64 precision from the seed's ~23 bits. Lengths outside
// the FP32 exponent range take the exact path. For the FP32 build's FP64 decisions; the exact build
// keeps vnorm (the reference's sqrt and divisions).
__device__ __forceinline__ V3<double> vnorm_fast(V3<double> v) {
    const double d = v.x * v.x + v.y * v.y + v.z * v.z;
    if (!(d > 0.0)) return v3<double>(0, 0, 0);
    if (d < 1e-30 || d > 1e30) return vnorm(v);
    double r = (double)rsqrtf((float)d);
    r = r * (1.5 - 0.5 * d * r * r);
    r = r * (1.5 - 0.5 * d * r * r);
    return v3<double>(v.x * r, v.y * r, v.z * r);
}
#endif
template <typename T> RP_HD bool veq(V3<T> a, V3<T> b) { return a.x == b.x && a.y == b.y && a.z == b.z; }

template <typename T> RP_HD Qt<T> qt(T x, T y, T z, T w) { Qt<T> q; q.x = x; q.y = y; q.z = z; q.w = w; return q; }
template <typename T, typename U> RP_HD Qt<T> qcast(const Qt<U>& a) { return qt<T>((T)a.x, (T)a.y, (T)a.z, (T)a.w); }
template <typename T> RP_HD Qt<T> qmul(Qt<T> a, Qt<T> b) {
    Qt<T> r;
    r.w = a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z;
    r.x = a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y;
    r.y = a.w * b.y + a.y * b.w + a.z * b.x - a.x * b.z;
    r.z = a.w * b.z + a.z * b.w + a.x * b.y - a.y * b.x;
    return r;
}
template <typename T> RP_HD Qt<T> qnormalize(Qt<T> q) {
    T l = sqrt(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w);
    return qt<T>(q.x / l, q.y / l, q.z / l, q.w / l);
}
template <typename T> RP_HD Qt<T> qinverse(Qt<T> q) { return qt<T>(-q.x, -q.y, -q.z, q.w); }
template <typename T> RP_HD V3<T> qrotate(Qt<T> q, V3<T> v) {
    T ix = q.w * v.x + q.y * v.z - q.z * v.y;
    T iy = q.w * v.y + q.z * v.x - q.x * v.z;
    T iz = q.w * v.z + q.x * v.y - q.y * v.x;
    T iw = -q.x * v.x - q.y * v.y - q.z * v.z;
    return v3<T>((ix * q.w) + (iw * -q.x) + (iy * -q.z) - (iz * -q.y),
                 (iy * q.w) + (iw * -q.y) + (iz * -q.x) - (ix * -q.z),
                 (iz * q.w) + (iw * -q.z) + (ix * -q.y) - (iy * -q.x));
}
template <typename T> RP_HD M3<T> qmat3(Qt<T> q) {
    M3<T> r;
    r.d[0][0] = (T)1.0 - (T)2.0 * q.y * q.y - (T)2.0 * q.z * q.z;
    r.d[1][0] = (T)2.0 * q.x * q.y + (T)2.0 * q.w * q.z;
    r.d[2][0] = (T)2.0 * q.x * q.z - (T)2.0 * q.w * q.y;
    r.d[0][1] = (T)2.0 * q.x * q.y - (T)2.0 * q.w * q.z;
    r.d[1][1] = (T)1.0 - ((T)2.0 * q.x * q.x) - ((T)2.0 * q.z * q.z);
    r.d[2][1] = (T)2.0 * q.y * q.z + (T)2.0 * q.w * q.x;
    r.d[0][2] = (T)2.0 * q.x * q.z + (T)2.0 * q.w * q.y;
    r.d[1][2] = (T)2.0 * q.y * q.z - (T)2.0 * q.w * q.x;
    r.d[2][2] = (T)1.0 - ((T)2.0 * q.x * q.x) - ((T)2.0 * q.y * q.y);
    return r;
}
// Body axes in world coordinates, indexed by PBD_Axis_Type (src/physics/pbd.cpp:219-243,
// src/quaternion.cpp:33-78).
template <typename T> RP_HD V3<T> qaxis(Qt<T> q, int axis) {
    const T one = 1.0, two = 2.0;
    switch (axis) {
    case 0: return v3<T>(one - two * q.y * q.y - two * q.z * q.z, two * q.x * q.y - two * -q.w * q.z, two * q.x * q.z + two * -q.w * q.y);
    case 1: return v3<T>(one - two * q.y * q.y - two * q.z * q.z, two * q.x * q.y - two * q.w * q.z, two * q.x * q.z + two * q.w * q.y);
    case 2: return v3<T>(two * q.x * q.y + two * -q.w * q.z, one - (two * q.x * q.x) - (two * q.z * q.z), two * q.y * q.z - two * -q.w * q.x);
    case 3: return v3<T>(two * q.x * q.y + two * q.w * q.z, one - (two * q.x * q.x) - (two * q.z * q.z), two * q.y * q.z - two * q.w * q.x);
    case 4: return v3<T>(two * q.x * q.z - two * -q.w * q.y, two * q.y * q.z + two * -q.w * q.x, one - (two * q.x * q.x) - (two * q.y * q.y));
    default: return v3<T>(two * q.x * q.z - two * q.w * q.y, two * q.y * q.z + two * q.w * q.x, one - (two * q.x * q.x) - (two * q.y * q.y));
    }
}

template <typename T> RP_HD M3<T> mmul(const M3<T>& a, const M3<T>& b) {
    M3<T> r;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) r.d[i][j] = a.d[i][0] * b.d[0][j] + a.d[i][1] * b.d[1][j] + a.d[i][2] * b.d[2][j];
    return r;
}
template <typename T> RP_HD M3<T> mtranspose(const M3<T>& a) {
    M3<T> r;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) r.d[i][j] = a.d[j][i];
    return r;
}
template <typename T> RP_HD V3<T> mmulv(const M3<T>& m, V3<T> v) {
    return v3<T>(m.d[0][0] * v.x + m.d[0][1] * v.y + m.d[0][2] * v.z, m.d[1][0] * v.x + m.d[1][1] * v.y + m.d[1][2] * v.z,
                 m.d[2][0] * v.x + m.d[2][1] * v.y + m.d[2][2] * v.z);
}
// Symmetric 3x3 stored as xx, yy, zz, xy, xz, yz (the reference's inertia tensors are exactly
// symmetric: colliders_get_default_inertia_tensor writes both off-diagonal halves with the same
// expression, and gm_mat3_inverse of a symmetric matrix multiplies the same operands).
template <typename T> RP_HD M3<T> msym(const T s[6]) {
    M3<T> r;
    r.d[0][0] = s[0]; r.d[1][1] = s[1]; r.d[2][2] = s[2];
    r.d[0][1] = s[3]; r.d[1][0] = s[3];
    r.d[0][2] = s[4]; r.d[2][0] = s[4];
    r.d[1][2] = s[5]; r.d[2][1] = s[5];
    return r;
}
// R * I_local * R^T (get_dynamic_(inverse_)inertia_tensor, src/physics/physics_util.cpp:26-63)
template <typename T> RP_HD M3<T> world_tensor(Qt<T> q, const M3<T>& local) {
    M3<T> r = qmat3(q);
    M3<T> rt = mtranspose(r);
    M3<T> aux = mmul(r, local);
    return mmul(aux, rt);
}

// util_get_model_matrix_no_scale (src/util.cpp:60-74) as the 4x4 product translation * rotation,
// evaluated term by term so the FP64 result matches the reference's, then the point transform of
// collider_update (src/physics/collider.cpp:414-422) including its divide by w.
template <typename T> struct M4 { T d[4][4]; };
template <typename T> RP_HD M4<T> model_matrix(Qt<T> q, V3<T> t) {
    M3<T> r = qmat3(q);
    T rr[4][4], tr[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            rr[i][j] = (i < 3 && j < 3) ? r.d[i][j] : ((i == 3 && j == 3) ? (T)1 : (T)0);
            tr[i][j] = (i == j) ? (T)1 : (T)0;
        }
    tr[0][3] = t.x; tr[1][3] = t.y; tr[2][3] = t.z;
    M4<T> m;
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) m.d[i][j] = tr[i][0] * rr[0][j] + tr[i][1] * rr[1][j] + tr[i][2] * rr[2][j] + tr[i][3] * rr[3][j];
    return m;
}
template <typename T> RP_HD V3<T> m4_point(const M4<T>& m, V3<T> p) {
    T x = p.x * m.d[0][0] + p.y * m.d[0][1] + p.z * m.d[0][2] + (T)1 * m.d[0][3];
    T y = p.x * m.d[1][0] + p.y * m.d[1][1] + p.z * m.d[1][2] + (T)1 * m.d[1][3];
    T z = p.x * m.d[2][0] + p.y * m.d[2][1] + p.z * m.d[2][2] + (T)1 * m.d[2][3];
    T w = p.x * m.d[3][0] + p.y * m.d[3][1] + p.z * m.d[3][2] + (T)1 * m.d[3][3];
    T s = (T)1 / w;
    return v3<T>(s * x, s * y, s * z);
}
template <typename T> RP_HD V3<T> m4_dir(const M4<T>& m, V3<T> v) {
    return v3<T>(m.d[0][0] * v.x + m.d[0][1] * v.y + m.d[0][2] * v.z, m.d[1][0] * v.x + m.d[1][1] * v.y + m.d[1][2] * v.z,
                 m.d[2][0] * v.x + m.d[2][1] * v.y + m.d[2][2] * v.z);
}

}  // namespace rp
