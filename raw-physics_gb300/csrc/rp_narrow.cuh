// Warp-per-pair narrowphase: support mapping, GJK, EPA and contact-manifold clipping.
//
// One warp handles one broad-phase pair. The pair's transformed hull vertices are staged in the
// warp's shared-memory slice; support mapping is a warp argmax; GJK's simplex logic runs
// redundantly on all lanes; EPA keeps its polytope in shared memory, tests face visibility and
// builds new faces lane-parallel, and replays the reference's order-dependent bookkeeping (the
// unordered removal of faces and horizon edges) on lane 0 so that face order — and so every
// tie-break — is the reference's. Clipping runs Sutherland–Hodgman one plane at a time with one
// lane per polygon edge and a warp prefix sum to keep the output order.
//
// References (raw-physics): support.cpp:5-39, gjk.cpp:7-379, epa.cpp:8-237, clipping.cpp:12-370,
// collider.cpp:523-571.
#pragma once
#include <type_traits>
#include <float.h>
#include "rp_math.cuh"
#include "rp_world.h"

namespace rp {

constexpr int WARP = 32;
constexpr int STAGE_V = 64;      // hull vertices staged per body in shared memory
constexpr int EPA_MAXV = 104;    // 4 simplex points + at most 100 EPA iterations
constexpr int EPA_MAXF = 192;    // faces of the EPA polytope
constexpr int EPA_MAXE = 64;     // horizon edges of one EPA iteration (two register slots per lane)
constexpr int CLIP_MAX = 96;     // vertices of a clipped polygon
constexpr int CMAX = 64;         // contacts of one body pair

// Precision policy. R: working type of geometry and solver. EPA face normals, distances and the
// termination test are always FP64.
// EPA of the FP32 build. 1 (default): polytope faces and the closest-face search in FP32, the
// termination test and the returned normal and depth in FP64 (the closest face re-evaluated from its
// three Minkowski points every iteration). 0: every face normal and distance in FP64, which on GB300
// (FP64 at 1/64 of the FP32 rate) made EPA the most expensive part of the batched narrowphase.
#ifndef RP_EPA_FAST
#define RP_EPA_FAST 1
#endif
constexpr bool kEpaFast = RP_EPA_FAST != 0;

template <bool EXACT> struct Prec;
template <> struct Prec<false> { typedef float R; static constexpr bool exact = false; };
template <> struct Prec<true> { typedef double R; static constexpr bool exact = true; };

// The FP32 build's EPA polytope (epa_fast): FP32 points, face normals and distances; the closest
// face is re-evaluated in FP64 before it is returned.
template <typename R>
struct EpaFastSmem {
    V3<float> poly[EPA_MAXV];
    V3<float> fn[EPA_MAXF];
    float fd[EPA_MAXF];
    uchar4 f[EPA_MAXF];
    uchar2 edge[3 * WARP];   // edges of this iteration's visible faces
    uchar2 hz[3 * WARP];     // the horizon
};

// The exact build's EPA polytope (epa): FP64 face normals and distances.
template <typename R>
struct EpaExactSmem {
    V3<R> poly[EPA_MAXV];
    V3<double> fn[EPA_MAXF];
    double fd[EPA_MAXF];
    uchar4 f[EPA_MAXF];      // x, y, z polytope indices, w = visibility
};

template <typename R>
struct NarrowSmem {
    V3<R> va[STAGE_V];
    V3<R> vb[STAGE_V];
    union U {
        // the FP32 build runs epa_fast only, so its scratch holds the FP32 polytope
        typename std::conditional<std::is_same<R, float>::value && (RP_EPA_FAST != 0), EpaFastSmem<R>, EpaExactSmem<R>>::type epa;
        struct {
            V3<R> buf[2][CLIP_MAX];
            V3<R> pn[CLIP_MAX];      // clip planes: normal
            V3<R> pp[CLIP_MAX];      // clip planes: point
            int32_t cand[WARP * 2];  // edge-pair candidates
        } clip;
        __device__ U() {}
    } u;
    V3<R> c_r1[CMAX];   // contacts of the pair (constraint-ready local offsets)
    V3<R> c_r2[CMAX];
    V3<R> c_n[CMAX];
    R gjk_saved[16];    // GJK state kept for cycle detection (simplex, size, direction)
    int ncontacts;
    int nf, ne, npoly;
    int status;
};

// ---------------------------------------------------------------------------------------------
// Warp utilities
__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

// argmax with the reference's "strict >, first index wins" rule (support.cpp:8-14)
template <typename T>
__device__ __forceinline__ void warp_argmax_first(T& v, int& idx) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        T ov = __shfl_xor_sync(0xffffffffu, v, o);
        int oi = __shfl_xor_sync(0xffffffffu, idx, o);
        if (ov > v || (ov == v && oi < idx)) { v = ov; idx = oi; }
    }
}
template <typename T>
__device__ __forceinline__ void warp_argmin_first(T& v, int& idx) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        T ov = __shfl_xor_sync(0xffffffffu, v, o);
        int oi = __shfl_xor_sync(0xffffffffu, idx, o);
        if (ov < v || (ov == v && oi < idx)) { v = ov; idx = oi; }
    }
}
// FP32 specialisations on the warp-reduce unit: the value as an order-preserving unsigned key
// (-0 folded onto +0, so equal floats give equal keys), one reduction for the extreme key, one for the
// smallest index among the lanes that hold it: the same "first index wins" result as the shuffle
// rounds above, in two instructions. (Lane values are never NaN: every caller starts from +-FLT_MAX
// and keeps a value only through a strict comparison.)
__device__ __forceinline__ unsigned f32_order_key(float f) {
    const unsigned b = __float_as_uint(f + 0.0f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float f32_from_order_key(unsigned k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}
__device__ __forceinline__ void warp_argmax_first(float& v, int& idx) {
    const unsigned k = f32_order_key(v);
    const unsigned m = __reduce_max_sync(0xffffffffu, k);
    idx = (int)__reduce_min_sync(0xffffffffu, k == m ? (unsigned)idx : 0xffffffffu);
    v = f32_from_order_key(m);
}
__device__ __forceinline__ void warp_argmin_first(float& v, int& idx) {
    const unsigned k = f32_order_key(v);
    const unsigned m = __reduce_min_sync(0xffffffffu, k);
    idx = (int)__reduce_min_sync(0xffffffffu, k == m ? (unsigned)idx : 0xffffffffu);
    v = f32_from_order_key(m);
}

__device__ __forceinline__ int warp_incl_scan(int x) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if ((int)lane_id() >= o) x += y;
    }
    return x;
}

// ---------------------------------------------------------------------------------------------
// A collider as seen by the narrowphase: transformed vertices and normals (exact build: world
// coordinates; FP32 build: rotated about the body origin, plus `off` for the pair-local frame).
template <typename R>
struct ColView {
    int type;
    R radius;
    V3<R> center;            // sphere centre (pair frame)
    V3<R> off;               // translation added to stored vertices (pair frame)
    const V3<R>* verts;      // stored transformed vertices (shared staging or global)
    bool staged;             // verts already include `off`
    const V3<R>* norms;      // transformed face normals (global)
    int nv, nf;
    const Shape* shape;
    int body;                // the body's slot (its FP64 orientation is read only for decisions made in FP64)
};

// A face normal of a hull rotated by the body's FP64 orientation (collider_update's normal
// transform, collider.cpp:425-429), for the FP32 build's FP64 reference-face decision.
template <typename R>
__device__ __forceinline__ V3<double> face_normal64(const WorldView<R>& W, const ColView<R>& c, int f) {
    const double* n = W.face_normal + 3 * (c.shape->face_off + f);
    const double4_32a q = W.rot[c.body];
    return vnorm_fast(mmulv(qmat3(qt<double>(q.x, q.y, q.z, q.w)), v3<double>(n[0], n[1], n[2])));
}

template <typename R>
__device__ __forceinline__ V3<R> cv_vertex(const ColView<R>& c, int i) {
    V3<R> v = c.verts[i];
    if (!c.staged) v = vadd(v, c.off);
    return v;
}

// support_point_get_index: warp argmax over the hull's transformed vertices
template <typename R>
__device__ int support_index(const ColView<R>& c, V3<R> d) {
    R best = -(R)DBL_MAX;
    if (sizeof(R) == 4) best = -FLT_MAX;
    int bi = 0x7fffffff;
    for (int i = (int)lane_id(); i < c.nv; i += WARP) {
        R dot = vdot(cv_vertex(c, i), d);
        if (dot > best) { best = dot; bi = i; }
    }
    warp_argmax_first(best, bi);
    return bi == 0x7fffffff ? 0 : bi;
}

template <typename R>
__device__ V3<R> support_point(const ColView<R>& c, V3<R> d) {
    if (c.type == COL_HULL) return cv_vertex(c, support_index(c, d));
    return vadd(c.center, vscale(c.radius, vnorm(d)));
}

// support_point_of_minkowski_difference (support.cpp:29-39): both hulls' argmax reductions run
// interleaved, so each shuffle round waits for one shuffle latency instead of two.
template <typename R>
__device__ __forceinline__ V3<R> support_mink(const ColView<R>& a, const ColView<R>& b, V3<R> d) {
    const V3<R> nd = vscale((R)-1.0, d);
    if (a.type != COL_HULL || b.type != COL_HULL) return vsub(support_point(a, d), support_point(b, nd));
    const R lowest = sizeof(R) == 4 ? (R)-FLT_MAX : (R)-DBL_MAX;
    R ba = lowest, bb = lowest;
    int ia = 0x7fffffff, ib = 0x7fffffff;
    for (int i = (int)lane_id(); i < a.nv; i += WARP) {
        R dot = vdot(cv_vertex(a, i), d);
        if (dot > ba) { ba = dot; ia = i; }
    }
    for (int i = (int)lane_id(); i < b.nv; i += WARP) {
        R dot = vdot(cv_vertex(b, i), nd);
        if (dot > bb) { bb = dot; ib = i; }
    }
    if constexpr (sizeof(R) == 4) {
        warp_argmax_first(ba, ia);
        warp_argmax_first(bb, ib);
    } else {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            R ova = __shfl_xor_sync(0xffffffffu, ba, o), ovb = __shfl_xor_sync(0xffffffffu, bb, o);
            int oia = __shfl_xor_sync(0xffffffffu, ia, o), oib = __shfl_xor_sync(0xffffffffu, ib, o);
            if (ova > ba || (ova == ba && oia < ia)) { ba = ova; ia = oia; }
            if (ovb > bb || (ovb == bb && oib < ib)) { bb = ovb; ib = oib; }
        }
    }
    if (ia == 0x7fffffff) ia = 0;
    if (ib == 0x7fffffff) ib = 0;
    return vsub(cv_vertex(a, ia), cv_vertex(b, ib));
}

// ---------------------------------------------------------------------------------------------
// GJK (gjk.cpp:7-379); all lanes hold the same simplex.
template <typename R>
struct Simplex { V3<R> a, b, c, d; int num; };

template <typename R>
__device__ __forceinline__ V3<R> triple_cross(V3<R> a, V3<R> b, V3<R> c) { return vcross(vcross(a, b), c); }

template <typename R>
__device__ bool do_simplex(Simplex<R>& s, V3<R>& dir) {
    const R zero = 0;
    if (s.num == 2) {
        V3<R> a = s.a, b = s.b, ao = vinv(a), ab = vsub(b, a);
        if (vdot(ab, ao) >= zero) { s.a = a; s.b = b; s.num = 2; dir = triple_cross(ab, ao, ab); }
        else { s.a = a; s.num = 1; dir = ao; }
        return false;
    }
    if (s.num == 3) {
        V3<R> a = s.a, b = s.b, c = s.c;
        V3<R> ao = vinv(a), ab = vsub(b, a), ac = vsub(c, a), abc = vcross(ab, ac);
        if (vdot(vcross(abc, ac), ao) >= zero) {
            if (vdot(ac, ao) >= zero) { s.a = a; s.b = c; s.num = 2; dir = triple_cross(ac, ao, ac); }
            else if (vdot(ab, ao) >= zero) { s.a = a; s.b = b; s.num = 2; dir = triple_cross(ab, ao, ab); }
            else { s.a = a; dir = ao; }
        } else {
            if (vdot(vcross(ab, abc), ao) >= zero) {
                if (vdot(ab, ao) >= zero) { s.a = a; s.b = b; s.num = 2; dir = triple_cross(ab, ao, ab); }
                else { s.a = a; dir = ao; }
            } else {
                if (vdot(abc, ao) >= zero) { s.a = a; s.b = b; s.c = c; s.num = 3; dir = abc; }
                else { s.a = a; s.b = c; s.c = b; s.num = 3; dir = vinv(abc); }
            }
        }
        return false;
    }
    V3<R> a = s.a, b = s.b, c = s.c, d = s.d;
    V3<R> ao = vinv(a), ab = vsub(b, a), ac = vsub(c, a), ad = vsub(d, a);
    V3<R> abc = vcross(ab, ac), acd = vcross(ac, ad), adb = vcross(ad, ab);
    int info = 0;
    if (vdot(abc, ao) >= zero) info |= 1;
    if (vdot(acd, ao) >= zero) info |= 2;
    if (vdot(adb, ao) >= zero) info |= 4;
    switch (info) {
    case 0: return true;
    case 1:
        if (vdot(vcross(abc, ac), ao) >= zero) {
            if (vdot(ac, ao) >= zero) { s.a = a; s.b = c; s.num = 2; dir = triple_cross(ac, ao, ac); }
            else if (vdot(ab, ao) >= zero) { s.a = a; s.b = b; s.num = 2; dir = triple_cross(ab, ao, ab); }
            else { s.a = a; dir = ao; }
        } else {
            if (vdot(vcross(ab, abc), ao) >= zero) {
                if (vdot(ab, ao) >= zero) { s.a = a; s.b = b; s.num = 2; dir = triple_cross(ab, ao, ab); }
                else { s.a = a; dir = ao; }
            } else { s.a = a; s.b = b; s.c = c; s.num = 3; dir = abc; }
        }
        break;
    case 2:
        if (vdot(vcross(acd, ad), ao) >= zero) {
            if (vdot(ad, ao) >= zero) { s.a = a; s.b = d; s.num = 2; dir = triple_cross(ad, ao, ad); }
            else if (vdot(ac, ao) >= zero) {
                // the reference pairs the AC simplex with the AB search direction here (gjk.cpp:213)
                s.a = a; s.b = c; s.num = 2; dir = triple_cross(ab, ao, ab);
            } else { s.a = a; dir = ao; }
        } else {
            if (vdot(vcross(ac, acd), ao) >= zero) {
                if (vdot(ac, ao) >= zero) { s.a = a; s.b = c; s.num = 2; dir = triple_cross(ac, ao, ac); }
                else { s.a = a; dir = ao; }
            } else { s.a = a; s.b = c; s.c = d; s.num = 3; dir = acd; }
        }
        break;
    case 3:
        if (vdot(ac, ao) >= zero) { s.a = a; s.b = c; s.num = 2; dir = triple_cross(ac, ao, ac); }
        else { s.a = a; s.num = 1; dir = ao; }
        break;
    case 4:
        if (vdot(vcross(adb, ab), ao) >= zero) {
            if (vdot(ab, ao) >= zero) { s.a = a; s.b = b; s.num = 2; dir = triple_cross(ab, ao, ab); }
            else if (vdot(ad, ao) >= zero) { s.a = a; s.b = d; s.num = 2; dir = triple_cross(ad, ao, ad); }
            else { s.a = a; dir = ao; }
        } else {
            if (vdot(vcross(ad, adb), ao) >= zero) {
                if (vdot(ad, ao) >= zero) { s.a = a; s.b = d; s.num = 2; dir = triple_cross(ad, ao, ad); }
                else { s.a = a; dir = ao; }
            } else { s.a = a; s.b = d; s.c = b; s.num = 3; dir = adb; }
        }
        break;
    case 5:
        if (vdot(ab, ao) >= zero) { s.a = a; s.b = b; s.num = 2; dir = triple_cross(ab, ao, ab); }
        else { s.a = a; s.num = 1; dir = ao; }
        break;
    case 6:
        if (vdot(ad, ao) >= zero) { s.a = a; s.b = d; s.num = 2; dir = triple_cross(ad, ao, ad); }
        else { s.a = a; s.num = 1; dir = ao; }
        break;
    default: s.a = a; s.num = 1; dir = ao; break;
    }
    return false;
}

// Component k (0..15) of the GJK iteration state: simplex points a, b, c, d, the simplex size and
// the search direction. All lanes hold the same state.
template <typename R>
__device__ __forceinline__ R gjk_state(const Simplex<R>& s, V3<R> dir, int k) {
    R v[16] = {s.a.x, s.a.y, s.a.z, s.b.x, s.b.y, s.b.z, s.c.x, s.c.y, s.c.z, s.d.x, s.d.y, s.d.z,
               (R)s.num, dir.x, dir.y, dir.z};
    R r = v[0];
#pragma unroll
    for (int i = 1; i < 16; ++i) r = (k == i) ? v[i] : r;
    return r;
}
__device__ __forceinline__ bool same_bits(float a, float b) { return __float_as_uint(a) == __float_as_uint(b); }
__device__ __forceinline__ bool same_bits(double a, double b) { return __double_as_longlong(a) == __double_as_longlong(b); }

// gjk_collides (gjk.cpp:350-379): at most 100 iterations, false when they run out.
// One iteration is a pure function of the state (simplex, size, direction), so once a state
// repeats bit for bit the run is periodic: it can neither find the origin nor separate any more
// and would end false at the iteration cap. Brent's cycle detection (one saved state, saved
// again at power-of-two distances, kept in `saved`, 16 values in shared memory) stops such runs
// early with the same result; the iteration count returned is then below 100 and `cycled` is set.
template <typename R>
__device__ bool gjk_collides(const ColView<R>& c1, const ColView<R>& c2, Simplex<R>& s, int& iters,
                             long long& support_cycles, R* saved, bool& cycled) {
    const int lane = (int)lane_id();
    long long t0 = clock64();
    s.a = support_mink(c1, c2, v3<R>(0, 0, 1));
    s.b = s.c = s.d = v3<R>(0, 0, 0);
    s.num = 1;
    V3<R> dir = vscale((R)-1.0, s.a);
    cycled = false;
    int power = 1, lam = 0;
    for (int i = 0; i < 100; ++i) {
        iters = i + 1;
        V3<R> p = support_mink(c1, c2, dir);
        support_cycles += clock64() - t0;
        if (vdot(p, dir) < (R)0) return false;
        if (s.num == 1) { s.b = s.a; s.a = p; }
        else if (s.num == 2) { s.c = s.b; s.b = s.a; s.a = p; }
        else { s.d = s.c; s.c = s.b; s.b = s.a; s.a = p; }
        s.num++;
        if (do_simplex(s, dir)) return true;
        if (i >= 8) {
            const R mine = gjk_state(s, dir, lane & 15);
            if (i > 8) {
                const bool eq = same_bits(saved[lane & 15], mine);
                if (__all_sync(0xffffffffu, eq)) { cycled = true; return false; }
            }
            if (i == 8 || ++lam == power) {
                __syncwarp();
                if (lane < 16) saved[lane] = mine;
                __syncwarp();
                if (i > 8) { power <<= 1; lam = 0; }
            }
        }
        t0 = clock64();
    }
    return false;
}

// ---------------------------------------------------------------------------------------------
// EPA (epa.cpp:8-237)
template <typename R>
__device__ void epa_face(NarrowSmem<R>& sm, int fi, int npoly) {
    uchar4 f = sm.u.epa.f[fi];
    V3<double> a = v3cast<double>(sm.u.epa.poly[f.x]), b = v3cast<double>(sm.u.epa.poly[f.y]),
               c = v3cast<double>(sm.u.epa.poly[f.z]);
    V3<double> n = vnorm(vcross(vsub(b, a), vsub(c, a)));
    if (!(n.x != 0.0 || n.y != 0.0 || n.z != 0.0)) atomicOr(&sm.status, (int)(ST_DEGENERATE | ST_DEG_EPA_NORMAL));
    double d = vdot(n, a);
    if (d < -0.0) {
        n = vinv(n);
        d = -d;
    } else if (d >= -0.0 && d <= 0.0) {
        bool ok = false;
        for (int i = 0; i < npoly; ++i) {
            double ad = vdot(n, v3cast<double>(sm.u.epa.poly[i]));
            if (ad < -0.0 || ad > 0.0) {
                n = ad < -0.0 ? n : vinv(n);
                ok = true;
                break;
            }
        }
        if (!ok) atomicOr(&sm.status, (int)(ST_DEGENERATE | ST_DEG_EPA_COPLANAR));
    }
    sm.u.epa.fn[fi] = n;
    sm.u.epa.fd[fi] = d;
}

// The horizon edge list of one EPA iteration, held in registers across the warp: slot s lives in
// lane s % 32, register s / 32 (up to 64 edges), with its endpoint positions for the reference's
// position-equality test (epa.cpp:92-106).
template <typename R>
struct EdgeRegs {
    int ex[2], ey[2];
    V3<R> p1[2], p2[2];
};

// add_edge (epa.cpp:79-110): remove the first edge equal to (x, y) in either orientation — by index
// or by endpoint positions — moving the last edge into its slot; otherwise append. Every lane takes
// part; ne is warp-uniform.
template <typename R>
__device__ __forceinline__ void epa_add_edge_warp(EdgeRegs<R>& E, int& ne, int x, int y, V3<R> px, V3<R> py, bool& overflow) {
    const unsigned lane = lane_id();
    int found = -1;
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        int slot = k * 32 + (int)lane;
        bool m = slot < ne && ((E.ex[k] == x && E.ey[k] == y) || (E.ex[k] == y && E.ey[k] == x) ||
                               (veq(E.p1[k], px) && veq(E.p2[k], py)) || (veq(E.p1[k], py) && veq(E.p2[k], px)));
        unsigned b = __ballot_sync(0xffffffffu, m);
        if (found < 0 && b) found = k * 32 + __ffs(b) - 1;
    }
    if (found >= 0) {
        const int last = ne - 1, lk = last >> 5, ll = last & 31;
        int lx = __shfl_sync(0xffffffffu, lk ? E.ex[1] : E.ex[0], ll);
        int ly = __shfl_sync(0xffffffffu, lk ? E.ey[1] : E.ey[0], ll);
        V3<R> q1, q2;
        q1.x = __shfl_sync(0xffffffffu, lk ? E.p1[1].x : E.p1[0].x, ll);
        q1.y = __shfl_sync(0xffffffffu, lk ? E.p1[1].y : E.p1[0].y, ll);
        q1.z = __shfl_sync(0xffffffffu, lk ? E.p1[1].z : E.p1[0].z, ll);
        q2.x = __shfl_sync(0xffffffffu, lk ? E.p2[1].x : E.p2[0].x, ll);
        q2.y = __shfl_sync(0xffffffffu, lk ? E.p2[1].y : E.p2[0].y, ll);
        q2.z = __shfl_sync(0xffffffffu, lk ? E.p2[1].z : E.p2[0].z, ll);
        if ((int)lane == (found & 31)) {
            const int fk = found >> 5;
            if (fk) { E.ex[1] = lx; E.ey[1] = ly; E.p1[1] = q1; E.p2[1] = q2; }
            else { E.ex[0] = lx; E.ey[0] = ly; E.p1[0] = q1; E.p2[0] = q2; }
        }
        ne = last;
    } else {
        if (ne >= EPA_MAXE) { overflow = true; return; }
        if ((int)lane == (ne & 31)) {
            if (ne >> 5) { E.ex[1] = x; E.ey[1] = y; E.p1[1] = px; E.p2[1] = py; }
            else { E.ex[0] = x; E.ey[0] = y; E.p1[0] = px; E.p2[0] = py; }
        }
        ne = ne + 1;
    }
}

// Returns true when converged; normal and penetration are then set (FP64).
template <typename R>
__device__ bool epa(NarrowSmem<R>& sm, const ColView<R>& c1, const ColView<R>& c2, const Simplex<R>& s,
                    V3<double>& out_n, double& out_pen, int& iters) {
    const unsigned lane = lane_id();
    if (lane == 0) {
        sm.u.epa.poly[0] = s.a; sm.u.epa.poly[1] = s.b; sm.u.epa.poly[2] = s.c; sm.u.epa.poly[3] = s.d;
        sm.u.epa.f[0] = make_uchar4(0, 1, 2, 0);
        sm.u.epa.f[1] = make_uchar4(0, 2, 3, 0);
        sm.u.epa.f[2] = make_uchar4(0, 3, 1, 0);
        sm.u.epa.f[3] = make_uchar4(1, 2, 3, 0);
        sm.nf = 4;
        sm.npoly = 4;
    }
    __syncwarp();
    if (lane < 4) epa_face(sm, (int)lane, 4);
    __syncwarp();
    // min over the initial faces, strict < with the first minimum kept (epa.cpp:141-144)
    double md = DBL_MAX;
    int mi = 0x7fffffff;
    for (int i = (int)lane; i < sm.nf; i += WARP)
        if (sm.u.epa.fd[i] < md) { md = sm.u.epa.fd[i]; mi = i; }
    warp_argmin_first(md, mi);
    V3<double> min_n = (mi == 0x7fffffff) ? v3<double>(0, 0, 0) : sm.u.epa.fn[mi];
    double min_d = md;
    for (int it = 0; it < 100; ++it) {
        iters = it + 1;
        V3<R> sp = support_mink(c1, c2, v3cast<R>(min_n));
        V3<double> spd = v3cast<double>(sp);
        double d = vdot(min_n, spd);
        if (fabs(d - min_d) < 0.0001) {
            out_n = min_n;
            out_pen = min_d;
            return true;
        }
        int np = sm.npoly;
        if (np >= EPA_MAXV) {
            if (lane == 0) atomicOr(&sm.status, (int)ST_EPA_OVERFLOW);
            __syncwarp();
            return false;
        }
        __syncwarp();
        if (lane == 0) { sm.u.epa.poly[np] = sp; sm.npoly = np + 1; sm.ne = 0; }
        // visibility of every face, lane-parallel (independent of the removal order)
        int nf = sm.nf;
        for (int i = (int)lane; i < nf; i += WARP) {
            uchar4 f = sm.u.epa.f[i];
            V3<double> cen = vadd(vadd(v3cast<double>(sm.u.epa.poly[f.y]), v3cast<double>(sm.u.epa.poly[f.z])),
                                  v3cast<double>(sm.u.epa.poly[f.x]));
            cen = vscale(1.0 / 3.0, cen);
            f.w = vdot(sm.u.epa.fn[i], vsub(spd, cen)) > 0.0 ? 1 : 0;
            sm.u.epa.f[i] = f;
        }
        __syncwarp();
        // the reference's removal loop: unordered remove, re-test the moved face (epa.cpp:167-197),
        // run by the whole warp with the horizon edges in registers
        EdgeRegs<R> E;
        int ne = 0;
        bool overflow = false;
        {
            int i = 0;
            while (i < nf) {
                uchar4 f = sm.u.epa.f[i];
                if (f.w) {
                    V3<R> px = sm.u.epa.poly[f.x], py = sm.u.epa.poly[f.y], pz = sm.u.epa.poly[f.z];
                    epa_add_edge_warp(E, ne, f.x, f.y, px, py, overflow);
                    epa_add_edge_warp(E, ne, f.y, f.z, py, pz, overflow);
                    epa_add_edge_warp(E, ne, f.z, f.x, pz, px, overflow);
                    nf--;
                    __syncwarp();
                    if (lane == 0) {
                        sm.u.epa.f[i] = sm.u.epa.f[nf];
                        sm.u.epa.fd[i] = sm.u.epa.fd[nf];
                        sm.u.epa.fn[i] = sm.u.epa.fn[nf];
                    }
                    __syncwarp();
                } else {
                    ++i;
                }
            }
        }
        if (overflow || nf + ne > EPA_MAXF) {
            if (lane == 0) atomicOr(&sm.status, (int)ST_EPA_OVERFLOW);
            __syncwarp();
            return false;
        }
        // new faces (edge, new point) in edge-slot order, normals lane-parallel
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            int slot = k * 32 + (int)lane;
            if (slot < ne) {
                sm.u.epa.f[nf + slot] = make_uchar4((unsigned char)E.ex[k], (unsigned char)E.ey[k], (unsigned char)np, 0);
            }
        }
        __syncwarp();
        for (int i = (int)lane; i < ne; i += WARP) epa_face(sm, nf + i, np + 1);
        __syncwarp();
        if (lane == 0) sm.nf = nf + ne;
        nf += ne;
        md = DBL_MAX;
        mi = 0x7fffffff;
        for (int i = (int)lane; i < nf; i += WARP)
            if (sm.u.epa.fd[i] < md) { md = sm.u.epa.fd[i]; mi = i; }
        warp_argmin_first(md, mi);
        min_d = md;
        if (mi != 0x7fffffff) min_n = sm.u.epa.fn[mi];
        __syncwarp();
    }
    return false;
}

// ---------------------------------------------------------------------------------------------
// EPA for the FP32 build: the same expansion, termination test and iteration cap as the reference,
// with every step warp-parallel. Faces are FP32 (their vertices are FP32 Minkowski points); the
// horizon is found set-wise: an edge of a visible face belongs to it when no other edge of a
// visible face joins the same two points (by index or position), which is what the reference's
// toggling add_edge leaves; surviving faces keep their relative order and new faces follow in
// horizon order, so only exact ties in the closest-face search can resolve differently. The
// closest face is re-evaluated in FP64 before it is returned.
__device__ __forceinline__ void epa_face_f32(const V3<float>* poly, int npoly, uchar4 f, V3<float>& n_out, float& d_out, int& status) {
    V3<float> a = poly[f.x], b = poly[f.y], c = poly[f.z];
    const V3<float> e1 = vsub(b, a), e2 = vsub(c, a), cr = vcross(e1, e2);
    V3<float> n;
    if (vdot(cr, cr) > 1e-8f * vdot(e1, e1) * vdot(e2, e2)) {
        n = vnorm(cr);
    } else {
        // A sliver face (|e1 x e2| <= 1e-4 |e1||e2|): FP32 resolves its normal only to about
        // 6e-8 |e1||e2| / |e1 x e2|, or loses it entirely, so it is recomputed in FP64 from the same
        // points. Only a normal that vanishes in FP64 too is the reference's degenerate face
        // (epa.cpp:41 asserts on it).
        const V3<double> A = v3cast<double>(a);
        const V3<double> n64 = vnorm(vcross(vsub(v3cast<double>(b), A), vsub(v3cast<double>(c), A)));
        if (!(n64.x != 0.0 || n64.y != 0.0 || n64.z != 0.0)) status |= ST_DEGENERATE | ST_DEG_EPA_NORMAL;
        n = v3cast<float>(n64);
    }
    float d = vdot(n, a);
    if (d < -0.f) {
        n = vinv(n);
        d = -d;
    } else if (d >= -0.f && d <= 0.f) {
        bool ok = false;
        for (int i = 0; i < npoly; ++i) {
            float ad = vdot(n, poly[i]);
            if (ad < -0.f || ad > 0.f) {
                n = ad < -0.f ? n : vinv(n);
                ok = true;
                break;
            }
        }
        if (!ok) status |= ST_DEGENERATE | ST_DEG_EPA_COPLANAR;
    }
    n_out = n;
    d_out = d;
}

// face_out (optional): when FP32 decides the termination, lane 0 writes the final face's three
// points and its FP32 normal there (12 floats) and *deferred is set, leaving the FP64 normal and depth
// to a thread-per-pair kernel (k_epa_finish) instead of the warp; otherwise they are computed here.
template <typename R>
__device__ bool epa_fast(NarrowSmem<R>& smr, const ColView<R>& c1, const ColView<R>& c2, const Simplex<R>& s,
                         V3<double>& out_n, double& out_pen, int& iters, long long* support_cycles = nullptr,
                         float* face_out = nullptr, bool* deferred = nullptr) {
    static_assert(sizeof(EpaFastSmem<R>) <= sizeof(typename NarrowSmem<R>::U), "EPA scratch must fit the union");
    EpaFastSmem<R>& sm = *reinterpret_cast<EpaFastSmem<R>*>(&smr.u);
    const unsigned lane = lane_id();
    int st = 0;
    if (lane == 0) {
        sm.poly[0] = v3cast<float>(s.a); sm.poly[1] = v3cast<float>(s.b);
        sm.poly[2] = v3cast<float>(s.c); sm.poly[3] = v3cast<float>(s.d);
        sm.f[0] = make_uchar4(0, 1, 2, 0);
        sm.f[1] = make_uchar4(0, 2, 3, 0);
        sm.f[2] = make_uchar4(0, 3, 1, 0);
        sm.f[3] = make_uchar4(1, 2, 3, 0);
    }
    __syncwarp();
    int nf = 4, npoly = 4;
    if (lane < 4) epa_face_f32(sm.poly, 4, sm.f[lane], sm.fn[lane], sm.fd[lane], st);
    __syncwarp();
    auto closest = [&](float& md, int& mi) {
        md = FLT_MAX;
        mi = 0x7fffffff;
        for (int i = (int)lane; i < nf; i += WARP)
            if (sm.fd[i] < md) { md = sm.fd[i]; mi = i; }
        warp_argmin_first(md, mi);
    };
    float min_d;
    int mi;
    closest(min_d, mi);
    for (int it = 0; it < 100; ++it) {
        iters = it + 1;
        V3<float> min_n = mi == 0x7fffffff ? v3<float>(0.f, 0.f, 0.f) : sm.fn[mi];
        const long long ts = clock64();
        V3<float> sp = v3cast<float>(support_mink(c1, c2, v3cast<R>(min_n)));
        if (support_cycles) *support_cycles += clock64() - ts;
        // Termination test (epa.cpp:153-160) with the FP64 outcome: |<n, s> - d| < 1e-4 for the
        // closest face. FP32 decides it when the FP32 gap is farther from 1e-4 than its error bound
        // (the face normal's error grows with the face's conditioning |e1||e2| / |e1 x e2|);
        // otherwise the face is re-evaluated in FP64. The returned normal and depth are FP64.
        bool done = false, need64 = true;
        if (mi != 0x7fffffff) {
            uchar4 f = sm.f[mi];
            V3<float> a = sm.poly[f.x], e1 = vsub(sm.poly[f.y], a), e2 = vsub(sm.poly[f.z], a);
            const float cr = vlen(vcross(e1, e2));
            const float cond = cr > 0.f ? vlen(e1) * vlen(e2) / cr : FLT_MAX;
            const float gap = fabsf(vdot(min_n, sp) - min_d);
            const float err = 1e-6f * (1.f + cond) * (vlen(sp) + vlen(a) + 1e-3f) + 1e-7f;
            if (cond < 1e6f && gap < 0.0001f - err) { done = true; need64 = false; }
            else if (cond < 1e6f && gap > 0.0001f + err) { need64 = false; }
        }
        if (done && !need64 && face_out) {
            if (lane == 0) {
                const uchar4 f = sm.f[mi];
                const V3<float> pa = sm.poly[f.x], pb = sm.poly[f.y], pc = sm.poly[f.z];
                const float v[12] = {pa.x, pa.y, pa.z, pb.x, pb.y, pb.z, pc.x, pc.y, pc.z, min_n.x, min_n.y, min_n.z};
                for (int i = 0; i < 12; ++i) face_out[i] = v[i];
                if (st) atomicOr(&smr.status, st);
            }
            *deferred = true;
            __syncwarp();
            return true;
        }
        V3<double> n64 = v3<double>(0, 0, 0);
        double d64 = 0.0;
        if (mi != 0x7fffffff && (need64 || done)) {
            uchar4 f = sm.f[mi];
            V3<double> a = v3cast<double>(sm.poly[f.x]), b = v3cast<double>(sm.poly[f.y]), c = v3cast<double>(sm.poly[f.z]);
            n64 = vnorm_fast(vcross(vsub(b, a), vsub(c, a)));
            if (vdot(n64, v3cast<double>(min_n)) < 0.0) n64 = vinv(n64);
            d64 = vdot(n64, a);
        }
        if (need64) done = fabs(vdot(n64, v3cast<double>(sp)) - d64) < 0.0001;
        if (done) {
            out_n = n64;
            out_pen = d64;
            if (st && lane == 0) atomicOr(&smr.status, st);
            return true;
        }
        if (npoly >= EPA_MAXV) break;
        const int np = npoly;
        if (lane == 0) sm.poly[np] = sp;
        // visibility (epa.cpp:171-179)
        for (int i = (int)lane; i < nf; i += WARP) {
            uchar4 f = sm.f[i];
            V3<float> cen = vscale(1.0f / 3.0f, vadd(vadd(sm.poly[f.y], sm.poly[f.z]), sm.poly[f.x]));
            f.w = vdot(sm.fn[i], vsub(sp, cen)) > 0.f ? 1 : 0;
            sm.f[i] = f;
        }
        __syncwarp();
        // edges of the visible faces, in face order
        int ne = 0;
        bool overflow = false;
        for (int base = 0; base < nf; base += WARP) {
            int i = base + (int)lane;
            uchar4 f = i < nf ? sm.f[i] : make_uchar4(0, 0, 0, 0);
            bool v = i < nf && f.w;
            unsigned m = __ballot_sync(0xffffffffu, v);
            int pos = ne + 3 * __popc(m & ((1u << lane) - 1u));
            if (v) {
                if (pos + 3 <= 3 * WARP) {
                    sm.edge[pos] = make_uchar2(f.x, f.y);
                    sm.edge[pos + 1] = make_uchar2(f.y, f.z);
                    sm.edge[pos + 2] = make_uchar2(f.z, f.x);
                } else {
                    overflow = true;
                }
            }
            ne += 3 * __popc(m);
        }
        overflow = __any_sync(0xffffffffu, overflow) || ne > 3 * WARP;
        __syncwarp();
        if (overflow) { st |= ST_EPA_OVERFLOW; break; }
        // horizon: the toggling add_edge keeps one edge of every class of coincident edges (same
        // two points, by index or position) that occurs an odd number of times
        int nh = 0;
        for (int base = 0; base < ne; base += WARP) {
            int k = base + (int)lane;
            bool keep = false;
            uchar2 e = make_uchar2(0, 0);
            if (k < ne) {
                e = sm.edge[k];
                V3<float> e1 = sm.poly[e.x], e2 = sm.poly[e.y];
                int partners = 0;
                bool first = true;
                for (int j = 0; j < ne; ++j) {
                    if (j == k) continue;
                    uchar2 g = sm.edge[j];
                    bool same = (g.x == e.x && g.y == e.y) || (g.x == e.y && g.y == e.x);
                    if (!same) {
                        V3<float> g1 = sm.poly[g.x], g2 = sm.poly[g.y];
                        same = (veq(g1, e1) && veq(g2, e2)) || (veq(g1, e2) && veq(g2, e1));
                    }
                    if (same) {
                        ++partners;
                        if (j < k) first = false;
                    }
                }
                keep = first && (partners & 1) == 0;
            }
            unsigned m = __ballot_sync(0xffffffffu, keep);
            int pos = nh + __popc(m & ((1u << lane) - 1u));
            nh += __popc(m);
            if (keep) sm.hz[pos] = e;
        }
        __syncwarp();
        // compact the surviving (invisible) faces in order
        int kept = 0;
        for (int base = 0; base < nf; base += WARP) {
            int i = base + (int)lane;
            uchar4 f;
            V3<float> n;
            float dd;
            bool alive = false;
            if (i < nf) {
                f = sm.f[i];
                alive = !f.w;
                n = sm.fn[i];
                dd = sm.fd[i];
            }
            unsigned m = __ballot_sync(0xffffffffu, alive);
            int pos = kept + __popc(m & ((1u << lane) - 1u));
            __syncwarp();
            if (alive) { sm.f[pos] = f; sm.fn[pos] = n; sm.fd[pos] = dd; }
            kept += __popc(m);
            __syncwarp();
        }
        if (kept + nh > EPA_MAXF || nh > 3 * WARP) { st |= ST_EPA_OVERFLOW; break; }
        for (int k = (int)lane; k < nh; k += WARP) {
            uchar2 e = sm.hz[k];
            uchar4 f = make_uchar4(e.x, e.y, (unsigned char)np, 0);
            sm.f[kept + k] = f;
            epa_face_f32(sm.poly, np + 1, f, sm.fn[kept + k], sm.fd[kept + k], st);
        }
        __syncwarp();
        nf = kept + nh;
        npoly = np + 1;
        closest(min_d, mi);
    }
    st = __reduce_or_sync(0xffffffffu, st);
    if (lane == 0 && st) atomicOr(&smr.status, st);
    __syncwarp();
    return false;
}

// The FP64 normal and depth of EPA's final face from its three points and FP32 normal (epa.cpp:32-77
// on the face EPA stopped at), as epa_fast computes them in the warp: one thread per pair.
__device__ __forceinline__ void epa_face_finish(const float* f, V3<double>& n64, double& d64) {
    const V3<double> a = v3<double>(f[0], f[1], f[2]), b = v3<double>(f[3], f[4], f[5]), c = v3<double>(f[6], f[7], f[8]);
    n64 = vnorm_fast(vcross(vsub(b, a), vsub(c, a)));
    if (vdot(n64, v3<double>(f[9], f[10], f[11])) < 0.0) n64 = vinv(n64);
    d64 = vdot(n64, a);
}

// ---------------------------------------------------------------------------------------------
// Clipping (clipping.cpp)
template <typename R>
__device__ __forceinline__ bool in_plane(V3<R> pn, V3<R> pp, V3<R> pos) {
    float distance = -vdot(pn, pp);
    return !(vdot(pos, pn) + (R)distance < (R)0.0);
}

template <typename R>
__device__ __forceinline__ bool plane_edge(V3<R> pn, V3<R> pp, V3<R> start, V3<R> end, V3<R>& out) {
    V3<R> ab = vsub(end, start);
    float ab_p = vdot(pn, ab);
    // (double)|ab_p| > 0.000001 (clipping.cpp:30): 1e-6f is the largest float below 1e-6 and no float
    // lies between them, so the FP32 comparison decides exactly the same
    if (fabsf(ab_p) > 1e-6f) {
        float distance = -vdot(pn, pp);
        V3<R> p_co = vscale((R)(-distance), pn);
        float fac = -vdot(pn, vsub(start, p_co)) / (R)ab_p;
        R mx = ((R)fac > (R)0.0) ? (R)fac : (R)0.0;
        fac = (float)((mx < (R)1.0) ? mx : (R)1.0);
        out = vadd(start, vscale((R)fac, ab));
        return true;
    }
    return false;
}

// One Sutherland–Hodgman pass against one plane, one lane per polygon edge. Returns the output count,
// or -1 when every vertex lies inside the plane: the pass would then emit its input unchanged and in
// order (each edge emits its end point), so the caller keeps the input buffer.
template <typename R>
__device__ int sh_pass(const V3<R>* in, int n, V3<R>* out, V3<R> pn, V3<R> pp, bool remove_only, int& status) {
    const unsigned lane = lane_id();
    bool all_in = true;
    for (int j = (int)lane; j < n; j += WARP) all_in = all_in && in_plane(pn, pp, in[j]);
    if (__all_sync(0xffffffffu, all_in)) return -1;
    int carry = 0;
    for (int base = 0; base < n; base += WARP) {
        int j = base + (int)lane;
        int cnt = 0;
        V3<R> o0 = v3<R>(0, 0, 0), o1 = v3<R>(0, 0, 0);
        if (j < n) {
            V3<R> end = in[j];
            V3<R> start = in[j == 0 ? n - 1 : j - 1];
            bool si = in_plane(pn, pp, start), ei = in_plane(pn, pp, end);
            if (remove_only) {
                if (ei) { o0 = end; cnt = 1; }
            } else if (si && ei) {
                o0 = end; cnt = 1;
            } else if (si && !ei) {
                V3<R> t;
                if (plane_edge(pn, pp, start, end, t)) { o0 = t; cnt = 1; }
            } else if (!si && ei) {
                V3<R> t;
                if (plane_edge(pn, pp, start, end, t)) { o0 = t; o1 = end; cnt = 2; }
                else { o0 = end; cnt = 1; }
            }
        }
        int incl = warp_incl_scan(cnt);
        int pos = carry + incl - cnt;
        if (cnt >= 1) { if (pos < CLIP_MAX) out[pos] = o0; else status |= ST_CLIP_OVERFLOW; }
        if (cnt == 2) { if (pos + 1 < CLIP_MAX) out[pos + 1] = o1; else status |= ST_CLIP_OVERFLOW; }
        carry += __shfl_sync(0xffffffffu, incl, 31);
    }
    __syncwarp();
    return carry < CLIP_MAX ? carry : CLIP_MAX;
}

template <typename R, bool EXACT>
struct PairFrame {
    // maps a contact point pair to constraint-local offsets r1_lc, r2_lc
    Qt<R> q1inv, q2inv;
    V3<R> x1, x2;     // body origins in the pair frame
    bool raw;         // keep the contact points themselves (known-answer queries)
};

template <typename R, bool EXACT>
__device__ void push_contact(NarrowSmem<R>& sm, const PairFrame<R, EXACT>& fr, V3<R> p1, V3<R> p2, V3<R> n, bool pred) {
    // clipping_contact_to_collision_constraint (pbd.cpp:408-424), compacted in warp order
    unsigned m = __ballot_sync(0xffffffffu, pred);
    int base = sm.ncontacts;
    int pos = base + __popc(m & ((1u << lane_id()) - 1u));
    if (pred) {
        if (pos < CMAX) {
            sm.c_r1[pos] = fr.raw ? p1 : qrotate(fr.q1inv, vsub(p1, fr.x1));
            sm.c_r2[pos] = fr.raw ? p2 : qrotate(fr.q2inv, vsub(p2, fr.x2));
            sm.c_n[pos] = n;
        } else {
            atomicOr(&sm.status, (int)ST_CONTACT_OVERFLOW);
        }
    }
    __syncwarp();
    if (lane_id() == 0) sm.ncontacts = min(base + __popc(m), CMAX);
    __syncwarp();
}

template <typename R>
__device__ __forceinline__ int csr_len(const int32_t* start, int row) { return start[row + 1] - start[row]; }

// convex_convex_contact_manifold (clipping.cpp:249-341)
template <typename R, bool EXACT>
__device__ void convex_convex_manifold(NarrowSmem<R>& sm, const WorldView<R>& W, const ColView<R>& h1, const ColView<R>& h2,
                                       V3<R> normal, V3<double> normal64, const PairFrame<R, EXACT>& fr) {
    const unsigned lane = lane_id();
    V3<R> inv_n = vinv(normal);
    int s1 = support_index(h1, normal);
    int s2 = support_index(h2, inv_n);
    const int32_t* cs = W.csr_start;
    const int32_t* cd = W.csr_data;
    // get_face_with_most_fitting_normal over vertex_to_faces (first max wins)
    int v2f1 = h1.shape->v2f_off + s1, v2f2 = h2.shape->v2f_off + s2;
    R best1 = sizeof(R) == 4 ? -FLT_MAX : -(R)DBL_MAX, best2 = best1;
    int f1 = 0x7fffffff, f2 = 0x7fffffff;
    for (int k = (int)lane; k < csr_len<R>(cs, v2f1); k += WARP) {
        int fi = cd[cs[v2f1] + k];
        R p = vdot(h1.norms[fi], normal);
        if (p > best1) { best1 = p; f1 = k; }
    }
    for (int k = (int)lane; k < csr_len<R>(cs, v2f2); k += WARP) {
        int fi = cd[cs[v2f2] + k];
        R p = vdot(h2.norms[fi], inv_n);
        if (p > best2) { best2 = p; f2 = k; }
    }
    warp_argmax_first(best1, f1);
    warp_argmax_first(best2, f2);
    f1 = cd[cs[v2f1] + (f1 == 0x7fffffff ? 0 : f1)];
    f2 = cd[cs[v2f2] + (f2 == 0x7fffffff ? 0 : f2)];
    V3<R> n1 = h1.norms[f1], n2 = h2.norms[f2];
    // get_edge_with_most_fitting_normal: candidates in (i, j, normal / inverted) order
    int v2n1 = h1.shape->v2n_off + s1, v2n2 = h2.shape->v2n_off + s2;
    int nn1 = csr_len<R>(cs, v2n1), nn2 = csr_len<R>(cs, v2n2);
    V3<R> sp1 = cv_vertex(h1, s1), sp2 = cv_vertex(h2, s2);
    R bestE = sizeof(R) == 4 ? -FLT_MAX : -(R)DBL_MAX;
    int bestK = 0x7fffffff;
    for (int k = (int)lane; k < nn1 * nn2; k += WARP) {
        int i = k / nn2, j = k % nn2;
        V3<R> e1 = vsub(sp1, cv_vertex(h1, cd[cs[v2n1] + i]));
        V3<R> e2 = vsub(sp2, cv_vertex(h2, cd[cs[v2n2] + j]));
        V3<R> cn = vnorm(vcross(e1, e2));
        V3<R> ci = vinv(cn);
        R d0 = vdot(cn, normal);
        if (d0 > bestE) { bestE = d0; bestK = 2 * k; }
        R d1 = vdot(ci, normal);
        if (d1 > bestE) { bestE = d1; bestK = 2 * k + 1; }
    }
    warp_argmax_first(bestE, bestK);
    V3<R> edge_normal = v3<R>(0, 0, 0);
    int ei = 0, ej = 0;
    if (bestK != 0x7fffffff) {
        int k = bestK >> 1;
        ei = cd[cs[v2n1] + k / nn2];
        ej = cd[cs[v2n2] + k % nn2];
        V3<R> e1 = vsub(sp1, cv_vertex(h1, ei));
        V3<R> e2 = vsub(sp2, cv_vertex(h2, ej));
        edge_normal = vnorm(vcross(e1, e2));
        if (bestK & 1) edge_normal = vinv(edge_normal);
    }
    R d1 = vdot(n1, normal), d2 = vdot(n2, inv_n), de = vdot(edge_normal, normal);
    if (de > d1 + (R)0.0001 && de > d2 + (R)0.0001) {
        // collision_distance_between_skew_lines (clipping.cpp:210-239)
        V3<R> p1 = sp1, dd1 = vsub(cv_vertex(h1, ei), p1);
        V3<R> p2 = sp2, dd2 = vsub(cv_vertex(h2, ej), p2);
        R nA = dd1.x * dd2.x + dd1.y * dd2.y + dd1.z * dd2.z;
        R nB = dd2.x * dd2.x + dd2.y * dd2.y + dd2.z * dd2.z;
        R mA = -dd1.x * dd1.x - dd1.y * dd1.y - dd1.z * dd1.z;
        R mB = -dd2.x * dd1.x - dd2.y * dd1.y - dd2.z * dd1.z;
        R rA = -dd1.x * p2.x + dd1.x * p1.x - dd1.y * p2.y + dd1.y * p1.y - dd1.z * p2.z + dd1.z * p1.z;
        R rB = -dd2.x * p2.x + dd2.x * p1.x - dd2.y * p2.y + dd2.y * p1.y - dd2.z * p2.z + dd2.z * p1.z;
        R den = (nA * mB) - (nB * mA);
        bool ok = den != (R)0;
        if (!ok && lane == 0) atomicOr(&sm.status, (int)(ST_DEGENERATE | ST_DEG_SKEW));
        R nn = ok ? ((rA * mB) - (rB * mA)) / den : (R)0;
        R mm = ok ? ((nA * rB) - (nB * rA)) / den : (R)0;
        V3<R> l1 = vadd(p1, vscale(mm, dd1));
        V3<R> l2 = vadd(p2, vscale(nn, dd2));
        push_contact(sm, fr, l1, l2, normal, ok && lane == 0);
        return;
    }
    bool ref1 = d1 > d2;
    // screen in FP32: |d1 - d2| below 1e-5 (within the float subtraction's rounding: 1.1e-5 covers it)
    if (!EXACT && fabsf((float)d1 - (float)d2) < 1.1e-5f) {
        // The reference face is the better-aligned of the two candidates (clipping.cpp:284). For
        // nearly parallel faces d1 and d2 differ by ~1e-11, below FP32 resolution; decide it from
        // FP64 normals so the FP32 build picks the reference's face (and so its contact order).
        // Outside 1e-5 (FP32 error of these unit-vector dot products: ~3e-7) FP32 decides the same.
        // one lane evaluates it (FP64 on GB300 issues at 1/64 of the FP32 rate) and broadcasts it
        int r = 0;
        if (lane == 0) {
            const V3<double> m1 = face_normal64(W, h1, f1), m2 = face_normal64(W, h2, f2);
            r = vdot(m1, normal64) > vdot(m2, vinv(normal64)) ? 1 : 0;
        }
        ref1 = __shfl_sync(0xffffffffu, r, 0) != 0;
    }
    const ColView<R>& rh = ref1 ? h1 : h2;
    const ColView<R>& ih = ref1 ? h2 : h1;
    int rf = ref1 ? f1 : f2, inf = ref1 ? f2 : f1;
    const int32_t* fes = W.face_elem_start;
    // incident polygon and boundary planes (build_boundary_planes, clipping.cpp:121-134)
    int fs_i = fes[ih.shape->elem_off + inf];
    int fe_i = fes[ih.shape->elem_off + inf + 1];
    int ninc = fe_i - fs_i;
    if (ninc > CLIP_MAX) { if (lane == 0) atomicOr(&sm.status, (int)ST_CLIP_OVERFLOW); ninc = CLIP_MAX; }
    for (int k = (int)lane; k < ninc; k += WARP) sm.u.clip.buf[0][k] = cv_vertex(ih, W.face_elem[fs_i + k]);
    int f2n_row = rh.shape->f2n_off + rf;
    int npl = csr_len<R>(cs, f2n_row);
    if (npl > CLIP_MAX) { if (lane == 0) atomicOr(&sm.status, (int)ST_CLIP_OVERFLOW); npl = CLIP_MAX; }
    for (int k = (int)lane; k < npl; k += WARP) {
        int nf = cd[cs[f2n_row] + k];
        sm.u.clip.pp[k] = cv_vertex(rh, W.face_elem[W.face_elem_start[rh.shape->elem_off + nf]]);
        sm.u.clip.pn[k] = vinv(rh.norms[nf]);
    }
    __syncwarp();
    int st = 0;
    int n = ninc, cur = 0;
    for (int p = 0; p < npl; ++p) {
        if (n == 0) break;
        const int m = sh_pass(sm.u.clip.buf[cur], n, sm.u.clip.buf[cur ^ 1], sm.u.clip.pn[p], sm.u.clip.pp[p], false, st);
        if (m >= 0) { n = m; cur ^= 1; }
    }
    V3<R> ref_n = vinv(rh.norms[rf]);
    V3<R> ref_p = cv_vertex(rh, W.face_elem[W.face_elem_start[rh.shape->elem_off + rf]]);
    if (n > 0) {
        const int m = sh_pass(sm.u.clip.buf[cur], n, sm.u.clip.buf[cur ^ 1], ref_n, ref_p, true, st);
        if (m >= 0) { n = m; cur ^= 1; }
    }
    if (st && lane == 0) atomicOr(&sm.status, (int)st);
    // contacts from the kept points (clipping.cpp:302-327)
    for (int base = 0; base < n; base += WARP) {
        int k = base + (int)lane;
        bool pred = false;
        V3<R> c1 = v3<R>(0, 0, 0), c2 = v3<R>(0, 0, 0);
        if (k < n) {
            V3<R> pt = sm.u.clip.buf[cur][k];
            R dd = vdot(vscale((R)-1.0, ref_n), ref_p);
            V3<R> cp = vsub(pt, vscale(vdot(ref_n, pt) + dd, ref_n));
            V3<R> diff = vsub(pt, cp);
            R pen;
            if (ref1) {
                pen = vdot(diff, normal);
                c1 = vsub(pt, vscale(pen, normal));
                c2 = pt;
            } else {
                pen = -vdot(diff, normal);
                c1 = pt;
                c2 = vadd(pt, vscale(pen, normal));
            }
            pred = pen < (R)0.0;
        }
        push_contact(sm, fr, c1, c2, normal, pred);
    }
}

// clipping_get_contact_manifold (clipping.cpp:343-370)
template <typename R, bool EXACT>
__device__ void contact_manifold(NarrowSmem<R>& sm, const WorldView<R>& W, const ColView<R>& c1, const ColView<R>& c2,
                                 V3<R> normal, V3<double> normal64, R pen, const PairFrame<R, EXACT>& fr) {
    if (c1.type == COL_SPHERE) {
        V3<R> sp = support_point(c1, normal);
        push_contact(sm, fr, sp, vsub(sp, vscale(pen, normal)), normal, lane_id() == 0);
    } else if (c2.type == COL_SPHERE) {
        V3<R> sp = support_point(c2, vinv(normal));
        push_contact(sm, fr, vadd(sp, vscale(pen, normal)), sp, normal, lane_id() == 0);
    } else {
        convex_convex_manifold<R, EXACT>(sm, W, c1, c2, normal, normal64, fr);
    }
}



// collider_get_contacts (collider.cpp:523-558)
template <typename R, bool EXACT>
__device__ void collider_contacts(NarrowSmem<R>& sm, const WorldView<R>& W, const ColView<R>& c1, const ColView<R>& c2,
                                  const PairFrame<R, EXACT>& fr, unsigned long long* counters) {
    if (c1.type == COL_SPHERE && c2.type == COL_SPHERE) {
        V3<R> dv = vsub(c1.center, c2.center);
        float dsq = vdot(dv, dv);
        float mind = (float)c1.radius + (float)c2.radius;
        if (dsq < (mind * mind)) {
            V3<R> normal = vnorm(vsub(c2.center, c1.center));
            R pen = (R)(float)(mind - sqrtf(dsq));
            contact_manifold<R, EXACT>(sm, W, c1, c2, normal, v3cast<double>(normal), pen, fr);
        }
        return;
    }
    Simplex<R> s;
    int gi = 0, ei = 0;
    const long long t0 = clock64();
    long long tsup = 0;
    bool cycled = false;
    bool hit = gjk_collides(c1, c2, s, gi, tsup, sm.gjk_saved, cycled);
    const long long t1 = clock64();
    if (counters && lane_id() == 0) {
        atomicAdd(&counters[0], (unsigned long long)gi);
        atomicAdd(&counters[12], (unsigned long long)(t1 - t0));
        atomicAdd(&counters[15], (unsigned long long)tsup);
        if (cycled) atomicAdd(&counters[16], 1ull);
        if (gi >= 100) atomicAdd(&counters[4], 1ull);
    }
    if (!hit) return;
    V3<double> n;
    double pen;
    bool ok;
    if constexpr (EXACT || !kEpaFast) ok = epa(sm, c1, c2, s, n, pen, ei);
    else ok = epa_fast(sm, c1, c2, s, n, pen, ei);
    const long long t2 = clock64();
    if (counters && lane_id() == 0) {
        atomicAdd(&counters[1], (unsigned long long)ei);
        atomicAdd(&counters[2], 1ull);
        atomicAdd(&counters[13], (unsigned long long)(t2 - t1));
        if (ei >= 100) atomicAdd(&counters[7], 1ull);
    }
    if (!ok) {
        if (lane_id() == 0) atomicOr(&sm.status, (int)ST_EPA_NOT_CONVERGED);
        __syncwarp();
        return;
    }
    contact_manifold<R, EXACT>(sm, W, c1, c2, v3cast<R>(n), n, (R)pen, fr);
    if (counters && lane_id() == 0) atomicAdd(&counters[14], (unsigned long long)(clock64() - t2));
}

}  // namespace rp
