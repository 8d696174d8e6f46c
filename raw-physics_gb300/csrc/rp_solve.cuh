// XPBD constraint solves, integration and velocity passes on the device.
//
// Bodies touched by one solver node (a broad-phase pair with its contacts, or one external joint)
// are loaded into registers, updated in the order the reference applies its corrections, and
// written back once; nodes of one level never share a non-fixed body, so no two threads write the
// same body.
//
// EXACT=true mirrors the reference's FP64 expressions term for term (built without FMA
// contraction it reproduces the reference bit for bit). EXACT=false keeps positions and
// orientations in FP64 and does the rest in FP32, forming position differences in FP64 before
// rounding so that precision does not depend on the distance from the world origin.
//
// References (raw-physics): pbd.cpp:81-406 (solves), :537-577 (predict), :623-643 (velocity
// update), :646-740 (velocity solver); pbd_base_constraints.cpp:6-227; physics_util.cpp:5-63.
#pragma once
#include "rp_math.cuh"
#include "rp_world.h"

namespace rp {

constexpr double PI_REF = 3.14159265358979;   // PI_F of include/gm.h:8

template <typename R>
struct Body {
    V3<double> x;
    Qt<double> q;
    R invm;
    M3<R> Iinv;       // local inverse inertia
    bool fixed;
    int idx;
};

template <typename R>
__device__ __forceinline__ Body<R> load_body(const WorldView<R>& W, int b) {
    Body<R> B;
    double4_32a p = W.pos[b], q = W.rot[b];
    B.x = v3<double>(p.x, p.y, p.z);
    B.q = qt<double>(q.x, q.y, q.z, q.w);
    B.invm = W.inv_mass[b];
    R s[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) s[i] = W.inv_inertia[6 * b + i];
    B.Iinv = msym(s);
    B.fixed = W.fixed[b] != 0;
    B.idx = b;
    return B;
}

template <typename R>
__device__ __forceinline__ void store_pose(const WorldView<R>& W, const Body<R>& B) {
    if (B.fixed) return;
    W.pos[B.idx] = make_double4_32a(B.x.x, B.x.y, B.x.z, 0.0);
    W.rot[B.idx] = make_double4_32a(B.q.x, B.q.y, B.q.z, B.q.w);
}

// Rotation used for the working-precision algebra of a body.
template <typename R>
__device__ __forceinline__ Qt<R> wq(const Qt<double>& q) { return qcast<R>(q); }

// --------------------------------------------------------------------------------------------
// Position_Constraint_Preprocessed_Data / positional constraint (pbd_base_constraints.cpp:6-123)
template <typename R>
struct Pcpd {
    V3<R> r1, r2;      // r_wc
    M3<R> I1, I2;      // world inverse inertia
};

template <typename R>
__device__ __forceinline__ Pcpd<R> pcpd(const Body<R>& a, const Body<R>& b, V3<R> r1_lc, V3<R> r2_lc) {
    Pcpd<R> p;
    Qt<R> qa = wq<R>(a.q), qb = wq<R>(b.q);
    p.r1 = qrotate(qa, r1_lc);
    p.r2 = qrotate(qb, r2_lc);
    p.I1 = world_tensor(qa, a.Iinv);
    p.I2 = world_tensor(qb, b.Iinv);
    return p;
}

template <typename R>
__device__ __forceinline__ R pos_dlambda(const Body<R>& a, const Body<R>& b, const Pcpd<R>& p, R h, R compliance, R lambda,
                                         V3<R> dx) {
    R c = vlen(dx);
    if (c <= Tiny<R>::v) return (R)0;
    V3<R> n = v3<R>(dx.x / c, dx.y / c, dx.z / c);
    R w1 = a.invm + vdot(vcross(p.r1, n), mmulv(p.I1, vcross(p.r1, n)));
    R w2 = b.invm + vdot(vcross(p.r2, n), mmulv(p.I2, vcross(p.r2, n)));
    R til = compliance / (h * h);
    return (-c - til * lambda) / (w1 + w2 + til);
}

// Normalisation of an FP64 quaternion in the FP32 build: an FP32 reciprocal square root refined by
// one FP64 Newton step (relative error ~1e-14), instead of an FP64 square root and four FP64
// divisions, which GB300 executes at a small fraction of its FP32 rate.
__device__ __forceinline__ Qt<double> qnormalize_fast(Qt<double> q) {
    double n2 = q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w;
    double r = (double)rsqrtf((float)n2);
    r = r * (1.5 - 0.5 * n2 * r * r);
    return qt<double>(q.x * r, q.y * r, q.z * r, q.w * r);
}

// q <- normalize(q + s * dq): the linearised orientation update, accumulated in FP64
template <typename R>
__device__ __forceinline__ void q_add_normalize(Qt<double>& q, Qt<R> d, double s) {
    if (sizeof(R) == 8) {
        q.x = q.x + s * (double)d.x; q.y = q.y + s * (double)d.y; q.z = q.z + s * (double)d.z; q.w = q.w + s * (double)d.w;
        q = qnormalize(q);
    } else {
        q.x = q.x + (double)((R)s * d.x); q.y = q.y + (double)((R)s * d.y);
        q.z = q.z + (double)((R)s * d.z); q.w = q.w + (double)((R)s * d.w);
        q = qnormalize_fast(q);
    }
}

template <typename R>
__device__ __forceinline__ void pos_apply(Body<R>& a, Body<R>& b, const Pcpd<R>& p, R dl, V3<R> dx) {
    R c = vlen(dx);
    if (c <= Tiny<R>::v) return;
    V3<R> n = v3<R>(dx.x / c, dx.y / c, dx.z / c);
    V3<R> imp = vscale(dl, n);
    if (!a.fixed) a.x = vadd(a.x, v3cast<double>(vscale(a.invm, imp)));
    if (!b.fixed) b.x = vadd(b.x, v3cast<double>(vscale(-b.invm, imp)));
    V3<R> a1 = mmulv(p.I1, vcross(p.r1, imp));
    V3<R> a2 = mmulv(p.I2, vcross(p.r2, imp));
    Qt<R> q1 = qmul(qt<R>(a1.x, a1.y, a1.z, (R)0), wq<R>(a.q));
    Qt<R> q2 = qmul(qt<R>(a2.x, a2.y, a2.z, (R)0), wq<R>(b.q));
    if (!a.fixed) q_add_normalize(a.q, q1, 0.5);
    if (!b.fixed) q_add_normalize(b.q, q2, -0.5);
}

// Angular constraint (pbd_base_constraints.cpp:125-227)
template <typename R>
struct Acpd { M3<R> I1, I2; };

template <typename R>
__device__ __forceinline__ Acpd<R> acpd(const Body<R>& a, const Body<R>& b) {
    Acpd<R> r;
    r.I1 = world_tensor(wq<R>(a.q), a.Iinv);
    r.I2 = world_tensor(wq<R>(b.q), b.Iinv);
    return r;
}

template <typename R>
__device__ __forceinline__ R ang_dlambda(const Acpd<R>& A, R h, R compliance, R lambda, V3<R> dq) {
    R th = vlen(dq);
    if (th <= Tiny<R>::v) return (R)0;
    V3<R> n = v3<R>(dq.x / th, dq.y / th, dq.z / th);
    R w1 = vdot(n, mmulv(A.I1, n));
    R w2 = vdot(n, mmulv(A.I2, n));
    R til = compliance / (h * h);
    return (-th - til * lambda) / (w1 + w2 + til);
}

template <typename R>
__device__ __forceinline__ void ang_apply(Body<R>& a, Body<R>& b, const Acpd<R>& A, R dl, V3<R> dq) {
    R th = vlen(dq);
    if (th <= Tiny<R>::v) return;
    V3<R> n = v3<R>(dq.x / th, dq.y / th, dq.z / th);
    V3<R> imp = vscale(-dl, n);
    V3<R> a1 = mmulv(A.I1, imp);
    V3<R> a2 = mmulv(A.I2, imp);
    Qt<R> q1 = qmul(qt<R>(a1.x, a1.y, a1.z, (R)0), wq<R>(a.q));
    Qt<R> q2 = qmul(qt<R>(a2.x, a2.y, a2.z, (R)0), wq<R>(b.q));
    if (!a.fixed) q_add_normalize(a.q, q1, 0.5);
    if (!b.fixed) q_add_normalize(b.q, q2, -0.5);
}

// x_a + r_a - (x_b + r_b), with the position difference formed in FP64 in the FP32 build
template <typename R, bool EXACT>
__device__ __forceinline__ V3<R> anchor_delta(const Body<R>& a, const Body<R>& b, V3<R> ra, V3<R> rb) {
    if (EXACT) return v3cast<R>(vsub(vadd(a.x, v3cast<double>(ra)), vadd(b.x, v3cast<double>(rb))));
    return vadd(v3cast<R>(vsub(a.x, b.x)), vsub(ra, rb));
}

// --------------------------------------------------------------------------------------------
// collision_constraint_solve (pbd.cpp:107-154). c points at the contact record
// {r1_lc, lambda_n, r2_lc, lambda_t, normal, -}.
template <typename R, bool EXACT>
__device__ void collision_solve(const WorldView<R>& W, Body<R>& a, Body<R>& b, R* c, R h, const R mus) {
    V3<R> r1 = v3<R>(c[0], c[1], c[2]), r2 = v3<R>(c[4], c[5], c[6]), n = v3<R>(c[8], c[9], c[10]);
    R lambda_n = c[3], lambda_t = c[7];
    Pcpd<R> p = pcpd(a, b, r1, r2);
    V3<R> d12 = anchor_delta<R, EXACT>(a, b, p.r1, p.r2);
    R d = vdot(d12, n);
    if (d > (R)0) {
        V3<R> dx = vscale(d, n);
        R dl = pos_dlambda(a, b, p, h, (R)0, lambda_n, dx);
        pos_apply(a, b, p, dl, dx);
        lambda_n += dl;
        p = pcpd(a, b, r1, r2);
        dl = pos_dlambda(a, b, p, h, (R)0, lambda_t, dx);
        R lt = lambda_t + dl;
        if (lt > mus * lambda_n) {
            // p1 - p1_til - (p2 - p2_til) with p_til from the previous pose (pbd.cpp:142-148)
            double4_32a pa = W.prev_pos[a.idx], qa = W.prev_rot[a.idx], pb = W.prev_pos[b.idx], qb = W.prev_rot[b.idx];
            V3<double> xa_prev = v3<double>(pa.x, pa.y, pa.z), xb_prev = v3<double>(pb.x, pb.y, pb.z);
            Qt<R> qa_prev = qcast<R>(qt<double>(qa.x, qa.y, qa.z, qa.w)), qb_prev = qcast<R>(qt<double>(qb.x, qb.y, qb.z, qb.w));
            V3<R> dp;
            if (EXACT) {
                V3<double> p1 = vadd(a.x, v3cast<double>(p.r1)), p2 = vadd(b.x, v3cast<double>(p.r2));
                V3<double> p1t = vadd(xa_prev, v3cast<double>(qrotate(qa_prev, r1)));
                V3<double> p2t = vadd(xb_prev, v3cast<double>(qrotate(qb_prev, r2)));
                dp = v3cast<R>(vsub(vsub(p1, p1t), vsub(p2, p2t)));
            } else {
                V3<R> da = vadd(v3cast<R>(vsub(a.x, xa_prev)), vsub(p.r1, qrotate(qa_prev, r1)));
                V3<R> db = vadd(v3cast<R>(vsub(b.x, xb_prev)), vsub(p.r2, qrotate(qb_prev, r2)));
                dp = vsub(da, db);
            }
            V3<R> dpt = vsub(dp, vscale(vdot(dp, n), n));
            pos_apply(a, b, p, dl, dpt);
            lambda_t += dl;
        }
    }
    c[3] = lambda_n;
    c[7] = lambda_t;
}

// limit_angle (pbd.cpp:175-217)
// Joint limits are evaluated in FP64 in both builds (the axes come from the FP64 orientations):
// asin's slope diverges at |s| -> 1, so at a +-90 degree limit an FP32 s (error 1e-7) would move
// phi by sqrt(2e-7) ~ 4.5e-4 rad; in FP64 the same amplification stays below 1e-7.
template <typename R>
__device__ bool limit_angle(V3<R> n, V3<R> n1, V3<R> n2, R alpha, R beta, V3<R>& dq) {
    const R pi = (R)PI_REF;
    R phi = asin(vdot(vcross(n1, n2), n));
    if (vdot(n1, n2) < (R)0) phi = pi - phi;
    if (phi > pi) phi = phi - (R)2.0 * pi;
    if (phi < -pi) phi = phi + (R)2.0 * pi;
    if (phi < alpha || phi > beta) {
        phi = (phi > beta) ? beta : ((phi < alpha) ? alpha : phi);
        V3<R> ax = n;
        if (vlen(ax) != (R)0) ax = vnorm(ax);
        R s = sin(phi / (R)2.0);
        Qt<R> rot = qt<R>(ax.x * s, ax.y * s, ax.z * s, cos(phi / (R)2.0));
        n1 = qrotate(rot, n1);
        dq = vcross(n1, n2);
        return true;
    }
    return false;
}

// True when limit_angle could apply a correction. With limits at or beyond +-pi the wrapped angle
// can never leave them (any build). Otherwise, in the FP32 build, an FP32 estimate of the angle from
// FP32 axes decides when it lies more than 0.01 rad inside both limits: its error stays below 1e-3 rad
// even where asin is ill-conditioned (|s| -> 1). Near a limit, near the +-pi wrap, or where the
// branch on <n1, n2> is within 1e-3 of flipping, the FP64 evaluation runs.
__device__ __forceinline__ bool limit_may_act(V3<float> n, V3<float> n1, V3<float> n2, double lo, double hi) {
    if (lo <= -PI_REF && hi >= PI_REF) return false;
    if (lo < -PI_REF + 0.02 || hi > PI_REF - 0.02) return true;
    const float c = vdot(n1, n2);
    if (fabsf(c) < 1e-3f) return true;
    const float pi = (float)PI_REF;
    float phi = asinf(fminf(fmaxf(vdot(vcross(n1, n2), n), -1.f), 1.f));
    if (c < 0.f) phi = pi - phi;
    if (phi > pi) phi -= 2.f * pi;
    if (phi < -pi) phi += 2.f * pi;
    return !(phi >= (float)lo + 0.01f && phi <= (float)hi - 0.01f);
}

template <typename R, bool EXACT>
__device__ void ext_solve(const WorldView<R>& W, const ExtConstraint& C, double* lam, R h) {
    Body<R> a = load_body(W, C.e1), b = load_body(W, C.e2);
    V3<R> r1 = v3<R>((R)C.r1[0], (R)C.r1[1], (R)C.r1[2]), r2 = v3<R>((R)C.r2[0], (R)C.r2[1], (R)C.r2[2]);
    switch (C.type) {
    case CON_POSITIONAL: {  // pbd.cpp:81-97
        V3<R> dx = vsub(v3cast<R>(vsub(a.x, b.x)), v3<R>((R)C.distance[0], (R)C.distance[1], (R)C.distance[2]));
        if (EXACT) dx = v3cast<R>(vsub(vsub(a.x, b.x), v3<double>(C.distance[0], C.distance[1], C.distance[2])));
        Pcpd<R> p = pcpd(a, b, r1, r2);
        R dl = pos_dlambda(a, b, p, h, (R)C.compliance, (R)lam[0], dx);
        pos_apply(a, b, p, dl, dx);
        lam[0] += (double)dl;
    } break;
    case CON_MUTUAL_ORIENTATION: {  // pbd.cpp:156-173
        Acpd<R> A = acpd(a, b);
        Qt<R> aux = qmul(wq<R>(a.q), qinverse(wq<R>(b.q)));
        V3<R> dq = v3<R>((R)2.0 * aux.x, (R)2.0 * aux.y, (R)2.0 * aux.z);
        R dl = ang_dlambda(A, h, (R)C.compliance, (R)lam[0], dq);
        ang_apply(a, b, A, dl, dq);
        lam[0] += (double)dl;
    } break;
    case CON_HINGE: {  // pbd.cpp:245-299
        Acpd<R> A = acpd(a, b);
        V3<R> dq = vcross(qaxis(wq<R>(a.q), C.a1), qaxis(wq<R>(b.q), C.a2));
        R dl = ang_dlambda(A, h, (R)C.compliance, (R)lam[1], dq);
        ang_apply(a, b, A, dl, dq);
        lam[1] += (double)dl;
        Pcpd<R> p = pcpd(a, b, r1, r2);
        V3<R> dx = anchor_delta<R, EXACT>(a, b, p.r1, p.r2);
        dl = pos_dlambda(a, b, p, h, (R)0, (R)lam[0], dx);
        pos_apply(a, b, p, dl, dx);
        lam[0] += (double)dl;
        bool act = C.limited != 0;
        if (act && !EXACT) {
            const Qt<float> qa = qcast<float>(a.q), qb = qcast<float>(b.q);
            act = limit_may_act(qaxis(qa, C.a1), qaxis(qa, C.l1), qaxis(qb, C.l2), C.lo, C.hi);
        }
        if (act) {
            V3<double> n1 = qaxis(a.q, C.l1), n2 = qaxis(b.q, C.l2), n = qaxis(a.q, C.a1), dq64;
            if (limit_angle<double>(n, n1, n2, C.lo, C.hi, dq64)) {
                dq = v3cast<R>(dq64);
                Acpd<R> B = acpd(a, b);
                R dl2 = ang_dlambda(B, h, (R)0, (R)lam[2], dq);
                ang_apply(a, b, B, dl2, dq);
                lam[2] += (double)dl2;
            }
        }
    } break;
    case CON_SPHERICAL: {  // pbd.cpp:301-379
        Pcpd<R> p = pcpd(a, b, r1, r2);
        V3<R> dx = anchor_delta<R, EXACT>(a, b, p.r1, p.r2);
        R dl = pos_dlambda(a, b, p, h, (R)0, (R)lam[0], dx);
        pos_apply(a, b, p, dl, dx);
        lam[0] += (double)dl;
        // swing and twist limits: axes and angles in FP64 (see limit_angle), after an FP32 screen
        const double EPS64 = 1e-50;
        bool swing = true, twist = true;
        if (!EXACT) {
            const Qt<float> qa = qcast<float>(a.q), qb = qcast<float>(b.q);
            V3<float> f1 = qaxis(qa, C.a1), f2 = qaxis(qb, C.a2), fn = vcross(f1, f2);
            const float fl = vlen(fn);
            // limits at or beyond +-pi never act, however parallel the swing axes are
            swing = !(C.lo <= -PI_REF && C.hi >= PI_REF) && (fl < 1e-3f || limit_may_act(vscale(1.f / fl, fn), f1, f2, C.lo, C.hi));
        }
        V3<double> n1 = qaxis(a.q, C.a1), n2 = qaxis(b.q, C.a2);
        V3<double> n = vcross(n1, n2);
        double nl = swing ? vlen(n) : 0.0;
        if (nl > EPS64) {
            n = v3<double>(n.x / nl, n.y / nl, n.z / nl);
            V3<double> dq64;
            if (limit_angle<double>(n, n1, n2, C.lo, C.hi, dq64)) {
                V3<R> dq = v3cast<R>(dq64);
                Acpd<R> A = acpd(a, b);
                R d2 = ang_dlambda(A, h, (R)0, (R)lam[1], dq);
                ang_apply(a, b, A, d2, dq);
                lam[1] += (double)d2;
            }
        }
        if (!EXACT) {   // screened on the orientations after the swing correction
            const Qt<float> qa = qcast<float>(a.q), qb = qcast<float>(b.q);
            V3<float> f1 = qaxis(qa, C.a1), f2 = qaxis(qb, C.a2);
            V3<float> g1 = qaxis(qa, C.l1), g2 = qaxis(qb, C.l2), gn = vadd(f1, f2);
            const float gl = vlen(gn);
            const bool never = C.lo2 <= -PI_REF && C.hi2 >= PI_REF;
            if (gl < 1e-3f) {
                twist = !never;
            } else {
                gn = vscale(1.f / gl, gn);
                V3<float> h1 = vsub(g1, vscale(vdot(gn, g1), gn)), h2 = vsub(g2, vscale(vdot(gn, g2), gn));
                const float l1 = vlen(h1), l2 = vlen(h2);
                twist = (l1 < 1e-3f || l2 < 1e-3f) ? !never
                                                   : limit_may_act(gn, vscale(1.f / l1, h1), vscale(1.f / l2, h2), C.lo2, C.hi2);
            }
        }
        V3<double> a1 = qaxis(a.q, C.a1), b1 = qaxis(a.q, C.l1);
        V3<double> a2 = qaxis(b.q, C.a2), b2 = qaxis(b.q, C.l2);
        n = vadd(a1, a2);
        nl = twist ? vlen(n) : 0.0;
        if (nl > EPS64) {
            n = v3<double>(n.x / nl, n.y / nl, n.z / nl);
            n1 = vsub(b1, vscale(vdot(n, b1), n));
            n2 = vsub(b2, vscale(vdot(n, b2), n));
            double l1 = vlen(n1), l2 = vlen(n2);
            if (l1 > EPS64 && l2 > EPS64) {
                n1 = v3<double>(n1.x / l1, n1.y / l1, n1.z / l1);
                n2 = v3<double>(n2.x / l2, n2.y / l2, n2.z / l2);
                V3<double> dq64;
                if (limit_angle<double>(n, n1, n2, C.lo2, C.hi2, dq64)) {
                    V3<R> dq = v3cast<R>(dq64);
                    Acpd<R> A = acpd(a, b);
                    R d2 = ang_dlambda(A, h, (R)0, (R)lam[2], dq);
                    ang_apply(a, b, A, d2, dq);
                    lam[2] += (double)d2;
                }
            }
        }
    } break;
    default: break;
    }
    store_pose(W, a);
    store_pose(W, b);
}

// --------------------------------------------------------------------------------------------
// FP32 build: a node's bodies as an FP64 base pose plus FP32 deltas.
//
// A solver node applies a handful of small corrections to its two bodies. Each body's pose is read
// once in FP64 (x0, q0); corrections accumulate in FP32 deltas (dx, dq) relative to it, and the FP64
// pose is written back once: x = x0 + dx, q = normalize(q0 + dq). The renormalisation after every
// orientation update (pbd_base_constraints.cpp:83-103) is carried out exactly in delta form:
// with u = dq + increment and e = |q0 + u|^2 - 1 = 2 q0.u + u.u, the normalised quaternion is
// q0 + q0 (r - 1) + u r with r - 1 = -e / (s (1 + s)), s = sqrt(1 + e), all of which are small,
// well-conditioned FP32 quantities. Per contact the solve then needs no FP64 arithmetic at all.
// FP32 build: a body during the substep's position sweep. Its FP64 pose stays at the predicted pose
// (pos / rot); the sweep's corrections accumulate per body in FP32 deltas (sdx, sdq), and the pose is
// folded into FP64 once per substep (fold_body), so FP64 carries the pose across substeps while the
// solve itself runs in FP32. A node loads the body's FP32 orientation (pose_f) and deltas and stores
// the deltas back.
struct FBody {
    V3<float> dx;
    Qt<float> q0f, dq;
    float invm;
    float S[6];   // local inverse inertia, symmetric storage (xx yy zz xy xz yz)
    bool fixed;
    int idx;
    __device__ __forceinline__ Qt<float> q() const { return qt<float>(q0f.x + dq.x, q0f.y + dq.y, q0f.z + dq.z, q0f.w + dq.w); }
};

__device__ __forceinline__ FBody load_fbody(const WorldView<float>& W, int b) {
    FBody B;
    const float4 qf = W.pose_f[2 * b + 1], d = W.sdx[b], q = W.sdq[b];
    B.q0f = qt<float>(qf.x, qf.y, qf.z, qf.w);
    B.dx = v3<float>(d.x, d.y, d.z);
    B.dq = qt<float>(q.x, q.y, q.z, q.w);
    B.invm = W.inv_mass[b];
#pragma unroll
    for (int i = 0; i < 6; ++i) B.S[i] = W.inv_inertia[6 * b + i];
    B.fixed = W.fixed[b] != 0;
    B.idx = b;
    return B;
}

__device__ __forceinline__ void store_fbody(const WorldView<float>& W, const FBody& B) {
    if (B.fixed) return;
    W.sdx[B.idx] = make_float4(B.dx.x, B.dx.y, B.dx.z, 0.f);
    W.sdq[B.idx] = make_float4(B.dq.x, B.dq.y, B.dq.z, B.dq.w);
}

// (float)(x_a - x_b) of two bodies' predicted positions, as stored in pair_base / ext_base
__device__ __forceinline__ float4 fbase4(const WorldView<float>& W, int a, int b) {
    const double4_32a pa = W.pos[a], pb = W.pos[b];
    return make_float4((float)(pa.x - pb.x), (float)(pa.y - pb.y), (float)(pa.z - pb.z), 0.f);
}


// The position sweep's corrections into the FP64 pose (x += dx, q = normalize(q + dq)), and the
// FP32 orientation copy the velocity sweep reads; bodies the sweep did not touch keep their pose.
__device__ __forceinline__ void fold_body(const WorldView<float>& W, int b) {
    const float4 d = W.sdx[b], q = W.sdq[b];
    if (d.x == 0.f && d.y == 0.f && d.z == 0.f && q.x == 0.f && q.y == 0.f && q.z == 0.f && q.w == 0.f) return;
    const double4_32a p4 = W.pos[b], q4 = W.rot[b];
    const Qt<double> nq = qnormalize_fast(qt<double>(q4.x + (double)q.x, q4.y + (double)q.y, q4.z + (double)q.z,
                                                     q4.w + (double)q.w));
    W.pos[b] = make_double4_32a(p4.x + (double)d.x, p4.y + (double)d.y, p4.z + (double)d.z, 0.0);
    W.rot[b] = make_double4_32a(nq.x, nq.y, nq.z, nq.w);
    W.pose_f[2 * b + 1] = make_float4((float)nq.x, (float)nq.y, (float)nq.z, (float)nq.w);
}

// q <- normalize(q + inc), in delta form
__device__ __forceinline__ void frot_update(FBody& B, Qt<float> inc) {
    Qt<float> u = qt<float>(B.dq.x + inc.x, B.dq.y + inc.y, B.dq.z + inc.z, B.dq.w + inc.w);
    float e = 2.f * (B.q0f.x * u.x + B.q0f.y * u.y + B.q0f.z * u.z + B.q0f.w * u.w) + (u.x * u.x + u.y * u.y + u.z * u.z + u.w * u.w);
    const float u1 = 1.f + e;   // |q0 + u|^2, close to 1
    float s = u1 * rsqrtf(u1);
    float rm1 = __fdividef(-e, s * (1.f + s));
    float r = 1.f + rm1;
    B.dq = qt<float>(B.q0f.x * rm1 + u.x * r, B.q0f.y * rm1 + u.y * r, B.q0f.z * rm1 + u.z * r, B.q0f.w * rm1 + u.w * r);
}

// FP32 delta-form arithmetic: unit vectors from the reciprocal square root of the special-function
// unit and divisions by __fdividef (each within 2 ulp), shorter dependent chains than IEEE sqrtf and
// division in the serial Gauss-Seidel chains; squared lengths at or below 1e-36 take the IEEE path
// (rsqrtf flushes subnormal inputs).
__device__ __forceinline__ float funit(V3<float> v, V3<float>& n) {
    const float c2 = v.x * v.x + v.y * v.y + v.z * v.z;
    if (c2 > 1e-36f) {
        const float r = rsqrtf(c2);
        n = v3<float>(v.x * r, v.y * r, v.z * r);
        return c2 * r;
    }
    const float c = vlen(v);
    if (c > 0.f) n = v3<float>(v.x / c, v.y / c, v.z / c);
    return c;
}

// The world inverse inertia applied to v at the body's current orientation, R (S (R^T v)): the
// products the reference forms with the world tensor R S R^T (physics_util.cpp:26-63), without
// keeping the tensor itself live through the solve (the FP32 path's register budget).
__device__ __forceinline__ V3<float> fIinv(const FBody& B, V3<float> v) {
    const M3<float> R = qmat3(B.q());
    const V3<float> l = v3<float>(R.d[0][0] * v.x + R.d[1][0] * v.y + R.d[2][0] * v.z,
                                  R.d[0][1] * v.x + R.d[1][1] * v.y + R.d[2][1] * v.z,
                                  R.d[0][2] * v.x + R.d[1][2] * v.y + R.d[2][2] * v.z);
    const V3<float> t = v3<float>(B.S[0] * l.x + B.S[3] * l.y + B.S[4] * l.z, B.S[3] * l.x + B.S[1] * l.y + B.S[5] * l.z,
                                  B.S[4] * l.x + B.S[5] * l.y + B.S[2] * l.z);
    return mmulv(R, t);
}

// calculate_positional_constraint_preprocessed_data on the FP32 path: the anchors in world axes (the
// inertia products are taken by fIinv at the same orientations, before the correction moves them)
struct FPcpd { V3<float> r1, r2; };
__device__ __forceinline__ FPcpd fpcpd(const FBody& a, const FBody& b, V3<float> r1_lc, V3<float> r2_lc) {
    FPcpd p;
    p.r1 = qrotate(a.q(), r1_lc);
    p.r2 = qrotate(b.q(), r2_lc);
    return p;
}

__device__ __forceinline__ float fpos_dlambda(const FBody& a, const FBody& b, const FPcpd& p, float lambda_til_free, V3<float> dx) {
    (void)lambda_til_free;
    V3<float> n;
    const float c = funit(dx, n);
    if (c <= 0.f) return 0.f;
    const V3<float> c1 = vcross(p.r1, n), c2 = vcross(p.r2, n);
    float w1 = a.invm + vdot(c1, fIinv(a, c1));
    float w2 = b.invm + vdot(c2, fIinv(b, c2));
    return __fdividef(-c, w1 + w2);   // contacts carry zero compliance (pbd.cpp:123,133)
}

__device__ __forceinline__ void fpos_apply(FBody& a, FBody& b, const FPcpd& p, float dl, V3<float> dx) {
    V3<float> n;
    const float c = funit(dx, n);
    if (c <= 0.f) return;
    V3<float> imp = vscale(dl, n);
    if (!a.fixed) a.dx = vadd(a.dx, vscale(a.invm, imp));
    if (!b.fixed) b.dx = vadd(b.dx, vscale(-b.invm, imp));
    V3<float> a1 = fIinv(a, vcross(p.r1, imp));
    V3<float> a2 = fIinv(b, vcross(p.r2, imp));
    Qt<float> q1 = qmul(qt<float>(a1.x, a1.y, a1.z, 0.f), a.q());
    Qt<float> q2 = qmul(qt<float>(a2.x, a2.y, a2.z, 0.f), b.q());
    if (!a.fixed) frot_update(a, qt<float>(0.5f * q1.x, 0.5f * q1.y, 0.5f * q1.z, 0.5f * q1.w));
    if (!b.fixed) frot_update(b, qt<float>(-0.5f * q2.x, -0.5f * q2.y, -0.5f * q2.z, -0.5f * q2.w));
}

// collision_constraint_solve (pbd.cpp:107-154) on FP32 deltas; base_ab = (float)(x0_a - x0_b)
static __device__ void fcollision_solve(const WorldView<float>& W, FBody& a, FBody& b, V3<float> base_ab, float* c, float mus) {
    V3<float> r1 = v3<float>(c[0], c[1], c[2]), r2 = v3<float>(c[4], c[5], c[6]), n = v3<float>(c[8], c[9], c[10]);
    float lambda_n = c[3], lambda_t = c[7];
    FPcpd p = fpcpd(a, b, r1, r2);
    V3<float> d12 = vadd(vadd(base_ab, vsub(a.dx, b.dx)), vsub(p.r1, p.r2));
    float d = vdot(d12, n);
    if (d > 0.f) {
        V3<float> dx = vscale(d, n);
        float dl = fpos_dlambda(a, b, p, 0.f, dx);
        fpos_apply(a, b, p, dl, dx);
        lambda_n += dl;
        p = fpcpd(a, b, r1, r2);
        dl = fpos_dlambda(a, b, p, 0.f, dx);
        float lt = lambda_t + dl;
        if (lt > mus * lambda_n) {
            // displacement since the substep began: the predict step's (pred_d, FP32 from the FP64 poses)
            // plus the sweep's; the previous orientations' FP32 copies (prev_qf)
            const float4 pda = W.pred_d[a.idx], pdb = W.pred_d[b.idx], qa = W.prev_qf[a.idx], qb = W.prev_qf[b.idx];
            Qt<float> qa_prev = qt<float>(qa.x, qa.y, qa.z, qa.w), qb_prev = qt<float>(qb.x, qb.y, qb.z, qb.w);
            V3<float> da = vadd(vadd(v3<float>(pda.x, pda.y, pda.z), a.dx), vsub(p.r1, qrotate(qa_prev, r1)));
            V3<float> db = vadd(vadd(v3<float>(pdb.x, pdb.y, pdb.z), b.dx), vsub(p.r2, qrotate(qb_prev, r2)));
            V3<float> dp = vsub(da, db);
            V3<float> dpt = vsub(dp, vscale(vdot(dp, n), n));
            fpos_apply(a, b, p, dl, dpt);
            lambda_t += dl;
        }
    }
    c[3] = lambda_n;
    c[7] = lambda_t;
}

// --------------------------------------------------------------------------------------------
// External constraints of the FP32 build on FP64-base / FP32-delta bodies (pbd.cpp:81-379): the
// same order of corrections as ext_solve, each applied to the FP32 deltas; joint-limit angles are
// screened in FP32 and evaluated in FP64 (from the FP64 orientation q0 + dq) where they may act.
__device__ __forceinline__ float fdlambda(float c, float w1, float w2, float h, float compliance, float lambda) {
    const float til = __fdividef(compliance, h * h);
    return __fdividef(-c - til * lambda, w1 + w2 + til);
}

__device__ __forceinline__ float fpos_dlambda_c(const FBody& a, const FBody& b, const FPcpd& p, float h,
                                                float compliance, float lambda, V3<float> dx) {
    V3<float> n;
    const float c = funit(dx, n);
    if (c <= 0.f) return 0.f;
    const V3<float> c1 = vcross(p.r1, n), c2 = vcross(p.r2, n);
    const float w1 = a.invm + vdot(c1, fIinv(a, c1));
    const float w2 = b.invm + vdot(c2, fIinv(b, c2));
    return fdlambda(c, w1, w2, h, compliance, lambda);
}

// ang_dlambda on the FP32 path
__device__ __forceinline__ float fang_dlambda(const FBody& a, const FBody& b, float h, float compliance, float lambda, V3<float> dq) {
    V3<float> n;
    const float th = funit(dq, n);
    if (th <= 0.f) return 0.f;
    return fdlambda(th, vdot(n, fIinv(a, n)), vdot(n, fIinv(b, n)), h, compliance, lambda);
}

__device__ __forceinline__ void fang_apply(FBody& a, FBody& b, float dl, V3<float> dq) {
    V3<float> n;
    const float th = funit(dq, n);
    if (th <= 0.f) return;
    const V3<float> imp = vscale(-dl, n);
    const V3<float> a1 = fIinv(a, imp), a2 = fIinv(b, imp);
    const Qt<float> q1 = qmul(qt<float>(a1.x, a1.y, a1.z, 0.f), a.q());
    const Qt<float> q2 = qmul(qt<float>(a2.x, a2.y, a2.z, 0.f), b.q());
    if (!a.fixed) frot_update(a, qt<float>(0.5f * q1.x, 0.5f * q1.y, 0.5f * q1.z, 0.5f * q1.w));
    if (!b.fixed) frot_update(b, qt<float>(-0.5f * q2.x, -0.5f * q2.y, -0.5f * q2.z, -0.5f * q2.w));
}

// the FP64 orientation of a body in delta form (the predicted FP64 orientation plus the sweep's delta)
__device__ __forceinline__ Qt<double> fq64(const WorldView<float>& W, const FBody& B) {
    const double4_32a q = W.rot[B.idx];
    return qt<double>(q.x + (double)B.dq.x, q.y + (double)B.dq.y, q.z + (double)B.dq.z, q.w + (double)B.dq.w);
}

// angular correction of one joint limit (limit_angle's dq, FP64) on the deltas
__device__ __forceinline__ void flimit_apply(FBody& a, FBody& b, V3<double> dq64, float h, float* lam) {
    const V3<float> dq = v3cast<float>(dq64);
    V3<float> n;
    const float th = funit(dq, n);
    if (th <= 0.f) return;
    const float dl = fdlambda(th, vdot(n, fIinv(a, n)), vdot(n, fIinv(b, n)), h, 0.f, *lam);
    fang_apply(a, b, dl, dq);
    *lam += dl;
}

// FP64 evaluation of a joint limit that the FP32 screen could not rule out (rare): kind 0 the hinge
// limit (pbd.cpp:279-298), 1 the spherical swing limit, 2 the spherical twist limit (pbd.cpp:327-378),
// each from the FP64 orientations q0 + dq, applying its correction to a and b. Out of line, so that
// the joint solve's common path keeps its values in registers.
static __device__ __noinline__ void flimit64(const WorldView<float>& W, FBody& a, FBody& b, const ExtConstraint& C, float h,
                                             float* lam, int kind) {
    const double EPS64 = 1e-50;
    const Qt<double> qa = fq64(W, a), qb = fq64(W, b);
    V3<double> dq64;
    if (kind == 0) {
        if (limit_angle<double>(qaxis(qa, C.a1), qaxis(qa, C.l1), qaxis(qb, C.l2), C.lo, C.hi, dq64))
            flimit_apply(a, b, dq64, h, &lam[2]);
    } else if (kind == 1) {
        const V3<double> n1 = qaxis(qa, C.a1), n2 = qaxis(qb, C.a2);
        const V3<double> n = vcross(n1, n2);
        const double nl = vlen(n);
        if (nl > EPS64 && limit_angle<double>(v3<double>(n.x / nl, n.y / nl, n.z / nl), n1, n2, C.lo, C.hi, dq64))
            flimit_apply(a, b, dq64, h, &lam[1]);
    } else {
        const V3<double> a1 = qaxis(qa, C.a1), b1 = qaxis(qa, C.l1), a2 = qaxis(qb, C.a2), b2 = qaxis(qb, C.l2);
        V3<double> n = vadd(a1, a2);
        const double nl = vlen(n);
        if (nl > EPS64) {
            n = v3<double>(n.x / nl, n.y / nl, n.z / nl);
            const V3<double> n1 = vsub(b1, vscale(vdot(n, b1), n)), n2 = vsub(b2, vscale(vdot(n, b2), n));
            const double l1 = vlen(n1), l2 = vlen(n2);
            if (l1 > EPS64 && l2 > EPS64 &&
                limit_angle<double>(n, v3<double>(n1.x / l1, n1.y / l1, n1.z / l1), v3<double>(n2.x / l2, n2.y / l2, n2.z / l2),
                                    C.lo2, C.hi2, dq64))
                flimit_apply(a, b, dq64, h, &lam[2]);
        }
    }
}

// lam: the joint's Lagrange multipliers of the substep as FP32 (they start at zero every substep and
// enter only through compliance, zero for the joints of the workloads); base: (float)(x_e1 - x_e2)
// of the predicted positions, rounded once per substep by the cull.
static __device__ void fext_solve(const WorldView<float>& W, const ExtConstraint& C, float4 base, float* lam, float h) {
    FBody a = load_fbody(W, C.e1), b = load_fbody(W, C.e2);
    const V3<float> r1 = v3<float>(C.r1f[0], C.r1f[1], C.r1f[2]);
    const V3<float> r2 = v3<float>(C.r2f[0], C.r2f[1], C.r2f[2]);
    const V3<float> base_ab = v3<float>(base.x, base.y, base.z);
    auto anchor = [&](const FPcpd& p) { return vadd(vadd(base_ab, vsub(a.dx, b.dx)), vsub(p.r1, p.r2)); };
    switch (C.type) {
    case CON_POSITIONAL: {  // pbd.cpp:81-97
        const double4_32a pa = W.pos[C.e1], pb = W.pos[C.e2];
        const V3<float> base = v3<float>((float)((pa.x - pb.x) - C.distance[0]), (float)((pa.y - pb.y) - C.distance[1]),
                                         (float)((pa.z - pb.z) - C.distance[2]));
        const V3<float> dx = vadd(base, vsub(a.dx, b.dx));
        const FPcpd p = fpcpd(a, b, r1, r2);
        const float dl = fpos_dlambda_c(a, b, p, h, C.compliance_f, lam[0], dx);
        fpos_apply(a, b, p, dl, dx);
        lam[0] += dl;
    } break;
    case CON_MUTUAL_ORIENTATION: {  // pbd.cpp:156-173
        const Qt<float> aux = qmul(a.q(), qinverse(b.q()));
        const V3<float> dq = v3<float>(2.f * aux.x, 2.f * aux.y, 2.f * aux.z);
        const float dl = fang_dlambda(a, b, h, C.compliance_f, lam[0], dq);
        fang_apply(a, b, dl, dq);
        lam[0] += dl;
    } break;
    case CON_HINGE: {  // pbd.cpp:245-299
        const V3<float> dq = vcross(qaxis(a.q(), C.a1), qaxis(b.q(), C.a2));
        float dl = fang_dlambda(a, b, h, C.compliance_f, lam[1], dq);
        fang_apply(a, b, dl, dq);
        lam[1] += dl;
        const FPcpd p = fpcpd(a, b, r1, r2);
        const V3<float> dx = anchor(p);
        dl = fpos_dlambda_c(a, b, p, h, 0.f, lam[0], dx);
        fpos_apply(a, b, p, dl, dx);
        lam[0] += dl;
        if (C.limited && limit_may_act(qaxis(a.q(), C.a1), qaxis(a.q(), C.l1), qaxis(b.q(), C.l2), C.lo, C.hi)) {
            flimit64(W, a, b, C, h, lam, 0);
        }
    } break;
    case CON_SPHERICAL: {  // pbd.cpp:301-379
        const FPcpd p = fpcpd(a, b, r1, r2);
        const V3<float> dx = anchor(p);
        const float dl = fpos_dlambda_c(a, b, p, h, 0.f, lam[0], dx);
        fpos_apply(a, b, p, dl, dx);
        lam[0] += dl;
        {   // swing
            const V3<float> f1 = qaxis(a.q(), C.a1), f2 = qaxis(b.q(), C.a2), fn = vcross(f1, f2);
            const float fl = vlen(fn);
            const bool never = C.lo <= -PI_REF && C.hi >= PI_REF;   // limits at or beyond +-pi never act
            if (!never && (fl < 1e-3f || limit_may_act(vscale(1.f / fl, fn), f1, f2, C.lo, C.hi))) {
                flimit64(W, a, b, C, h, lam, 1);
            }
        }
        {   // twist, on the orientations after the swing correction
            const V3<float> f1 = qaxis(a.q(), C.a1), f2 = qaxis(b.q(), C.a2);
            const V3<float> g1 = qaxis(a.q(), C.l1), g2 = qaxis(b.q(), C.l2);
            V3<float> gn = vadd(f1, f2);
            const float gl = vlen(gn);
            const bool never = C.lo2 <= -PI_REF && C.hi2 >= PI_REF;
            bool act;
            if (gl < 1e-3f) {
                act = !never;
            } else {
                gn = vscale(1.f / gl, gn);
                const V3<float> h1 = vsub(g1, vscale(vdot(gn, g1), gn)), h2 = vsub(g2, vscale(vdot(gn, g2), gn));
                const float l1 = vlen(h1), l2 = vlen(h2);
                act = (l1 < 1e-3f || l2 < 1e-3f) ? !never
                                                 : limit_may_act(gn, vscale(1.f / l1, h1), vscale(1.f / l2, h2), C.lo2, C.hi2);
            }
            if (act) flimit64(W, a, b, C, h, lam, 2);
        }
    } break;
    default: break;
    }
    store_fbody(W, a);
    store_fbody(W, b);
}

// FP32 build: after predict, the FP32 copies the substep's sweeps work from (the pose, the predict
// step's displacement and the previous orientation) and zero sweep deltas.
__device__ __forceinline__ void stage_body(const WorldView<float>& W, int b) {
    const double4_32a p = W.pos[b], q = W.rot[b], pp = W.prev_pos[b], pq = W.prev_rot[b];
    W.pose_f[2 * b] = make_float4((float)p.x, (float)p.y, (float)p.z, 0.f);
    W.pose_f[2 * b + 1] = make_float4((float)q.x, (float)q.y, (float)q.z, (float)q.w);
    W.sdx[b] = make_float4(0.f, 0.f, 0.f, 0.f);
    W.sdq[b] = make_float4(0.f, 0.f, 0.f, 0.f);
    W.pred_d[b] = make_float4((float)(p.x - pp.x), (float)(p.y - pp.y), (float)(p.z - pp.z), 0.f);
    W.prev_qf[b] = make_float4((float)pq.x, (float)pq.y, (float)pq.z, (float)pq.w);
}

// --------------------------------------------------------------------------------------------
// Predict (pbd.cpp:537-577) for one body
template <typename R, bool EXACT>
__device__ void predict_body(const WorldView<R>& W, int b, double h) {
    double4_32a p = W.pos[b], q4 = W.rot[b];
    W.prev_pos[b] = p;
    W.prev_rot[b] = q4;
    if (W.fixed[b] || !W.active[b]) return;
    V3<double> x = v3<double>(p.x, p.y, p.z);
    Qt<double> q = qt<double>(q4.x, q4.y, q4.z, q4.w);
    V3<R> v = v3<R>(W.vel[3 * b], W.vel[3 * b + 1], W.vel[3 * b + 2]);
    V3<R> w = v3<R>(W.omega[3 * b], W.omega[3 * b + 1], W.omega[3 * b + 2]);
    V3<R> F = v3<R>((R)W.force[3 * b], (R)W.force[3 * b + 1], (R)W.force[3 * b + 2]);
    V3<R> T = v3<R>((R)W.torque[3 * b], (R)W.torque[3 * b + 1], (R)W.torque[3 * b + 2]);
    R invm = W.inv_mass[b];
    R si[6], sI[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) { si[i] = W.inv_inertia[6 * b + i]; sI[i] = W.inertia[6 * b + i]; }
    R hR = (R)h;
    v = vadd(v, vscale(hR * invm, F));
    if (EXACT) x = vadd(x, v3cast<double>(vscale(hR, v)));
    else x = vadd(x, vscale(h, v3cast<double>(v)));
    Qt<R> qw = wq<R>(q);
    M3<R> Iinv = world_tensor(qw, msym(si)), I = world_tensor(qw, msym(sI));
    w = vadd(w, vscale(hR, mmulv(Iinv, vsub(T, vcross(w, mmulv(I, w))))));
    Qt<R> qd = qmul(qt<R>(w.x, w.y, w.z, (R)0), qw);
    if (EXACT) {
        q.x = q.x + h * 0.5 * (double)qd.x; q.y = q.y + h * 0.5 * (double)qd.y;
        q.z = q.z + h * 0.5 * (double)qd.z; q.w = q.w + h * 0.5 * (double)qd.w;
        q = qnormalize(q);
    } else {
        R s = hR * (R)0.5;
        q.x = q.x + (double)(s * qd.x); q.y = q.y + (double)(s * qd.y);
        q.z = q.z + (double)(s * qd.z); q.w = q.w + (double)(s * qd.w);
        q = qnormalize_fast(q);
    }
    W.pos[b] = make_double4_32a(x.x, x.y, x.z, 0.0);
    W.rot[b] = make_double4_32a(q.x, q.y, q.z, q.w);
    W.vel[3 * b] = v.x; W.vel[3 * b + 1] = v.y; W.vel[3 * b + 2] = v.z;
    W.omega[3 * b] = w.x; W.omega[3 * b + 1] = w.y; W.omega[3 * b + 2] = w.z;
}

// PBD velocity update (pbd.cpp:623-643) for one body
template <typename R, bool EXACT>
__device__ void velocity_body(const WorldView<R>& W, int b, double h) {
    if (W.fixed[b] || !W.active[b]) return;
#pragma unroll
    for (int i = 0; i < 3; ++i) { W.prev_vel[3 * b + i] = W.vel[3 * b + i]; W.prev_omega[3 * b + i] = W.omega[3 * b + i]; }
    double4_32a p = W.pos[b], pp = W.prev_pos[b], q4 = W.rot[b], pq4 = W.prev_rot[b];
    V3<double> dx = vsub(v3<double>(p.x, p.y, p.z), v3<double>(pp.x, pp.y, pp.z));
    if (EXACT) {
        V3<double> v = vscale(1.0 / h, dx);
        Qt<double> dq = qmul(qt<double>(q4.x, q4.y, q4.z, q4.w), qinverse(qt<double>(pq4.x, pq4.y, pq4.z, pq4.w)));
        V3<double> w = (dq.w >= 0.0) ? vscale(2.0 / h, v3<double>(dq.x, dq.y, dq.z)) : vscale(-2.0 / h, v3<double>(dq.x, dq.y, dq.z));
        W.vel[3 * b] = (R)v.x; W.vel[3 * b + 1] = (R)v.y; W.vel[3 * b + 2] = (R)v.z;
        W.omega[3 * b] = (R)w.x; W.omega[3 * b + 1] = (R)w.y; W.omega[3 * b + 2] = (R)w.z;
        return;
    }
    // FP32 build: only the pose differences are formed in FP64. With q = q_prev + d,
    // q * q_prev^-1 = (0, 0, 0, |q_prev|^2) + d * q_prev^-1, so its vector part is d * q_prev^-1.
    const R inv_h = (R)(1.0 / h);
    V3<R> v = vscale(inv_h, v3cast<R>(dx));
    Qt<R> d = qt<R>((R)(q4.x - pq4.x), (R)(q4.y - pq4.y), (R)(q4.z - pq4.z), (R)(q4.w - pq4.w));
    Qt<R> qpi = qinverse(qt<R>((R)pq4.x, (R)pq4.y, (R)pq4.z, (R)pq4.w));
    Qt<R> dq = qmul(d, qpi);
    R sgn = ((R)1 + dq.w >= (R)0) ? (R)2 * inv_h : (R)-2 * inv_h;
    W.vel[3 * b] = v.x; W.vel[3 * b + 1] = v.y; W.vel[3 * b + 2] = v.z;
    W.omega[3 * b] = sgn * dq.x; W.omega[3 * b + 1] = sgn * dq.y; W.omega[3 * b + 2] = sgn * dq.z;
}

// Velocity solver for one contact (pbd.cpp:646-711); velocities of the two bodies are in registers.
// p: the contact's preprocessed data from the current poses (anchors in world orientation, world
// inverse inertias); a / b: inverse mass and fixed flag of the two bodies.
template <typename R>
struct VelBody { R invm; bool fixed; };

template <typename R, bool EXACT>
__device__ void contact_velocity(const Pcpd<R>& p, VelBody<R> a, VelBody<R> b, const R* c, R h, R mud, R e,
                                 V3<R>& va, V3<R>& wa, V3<R>& vb, V3<R>& wb, V3<R> pva, V3<R> pwa, V3<R> pvb, V3<R> pwb) {
    V3<R> n = v3<R>(c[8], c[9], c[10]);
    R lambda_n = c[3];
    V3<R> v = vsub(vadd(va, vcross(wa, p.r1)), vadd(vb, vcross(wb, p.r2)));
    R vn = vdot(n, v);
    V3<R> vt = vsub(v, vscale(vn, n));
    V3<R> dv = v3<R>(0, 0, 0);
    R fn = lambda_n / h;
    R x1 = mud * fabs(fn), x2 = vlen(vt);
    R fact = (x1 < x2) ? x1 : x2;
    dv = vadd(dv, vscale(-fact, vnorm(vt)));
    V3<R> vtil = vsub(vadd(pva, vcross(pwa, p.r1)), vadd(pvb, vcross(pwb, p.r2)));
    R vntil = vdot(n, vtil);
    R m = -e * vntil;
    fact = -vn + ((m < (R)0.0) ? m : (R)0.0);
    dv = vadd(dv, vscale(fact, n));
    R w1 = a.invm + vdot(vcross(p.r1, n), mmulv(p.I1, vcross(p.r1, n)));
    R w2 = b.invm + vdot(vcross(p.r2, n), mmulv(p.I2, vcross(p.r2, n)));
    V3<R> P = vscale((R)1.0 / (w1 + w2), dv);
    if (!a.fixed) {
        va = vadd(va, vscale(a.invm, P));
        wa = vadd(wa, mmulv(p.I1, vcross(p.r1, P)));
    }
    if (!b.fixed) {
        vb = vadd(vb, vinv(vscale(b.invm, P)));
        wb = vadd(wb, vinv(mmulv(p.I2, vcross(p.r2, P))));
    }
}

}  // namespace rp
