// Reverse-mode derivative of the XPBD substep (the adjoint of pbd_simulate_with_constraints,
// src/physics/pbd.cpp:468-747): free bodies under gravity, the external joints (positional, mutual
// orientation, hinge, spherical, with limits) and, with collisions enabled, hull-hull contacts
// (GJK/EPA normal, clipped manifold, normal and static-friction solve, velocity solver with dynamic
// friction and restitution; rp_adjoint_contact.cuh).
//
// One thread differentiates one scene. The forward substep is written once, templated on its scalar
// type S: with S = double it reproduces the all-FP64 step (same operations in the same order, built
// without FMA contraction) and runs the trajectory and its checkpoints; with S = AVar every operation
// also appends (parent ids, partial derivatives) to the thread's tape, and the tape swept backwards
// turns the adjoint of a substep's end state into the adjoint of its start state. Trajectories are
// checkpointed every K frames; the backward pass recomputes each K-frame segment from its checkpoint,
// keeping the start state of every substep and the discrete state of every frame (broad-phase
// pairs, awake bodies), then replays and reverses the substeps last to first.
//
// Held fixed, as derivatives of discrete events: the broad-phase pair list and the set of awake
// bodies of each frame, every branch taken at a comparison (a joint limit or a contact acting or
// not, static friction holding or not, a clipping test), the support vertices and faces that GJK,
// EPA and the clipping select, and the FP32 roundings of the clipping (differentiated as identity).
#pragma once
#include <math.h>
#include "rp_math.cuh"
#include "rp_world.h"

namespace rp {

// ---------------------------------------------------------------------------------------------
// Tape
struct Tape {
    int2* ab;          // parents of each entry (-1: none)
    double2* d;        // partial derivatives with respect to the two parents
    double* adj;       // adjoints, swept backwards
    int n, cap, overflow;
};

constexpr int ADJ_BLOCK = 32;
__shared__ Tape s_tape[ADJ_BLOCK];

struct AVar {
    double v;
    int id;            // tape entry, -1 for a constant
    __device__ AVar() : v(0.0), id(-1) {}
    __device__ AVar(double x) : v(x), id(-1) {}
    __device__ AVar(double x, int i) : v(x), id(i) {}
};

__device__ __forceinline__ int tape_push(int a, double da, int b, double db) {
    Tape& t = s_tape[threadIdx.x];
    int i = t.n;
    if (i >= t.cap) {
        t.overflow = 1;
        i = t.cap - 1;
    } else {
        t.n = i + 1;
    }
    t.ab[i] = make_int2(a, b);
    t.d[i] = make_double2(da, db);
    return i;
}

__device__ __forceinline__ AVar a_leaf(double x) { return AVar(x, tape_push(-1, 0.0, -1, 0.0)); }
__device__ __forceinline__ AVar a_op1(double v, const AVar& a, double da) {
    return a.id < 0 ? AVar(v) : AVar(v, tape_push(a.id, da, -1, 0.0));
}
__device__ __forceinline__ AVar a_op2(double v, const AVar& a, double da, const AVar& b, double db) {
    if (a.id < 0 && b.id < 0) return AVar(v);
    return AVar(v, tape_push(a.id, da, b.id, db));
}

__device__ __forceinline__ AVar operator+(const AVar& a, const AVar& b) { return a_op2(a.v + b.v, a, 1.0, b, 1.0); }
__device__ __forceinline__ AVar operator-(const AVar& a, const AVar& b) { return a_op2(a.v - b.v, a, 1.0, b, -1.0); }
__device__ __forceinline__ AVar operator*(const AVar& a, const AVar& b) { return a_op2(a.v * b.v, a, b.v, b, a.v); }
__device__ __forceinline__ AVar operator/(const AVar& a, const AVar& b) {
    const double q = a.v / b.v;
    return a_op2(q, a, 1.0 / b.v, b, -q / b.v);
}
__device__ __forceinline__ AVar operator-(const AVar& a) { return a_op1(-a.v, a, -1.0); }
__device__ __forceinline__ AVar operator+(const AVar& a, double b) { return a + AVar(b); }
__device__ __forceinline__ AVar operator-(const AVar& a, double b) { return a - AVar(b); }
__device__ __forceinline__ AVar operator*(const AVar& a, double b) { return a * AVar(b); }
__device__ __forceinline__ AVar operator/(const AVar& a, double b) { return a / AVar(b); }
__device__ __forceinline__ AVar operator+(double a, const AVar& b) { return AVar(a) + b; }
__device__ __forceinline__ AVar operator-(double a, const AVar& b) { return AVar(a) - b; }
__device__ __forceinline__ AVar operator*(double a, const AVar& b) { return AVar(a) * b; }
__device__ __forceinline__ AVar operator/(double a, const AVar& b) { return AVar(a) / b; }
__device__ __forceinline__ bool operator<(const AVar& a, const AVar& b) { return a.v < b.v; }
__device__ __forceinline__ bool operator>(const AVar& a, const AVar& b) { return a.v > b.v; }
__device__ __forceinline__ bool operator<=(const AVar& a, const AVar& b) { return a.v <= b.v; }
__device__ __forceinline__ bool operator>=(const AVar& a, const AVar& b) { return a.v >= b.v; }
__device__ __forceinline__ bool operator==(const AVar& a, const AVar& b) { return a.v == b.v; }
__device__ __forceinline__ bool operator!=(const AVar& a, const AVar& b) { return a.v != b.v; }
__device__ __forceinline__ AVar sqrt(const AVar& a) {
    const double r = ::sqrt(a.v);
    return a_op1(r, a, r > 0.0 ? 0.5 / r : 0.0);
}
__device__ __forceinline__ AVar sin(const AVar& a) { return a_op1(::sin(a.v), a, ::cos(a.v)); }
__device__ __forceinline__ AVar cos(const AVar& a) { return a_op1(::cos(a.v), a, -::sin(a.v)); }
__device__ __forceinline__ AVar asin(const AVar& a) {
    const double s = 1.0 - a.v * a.v;
    return a_op1(::asin(a.v), a, s > 0.0 ? 1.0 / ::sqrt(s) : 0.0);
}
__device__ __forceinline__ AVar fabs(const AVar& a) { return a_op1(::fabs(a.v), a, a.v < 0.0 ? -1.0 : 1.0); }
// the clipping's float roundings (clipping.cpp:13,27,30,36): the value rounds, the derivative is 1
__device__ __forceinline__ AVar g_f32(const AVar& a) { return a_op1((double)(float)a.v, a, 1.0); }
__device__ __forceinline__ double g_f32(double a) { return (double)(float)a; }

// the scalar pass calls the same names on doubles
__device__ __forceinline__ double sqrt(double a) { return ::sqrt(a); }
__device__ __forceinline__ double sin(double a) { return ::sin(a); }
__device__ __forceinline__ double cos(double a) { return ::cos(a); }
__device__ __forceinline__ double asin(double a) { return ::asin(a); }
__device__ __forceinline__ double fabs(double a) { return ::fabs(a); }

template <> struct Tiny<AVar> { static constexpr double v = 1e-50; };
__device__ __forceinline__ double val(double x) { return x; }
__device__ __forceinline__ double val(const AVar& x) { return x.v; }
template <typename S> __device__ __forceinline__ V3<double> vval(const V3<S>& a) { return v3<double>(val(a.x), val(a.y), val(a.z)); }

// ---------------------------------------------------------------------------------------------
// The substep on bodies held in registers (mirrors rp_solve.cuh's all-FP64 path term for term)
template <typename S>
struct GBody {
    V3<S> x, px;       // position, position at the substep start
    Qt<S> q, pq;       // orientation, orientation at the substep start
    V3<S> v, w;        // velocities
    V3<S> pv, pw;      // velocities before the velocity update (previous_linear/angular_velocity)
    S invm;
    M3<S> Iinv, I;     // local inverse inertia and inertia
    S mus, mud, rest;  // static and dynamic friction, restitution
    bool fixed, active;
};

template <typename S>
__device__ __forceinline__ void g_qadd(Qt<S>& q, Qt<S> d, double s) {
    q.x = q.x + s * d.x; q.y = q.y + s * d.y; q.z = q.z + s * d.z; q.w = q.w + s * d.w;
    q = qnormalize(q);
}

// predict (pbd.cpp:537-577) with the caller's force F and no torque
template <typename S>
__device__ __noinline__ void g_predict(GBody<S>& B, V3<S> F, double h) {
    B.px = B.x;
    B.pq = B.q;
    if (B.fixed || !B.active) return;
    const V3<S> T = v3<S>(S(0.0), S(0.0), S(0.0));
    B.v = vadd(B.v, vscale(S(h) * B.invm, F));
    B.x = vadd(B.x, vscale(S(h), B.v));
    const M3<S> Iinv = world_tensor(B.q, B.Iinv), I = world_tensor(B.q, B.I);
    B.w = vadd(B.w, vscale(S(h), mmulv(Iinv, vsub(T, vcross(B.w, mmulv(I, B.w))))));
    const Qt<S> qd = qmul(qt<S>(B.w.x, B.w.y, B.w.z, S(0.0)), B.q);
    B.q.x = B.q.x + h * 0.5 * qd.x; B.q.y = B.q.y + h * 0.5 * qd.y;
    B.q.z = B.q.z + h * 0.5 * qd.z; B.q.w = B.q.w + h * 0.5 * qd.w;
    B.q = qnormalize(B.q);
}

// velocity update (pbd.cpp:623-643)
template <typename S>
__device__ void g_velocity(GBody<S>& B, double h) {
    if (B.fixed || !B.active) return;
    B.pv = B.v;
    B.pw = B.w;
    const V3<S> dx = vsub(B.x, B.px);
    B.v = vscale(S(1.0 / h), dx);
    const Qt<S> dq = qmul(B.q, qinverse(B.pq));
    B.w = (val(dq.w) >= 0.0) ? vscale(S(2.0 / h), v3<S>(dq.x, dq.y, dq.z)) : vscale(S(-2.0 / h), v3<S>(dq.x, dq.y, dq.z));
}

template <typename S> struct GPcpd { V3<S> r1, r2; M3<S> I1, I2; };

template <typename S>
__device__ __forceinline__ GPcpd<S> g_pcpd(const GBody<S>& a, const GBody<S>& b, V3<S> r1, V3<S> r2) {
    GPcpd<S> p;
    p.r1 = qrotate(a.q, r1);
    p.r2 = qrotate(b.q, r2);
    p.I1 = world_tensor(a.q, a.Iinv);
    p.I2 = world_tensor(b.q, b.Iinv);
    return p;
}

template <typename S>
__device__ S g_pos_dlambda(const GBody<S>& a, const GBody<S>& b, const GPcpd<S>& p, double h, double compliance, S lambda, V3<S> dx) {
    const S c = vlen(dx);
    if (c <= Tiny<S>::v) return S(0.0);
    const V3<S> n = v3<S>(dx.x / c, dx.y / c, dx.z / c);
    const S w1 = a.invm + vdot(vcross(p.r1, n), mmulv(p.I1, vcross(p.r1, n)));
    const S w2 = b.invm + vdot(vcross(p.r2, n), mmulv(p.I2, vcross(p.r2, n)));
    const S til = S(compliance) / (S(h) * S(h));
    return (-c - til * lambda) / (w1 + w2 + til);
}

template <typename S>
__device__ void g_pos_apply(GBody<S>& a, GBody<S>& b, const GPcpd<S>& p, S dl, V3<S> dx) {
    const S c = vlen(dx);
    if (c <= Tiny<S>::v) return;
    const V3<S> n = v3<S>(dx.x / c, dx.y / c, dx.z / c);
    const V3<S> imp = vscale(dl, n);
    if (!a.fixed) a.x = vadd(a.x, vscale(a.invm, imp));
    if (!b.fixed) b.x = vadd(b.x, vscale(-b.invm, imp));
    const V3<S> a1 = mmulv(p.I1, vcross(p.r1, imp));
    const V3<S> a2 = mmulv(p.I2, vcross(p.r2, imp));
    const Qt<S> q1 = qmul(qt<S>(a1.x, a1.y, a1.z, S(0.0)), a.q);
    const Qt<S> q2 = qmul(qt<S>(a2.x, a2.y, a2.z, S(0.0)), b.q);
    if (!a.fixed) g_qadd(a.q, q1, 0.5);
    if (!b.fixed) g_qadd(b.q, q2, -0.5);
}

template <typename S> struct GAcpd { M3<S> I1, I2; };

template <typename S>
__device__ __forceinline__ GAcpd<S> g_acpd(const GBody<S>& a, const GBody<S>& b) {
    GAcpd<S> r;
    r.I1 = world_tensor(a.q, a.Iinv);
    r.I2 = world_tensor(b.q, b.Iinv);
    return r;
}

template <typename S>
__device__ S g_ang_dlambda(const GAcpd<S>& A, double h, double compliance, S lambda, V3<S> dq) {
    const S th = vlen(dq);
    if (th <= Tiny<S>::v) return S(0.0);
    const V3<S> n = v3<S>(dq.x / th, dq.y / th, dq.z / th);
    const S w1 = vdot(n, mmulv(A.I1, n));
    const S w2 = vdot(n, mmulv(A.I2, n));
    const S til = S(compliance) / (S(h) * S(h));
    return (-th - til * lambda) / (w1 + w2 + til);
}

template <typename S>
__device__ void g_ang_apply(GBody<S>& a, GBody<S>& b, const GAcpd<S>& A, S dl, V3<S> dq) {
    const S th = vlen(dq);
    if (th <= Tiny<S>::v) return;
    const V3<S> n = v3<S>(dq.x / th, dq.y / th, dq.z / th);
    const V3<S> imp = vscale(-dl, n);
    const V3<S> a1 = mmulv(A.I1, imp);
    const V3<S> a2 = mmulv(A.I2, imp);
    const Qt<S> q1 = qmul(qt<S>(a1.x, a1.y, a1.z, S(0.0)), a.q);
    const Qt<S> q2 = qmul(qt<S>(a2.x, a2.y, a2.z, S(0.0)), b.q);
    if (!a.fixed) g_qadd(a.q, q1, 0.5);
    if (!b.fixed) g_qadd(b.q, q2, -0.5);
}

template <typename S>
__device__ bool g_limit_angle(V3<S> n, V3<S> n1, V3<S> n2, double alpha, double beta, V3<S>& dq) {
    const S pi = S(3.14159265358979);
    S phi = asin(vdot(vcross(n1, n2), n));
    if (vdot(n1, n2) < S(0.0)) phi = pi - phi;
    if (phi > pi) phi = phi - S(2.0) * pi;
    if (phi < -pi) phi = phi + S(2.0) * pi;
    if (phi < S(alpha) || phi > S(beta)) {
        phi = (phi > S(beta)) ? S(beta) : ((phi < S(alpha)) ? S(alpha) : phi);
        V3<S> ax = n;
        if (vlen(ax) != S(0.0)) ax = vnorm(ax);
        const S s = sin(phi / S(2.0));
        const Qt<S> rot = qt<S>(ax.x * s, ax.y * s, ax.z * s, cos(phi / S(2.0)));
        n1 = qrotate(rot, n1);
        dq = vcross(n1, n2);
        return true;
    }
    return false;
}

template <typename S>
__device__ void g_angle_correction(GBody<S>& a, GBody<S>& b, V3<S> dq, double h, S& lam) {
    const GAcpd<S> A = g_acpd(a, b);
    const S d2 = g_ang_dlambda(A, h, 0.0, lam, dq);
    g_ang_apply(a, b, A, d2, dq);
    lam = lam + d2;
}

// one external constraint (pbd.cpp:81-379); lam: its 4 per-substep lambdas
template <typename S>
__device__ __noinline__ void g_ext_solve(GBody<S>& a, GBody<S>& b, const ExtConstraint& C, S* lam, double h) {
    const V3<S> r1 = v3<S>(S(C.r1[0]), S(C.r1[1]), S(C.r1[2])), r2 = v3<S>(S(C.r2[0]), S(C.r2[1]), S(C.r2[2]));
    auto anchor = [&](const GPcpd<S>& p) { return vsub(vadd(a.x, p.r1), vadd(b.x, p.r2)); };
    switch (C.type) {
    case CON_POSITIONAL: {
        const V3<S> dx = vsub(vsub(a.x, b.x), v3<S>(S(C.distance[0]), S(C.distance[1]), S(C.distance[2])));
        const GPcpd<S> p = g_pcpd(a, b, r1, r2);
        const S dl = g_pos_dlambda(a, b, p, h, C.compliance, lam[0], dx);
        g_pos_apply(a, b, p, dl, dx);
        lam[0] = lam[0] + dl;
    } break;
    case CON_MUTUAL_ORIENTATION: {
        const GAcpd<S> A = g_acpd(a, b);
        const Qt<S> aux = qmul(a.q, qinverse(b.q));
        const V3<S> dq = v3<S>(S(2.0) * aux.x, S(2.0) * aux.y, S(2.0) * aux.z);
        const S dl = g_ang_dlambda(A, h, C.compliance, lam[0], dq);
        g_ang_apply(a, b, A, dl, dq);
        lam[0] = lam[0] + dl;
    } break;
    case CON_HINGE: {
        const GAcpd<S> A = g_acpd(a, b);
        const V3<S> dq = vcross(qaxis(a.q, C.a1), qaxis(b.q, C.a2));
        S dl = g_ang_dlambda(A, h, C.compliance, lam[1], dq);
        g_ang_apply(a, b, A, dl, dq);
        lam[1] = lam[1] + dl;
        const GPcpd<S> p = g_pcpd(a, b, r1, r2);
        const V3<S> dx = anchor(p);
        dl = g_pos_dlambda(a, b, p, h, 0.0, lam[0], dx);
        g_pos_apply(a, b, p, dl, dx);
        lam[0] = lam[0] + dl;
        if (C.limited) {
            V3<S> dq2;
            if (g_limit_angle(qaxis(a.q, C.a1), qaxis(a.q, C.l1), qaxis(b.q, C.l2), C.lo, C.hi, dq2))
                g_angle_correction(a, b, dq2, h, lam[2]);
        }
    } break;
    case CON_SPHERICAL: {
        const GPcpd<S> p = g_pcpd(a, b, r1, r2);
        const V3<S> dx = anchor(p);
        const S dl = g_pos_dlambda(a, b, p, h, 0.0, lam[0], dx);
        g_pos_apply(a, b, p, dl, dx);
        lam[0] = lam[0] + dl;
        const double EPS64 = 1e-50;
        {
            const V3<S> n1 = qaxis(a.q, C.a1), n2 = qaxis(b.q, C.a2);
            V3<S> n = vcross(n1, n2);
            const S nl = vlen(n);
            if (val(nl) > EPS64) {
                n = v3<S>(n.x / nl, n.y / nl, n.z / nl);
                V3<S> dq2;
                if (g_limit_angle(n, n1, n2, C.lo, C.hi, dq2)) g_angle_correction(a, b, dq2, h, lam[1]);
            }
        }
        {
            const V3<S> a1 = qaxis(a.q, C.a1), b1 = qaxis(a.q, C.l1), a2 = qaxis(b.q, C.a2), b2 = qaxis(b.q, C.l2);
            V3<S> n = vadd(a1, a2);
            const S nl = vlen(n);
            if (val(nl) > EPS64) {
                n = v3<S>(n.x / nl, n.y / nl, n.z / nl);
                V3<S> n1 = vsub(b1, vscale(vdot(n, b1), n)), n2 = vsub(b2, vscale(vdot(n, b2), n));
                const S l1 = vlen(n1), l2 = vlen(n2);
                if (val(l1) > EPS64 && val(l2) > EPS64) {
                    n1 = v3<S>(n1.x / l1, n1.y / l1, n1.z / l1);
                    n2 = v3<S>(n2.x / l2, n2.y / l2, n2.z / l2);
                    V3<S> dq2;
                    if (g_limit_angle(n, n1, n2, C.lo2, C.hi2, dq2)) g_angle_correction(a, b, dq2, h, lam[2]);
                }
            }
        }
    } break;
    default: break;
    }
}

}  // namespace rp
