// Adjoint kernel of the substep (rp_adjoint.cuh, rp_adjoint_contact.cuh) and its launcher.
// Built without FMA contraction: the scalar forward pass then reproduces the all-FP64 step.
#include "rp_adjoint_contact.cuh"

namespace rp {

// Body state at a substep boundary: x[3], q[4], v[3], w[3]
constexpr int ADJ_STATE = 13;
// Tape leaves per body: the 13 state values, the inverse mass, static and dynamic friction
constexpr int ADJ_LEAVES = 16;
// Checkpoint per body: the state, the deactivation time and the awake flag
constexpr int ADJ_CKPT = 15;

// The body's inertia tensors at its exact FP64 values, as functions of its inverse mass: the default
// inertia is a point-mass sum (colliders_get_default_inertia_tensor, collider.cpp:448-494), so
// I = m I_unit and I^-1 = invm I_unit^-1, with d I^-1 / d invm = I^-1 / invm, d I / d invm = -I / invm.
template <typename S>
__device__ void g_inertia(GBody<S>& B, const AdjointScene& sc, int i, double invm) {
    S si[6], sI[6];
    for (int k = 0; k < 6; ++k) {
        const double vi = sc.inv_inertia[6 * i + k], vI = sc.inertia[6 * i + k];
        if constexpr (sizeof(S) == sizeof(double)) {
            si[k] = vi;
            sI[k] = vI;
        } else {
            si[k] = a_op1(vi, B.invm, vi / invm);
            sI[k] = a_op1(vI, B.invm, -vI / invm);
        }
    }
    B.Iinv = msym(si);
    B.I = msym(sI);
}

template <typename S>
__device__ __forceinline__ S g_input(double x) {
    if constexpr (sizeof(S) == sizeof(double)) return x;
    else return a_leaf(x);
}

// The substep from `start` (nb bodies) with scalar type S, given the frame's broad-phase pairs and
// awake flags. With S = AVar every body's 16 inputs become tape leaves first, in body order (ids
// 16 i .. 16 i + 15): 13 state values, inverse mass, static and dynamic friction.
template <typename S>
__device__ void g_substep(GBody<S>* B, const double* start, const AdjointScene& sc, const AdjointParams& P, S* lam,
                          const int2* pairs, int np, const uint8_t* active, GScene<S>& X) {
    const int nb = sc.nb;
    for (int i = 0; i < nb; ++i) {
        const double* st = start + ADJ_STATE * i;
        S vals[ADJ_LEAVES];
        for (int k = 0; k < ADJ_STATE; ++k) vals[k] = g_input<S>(st[k]);
        vals[13] = g_input<S>(sc.invm[i]);
        vals[14] = g_input<S>(sc.material[3 * i]);
        vals[15] = g_input<S>(sc.material[3 * i + 1]);
        GBody<S>& b = B[i];
        b.x = v3<S>(vals[0], vals[1], vals[2]);
        b.q = qt<S>(vals[3], vals[4], vals[5], vals[6]);
        b.v = v3<S>(vals[7], vals[8], vals[9]);
        b.w = v3<S>(vals[10], vals[11], vals[12]);
        b.invm = vals[13];
        b.mus = vals[14];
        b.mud = vals[15];
        b.rest = S(sc.material[3 * i + 2]);
        const double* pv = sc.prev_vel + 6 * i;
        b.pv = v3<S>(S(pv[0]), S(pv[1]), S(pv[2]));
        b.pw = v3<S>(S(pv[3]), S(pv[4]), S(pv[5]));
        b.fixed = sc.fixed[i] != 0;
        b.active = active[i] != 0;
    }
    for (int i = 0; i < nb; ++i) {
        if (!B[i].fixed) {
            g_inertia(B[i], sc, i, sc.invm[i]);
        } else {
            // a fixed body's tensors are zero (entity_create_fixed): constants, as its inverse mass
            const S z[6] = {S(0.0), S(0.0), S(0.0), S(0.0), S(0.0), S(0.0)};
            B[i].Iinv = msym(z);
            B[i].I = msym(z);
        }
    }
    const double h = P.dt / P.substeps;
    for (int i = 0; i < nb; ++i) {
        // gravity as the caller's force -g m (stack.cpp:93-96), formed as the host forms it
        const S Fy = B[i].fixed ? S(0.0) : S(-P.gravity * 1.0) / B[i].invm;
        g_predict(B[i], v3<S>(S(0.0), Fy, S(0.0)), h);
    }
    X.ncon = 0;
    if (P.collisions) {
        // pairs whose bodies are both fixed or asleep are skipped (pbd.cpp:590-593); each body's hulls
        // are transformed once per substep, at its predicted pose
        const int stamp = ++*X.stamp;
        for (int k = 0; k < np; ++k) {
            const int a = pairs[k].x, c = pairs[k].y;
            if ((B[a].fixed || !B[a].active) && (B[c].fixed || !B[c].active)) continue;
            if (sc.stamp[a] != stamp) { g_transform(sc, P.geom, B[a], a, X); sc.stamp[a] = stamp; }
            if (sc.stamp[c] != stamp) { g_transform(sc, P.geom, B[c], c, X); sc.stamp[c] = stamp; }
            g_pair_contacts(sc, P.geom, X, B, a, c);
        }
    }
    for (int it = 0; it < P.pos_iters; ++it) {
        for (int e = 0; e < sc.ne; ++e) {
            if (it == 0)
                for (int k = 0; k < 4; ++k) lam[4 * e + k] = S(0.0);
            const ExtConstraint& C = sc.ext[e];
            g_ext_solve(B[C.e1 - sc.body0], B[C.e2 - sc.body0], C, lam + 4 * e, h);
        }
        for (int c = 0; c < X.ncon; ++c) g_collision_solve(B[X.con[c].a], B[X.con[c].b], X.con[c], h);
    }
    for (int i = 0; i < nb; ++i) g_velocity(B[i], h);
    for (int c = 0; c < X.ncon; ++c) g_contact_velocity(B[X.con[c].a], B[X.con[c].b], X.con[c], h);
}

__device__ void g_store(const GBody<double>* B, double* out, int nb) {
    for (int i = 0; i < nb; ++i) {
        double* o = out + ADJ_STATE * i;
        o[0] = B[i].x.x; o[1] = B[i].x.y; o[2] = B[i].x.z;
        o[3] = B[i].q.x; o[4] = B[i].q.y; o[5] = B[i].q.z; o[6] = B[i].q.w;
        o[7] = B[i].v.x; o[8] = B[i].v.y; o[9] = B[i].v.z;
        o[10] = B[i].w.x; o[11] = B[i].w.y; o[12] = B[i].w.z;
    }
}

template <typename S>
__device__ GScene<S> g_scene_view(const AdjointScene& sc, bool tape, int* counter) {
    GScene<S> X;
    X.tv = reinterpret_cast<V3<S>*>(tape ? sc.tv_a : sc.tv_d);
    X.tn = reinterpret_cast<V3<S>*>(tape ? sc.tn_a : sc.tn_d);
    X.tvv = reinterpret_cast<V3<double>*>(sc.tv_val);
    X.tnv = reinterpret_cast<V3<double>*>(sc.tn_val);
    X.con = reinterpret_cast<GCon<S>*>(tape ? sc.con_a : sc.con_d);
    X.ncon = 0;
    X.clip = reinterpret_cast<GClip<S>*>(tape ? sc.clip_a : sc.clip_d);
    X.epa = reinterpret_cast<GEpa*>(sc.epa);
    X.stamp = counter;
    return X;
}

// The frame's discrete state from the state at its start: pairs, then islands and sleeping
__device__ int g_frame_begin(const AdjointScene& sc, const AdjointParams& P, const double* st, int2* pairs) {
    const int np = g_broad(sc, P.geom, st, pairs);
    g_islands(sc, st, pairs, np, P.dt);
    return np;
}

// Reverse sweep of one substep's tape. The adjoints of entries at or above `leaves` live in a window
// of W values in shared memory that slides down the tape (an entry's parents are mostly a few hundred
// entries below it); parents below the window, the leaves among them, accumulate in the global array.
// Tape records are fetched eight at a time so that their loads overlap. Returns false on an entry
// whose parent does not precede it (a corrupt tape, reported and not followed).
__device__ bool g_reverse(Tape& t, int n, int leaves, double* win, int W) {
    bool ok = true;
    int hi = n, lo = max(leaves, n - W);
    for (int k = lo; k < hi; ++k) win[k - lo] = t.adj[k];
    int i = n - 1;
    while (i >= leaves) {
        if (i < lo) {
            hi = lo;
            lo = max(leaves, hi - W);
            for (int k = lo; k < hi; ++k) win[k - lo] = t.adj[k];
        }
        const int c0 = max(lo, i - 7);
        int2 ab[8];
        double2 dd[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int j = i - k;
            if (j >= c0) { ab[k] = t.ab[j]; dd[k] = t.d[j]; }
        }
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int j = i - k;
            if (j < c0) break;
            const double a = win[j - lo];
            if (a == 0.0) continue;
            const int2 p = ab[k];
            if (p.x >= j || p.y >= j) { ok = false; continue; }
            if (p.x >= 0) {
                if (p.x >= lo) win[p.x - lo] += a * dd[k].x;
                else t.adj[p.x] += a * dd[k].x;
            }
            if (p.y >= 0) {
                if (p.y >= lo) win[p.y - lo] += a * dd[k].y;
                else t.adj[p.y] += a * dd[k].y;
            }
        }
        i = c0 - 1;
    }
    return ok;
}

// One thread per scene: forward trajectory with checkpoints, the loss, then the backward sweep.
// Dynamic shared memory: a reverse-sweep window of `win` doubles per thread.
__global__ void __launch_bounds__(ADJ_BLOCK) k_adjoint(AdjointScene* scenes, int nscenes, AdjointParams P, int win) {
    extern __shared__ double s_win[];
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    Tape& tape = s_tape[threadIdx.x];
    if (s >= nscenes) return;
    long long prof[6] = {0, 0, 0, 0, 0, 0};
    long long t0 = clock64();
    const AdjointScene sc = scenes[s];
    tape.ab = sc.tape_ab;
    tape.d = sc.tape_d;
    tape.adj = sc.tape_adj;
    tape.cap = sc.tape_cap;
    tape.n = 0;
    tape.overflow = 0;
    sc.status[0] = 0;
    const int nb = sc.nb, S_ = P.substeps, K = P.checkpoint_every;
    const size_t stride = (size_t)ADJ_STATE * nb, cstride = (size_t)ADJ_CKPT * nb;
    GBody<double>* Bd = reinterpret_cast<GBody<double>*>(sc.bodies_d);
    GBody<AVar>* Ba = reinterpret_cast<GBody<AVar>*>(sc.bodies_a);
    double* lamd = sc.lam_d;
    AVar* lama = reinterpret_cast<AVar*>(sc.lam_a);
    int counter = 0;
    GScene<double> Xd = g_scene_view<double>(sc, false, &counter);
    GScene<AVar> Xa = g_scene_view<AVar>(sc, true, &counter);
    for (int i = 0; i < nb; ++i) sc.stamp[i] = -1;
    auto save = [&](double* ck, const double* st) {
        for (size_t k = 0; k < stride; ++k) ck[k] = st[k];
        for (int i = 0; i < nb; ++i) { ck[stride + i] = sc.deact[i]; ck[stride + nb + i] = sc.active[i]; }
    };
    auto restore = [&](const double* ck, double* st) {
        for (size_t k = 0; k < stride; ++k) st[k] = ck[k];
        for (int i = 0; i < nb; ++i) { sc.deact[i] = ck[stride + i]; sc.active[i] = ck[stride + nb + i] != 0.0 ? 1 : 0; }
    };
    // forward, checkpoint at every K-th frame start
    double* cur = sc.work;
    for (size_t k = 0; k < stride; ++k) cur[k] = sc.start[k];
    for (int i = 0; i < nb; ++i) { sc.deact[i] = sc.deact0[i]; sc.active[i] = sc.active0[i]; }
    for (int f = 0; f < P.frames; ++f) {
        if (f % K == 0) save(sc.checkpoints + (size_t)(f / K) * cstride, cur);
        const int np = g_frame_begin(sc, P, cur, sc.pairs);
        for (int u = 0; u < S_; ++u) {
            g_substep<double>(Bd, cur, sc, P, lamd, sc.pairs, np, sc.active, Xd);
            g_store(Bd, cur, nb);
        }
    }
    prof[0] = clock64() - t0;
    // loss |x_target_body - target|^2 and its seed
    const int lb = sc.loss_body;
    const double dx = cur[ADJ_STATE * lb + 0] - sc.target[0], dy = cur[ADJ_STATE * lb + 1] - sc.target[1],
                 dz = cur[ADJ_STATE * lb + 2] - sc.target[2];
    sc.loss[0] = dx * dx + dy * dy + dz * dz;
    double* g = sc.grad_state;  // adjoint of the current state
    for (size_t k = 0; k < stride; ++k) g[k] = 0.0;
    for (int i = 0; i < nb; ++i) { sc.grad_invm[i] = 0.0; sc.grad_mu[2 * i] = 0.0; sc.grad_mu[2 * i + 1] = 0.0; }
    g[ADJ_STATE * lb + 0] = 2.0 * dx;
    g[ADJ_STATE * lb + 1] = 2.0 * dy;
    g[ADJ_STATE * lb + 2] = 2.0 * dz;
    // backward, segment by segment
    bool bad = false;
    const int nseg = (P.frames + K - 1) / K;
    for (int seg = nseg - 1; seg >= 0; --seg) {
        const int f0 = seg * K, f1 = min(P.frames, f0 + K);
        const int nsub = (f1 - f0) * S_;
        // recompute the segment, keeping every substep's start state and every frame's pairs and awake flags
        t0 = clock64();
        restore(sc.checkpoints + (size_t)seg * cstride, sc.segment);
        for (int fl = 0; fl < f1 - f0; ++fl) {
            int2* fp = sc.pairs + (size_t)fl * sc.pair_cap;
            uint8_t* fa = sc.active_seg + (size_t)fl * nb;
            sc.npairs[fl] = g_frame_begin(sc, P, sc.segment + (size_t)fl * S_ * stride, fp);
            for (int i = 0; i < nb; ++i) fa[i] = sc.active[i];
            for (int u = 0; u < S_; ++u) {
                const int idx = fl * S_ + u;
                if (idx + 1 >= nsub) break;
                g_substep<double>(Bd, sc.segment + (size_t)idx * stride, sc, P, lamd, fp, sc.npairs[fl], fa, Xd);
                g_store(Bd, sc.segment + (size_t)(idx + 1) * stride, nb);
            }
        }
        prof[1] += clock64() - t0;
        for (int u = nsub - 1; u >= 0; --u) {
            const int fl = u / S_;
            t0 = clock64();
            tape.n = 0;
            g_substep<AVar>(Ba, sc.segment + (size_t)u * stride, sc, P, lama, sc.pairs + (size_t)fl * sc.pair_cap,
                            sc.npairs[fl], sc.active_seg + (size_t)fl * nb, Xa);
            const int n = tape.n;
            prof[4] = max(prof[4], (long long)n);
            prof[5] += n;
            const long long t1 = clock64();
            prof[2] += t1 - t0;
            for (int i = 0; i < n; ++i) tape.adj[i] = 0.0;
            // seed the outputs (a constant output has no path to the leaves)
            for (int i = 0; i < nb; ++i) {
                const AVar out[ADJ_STATE] = {Ba[i].x.x, Ba[i].x.y, Ba[i].x.z, Ba[i].q.x, Ba[i].q.y, Ba[i].q.z, Ba[i].q.w,
                                             Ba[i].v.x, Ba[i].v.y, Ba[i].v.z, Ba[i].w.x, Ba[i].w.y, Ba[i].w.z};
                for (int k = 0; k < ADJ_STATE; ++k) {
                    const int id = out[k].id;
                    if (id >= n) bad = true;
                    else if (id >= 0) tape.adj[id] += g[ADJ_STATE * i + k];
                }
            }
            if (!g_reverse(tape, n, min(n, ADJ_LEAVES * nb), s_win + (size_t)threadIdx.x * win, win)) bad = true;
            // leaves: 16 per body, in creation order
            for (int i = 0; i < nb; ++i) {
                const double* L = tape.adj + ADJ_LEAVES * i;
                for (int k = 0; k < ADJ_STATE; ++k) g[ADJ_STATE * i + k] = L[k];
                sc.grad_invm[i] += L[13];
                sc.grad_mu[2 * i] += L[14];
                sc.grad_mu[2 * i + 1] += L[15];
            }
            prof[3] += clock64() - t1;
        }
    }
    for (int k = 0; k < 6; ++k) sc.prof[k] = prof[k];
    sc.status[0] |= (tape.overflow ? ADJ_ST_TAPE : 0) | (bad ? ADJ_ST_BAD_TAPE : 0);
}

cudaError_t adjoint_launch(AdjointScene* d_scenes, int nscenes, const AdjointParams& P, cudaStream_t st) {
    // one serial thread per scene: spread the scenes over every SM rather than filling few
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int tpb = max(1, min(ADJ_BLOCK, (nscenes + sms - 1) / max(sms, 1)));
    const int blocks = (nscenes + tpb - 1) / tpb;
    // reverse-sweep windows: 200 KB of shared memory per block, split between its threads
    const int win = 25600 / tpb;
    const size_t smem = (size_t)win * tpb * sizeof(double);
    cudaError_t e = cudaFuncSetAttribute(k_adjoint, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_adjoint<<<blocks, tpb, smem, st>>>(d_scenes, nscenes, P, win);
    return cudaGetLastError();
}

size_t adjoint_body_bytes(bool tape) { return tape ? sizeof(GBody<AVar>) : sizeof(GBody<double>); }
size_t adjoint_var_bytes() { return sizeof(AVar); }
size_t adjoint_contact_bytes(bool tape) { return tape ? sizeof(GCon<AVar>) : sizeof(GCon<double>); }
size_t adjoint_clip_bytes(bool tape) { return tape ? sizeof(GClip<AVar>) : sizeof(GClip<double>); }
size_t adjoint_epa_bytes() { return sizeof(GEpa); }

}  // namespace rp
