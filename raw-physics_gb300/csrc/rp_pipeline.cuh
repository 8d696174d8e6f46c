// Phase-major form of the step: one kernel per phase over every scene of the batch.
//
// The persistent step kernels (rp_step.cuh) run a whole frame inside one launch, so every SM
// interleaves all phases' code — broad phase, schedule, GJK, EPA, clipping, solves — and the
// instruction working set (~0.8 MB) thrashes the instruction caches. Here each phase is its own
// small kernel, launched over the whole batch, and a frame is the fixed sequence
//
//   setup (per scene: broad phase, islands, schedule, work-list reservation)
//   per substep: predict, hull transform, GJK, EPA, contact manifold, position sweep(s),
//                velocity update, velocity sweep
//
// replayed from a CUDA graph. Every SM then runs one phase's code at a time, the narrowphase
// kernels run at the occupancy their register and shared-memory needs allow, and the work is
// spread over all SMs regardless of how it is split into scenes. Results are identical to the
// persistent kernels: the same device functions run in the same order per scene.
//
// Narrowphase hand-off, per broad-phase pair of the frame's work list (work_state), through two
// compacted lists rebuilt every substep:
//   k_cull      thread per pair: liveness and bounds test; GJK candidates -> gjk_list, pairs needing
//               the general path (compound bodies, sphere colliders) -> hit_list
//   k_gjk       warp per GJK candidate: GJK on the two staged hulls; a hit stores its simplex and
//               joins hit_list
//   k_epa       warp per hit: EPA from the stored simplex; stores the FP64 normal and the penetration
//   k_manifold  warp per hit_list entry: contact manifold (or the general path); writes contacts
#pragma once
#include "rp_step.cuh"
#include "rp_launch.h"

namespace rp {

constexpr int PIPE_BLOCK = 256;
constexpr int PIPE_WARPS = PIPE_BLOCK / 32;

// Shared memory of one warp in k_gjk: the two staged hulls and the cycle-detection state.
template <typename R>
struct GjkSmem {
    V3<R> va[STAGE_V];
    V3<R> vb[STAGE_V];
    R saved[16];
};

// Per-warp diagnostic totals, flushed with one atomic each when the warp finishes.
struct WarpTally {
    unsigned long long v[8];
    __device__ WarpTally() {
        for (int i = 0; i < 8; ++i) v[i] = 0;
    }
    __device__ void flush(unsigned long long* counters, const int* slots) {
        if (lane_id() != 0 || !counters) return;
        for (int i = 0; i < 8; ++i)
            if (slots[i] >= 0 && v[i]) atomicAdd(&counters[slots[i]], v[i]);
    }
};

// Views of a pair of single-hull bodies in the pair frame of pair_contacts (FP32 build: body a's
// origin; exact build: world coordinates), staging both hulls' vertices in shared memory. The FP32
// build reads the pair's FP32 offset (work_off, rounded from the FP64 poses by k_cull) and the FP32
// orientations of the predict phase (pose_f), which equal the casts of the FP64 values: no FP64
// arithmetic or conversion runs in the warp.
template <typename R, bool EXACT>
__device__ void single_views(const WorldView<R>& W, V3<R>* stage_a, V3<R>* stage_b, int a, int b, int k, ColView<R>& va,
                             ColView<R>& vb, PairFrame<R, EXACT>& fr) {
    fr.raw = false;
    V3<R> offa = v3<R>(0, 0, 0), offb;
    if constexpr (EXACT) {
        double4_32a pa = W.pos[a], pb = W.pos[b], qa4 = W.rot[a], qb4 = W.rot[b];
        offb = v3<R>(0, 0, 0);
        fr.x1 = v3<R>((R)pa.x, (R)pa.y, (R)pa.z);
        fr.x2 = v3<R>((R)pb.x, (R)pb.y, (R)pb.z);
        fr.q1inv = qinverse(qt<R>((R)qa4.x, (R)qa4.y, (R)qa4.z, (R)qa4.w));
        fr.q2inv = qinverse(qt<R>((R)qb4.x, (R)qb4.y, (R)qb4.z, (R)qb4.w));
    } else {
        const float4 o = W.work_off[k], qa = W.pose_f[2 * a + 1], qb = W.pose_f[2 * b + 1];
        offb = v3<R>(o.x, o.y, o.z);
        fr.x1 = offa;
        fr.x2 = offb;
        fr.q1inv = qinverse(qt<R>(qa.x, qa.y, qa.z, qa.w));
        fr.q2inv = qinverse(qt<R>(qb.x, qb.y, qb.z, qb.w));
    }
    va = make_view<R, EXACT>(W, W.col_start[a], EXACT ? fr.x1 : offa, offa, stage_a, a);
    vb = make_view<R, EXACT>(W, W.col_start[b], EXACT ? fr.x2 : offb, offb, stage_b, b);
}

// True when both bodies have exactly one collider, a hull whose vertices fit the staging area.
template <typename R>
__device__ __forceinline__ bool single_hulls(const WorldView<R>& W, int a, int b) {
    static_assert(STAGE_V == 64, "single_hull flags are built for hulls of at most 64 vertices");
    return W.single_hull[a] && W.single_hull[b];
}

// Copies the warp's contacts of global pair slot gp into the scene's contact buffer.
template <typename R>
__device__ void emit_contacts(const WorldView<R>& W, NarrowSmem<R>& sm, int s, int gp, unsigned long long& tally) {
    const int lane = (int)lane_id();
    const int cbase = W.scene_contact_cap[s];
    const int ccap = W.scene_contact_cap[s + 1] - cbase;
    int nc = sm.ncontacts, start = 0;
    if (lane == 0) {
        start = nc ? atomicAdd(&W.contact_count[s], nc) : 0;
        if (start + nc > ccap) {
            atomicOr(&W.status[s], (uint32_t)ST_CONTACT_OVERFLOW);
            nc = 0;
        }
        if (sm.status) {
            atomicOr(&W.status[s], (uint32_t)sm.status);
            const int2 pr = W.pairs[gp];
            note_degenerate(W, (uint32_t)sm.status, s, pr.x, pr.y);
        }
        tally += (unsigned long long)nc;
        W.pair_cstart[gp] = start;
        W.pair_ccount[gp] = nc;
        if (nc > 0) {
            // the pair's solver node (after the scene's external constraints) acts this substep
            const int node = W.scene_node_cap[s] + (W.scene_ext[s + 1] - W.scene_ext[s]) + (gp - W.scene_pair_cap[s]);
            atomicOr(&W.node_bits[node >> 5], 1u << (node & 31));
        }
    }
    start = __shfl_sync(0xffffffffu, start, 0);
    nc = __shfl_sync(0xffffffffu, nc, 0);
    for (int k = lane; k < nc; k += 32) {
        R* c = W.contacts + 12 * (size_t)(cbase + start + k);
        V3<R> r1 = sm.c_r1[k], r2 = sm.c_r2[k], n = sm.c_n[k];
        c[0] = r1.x; c[1] = r1.y; c[2] = r1.z; c[3] = 0;
        c[4] = r2.x; c[5] = r2.y; c[6] = r2.z; c[7] = 0;
        c[8] = n.x; c[9] = n.y; c[10] = n.z; c[11] = 0;
    }
    __syncwarp();
}

// ---------------------------------------------------------------------------------------------
// Frame setup: broad phase, islands, schedule, then the frame's narrowphase work list.
template <typename R, class G>
__device__ void setup_scene(const WorldView<R>& W, const G& g, int s, double dt, int* smem, int* base_smem) {
    broad_phase(W, g, s, smem);
    islands(W, g, s, dt);
    schedule(W, g, s, smem);
    const int np = min(W.pair_count[s], W.scene_pair_cap[s + 1] - W.scene_pair_cap[s]);
    if (threadIdx.x == 0 && g.block() == 0) *base_smem = np ? atomicAdd(&W.queue[0], np) : 0;
    if (g.nblocks() == 1) {
        __syncthreads();
        const int base = *base_smem;
        for (int p = g.rank(); p < np; p += g.size()) W.work_list[base + p] = W.scene_pair_cap[s] + p;
    } else {
        // one reservation per scene; block 0 publishes it through the scan scratch
        if (threadIdx.x == 0 && g.block() == 0) W.scan_tmp[0] = *base_smem;
        g.sync();
        const int base = W.scan_tmp[0];
        for (int p = g.rank(); p < np; p += g.size()) W.work_list[base + p] = W.scene_pair_cap[s] + p;
        g.sync();
    }
}

template <typename R>
__global__ void __launch_bounds__(BLOCK) k_setup_cta(WorldView<R> W, double dt) {
    if (frame_abandoned(W.status)) return;
    __shared__ int scan_smem[32];
    __shared__ int base_smem;
    CtaGroup g;
    for (int s = blockIdx.x; s < W.num_scenes; s += gridDim.x) {
        setup_scene(W, g, s, dt, scan_smem, &base_smem);
        __syncthreads();
    }
}

template <typename R>
__global__ void __launch_bounds__(BLOCK) k_setup_grid(WorldView<R> W, double dt) {
    __shared__ int scan_smem[32];
    __shared__ int base_smem;
    if (frame_abandoned(W.status)) return;
    GridGroup g;
    g.bar = W.barrier;
    g.status = W.status;
    g.limit_ns = W.wait_ns;
    setup_scene(W, g, 0, dt, scan_smem, &base_smem);
}

// ---------------------------------------------------------------------------------------------
// Per-substep body phases
template <typename R, bool EXACT>
__global__ void __launch_bounds__(PIPE_BLOCK) k_predict(WorldView<R> W, int nbodies, int next, double h) {
    if (frame_abandoned(W.status)) return;
    const int t = blockIdx.x * blockDim.x + threadIdx.x, n = gridDim.x * blockDim.x;
    for (int b = t; b < nbodies; b += n) {
        predict_body<R, EXACT>(W, b, h);
        if constexpr (EXACT) {
            const double4_32a p = W.pos[b], q = W.rot[b];
            W.pose_f[2 * b] = make_float4((float)p.x, (float)p.y, (float)p.z, 0.f);
            W.pose_f[2 * b + 1] = make_float4((float)q.x, (float)q.y, (float)q.z, (float)q.w);
        } else {
            stage_body(W, b);
        }
    }
    for (int e = t; e < next; e += n)
        for (int k = 0; k < 4; ++k) W.ext_lambda[4 * (size_t)e + k] = 0.0;
    for (int s = t; s < W.num_scenes; s += n) {
        W.contact_count[s] = 0;
        W.act_count[2 * s] = 0;
        W.act_count[2 * s + 1] = 0;
    }
    if (t == 0) { W.queue[2] = 0; W.queue[3] = 0; W.queue[4] += 1; W.queue[5] = 0; W.queue[7] = 0; }
}

// The hulls of the bodies k_cull listed for this substep (tlist: bodies of the pairs that go on to
// GJK or the general path; the narrowphase reads no other transformed hull), `group` threads per
// collider (a power of two up to 32; 4 by default: the typical hull has 8-64 vertices, so a whole
// warp per collider would leave most lanes idle).
template <typename R, bool EXACT>
__global__ void __launch_bounds__(PIPE_BLOCK) k_transform(WorldView<R> W, int group) {
    if (frame_abandoned(W.status)) return;
    const int sub = threadIdx.x % group;
    const int gi = (blockIdx.x * blockDim.x + threadIdx.x) / group;
    const int ng = (gridDim.x * blockDim.x) / group;
    const int n = W.queue[7];
    for (int i = gi; i < n; i += ng) {
        const int b = W.tlist[i];
        for (int ci = W.col_start[b]; ci < W.col_start[b + 1]; ++ci) {
            const Collider col = W.colliders[ci];
            if (col.type == COL_HULL) transform_collider<R, EXACT, !EXACT>(W, col, b, sub, group);
        }
    }
}

template <typename R, bool EXACT>
__global__ void __launch_bounds__(PIPE_BLOCK) k_velocity(WorldView<R> W, int nbodies, double h) {
    if (frame_abandoned(W.status)) return;
    const int t = blockIdx.x * blockDim.x + threadIdx.x, n = gridDim.x * blockDim.x;
    for (int b = t; b < nbodies; b += n) {
        if constexpr (!EXACT) fold_body(W, b);   // the position sweep's corrections into the FP64 pose
        velocity_body<R, EXACT>(W, b, h);
    }
}

// ---------------------------------------------------------------------------------------------
// Narrowphase kernels
// Appends `item` (valid where `take`) to list[*count ...] with one atomic per CTA: a block-wide
// scan of the flags, then thread 0 reserves the block's range. Every thread of the block calls it.
__device__ __forceinline__ void block_append(int32_t* list, int32_t* count, bool take, int item, int* smem, int* base_smem) {
    int total;
    const int incl = block_incl_scan(take ? 1 : 0, smem, total);
    if (threadIdx.x == 0) *base_smem = total ? atomicAdd(count, total) : 0;
    __syncthreads();
    if (take) list[*base_smem + incl - 1] = item;
    __syncthreads();
}

// Thread per work item: liveness (pbd.cpp:583-590 skips pairs of two fixed or sleeping bodies), the
// bounds test, and the split into the GJK list (pairs of two single hulls that may touch) and the
// general path (compound bodies, sphere colliders), which goes straight to the contact list.
template <typename R>
__global__ void __launch_bounds__(PIPE_BLOCK) k_cull(WorldView<R> W, int enabled) {
    if (frame_abandoned(W.status)) return;
    __shared__ int scan_smem[32];
    __shared__ int base_smem;
    if constexpr (!std::is_same<R, double>::value) {   // the joints' FP32 solve frames of this substep
        const int ne = W.scene_ext[W.num_scenes];
        for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += gridDim.x * blockDim.x) {
            const ExtConstraint& C = W.ext[e];
            const double4_32a pa = W.pos[C.e1], pb = W.pos[C.e2];
            W.ext_base[e] = make_float4((float)(pa.x - pb.x), (float)(pa.y - pb.y), (float)(pa.z - pb.z), 0.f);
        }
    }
    const int n = W.queue[0];
    unsigned long long apart = 0;
    for (int base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const int k = base + (int)threadIdx.x;
        int state = WS_NONE;
        bool gjk = false;
        int ta = -1, tb = -1;
        if (k < n) {
            const int gp = W.work_list[k];
            const int2 pr = W.pairs[gp];
            const int a = pr.x, b = pr.y;
            const bool live = !((W.fixed[a] || !W.active[a]) && (W.fixed[b] || !W.active[b]));
            if (live && enabled) {
                if (!single_hulls(W, a, b)) state = WS_GENERAL;
                else if (bounds_apart_f(W, a, b)) ++apart;
                else gjk = true;
            }
            if ((gjk || state == WS_GENERAL) && !std::is_same<R, double>::value) {
                // one FP64 difference per pair and substep: the pair frame's offset for the warp kernels
                // and the FP32 sweeps' solve frame of the pair
                const double4_32a pa = W.pos[a], pb = W.pos[b];
                if (gjk) W.work_off[k] = make_float4((float)(pb.x - pa.x), (float)(pb.y - pa.y), (float)(pb.z - pa.z), 0.f);
                W.pair_base[gp] = make_float4((float)(pa.x - pb.x), (float)(pa.y - pb.y), (float)(pa.z - pb.z), 0.f);
            }
            W.work_state[k] = state;
            if (state == WS_NONE && !gjk) { W.pair_ccount[gp] = 0; W.pair_cstart[gp] = 0; }
            if (gjk || state == WS_GENERAL) {   // both hulls are read this substep: list each body once
                const int stamp = W.queue[4];
                ta = atomicExch(&W.tstamp[a], stamp) != stamp ? a : -1;
                tb = atomicExch(&W.tstamp[b], stamp) != stamp ? b : -1;
            }
        }
        {   // warp-aggregated append of the newly listed bodies
            const int lane = threadIdx.x & 31;
            const int c = (ta >= 0) + (tb >= 0);
            int incl = c;
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += y;
            }
            const int total = __shfl_sync(0xffffffffu, incl, 31);
            int base = 0;
            if (lane == 31 && total) base = atomicAdd(&W.queue[7], total);
            base = __shfl_sync(0xffffffffu, base, 31) + incl - c;
            if (ta >= 0) W.tlist[base++] = ta;
            if (tb >= 0) W.tlist[base] = tb;
        }
        block_append(W.gjk_list, &W.queue[2], gjk, k, scan_smem, &base_smem);
        block_append(W.hit_list, &W.queue[3], state == WS_GENERAL, k, scan_smem, &base_smem);
    }
    for (int o = 16; o > 0; o >>= 1) apart += __shfl_xor_sync(0xffffffffu, apart, o);
    if ((threadIdx.x & 31) == 0 && apart && W.counters) atomicAdd(&W.counters[11], apart);
}

// Warp per GJK candidate: GJK on the two staged hulls. A hit keeps its simplex and joins the
// contact list; the list entries are gathered per warp and appended 32 at a time.
template <typename R, bool EXACT>
__global__ void __launch_bounds__(PIPE_BLOCK, 3) k_gjk(WorldView<R> W) {
    if (frame_abandoned(W.status)) return;
    extern __shared__ __align__(16) unsigned char dyn_smem[];
    GjkSmem<R>& sm = reinterpret_cast<GjkSmem<R>*>(dyn_smem)[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    const int n = W.queue[2];
    WarpTally t;   // GJK iterations, cap hits, cycles, support cycles, cycle exits, -, GJK runs
    int pending = 0, mine = 0;
    for (int j = gw; j < n; j += nw) {
        const int k = W.gjk_list[j];
        const int gp = W.work_list[k];
        const int2 pr = W.pairs[gp];
        const int a = pr.x, b = pr.y;
        ColView<R> va, vb;
        PairFrame<R, EXACT> fr;
        single_views<R, EXACT>(W, sm.va, sm.vb, a, b, k, va, vb, fr);
        Simplex<R> sx;
        int gi = 0;
        long long tsup = 0;
        bool cycled = false;
        const long long t0 = clock64();
        const bool hit = gjk_collides(va, vb, sx, gi, tsup, sm.saved, cycled);
        t.v[0] += gi;
        t.v[1] += gi >= 100;
        t.v[2] += clock64() - t0;
        t.v[3] += tsup;
        t.v[4] += cycled;
        t.v[6] += 1;
        if (hit) {
            R* out = W.work_simplex + 16 * (size_t)k;
            const R comp[12] = {sx.a.x, sx.a.y, sx.a.z, sx.b.x, sx.b.y, sx.b.z,
                                sx.c.x, sx.c.y, sx.c.z, sx.d.x, sx.d.y, sx.d.z};
#pragma unroll
            for (int i = 0; i < 12; ++i)
                if (lane == i) out[i] = comp[i];
            if (lane == pending) mine = k;
            if (++pending == 32) {
                int base = 0;
                if (lane == 0) base = atomicAdd(&W.queue[3], 32);
                base = __shfl_sync(0xffffffffu, base, 0);
                W.hit_list[base + lane] = mine;
                pending = 0;
            }
        }
        if (lane == 0) {
            W.work_state[k] = hit ? WS_HIT : WS_NONE;
            if (!hit) { W.pair_ccount[gp] = 0; W.pair_cstart[gp] = 0; }
        }
        __syncwarp();
    }
    if (pending) {
        int base = 0;
        if (lane == 0) base = atomicAdd(&W.queue[3], pending);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (lane < pending) W.hit_list[base + lane] = mine;
    }
    const int slots[8] = {0, 4, 12, 15, 16, -1, 10, -1};
    t.flush(W.counters, slots);
}

template <typename R, bool EXACT>
__global__ void __launch_bounds__(PIPE_BLOCK, EXACT ? 2 : 3) k_epa(WorldView<R> W) {
    if (frame_abandoned(W.status)) return;
    extern __shared__ __align__(16) unsigned char dyn_smem[];
    NarrowSmem<R>& sm = reinterpret_cast<NarrowSmem<R>*>(dyn_smem)[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    const int n = W.queue[3];
    WarpTally t;   // EPA iterations, EPA calls, EPA cycles, EPA cap hits
    for (int j = gw; j < n; j += nw) {
        const int k = W.hit_list[j];
        if (W.work_state[k] != WS_HIT) continue;
        {
            const int gp = W.work_list[k];
            const int2 pr = W.pairs[gp];
            const int a = pr.x, b = pr.y;
            if (lane == 0) { sm.status = 0; }
            const long long tv = clock64();
            ColView<R> va, vb;
            PairFrame<R, EXACT> fr;
            single_views<R, EXACT>(W, sm.va, sm.vb, a, b, k, va, vb, fr);
            const R* in = W.work_simplex + 16 * (size_t)k;
            Simplex<R> sx;
            sx.a = v3<R>(in[0], in[1], in[2]);
            sx.b = v3<R>(in[3], in[4], in[5]);
            sx.c = v3<R>(in[6], in[7], in[8]);
            sx.d = v3<R>(in[9], in[10], in[11]);
            sx.num = 4;
            V3<double> nrm;
            double pen = 0.0;
            int ei = 0;
            const long long t0 = clock64();
            long long tsup = 0;
            bool deferred = false;
            bool ok;
            if constexpr (EXACT || !kEpaFast) ok = epa(sm, va, vb, sx, nrm, pen, ei);
            else ok = epa_fast(sm, va, vb, sx, nrm, pen, ei, &tsup, W.work_face + 12 * (size_t)k, &deferred);
            t.v[0] += ei;
            t.v[1] += 1;
            t.v[2] += clock64() - t0;
            t.v[3] += ei >= 100;
            t.v[4] += t0 - tv;
            t.v[5] += tsup;
            const int s = W.body_scene[a];
            if (!EXACT && (sm.status & (ST_DEG_EPA_NORMAL | ST_DEG_EPA_COPLANAR))) {
                // FP32 resolved this polytope to a degenerate one: the pair is redone in FP64 (k_fallback),
                // which decides it as the reference would
                if (lane == 0) {
                    W.work_state[k] = WS_FALLBACK;
                    W.fallback_list[atomicAdd(&W.queue[5], 1)] = k;
                }
                __syncwarp();
                continue;
            }
            if (lane == 0) {
                if (!ok) atomicOr(&W.status[s], (uint32_t)ST_EPA_NOT_CONVERGED);
                if (sm.status) {
                    atomicOr(&W.status[s], (uint32_t)sm.status);
                    note_degenerate(W, (uint32_t)sm.status, s, a, b);
                }
                if (ok && deferred) {
                    W.work_state[k] = WS_EPA_FACE;
                } else if (ok) {
                    double* o = W.work_epa + 4 * (size_t)k;
                    o[0] = nrm.x; o[1] = nrm.y; o[2] = nrm.z; o[3] = pen;
                    if (!EXACT) {
                        float* fo = W.work_face + 12 * (size_t)k;
                        fo[0] = (float)nrm.x; fo[1] = (float)nrm.y; fo[2] = (float)nrm.z; fo[3] = (float)pen;
                    }
                    W.work_state[k] = WS_EPA_OK;
                } else {
                    W.work_state[k] = WS_NONE;
                    W.pair_ccount[gp] = 0;
                    W.pair_cstart[gp] = 0;
                }
            }
            __syncwarp();
        }
    }
    const int slots[8] = {1, 2, 13, 7, 17, 18, -1, -1};
    t.flush(W.counters, slots);
}

// Thread per hit: the FP64 normal and depth of every EPA whose termination FP32 decided (WS_EPA_FACE),
// 32 pairs per warp instruction instead of one pair's arithmetic repeated by all 32 lanes; the FP32
// copies the manifold kernel works with are stored beside them.
template <typename R>
__global__ void __launch_bounds__(PIPE_BLOCK) k_epa_finish(WorldView<R> W) {
    if (frame_abandoned(W.status)) return;
    const int n = W.queue[3];
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const int k = W.hit_list[j];
        if (W.work_state[k] != WS_EPA_FACE) continue;
        float* f = W.work_face + 12 * (size_t)k;
        V3<double> n64;
        double d64;
        epa_face_finish(f, n64, d64);
        double* o = W.work_epa + 4 * (size_t)k;
        o[0] = n64.x; o[1] = n64.y; o[2] = n64.z; o[3] = d64;
        f[0] = (float)n64.x; f[1] = (float)n64.y; f[2] = (float)n64.z; f[3] = (float)d64;
        W.work_state[k] = WS_EPA_OK;
    }
}

// GENERAL: the pairs of the general path (compound bodies, sphere colliders: the whole
// colliders_get_contacts per pair); otherwise the contact manifolds of the EPA hits. Two instantiations
// keep the common kernel's code and registers free of the general path.
template <typename R, bool EXACT, bool GENERAL>
__global__ void __launch_bounds__(PIPE_BLOCK, (GENERAL || EXACT) ? 2 : 3) k_manifold(WorldView<R> W) {
    if (frame_abandoned(W.status)) return;
    extern __shared__ __align__(16) unsigned char dyn_smem[];
    NarrowSmem<R>& sm = reinterpret_cast<NarrowSmem<R>*>(dyn_smem)[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    const int n = W.queue[3];
    WarpTally t;   // contacts, manifold cycles
    for (int j = gw; j < n; j += nw) {
        const int k = W.hit_list[j];
        const int st = W.work_state[k];
        if (st != (GENERAL ? WS_GENERAL : WS_EPA_OK)) continue;
        {
            const int gp = W.work_list[k];
            const int2 pr = W.pairs[gp];
            const int a = pr.x, b = pr.y;
            const int s = W.body_scene[a];
            const long long t0 = clock64();
            long long t1 = t0;
            if constexpr (GENERAL) {
                pair_contacts<R, EXACT>(W, sm, a, b, false);
            } else {
                if (lane == 0) { sm.ncontacts = 0; sm.status = 0; }
                __syncwarp();
                ColView<R> va, vb;
                PairFrame<R, EXACT> fr;
                single_views<R, EXACT>(W, sm.va, sm.vb, a, b, k, va, vb, fr);
                const double* e = W.work_epa + 4 * (size_t)k;
                const V3<double> n64 = v3<double>(e[0], e[1], e[2]);
                t1 = clock64();
                if constexpr (EXACT) {
                    contact_manifold<R, EXACT>(sm, W, va, vb, v3cast<R>(n64), n64, (R)e[3], fr);
                } else {
                    // the FP32 normal and depth stored beside the FP64 ones (no conversion in the warp)
                    const float* f = W.work_face + 12 * (size_t)k;
                    contact_manifold<R, EXACT>(sm, W, va, vb, v3<R>(f[0], f[1], f[2]), n64, (R)f[3], fr);
                }
            }
            const long long t2 = clock64();
            t.v[1] += t2 - t0;
            t.v[2] += t1 - t0;
            if (!EXACT && !GENERAL && (sm.status & ST_DEG_SKEW)) {
                if (lane == 0) {
                    W.work_state[k] = WS_FALLBACK;
                    W.fallback_list[atomicAdd(&W.queue[5], 1)] = k;
                }
                __syncwarp();
                continue;
            }
            emit_contacts(W, sm, s, gp, t.v[0]);
            t.v[3] += clock64() - t2;
        }
    }
    const int slots[8] = {3, 14, 19, 20, -1, -1, -1, -1};
    t.flush(W.counters, slots);
}

// ---------------------------------------------------------------------------------------------
// FP64 redo of the FP32 build's degenerate pairs. Where FP32 rounding makes EPA's polytope degenerate
// (its points coplanar, a face normal that vanishes: typically two boxes resting face to face, as the
// links of a joint chain do) or the edge-edge contact's lines parallel, the reference, in FP64,
// usually is not: the pair's GJK, EPA and contact manifold run again in FP64 from the FP64 poses and
// hull geometry (the exact build's code), and its contacts replace the FP32 ones. One warp per pair.
constexpr int FALLBACK_MAXF = 128;   // face normals staged per hull

template <typename R>
__device__ WorldView<double> fp64_geometry(const WorldView<R>& W) {
    WorldView<double> G;
    memset(&G, 0, sizeof(G));
    G.colliders = W.colliders;
    G.shapes = W.shapes;
    G.shape_verts = W.shape_verts;
    G.face_normal = W.face_normal;
    G.face_elem_start = W.face_elem_start;
    G.face_elem = W.face_elem;
    G.csr_start = W.csr_start;
    G.csr_data = W.csr_data;
    G.pos = W.pos;
    G.rot = W.rot;
    return G;
}

template <typename R>
__global__ void __launch_bounds__(32) k_fallback(WorldView<R> W) {
    if (frame_abandoned(W.status)) return;
    extern __shared__ __align__(16) unsigned char dyn_smem[];
    NarrowSmem<double>& sm = *reinterpret_cast<NarrowSmem<double>*>(dyn_smem);
    V3<double>* norms = reinterpret_cast<V3<double>*>(dyn_smem + sizeof(NarrowSmem<double>));
    const int lane = threadIdx.x & 31;
    const int n = W.queue[5];
    const WorldView<double> G = fp64_geometry(W);
    for (int j = blockIdx.x; j < n; j += gridDim.x) {
        const int k = W.fallback_list[j];
        const int gp = W.work_list[k];
        const int2 pr = W.pairs[gp];
        const int s = W.body_scene[pr.x];
        ColView<double> v[2];
        const double4_32a pa = W.pos[pr.x], pb = W.pos[pr.y], qa = W.rot[pr.x], qb = W.rot[pr.y];
        for (int side = 0; side < 2; ++side) {
            const int body = side ? pr.y : pr.x;
            const Collider col = W.colliders[W.col_start[body]];
            const Shape* sh = W.shapes + col.shape;
            const double4_32a p4 = side ? pb : pa, q4 = side ? qb : qa;
            const M4<double> M = model_matrix(qt<double>(q4.x, q4.y, q4.z, q4.w), v3<double>(p4.x, p4.y, p4.z));
            V3<double>* tv = side ? sm.vb : sm.va;
            V3<double>* tn = norms + side * FALLBACK_MAXF;
            for (int i = lane; i < sh->nv; i += 32) {
                const double* x = W.shape_verts + 3 * (size_t)(sh->vert_off + i);
                tv[i] = m4_point(M, v3<double>(x[0], x[1], x[2]));
            }
            for (int i = lane; i < sh->nf; i += 32) {
                const double* x = W.face_normal + 3 * (size_t)(sh->face_off + i);
                tn[i] = vnorm(m4_dir(M, v3<double>(x[0], x[1], x[2])));
            }
            ColView<double>& c = v[side];
            c.type = COL_HULL;
            c.radius = 0.0;
            c.center = v3<double>(p4.x, p4.y, p4.z);
            c.off = v3<double>(0, 0, 0);
            c.verts = tv;
            c.staged = true;
            c.norms = tn;
            c.nv = sh->nv;
            c.nf = sh->nf;
            c.shape = sh;
            c.body = body;
        }
        PairFrame<double, true> fr;
        fr.raw = false;
        fr.x1 = v3<double>(pa.x, pa.y, pa.z);
        fr.x2 = v3<double>(pb.x, pb.y, pb.z);
        fr.q1inv = qinverse(qt<double>(qa.x, qa.y, qa.z, qa.w));
        fr.q2inv = qinverse(qt<double>(qb.x, qb.y, qb.z, qb.w));
        if (lane == 0) { sm.ncontacts = 0; sm.status = 0; }
        __syncwarp();
        collider_contacts<double, true>(sm, G, v[0], v[1], fr, nullptr);
        __syncwarp();
        // write the contacts as the FP32 build stores them (emit_contacts)
        const int cbase = W.scene_contact_cap[s];
        const int ccap = W.scene_contact_cap[s + 1] - cbase;
        int nc = sm.ncontacts, start = 0;
        if (lane == 0) {
            start = nc ? atomicAdd(&W.contact_count[s], nc) : 0;
            if (start + nc > ccap) {
                atomicOr(&W.status[s], (uint32_t)ST_CONTACT_OVERFLOW);
                nc = 0;
            }
            if (sm.status) {
                atomicOr(&W.status[s], (uint32_t)sm.status);
                note_degenerate(W, (uint32_t)sm.status, s, pr.x, pr.y);
            }
            W.pair_cstart[gp] = start;
            W.pair_ccount[gp] = nc;
            W.work_state[k] = nc ? WS_EPA_OK : WS_NONE;
            if (nc > 0) {
                const int node = W.scene_node_cap[s] + (W.scene_ext[s + 1] - W.scene_ext[s]) + (gp - W.scene_pair_cap[s]);
                atomicOr(&W.node_bits[node >> 5], 1u << (node & 31));
            }
            if (W.counters) {
                atomicAdd(&W.counters[3], (unsigned long long)nc);
                atomicAdd(&W.counters[23], 1ull);
            }
        }
        start = __shfl_sync(0xffffffffu, start, 0);
        nc = __shfl_sync(0xffffffffu, nc, 0);
        for (int c = lane; c < nc; c += 32) {
            R* o = W.contacts + 12 * (size_t)(cbase + start + c);
            const V3<double> r1 = sm.c_r1[c], r2 = sm.c_r2[c], nn = sm.c_n[c];
            o[0] = (R)r1.x; o[1] = (R)r1.y; o[2] = (R)r1.z; o[3] = 0;
            o[4] = (R)r2.x; o[5] = (R)r2.y; o[6] = (R)r2.z; o[7] = 0;
            o[8] = (R)nn.x; o[9] = (R)nn.y; o[10] = (R)nn.z; o[11] = 0;
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------------------------
// Gauss–Seidel sweeps: one CTA per scene, or the whole cooperative grid on one large scene.
template <typename R, bool EXACT, bool VELOCITY>
__global__ void __launch_bounds__(BLOCK) k_sweep_cta(WorldView<R> W, double h, int resched_first) {
    if (frame_abandoned(W.status)) return;
    CtaGroup g;
    for (int s = blockIdx.x; s < W.num_scenes; s += gridDim.x) {
        if (!VELOCITY && resched_first) resched(W, g, s);
        sweep_levels<R, EXACT, VELOCITY>(W, g, s, (R)h);
        __syncthreads();
    }
}

// One warp per scene: a scene's levels are mostly a few nodes wide, so a warp (barrier: __syncwarp)
// sweeps them as fast as a CTA would while many more scenes are in flight per SM. Warps take scenes
// from a counter (queue[1], zeroed before the launch) in decreasing-size order. The first position
// sweep of a substep builds the substep's schedules first (resched).
constexpr int SWEEP_WARP_BLOCK = 128;

// Both per-substep schedules of scene s by one warp, in one ordered pass (the result resched would
// give). The active nodes are gathered in constraint order (external constraints, then the pairs
// whose bit the contact write-out set), then lane 0 walks them once: in reference order a node's level
// is one more than the latest level on either of its bodies (the longest path, since a body's nodes
// are visited in order); in coloured order it takes the smallest colour neither body has used yet
// (first-fit, so a joint chain alternates two colours). One pass instead of one relaxation round per
// dependent step (a 64-link chain would take 64). Scenes beyond the shared tables take resched.
constexpr int SERIAL_MAX_BODIES = 512;
constexpr int SERIAL_MAX_WORDS = 256;   // node bitmap words staged per warp (8192 nodes)
constexpr int SERIAL_MAX_LEVELS = 256;  // levels (colours) counted in shared memory
struct SerialSmem {
    uint64_t mask[SERIAL_MAX_BODIES];   // per body: 1 + latest level, or the colours used (position sweep)
    uint64_t vmask[SERIAL_MAX_BODIES];  // (velocity sweep)
    uint32_t words[SERIAL_MAX_WORDS + 2];
    int cnt[2][SERIAL_MAX_LEVELS];      // nodes per level, then the fill cursors
    int n[2], L[2], overflow;
};

template <typename R>
__device__ bool resched_serial(const WorldView<R>& W, int s, SerialSmem& sm) {
    const int lane = threadIdx.x & 31;
    const int b0 = W.scene_body[s], nb = W.scene_body[s + 1] - b0;
    const int ne = W.scene_ext[s + 1] - W.scene_ext[s];
    const int nbase = W.scene_node_cap[s];
    const int nn = W.scene_nodes[s];
    const int w0 = (nbase + ne) >> 5, w1 = (nbase + nn + 31) >> 5;
    if (nb > SERIAL_MAX_BODIES || w1 - w0 > SERIAL_MAX_WORDS) return false;
    const int* nbody = W.node_body + 2 * nbase;
    const SchedView<R> v0 = sched_view(W, s, 0), v1 = sched_view(W, s, 1);
    const bool coloured = W.sweep_order == SWEEP_COLOURED;
    // clear the level tables the previous substep used, and the per-body tables
    const int used0 = min(*(volatile int*)v0.levels + 1, W.max_levels), used1 = min(*(volatile int*)v1.levels + 1, W.max_levels);
    for (int l = lane; l <= used0; l += 32) { v0.count[l] = 0; v0.fill[l] = 0; }
    for (int l = lane; l <= used1; l += 32) { v1.count[l] = 0; v1.fill[l] = 0; }
    for (int b = lane; b < nb; b += 32) { sm.mask[b] = 0ull; sm.vmask[b] = 0ull; }
    for (int w = lane; w < w1 - w0; w += 32) sm.words[w] = W.node_bits[w0 + w];
    for (int l = lane; l < SERIAL_MAX_LEVELS; l += 32) { sm.cnt[0][l] = 0; sm.cnt[1][l] = 0; }
    __syncwarp();
    if (lane == 0) {
        // per body: reference order keeps 1 + its latest level (0: none yet), coloured order the set
        // of colours its nodes use
        int n0 = 0, n1 = 0, extra = 0;
        auto place = [&](int k, bool pair) {
            const int a = nbody[2 * k], c = nbody[2 * k + 1];
            const int ia = a >= 0 ? a - b0 : -1, ic = c >= 0 ? c - b0 : -1;
            if (ia < 0 && ic < 0) return;                       // no dynamic body: a no-op node
            for (int which = 0; which < (pair ? 2 : 1); ++which) {
                uint64_t* m = which ? sm.vmask : sm.mask;
                const uint64_t ma = ia >= 0 ? m[ia] : 0ull, mc = ic >= 0 ? m[ic] : 0ull;
                int l;
                if (coloured) {
                    const uint64_t used = ma | mc;
                    if (~used) {
                        l = __ffsll((long long)~used) - 1;
                        if (ia >= 0) m[ia] = ma | (1ull << l);
                        if (ic >= 0) m[ic] = mc | (1ull << l);
                    } else {
                        l = 64 + extra++;                          // every small colour taken: a colour of its own
                    }
                } else {
                    l = (int)(ma > mc ? ma : mc);
                    if (ia >= 0) m[ia] = (uint64_t)l + 1ull;
                    if (ic >= 0) m[ic] = (uint64_t)l + 1ull;
                }
                const SchedView<R>& v = which ? v1 : v0;
                v.lev[k] = l;
                v.list[which ? n1++ : n0++] = k;
                if (l < SERIAL_MAX_LEVELS) {
                    sm.cnt[which][l]++;
                    sm.L[which] = max(sm.L[which], l + 1);
                } else {
                    sm.overflow = 1;
                }
            }
        };
        sm.L[0] = sm.L[1] = 0;
        sm.overflow = 0;
        for (int k = 0; k < ne; ++k) place(k, false);
        for (int w = 0; w < w1 - w0; ++w) {
            uint32_t bits = sm.words[w];
            const int base = ((w0 + w) << 5) - nbase;
            while (bits) {
                const int k = base + __ffs(bits) - 1;
                bits &= bits - 1u;
                if (k >= ne && k < nn) place(k, true);
            }
        }
        sm.n[0] = n0;
        sm.n[1] = n1;
        *v0.active = n0;
        *v1.active = n1;
        *v0.levels = 0;
        *v1.levels = 0;
    }
    __syncwarp();
    if (sm.overflow) return false;
    // bucket by level from the shared counts: prefix (the level table the sweep reads), then every
    // lane places list entries at its level's cursor (shared-memory atomics)
    for (int which = 0; which < 2; ++which) {
        const SchedView<R>& v = which ? v1 : v0;
        const int L = sm.L[which], n = sm.n[which];
        int carry = 0;
        for (int base = 0; base < L; base += 32) {
            const int l = base + lane;
            const int c = l < L ? sm.cnt[which][l] : 0;
            const int incl = warp_incl_scan(c);
            if (l < L) {
                v.count[l] = carry + incl - c;
                sm.cnt[which][l] = carry + incl - c;
            }
            carry += __shfl_sync(0xffffffffu, incl, 31);
        }
        if (lane == 0) {
            v.count[L] = carry;
            *v.levels = L;
            if (which == 0) atomicAdd(&W.counters[6], (unsigned long long)L);
        }
        __syncwarp();
        for (int i = lane; i < n; i += 32) {
            const int k = v.list[i];
            const int l = v.lev[k];
            v.nodes[atomicAdd(&sm.cnt[which][l], 1)] = k;
        }
        __syncwarp();
    }
    return true;
}

// The relaxation schedule by one warp, for scenes beyond resched_serial's shared tables (rare): out of
// line, so that the sweep's own path keeps its registers.
template <typename R>
__device__ __noinline__ void resched_warp_cold(const WorldView<R>& W, int s) {
    WarpGroup g;
    resched(W, g, s);
}

// CTA: the instantiation with the CTA phase (W.cta_scenes > 0); without it the kernel's code holds
// only the warp path.
template <typename R, bool EXACT, bool VELOCITY, bool CTA>
__global__ void __launch_bounds__(SWEEP_WARP_BLOCK, 4) k_sweep_warp(WorldView<R> W, double h, int resched_first) {
    if (frame_abandoned(W.status)) return;
    __shared__ SerialSmem ssm[VELOCITY ? 1 : SWEEP_WARP_BLOCK / 32];
    __shared__ int s_next, s_ok;
    // the W.cta_scenes largest scenes first, each swept by a whole CTA (queue[6] hands them out), so
    // the biggest scenes do not leave one warp finishing alone; then one warp per scene (queue[1])
    for (; CTA;) {
        if (threadIdx.x == 0) s_next = atomicAdd(&W.queue[6], 1);
        __syncthreads();
        const int i = s_next;
        __syncthreads();
        if (i >= W.cta_scenes) break;
        const int s = W.scene_order[i];
        CtaGroup cg;
        if (!VELOCITY && resched_first) {
            if (threadIdx.x < 32) {
                const bool ok = resched_serial(W, s, ssm[0]);
                if (threadIdx.x == 0) s_ok = ok ? 1 : 0;
            }
            __syncthreads();
            if (!s_ok) resched(W, cg, s);
            __syncthreads();
        }
        sweep_levels<R, EXACT, VELOCITY>(W, cg, s, (R)h);
        __syncthreads();
    }
    WarpGroup g;
    const int lane = threadIdx.x & 31;
    for (;;) {
        int i = 0;
        if (lane == 0) i = W.cta_scenes + atomicAdd(&W.queue[1], 1);
        i = __shfl_sync(0xffffffffu, i, 0);
        if (i >= W.num_scenes) break;
        const int s = W.scene_order[i];
        if (!VELOCITY && resched_first) {
            if (!resched_serial(W, s, ssm[(threadIdx.x >> 5) % (VELOCITY ? 1 : SWEEP_WARP_BLOCK / 32)])) resched_warp_cold(W, s);
        }
        sweep_levels<R, EXACT, VELOCITY>(W, g, s, (R)h);
        __syncwarp();
    }
}

template <typename R, bool EXACT, bool VELOCITY>
__global__ void __launch_bounds__(BLOCK) k_sweep_grid(WorldView<R> W, double h, int resched_first) {
    if (frame_abandoned(W.status)) return;
    GridGroup g;
    g.bar = W.barrier;
    g.status = W.status;
    g.limit_ns = W.wait_ns;
    if (!VELOCITY && resched_first) resched(W, g, 0);
    sweep_levels<R, EXACT, VELOCITY>(W, g, 0, (R)h);
}

}  // namespace rp

namespace rp {

// Host-side launch sequence of one frame of the phase-major form.
template <typename R, bool EXACT>
struct PipeLauncher {
    static size_t gjk_smem() { return sizeof(GjkSmem<R>) * PIPE_WARPS; }
    static size_t narrow_smem() { return sizeof(NarrowSmem<R>) * PIPE_WARPS; }
    static size_t fallback_smem() { return sizeof(NarrowSmem<double>) + 2 * FALLBACK_MAXF * sizeof(V3<double>); }

    static cudaError_t configure(PipeConfig& c, int sms) {
        cudaError_t e = cudaFuncSetAttribute(k_gjk<R, EXACT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gjk_smem());
        if (e == cudaSuccess) e = cudaFuncSetAttribute(k_epa<R, EXACT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)narrow_smem());
        if (e == cudaSuccess) e = cudaFuncSetAttribute(k_manifold<R, EXACT, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)narrow_smem());
        if (e == cudaSuccess) e = cudaFuncSetAttribute(k_manifold<R, EXACT, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)narrow_smem());
        if (e == cudaSuccess && !EXACT)
            e = cudaFuncSetAttribute(k_fallback<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fallback_smem());
        if (e != cudaSuccess) return e;
        int nb = 0;
        auto occ = [&](const void* f, int block, size_t smem) {
            int b = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, f, block, smem) != cudaSuccess) b = 1;
            return b < 1 ? 1 : b;
        };
        nb = occ((const void*)k_gjk<R, EXACT>, PIPE_BLOCK, gjk_smem());
        c.gjk_blocks = nb * sms;
        nb = occ((const void*)k_epa<R, EXACT>, PIPE_BLOCK, narrow_smem());
        c.epa_blocks = nb * sms;
        nb = occ((const void*)k_manifold<R, EXACT, false>, PIPE_BLOCK, narrow_smem());
        c.manifold_blocks = nb * sms;
        nb = occ((const void*)k_manifold<R, EXACT, true>, PIPE_BLOCK, narrow_smem());
        c.general_blocks = nb * sms;
        c.sweep_warp_blocks = occ((const void*)k_sweep_warp<R, EXACT, false, true>, SWEEP_WARP_BLOCK, 0) * sms;
        c.cull_blocks = occ((const void*)k_cull<R>, PIPE_BLOCK, 0) * sms;
        // cooperative kernels: one CTA per SM keeps the grid barrier's arrival count low
        (void)occ((const void*)k_setup_grid<R>, BLOCK, 0);
        c.setup_grid_blocks = sms;
        c.sweep_grid_blocks = sms;
        c.vsweep_grid_blocks = sms;
        c.sms = sms;
        return cudaSuccess;
    }

    template <typename... Args>
    static cudaError_t coop(void (*kernel)(Args...), int blocks, int block, cudaStream_t st, Args... args) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(blocks);
        cfg.blockDim = dim3(block);
        cfg.dynamicSmemBytes = 0;
        cfg.stream = st;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        return cudaLaunchKernelEx(&cfg, kernel, args...);
    }

    template <bool VELOCITY>
    static cudaError_t sweep_warp(const WorldView<R>& W, const PipeConfig& c, cudaStream_t st, double h, int first) {
        cudaError_t e = cudaMemsetAsync(W.queue + 1, 0, sizeof(int32_t), st);
        if (e == cudaSuccess) e = cudaMemsetAsync(W.queue + 6, 0, sizeof(int32_t), st);
        if (e != cudaSuccess) return e;
        if (W.cta_scenes > 0) k_sweep_warp<R, EXACT, VELOCITY, true><<<c.sweep_warp_blocks, SWEEP_WARP_BLOCK, 0, st>>>(W, h, first);
        else k_sweep_warp<R, EXACT, VELOCITY, false><<<c.sweep_warp_blocks, SWEEP_WARP_BLOCK, 0, st>>>(W, h, first);
        return cudaGetLastError();
    }

    static cudaError_t frame(const WorldView<R>& W, const StepParams& P, const PipeConfig& c, const PipeDims& d,
                             cudaStream_t st, PipeMarks* marks) {
        cudaError_t e = cudaMemsetAsync(W.queue, 0, sizeof(int32_t), st);
        if (e != cudaSuccess) return e;
        // the grid barrier's arrival counter starts every frame at zero (its cooperative kernels all
        // run c.sms CTAs)
        if (d.grid_mode && (e = cudaMemsetAsync(W.barrier, 0, sizeof(unsigned), st)) != cudaSuccess) return e;
        auto mark = [&](int phase) -> cudaError_t {
            if (!marks || marks->n >= marks->cap) return cudaSuccess;
            marks->phase[marks->n] = phase;
            return cudaEventRecord(marks->ev[marks->n++], st);
        };
        const double h = P.dt / P.num_substeps;
        const int body_blocks = (d.nbodies + d.next + PIPE_BLOCK - 1) / PIPE_BLOCK + 1;
        const int col_blocks = (d.ncolliders * c.transform_group + PIPE_BLOCK - 1) / PIPE_BLOCK + 1;
        if ((e = mark(-1)) != cudaSuccess) return e;
        if (d.grid_mode) e = coop(k_setup_grid<R>, c.setup_grid_blocks, BLOCK, st, W, P.dt);
        else k_setup_cta<R><<<d.num_scenes, BLOCK, 0, st>>>(W, P.dt), e = cudaGetLastError();
        if (e != cudaSuccess || (e = mark(PH_BROAD)) != cudaSuccess) return e;
        for (int sub = 0; sub < P.num_substeps; ++sub) {
            k_predict<R, EXACT><<<body_blocks, PIPE_BLOCK, 0, st>>>(W, d.nbodies, d.next, h);
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
            if ((e = cudaMemsetAsync(W.node_bits, 0, (size_t)d.node_words * 4, st)) != cudaSuccess) return e;
            if ((e = mark(PH_PREDICT)) != cudaSuccess) return e;
            k_cull<R><<<c.cull_blocks, PIPE_BLOCK, 0, st>>>(W, P.enable_collisions);
            if ((e = cudaGetLastError()) != cudaSuccess || (e = mark(PH_NARROW)) != cudaSuccess) return e;
            if (P.enable_collisions) {
                k_transform<R, EXACT><<<col_blocks, PIPE_BLOCK, 0, st>>>(W, c.transform_group);
                if ((e = cudaGetLastError()) != cudaSuccess || (e = mark(PH_TRANSFORM)) != cudaSuccess) return e;
                k_gjk<R, EXACT><<<c.gjk_blocks, PIPE_BLOCK, gjk_smem(), st>>>(W);
                if ((e = cudaGetLastError()) != cudaSuccess || (e = mark(PH_GJK)) != cudaSuccess) return e;
                k_epa<R, EXACT><<<c.epa_blocks, PIPE_BLOCK, narrow_smem(), st>>>(W);
                if ((e = cudaGetLastError()) != cudaSuccess) return e;
                if (!EXACT) {
                    k_epa_finish<R><<<c.cull_blocks, PIPE_BLOCK, 0, st>>>(W);
                    if ((e = cudaGetLastError()) != cudaSuccess) return e;
                }
                if ((e = mark(PH_EPA)) != cudaSuccess) return e;
                k_manifold<R, EXACT, false><<<c.manifold_blocks, PIPE_BLOCK, narrow_smem(), st>>>(W);
                if ((e = cudaGetLastError()) != cudaSuccess) return e;
                k_manifold<R, EXACT, true><<<c.general_blocks, PIPE_BLOCK, narrow_smem(), st>>>(W);
                if ((e = cudaGetLastError()) != cudaSuccess) return e;
                if (!EXACT) {
                    k_fallback<R><<<c.sms, 32, fallback_smem(), st>>>(W);
                    if ((e = cudaGetLastError()) != cudaSuccess) return e;
                }
                if ((e = mark(PH_MANIFOLD)) != cudaSuccess) return e;
            }
            for (int it = 0; it < P.num_pos_iters; ++it) {
                const int first = it == 0 ? 1 : 0;   // the substep's schedules are built by its first sweep
                if (d.grid_mode) e = coop(k_sweep_grid<R, EXACT, false>, c.sweep_grid_blocks, BLOCK, st, W, h, first);
                else if (c.sweep_cta) k_sweep_cta<R, EXACT, false><<<d.num_scenes, BLOCK, 0, st>>>(W, h, first), e = cudaGetLastError();
                else e = sweep_warp<false>(W, c, st, h, first);
                if (e != cudaSuccess) return e;
            }
            if ((e = mark(PH_SOLVE)) != cudaSuccess) return e;
            k_velocity<R, EXACT><<<body_blocks, PIPE_BLOCK, 0, st>>>(W, d.nbodies, h);
            if ((e = cudaGetLastError()) != cudaSuccess || (e = mark(PH_VELOCITY)) != cudaSuccess) return e;
            if (d.grid_mode) e = coop(k_sweep_grid<R, EXACT, true>, c.vsweep_grid_blocks, BLOCK, st, W, h, 0);
            else if (c.sweep_cta) k_sweep_cta<R, EXACT, true><<<d.num_scenes, BLOCK, 0, st>>>(W, h, 0), e = cudaGetLastError();
            else e = sweep_warp<true>(W, c, st, h, 0);
            if (e != cudaSuccess || (e = mark(PH_VSOLVE)) != cudaSuccess) return e;
        }
        return cudaSuccess;
    }

    static int launches_per_frame(const StepParams& P) {
        const int per_sub = 2 + (P.enable_collisions ? (EXACT ? 6 : 8) : 1) + P.num_pos_iters + 1;
        return 1 + P.num_substeps * per_sub;
    }
};

}  // namespace rp
