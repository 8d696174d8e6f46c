// Kernel entry points and host-side launchers of one precision build.
// rp_kernels_f32.cu and rp_kernels_f64.cu include this file with RP_EXACT 0 / 1; the FP64 build is
// compiled without FMA contraction so that it evaluates the reference's FP64 expressions exactly.
#pragma once
#include "rp_step.cuh"
#include "rp_launch.h"
#include <algorithm>

namespace rp {

// Broad phase of one scene (known-answer entry point rp_broad_pairs), with the group the step uses
// for it: one CTA for a scene of a batch, the cooperative grid (sort-based) for one large scene.
template <typename R>
__global__ void __launch_bounds__(BLOCK) broad_kernel(WorldView<R> W, int s) {
    __shared__ int scan_smem[32];
    CtaGroup g;
    broad_phase(W, g, s, scan_smem);
}

template <typename R>
__global__ void __launch_bounds__(BLOCK) broad_grid_kernel(WorldView<R> W) {
    __shared__ int scan_smem[32];
    if (frame_abandoned(W.status)) return;
    GridGroup g;
    g.bar = W.barrier;
    g.status = W.status;
    g.limit_ns = W.wait_ns;
    broad_phase(W, g, 0, scan_smem);
}

// Narrowphase of one body pair with one warp (known-answer entry point rp_contacts): transform the
// two bodies' hulls, then colliders_get_contacts; writes contact points in world coordinates.
template <typename R, bool EXACT>
__global__ void __launch_bounds__(32) contacts_kernel(WorldView<R> W, int a, int b, double* out, int cap, int* count) {
    extern __shared__ __align__(16) unsigned char dyn_smem[];
    NarrowSmem<R>& sm = *reinterpret_cast<NarrowSmem<R>*>(dyn_smem);
    const int lane = threadIdx.x;
    for (int side = 0; side < 2; ++side) {
        int body = side ? b : a;
        for (int ci = W.col_start[body]; ci < W.col_start[body + 1]; ++ci) {
            const Collider col = W.colliders[ci];
            if (col.type == COL_HULL) transform_collider<R, EXACT>(W, col, body, lane);
        }
    }
    __syncwarp();
    __threadfence_block();
    pair_contacts<R, EXACT>(W, sm, a, b, true);
    double4_32a pa = W.pos[a];
    int nc = sm.ncontacts;
    for (int k = lane; k < nc && k < cap; k += 32) {
        V3<R> p1 = sm.c_r1[k], p2 = sm.c_r2[k], n = sm.c_n[k];
        double ox = EXACT ? 0.0 : pa.x, oy = EXACT ? 0.0 : pa.y, oz = EXACT ? 0.0 : pa.z;
        double* o = out + 9 * k;
        o[0] = (double)p1.x + ox; o[1] = (double)p1.y + oy; o[2] = (double)p1.z + oz;
        o[3] = (double)p2.x + ox; o[4] = (double)p2.y + oy; o[5] = (double)p2.z + oz;
        o[6] = (double)n.x; o[7] = (double)n.y; o[8] = (double)n.z;
    }
    if (lane == 0) {
        *count = nc;
        if (sm.status) atomicOr(&W.status[0], (uint32_t)sm.status);
    }
}

// rp_state_set / rp_state_get on the device: the entity-ordered 28-double records (include/rp.h,
// RP_STATE_DOUBLES) to and from the body-slot SoA state, thread per body.
template <typename R>
__global__ void __launch_bounds__(256) state_unpack_kernel(WorldView<R> W, const double* rec, const int32_t* slot_entity, int n) {
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < n; b += gridDim.x * blockDim.x) {
        const double* o = rec + 28 * (size_t)slot_entity[b];
        W.pos[b] = make_double4_32a(o[0], o[1], o[2], 0.0);
        W.rot[b] = make_double4_32a(o[3], o[4], o[5], o[6]);
        W.prev_pos[b] = make_double4_32a(o[13], o[14], o[15], 0.0);
        W.prev_rot[b] = make_double4_32a(o[16], o[17], o[18], o[19]);
        for (int k = 0; k < 3; ++k) {
            W.vel[3 * b + k] = (R)o[7 + k];
            W.omega[3 * b + k] = (R)o[10 + k];
            W.prev_vel[3 * b + k] = (R)o[20 + k];
            W.prev_omega[3 * b + k] = (R)o[23 + k];
        }
        W.active[b] = o[26] != 0.0 ? 1 : 0;
        W.deact[b] = o[27];
    }
}

template <typename R>
__global__ void __launch_bounds__(256) state_pack_kernel(WorldView<R> W, double* rec, const int32_t* slot_entity, int n) {
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < n; b += gridDim.x * blockDim.x) {
        double* o = rec + 28 * (size_t)slot_entity[b];
        const double4_32a p = W.pos[b], q = W.rot[b], pp = W.prev_pos[b], pq = W.prev_rot[b];
        o[0] = p.x; o[1] = p.y; o[2] = p.z;
        o[3] = q.x; o[4] = q.y; o[5] = q.z; o[6] = q.w;
        for (int k = 0; k < 3; ++k) {
            o[7 + k] = (double)W.vel[3 * b + k];
            o[10 + k] = (double)W.omega[3 * b + k];
            o[20 + k] = (double)W.prev_vel[3 * b + k];
            o[23 + k] = (double)W.prev_omega[3 * b + k];
        }
        o[13] = pp.x; o[14] = pp.y; o[15] = pp.z;
        o[16] = pq.x; o[17] = pq.y; o[18] = pq.z; o[19] = pq.w;
        o[26] = W.active[b] ? 1.0 : 0.0;
        o[27] = W.deact[b];
    }
}

template <typename R, bool EXACT>
struct Launcher {
    static size_t smem_bytes() { return sizeof(NarrowSmem<R>) * WARPS_PER_BLOCK; }

    static cudaError_t configure() {
        cudaError_t e = cudaFuncSetAttribute(step_kernel_cta<R, EXACT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes());
        if (e != cudaSuccess) return e;
        e = cudaFuncSetAttribute(step_kernel_grid<R, EXACT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes());
        if (e != cudaSuccess) return e;
        return cudaFuncSetAttribute(contacts_kernel<R, EXACT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(NarrowSmem<R>));
    }

    static int grid_blocks_per_sm() {
        int nb = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, step_kernel_grid<R, EXACT>, BLOCK, smem_bytes()) != cudaSuccess) return 0;
        return nb;
    }

    static cudaError_t step(const WorldView<R>& W, const StepParams& P, bool grid, int blocks, cudaStream_t st) {
        if (grid) {
            cudaError_t e = cudaMemsetAsync(W.barrier, 0, sizeof(unsigned), st);   // grid barrier counter
            if (e != cudaSuccess) return e;
            void* args[] = {(void*)&W, (void*)&P};
            return cudaLaunchCooperativeKernel((const void*)step_kernel_grid<R, EXACT>, dim3(blocks), dim3(BLOCK), args,
                                               smem_bytes(), st);
        }
        step_kernel_cta<R, EXACT><<<blocks, BLOCK, smem_bytes(), st>>>(W, P);
        return cudaGetLastError();
    }

    static cudaError_t broad(const WorldView<R>& W, int s, int grid_blocks, cudaStream_t st) {
        if (grid_blocks > 0) {
            cudaError_t e = cudaMemsetAsync(W.barrier, 0, sizeof(unsigned), st);   // grid barrier counter
            if (e != cudaSuccess) return e;
            void* args[] = {(void*)&W};
            return cudaLaunchCooperativeKernel((const void*)broad_grid_kernel<R>, dim3(grid_blocks), dim3(BLOCK), args, 0, st);
        }
        broad_kernel<R><<<1, BLOCK, 0, st>>>(W, s);
        return cudaGetLastError();
    }

    static cudaError_t state_io(const WorldView<R>& W, double* rec, const int32_t* slot_entity, int n, bool pack,
                                cudaStream_t st) {
        if (n <= 0) return cudaSuccess;
        const int blocks = std::min((n + 255) / 256, 4096);
        if (pack) state_pack_kernel<R><<<blocks, 256, 0, st>>>(W, rec, slot_entity, n);
        else state_unpack_kernel<R><<<blocks, 256, 0, st>>>(W, rec, slot_entity, n);
        return cudaGetLastError();
    }

    static cudaError_t contacts(const WorldView<R>& W, int a, int b, double* out, int cap, int* count, cudaStream_t st) {
        contacts_kernel<R, EXACT><<<1, 32, sizeof(NarrowSmem<R>), st>>>(W, a, b, out, cap, count);
        return cudaGetLastError();
    }
};

}  // namespace rp
