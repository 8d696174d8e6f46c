// All-FP64 build of the step kernels, compiled with -fmad=false: the reference's FP64 arithmetic.
#include "rp_kernels.cuh"

namespace rp {
size_t smem_bytes_f64() { return Launcher<double, true>::smem_bytes(); }
cudaError_t configure_f64() { return Launcher<double, true>::configure(); }
int grid_blocks_per_sm_f64() { return Launcher<double, true>::grid_blocks_per_sm(); }
cudaError_t step_f64(const WorldView<double>& W, const StepParams& P, bool grid, int blocks, cudaStream_t st) {
    return Launcher<double, true>::step(W, P, grid, blocks, st);
}
cudaError_t broad_f64(const WorldView<double>& W, int scene, int grid_blocks, cudaStream_t st) {
    return Launcher<double, true>::broad(W, scene, grid_blocks, st);
}
cudaError_t state_io_f64(const WorldView<double>& W, double* rec, const int32_t* slot_entity, int n, bool pack, cudaStream_t st) {
    return Launcher<double, true>::state_io(W, rec, slot_entity, n, pack, st);
}
cudaError_t contacts_f64(const WorldView<double>& W, int a, int b, double* out, int cap, int* count, cudaStream_t st) {
    return Launcher<double, true>::contacts(W, a, b, out, cap, count, st);
}

// One warp per hull collider; the exact build's transform (model matrix, point with its divide by w,
// normalised direction), so the result is what colliders_update computes on the host.
__global__ void __launch_bounds__(256) world_hulls_kernel(WorldHullsArgs a) {
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int ci = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); ci < a.ncolliders; ci += nw) {
        const Collider col = a.colliders[ci];
        if (col.type != COL_HULL) continue;
        const Shape sh = a.shapes[col.shape];
        const double4_32a p4 = a.pos[a.col_body[ci]], q4 = a.rot[a.col_body[ci]];
        const M4<double> M = model_matrix(qt<double>(q4.x, q4.y, q4.z, q4.w), v3<double>(p4.x, p4.y, p4.z));
        for (int i = lane; i < sh.nv; i += 32) {
            const double* v = a.shape_verts + 3 * (size_t)(sh.vert_off + i);
            const V3<double> o = m4_point(M, v3<double>(v[0], v[1], v[2]));
            double* d = a.vertices_out + 3 * (size_t)(col.tv_off + i);
            d[0] = o.x; d[1] = o.y; d[2] = o.z;
        }
        for (int i = lane; i < sh.nf; i += 32) {
            const double* n = a.face_normal + 3 * (size_t)(sh.face_off + i);
            const V3<double> o = vnorm(m4_dir(M, v3<double>(n[0], n[1], n[2])));
            double* d = a.normals_out + 3 * (size_t)(col.tn_off + i);
            d[0] = o.x; d[1] = o.y; d[2] = o.z;
        }
    }
}

cudaError_t world_hulls(const WorldHullsArgs& a, cudaStream_t st) {
    if (a.ncolliders <= 0) return cudaSuccess;
    const int blocks = (a.ncolliders * 32 + 255) / 256;
    world_hulls_kernel<<<blocks < 4096 ? blocks : 4096, 256, 0, st>>>(a);
    return cudaGetLastError();
}
}  // namespace rp
