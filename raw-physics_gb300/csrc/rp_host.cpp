// Host runtime of the GB300 rigid-body step and the C ABI of include/rp.h.
//
// The world keeps a host mirror of the reference's entity / collider / constraint data (set-up
// only), lays it out in HBM scene by scene (rp_world.h), and drives the persistent step kernel.
// After the first upload the device copy of the body state is authoritative: stepping never
// touches the host, and rp_state_get / rp_state_set are the only transfers.
#include "../../include/rp.h"
#include "rp_hull.h"
#include "rp_launch.h"
#include "rp_world.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <atomic>
#include <map>
#include <memory>
#include <thread>
#include <string>
#include <vector>

namespace rp {

static thread_local std::string g_last_error;
static rp_status fail(rp_status code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

// the same error reporting for the host units outside this file (rp_hull_io.cpp)
rp_status report_error(rp_status code, const char* msg) { return fail(code, msg); }

#define RP_CUDA(call)                                                                                        \
    do {                                                                                                     \
        cudaError_t e_ = (call);                                                                             \
        if (e_ != cudaSuccess) return fail(RP_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// Page-locked host staging: copies from and to it run at full link bandwidth, asynchronously
struct HostBuf {
    void* p = nullptr;
    size_t bytes = 0;
    HostBuf() = default;
    HostBuf(const HostBuf&) = delete;
    HostBuf& operator=(const HostBuf&) = delete;
    ~HostBuf() { release(); }
    void release() {
        if (p) cudaFreeHost(p);
        p = nullptr;
        bytes = 0;
    }
    cudaError_t ensure(size_t n) {
        if (n <= bytes && p) return cudaSuccess;
        release();
        size_t want = n ? n : 16;
        cudaError_t e = cudaHostAlloc(&p, want, cudaHostAllocDefault);
        if (e == cudaSuccess) bytes = want;
        return e;
    }
};

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    cudaError_t ensure(size_t n) {
        if (n <= bytes && p) return cudaSuccess;
        release();
        size_t want = n ? n : 16;
        cudaError_t e = cudaMalloc(&p, want);
        if (e == cudaSuccess) bytes = want;
        return e;
    }
    template <typename T> T* as() const { return (T*)p; }
};

struct Force { double pos[3], f[3]; };

struct HostBody {
    int scene = 0;
    double pos[3], rot[4], v[3] = {0, 0, 0}, w[3] = {0, 0, 0};
    double ppos[3] = {0, 0, 0}, prot[4] = {0, 0, 0, 1}, pv[3] = {0, 0, 0}, pw[3] = {0, 0, 0};
    double active = 1.0, deact = 0.0;
    double invm = 0.0, I[9], Iinv[9], radius = 0.0;
    int fixed = 0;
    double mus = 0, mud = 0, rest = 0;
    std::vector<rp_collider_desc> cols;
    std::vector<Force> forces;
    int slot = -1;   // index in the device layout (bodies grouped by scene)
};

struct HostExt {
    ExtConstraint c;   // e1/e2 hold entity indices here; slots are substituted at upload
    int scene;
};

}  // namespace rp

using namespace rp;

struct rp_world {
    int device = 0;
    int precision = RP_PRECISION_FP32;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int num_sms = 0;
    int grid_blocks = 0;

    std::vector<std::unique_ptr<Hull>> hulls;
    std::map<std::vector<double>, int> hull_index;   // content -> hull id (identical hulls are shared)
    int num_scenes = 1;
    std::vector<HostBody> bodies;
    std::vector<HostExt> exts;
    double gravity = 0.0;

    // upload state
    bool static_dirty = true;    // layout or constants changed: rebuild the device copy
    bool forces_dirty = true;
    bool device_state_valid = false;   // device holds the authoritative body state
    std::vector<int> slot_to_entity;

    // layout
    std::vector<int32_t> scene_body, scene_ext, scene_pair_cap, scene_contact_cap, scene_node_cap;
    int max_levels = 1024;
    bool grid_mode = false;
    double pair_mult = 1.0, contact_mult = 1.0;   // grown when a step overflows its scratch

    // device buffers
    DevBuf d_scene_body, d_scene_ext, d_scene_pair_cap, d_scene_contact_cap, d_scene_node_cap;
    DevBuf d_pos, d_rot, d_ppos, d_prot, d_vel, d_omega, d_pvel, d_pomega, d_active, d_deact;
    DevBuf d_backup;
    DevBuf d_invm, d_I, d_Iinv, d_mat, d_radius, d_bound, d_fixed, d_col_start, d_force, d_torque;
    DevBuf d_colliders, d_shapes, d_shape_verts, d_face_normal, d_shape_verts_f, d_face_normal_f, d_face_elem_start, d_face_elem, d_csr_start, d_csr_data;
    DevBuf d_tverts, d_tnorms, d_ext;
    DevBuf d_sort_key, d_sort_val, d_sort_hist, d_sort_hi;
    DevBuf d_pair_count, d_pairs, d_row_count, d_uf_parent, d_island_awake, d_node_body, d_node_pred, d_node_level;
    DevBuf d_tl_count, d_tl_start, d_tl, d_level_count, d_level_fill, d_scan_tmp, d_level_nodes, d_scene_levels,
        d_scene_nodes, d_pair_cstart, d_pair_ccount, d_contact_count, d_work, d_contacts, d_ext_lambda, d_status, d_barrier,
        d_counters, d_phase, d_kat_out, d_kat_count, d_deg;
    DevBuf d_hull_v, d_hull_n;   // rp_transformed_hulls output (device)
    HostBuf h_hull;              // and its pinned staging
    std::vector<int64_t> hull_v_off, hull_n_off;   // per entity: first vertex / normal in entity order
    int64_t hull_nv = 0, hull_nn = 0;              // totals (vertices, normals) over every hull collider
    DevBuf d_node_bits, d_sdx, d_sdq, d_pred_d, d_prev_qf;
    DevBuf d_node_vpred, d_node_vlevel, d_vlevel_count, d_vlevel_fill, d_vlevel_nodes, d_scene_vlevels, d_act_list, d_act_count;

    // phase-major pipeline
    DevBuf d_adj_scenes, d_adj_data, d_adj_ext;   // adjoint scratch
    HostBuf h_state;                               // pinned staging of the body state (rp_state_set / _get)
    HostBuf h_rec;                                 // pinned staging of the state records (device-side packing)
    DevBuf d_rec, d_slot_entity;                   // the records on the device; entity of each body slot
    cudaEvent_t ev_rec = nullptr;                  // the last record upload (h_rec is refilled after it)
    double adj_prof[6] = {0, 0, 0, 0, 0, 0};      // last adjoint's slowest scene (rp_adjoint_profile)
    DevBuf d_pose_f, d_body_scene, d_col_body, d_scene_order, d_gjk_list, d_hit_list, d_work_list, d_work_state, d_work_simplex, d_work_epa, d_queue, d_work_off, d_work_face, d_fallback, d_tstamp, d_tlist, d_single_hull, d_pair_base, d_ext_base;
    int mode = RP_MODE_AUTO;          // RP_MODE_*: how a frame is launched
    int solo_nodes = 512;             // tunable: grid sweeps run levels up to this size on one CTA
    int cta_from = 0;                 // tunable: batched sweeps give a whole CTA to scenes of this cost or more (0: none)
    std::vector<int64_t> order_cost;  // sweep cost of the scenes in scene_order (decreasing)
    int cta_scenes = 0;               // how many leading scenes of scene_order that is
    uint64_t wait_ns = 1000000000ull; // bound of every device-side wait (rp_world_set_wait_limit)
    int sweep_order = RP_SWEEP_REFERENCE;   // Gauss–Seidel order of the sweeps (rp_world_set_sweep_order)
    bool pipe_ready = false;
    PipeConfig pipe;
    PipeDims dims;
    uint64_t layout_gen = 0;          // bumped whenever device buffers are (re)allocated
    cudaGraphExec_t graph = nullptr;  // one captured frame of the pipeline
    uint64_t graph_gen = ~0ull;
    StepParams graph_params = {};
    std::vector<cudaEvent_t> marks;   // phase events of a timed frame
    std::vector<int> mark_phase;
    double phase_ms[PHASES] = {};

    uint64_t launches = 0;
    uint64_t h2d_bytes = 0, d2h_bytes = 0;
    uint64_t steps = 0, substeps = 0;
    uint32_t status_accum = 0;
    bool timing = false;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    double last_ms = 0.0;
    uint32_t last_launches = 0;

    size_t rsize() const { return precision == RP_PRECISION_FP64 ? 8 : 4; }
};

namespace {

rp_status check_world(rp_world* w) {
    if (!w) return fail(RP_ERR_INVALID, "null world");
    return RP_OK;
}

bool finite3(const double* v) { return std::isfinite(v[0]) && std::isfinite(v[1]) && std::isfinite(v[2]); }

std::vector<ColliderDesc> descs(rp_world* w, const std::vector<rp_collider_desc>& cols) {
    std::vector<ColliderDesc> d;
    for (const rp_collider_desc& c : cols)
        d.push_back({c.type, c.type == RP_COLLIDER_HULL ? w->hulls[(size_t)c.hull].get() : nullptr, c.radius});
    return d;
}

template <typename T>
cudaError_t upload(DevBuf& b, const std::vector<T>& v, cudaStream_t st) {
    cudaError_t e = b.ensure(v.size() * sizeof(T));
    if (e != cudaSuccess || v.empty()) return e;
    return cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st);
}

// convert FP64 host values to the build's working type
template <typename T>
std::vector<unsigned char> as_working(const std::vector<double>& v, size_t rsize) {
    std::vector<unsigned char> out(v.size() * rsize);
    for (size_t i = 0; i < v.size(); ++i) {
        if (rsize == 8) std::memcpy(&out[i * 8], &v[i], 8);
        else { float f = (float)v[i]; std::memcpy(&out[i * 4], &f, 4); }
    }
    return out;
}

rp_status sync_state_to_host(rp_world* w);

// Copies n doubles in parallel chunks (state records of a large batch are hundreds of MB: one core's
// memcpy would dominate a frame); with `check`, also returns false if any is not finite.
bool copy_records(double* dst, const double* src, size_t n, bool check) {
    const size_t chunk_min = (size_t)1 << 18;
    const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    const size_t chunks = std::max<size_t>(1, std::min<size_t>(hw, (n + chunk_min - 1) / chunk_min));
    std::atomic<bool> ok(true);
    auto work = [&](size_t c) {
        const size_t lo = n * c / chunks, hi = n * (c + 1) / chunks;
        bool good = true;
        if (check)
            for (size_t i = lo; i < hi; ++i) good = good && std::isfinite(src[i]);
        if (!good) ok = false;
        std::memcpy(dst + lo, src + lo, (hi - lo) * sizeof(double));
    };
    if (chunks == 1) {
        work(0);
    } else {
        std::vector<std::thread> th;
        for (size_t c = 1; c < chunks; ++c) th.emplace_back(work, c);
        work(0);
        for (std::thread& t : th) t.join();
    }
    return ok;
}

// Scenes whose sweep cost (bodies + 8 per joint) reaches cta_from get a whole CTA in the warp sweeps.
void set_cta_scenes(rp_world* w) {
    int n = 0;
    while (n < (int)w->order_cost.size() && w->cta_from > 0 && w->order_cost[(size_t)n] >= (int64_t)w->cta_from) ++n;
    w->cta_scenes = n;
}

// (Re)build the device layout: bodies grouped by scene, shapes, colliders, constraints, scratch.
rp_status build_device(rp_world* w) {
    if (w->device_state_valid) {
        rp_status s = sync_state_to_host(w);
        if (s != RP_OK) return s;
    }
    cudaStream_t st = w->stream;
    const int S = w->num_scenes;
    const size_t N = w->bodies.size();
    // slots: stable by scene
    w->scene_body.assign((size_t)S + 1, 0);
    for (const HostBody& b : w->bodies) w->scene_body[(size_t)b.scene + 1]++;
    for (int s = 0; s < S; ++s) w->scene_body[(size_t)s + 1] += w->scene_body[(size_t)s];
    std::vector<int> fill(w->scene_body.begin(), w->scene_body.end() - 1);
    w->slot_to_entity.assign(N, 0);
    for (size_t e = 0; e < N; ++e) {
        HostBody& b = w->bodies[e];
        b.slot = fill[(size_t)b.scene]++;
        w->slot_to_entity[(size_t)b.slot] = (int)e;
    }
    // external constraints grouped by scene
    w->scene_ext.assign((size_t)S + 1, 0);
    for (const HostExt& x : w->exts) w->scene_ext[(size_t)x.scene + 1]++;
    for (int s = 0; s < S; ++s) w->scene_ext[(size_t)s + 1] += w->scene_ext[(size_t)s];
    std::vector<ExtConstraint> ext(w->exts.size());
    {
        std::vector<int> ef(w->scene_ext.begin(), w->scene_ext.end() - 1);
        for (const HostExt& x : w->exts) {
            ExtConstraint c = x.c;
            c.e1 = w->bodies[(size_t)c.e1].slot;
            c.e2 = w->bodies[(size_t)c.e2].slot;
            for (int k = 0; k < 3; ++k) { c.r1f[k] = (float)c.r1[k]; c.r2f[k] = (float)c.r2[k]; }
            c.compliance_f = (float)c.compliance;
            ext[(size_t)ef[(size_t)x.scene]++] = c;
        }
    }
    // scratch capacities per scene
    w->scene_pair_cap.assign((size_t)S + 1, 0);
    w->scene_contact_cap.assign((size_t)S + 1, 0);
    w->scene_node_cap.assign((size_t)S + 1, 0);
    int max_bodies = 0;
    // RP_SCRATCH_SCALE (tests only) shrinks the initial scratch so the overflow-and-regrow path runs
    const char* scale_env = std::getenv("RP_SCRATCH_SCALE");
    const double scale = scale_env ? std::max(1e-6, std::atof(scale_env)) : 1.0;
    for (int s = 0; s < S; ++s) {
        long long n = w->scene_body[(size_t)s + 1] - w->scene_body[(size_t)s];
        max_bodies = std::max(max_bodies, (int)n);
        long long all = n * (n - 1) / 2;
        long long pc = std::min(all, std::max(1LL, (long long)(std::max(256.0, 16.0 * (double)n) * w->pair_mult * scale)));
        long long cc = std::max(1LL, (long long)(std::max(256.0, 2.0 * (double)pc) * w->contact_mult * scale));
        if (pc > (1LL << 30) || cc > (1LL << 30)) return fail(RP_ERR_CAPACITY, "scratch sizes beyond 2^30 entries");
        w->scene_pair_cap[(size_t)s + 1] = w->scene_pair_cap[(size_t)s] + (int32_t)pc;
        w->scene_contact_cap[(size_t)s + 1] = w->scene_contact_cap[(size_t)s] + (int32_t)cc;
        w->scene_node_cap[(size_t)s + 1] = w->scene_node_cap[(size_t)s] + (int32_t)pc +
                                           (w->scene_ext[(size_t)s + 1] - w->scene_ext[(size_t)s]);
    }
    w->grid_mode = (S == 1 && max_bodies >= 256);
    w->max_levels = w->grid_mode ? 8192 : 1024;
    // shapes: every hull id used by a collider, in hull-id order
    std::vector<Shape> shapes;
    std::vector<double> sverts, snorm;
    std::vector<int32_t> fstart, felem, cstart, cdata;
    std::vector<int> shape_of_hull(w->hulls.size(), -1);
    // topology tables once per distinct topology: scaled copies of one mesh share them, which keeps
    // the contact manifold's lookups in a few kilobytes
    std::map<std::vector<int32_t>, Shape> topo;
    for (size_t h = 0; h < w->hulls.size(); ++h) {
        const Hull& H = *w->hulls[h];
        Shape sh;
        sh.nv = H.nv();
        sh.nf = H.nf();
        sh.vert_off = (int32_t)(sverts.size() / 3);
        sh.face_off = (int32_t)(snorm.size() / 3);
        sverts.insert(sverts.end(), H.verts.begin(), H.verts.end());
        snorm.insert(snorm.end(), H.normals.begin(), H.normals.end());
        std::vector<int32_t> key{sh.nv};
        for (const auto* rows : {&H.faces, &H.v2f, &H.v2n, &H.f2n}) {
            key.push_back((int32_t)rows->size());
            for (const auto& r : *rows) {
                key.push_back((int32_t)r.size());
                key.insert(key.end(), r.begin(), r.end());
            }
        }
        auto it = topo.find(key);
        if (it == topo.end()) {
            Shape t;
            t.max_face_valence = 0;
            t.max_face_neighbours = 0;
            // face element CSR over one global face numbering (elem_off = the topology's first face);
            // a single sentinel after the last topology closes the final face
            t.elem_off = (int32_t)fstart.size();
            for (int f = 0; f < sh.nf; ++f) {
                fstart.push_back((int32_t)felem.size());
                felem.insert(felem.end(), H.faces[(size_t)f].begin(), H.faces[(size_t)f].end());
                t.max_face_valence = std::max(t.max_face_valence, (int32_t)H.faces[(size_t)f].size());
                t.max_face_neighbours = std::max(t.max_face_neighbours, (int32_t)H.f2n[(size_t)f].size());
            }
            auto add_csr = [&](const std::vector<std::vector<int>>& rows) {
                int32_t off = (int32_t)cstart.size();
                for (const auto& r : rows) {
                    cstart.push_back((int32_t)cdata.size());
                    cdata.insert(cdata.end(), r.begin(), r.end());
                }
                cstart.push_back((int32_t)cdata.size());
                return off;
            };
            t.v2f_off = add_csr(H.v2f);
            t.v2n_off = add_csr(H.v2n);
            t.f2n_off = add_csr(H.f2n);
            it = topo.emplace(std::move(key), t).first;
        }
        sh.elem_off = it->second.elem_off;
        sh.v2f_off = it->second.v2f_off;
        sh.v2n_off = it->second.v2n_off;
        sh.f2n_off = it->second.f2n_off;
        sh.max_face_valence = it->second.max_face_valence;
        sh.max_face_neighbours = it->second.max_face_neighbours;
        shape_of_hull[h] = (int)shapes.size();
        shapes.push_back(sh);
    }
    fstart.push_back((int32_t)felem.size());
    // colliders, transformed-geometry offsets
    std::vector<Collider> cols;
    std::vector<int32_t> col_start(N + 1, 0);
    int32_t tv = 0, tn = 0;
    for (size_t slot = 0; slot < N; ++slot) {
        const HostBody& b = w->bodies[(size_t)w->slot_to_entity[slot]];
        col_start[slot] = (int32_t)cols.size();
        for (const rp_collider_desc& d : b.cols) {
            Collider c;
            c.type = d.type;
            c.shape = d.type == RP_COLLIDER_HULL ? shape_of_hull[(size_t)d.hull] : -1;
            c.radius = d.radius;
            c.tv_off = tv;
            c.tn_off = tn;
            if (d.type == RP_COLLIDER_HULL) {
                tv += shapes[(size_t)c.shape].nv;
                tn += shapes[(size_t)c.shape].nf;
            }
            cols.push_back(c);
        }
    }
    col_start[N] = (int32_t)cols.size();
    // entity-order offsets of each entity's transformed geometry (rp_transformed_hulls)
    w->hull_v_off.assign(N + 1, 0);
    w->hull_n_off.assign(N + 1, 0);
    for (size_t e = 0; e < N; ++e) {
        int64_t nv = 0, nf = 0;
        for (const rp_collider_desc& d : w->bodies[e].cols)
            if (d.type == RP_COLLIDER_HULL) { nv += w->hulls[(size_t)d.hull]->nv(); nf += w->hulls[(size_t)d.hull]->nf(); }
        w->hull_v_off[e + 1] = w->hull_v_off[e] + nv;
        w->hull_n_off[e + 1] = w->hull_n_off[e] + nf;
    }
    w->hull_nv = tv;
    w->hull_nn = tn;
    // body constants
    std::vector<double> invm(N), I6(6 * N), Ii6(6 * N), mat(4 * N), rad(N);
    std::vector<uint8_t> fixedv(N);
    for (size_t slot = 0; slot < N; ++slot) {
        const HostBody& b = w->bodies[(size_t)w->slot_to_entity[slot]];
        invm[slot] = b.invm;
        const int sym[6] = {0, 4, 8, 1, 2, 5};
        for (int k = 0; k < 6; ++k) { I6[6 * slot + (size_t)k] = b.I[sym[k]]; Ii6[6 * slot + (size_t)k] = b.Iinv[sym[k]]; }
        mat[4 * slot] = b.mus;
        mat[4 * slot + 1] = b.mud;
        mat[4 * slot + 2] = b.rest;
        mat[4 * slot + 3] = 0.0;
        rad[slot] = b.radius;
        fixedv[slot] = (uint8_t)b.fixed;
    }
    // geometric bounds for the narrowphase's separation test: a box and a sphere about the body
    // origin enclosing every hull vertex, rounded outwards to float; bodies with sphere colliders
    // get no box and an infinite radius (never separated by this test)
    std::vector<float4> bound(2 * N);
    for (size_t slot = 0; slot < N; ++slot) {
        const HostBody& b = w->bodies[(size_t)w->slot_to_entity[slot]];
        double lo[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, hi[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX}, r2 = 0.0;
        bool hulls = !b.cols.empty();
        for (const rp_collider_desc& d : b.cols) {
            if (d.type != RP_COLLIDER_HULL) { hulls = false; break; }
            const Hull& H = *w->hulls[(size_t)d.hull];
            for (int i = 0; i < H.nv(); ++i) {
                const double* v = &H.verts[(size_t)(3 * i)];
                for (int k = 0; k < 3; ++k) { lo[k] = std::min(lo[k], v[k]); hi[k] = std::max(hi[k], v[k]); }
                r2 = std::max(r2, v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
            }
        }
        if (!hulls) {
            bound[2 * slot] = make_float4(0.f, 0.f, 0.f, INFINITY);
            bound[2 * slot + 1] = make_float4(0.f, 0.f, 0.f, 0.f);
            continue;
        }
        float c[3], hx[3];
        for (int k = 0; k < 3; ++k) {
            double cd = 0.5 * (lo[k] + hi[k]);
            c[k] = (float)cd;
            double half = 0.5 * (hi[k] - lo[k]) + std::fabs(cd - (double)c[k]);
            hx[k] = std::nextafter((float)(half * (1.0 + 1e-6)), INFINITY);
        }
        float r = std::nextafter((float)(std::sqrt(r2) * (1.0 + 1e-6)), INFINITY);
        bound[2 * slot] = make_float4(c[0], c[1], c[2], r);
        bound[2 * slot + 1] = make_float4(hx[0], hx[1], hx[2], 1.f);
    }
    const size_t R = w->rsize();
    RP_CUDA(upload(w->d_scene_body, w->scene_body, st));
    RP_CUDA(upload(w->d_scene_ext, w->scene_ext, st));
    RP_CUDA(upload(w->d_scene_pair_cap, w->scene_pair_cap, st));
    RP_CUDA(upload(w->d_scene_contact_cap, w->scene_contact_cap, st));
    RP_CUDA(upload(w->d_scene_node_cap, w->scene_node_cap, st));
    RP_CUDA(upload(w->d_invm, as_working<double>(invm, R), st));
    RP_CUDA(upload(w->d_I, as_working<double>(I6, R), st));
    RP_CUDA(upload(w->d_Iinv, as_working<double>(Ii6, R), st));
    RP_CUDA(upload(w->d_mat, as_working<double>(mat, R), st));
    RP_CUDA(upload(w->d_radius, rad, st));
    RP_CUDA(upload(w->d_bound, bound, st));
    RP_CUDA(upload(w->d_fixed, fixedv, st));
    RP_CUDA(upload(w->d_col_start, col_start, st));
    RP_CUDA(upload(w->d_colliders, cols, st));
    RP_CUDA(upload(w->d_shapes, shapes, st));
    RP_CUDA(upload(w->d_shape_verts, sverts, st));
    RP_CUDA(upload(w->d_face_normal, snorm, st));
    {
        std::vector<float> fv(sverts.begin(), sverts.end()), fn(snorm.begin(), snorm.end());
        RP_CUDA(upload(w->d_shape_verts_f, fv, st));
        RP_CUDA(upload(w->d_face_normal_f, fn, st));
    }
    RP_CUDA(upload(w->d_face_elem_start, fstart, st));
    RP_CUDA(upload(w->d_face_elem, felem, st));
    RP_CUDA(upload(w->d_csr_start, cstart, st));
    RP_CUDA(upload(w->d_csr_data, cdata, st));
    RP_CUDA(upload(w->d_ext, ext, st));
    RP_CUDA(w->d_tverts.ensure((size_t)std::max(tv, 1) * 3 * R));
    RP_CUDA(w->d_tnorms.ensure((size_t)std::max(tn, 1) * 3 * R));
    // mutable state
    RP_CUDA(w->d_pos.ensure(std::max<size_t>(N, 1) * 32));
    RP_CUDA(w->d_rot.ensure(std::max<size_t>(N, 1) * 32));
    RP_CUDA(w->d_ppos.ensure(std::max<size_t>(N, 1) * 32));
    RP_CUDA(w->d_prot.ensure(std::max<size_t>(N, 1) * 32));
    RP_CUDA(w->d_vel.ensure(std::max<size_t>(N, 1) * 3 * R));
    RP_CUDA(w->d_omega.ensure(std::max<size_t>(N, 1) * 3 * R));
    RP_CUDA(w->d_pvel.ensure(std::max<size_t>(N, 1) * 3 * R));
    RP_CUDA(w->d_pomega.ensure(std::max<size_t>(N, 1) * 3 * R));
    RP_CUDA(w->d_active.ensure(std::max<size_t>(N, 1)));
    RP_CUDA(w->d_deact.ensure(std::max<size_t>(N, 1) * 8));
    RP_CUDA(w->d_force.ensure(std::max<size_t>(N, 1) * 24));
    RP_CUDA(w->d_torque.ensure(std::max<size_t>(N, 1) * 24));
    // scratch
    const size_t P = (size_t)w->scene_pair_cap[(size_t)S], C = (size_t)w->scene_contact_cap[(size_t)S],
                 NN = (size_t)w->scene_node_cap[(size_t)S], E = w->exts.size();
    RP_CUDA(w->d_pair_count.ensure((size_t)S * 4));
    RP_CUDA(w->d_pairs.ensure(std::max<size_t>(P, 1) * 8));
    RP_CUDA(w->d_row_count.ensure(std::max<size_t>(N, 1) * 4));
    RP_CUDA(w->d_sort_key.ensure(std::max<size_t>(2 * N, 1) * 4));
    RP_CUDA(w->d_sort_val.ensure(std::max<size_t>(2 * N, 1) * 4));
    RP_CUDA(w->d_sort_hist.ensure(256 * ((std::max<size_t>(N, 1) + 255) / 256) * 4));
    RP_CUDA(w->d_sort_hi.ensure(std::max<size_t>(N, 1) * 4));
    RP_CUDA(w->d_uf_parent.ensure(std::max<size_t>(N, 1) * 4));
    RP_CUDA(w->d_island_awake.ensure(std::max<size_t>(N, 1)));
    RP_CUDA(w->d_node_body.ensure(std::max<size_t>(NN, 1) * 8));
    RP_CUDA(w->d_node_pred.ensure(std::max<size_t>(NN, 1) * 8));
    RP_CUDA(w->d_node_level.ensure(std::max<size_t>(NN, 1) * 4));
    RP_CUDA(w->d_tl_count.ensure(std::max<size_t>(N, 1) * 4));
    RP_CUDA(w->d_tl_start.ensure((N + 1) * 4));
    RP_CUDA(w->d_tl.ensure(std::max<size_t>(NN, 1) * 8));
    RP_CUDA(w->d_level_count.ensure((size_t)S * (size_t)(w->max_levels + 1) * 4));
    RP_CUDA(w->d_level_fill.ensure((size_t)S * (size_t)(w->max_levels + 1) * 4));
    RP_CUDA(w->d_scan_tmp.ensure(4096 * 4));
    RP_CUDA(w->d_level_nodes.ensure(std::max<size_t>(NN, 1) * 4));
    RP_CUDA(w->d_scene_levels.ensure((size_t)S * 4));
    RP_CUDA(w->d_node_vpred.ensure(std::max<size_t>(NN, 1) * 8));
    RP_CUDA(w->d_node_vlevel.ensure(std::max<size_t>(NN, 1) * 4));
    RP_CUDA(w->d_vlevel_count.ensure((size_t)S * (size_t)(w->max_levels + 1) * 4));
    RP_CUDA(w->d_vlevel_fill.ensure((size_t)S * (size_t)(w->max_levels + 1) * 4));
    RP_CUDA(w->d_vlevel_nodes.ensure(std::max<size_t>(NN, 1) * 4));
    RP_CUDA(w->d_scene_vlevels.ensure((size_t)S * 4));
    RP_CUDA(w->d_act_list.ensure(std::max<size_t>(2 * NN, 1) * 4));
    RP_CUDA(w->d_act_count.ensure((size_t)S * 8));
    RP_CUDA(w->d_node_bits.ensure((NN / 32 + 1) * 4));
    RP_CUDA(cudaMemsetAsync(w->d_node_bits.p, 0, (NN / 32 + 1) * 4, st));
    w->dims.node_words = (int)(NN / 32 + 1);
    RP_CUDA(w->d_scene_nodes.ensure((size_t)S * 4));
    RP_CUDA(w->d_pair_cstart.ensure(std::max<size_t>(P, 1) * 4));
    RP_CUDA(w->d_pair_ccount.ensure(std::max<size_t>(P, 1) * 4));
    RP_CUDA(w->d_contact_count.ensure((size_t)S * 4));
    RP_CUDA(w->d_work.ensure((size_t)S * 4));
    RP_CUDA(w->d_contacts.ensure(std::max<size_t>(C, 1) * 12 * R));
    RP_CUDA(w->d_ext_lambda.ensure(std::max<size_t>(E, 1) * 4 * 8));
    {   // phase-major pipeline: body -> scene, collider -> body, per-pair narrowphase hand-off
        std::vector<int32_t> body_scene(std::max<size_t>(N, 1), 0), col_body(std::max<size_t>(cols.size(), 1), 0);
        for (int sc = 0; sc < S; ++sc)
            for (int32_t b = w->scene_body[(size_t)sc]; b < w->scene_body[(size_t)sc + 1]; ++b) body_scene[(size_t)b] = sc;
        for (size_t slot = 0; slot < N; ++slot)
            for (int32_t c = col_start[slot]; c < col_start[slot + 1]; ++c) col_body[(size_t)c] = (int32_t)slot;
        RP_CUDA(upload(w->d_body_scene, body_scene, st));
        RP_CUDA(upload(w->d_slot_entity, w->slot_to_entity, st));
        RP_CUDA(upload(w->d_col_body, col_body, st));
        std::vector<uint8_t> single(std::max<size_t>(N, 1), 0);
        for (size_t slot = 0; slot < N; ++slot) {
            const int32_t c = col_start[slot];
            single[slot] = col_start[slot + 1] - c == 1 && cols[(size_t)c].type == COL_HULL &&
                           shapes[(size_t)cols[(size_t)c].shape].nv <= 64;
        }
        RP_CUDA(upload(w->d_single_hull, single, st));
        RP_CUDA(w->d_pose_f.ensure(std::max<size_t>(N, 1) * 32));
        for (DevBuf* b : {&w->d_sdx, &w->d_sdq, &w->d_pred_d, &w->d_prev_qf}) {
            RP_CUDA(b->ensure(std::max<size_t>(N, 1) * 16));
            RP_CUDA(cudaMemsetAsync(b->p, 0, std::max<size_t>(N, 1) * 16, st));
        }
        RP_CUDA(w->d_work_list.ensure(std::max<size_t>(P, 1) * 4));
        RP_CUDA(w->d_work_state.ensure(std::max<size_t>(P, 1) * 4));
        RP_CUDA(w->d_gjk_list.ensure(std::max<size_t>(P, 1) * 4));
        RP_CUDA(w->d_hit_list.ensure(std::max<size_t>(P, 1) * 4));
        RP_CUDA(w->d_work_simplex.ensure(std::max<size_t>(P, 1) * 16 * R));
        RP_CUDA(w->d_work_epa.ensure(std::max<size_t>(P, 1) * 4 * 8));
        RP_CUDA(w->d_work_off.ensure(std::max<size_t>(P, 1) * 16));
        RP_CUDA(w->d_pair_base.ensure(std::max<size_t>(P, 1) * 16));
        RP_CUDA(w->d_ext_base.ensure(std::max<size_t>(E, 1) * 16));
        RP_CUDA(w->d_fallback.ensure(std::max<size_t>(P, 1) * 4));
        RP_CUDA(w->d_work_face.ensure(std::max<size_t>(P, 1) * 12 * 4));
        std::vector<int32_t> order((size_t)S);
        for (int sc = 0; sc < S; ++sc) order[(size_t)sc] = sc;
        // largest estimated sweep cost first: bodies, plus joints weighted for their serial chains
        auto cost = [&](int32_t x) {
            return (long long)(w->scene_body[(size_t)x + 1] - w->scene_body[(size_t)x]) +
                   8LL * (w->scene_ext[(size_t)x + 1] - w->scene_ext[(size_t)x]);
        };
        std::stable_sort(order.begin(), order.end(), [&](int32_t x, int32_t y) { return cost(x) > cost(y); });
        RP_CUDA(upload(w->d_scene_order, order, st));
        w->order_cost.assign((size_t)S, 0);
        for (int sc = 0; sc < S; ++sc) w->order_cost[(size_t)sc] = cost(order[(size_t)sc]);
        set_cta_scenes(w);
        RP_CUDA(w->d_queue.ensure(64));
        RP_CUDA(cudaMemsetAsync(w->d_queue.p, 0, 64, st));
        // transform-list stamps restart with the substep counter
        RP_CUDA(w->d_tstamp.ensure(std::max<size_t>(N, 1) * 4));
        RP_CUDA(cudaMemsetAsync(w->d_tstamp.p, 0, std::max<size_t>(N, 1) * 4, st));
        RP_CUDA(w->d_tlist.ensure(std::max<size_t>(N, 1) * 4));
        w->dims.nbodies = (int)N;
        w->dims.ncolliders = (int)cols.size();
        w->dims.next = (int)E;
        w->dims.num_scenes = S;
        w->dims.grid_mode = w->grid_mode ? 1 : 0;
        w->layout_gen++;
    }
    if (!w->d_status.p) {
        RP_CUDA(w->d_barrier.ensure(64));
        RP_CUDA(cudaMemsetAsync(w->d_barrier.p, 0, 64, st));
        RP_CUDA(w->d_counters.ensure(32 * 8));
        RP_CUDA(cudaMemsetAsync(w->d_counters.p, 0, 256, st));
        RP_CUDA(w->d_phase.ensure(PHASES * 8));
        RP_CUDA(cudaMemsetAsync(w->d_phase.p, 0, PHASES * 8, st));
        RP_CUDA(w->d_deg.ensure(32));
        RP_CUDA(cudaMemsetAsync(w->d_deg.p, 0, 32, st));
    }
    RP_CUDA(w->d_status.ensure((size_t)S * 4));
    RP_CUDA(cudaMemsetAsync(w->d_status.p, 0, (size_t)S * 4, st));
    RP_CUDA(cudaMemsetAsync(w->d_pair_count.p, 0, (size_t)S * 4, st));
    RP_CUDA(cudaMemsetAsync(w->d_scene_levels.p, 0, (size_t)S * 4, st));
    RP_CUDA(cudaMemsetAsync(w->d_scene_vlevels.p, 0, (size_t)S * 4, st));
    {   // level tables start at zero; each substep's schedule clears what the previous one used
        const size_t lt = (size_t)S * (size_t)(w->max_levels + 1) * 4;
        RP_CUDA(cudaMemsetAsync(w->d_level_count.p, 0, lt, st));
        RP_CUDA(cudaMemsetAsync(w->d_level_fill.p, 0, lt, st));
        RP_CUDA(cudaMemsetAsync(w->d_vlevel_count.p, 0, lt, st));
        RP_CUDA(cudaMemsetAsync(w->d_vlevel_fill.p, 0, lt, st));
    }
    RP_CUDA(cudaMemsetAsync(w->d_act_count.p, 0, (size_t)S * 8, st));
    w->static_dirty = false;
    w->forces_dirty = true;
    // upload the host state
    w->device_state_valid = false;
    return RP_OK;
}

template <typename R>
WorldView<R> make_view(rp_world* w) {
    WorldView<R> V;
    std::memset(&V, 0, sizeof(V));
    V.num_scenes = w->num_scenes;
    V.scene_body = w->d_scene_body.as<int32_t>();
    V.scene_ext = w->d_scene_ext.as<int32_t>();
    V.scene_pair_cap = w->d_scene_pair_cap.as<int32_t>();
    V.scene_contact_cap = w->d_scene_contact_cap.as<int32_t>();
    V.scene_node_cap = w->d_scene_node_cap.as<int32_t>();
    V.pos = w->d_pos.as<double4_32a>();
    V.rot = w->d_rot.as<double4_32a>();
    V.prev_pos = w->d_ppos.as<double4_32a>();
    V.prev_rot = w->d_prot.as<double4_32a>();
    V.vel = w->d_vel.as<R>();
    V.omega = w->d_omega.as<R>();
    V.prev_vel = w->d_pvel.as<R>();
    V.prev_omega = w->d_pomega.as<R>();
    V.active = w->d_active.as<uint8_t>();
    V.deact = w->d_deact.as<double>();
    V.inv_mass = w->d_invm.as<R>();
    V.inertia = w->d_I.as<R>();
    V.inv_inertia = w->d_Iinv.as<R>();
    V.material = w->d_mat.as<R>();
    V.radius = w->d_radius.as<double>();
    V.bound = w->d_bound.as<float4>();
    V.fixed = w->d_fixed.as<uint8_t>();
    V.col_start = w->d_col_start.as<int32_t>();
    V.force = w->d_force.as<double>();
    V.torque = w->d_torque.as<double>();
    V.colliders = w->d_colliders.as<Collider>();
    V.shapes = w->d_shapes.as<Shape>();
    V.shape_verts = w->d_shape_verts.as<double>();
    V.face_normal = w->d_face_normal.as<double>();
    V.shape_verts_f = w->d_shape_verts_f.as<float>();
    V.face_normal_f = w->d_face_normal_f.as<float>();
    V.face_elem_start = w->d_face_elem_start.as<int32_t>();
    V.face_elem = w->d_face_elem.as<int32_t>();
    V.csr_start = w->d_csr_start.as<int32_t>();
    V.csr_data = w->d_csr_data.as<int32_t>();
    V.tverts = w->d_tverts.as<R>();
    V.tnorms = w->d_tnorms.as<R>();
    V.ext = w->d_ext.as<ExtConstraint>();
    V.pair_count = w->d_pair_count.as<int32_t>();
    V.pairs = w->d_pairs.as<int2>();
    V.row_count = w->d_row_count.as<int32_t>();
    V.sort_key = w->d_sort_key.as<uint32_t>();
    V.sort_val = w->d_sort_val.as<int32_t>();
    V.sort_hist = w->d_sort_hist.as<int32_t>();
    V.sort_hi = w->d_sort_hi.as<float>();
    V.uf_parent = w->d_uf_parent.as<int32_t>();
    V.island_awake = w->d_island_awake.as<uint8_t>();
    V.node_body = w->d_node_body.as<int32_t>();
    V.node_pred = w->d_node_pred.as<int32_t>();
    V.node_level = w->d_node_level.as<int32_t>();
    V.body_tl_count = w->d_tl_count.as<int32_t>();
    V.body_tl_start = w->d_tl_start.as<int32_t>();
    V.body_tl = w->d_tl.as<int32_t>();
    V.level_count = w->d_level_count.as<int32_t>();
    V.level_fill = w->d_level_fill.as<int32_t>();
    V.scan_tmp = w->d_scan_tmp.as<int32_t>();
    V.level_nodes = w->d_level_nodes.as<int32_t>();
    V.scene_levels = w->d_scene_levels.as<int32_t>();
    V.scene_nodes = w->d_scene_nodes.as<int32_t>();
    V.pair_cstart = w->d_pair_cstart.as<int32_t>();
    V.pair_ccount = w->d_pair_ccount.as<int32_t>();
    V.contact_count = w->d_contact_count.as<int32_t>();
    V.work = w->d_work.as<int32_t>();
    V.contacts = w->d_contacts.as<R>();
    V.ext_lambda = w->d_ext_lambda.as<double>();
    V.max_levels = w->max_levels;
    V.node_vpred = w->d_node_vpred.as<int32_t>();
    V.node_vlevel = w->d_node_vlevel.as<int32_t>();
    V.vlevel_count = w->d_vlevel_count.as<int32_t>();
    V.vlevel_fill = w->d_vlevel_fill.as<int32_t>();
    V.vlevel_nodes = w->d_vlevel_nodes.as<int32_t>();
    V.scene_vlevels = w->d_scene_vlevels.as<int32_t>();
    V.act_list = w->d_act_list.as<int32_t>();
    V.act_count = w->d_act_count.as<int32_t>();
    V.sweep_order = w->sweep_order;
    V.node_bits = w->d_node_bits.as<uint32_t>();
    V.status = w->d_status.as<uint32_t>();
    V.barrier = w->d_barrier.as<unsigned int>();
    V.counters = w->d_counters.as<unsigned long long>();
    V.phase_ns = w->d_phase.as<unsigned long long>();
    V.body_scene = w->d_body_scene.as<int32_t>();
    V.pose_f = w->d_pose_f.as<float4>();
    V.sdx = w->d_sdx.as<float4>();
    V.sdq = w->d_sdq.as<float4>();
    V.pred_d = w->d_pred_d.as<float4>();
    V.prev_qf = w->d_prev_qf.as<float4>();
    V.col_body = w->d_col_body.as<int32_t>();
    V.single_hull = w->d_single_hull.as<uint8_t>();
    V.work_list = w->d_work_list.as<int32_t>();
    V.work_state = w->d_work_state.as<int32_t>();
    V.gjk_list = w->d_gjk_list.as<int32_t>();
    V.hit_list = w->d_hit_list.as<int32_t>();
    V.work_simplex = w->d_work_simplex.as<R>();
    V.work_epa = w->d_work_epa.as<double>();
    V.work_off = w->d_work_off.as<float4>();
    V.pair_base = w->d_pair_base.as<float4>();
    V.ext_base = w->d_ext_base.as<float4>();
    V.fallback_list = w->d_fallback.as<int32_t>();
    V.work_face = w->d_work_face.as<float>();
    V.queue = w->d_queue.as<int32_t>();
    V.tstamp = w->d_tstamp.as<int32_t>();
    V.tlist = w->d_tlist.as<int32_t>();
    V.scene_order = w->d_scene_order.as<int32_t>();
    V.solo_nodes = w->solo_nodes;
    V.cta_scenes = w->cta_scenes;
    V.wait_ns = w->wait_ns;
    V.deg_first = w->d_deg.as<int32_t>();
    return V;
}

// Mutable per-body state layout on the device, for snapshots.
struct StateSlices {
    DevBuf* b[10];
    size_t bytes[10];
};
StateSlices state_slices(rp_world* w) {
    const size_t N = w->bodies.size(), R = w->rsize();
    StateSlices s = {{&w->d_pos, &w->d_rot, &w->d_ppos, &w->d_prot, &w->d_vel, &w->d_omega, &w->d_pvel, &w->d_pomega,
                      &w->d_active, &w->d_deact},
                     {N * 32, N * 32, N * 32, N * 32, N * 3 * R, N * 3 * R, N * 3 * R, N * 3 * R, N, N * 8}};
    return s;
}

// The body state's staging layout in the pinned buffer: pose arrays (double4 each), deactivation
// times, the four velocity arrays in the working type, the awake flags.
struct StateLayout {
    size_t pos, rot, ppos, prot, deact, vel, om, pvel, pom, act, total;
    StateLayout(size_t N, size_t R) {
        pos = 0; rot = pos + 32 * N; ppos = rot + 32 * N; prot = ppos + 32 * N; deact = prot + 32 * N;
        vel = deact + 8 * N; om = vel + 3 * R * N; pvel = om + 3 * R * N; pom = pvel + 3 * R * N; act = pom + 3 * R * N;
        total = act + N;
    }
};

rp_status upload_state(rp_world* w) {
    const size_t N = w->bodies.size(), R = w->rsize();
    const StateLayout L(N, R);
    RP_CUDA(w->h_state.ensure(L.total));
    char* h = (char*)w->h_state.p;
    double* pos = (double*)(h + L.pos);
    double* rot = (double*)(h + L.rot);
    double* ppos = (double*)(h + L.ppos);
    double* prot = (double*)(h + L.prot);
    double* deact = (double*)(h + L.deact);
    uint8_t* act = (uint8_t*)(h + L.act);
    auto put = [&](size_t off, size_t i, double v) {
        if (R == 8) ((double*)(h + off))[i] = v;
        else ((float*)(h + off))[i] = (float)v;
    };
    for (size_t slot = 0; slot < N; ++slot) {
        const HostBody& b = w->bodies[(size_t)w->slot_to_entity[slot]];
        for (int k = 0; k < 3; ++k) {
            pos[4 * slot + (size_t)k] = b.pos[k];
            ppos[4 * slot + (size_t)k] = b.ppos[k];
            put(L.vel, 3 * slot + (size_t)k, b.v[k]);
            put(L.om, 3 * slot + (size_t)k, b.w[k]);
            put(L.pvel, 3 * slot + (size_t)k, b.pv[k]);
            put(L.pom, 3 * slot + (size_t)k, b.pw[k]);
        }
        pos[4 * slot + 3] = 0.0;
        ppos[4 * slot + 3] = 0.0;
        for (int k = 0; k < 4; ++k) { rot[4 * slot + (size_t)k] = b.rot[k]; prot[4 * slot + (size_t)k] = b.prot[k]; }
        act[slot] = b.active != 0.0 ? 1 : 0;
        deact[slot] = b.deact;
    }
    cudaStream_t st = w->stream;
    w->h2d_bytes += N * (4 * 32 + 4 * 3 * R + 1 + 8);
    auto send = [&](DevBuf& d, size_t off, size_t bytes) -> cudaError_t {
        cudaError_t e = d.ensure(bytes);
        if (e != cudaSuccess || bytes == 0) return e;
        return cudaMemcpyAsync(d.p, h + off, bytes, cudaMemcpyHostToDevice, st);
    };
    RP_CUDA(send(w->d_pos, L.pos, 32 * N));
    RP_CUDA(send(w->d_rot, L.rot, 32 * N));
    RP_CUDA(send(w->d_ppos, L.ppos, 32 * N));
    RP_CUDA(send(w->d_prot, L.prot, 32 * N));
    RP_CUDA(send(w->d_vel, L.vel, 3 * R * N));
    RP_CUDA(send(w->d_omega, L.om, 3 * R * N));
    RP_CUDA(send(w->d_pvel, L.pvel, 3 * R * N));
    RP_CUDA(send(w->d_pomega, L.pom, 3 * R * N));
    RP_CUDA(send(w->d_active, L.act, N));
    RP_CUDA(send(w->d_deact, L.deact, 8 * N));
    RP_CUDA(cudaStreamSynchronize(st));   // the staging buffer is refilled by the next call
    w->device_state_valid = true;
    return RP_OK;
}

rp_status sync_state_to_host(rp_world* w) {
    if (!w->device_state_valid) return RP_OK;
    const size_t N = w->bodies.size(), R = w->rsize();
    cudaStream_t st = w->stream;
    const StateLayout L(N, R);
    RP_CUDA(w->h_state.ensure(L.total));
    char* h = (char*)w->h_state.p;
    if (N) {
        RP_CUDA(cudaMemcpyAsync(h + L.pos, w->d_pos.p, N * 32, cudaMemcpyDeviceToHost, st));
        RP_CUDA(cudaMemcpyAsync(h + L.rot, w->d_rot.p, N * 32, cudaMemcpyDeviceToHost, st));
        RP_CUDA(cudaMemcpyAsync(h + L.ppos, w->d_ppos.p, N * 32, cudaMemcpyDeviceToHost, st));
        RP_CUDA(cudaMemcpyAsync(h + L.prot, w->d_prot.p, N * 32, cudaMemcpyDeviceToHost, st));
        RP_CUDA(cudaMemcpyAsync(h + L.deact, w->d_deact.p, N * 8, cudaMemcpyDeviceToHost, st));
        RP_CUDA(cudaMemcpyAsync(h + L.vel, w->d_vel.p, 3 * R * N, cudaMemcpyDeviceToHost, st));
        RP_CUDA(cudaMemcpyAsync(h + L.om, w->d_omega.p, 3 * R * N, cudaMemcpyDeviceToHost, st));
        RP_CUDA(cudaMemcpyAsync(h + L.pvel, w->d_pvel.p, 3 * R * N, cudaMemcpyDeviceToHost, st));
        RP_CUDA(cudaMemcpyAsync(h + L.pom, w->d_pomega.p, 3 * R * N, cudaMemcpyDeviceToHost, st));
        RP_CUDA(cudaMemcpyAsync(h + L.act, w->d_active.p, N, cudaMemcpyDeviceToHost, st));
    }
    w->d2h_bytes += N * (4 * 32 + 4 * 3 * R + 1 + 8);
    RP_CUDA(cudaStreamSynchronize(st));
    const double* pos = (const double*)(h + L.pos);
    const double* rot = (const double*)(h + L.rot);
    const double* ppos = (const double*)(h + L.ppos);
    const double* prot = (const double*)(h + L.prot);
    const double* deact = (const double*)(h + L.deact);
    const uint8_t* act = (const uint8_t*)(h + L.act);
    auto get = [&](size_t off, size_t i) -> double {
        return R == 8 ? ((const double*)(h + off))[i] : (double)((const float*)(h + off))[i];
    };
    for (size_t slot = 0; slot < N; ++slot) {
        HostBody& b = w->bodies[(size_t)w->slot_to_entity[slot]];
        for (int k = 0; k < 3; ++k) {
            b.pos[k] = pos[4 * slot + (size_t)k];
            b.ppos[k] = ppos[4 * slot + (size_t)k];
            b.v[k] = get(L.vel, 3 * slot + (size_t)k);
            b.w[k] = get(L.om, 3 * slot + (size_t)k);
            b.pv[k] = get(L.pvel, 3 * slot + (size_t)k);
            b.pw[k] = get(L.pom, 3 * slot + (size_t)k);
        }
        for (int k = 0; k < 4; ++k) { b.rot[k] = rot[4 * slot + (size_t)k]; b.prot[k] = prot[4 * slot + (size_t)k]; }
        b.active = act[slot] ? 1.0 : 0.0;
        b.deact = deact[slot];
    }
    return RP_OK;
}

rp_status ensure_device(rp_world* w) {
    if (w->device < 0) return fail(RP_ERR_NO_DEVICE, "host-only world (created with device -1)");
    if (w->static_dirty) {
        rp_status s = build_device(w);
        if (s != RP_OK) return s;
    }
    if (!w->device_state_valid) {
        rp_status s = upload_state(w);
        if (s != RP_OK) return s;
    }
    return RP_OK;
}

// calculate_external_force / _torque (physics_util.cpp:5-24) over the step's forces, then gravity
rp_status upload_forces(rp_world* w) {
    const size_t N = w->bodies.size();
    std::vector<double> F(3 * N, 0.0), T(3 * N, 0.0);
    for (size_t slot = 0; slot < N; ++slot) {
        const HostBody& b = w->bodies[(size_t)w->slot_to_entity[slot]];
        if (b.fixed) continue;
        double f[3] = {0.0, 0.0, 0.0}, t[3] = {0.0, 0.0, 0.0};
        std::vector<Force> all = b.forces;
        if (w->gravity != 0.0) all.push_back({{0.0, 0.0, 0.0}, {0.0, -w->gravity * 1.0 / b.invm, 0.0}});
        for (const Force& x : all) { f[0] = f[0] + x.f[0]; f[1] = f[1] + x.f[1]; f[2] = f[2] + x.f[2]; }
        for (const Force& x : all) {
            double d[3] = {x.pos[0] - 0.0, x.pos[1] - 0.0, x.pos[2] - 0.0};
            double c[3] = {d[1] * x.f[2] - d[2] * x.f[1], d[2] * x.f[0] - d[0] * x.f[2], d[0] * x.f[1] - d[1] * x.f[0]};
            t[0] = t[0] + c[0]; t[1] = t[1] + c[1]; t[2] = t[2] + c[2];
        }
        for (int k = 0; k < 3; ++k) { F[3 * slot + (size_t)k] = f[k]; T[3 * slot + (size_t)k] = t[k]; }
    }
    w->h2d_bytes += 2 * F.size() * sizeof(double);
    RP_CUDA(upload(w->d_force, F, w->stream));
    RP_CUDA(upload(w->d_torque, T, w->stream));
    RP_CUDA(cudaStreamSynchronize(w->stream));
    w->forces_dirty = false;
    return RP_OK;
}

// The launch mode a frame uses: the persistent kernel (one launch per frame) or the phase-major
// pipeline (one kernel per phase, replayed from a captured CUDA graph).
bool use_pipeline(const rp_world* w) {
    if (w->mode == RP_MODE_PERSISTENT) return false;
    if (w->mode == RP_MODE_PHASED) return true;
    const char* env = std::getenv("RP_MODE");
    if (env && std::strcmp(env, "persistent") == 0) return false;
    return true;
}

cudaError_t pipe_frame(rp_world* w, const StepParams& P, PipeMarks* marks) {
    if (w->precision == RP_PRECISION_FP64) return pipe_frame_f64(make_view<double>(w), P, w->pipe, w->dims, w->stream, marks);
    return pipe_frame_f32(make_view<float>(w), P, w->pipe, w->dims, w->stream, marks);
}

cudaError_t launch_pipeline(rp_world* w, const StepParams& P) {
    cudaError_t e;
    if (!w->pipe_ready) {
        e = w->precision == RP_PRECISION_FP64 ? pipe_configure_f64(w->pipe, w->num_sms) : pipe_configure_f32(w->pipe, w->num_sms);
        if (e != cudaSuccess) return e;
        w->pipe_ready = true;
    }
    w->launches += (uint64_t)(w->precision == RP_PRECISION_FP64 ? pipe_launches_f64(P) : pipe_launches_f32(P));
    if (!w->timing && w->stream == nullptr) {
        // the legacy default stream cannot be captured: launch the frame's kernels directly
        return pipe_frame(w, P, nullptr);
    }
    if (w->timing) {
        // a timed frame runs without the graph, with an event after every phase
        const int cap = 2 + P.num_substeps * 12;
        while ((int)w->marks.size() < cap) {
            cudaEvent_t ev;
            e = cudaEventCreate(&ev);
            if (e != cudaSuccess) return e;
            w->marks.push_back(ev);
        }
        w->mark_phase.assign((size_t)cap, 0);
        PipeMarks m;
        m.ev = w->marks.data();
        m.phase = w->mark_phase.data();
        m.cap = cap;
        e = pipe_frame(w, P, &m);
        if (e != cudaSuccess) return e;
        e = cudaEventSynchronize(w->marks[(size_t)m.n - 1]);
        if (e != cudaSuccess) return e;
        for (int i = 1; i < m.n; ++i) {
            float ms = 0.f;
            e = cudaEventElapsedTime(&ms, w->marks[(size_t)i - 1], w->marks[(size_t)i]);
            if (e != cudaSuccess) return e;
            const int ph = m.phase[i];
            if (ph >= 0 && ph < PHASES) w->phase_ms[ph] += ms;
        }
        return cudaSuccess;
    }
    const StepParams& G = w->graph_params;
    if (!w->graph || w->graph_gen != w->layout_gen || G.dt != P.dt || G.num_substeps != P.num_substeps ||
        G.num_pos_iters != P.num_pos_iters || G.enable_collisions != P.enable_collisions) {
        if (w->graph) { cudaGraphExecDestroy(w->graph); w->graph = nullptr; }
        cudaGraph_t g = nullptr;
        e = cudaStreamBeginCapture(w->stream, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return e;
        cudaError_t le = pipe_frame(w, P, nullptr);
        e = cudaStreamEndCapture(w->stream, &g);
        if (le != cudaSuccess) { if (g) cudaGraphDestroy(g); return le; }
        if (e != cudaSuccess) return e;
        e = cudaGraphInstantiate(&w->graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) { w->graph = nullptr; return e; }
        w->graph_gen = w->layout_gen;
        w->graph_params = P;
    }
    return cudaGraphLaunch(w->graph, w->stream);
}

cudaError_t launch_step(rp_world* w, const StepParams& P) {
    if (use_pipeline(w)) return launch_pipeline(w, P);
    cudaError_t e;
    if (w->precision == RP_PRECISION_FP64) e = step_f64(make_view<double>(w), P, w->grid_mode, w->grid_mode ? w->grid_blocks : w->num_scenes, w->stream);
    else e = step_f32(make_view<float>(w), P, w->grid_mode, w->grid_mode ? w->grid_blocks : w->num_scenes, w->stream);
    w->launches++;
    return e;
}

rp_status snapshot(rp_world* w, bool restore) {
    StateSlices s = state_slices(w);
    size_t total = 0;
    for (int i = 0; i < 10; ++i) total += (s.bytes[i] + 255) & ~(size_t)255;
    if (!restore) RP_CUDA(w->d_backup.ensure(total));
    size_t off = 0;
    for (int i = 0; i < 10; ++i) {
        char* bk = (char*)w->d_backup.p + off;
        if (s.bytes[i]) {
            if (restore) RP_CUDA(cudaMemcpyAsync(s.b[i]->p, bk, s.bytes[i], cudaMemcpyDeviceToDevice, w->stream));
            else RP_CUDA(cudaMemcpyAsync(bk, s.b[i]->p, s.bytes[i], cudaMemcpyDeviceToDevice, w->stream));
        }
        off += (s.bytes[i] + 255) & ~(size_t)255;
    }
    return RP_OK;
}

uint32_t read_status(rp_world* w, cudaError_t& e) {
    std::vector<uint32_t> st((size_t)w->num_scenes, 0);
    e = cudaMemcpyAsync(st.data(), w->d_status.p, st.size() * 4, cudaMemcpyDeviceToHost, w->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(w->stream);
    uint32_t bits = 0;
    for (uint32_t x : st) bits |= x;
    if (e == cudaSuccess) e = cudaMemsetAsync(w->d_status.p, 0, st.size() * 4, w->stream);
    return bits;
}

}  // namespace

// =====================================================================================================
// C ABI
extern "C" {

const char* rp_last_error(void) { return g_last_error.c_str(); }

rp_status rp_world_create(rp_world** out, int32_t device, int32_t precision) {
    if (!out) return fail(RP_ERR_INVALID, "null out");
    *out = nullptr;
    if (precision != RP_PRECISION_FP32 && precision != RP_PRECISION_FP64) return fail(RP_ERR_INVALID, "bad precision");
    if (device == -1) {
        rp_world* hw = new rp_world();
        hw->device = -1;
        hw->precision = precision;
        hw->scene_body.assign(2, 0);
        *out = hw;
        return RP_OK;
    }
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return fail(RP_ERR_NO_DEVICE, "no CUDA device");
    if (device < 0 || device >= n) return fail(RP_ERR_INVALID, "bad device index");
    RP_CUDA(cudaSetDevice(device));
    cudaDeviceProp prop;
    RP_CUDA(cudaGetDeviceProperties(&prop, device));
    if (prop.major < 10) return fail(RP_ERR_NO_DEVICE, "the kernels are built for sm_103a (GB300)");
    std::unique_ptr<rp_world> w(new rp_world());
    w->device = device;
    w->precision = precision;
    w->num_sms = prop.multiProcessorCount;
    RP_CUDA(precision == RP_PRECISION_FP64 ? configure_f64() : configure_f32());
    int per_sm = precision == RP_PRECISION_FP64 ? grid_blocks_per_sm_f64() : grid_blocks_per_sm_f32();
    if (per_sm <= 0) return fail(RP_ERR_CUDA, "step kernel cannot be resident");
    w->grid_blocks = std::min(per_sm * w->num_sms, 4096);
    RP_CUDA(cudaStreamCreateWithFlags(&w->stream, cudaStreamNonBlocking));
    w->own_stream = true;
    RP_CUDA(cudaEventCreate(&w->ev0));
    RP_CUDA(cudaEventCreate(&w->ev1));
    w->scene_body.assign(2, 0);
    *out = w.release();
    return RP_OK;
}

void rp_world_destroy(rp_world* w) {
    if (!w) return;
    if (w->device < 0) {
        delete w;
        return;
    }
    cudaSetDevice(w->device);
    if (w->stream) cudaStreamSynchronize(w->stream);
    if (w->ev0) cudaEventDestroy(w->ev0);
    if (w->ev1) cudaEventDestroy(w->ev1);
    if (w->ev_rec) cudaEventDestroy(w->ev_rec);
    if (w->graph) cudaGraphExecDestroy(w->graph);
    for (cudaEvent_t ev : w->marks) cudaEventDestroy(ev);
    if (w->own_stream && w->stream) cudaStreamDestroy(w->stream);
    delete w;
}

rp_status rp_world_set_stream(rp_world* w, void* stream) {
    if (check_world(w)) return RP_ERR_INVALID;
    if (w->device < 0) return fail(RP_ERR_NO_DEVICE, "host-only world");
    RP_CUDA(cudaStreamSynchronize(w->stream));
    if (w->own_stream) cudaStreamDestroy(w->stream);
    w->stream = (cudaStream_t)stream;
    w->own_stream = false;
    return RP_OK;
}

rp_status rp_scene_create(rp_world* w, int32_t* out) {
    if (check_world(w)) return RP_ERR_INVALID;
    if (out) *out = w->num_scenes;
    w->num_scenes++;
    w->static_dirty = true;
    return RP_OK;
}

rp_status rp_hull_create(rp_world* w, const double* v, uint32_t nv, const uint32_t* idx, uint32_t ni, int32_t* out) {
    if (check_world(w) || !v || !idx || !out) return fail(RP_ERR_INVALID, "null argument");
    std::vector<double> key(v, v + 3 * (size_t)nv);
    key.push_back(-1.0);
    for (uint32_t i = 0; i < ni; ++i) key.push_back((double)idx[i]);
    auto it = w->hull_index.find(key);
    if (it != w->hull_index.end()) { *out = it->second; return RP_OK; }
    std::unique_ptr<Hull> h(new Hull());
    std::string err = build_hull(v, nv, idx, ni, *h);
    if (!err.empty()) return fail(RP_ERR_DEGENERATE, err);
    *out = (int32_t)w->hulls.size();
    w->hulls.push_back(std::move(h));
    w->hull_index.emplace(std::move(key), *out);
    w->static_dirty = true;
    return RP_OK;
}

rp_status rp_hull_create_from_topology(rp_world* w, const double* verts, int32_t nv, const double* normals, int32_t nf,
                                       const int32_t* fstart, const int32_t* felem, const int32_t* v2f_start,
                                       const int32_t* v2f, const int32_t* v2n_start, const int32_t* v2n,
                                       const int32_t* f2n_start, const int32_t* f2n, int32_t* out) {
    if (check_world(w) || !verts || !normals || !fstart || !felem || !v2f_start || !v2f || !v2n_start || !v2n ||
        !f2n_start || !f2n || !out || nv <= 0 || nf <= 0)
        return fail(RP_ERR_INVALID, "bad hull topology");
    std::unique_ptr<Hull> h(new Hull());
    h->verts.assign(verts, verts + 3 * (size_t)nv);
    h->normals.assign(normals, normals + 3 * (size_t)nf);
    auto rows = [](const int32_t* start, const int32_t* data, int32_t n, int32_t bound, std::vector<std::vector<int>>& dst) {
        dst.assign((size_t)n, {});
        for (int32_t r = 0; r < n; ++r) {
            if (start[r + 1] < start[r]) return false;
            for (int32_t k = start[r]; k < start[r + 1]; ++k) {
                if (data[k] < 0 || data[k] >= bound) return false;
                dst[(size_t)r].push_back(data[k]);
            }
        }
        return true;
    };
    if (!rows(fstart, felem, nf, nv, h->faces) || !rows(v2f_start, v2f, nv, nf, h->v2f) ||
        !rows(v2n_start, v2n, nv, nv, h->v2n) || !rows(f2n_start, f2n, nf, nf, h->f2n))
        return fail(RP_ERR_INVALID, "hull topology index out of range");
    *out = (int32_t)w->hulls.size();
    w->hulls.push_back(std::move(h));
    w->static_dirty = true;
    return RP_OK;
}

rp_status rp_hull_info(rp_world* w, int32_t hull, int32_t* nv, int32_t* nf) {
    if (check_world(w) || hull < 0 || hull >= (int32_t)w->hulls.size()) return fail(RP_ERR_INVALID, "bad hull");
    if (nv) *nv = w->hulls[(size_t)hull]->nv();
    if (nf) *nf = w->hulls[(size_t)hull]->nf();
    return RP_OK;
}

rp_status rp_hull_topology(rp_world* w, int32_t hull, int32_t which, int32_t* start, int32_t* data, int32_t cap, int32_t* nrows,
                           int32_t* ndata) {
    if (check_world(w) || hull < 0 || hull >= (int32_t)w->hulls.size() || which < 0 || which > 3)
        return fail(RP_ERR_INVALID, "bad hull or table");
    const Hull& H = *w->hulls[(size_t)hull];
    const std::vector<std::vector<int>>& t = which == 0 ? H.faces : which == 1 ? H.v2f : which == 2 ? H.v2n : H.f2n;
    int32_t total = 0;
    for (const auto& r : t) total += (int32_t)r.size();
    if (nrows) *nrows = (int32_t)t.size();
    if (ndata) *ndata = total;
    int32_t k = 0;
    for (size_t r = 0; r < t.size(); ++r) {
        if (start) start[r] = k;
        for (int x : t[r]) {
            if (data && k < cap) data[k] = x;
            ++k;
        }
    }
    if (start) start[t.size()] = k;
    return RP_OK;
}

rp_status rp_hull_geometry(rp_world* w, int32_t hull, double* verts, double* normals) {
    if (check_world(w) || hull < 0 || hull >= (int32_t)w->hulls.size()) return fail(RP_ERR_INVALID, "bad hull");
    const Hull& H = *w->hulls[(size_t)hull];
    if (verts) std::memcpy(verts, H.verts.data(), H.verts.size() * sizeof(double));
    if (normals) std::memcpy(normals, H.normals.data(), H.normals.size() * sizeof(double));
    return RP_OK;
}

rp_status rp_hull_face(rp_world* w, int32_t hull, int32_t face, double normal[3], int32_t* elems, int32_t cap, int32_t* ne) {
    if (check_world(w) || hull < 0 || hull >= (int32_t)w->hulls.size()) return fail(RP_ERR_INVALID, "bad hull");
    const Hull& H = *w->hulls[(size_t)hull];
    if (face < 0 || face >= H.nf()) return fail(RP_ERR_INVALID, "bad face");
    if (normal)
        for (int k = 0; k < 3; ++k) normal[k] = H.normals[(size_t)(3 * face + k)];
    const std::vector<int>& f = H.faces[(size_t)face];
    if (ne) *ne = (int32_t)f.size();
    for (int32_t i = 0; i < cap && i < (int32_t)f.size(); ++i) elems[i] = f[(size_t)i];
    return RP_OK;
}

rp_status rp_entity_create(rp_world* w, int32_t scene, const double p[3], const double q[4], double mass, int32_t fixed,
                           const rp_collider_desc* cols, uint32_t ncols, double mus, double mud, double rest, int32_t* out) {
    if (check_world(w) || !p || !q || (!cols && ncols) || !out) return fail(RP_ERR_INVALID, "null argument");
    if (scene < 0 || scene >= w->num_scenes) return fail(RP_ERR_INVALID, "bad scene");
    if (ncols == 0) return fail(RP_ERR_INVALID, "an entity needs at least one collider");
    if (!finite3(p) || !std::isfinite(q[0]) || !std::isfinite(q[1]) || !std::isfinite(q[2]) || !std::isfinite(q[3]))
        return fail(RP_ERR_INVALID, "pose is not finite");
    if (!fixed && !(mass > 0.0)) return fail(RP_ERR_INVALID, "mass must be positive");
    if (!(mus >= 0.0 && mus <= 1.0 && mud >= 0.0 && mud <= 1.0 && rest >= 0.0 && rest <= 1.0))
        return fail(RP_ERR_INVALID, "friction and restitution must lie in [0, 1] (entity.cpp:55-57)");
    HostBody b;
    b.scene = scene;
    for (uint32_t i = 0; i < ncols; ++i) {
        if (cols[i].type == RP_COLLIDER_HULL) {
            if (cols[i].hull < 0 || cols[i].hull >= (int32_t)w->hulls.size()) return fail(RP_ERR_INVALID, "bad hull id");
        } else if (cols[i].type != RP_COLLIDER_SPHERE || !(cols[i].radius > 0.0f)) {
            return fail(RP_ERR_INVALID, "bad collider");
        }
        b.cols.push_back(cols[i]);
    }
    std::vector<ColliderDesc> d = descs(w, b.cols);
    b.radius = bounding_radius(d);
    if (fixed) {
        b.invm = 0.0;
        for (int k = 0; k < 9; ++k) b.I[k] = b.Iinv[k] = 0.0;
    } else {
        b.invm = 1.0 / mass;
        std::string err = inertia(d, mass, b.I, b.Iinv);
        if (!err.empty()) return fail(RP_ERR_DEGENERATE, err);
    }
    for (int k = 0; k < 3; ++k) b.pos[k] = p[k];
    for (int k = 0; k < 4; ++k) b.rot[k] = q[k];
    b.fixed = fixed ? 1 : 0;
    b.mus = mus;
    b.mud = mud;
    b.rest = rest;
    if (w->device_state_valid) {
        rp_status s = sync_state_to_host(w);
        if (s != RP_OK) return s;
        w->device_state_valid = false;
    }
    w->bodies.push_back(b);
    w->static_dirty = true;
    *out = (int32_t)w->bodies.size() - 1;
    return RP_OK;
}

rp_status rp_entities_create(rp_world* w, uint32_t n, const int32_t* scene, const double* pos, const double* rot,
                             const double* mass, const int32_t* fixed, const rp_collider_desc* cols, const double* mus,
                             const double* mud, const double* rest, const double* vel, const double* omega,
                             int32_t* out_first) {
    if (check_world(w) || !out_first || (n && (!scene || !pos || !rot || !mass || !fixed || !cols || !mus || !mud || !rest)))
        return fail(RP_ERR_INVALID, "null argument");
    *out_first = (int32_t)w->bodies.size();
    if (w->device_state_valid) {
        rp_status s = sync_state_to_host(w);
        if (s != RP_OK) return s;
        w->device_state_valid = false;
    }
    const size_t first = w->bodies.size();
    w->bodies.reserve(first + n);
    static const double zero[3] = {0.0, 0.0, 0.0};
    for (uint32_t i = 0; i < n; ++i) {
        int32_t e = 0;
        rp_status s = rp_entity_create(w, scene[i], pos + 3 * (size_t)i, rot + 4 * (size_t)i, mass[i], fixed[i], cols + i, 1,
                                       mus[i], mud[i], rest[i], &e);
        if (s == RP_OK && (vel || omega)) {
            HostBody& b = w->bodies[(size_t)e];
            const double* v = vel ? vel + 3 * (size_t)i : zero;
            const double* om = omega ? omega + 3 * (size_t)i : zero;
            for (int k = 0; k < 3; ++k) { b.v[k] = v[k]; b.w[k] = om[k]; }
        }
        if (s != RP_OK) {
            w->bodies.resize(first);   // all or nothing
            return s;
        }
    }
    return RP_OK;
}

rp_status rp_entity_set_velocity(rp_world* w, int32_t e, const double v[3], const double om[3]) {
    if (check_world(w) || e < 0 || e >= (int32_t)w->bodies.size() || !v || !om) return fail(RP_ERR_INVALID, "bad entity");
    if (w->device_state_valid) {
        rp_status s = sync_state_to_host(w);
        if (s != RP_OK) return s;
        w->device_state_valid = false;
    }
    for (int k = 0; k < 3; ++k) { w->bodies[(size_t)e].v[k] = v[k]; w->bodies[(size_t)e].w[k] = om[k]; }
    return RP_OK;
}

rp_status rp_entity_add_force(rp_world* w, int32_t e, const double pos[3], const double f[3], int32_t local) {
    if (check_world(w) || e < 0 || e >= (int32_t)w->bodies.size() || !pos || !f) return fail(RP_ERR_INVALID, "bad entity");
    Force x;
    if (local) {
        // entity_add_force with local coordinates (entity.cpp:176-191): rotate the force and the
        // point by the entity's current orientation (unit scale)
        if (w->device_state_valid) {
            rp_status s = sync_state_to_host(w);
            if (s != RP_OK) return s;
        }
        const double* q = w->bodies[(size_t)e].rot;
        double ix = q[3] * f[0] + q[1] * f[2] - q[2] * f[1];
        double iy = q[3] * f[1] + q[2] * f[0] - q[0] * f[2];
        double iz = q[3] * f[2] + q[0] * f[1] - q[1] * f[0];
        double iw = -q[0] * f[0] - q[1] * f[1] - q[2] * f[2];
        x.f[0] = (ix * q[3]) + (iw * -q[0]) + (iy * -q[2]) - (iz * -q[1]);
        x.f[1] = (iy * q[3]) + (iw * -q[1]) + (iz * -q[0]) - (ix * -q[2]);
        x.f[2] = (iz * q[3]) + (iw * -q[2]) + (ix * -q[1]) - (iy * -q[0]);
        double m[3][3];
        m[0][0] = 1.0 - 2.0 * q[1] * q[1] - 2.0 * q[2] * q[2];
        m[1][0] = 2.0 * q[0] * q[1] + 2.0 * q[3] * q[2];
        m[2][0] = 2.0 * q[0] * q[2] - 2.0 * q[3] * q[1];
        m[0][1] = 2.0 * q[0] * q[1] - 2.0 * q[3] * q[2];
        m[1][1] = 1.0 - (2.0 * q[0] * q[0]) - (2.0 * q[2] * q[2]);
        m[2][1] = 2.0 * q[1] * q[2] + 2.0 * q[3] * q[0];
        m[0][2] = 2.0 * q[0] * q[2] + 2.0 * q[3] * q[1];
        m[1][2] = 2.0 * q[1] * q[2] - 2.0 * q[3] * q[0];
        m[2][2] = 1.0 - (2.0 * q[0] * q[0]) - (2.0 * q[1] * q[1]);
        // rotation * identity scale, then the point transform with a zero translation column
        double r[3][4];
        for (int i = 0; i < 3; ++i) {
            for (int j = 0; j < 3; ++j) {
                double sc[3] = {j == 0 ? 1.0 : 0.0, j == 1 ? 1.0 : 0.0, j == 2 ? 1.0 : 0.0};
                r[i][j] = m[i][0] * sc[0] + m[i][1] * sc[1] + m[i][2] * sc[2] + 0.0 * 0.0;
            }
            r[i][3] = m[i][0] * 0.0 + m[i][1] * 0.0 + m[i][2] * 0.0 + 0.0 * 1.0;
        }
        for (int i = 0; i < 3; ++i) x.pos[i] = r[i][0] * pos[0] + r[i][1] * pos[1] + r[i][2] * pos[2] + r[i][3] * 1.0;
    } else {
        for (int k = 0; k < 3; ++k) { x.pos[k] = pos[k]; x.f[k] = f[k]; }
    }
    w->bodies[(size_t)e].forces.push_back(x);
    w->forces_dirty = true;
    return RP_OK;
}

rp_status rp_entity_clear_forces(rp_world* w, int32_t e) {
    if (check_world(w) || e < 0 || e >= (int32_t)w->bodies.size()) return fail(RP_ERR_INVALID, "bad entity");
    if (!w->bodies[(size_t)e].forces.empty()) w->forces_dirty = true;
    w->bodies[(size_t)e].forces.clear();
    return RP_OK;
}

rp_status rp_world_set_gravity(rp_world* w, double g) {
    if (check_world(w) || !std::isfinite(g)) return fail(RP_ERR_INVALID, "bad gravity");
    if (g != w->gravity) w->forces_dirty = true;
    w->gravity = g;
    return RP_OK;
}

rp_status rp_entity_get_mass_properties(rp_world* w, int32_t e, double* invm, double I[9], double Iinv[9], double* radius) {
    if (check_world(w) || e < 0 || e >= (int32_t)w->bodies.size()) return fail(RP_ERR_INVALID, "bad entity");
    const HostBody& b = w->bodies[(size_t)e];
    if (invm) *invm = b.invm;
    if (I) std::memcpy(I, b.I, sizeof(b.I));
    if (Iinv) std::memcpy(Iinv, b.Iinv, sizeof(b.Iinv));
    if (radius) *radius = b.radius;
    return RP_OK;
}

rp_status rp_entity_set_mass_properties(rp_world* w, int32_t e, double invm, const double I[9], const double Iinv[9],
                                        double radius) {
    if (check_world(w) || e < 0 || e >= (int32_t)w->bodies.size() || !I || !Iinv) return fail(RP_ERR_INVALID, "bad entity");
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c)
            if (I[3 * r + c] != I[3 * c + r] || Iinv[3 * r + c] != Iinv[3 * c + r])
                return fail(RP_ERR_INVALID, "inertia tensors must be symmetric");
    HostBody& b = w->bodies[(size_t)e];
    b.invm = invm;
    std::memcpy(b.I, I, sizeof(b.I));
    std::memcpy(b.Iinv, Iinv, sizeof(b.Iinv));
    b.radius = radius;
    if (w->device_state_valid) {
        rp_status s = sync_state_to_host(w);
        if (s != RP_OK) return s;
        w->device_state_valid = false;
    }
    w->static_dirty = true;
    w->forces_dirty = true;
    return RP_OK;
}

int32_t rp_num_entities(const rp_world* w) { return w ? (int32_t)w->bodies.size() : 0; }

static rp_status add_ext(rp_world* w, ExtConstraint c, int32_t* out) {
    if (c.e1 < 0 || c.e2 < 0 || c.e1 >= (int32_t)w->bodies.size() || c.e2 >= (int32_t)w->bodies.size())
        return fail(RP_ERR_INVALID, "bad entity");
    if (w->bodies[(size_t)c.e1].scene != w->bodies[(size_t)c.e2].scene) return fail(RP_ERR_INVALID, "entities in different scenes");
    if (c.e1 == c.e2) return fail(RP_ERR_INVALID, "a constraint needs two distinct entities");
    if (w->device_state_valid) {
        rp_status s = sync_state_to_host(w);
        if (s != RP_OK) return s;
        w->device_state_valid = false;
    }
    HostExt x;
    x.c = c;
    x.scene = w->bodies[(size_t)c.e1].scene;
    w->exts.push_back(x);
    w->static_dirty = true;
    if (out) *out = (int32_t)w->exts.size() - 1;
    return RP_OK;
}

static ExtConstraint ext_base(int32_t type, int32_t e1, int32_t e2, const double* r1, const double* r2) {
    ExtConstraint c;
    std::memset(&c, 0, sizeof(c));
    c.type = type;
    c.e1 = e1;
    c.e2 = e2;
    for (int k = 0; k < 3; ++k) { c.r1[k] = r1 ? r1[k] : 0.0; c.r2[k] = r2 ? r2[k] : 0.0; }
    return c;
}

rp_status rp_constraint_positional(rp_world* w, int32_t e1, int32_t e2, const double r1[3], const double r2[3], double compliance,
                                   const double distance[3], int32_t* out) {
    if (check_world(w) || !r1 || !r2 || !distance) return fail(RP_ERR_INVALID, "null argument");
    ExtConstraint c = ext_base(CON_POSITIONAL, e1, e2, r1, r2);
    c.compliance = compliance;
    for (int k = 0; k < 3; ++k) c.distance[k] = distance[k];
    return add_ext(w, c, out);
}

rp_status rp_constraint_mutual_orientation(rp_world* w, int32_t e1, int32_t e2, double compliance, int32_t* out) {
    if (check_world(w)) return RP_ERR_INVALID;
    ExtConstraint c = ext_base(CON_MUTUAL_ORIENTATION, e1, e2, nullptr, nullptr);
    c.compliance = compliance;
    return add_ext(w, c, out);
}

rp_status rp_constraint_hinge(rp_world* w, int32_t e1, int32_t e2, const double r1[3], const double r2[3], double compliance,
                              int32_t a1, int32_t a2, int32_t limited, int32_t l1, int32_t l2, double lower, double upper,
                              int32_t* out) {
    if (check_world(w) || !r1 || !r2) return fail(RP_ERR_INVALID, "null argument");
    if (a1 < 0 || a1 > 5 || a2 < 0 || a2 > 5 || (limited && (l1 < 0 || l1 > 5 || l2 < 0 || l2 > 5)))
        return fail(RP_ERR_INVALID, "bad axis");
    ExtConstraint c = ext_base(CON_HINGE, e1, e2, r1, r2);
    c.compliance = compliance;
    c.a1 = a1; c.a2 = a2; c.limited = limited ? 1 : 0;
    c.l1 = limited ? l1 : 0; c.l2 = limited ? l2 : 0;
    c.lo = limited ? lower : 0.0; c.hi = limited ? upper : 0.0;
    return add_ext(w, c, out);
}

rp_status rp_constraint_spherical(rp_world* w, int32_t e1, int32_t e2, const double r1[3], const double r2[3], int32_t s1,
                                  int32_t s2, int32_t t1, int32_t t2, double slo, double shi, double tlo, double thi,
                                  int32_t* out) {
    if (check_world(w) || !r1 || !r2) return fail(RP_ERR_INVALID, "null argument");
    if (s1 < 0 || s1 > 5 || s2 < 0 || s2 > 5 || t1 < 0 || t1 > 5 || t2 < 0 || t2 > 5) return fail(RP_ERR_INVALID, "bad axis");
    ExtConstraint c = ext_base(CON_SPHERICAL, e1, e2, r1, r2);
    c.a1 = s1; c.a2 = s2; c.l1 = t1; c.l2 = t2;
    c.lo = slo; c.hi = shi; c.lo2 = tlo; c.hi2 = thi;
    return add_ext(w, c, out);
}

rp_status rp_simulate(rp_world* w, double dt, uint32_t substeps, uint32_t iters, int32_t collisions, uint32_t nsteps) {
    if (check_world(w)) return RP_ERR_INVALID;
    if (!std::isfinite(dt) || substeps == 0) return fail(RP_ERR_INVALID, "bad dt or substep count");
    if (w->device < 0) return fail(RP_ERR_NO_DEVICE, "host-only world (created with device -1)");
    if (w->bodies.empty() || nsteps == 0 || !(dt > 0.0)) return RP_OK;
    RP_CUDA(cudaSetDevice(w->device));
    rp_status s = ensure_device(w);
    if (s != RP_OK) return s;
    if (w->forces_dirty) {
        s = upload_forces(w);
        if (s != RP_OK) return s;
    }
    StepParams P;
    P.dt = dt;
    P.num_substeps = (int32_t)substeps;
    P.num_pos_iters = (int32_t)iters;
    P.enable_collisions = collisions ? 1 : 0;
    P.pad = 0;
    for (int attempt = 0; attempt < 6; ++attempt) {
        s = snapshot(w, false);
        if (s != RP_OK) return s;
        if (w->timing) RP_CUDA(cudaEventRecord(w->ev0, w->stream));
        for (uint32_t k = 0; k < nsteps; ++k) RP_CUDA(launch_step(w, P));
        if (w->timing) RP_CUDA(cudaEventRecord(w->ev1, w->stream));
        cudaError_t e;
        uint32_t bits = read_status(w, e);
        if (e != cudaSuccess) return fail(RP_ERR_CUDA, cudaGetErrorString(e));
        if (w->timing) {
            float ms = 0.f;
            RP_CUDA(cudaEventElapsedTime(&ms, w->ev0, w->ev1));
            w->last_ms = ms / nsteps;
        }
        if (bits & (ST_PAIR_OVERFLOW | ST_CONTACT_OVERFLOW)) {
            // restore the frames' starting state, grow the scratch 4x and redo them
            s = snapshot(w, true);
            if (s != RP_OK) return s;
            s = sync_state_to_host(w);
            if (s != RP_OK) return s;
            if (bits & ST_PAIR_OVERFLOW) w->pair_mult *= 4.0;
            if (bits & ST_CONTACT_OVERFLOW) w->contact_mult *= 4.0;
            w->static_dirty = true;
            s = ensure_device(w);
            if (s != RP_OK) return s;
            s = upload_forces(w);
            if (s != RP_OK) return s;
            continue;
        }
        if (bits & ST_BARRIER_TIMEOUT) {
            // a bounded wait gave up and the frame was abandoned: restore the call's starting state
            // and leave forces pending, as if the call had not run
            s = snapshot(w, true);
            if (s != RP_OK) return s;
            RP_CUDA(cudaStreamSynchronize(w->stream));
            return fail(RP_ERR_TIMEOUT, "a device-side wait exceeded its limit; the call was undone");
        }
        w->status_accum |= bits;
        break;
    }
    w->steps += nsteps;
    w->substeps += (uint64_t)nsteps * substeps;
    for (HostBody& b : w->bodies)
        if (!b.forces.empty()) { b.forces.clear(); w->forces_dirty = true; }
    return RP_OK;
}

rp_status rp_sync(rp_world* w) {
    if (check_world(w)) return RP_ERR_INVALID;
    if (w->device < 0) return fail(RP_ERR_NO_DEVICE, "host-only world");
    RP_CUDA(cudaStreamSynchronize(w->stream));
    return RP_OK;
}

rp_status rp_last_status(rp_world* w, uint32_t* bits) {
    if (check_world(w) || !bits) return RP_ERR_INVALID;
    *bits = w->status_accum;
    w->status_accum = 0;
    return RP_OK;
}

rp_status rp_state_get(rp_world* w, double* out) {
    if (check_world(w) || (!out && !w->bodies.empty())) return fail(RP_ERR_INVALID, "null argument");
    const size_t n = w->bodies.size();
    if (w->device_state_valid && !w->static_dirty && n && w->d_slot_entity.p) {
        // the device holds the state: pack the records there, one copy back, a parallel host copy
        const size_t bytes = n * RP_STATE_DOUBLES * sizeof(double);
        RP_CUDA(cudaSetDevice(w->device));
        if (w->ev_rec) RP_CUDA(cudaEventSynchronize(w->ev_rec));
        RP_CUDA(w->d_rec.ensure(bytes));
        RP_CUDA(w->h_rec.ensure(bytes));
        if (w->precision == RP_PRECISION_FP64)
            RP_CUDA(state_io_f64(make_view<double>(w), w->d_rec.as<double>(), w->d_slot_entity.as<int32_t>(), (int)n, true, w->stream));
        else
            RP_CUDA(state_io_f32(make_view<float>(w), w->d_rec.as<double>(), w->d_slot_entity.as<int32_t>(), (int)n, true, w->stream));
        w->launches++;
        RP_CUDA(cudaMemcpyAsync(w->h_rec.p, w->d_rec.p, bytes, cudaMemcpyDeviceToHost, w->stream));
        RP_CUDA(cudaStreamSynchronize(w->stream));
        w->d2h_bytes += bytes;
        copy_records(out, (const double*)w->h_rec.p, n * RP_STATE_DOUBLES, false);
        return RP_OK;
    }
    if (w->device_state_valid) {
        rp_status s = sync_state_to_host(w);
        if (s != RP_OK) return s;
    }
    for (size_t e = 0; e < w->bodies.size(); ++e) {
        const HostBody& b = w->bodies[e];
        double* o = out + e * RP_STATE_DOUBLES;
        for (int k = 0; k < 3; ++k) { o[k] = b.pos[k]; o[7 + k] = b.v[k]; o[10 + k] = b.w[k]; o[13 + k] = b.ppos[k]; o[20 + k] = b.pv[k]; o[23 + k] = b.pw[k]; }
        for (int k = 0; k < 4; ++k) { o[3 + k] = b.rot[k]; o[16 + k] = b.prot[k]; }
        o[26] = b.active;
        o[27] = b.deact;
    }
    return RP_OK;
}

rp_status rp_state_set(rp_world* w, const double* in) {
    if (check_world(w) || (!in && !w->bodies.empty())) return fail(RP_ERR_INVALID, "null argument");
    const size_t n = w->bodies.size();
    if (w->device >= 0 && !w->static_dirty && n && w->d_slot_entity.p && w->d_pos.p) {
        // a built world: the records go to the device as they are and are unpacked there; the
        // device then holds the state (the host mirror is refreshed from it when needed)
        const size_t bytes = n * RP_STATE_DOUBLES * sizeof(double);
        RP_CUDA(cudaSetDevice(w->device));
        if (w->ev_rec) RP_CUDA(cudaEventSynchronize(w->ev_rec));
        RP_CUDA(w->h_rec.ensure(bytes));
        RP_CUDA(w->d_rec.ensure(bytes));
        if (!copy_records((double*)w->h_rec.p, in, n * RP_STATE_DOUBLES, true))
            return fail(RP_ERR_INVALID, "state is not finite");
        RP_CUDA(cudaMemcpyAsync(w->d_rec.p, w->h_rec.p, bytes, cudaMemcpyHostToDevice, w->stream));
        if (!w->ev_rec) RP_CUDA(cudaEventCreateWithFlags(&w->ev_rec, cudaEventDisableTiming));
        RP_CUDA(cudaEventRecord(w->ev_rec, w->stream));
        if (w->precision == RP_PRECISION_FP64)
            RP_CUDA(state_io_f64(make_view<double>(w), w->d_rec.as<double>(), w->d_slot_entity.as<int32_t>(), (int)n, false, w->stream));
        else
            RP_CUDA(state_io_f32(make_view<float>(w), w->d_rec.as<double>(), w->d_slot_entity.as<int32_t>(), (int)n, false, w->stream));
        w->launches++;
        w->h2d_bytes += bytes;
        w->device_state_valid = true;
        return RP_OK;
    }
    for (size_t e = 0; e < w->bodies.size(); ++e) {
        const double* o = in + e * RP_STATE_DOUBLES;
        for (int k = 0; k < RP_STATE_DOUBLES; ++k)
            if (!std::isfinite(o[k])) return fail(RP_ERR_INVALID, "state is not finite");
    }
    for (size_t e = 0; e < w->bodies.size(); ++e) {
        HostBody& b = w->bodies[e];
        const double* o = in + e * RP_STATE_DOUBLES;
        for (int k = 0; k < 3; ++k) { b.pos[k] = o[k]; b.v[k] = o[7 + k]; b.w[k] = o[10 + k]; b.ppos[k] = o[13 + k]; b.pv[k] = o[20 + k]; b.pw[k] = o[23 + k]; }
        for (int k = 0; k < 4; ++k) { b.rot[k] = o[3 + k]; b.prot[k] = o[16 + k]; }
        b.active = o[26] != 0.0 ? 1.0 : 0.0;
        b.deact = o[27];
    }
    w->device_state_valid = false;
    if (!w->static_dirty) return upload_state(w);
    return RP_OK;
}

rp_status rp_broad_pairs(rp_world* w, int32_t scene, uint32_t* out, uint32_t cap, uint32_t* count) {
    if (check_world(w) || scene < 0 || scene >= w->num_scenes || (!out && cap)) return fail(RP_ERR_INVALID, "bad argument");
    if (w->device < 0) return fail(RP_ERR_NO_DEVICE, "host-only world");
    RP_CUDA(cudaSetDevice(w->device));
    rp_status s = ensure_device(w);
    if (s != RP_OK) return s;
    // the step's own broad phase for this world: the grid (sort-based) for one large scene
    const int gb = w->grid_mode ? w->num_sms : 0;
    if (w->precision == RP_PRECISION_FP64) RP_CUDA(broad_f64(make_view<double>(w), scene, gb, w->stream));
    else RP_CUDA(broad_f32(make_view<float>(w), scene, gb, w->stream));
    w->launches++;
    {
        cudaError_t e;
        const uint32_t bits = read_status(w, e);
        if (e != cudaSuccess) return fail(RP_ERR_CUDA, cudaGetErrorString(e));
        if (bits & ST_BARRIER_TIMEOUT) return fail(RP_ERR_TIMEOUT, "a device-side wait of the broad phase exceeded its limit");
    }
    int32_t n = 0;
    RP_CUDA(cudaMemcpyAsync(&n, w->d_pair_count.as<int32_t>() + scene, 4, cudaMemcpyDeviceToHost, w->stream));
    RP_CUDA(cudaStreamSynchronize(w->stream));
    int32_t pc = w->scene_pair_cap[(size_t)scene + 1] - w->scene_pair_cap[(size_t)scene];
    if (count) *count = (uint32_t)n;
    if (n > pc) return fail(RP_ERR_CAPACITY, "more pairs than the scratch holds");
    std::vector<int2> pr((size_t)n);
    if (n) RP_CUDA(cudaMemcpyAsync(pr.data(), w->d_pairs.as<int2>() + w->scene_pair_cap[(size_t)scene], (size_t)n * 8,
                                   cudaMemcpyDeviceToHost, w->stream));
    RP_CUDA(cudaStreamSynchronize(w->stream));
    for (int32_t k = 0; k < n && (uint32_t)k < cap; ++k) {
        out[2 * k] = (uint32_t)w->slot_to_entity[(size_t)pr[(size_t)k].x];
        out[2 * k + 1] = (uint32_t)w->slot_to_entity[(size_t)pr[(size_t)k].y];
    }
    return RP_OK;
}

rp_status rp_contacts(rp_world* w, int32_t e1, int32_t e2, double* out, uint32_t cap, uint32_t* count) {
    if (check_world(w) || e1 < 0 || e2 < 0 || e1 >= (int32_t)w->bodies.size() || e2 >= (int32_t)w->bodies.size() || e1 == e2)
        return fail(RP_ERR_INVALID, "bad entity");
    if (w->device < 0) return fail(RP_ERR_NO_DEVICE, "host-only world");
    RP_CUDA(cudaSetDevice(w->device));
    rp_status s = ensure_device(w);
    if (s != RP_OK) return s;
    const int kcap = 64;
    RP_CUDA(w->d_kat_out.ensure((size_t)kcap * 9 * 8));
    RP_CUDA(w->d_kat_count.ensure(4));
    int a = w->bodies[(size_t)e1].slot, b = w->bodies[(size_t)e2].slot;
    if (w->precision == RP_PRECISION_FP64)
        RP_CUDA(contacts_f64(make_view<double>(w), a, b, w->d_kat_out.as<double>(), kcap, w->d_kat_count.as<int>(), w->stream));
    else
        RP_CUDA(contacts_f32(make_view<float>(w), a, b, w->d_kat_out.as<double>(), kcap, w->d_kat_count.as<int>(), w->stream));
    w->launches++;
    int n = 0;
    std::vector<double> buf((size_t)kcap * 9);
    RP_CUDA(cudaMemcpyAsync(&n, w->d_kat_count.p, 4, cudaMemcpyDeviceToHost, w->stream));
    RP_CUDA(cudaMemcpyAsync(buf.data(), w->d_kat_out.p, buf.size() * 8, cudaMemcpyDeviceToHost, w->stream));
    RP_CUDA(cudaStreamSynchronize(w->stream));
    if (count) *count = (uint32_t)n;
    for (int k = 0; k < n && (uint32_t)k < cap && k < kcap; ++k)
        for (int j = 0; j < 9; ++j) out[9 * k + j] = buf[(size_t)(9 * k + j)];
    return RP_OK;
}

rp_status rp_contacts_noalloc(rp_world* w, int32_t e1, int32_t e2, double* out, uint32_t cap, uint32_t* count) {
    if (check_world(w) || e1 < 0 || e2 < 0 || e1 >= (int32_t)w->bodies.size() || e2 >= (int32_t)w->bodies.size() || e1 == e2)
        return fail(RP_ERR_INVALID, "bad entity");
    if (!out || !count) return fail(RP_ERR_INVALID, "null argument");
    if (cap > (uint32_t)NOALLOC_MAX_CONTACTS)
        return fail(RP_ERR_CAPACITY, "rp_contacts_noalloc: cap exceeds the static scratch (64 contacts per call)");
    if (w->device < 0) return fail(RP_ERR_NO_DEVICE, "host-only world");
    if (w->static_dirty || !w->d_pos.p)
        return fail(RP_ERR_STATE, "rp_contacts_noalloc: the device world is not built (new entities, constraints or "
                                  "hulls since the last step); step the world (rp_simulate) first");
    RP_CUDA(cudaSetDevice(w->device));
    if (!w->device_state_valid) {
        // host-side edits since the last step: re-upload them through the existing pinned staging
        // buffer (no allocation); a staging buffer too small would need one, so that case is refused
        const StateLayout L(w->bodies.size(), w->rsize());
        if (!w->h_state.p || w->h_state.bytes < L.total)
            return fail(RP_ERR_STATE, "rp_contacts_noalloc: host-side edits since the last step need a step first");
        rp_status s = upload_state(w);
        if (s != RP_OK) return s;
    }
    double* scratch = nullptr;
    int* d_count = nullptr;
    RP_CUDA(noalloc_scratch(w->device, &scratch, &d_count));
    const int a = w->bodies[(size_t)e1].slot, b = w->bodies[(size_t)e2].slot;
    if (w->precision == RP_PRECISION_FP64)
        RP_CUDA(contacts_f64(make_view<double>(w), a, b, scratch, NOALLOC_MAX_CONTACTS, d_count, w->stream));
    else
        RP_CUDA(contacts_f32(make_view<float>(w), a, b, scratch, NOALLOC_MAX_CONTACTS, d_count, w->stream));
    w->launches++;
    int n = 0;
    RP_CUDA(cudaMemcpyAsync(&n, d_count, sizeof(int), cudaMemcpyDeviceToHost, w->stream));
    RP_CUDA(cudaStreamSynchronize(w->stream));
    const int m = std::min(std::min(n, NOALLOC_MAX_CONTACTS), (int)cap);
    if (m > 0) {
        RP_CUDA(cudaMemcpyAsync(out, scratch, (size_t)m * 9 * sizeof(double), cudaMemcpyDeviceToHost, w->stream));
        RP_CUDA(cudaStreamSynchronize(w->stream));
    }
    *count = (uint32_t)n;
    return RP_OK;
}

rp_status rp_last_contacts(rp_world* w, int32_t scene, int32_t* pairs_out, double* out, uint32_t cap, uint32_t* count) {
    if (check_world(w) || scene < 0 || scene >= w->num_scenes) return fail(RP_ERR_INVALID, "bad argument");
    if (w->device < 0 || !w->d_pair_count.p || w->static_dirty) return fail(RP_ERR_STATE, "no step has run");
    int32_t np = 0;
    RP_CUDA(cudaMemcpyAsync(&np, w->d_pair_count.as<int32_t>() + scene, 4, cudaMemcpyDeviceToHost, w->stream));
    RP_CUDA(cudaStreamSynchronize(w->stream));
    const int32_t pbase = w->scene_pair_cap[(size_t)scene], cbase = w->scene_contact_cap[(size_t)scene];
    np = std::min(np, w->scene_pair_cap[(size_t)scene + 1] - pbase);
    std::vector<int2> pr((size_t)np);
    std::vector<int32_t> cs((size_t)np), cc((size_t)np);
    const int32_t ncap = w->scene_contact_cap[(size_t)scene + 1] - cbase;
    const size_t R = w->rsize();
    std::vector<unsigned char> con((size_t)ncap * 12 * R);
    if (np) {
        RP_CUDA(cudaMemcpyAsync(pr.data(), w->d_pairs.as<int2>() + pbase, (size_t)np * 8, cudaMemcpyDeviceToHost, w->stream));
        RP_CUDA(cudaMemcpyAsync(cs.data(), w->d_pair_cstart.as<int32_t>() + pbase, (size_t)np * 4, cudaMemcpyDeviceToHost, w->stream));
        RP_CUDA(cudaMemcpyAsync(cc.data(), w->d_pair_ccount.as<int32_t>() + pbase, (size_t)np * 4, cudaMemcpyDeviceToHost, w->stream));
        RP_CUDA(cudaMemcpyAsync(con.data(), (char*)w->d_contacts.p + (size_t)cbase * 12 * R, con.size(), cudaMemcpyDeviceToHost, w->stream));
    }
    RP_CUDA(cudaStreamSynchronize(w->stream));
    uint32_t k = 0;
    const int map[11] = {0, 1, 2, 4, 5, 6, 8, 9, 10, 3, 7};
    for (int32_t p = 0; p < np; ++p) {
        for (int32_t c = 0; c < cc[(size_t)p]; ++c, ++k) {
            if (k >= cap) continue;
            size_t base = (size_t)(cs[(size_t)p] + c) * 12;
            pairs_out[2 * k] = w->slot_to_entity[(size_t)pr[(size_t)p].x];
            pairs_out[2 * k + 1] = w->slot_to_entity[(size_t)pr[(size_t)p].y];
            for (int j = 0; j < 11; ++j) {
                size_t at = base + (size_t)map[j];
                if (R == 8) std::memcpy(&out[11 * k + j], &con[at * 8], 8);
                else { float f; std::memcpy(&f, &con[at * 4], 4); out[11 * k + j] = f; }
            }
        }
    }
    if (count) *count = k;
    return RP_OK;
}

rp_status rp_counters(rp_world* w, uint64_t out[RP_NUM_COUNTERS]) {
    if (check_world(w) || !out) return RP_ERR_INVALID;
    for (int k = 0; k < RP_NUM_COUNTERS; ++k) out[k] = 0;
    if (w->d_counters.p) {
        unsigned long long c[32];
        RP_CUDA(cudaMemcpyAsync(c, w->d_counters.p, sizeof(c), cudaMemcpyDeviceToHost, w->stream));
        int32_t cc = 0, pc = 0, lv = 0;
        if (w->d_contact_count.p) RP_CUDA(cudaMemcpyAsync(&cc, w->d_contact_count.p, 4, cudaMemcpyDeviceToHost, w->stream));
        if (w->d_pair_count.p) RP_CUDA(cudaMemcpyAsync(&pc, w->d_pair_count.p, 4, cudaMemcpyDeviceToHost, w->stream));
        if (w->d_scene_levels.p) RP_CUDA(cudaMemcpyAsync(&lv, w->d_scene_levels.p, 4, cudaMemcpyDeviceToHost, w->stream));
        RP_CUDA(cudaStreamSynchronize(w->stream));
        (void)cc; (void)pc; (void)lv;
        out[0] = c[0]; out[1] = c[1]; out[2] = c[2];
        out[5] = c[3]; out[6] = c[5]; out[7] = c[6];
        out[8] = c[4]; out[9] = c[7]; out[10] = c[8]; out[11] = c[9]; out[12] = c[10]; out[13] = c[11];
        out[14] = c[12]; out[15] = c[13]; out[16] = c[14]; out[17] = c[15]; out[18] = c[16];
        out[19] = c[17]; out[20] = c[18]; out[21] = c[19]; out[22] = c[20];
        out[23] = c[23];
    }
    out[3] = w->steps;
    out[4] = w->substeps;
    return RP_OK;
}

uint64_t rp_kernel_launches(const rp_world* w) { return w ? w->launches : 0; }

rp_status rp_phase_times(rp_world* w, double out[RP_NUM_PHASES]) {
    if (check_world(w) || !out) return RP_ERR_INVALID;
    for (int k = 0; k < PHASES; ++k) out[k] = 0.0;
    for (int k = 0; k < PHASES; ++k) out[k] = w->phase_ms[k];
    if (!w->d_phase.p) return RP_OK;
    unsigned long long ns[PHASES];
    RP_CUDA(cudaMemcpyAsync(ns, w->d_phase.p, sizeof(ns), cudaMemcpyDeviceToHost, w->stream));
    RP_CUDA(cudaStreamSynchronize(w->stream));
    for (int k = 0; k < PHASES; ++k) out[k] += (double)ns[k] * 1e-6;
    return RP_OK;
}

rp_status rp_transfer_bytes(rp_world* w, uint64_t out[2]) {
    if (check_world(w) || !out) return RP_ERR_INVALID;
    out[0] = w->h2d_bytes;
    out[1] = w->d2h_bytes;
    return RP_OK;
}

rp_status rp_set_timing(rp_world* w, int32_t enabled) {
    if (check_world(w)) return RP_ERR_INVALID;
    w->timing = enabled != 0;
    return RP_OK;
}

rp_status rp_autotune(rp_world* w, double dt, uint32_t substeps, uint32_t iters, int32_t collisions, uint32_t frames,
                      int32_t choice[4]) {
    if (check_world(w) || !choice) return RP_ERR_INVALID;
    if (w->device < 0) return fail(RP_ERR_NO_DEVICE, "host-only world");
    if (!(dt > 0.0) || substeps == 0 || frames == 0) return fail(RP_ERR_INVALID, "bad step arguments");
    for (const HostBody& b : w->bodies)
        if (!b.forces.empty()) return fail(RP_ERR_STATE, "autotune runs before forces are added for the next frame");
    if (w->bodies.empty()) return RP_OK;
    // trials run from the same state, which is restored at the end; results do not depend on the choice
    const size_t n = w->bodies.size();
    std::vector<double> saved(n * RP_STATE_DOUBLES);
    rp_status s = rp_state_get(w, saved.data());
    if (s != RP_OK) return s;
    const uint64_t steps0 = w->steps, substeps0 = w->substeps;
    const uint32_t status0 = w->status_accum;
    cudaEvent_t e0, e1;
    RP_CUDA(cudaEventCreate(&e0));
    RP_CUDA(cudaEventCreate(&e1));
    auto trial = [&](float& ms) -> rp_status {
        rp_status r = rp_state_set(w, saved.data());
        if (r == RP_OK) r = rp_simulate(w, dt, substeps, iters, collisions, 1);   // warm-up, graph capture
        if (r != RP_OK) return r;
        if (cudaEventRecord(e0, w->stream) != cudaSuccess) return fail(RP_ERR_CUDA, "event");
        r = rp_simulate(w, dt, substeps, iters, collisions, frames);
        if (r != RP_OK) return r;
        if (cudaEventRecord(e1, w->stream) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
            cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess)
            return fail(RP_ERR_CUDA, "event timing");
        return RP_OK;
    };
    // cta: how a batch's sweeps assign scenes: 1 = one CTA per scene (k_sweep_cta); 0 = one warp per
    // scene; n >= 2 = scenes of sweep cost n or more get a whole CTA, the rest a warp each
    auto set_tune = [&](int mode, int group, int cta, int solo) {
        w->mode = mode;
        w->pipe.transform_group = group;
        w->pipe.sweep_cta = cta == 1 ? 1 : 0;
        w->cta_from = cta == 1 ? 0 : cta;
        set_cta_scenes(w);
        w->solo_nodes = solo;
        w->layout_gen++;   // recapture the frame graph with the new launch shapes
    };
    const int cta0 = w->pipe.sweep_cta ? 1 : w->cta_from;
    int best[4] = {RP_MODE_PHASED, 4, cta0, 512};
    float best_ms = 0.f;
    // each candidate timed twice (the faster run counts); a later candidate replaces the best only
    // when it is at least 1 % faster, so timing noise does not move the choice off the default
    auto consider = [&](int mode, int group, int cta, int solo) -> rp_status {
        set_tune(mode, group, cta, solo);
        float ms = 0.f, ms2 = 0.f;
        rp_status r = trial(ms);
        if (r == RP_OK) r = trial(ms2);
        if (r != RP_OK) return r;
        ms = std::min(ms, ms2);
        if (best_ms == 0.f || ms < 0.99f * best_ms) {
            best_ms = ms;
            best[0] = mode; best[1] = group; best[2] = cta; best[3] = solo;
        }
        return RP_OK;
    };
    // coordinate search: launch mode, then the hull-transform group, then the sweep layout
    s = consider(RP_MODE_PHASED, 4, cta0, 512);
    if (s == RP_OK) s = consider(RP_MODE_PERSISTENT, 4, cta0, 512);
    if (s == RP_OK && best[0] == RP_MODE_PHASED) {
        for (int g : {8, 16, 32})
            if (s == RP_OK) s = consider(RP_MODE_PHASED, g, cta0, 512);
        const int g = best[1];
        if (w->grid_mode) {
            for (int solo : {128, 256, 1024, 2048})
                if (s == RP_OK) s = consider(RP_MODE_PHASED, g, cta0, solo);
        } else {
            // the sweeps' scene assignment: every scene a warp, every scene a CTA, or the largest a CTA
            for (int cta : {0, 1, 96, 160, 256, 384})
                if (s == RP_OK && cta != cta0) s = consider(RP_MODE_PHASED, g, cta, 512);
        }
    } else if (s == RP_OK && w->grid_mode) {
        for (int solo : {128, 256, 1024, 2048})
            if (s == RP_OK) s = consider(RP_MODE_PERSISTENT, 4, 0, solo);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    set_tune(best[0], best[1], best[2], best[3]);
    rp_status r = rp_state_set(w, saved.data());
    w->steps = steps0;
    w->substeps = substeps0;
    w->status_accum = status0;
    for (int k = 0; k < 4; ++k) choice[k] = best[k];
    return s != RP_OK ? s : r;
}

rp_status rp_adjoint_trajectory(rp_world* w, double dt, uint32_t substeps, uint32_t iters, int32_t collisions,
                                uint32_t frames, uint32_t checkpoint_every, const int32_t* loss_entity, const double* target,
                                double* loss_out, double* grad_v, double* grad_w, double* grad_mass, double* grad_friction) {
    if (check_world(w) || !loss_entity || !target || !loss_out || !grad_v || !grad_w || !grad_mass)
        return fail(RP_ERR_INVALID, "null argument");
    if (!(dt > 0.0) || substeps == 0 || iters == 0 || frames == 0 || checkpoint_every == 0)
        return fail(RP_ERR_INVALID, "bad step arguments");
    const int S = w->num_scenes;
    for (int s = 0; s < S; ++s) {
        const int e = loss_entity[s];
        if (e < 0 || e >= (int)w->bodies.size() || w->bodies[(size_t)e].scene != s)
            return fail(RP_ERR_INVALID, "loss entity must belong to its scene");
    }
    for (const HostBody& b : w->bodies)
        if (!b.forces.empty()) return fail(RP_ERR_STATE, "the adjoint covers gravity only: clear the pending forces");
    if (w->device < 0) return fail(RP_ERR_NO_DEVICE, "host-only world");
    RP_CUDA(cudaSetDevice(w->device));
    rp_status st = ensure_device(w);   // slots, the scene layout and the geometry
    if (st != RP_OK) return st;
    if (w->device_state_valid) {
        st = sync_state_to_host(w);
        if (st != RP_OK) return st;
    }
    // host copies by slot: start states, mass properties, materials, sleeping state
    const size_t N = w->bodies.size();
    std::vector<double> start(13 * N), invm(N), I6(6 * N), Ii6(6 * N), mat(3 * N), pvel(6 * N), deact(N);
    std::vector<uint8_t> fixedv(N), activev(N);
    std::vector<int> tv_of(N + 1, 0), tn_of(N + 1, 0);   // transformed vertices / normals before each slot
    const int sym[6] = {0, 4, 8, 1, 2, 5};
    for (size_t slot = 0; slot < N; ++slot) {
        const HostBody& b = w->bodies[(size_t)w->slot_to_entity[slot]];
        double* o = &start[13 * slot];
        for (int k = 0; k < 3; ++k) { o[k] = b.pos[k]; o[7 + k] = b.v[k]; o[10 + k] = b.w[k]; }
        for (int k = 0; k < 4; ++k) o[3 + k] = b.rot[k];
        invm[slot] = b.invm;
        for (int k = 0; k < 6; ++k) { I6[6 * slot + (size_t)k] = b.I[sym[k]]; Ii6[6 * slot + (size_t)k] = b.Iinv[sym[k]]; }
        mat[3 * slot] = b.mus;
        mat[3 * slot + 1] = b.mud;
        mat[3 * slot + 2] = b.rest;
        for (int k = 0; k < 3; ++k) { pvel[6 * slot + (size_t)k] = b.pv[k]; pvel[6 * slot + 3 + (size_t)k] = b.pw[k]; }
        deact[slot] = b.deact;
        activev[slot] = b.active != 0.0 ? 1 : 0;
        fixedv[slot] = (uint8_t)b.fixed;
        int nv = 0, nf = 0;
        for (const rp_collider_desc& d : b.cols) {
            if (d.type != RP_COLLIDER_HULL) continue;
            nv += w->hulls[(size_t)d.hull]->nv();
            nf += w->hulls[(size_t)d.hull]->nf();
        }
        tv_of[slot + 1] = tv_of[slot] + nv;
        tn_of[slot + 1] = tn_of[slot] + nf;
    }
    std::vector<ExtConstraint> ext;
    std::vector<int> ext_start((size_t)S + 1, 0);
    for (int s = 0; s < S; ++s) {
        ext_start[(size_t)s] = (int)ext.size();
        for (const HostExt& x : w->exts) {
            if (x.scene != s) continue;
            ExtConstraint c = x.c;
            c.e1 = w->bodies[(size_t)c.e1].slot;
            c.e2 = w->bodies[(size_t)c.e2].slot;
            for (int k = 0; k < 3; ++k) { c.r1f[k] = (float)c.r1[k]; c.r2f[k] = (float)c.r2[k]; }
            c.compliance_f = (float)c.compliance;
            ext.push_back(c);
        }
    }
    ext_start[(size_t)S] = (int)ext.size();
    const size_t K = checkpoint_every;
    const size_t body_d = adjoint_body_bytes(false), body_a = adjoint_body_bytes(true), var = adjoint_var_bytes();
    const size_t con_d = adjoint_contact_bytes(false), con_a = adjoint_contact_bytes(true);
    const size_t clip_d = adjoint_clip_bytes(false), clip_a = adjoint_clip_bytes(true), epa = adjoint_epa_bytes();
    struct Off {
        size_t ckpt, seg, work, deact, active, aseg, pairs, npairs, uf, awake, stamp, tvd, tnd, tva, tna, tvv, tnv, cond, cona,
            clipd, clipa, epa, grad, ginv, gmu, loss, status, prof, bd, ba, lamd, lama, tab, td, tadj;
        int cap, pcap, ccap;
    };
    std::vector<Off> off((size_t)S);
    // the tape of one substep: bodies, joints, and with collisions the hull transforms, narrowphase
    // and contact solves; an overflow doubles it and runs again
    size_t tape_scale = 1;
    rp_status result = RP_OK;
    for (int attempt = 0; attempt < 3; ++attempt) {
        size_t total = 0;
        auto take = [&](size_t bytes) { size_t o = total; total += (bytes + 255) & ~(size_t)255; return o; };
        for (int s = 0; s < S; ++s) {
            const int b0 = w->scene_body[(size_t)s];
            const size_t nb = (size_t)(w->scene_body[(size_t)s + 1] - b0);
            const size_t ne = (size_t)(ext_start[(size_t)s + 1] - ext_start[(size_t)s]);
            const size_t ntv = (size_t)(tv_of[(size_t)b0 + nb] - tv_of[(size_t)b0]);
            const size_t ntn = (size_t)(tn_of[(size_t)b0 + nb] - tn_of[(size_t)b0]);
            const size_t stride = 13 * nb * 8;
            Off& o = off[(size_t)s];
            o.pcap = (int)std::min<size_t>(nb * (nb - 1) / 2 + 1, 16 * nb + 64);
            o.ccap = collisions ? (int)(32 * nb + 256) : 1;
            const size_t cap = (600 * nb + 2500 * ne * iters + (collisions ? 8000 * nb * iters : 0) + 4096) * tape_scale;
            o.cap = (int)std::min<size_t>((size_t)1 << 30, cap);
            o.ckpt = take(((frames + K - 1) / K + 1) * 15 * nb * 8);
            o.seg = take((K * substeps + 1) * stride);
            o.work = take(stride);
            o.deact = take(nb * 8);
            o.active = take(nb);
            o.aseg = take(K * nb);
            o.pairs = take(K * (size_t)o.pcap * 8);
            o.npairs = take(K * 4);
            o.uf = take(nb * 4);
            o.awake = take(nb);
            o.stamp = take(nb * 4);
            o.tvd = take(ntv * 24 + 8);
            o.tnd = take(ntn * 24 + 8);
            o.tva = take(ntv * 3 * var + var);
            o.tna = take(ntn * 3 * var + var);
            o.tvv = take(ntv * 24 + 8);
            o.tnv = take(ntn * 24 + 8);
            o.cond = take((size_t)o.ccap * con_d);
            o.cona = take((size_t)o.ccap * con_a);
            o.clipd = take(collisions ? clip_d : 8);
            o.clipa = take(collisions ? clip_a : 8);
            o.epa = take(collisions ? epa : 8);
            o.grad = take(stride);
            o.ginv = take(nb * 8);
            o.gmu = take(2 * nb * 8);
            o.loss = take(8);
            o.status = take(8);
            o.prof = take(6 * 8);
            o.bd = take(nb * body_d);
            o.ba = take(nb * body_a);
            o.lamd = take(4 * ne * 8 + 8);
            o.lama = take(4 * ne * var + var);
            o.tab = take((size_t)o.cap * 8);
            o.td = take((size_t)o.cap * 16);
            o.tadj = take((size_t)o.cap * 8);
        }
        const size_t inputs = (13 + 1 + 12 + 3 + 6 + 1) * N * 8 + 2 * N + 256;
        RP_CUDA(w->d_adj_data.ensure(total + inputs + 1024));
        RP_CUDA(w->d_adj_ext.ensure(std::max<size_t>(ext.size(), 1) * sizeof(ExtConstraint)));
        RP_CUDA(w->d_adj_scenes.ensure((size_t)S * sizeof(AdjointScene)));
        char* base = (char*)w->d_adj_data.p;
        char* in = base + total;
        double* d_start = (double*)in;
        double* d_invm = d_start + 13 * N;
        double* d_I = d_invm + N;
        double* d_Ii = d_I + 6 * N;
        double* d_mat = d_Ii + 6 * N;
        double* d_pvel = d_mat + 3 * N;
        double* d_deact = d_pvel + 6 * N;
        uint8_t* d_fixed = (uint8_t*)(d_deact + N);
        uint8_t* d_active = d_fixed + N;
        RP_CUDA(cudaMemcpyAsync(d_start, start.data(), start.size() * 8, cudaMemcpyHostToDevice, w->stream));
        RP_CUDA(cudaMemcpyAsync(d_invm, invm.data(), N * 8, cudaMemcpyHostToDevice, w->stream));
        RP_CUDA(cudaMemcpyAsync(d_I, I6.data(), I6.size() * 8, cudaMemcpyHostToDevice, w->stream));
        RP_CUDA(cudaMemcpyAsync(d_Ii, Ii6.data(), Ii6.size() * 8, cudaMemcpyHostToDevice, w->stream));
        RP_CUDA(cudaMemcpyAsync(d_mat, mat.data(), mat.size() * 8, cudaMemcpyHostToDevice, w->stream));
        RP_CUDA(cudaMemcpyAsync(d_pvel, pvel.data(), pvel.size() * 8, cudaMemcpyHostToDevice, w->stream));
        RP_CUDA(cudaMemcpyAsync(d_deact, deact.data(), N * 8, cudaMemcpyHostToDevice, w->stream));
        RP_CUDA(cudaMemcpyAsync(d_fixed, fixedv.data(), N, cudaMemcpyHostToDevice, w->stream));
        RP_CUDA(cudaMemcpyAsync(d_active, activev.data(), N, cudaMemcpyHostToDevice, w->stream));
        if (!ext.empty())
            RP_CUDA(cudaMemcpyAsync(w->d_adj_ext.p, ext.data(), ext.size() * sizeof(ExtConstraint), cudaMemcpyHostToDevice,
                                    w->stream));
        std::vector<AdjointScene> scenes((size_t)S);
        for (int s = 0; s < S; ++s) {
            AdjointScene& a = scenes[(size_t)s];
            const Off& o = off[(size_t)s];
            const int b0 = w->scene_body[(size_t)s];
            a.nb = w->scene_body[(size_t)s + 1] - b0;
            a.ne = ext_start[(size_t)s + 1] - ext_start[(size_t)s];
            a.body0 = b0;
            a.ext = w->d_adj_ext.as<ExtConstraint>() + ext_start[(size_t)s];
            a.start = d_start + 13 * (size_t)b0;
            a.invm = d_invm + b0;
            a.inertia = d_I + 6 * (size_t)b0;
            a.inv_inertia = d_Ii + 6 * (size_t)b0;
            a.material = d_mat + 3 * (size_t)b0;
            a.prev_vel = d_pvel + 6 * (size_t)b0;
            a.deact0 = d_deact + b0;
            a.active0 = d_active + b0;
            a.fixed = d_fixed + b0;
            a.loss_body = w->bodies[(size_t)loss_entity[s]].slot - b0;
            for (int k = 0; k < 3; ++k) a.target[k] = target[3 * s + k];
            a.tv0 = tv_of[(size_t)b0];
            a.tn0 = tn_of[(size_t)b0];
            a.ntv = tv_of[(size_t)b0 + (size_t)a.nb] - a.tv0;
            a.ntn = tn_of[(size_t)b0 + (size_t)a.nb] - a.tn0;
            a.pair_cap = o.pcap;
            a.contact_cap = o.ccap;
            a.checkpoints = (double*)(base + o.ckpt);
            a.segment = (double*)(base + o.seg);
            a.work = (double*)(base + o.work);
            a.deact = (double*)(base + o.deact);
            a.active = (uint8_t*)(base + o.active);
            a.active_seg = (uint8_t*)(base + o.aseg);
            a.pairs = (int2*)(base + o.pairs);
            a.npairs = (int*)(base + o.npairs);
            a.uf = (int*)(base + o.uf);
            a.awake = (uint8_t*)(base + o.awake);
            a.stamp = (int*)(base + o.stamp);
            a.tv_d = base + o.tvd;
            a.tn_d = base + o.tnd;
            a.tv_a = base + o.tva;
            a.tn_a = base + o.tna;
            a.tv_val = (double*)(base + o.tvv);
            a.tn_val = (double*)(base + o.tnv);
            a.con_d = base + o.cond;
            a.con_a = base + o.cona;
            a.clip_d = base + o.clipd;
            a.clip_a = base + o.clipa;
            a.epa = base + o.epa;
            a.grad_state = (double*)(base + o.grad);
            a.grad_invm = (double*)(base + o.ginv);
            a.grad_mu = (double*)(base + o.gmu);
            a.loss = (double*)(base + o.loss);
            a.status = (int*)(base + o.status);
            a.prof = (long long*)(base + o.prof);
            a.bodies_d = base + o.bd;
            a.bodies_a = base + o.ba;
            a.lam_d = (double*)(base + o.lamd);
            a.lam_a = base + o.lama;
            a.tape_ab = (int2*)(base + o.tab);
            a.tape_d = (double2*)(base + o.td);
            a.tape_adj = (double*)(base + o.tadj);
            a.tape_cap = o.cap;
        }
        RP_CUDA(cudaMemcpyAsync(w->d_adj_scenes.p, scenes.data(), scenes.size() * sizeof(AdjointScene),
                                cudaMemcpyHostToDevice, w->stream));
        AdjointParams P;
        P.dt = dt;
        P.gravity = w->gravity;
        P.substeps = (int)substeps;
        P.pos_iters = (int)iters;
        P.frames = (int)frames;
        P.checkpoint_every = (int)checkpoint_every;
        P.collisions = collisions ? 1 : 0;
        P.geom.colliders = w->d_colliders.as<Collider>();
        P.geom.shapes = w->d_shapes.as<Shape>();
        P.geom.shape_verts = w->d_shape_verts.as<double>();
        P.geom.face_normal = w->d_face_normal.as<double>();
        P.geom.face_elem_start = w->d_face_elem_start.as<int32_t>();
        P.geom.face_elem = w->d_face_elem.as<int32_t>();
        P.geom.csr_start = w->d_csr_start.as<int32_t>();
        P.geom.csr_data = w->d_csr_data.as<int32_t>();
        P.geom.col_start = w->d_col_start.as<int32_t>();
        P.geom.radius = w->d_radius.as<double>();
        RP_CUDA(adjoint_launch(w->d_adj_scenes.as<AdjointScene>(), S, P, w->stream));
        w->launches++;
        // results
        std::vector<double> g(13 * N), gi(N), gmu(2 * N);
        std::vector<int> status((size_t)S, 0);
        std::vector<long long> prof(6 * (size_t)S, 0);
        for (int s = 0; s < S; ++s) {
            const Off& o = off[(size_t)s];
            const int b0 = w->scene_body[(size_t)s], nb = w->scene_body[(size_t)s + 1] - b0;
            RP_CUDA(cudaMemcpyAsync(&g[13 * (size_t)b0], base + o.grad, 13 * (size_t)nb * 8, cudaMemcpyDeviceToHost, w->stream));
            RP_CUDA(cudaMemcpyAsync(&gi[(size_t)b0], base + o.ginv, (size_t)nb * 8, cudaMemcpyDeviceToHost, w->stream));
            RP_CUDA(cudaMemcpyAsync(&gmu[2 * (size_t)b0], base + o.gmu, 2 * (size_t)nb * 8, cudaMemcpyDeviceToHost, w->stream));
            RP_CUDA(cudaMemcpyAsync(&loss_out[s], base + o.loss, 8, cudaMemcpyDeviceToHost, w->stream));
            RP_CUDA(cudaMemcpyAsync(&status[(size_t)s], base + o.status, 4, cudaMemcpyDeviceToHost, w->stream));
            RP_CUDA(cudaMemcpyAsync(&prof[6 * (size_t)s], base + o.prof, 48, cudaMemcpyDeviceToHost, w->stream));
        }
        RP_CUDA(cudaStreamSynchronize(w->stream));
        {
            // the slowest scene's phase split, in ms at the SM clock
            int clock_khz = 1;
            cudaDeviceGetAttribute(&clock_khz, cudaDevAttrClockRate, w->device);
            size_t worst = 0;
            long long worst_c = -1;
            for (size_t s = 0; s < (size_t)S; ++s) {
                const long long c = prof[6 * s] + prof[6 * s + 1] + prof[6 * s + 2] + prof[6 * s + 3];
                if (c > worst_c) { worst_c = c; worst = s; }
            }
            for (int k = 0; k < 4; ++k) w->adj_prof[k] = (double)prof[6 * worst + (size_t)k] / (double)std::max(clock_khz, 1);
            w->adj_prof[4] = (double)prof[6 * worst + 4];
            w->adj_prof[5] = (double)prof[6 * worst + 5];
        }
        int bad = 0;
        for (int v : status) bad |= v;
        if (bad & ADJ_ST_TAPE) {
            if (attempt < 2) { tape_scale *= 4; continue; }
            return fail(RP_ERR_CAPACITY, "adjoint tape overflow");
        }
        if (bad & ADJ_ST_BAD_TAPE) return fail(RP_ERR_STATE, "adjoint tape inconsistent (an entry refers to a later one)");
        if (bad & ADJ_ST_UNSUPPORTED) return fail(RP_ERR_INVALID, "the adjoint's contacts cover hull colliders only");
        if (bad & (ADJ_ST_PAIRS | ADJ_ST_CONTACTS)) return fail(RP_ERR_CAPACITY, "adjoint pair or contact scratch overflow");
        if (bad & ADJ_ST_NARROW) return fail(RP_ERR_DEGENERATE, "degenerate or oversized narrowphase in the adjoint");
        for (size_t e = 0; e < N; ++e) {
            const HostBody& b = w->bodies[e];
            const size_t slot = (size_t)b.slot;
            for (int k = 0; k < 3; ++k) {
                grad_v[3 * e + k] = g[13 * slot + 7 + (size_t)k];
                grad_w[3 * e + k] = g[13 * slot + 10 + (size_t)k];
            }
            // d loss / d m = d loss / d invm * d invm / d m = -invm^2 d loss / d invm
            grad_mass[e] = b.fixed ? 0.0 : -b.invm * b.invm * gi[slot];
            if (grad_friction) {
                grad_friction[2 * e] = gmu[2 * slot];
                grad_friction[2 * e + 1] = gmu[2 * slot + 1];
            }
        }
        result = RP_OK;
        break;
    }
    return result;
}

rp_status rp_adjoint_profile(rp_world* w, double out[6]) {
    if (check_world(w) || !out) return RP_ERR_INVALID;
    for (int k = 0; k < 6; ++k) out[k] = w->adj_prof[k];
    return RP_OK;
}

rp_status rp_degenerate_info(rp_world* w, int64_t out[5]) {
    if (check_world(w) || !out) return fail(RP_ERR_INVALID, "null argument");
    for (int k = 0; k < 5; ++k) out[k] = k == 0 ? 0 : -1;
    if (w->device < 0 || !w->d_deg.p) return RP_OK;
    RP_CUDA(cudaSetDevice(w->device));
    int32_t rec[8];
    RP_CUDA(cudaMemcpyAsync(rec, w->d_deg.p, sizeof(rec), cudaMemcpyDeviceToHost, w->stream));
    RP_CUDA(cudaMemsetAsync(w->d_deg.p, 0, sizeof(rec), w->stream));
    RP_CUDA(cudaStreamSynchronize(w->stream));
    if (rec[0] == 0) return RP_OK;
    out[0] = rec[0];
    out[1] = rec[1];
    out[2] = rec[2] >= 0 && rec[2] < (int32_t)w->slot_to_entity.size() ? w->slot_to_entity[(size_t)rec[2]] : -1;
    out[3] = rec[3] >= 0 && rec[3] < (int32_t)w->slot_to_entity.size() ? w->slot_to_entity[(size_t)rec[3]] : -1;
    out[4] = rec[4];
    return RP_OK;
}

rp_status rp_transformed_hulls_size(rp_world* w, uint64_t* num_vertices, uint64_t* num_normals) {
    if (check_world(w) || !num_vertices || !num_normals) return fail(RP_ERR_INVALID, "null argument");
    int64_t nv = 0, nn = 0;
    for (const HostBody& b : w->bodies)
        for (const rp_collider_desc& d : b.cols)
            if (d.type == RP_COLLIDER_HULL) { nv += w->hulls[(size_t)d.hull]->nv(); nn += w->hulls[(size_t)d.hull]->nf(); }
    *num_vertices = (uint64_t)nv;
    *num_normals = (uint64_t)nn;
    return RP_OK;
}

rp_status rp_transformed_hulls(rp_world* w, double* vertices_out, double* normals_out) {
    if (check_world(w) || !vertices_out || !normals_out) return fail(RP_ERR_INVALID, "null argument");
    if (w->device < 0) return fail(RP_ERR_NO_DEVICE, "host-only world");
    if (w->bodies.empty()) return RP_OK;
    RP_CUDA(cudaSetDevice(w->device));
    rp_status s = ensure_device(w);
    if (s != RP_OK) return s;
    const size_t vb = (size_t)std::max<int64_t>(w->hull_nv, 1) * 24, nb = (size_t)std::max<int64_t>(w->hull_nn, 1) * 24;
    RP_CUDA(w->d_hull_v.ensure(vb));
    RP_CUDA(w->d_hull_n.ensure(nb));
    RP_CUDA(w->h_hull.ensure(vb + nb));
    WorldHullsArgs a;
    a.colliders = w->d_colliders.as<Collider>();
    a.col_body = w->d_col_body.as<int32_t>();
    a.shapes = w->d_shapes.as<Shape>();
    a.shape_verts = w->d_shape_verts.as<double>();
    a.face_normal = w->d_face_normal.as<double>();
    a.pos = w->d_pos.as<double4_32a>();
    a.rot = w->d_rot.as<double4_32a>();
    a.ncolliders = w->dims.ncolliders;
    a.vertices_out = w->d_hull_v.as<double>();
    a.normals_out = w->d_hull_n.as<double>();
    RP_CUDA(world_hulls(a, w->stream));
    w->launches++;
    char* h = (char*)w->h_hull.p;
    RP_CUDA(cudaMemcpyAsync(h, a.vertices_out, (size_t)w->hull_nv * 24, cudaMemcpyDeviceToHost, w->stream));
    RP_CUDA(cudaMemcpyAsync(h + vb, a.normals_out, (size_t)w->hull_nn * 24, cudaMemcpyDeviceToHost, w->stream));
    RP_CUDA(cudaStreamSynchronize(w->stream));
    w->d2h_bytes += (uint64_t)(w->hull_nv + w->hull_nn) * 24;
    // device order is slot order (bodies grouped by scene); the output is in entity order
    const double* hv = (const double*)h;
    const double* hn = (const double*)(h + vb);
    int64_t sv = 0, sn = 0;
    for (size_t slot = 0; slot < w->bodies.size(); ++slot) {
        const size_t e = (size_t)w->slot_to_entity[slot];
        const int64_t nv = w->hull_v_off[e + 1] - w->hull_v_off[e], nn = w->hull_n_off[e + 1] - w->hull_n_off[e];
        std::memcpy(vertices_out + 3 * w->hull_v_off[e], hv + 3 * sv, (size_t)nv * 24);
        std::memcpy(normals_out + 3 * w->hull_n_off[e], hn + 3 * sn, (size_t)nn * 24);
        sv += nv;
        sn += nn;
    }
    return RP_OK;
}

rp_status rp_last_schedule(rp_world* w, int32_t scene, int32_t which, int32_t* level_out, int32_t* bodies_out,
                           uint32_t cap, uint32_t* count) {
    if (check_world(w) || scene < 0 || scene >= w->num_scenes || (which != 0 && which != 1) || !count)
        return fail(RP_ERR_INVALID, "bad argument");
    if (w->device < 0 || !w->d_scene_nodes.p || w->static_dirty) return fail(RP_ERR_STATE, "no step has run");
    RP_CUDA(cudaSetDevice(w->device));
    int32_t nn = 0;
    RP_CUDA(cudaMemcpyAsync(&nn, w->d_scene_nodes.as<int32_t>() + scene, 4, cudaMemcpyDeviceToHost, w->stream));
    RP_CUDA(cudaStreamSynchronize(w->stream));
    *count = (uint32_t)nn;
    const int32_t nbase = w->scene_node_cap[(size_t)scene];
    const uint32_t m = std::min<uint32_t>((uint32_t)nn, cap);
    if (m == 0) return RP_OK;
    // the schedule is what the sweeps read: the level table and the nodes bucketed by level
    const DevBuf& Lv = which ? w->d_scene_vlevels : w->d_scene_levels;
    const DevBuf& Lc = which ? w->d_vlevel_count : w->d_level_count;
    const DevBuf& Ln = which ? w->d_vlevel_nodes : w->d_level_nodes;
    int32_t L = 0;
    RP_CUDA(cudaMemcpyAsync(&L, Lv.as<int32_t>() + scene, 4, cudaMemcpyDeviceToHost, w->stream));
    RP_CUDA(cudaStreamSynchronize(w->stream));
    L = std::max(0, std::min(L, w->max_levels));
    std::vector<int32_t> start((size_t)L + 1);
    RP_CUDA(cudaMemcpyAsync(start.data(), Lc.as<int32_t>() + (size_t)scene * (size_t)(w->max_levels + 1),
                            ((size_t)L + 1) * 4, cudaMemcpyDeviceToHost, w->stream));
    RP_CUDA(cudaStreamSynchronize(w->stream));
    const int32_t total = std::max(0, std::min(start[(size_t)L], nn));
    std::vector<int32_t> nodes((size_t)std::max(total, 1)), bod(2 * (size_t)m);
    if (total) RP_CUDA(cudaMemcpyAsync(nodes.data(), Ln.as<int32_t>() + nbase, (size_t)total * 4, cudaMemcpyDeviceToHost, w->stream));
    RP_CUDA(cudaMemcpyAsync(bod.data(), w->d_node_body.as<int32_t>() + 2 * (size_t)nbase, 2 * (size_t)m * 4,
                            cudaMemcpyDeviceToHost, w->stream));
    RP_CUDA(cudaStreamSynchronize(w->stream));
    std::vector<int32_t> lev(m, -1);
    for (int32_t l = 0; l < L; ++l)
        for (int32_t i = start[(size_t)l]; i < start[(size_t)l + 1] && i < total; ++i)
            if (nodes[(size_t)i] >= 0 && (uint32_t)nodes[(size_t)i] < m) lev[(size_t)nodes[(size_t)i]] = l;
    for (uint32_t k = 0; k < m; ++k) {
        if (level_out) level_out[k] = lev[k];
        if (bodies_out)
            for (int j = 0; j < 2; ++j) {
                const int32_t b = bod[2 * (size_t)k + (size_t)j];
                bodies_out[2 * (size_t)k + (size_t)j] = b >= 0 ? w->slot_to_entity[(size_t)b] : -1;
            }
    }
    return RP_OK;
}

rp_status rp_world_set_sweep_order(rp_world* w, int32_t order) {
    if (check_world(w)) return RP_ERR_INVALID;
    if (order != RP_SWEEP_REFERENCE && order != RP_SWEEP_COLOURED) return fail(RP_ERR_INVALID, "bad sweep order");
    w->sweep_order = order;
    if (w->graph) { cudaGraphExecDestroy(w->graph); w->graph = nullptr; }   // the order is a kernel argument
    return RP_OK;
}

rp_status rp_world_set_sweep_assignment(rp_world* w, int32_t cta) {
    if (check_world(w)) return RP_ERR_INVALID;
    if (cta < 0) return fail(RP_ERR_INVALID, "bad sweep assignment");
    w->pipe.sweep_cta = cta == 1 ? 1 : 0;
    w->cta_from = cta == 1 ? 0 : cta;
    set_cta_scenes(w);
    w->layout_gen++;   // recapture the frame graph with the new launch shapes
    return RP_OK;
}

rp_status rp_world_set_wait_limit(rp_world* w, uint64_t microseconds) {
    if (check_world(w)) return RP_ERR_INVALID;
    if (microseconds > 60000000ull) return fail(RP_ERR_INVALID, "wait limit above 60 s");
    w->wait_ns = microseconds * 1000ull;
    if (w->graph) { cudaGraphExecDestroy(w->graph); w->graph = nullptr; }   // the limit is a kernel argument
    return RP_OK;
}

rp_status rp_world_set_mode(rp_world* w, int32_t mode) {
    if (check_world(w)) return RP_ERR_INVALID;
    if (mode != RP_MODE_AUTO && mode != RP_MODE_PERSISTENT && mode != RP_MODE_PHASED) return fail(RP_ERR_INVALID, "bad mode");
    w->mode = mode;
    return RP_OK;
}

rp_status rp_last_step_ms(rp_world* w, double* ms) {
    if (check_world(w) || !ms) return RP_ERR_INVALID;
    *ms = w->last_ms;
    return RP_OK;
}

}  // extern "C"
