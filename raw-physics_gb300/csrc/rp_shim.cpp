// The C++-mangled pbd_simulate / pbd_simulate_with_constraints drop-in (include/rp_compat.h).
//
// Each call: (1) if the set of entities, their colliders, mass properties or the external
// constraints changed since the last call, rebuild the device world from the caller's own data
// (hull topology forwarded as-is, mass properties as stored in the entities); (2) upload the
// entities' state and this frame's forces; (3) run the step on the GPU; (4) write the results back
// into the Entity structs and refresh the colliders' transformed geometry.
#include "../../include/rp_compat.h"
#include "../../include/rp.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <vector>

namespace {

template <typename T>
size_t la_len(const T* a) {   // light_array length (include/light_array.h:72)
    return a ? ((const size_t*)(const void*)a)[-1] : 0;
}

rp_world* g_world = nullptr;
std::vector<double> g_signature;
std::map<uint64_t, int32_t> g_entity_of_id;

void report(const char* what) { std::fprintf(stderr, "raw-physics GB300 drop-in: %s: %s\n", what, rp_last_error()); }

void push(std::vector<double>& sig, const void* p, size_t n) {
    const unsigned char* b = (const unsigned char*)p;
    for (size_t i = 0; i < n; i += 8) {
        uint64_t x = 0;
        std::memcpy(&x, b + i, (n - i) < 8 ? (n - i) : 8);
        double d;
        std::memcpy(&d, &x, 8);
        sig.push_back(d);
    }
}

// Everything that determines the device layout and constants (not the per-frame state).
std::vector<double> signature(Entity** es, size_t n, const Constraint* cons, size_t nc) {
    std::vector<double> sig;
    for (size_t i = 0; i < n; ++i) {
        const Entity* e = es[i];
        push(sig, &e->id, 8);
        const void* cp = e->colliders;
        push(sig, &cp, sizeof(cp));
        size_t ncol = la_len(e->colliders);
        push(sig, &ncol, 8);
        for (size_t c = 0; c < ncol; ++c) push(sig, &e->colliders[c], sizeof(rpc_collider));
        push(sig, &e->inverse_mass, 8);
        push(sig, &e->inertia_tensor, sizeof(rpc_mat3));
        push(sig, &e->inverse_inertia_tensor, sizeof(rpc_mat3));
        push(sig, &e->bounding_sphere_radius, 8);
        push(sig, &e->fixed, 4);
        push(sig, &e->static_friction_coefficient, 24);
    }
    for (size_t k = 0; k < nc; ++k) {
        Constraint c = cons[k];
        // lambdas do not matter (copy_constraints resets them every substep, pbd.cpp:426-462)
        switch (c.type) {
        case 0: c.positional_constraint.lambda = 0; break;
        case 2: c.mutual_orientation_constraint.lambda = 0; break;
        case 3: c.hinge_joint_constraint.lambda_pos = c.hinge_joint_constraint.lambda_aligned_axes = c.hinge_joint_constraint.lambda_limit_axes = 0; break;
        case 4: c.spherical_joint_constraint.lambda_pos = c.spherical_joint_constraint.lambda_swing = c.spherical_joint_constraint.lambda_twist = 0; break;
        default: break;
        }
        push(sig, &c, sizeof(c));
    }
    return sig;
}

bool build(Entity** es, size_t n, const Constraint* cons, size_t nc) {
    if (g_world) rp_world_destroy(g_world);
    g_world = nullptr;
    g_entity_of_id.clear();
    const char* prec = std::getenv("RP_SHIM_PRECISION");
    const char* dev = std::getenv("RP_SHIM_DEVICE");
    int precision = (prec && std::strcmp(prec, "fp64") == 0) ? RP_PRECISION_FP64 : RP_PRECISION_FP32;
    if (rp_world_create(&g_world, dev ? std::atoi(dev) : 0, precision) != RP_OK) { report("world"); return false; }
    std::map<const rpc_collider*, int32_t> hull_of;
    for (size_t i = 0; i < n; ++i) {
        const Entity* e = es[i];
        std::vector<rp_collider_desc> descs;
        for (size_t c = 0; c < la_len(e->colliders); ++c) {
            const rpc_collider* col = &e->colliders[c];
            rp_collider_desc d;
            d.type = col->type;
            d.hull = -1;
            d.radius = 0.0f;
            if (col->type == 0) {
                d.radius = col->sphere.radius;
            } else {
                const rpc_hull& h = col->convex_hull;
                int32_t nv = (int32_t)la_len(h.vertices), nf = (int32_t)la_len(h.faces);
                std::vector<double> v, nrm;
                std::vector<int32_t> fs{0}, fe, vfs{0}, vf, vns{0}, vn, ffs{0}, ff;
                for (int32_t k = 0; k < nv; ++k) { v.push_back(h.vertices[k].x); v.push_back(h.vertices[k].y); v.push_back(h.vertices[k].z); }
                for (int32_t f = 0; f < nf; ++f) {
                    nrm.push_back(h.faces[f].normal.x); nrm.push_back(h.faces[f].normal.y); nrm.push_back(h.faces[f].normal.z);
                    for (size_t k = 0; k < la_len(h.faces[f].elements); ++k) fe.push_back((int32_t)h.faces[f].elements[k]);
                    fs.push_back((int32_t)fe.size());
                    for (size_t k = 0; k < la_len(h.face_to_neighbors[f]); ++k) ff.push_back((int32_t)h.face_to_neighbors[f][k]);
                    ffs.push_back((int32_t)ff.size());
                }
                for (int32_t k = 0; k < nv; ++k) {
                    for (size_t j = 0; j < la_len(h.vertex_to_faces[k]); ++j) vf.push_back((int32_t)h.vertex_to_faces[k][j]);
                    vfs.push_back((int32_t)vf.size());
                    for (size_t j = 0; j < la_len(h.vertex_to_neighbors[k]); ++j) vn.push_back((int32_t)h.vertex_to_neighbors[k][j]);
                    vns.push_back((int32_t)vn.size());
                }
                if (rp_hull_create_from_topology(g_world, v.data(), nv, nrm.data(), nf, fs.data(), fe.data(), vfs.data(), vf.data(),
                                                 vns.data(), vn.data(), ffs.data(), ff.data(), &d.hull) != RP_OK) {
                    report("hull");
                    return false;
                }
            }
            descs.push_back(d);
        }
        double p[3] = {e->world_position.x, e->world_position.y, e->world_position.z};
        double q[4] = {e->world_rotation.x, e->world_rotation.y, e->world_rotation.z, e->world_rotation.w};
        double mass = e->fixed ? 0.0 : 1.0;
        int32_t id = -1;
        // mass properties are forwarded as stored (they may have been edited after entity_create)
        if (rp_entity_create(g_world, 0, p, q, mass, e->fixed, descs.data(), (uint32_t)descs.size(),
                             e->static_friction_coefficient, e->dynamic_friction_coefficient, e->restitution_coefficient,
                             &id) != RP_OK) {
            report("entity");
            return false;
        }
        double I[9], Ii[9];
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) { I[3 * r + c] = e->inertia_tensor.data[r][c]; Ii[3 * r + c] = e->inverse_inertia_tensor.data[r][c]; }
        if (rp_entity_set_mass_properties(g_world, id, e->inverse_mass, I, Ii, e->bounding_sphere_radius) != RP_OK) {
            report("mass properties");
            return false;
        }
        g_entity_of_id[e->id] = id;
    }
    for (size_t k = 0; k < nc; ++k) {
        const Constraint& c = cons[k];
        auto a = g_entity_of_id.find(c.e1_id), b = g_entity_of_id.find(c.e2_id);
        if (a == g_entity_of_id.end() || b == g_entity_of_id.end()) {
            std::fprintf(stderr, "raw-physics GB300 drop-in: constraint on an entity not passed to pbd_simulate\n");
            return false;
        }
        rp_status s = RP_ERR_INVALID;
        if (c.type == 0) {
            const auto& x = c.positional_constraint;
            double r1[3] = {x.r1_lc.x, x.r1_lc.y, x.r1_lc.z}, r2[3] = {x.r2_lc.x, x.r2_lc.y, x.r2_lc.z};
            double d[3] = {x.distance.x, x.distance.y, x.distance.z};
            s = rp_constraint_positional(g_world, a->second, b->second, r1, r2, x.compliance, d, nullptr);
        } else if (c.type == 2) {
            s = rp_constraint_mutual_orientation(g_world, a->second, b->second, c.mutual_orientation_constraint.compliance, nullptr);
        } else if (c.type == 3) {
            const auto& x = c.hinge_joint_constraint;
            double r1[3] = {x.r1_lc.x, x.r1_lc.y, x.r1_lc.z}, r2[3] = {x.r2_lc.x, x.r2_lc.y, x.r2_lc.z};
            s = rp_constraint_hinge(g_world, a->second, b->second, r1, r2, x.compliance, x.e1_aligned_axis, x.e2_aligned_axis,
                                    x.limited, x.e1_limit_axis, x.e2_limit_axis, x.lower_limit, x.upper_limit, nullptr);
        } else if (c.type == 4) {
            const auto& x = c.spherical_joint_constraint;
            double r1[3] = {x.r1_lc.x, x.r1_lc.y, x.r1_lc.z}, r2[3] = {x.r2_lc.x, x.r2_lc.y, x.r2_lc.z};
            s = rp_constraint_spherical(g_world, a->second, b->second, r1, r2, x.e1_swing_axis, x.e2_swing_axis, x.e1_twist_axis,
                                        x.e2_twist_axis, x.swing_lower_limit, x.swing_upper_limit, x.twist_lower_limit,
                                        x.twist_upper_limit, nullptr);
        }
        if (s != RP_OK) { report("constraint"); return false; }
    }
    return true;
}

// colliders_update (collider.cpp:409-438) at the entity's final pose
void refresh_colliders(Entity* e) {
    const rpc_quat& q = e->world_rotation;
    double m[3][3];
    m[0][0] = 1.0 - 2.0 * q.y * q.y - 2.0 * q.z * q.z;
    m[1][0] = 2.0 * q.x * q.y + 2.0 * q.w * q.z;
    m[2][0] = 2.0 * q.x * q.z - 2.0 * q.w * q.y;
    m[0][1] = 2.0 * q.x * q.y - 2.0 * q.w * q.z;
    m[1][1] = 1.0 - (2.0 * q.x * q.x) - (2.0 * q.z * q.z);
    m[2][1] = 2.0 * q.y * q.z + 2.0 * q.w * q.x;
    m[0][2] = 2.0 * q.x * q.z + 2.0 * q.w * q.y;
    m[1][2] = 2.0 * q.y * q.z - 2.0 * q.w * q.x;
    m[2][2] = 1.0 - (2.0 * q.x * q.x) - (2.0 * q.y * q.y);
    const double t[3] = {e->world_position.x, e->world_position.y, e->world_position.z};
    for (size_t c = 0; c < la_len(e->colliders); ++c) {
        rpc_collider* col = &e->colliders[c];
        if (col->type == 0) { col->sphere.center = e->world_position; continue; }
        rpc_hull& h = col->convex_hull;
        for (size_t i = 0; i < la_len(h.vertices); ++i) {
            const rpc_vec3 v = h.vertices[i];
            double o[3];
            for (int r = 0; r < 3; ++r) o[r] = v.x * m[r][0] + v.y * m[r][1] + v.z * m[r][2] + 1.0 * t[r];
            h.transformed_vertices[i].x = o[0];
            h.transformed_vertices[i].y = o[1];
            h.transformed_vertices[i].z = o[2];
        }
        for (size_t f = 0; f < la_len(h.faces); ++f) {
            const rpc_vec3 nn = h.faces[f].normal;
            double o[3];
            for (int r = 0; r < 3; ++r) o[r] = m[r][0] * nn.x + m[r][1] * nn.y + m[r][2] * nn.z;
            double l = std::sqrt(o[0] * o[0] + o[1] * o[1] + o[2] * o[2]);
            if (l != 0.0) { o[0] /= l; o[1] /= l; o[2] /= l; }
            h.transformed_faces[f].normal.x = o[0];
            h.transformed_faces[f].normal.y = o[1];
            h.transformed_faces[f].normal.z = o[2];
        }
    }
}

}  // namespace

extern "C" void rp_compat_reset(void) {
    if (g_world) rp_world_destroy(g_world);
    g_world = nullptr;
    g_signature.clear();
    g_entity_of_id.clear();
}

void pbd_simulate_with_constraints(double dt, Entity** entities, Constraint* cons, uint32_t num_substeps, uint32_t num_pos_iters,
                                   int32_t enable_collisions) {
    if (!(dt > 0.0) || !entities) return;   // pbd.cpp:471
    const size_t n = la_len(entities), nc = cons ? la_len(cons) : 0;
    if (n == 0) return;
    std::vector<double> sig = signature(entities, n, cons, nc);
    if (!g_world || sig != g_signature) {
        if (!build(entities, n, cons, nc)) { rp_compat_reset(); return; }
        g_signature = sig;
    }
    std::vector<double> st(n * RP_STATE_DOUBLES);
    for (size_t i = 0; i < n; ++i) {
        const Entity* e = entities[i];
        double* o = &st[i * RP_STATE_DOUBLES];
        const rpc_vec3* v3s[8] = {&e->world_position, nullptr, &e->linear_velocity, &e->angular_velocity,
                                  &e->previous_world_position, nullptr, &e->previous_linear_velocity, &e->previous_angular_velocity};
        const int off[8] = {0, 3, 7, 10, 13, 16, 20, 23};
        for (int k = 0; k < 8; ++k)
            if (v3s[k]) { o[off[k]] = v3s[k]->x; o[off[k] + 1] = v3s[k]->y; o[off[k] + 2] = v3s[k]->z; }
        o[3] = e->world_rotation.x; o[4] = e->world_rotation.y; o[5] = e->world_rotation.z; o[6] = e->world_rotation.w;
        o[16] = e->previous_world_rotation.x; o[17] = e->previous_world_rotation.y;
        o[18] = e->previous_world_rotation.z; o[19] = e->previous_world_rotation.w;
        o[26] = e->active ? 1.0 : 0.0;
        o[27] = e->deactivation_time;
    }
    if (rp_state_set(g_world, st.data()) != RP_OK) { report("state"); return; }
    rp_world_set_gravity(g_world, 0.0);
    for (size_t i = 0; i < n; ++i) {
        const Entity* e = entities[i];
        int32_t id = g_entity_of_id[e->id];
        for (size_t k = 0; k < la_len(e->forces); ++k) {
            // entity_add_force already stored world-frame values (entity.cpp:176-191)
            double p[3] = {e->forces[k].position.x, e->forces[k].position.y, e->forces[k].position.z};
            double f[3] = {e->forces[k].force.x, e->forces[k].force.y, e->forces[k].force.z};
            rp_entity_add_force(g_world, id, p, f, 0);
        }
    }
    if (rp_simulate(g_world, dt, num_substeps, num_pos_iters, enable_collisions, 1) != RP_OK) { report("simulate"); return; }
    if (rp_state_get(g_world, st.data()) != RP_OK) { report("state"); return; }
    for (size_t i = 0; i < n; ++i) {
        Entity* e = entities[i];
        const double* o = &st[i * RP_STATE_DOUBLES];
        e->world_position = {o[0], o[1], o[2]};
        e->world_rotation = {o[3], o[4], o[5], o[6]};
        e->linear_velocity = {o[7], o[8], o[9]};
        e->angular_velocity = {o[10], o[11], o[12]};
        e->previous_world_position = {o[13], o[14], o[15]};
        e->previous_world_rotation = {o[16], o[17], o[18], o[19]};
        e->previous_linear_velocity = {o[20], o[21], o[22]};
        e->previous_angular_velocity = {o[23], o[24], o[25]};
        e->active = o[26] != 0.0;
        e->deactivation_time = o[27];
        refresh_colliders(e);
    }
}

void pbd_simulate(double dt, Entity** entities, uint32_t num_substeps, uint32_t num_pos_iters, int32_t enable_collisions) {
    pbd_simulate_with_constraints(dt, entities, nullptr, num_substeps, num_pos_iters, enable_collisions);
}
