// The C++-mangled pbd_simulate / pbd_simulate_with_constraints drop-in (include/rp_compat.h).
//
// Each call: (1) if the set of entities, their colliders, mass properties or the external
// constraints changed since the last call, rebuild the device world from the caller's own data
// (hull topology forwarded as-is, mass properties as stored in the entities); (2) upload the
// entities' state only when the caller changed it since the last call wrote it back, and the
// frame's forces only when they are not the examples' plain gravity (0, -g / inverse_mass, 0) at the
// origin, which is kept on the device as the world's gravity instead; (3) run the step on the GPU;
// (4) write the results back into the Entity structs and refresh the colliders' transformed geometry
// from the device (colliders_update at the final pose, computed there in FP64).
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
std::vector<double> g_written;      // the state the last call wrote back (the device still holds it)
double g_gravity = 0.0;             // gravity the device world applies (0: forces are uploaded)
std::vector<double> g_hull_v, g_hull_n;   // staging of rp_transformed_hulls

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

// The caller's forces when every dynamic entity carries exactly the examples' gravity force,
// entity_add_force(e, 0, (0, -g * 1 / inverse_mass, 0)) (src/examples/stack.cpp:93-96), for one g:
// returns that g (bit for bit the value the device recomputes per entity), else 0.
double plain_gravity(Entity** es, size_t n) {
    double g = 0.0;
    for (size_t i = 0; i < n; ++i) {
        const Entity* e = es[i];
        if (e->fixed) continue;
        if (la_len(e->forces) != 1) return 0.0;
        const rpc_force& f = e->forces[0];
        if (f.local_coords || f.position.x != 0.0 || f.position.y != 0.0 || f.position.z != 0.0 || f.force.x != 0.0 ||
            f.force.z != 0.0 || !(e->inverse_mass > 0.0))
            return 0.0;
        if (g == 0.0) g = -f.force.y * e->inverse_mass;
        if (!(g != 0.0) || -g * 1.0 / e->inverse_mass != f.force.y) return 0.0;
    }
    return g;
}

// colliders_update (collider.cpp:409-446) of every entity at its final pose, computed on the device
// (rp_transformed_hulls) and copied into the caller's transformed vertices and face normals. The
// reference itself leaves them at the last substep's predicted pose, and only for the bodies of that
// substep's live pairs (pbd.cpp:598-599); its step recomputes them before every use, and callers run
// colliders_update on every entity before the next call (stack.cpp:88-91), so the final pose is what a
// caller reads. RP_SHIM_COLLIDERS=none skips the refresh (such callers recompute them anyway).
bool refresh_colliders(Entity** es, size_t n) {
    const char* mode = std::getenv("RP_SHIM_COLLIDERS");
    if (mode && std::strcmp(mode, "none") == 0) return true;
    uint64_t nv = 0, nn = 0;
    if (rp_transformed_hulls_size(g_world, &nv, &nn) != RP_OK) return false;
    g_hull_v.resize(3 * nv + 3);
    g_hull_n.resize(3 * nn + 3);
    if (rp_transformed_hulls(g_world, g_hull_v.data(), g_hull_n.data()) != RP_OK) return false;
    size_t iv = 0, in = 0;
    for (size_t i = 0; i < n; ++i) {
        Entity* e = es[i];
        for (size_t c = 0; c < la_len(e->colliders); ++c) {
            rpc_collider* col = &e->colliders[c];
            if (col->type == 0) { col->sphere.center = e->world_position; continue; }
            rpc_hull& h = col->convex_hull;
            const size_t hv = la_len(h.vertices), hf = la_len(h.faces);
            for (size_t k = 0; k < hv; ++k, ++iv)
                h.transformed_vertices[k] = {g_hull_v[3 * iv], g_hull_v[3 * iv + 1], g_hull_v[3 * iv + 2]};
            for (size_t f = 0; f < hf; ++f, ++in)
                h.transformed_faces[f].normal = {g_hull_n[3 * in], g_hull_n[3 * in + 1], g_hull_n[3 * in + 2]};
        }
    }
    return true;
}

}  // namespace

extern "C" rp_world* rp_compat_world(void) { return g_world; }

extern "C" void rp_compat_reset(void) {
    if (g_world) rp_world_destroy(g_world);
    g_world = nullptr;
    g_signature.clear();
    g_entity_of_id.clear();
    g_written.clear();
    g_gravity = 0.0;
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
        g_written.clear();
        g_gravity = 0.0;
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
    // the device already holds the state this call would upload when the caller left it as written
    if (g_written.size() != st.size() || std::memcmp(g_written.data(), st.data(), st.size() * sizeof(double)) != 0) {
        if (rp_state_set(g_world, st.data()) != RP_OK) { report("state"); return; }
    }
    const double g = plain_gravity(entities, n);
    if (g != g_gravity) {
        rp_world_set_gravity(g_world, g);
        g_gravity = g;
    }
    if (g == 0.0) {
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
    }
    g_written.swap(st);
    if (!refresh_colliders(entities, n)) report("colliders");
}

void pbd_simulate(double dt, Entity** entities, uint32_t num_substeps, uint32_t num_pos_iters, int32_t enable_collisions) {
    pbd_simulate_with_constraints(dt, entities, nullptr, num_substeps, num_pos_iters, enable_collisions);
}
