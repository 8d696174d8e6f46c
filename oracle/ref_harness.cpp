// Oracle harness around the reference's own physics sources — TEST INFRASTRUCTURE ONLY.
//
// oracle/Makefile compiles this file together with the reference's src/physics/*.cpp,
// src/entity.cpp, src/quaternion.cpp, src/util.cpp and src/render/obj.cpp (the OBJ reader, for
// the hull-from-OBJ fixtures), taken from where they lie in the
// reference checkout, into oracle/_ref/libref_harness.so. It implements oracle/harness.h by
// calling the reference's public functions exactly as its example scenes do
// (src/examples/stack.cpp:86-104, src/examples/examples_util.cpp:5-24).
#define DYNAMIC_ARRAY_IMPLEMENT
#define GRAPHICS_MATH_IMPLEMENT
#define C_FEK_HASH_MAP_IMPLEMENT
#include <light_array.h>
#include <hash_map.h>
#include <gm.h>
#include "entity.h"
#include "physics/pbd.h"
#include "physics/broad.h"
#include "physics/collider.h"
#include "physics/gjk.h"
#include "physics/epa.h"
#include "physics/clipping.h"
#include "render/obj.h"
#include <vector>
#include <string.h>
#include "harness.h"

extern Entity** entities;  // the reference's process-global registry (src/entity.cpp:7)

namespace {

struct MeshData {
    std::vector<float> pos;        // 3 per vertex
    std::vector<uint32_t> idx;
};

std::vector<MeshData> g_meshes;
Collider* g_pending = nullptr;     // light_array of colliders for the next entity
std::vector<eid> g_ids;            // entity index -> eid
Constraint* g_constraints = nullptr;
bool g_initialised = false;

Entity* ent(int i) { return entity_get_by_id(g_ids[(size_t)i]); }

Collider make_hull(const MeshData& m, const double s[3]) {
    // examples_util_create_single_convex_hull_collider_array: (r64)float position, scaled in FP64
    vec3* verts = array_new(vec3);
    size_t nv = m.pos.size() / 3;
    for (size_t i = 0; i < nv; ++i) {
        vec3 p = (vec3){(r64)m.pos[3 * i + 0], (r64)m.pos[3 * i + 1], (r64)m.pos[3 * i + 2]};
        p.x *= s[0];
        p.y *= s[1];
        p.z *= s[2];
        array_push(verts, p);
    }
    u32* idx = array_new(u32);
    for (uint32_t v : m.idx) array_push(idx, v);
    Collider c = collider_convex_hull_create(verts, idx);
    array_free(verts);
    array_free(idx);
    return c;
}

}  // namespace

extern "C" {

void orc_reset(void) {
    if (g_initialised) {
        // Destroy from the back so the unordered removal in entity_destroy never skips one.
        while (array_length(entities) > 0) {
            Entity* e = entities[array_length(entities) - 1];
            colliders_destroy(e->colliders);
            array_free(e->colliders);
            entity_destroy(e);
        }
        entity_module_destroy();
    }
    entity_module_init();
    g_initialised = true;
    g_meshes.clear();
    g_ids.clear();
    if (g_pending) { array_free(g_pending); g_pending = nullptr; }
    if (g_constraints) { array_free(g_constraints); g_constraints = nullptr; }
}

int orc_mesh_add(const float* positions, uint32_t num_vertices, const uint32_t* indices, uint32_t num_indices) {
    MeshData m;
    m.pos.assign(positions, positions + 3 * (size_t)num_vertices);
    m.idx.assign(indices, indices + num_indices);
    g_meshes.push_back(std::move(m));
    return (int)g_meshes.size() - 1;
}

void orc_colliders_begin(void) {
    if (g_pending) array_free(g_pending);
    g_pending = array_new(Collider);
}

int orc_colliders_add_hull(int mesh, const double scale[3]) {
    Collider c = make_hull(g_meshes[(size_t)mesh], scale);
    array_push(g_pending, c);
    return (int)array_length(g_pending) - 1;
}

int orc_colliders_add_sphere(float radius) {
    Collider c = collider_sphere_create(radius);
    array_push(g_pending, c);
    return (int)array_length(g_pending) - 1;
}

int orc_entity_create(const double pos[3], const double rot[4], double mass, int fixed,
                      double mus, double mud, double rest) {
    Mesh mesh;
    memset(&mesh, 0, sizeof(mesh));
    vec3 p = (vec3){pos[0], pos[1], pos[2]};
    Quaternion q = (Quaternion){rot[0], rot[1], rot[2], rot[3]};
    vec3 one = (vec3){1.0, 1.0, 1.0};
    vec4 white = (vec4){1.0, 1.0, 1.0, 1.0};
    eid id;
    if (fixed) {
        id = entity_create_fixed(mesh, p, q, one, white, g_pending, mus, mud, rest);
    } else {
        id = entity_create(mesh, p, q, one, white, mass, g_pending, mus, mud, rest);
    }
    g_pending = nullptr;  // ownership moved to the entity
    g_ids.push_back(id);
    return (int)g_ids.size() - 1;
}

void orc_entity_set_velocity(int i, const double v[3], const double w[3]) {
    Entity* e = ent(i);
    e->linear_velocity = (vec3){v[0], v[1], v[2]};
    e->angular_velocity = (vec3){w[0], w[1], w[2]};
}

void orc_entity_add_force(int i, const double position[3], const double force[3], int local_coords) {
    entity_add_force(ent(i), (vec3){position[0], position[1], position[2]},
                     (vec3){force[0], force[1], force[2]}, local_coords);
}

double orc_entity_get_inverse_mass(int i) { return ent(i)->inverse_mass; }

void orc_entity_get_inertia(int i, double inertia[9], double inverse_inertia[9]) {
    Entity* e = ent(i);
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            inertia[3 * r + c] = e->inertia_tensor.data[r][c];
            inverse_inertia[3 * r + c] = e->inverse_inertia_tensor.data[r][c];
        }
}

double orc_entity_get_radius(int i) { return ent(i)->bounding_sphere_radius; }

int orc_hull_topology(int i, int k, int which, int32_t* start, int32_t* data, int32_t cap, int32_t* ndata) {
    const Collider_Convex_Hull& h = ent(i)->colliders[k].convex_hull;
    int rows = which == 0 || which == 3 ? (int)array_length(h.faces) : (int)array_length(h.vertices);
    int32_t n = 0;
    for (int r = 0; r < rows; ++r) {
        const u32* row = which == 0 ? h.faces[r].elements : which == 1 ? h.vertex_to_faces[r]
                       : which == 2 ? h.vertex_to_neighbors[r] : h.face_to_neighbors[r];
        if (start) start[r] = n;
        for (u32 c = 0; c < array_length(row); ++c) {
            if (data && n < cap) data[n] = (int32_t)row[c];
            ++n;
        }
    }
    if (start) start[rows] = n;
    if (ndata) *ndata = n;
    return rows;
}

int orc_hull_geometry(int i, int k, double* verts, double* normals, int32_t capv, int32_t capf, int32_t* nf) {
    const Collider_Convex_Hull& h = ent(i)->colliders[k].convex_hull;
    int nv = (int)array_length(h.vertices), f = (int)array_length(h.faces);
    for (int v = 0; v < nv && v < capv; ++v) { verts[3 * v] = h.vertices[v].x; verts[3 * v + 1] = h.vertices[v].y; verts[3 * v + 2] = h.vertices[v].z; }
    for (int j = 0; j < f && j < capf; ++j) { normals[3 * j] = h.faces[j].normal.x; normals[3 * j + 1] = h.faces[j].normal.y; normals[3 * j + 2] = h.faces[j].normal.z; }
    if (nf) *nf = f;
    return nv;
}

static void push_constraint(const Constraint& c) {
    if (!g_constraints) g_constraints = array_new(Constraint);
    array_push(g_constraints, c);
}

int orc_constraint_positional(int e1, int e2, const double r1[3], const double r2[3], double compliance,
                              const double distance[3]) {
    Constraint c;
    memset(&c, 0, sizeof(c));
    pbd_positional_constraint_init(&c, g_ids[(size_t)e1], g_ids[(size_t)e2], (vec3){r1[0], r1[1], r1[2]},
                                   (vec3){r2[0], r2[1], r2[2]}, compliance,
                                   (vec3){distance[0], distance[1], distance[2]});
    push_constraint(c);
    return (int)array_length(g_constraints) - 1;
}

int orc_constraint_mutual_orientation(int e1, int e2, double compliance) {
    Constraint c;
    memset(&c, 0, sizeof(c));
    pbd_mutual_orientation_constraint_init(&c, g_ids[(size_t)e1], g_ids[(size_t)e2], compliance);
    push_constraint(c);
    return (int)array_length(g_constraints) - 1;
}

int orc_constraint_hinge(int e1, int e2, const double r1[3], const double r2[3], double compliance,
                         int a1, int a2, int limited, int l1, int l2, double lower, double upper) {
    Constraint c;
    memset(&c, 0, sizeof(c));
    vec3 v1 = (vec3){r1[0], r1[1], r1[2]};
    vec3 v2 = (vec3){r2[0], r2[1], r2[2]};
    if (limited) {
        pbd_hinge_joint_constraint_limited_init(&c, g_ids[(size_t)e1], g_ids[(size_t)e2], v1, v2, compliance,
                                                (PBD_Axis_Type)a1, (PBD_Axis_Type)a2, (PBD_Axis_Type)l1,
                                                (PBD_Axis_Type)l2, lower, upper);
    } else {
        pbd_hinge_joint_constraint_unlimited_init(&c, g_ids[(size_t)e1], g_ids[(size_t)e2], v1, v2, compliance,
                                                  (PBD_Axis_Type)a1, (PBD_Axis_Type)a2);
    }
    push_constraint(c);
    return (int)array_length(g_constraints) - 1;
}

int orc_constraint_spherical(int e1, int e2, const double r1[3], const double r2[3], int s1, int s2, int t1,
                             int t2, double slo, double shi, double tlo, double thi) {
    Constraint c;
    memset(&c, 0, sizeof(c));
    pbd_spherical_joint_constraint_init(&c, g_ids[(size_t)e1], g_ids[(size_t)e2], (vec3){r1[0], r1[1], r1[2]},
                                        (vec3){r2[0], r2[1], r2[2]}, (PBD_Axis_Type)s1, (PBD_Axis_Type)s2,
                                        (PBD_Axis_Type)t1, (PBD_Axis_Type)t2, slo, shi, tlo, thi);
    push_constraint(c);
    return (int)array_length(g_constraints) - 1;
}

void orc_step(double dt, uint32_t num_substeps, uint32_t num_pos_iters, int enable_collisions, double gravity) {
    Entity** all = entity_get_all();
    for (u32 i = 0; i < array_length(all); ++i) {
        Entity* e = all[i];
        colliders_update(e->colliders, e->world_position, &e->world_rotation);
    }
    for (u32 i = 0; i < array_length(all); ++i) {
        entity_add_force(all[i], (vec3){0.0, 0.0, 0.0}, (vec3){0.0, -gravity * 1.0 / all[i]->inverse_mass, 0.0}, false);
    }
    pbd_simulate_with_constraints(dt, all, g_constraints, num_substeps, num_pos_iters, enable_collisions);
    for (u32 i = 0; i < array_length(all); ++i) {
        entity_clear_forces(all[i]);
    }
    array_free(all);
}

uint32_t orc_num_entities(void) { return (uint32_t)g_ids.size(); }

void orc_get_state(double* out) {
    for (size_t i = 0; i < g_ids.size(); ++i) {
        Entity* e = ent((int)i);
        double* o = out + i * ORC_STATE_DOUBLES;
        o[0] = e->world_position.x; o[1] = e->world_position.y; o[2] = e->world_position.z;
        o[3] = e->world_rotation.x; o[4] = e->world_rotation.y; o[5] = e->world_rotation.z; o[6] = e->world_rotation.w;
        o[7] = e->linear_velocity.x; o[8] = e->linear_velocity.y; o[9] = e->linear_velocity.z;
        o[10] = e->angular_velocity.x; o[11] = e->angular_velocity.y; o[12] = e->angular_velocity.z;
        o[13] = e->previous_world_position.x; o[14] = e->previous_world_position.y; o[15] = e->previous_world_position.z;
        o[16] = e->previous_world_rotation.x; o[17] = e->previous_world_rotation.y;
        o[18] = e->previous_world_rotation.z; o[19] = e->previous_world_rotation.w;
        o[20] = e->previous_linear_velocity.x; o[21] = e->previous_linear_velocity.y; o[22] = e->previous_linear_velocity.z;
        o[23] = e->previous_angular_velocity.x; o[24] = e->previous_angular_velocity.y; o[25] = e->previous_angular_velocity.z;
        o[26] = e->active ? 1.0 : 0.0;
        o[27] = e->deactivation_time;
    }
}

void orc_set_state(const double* in) {
    for (size_t i = 0; i < g_ids.size(); ++i) {
        Entity* e = ent((int)i);
        const double* o = in + i * ORC_STATE_DOUBLES;
        e->world_position = (vec3){o[0], o[1], o[2]};
        e->world_rotation = (Quaternion){o[3], o[4], o[5], o[6]};
        e->linear_velocity = (vec3){o[7], o[8], o[9]};
        e->angular_velocity = (vec3){o[10], o[11], o[12]};
        e->previous_world_position = (vec3){o[13], o[14], o[15]};
        e->previous_world_rotation = (Quaternion){o[16], o[17], o[18], o[19]};
        e->previous_linear_velocity = (vec3){o[20], o[21], o[22]};
        e->previous_angular_velocity = (vec3){o[23], o[24], o[25]};
        e->active = o[26] != 0.0;
        e->deactivation_time = o[27];
    }
}

uint32_t orc_broad_pairs(uint32_t* out, uint32_t cap) {
    Entity** all = entity_get_all();
    Broad_Collision_Pair* pairs = broad_get_collision_pairs(all);
    uint32_t n = (uint32_t)array_length(pairs);
    // eid -> index: ids are assigned in creation order but keep counting across resets
    for (uint32_t k = 0; k < n && k < cap; ++k) {
        uint32_t a = 0, b = 0;
        for (size_t i = 0; i < g_ids.size(); ++i) {
            if (g_ids[i] == pairs[k].e1_id) a = (uint32_t)i;
            if (g_ids[i] == pairs[k].e2_id) b = (uint32_t)i;
        }
        out[2 * k] = a;
        out[2 * k + 1] = b;
    }
    array_free(pairs);
    array_free(all);
    return n;
}

uint32_t orc_contacts(int e1, int e2, double* out, uint32_t cap) {
    Entity* a = ent(e1);
    Entity* b = ent(e2);
    colliders_update(a->colliders, a->world_position, &a->world_rotation);
    colliders_update(b->colliders, b->world_position, &b->world_rotation);
    Collider_Contact* contacts = colliders_get_contacts(a->colliders, b->colliders);
    uint32_t n = (uint32_t)array_length(contacts);
    for (uint32_t k = 0; k < n && k < cap; ++k) {
        double* o = out + (size_t)k * ORC_CONTACT_DOUBLES;
        o[0] = contacts[k].collision_point1.x; o[1] = contacts[k].collision_point1.y; o[2] = contacts[k].collision_point1.z;
        o[3] = contacts[k].collision_point2.x; o[4] = contacts[k].collision_point2.y; o[5] = contacts[k].collision_point2.z;
        o[6] = contacts[k].normal.x; o[7] = contacts[k].normal.y; o[8] = contacts[k].normal.z;
    }
    array_free(contacts);
    return n;
}

uint32_t orc_manifold(int e1, int e2, const double* normal, double penetration, double* out, uint32_t cap) {
    Entity* a = ent(e1);
    Entity* b = ent(e2);
    colliders_update(a->colliders, a->world_position, &a->world_rotation);
    colliders_update(b->colliders, b->world_position, &b->world_rotation);
    Collider_Contact* contacts = array_new(Collider_Contact);
    vec3 n;
    n.x = normal[0];
    n.y = normal[1];
    n.z = normal[2];
    clipping_get_contact_manifold(&a->colliders[0], &b->colliders[0], n, penetration, &contacts);
    uint32_t cnt = (uint32_t)array_length(contacts);
    for (uint32_t k = 0; k < cnt && k < cap; ++k) {
        double* o = out + (size_t)k * ORC_CONTACT_DOUBLES;
        o[0] = contacts[k].collision_point1.x; o[1] = contacts[k].collision_point1.y; o[2] = contacts[k].collision_point1.z;
        o[3] = contacts[k].collision_point2.x; o[4] = contacts[k].collision_point2.y; o[5] = contacts[k].collision_point2.z;
        o[6] = contacts[k].normal.x; o[7] = contacts[k].normal.y; o[8] = contacts[k].normal.z;
    }
    array_free(contacts);
    return cnt;
}

int orc_gjk_epa(int e1, int e2, double* out) {
    Entity* a = ent(e1);
    Entity* b = ent(e2);
    colliders_update(a->colliders, a->world_position, &a->world_rotation);
    colliders_update(b->colliders, b->world_position, &b->world_rotation);
    GJK_Simplex simplex;
    if (!gjk_collides(&a->colliders[0], &b->colliders[0], &simplex)) return 0;
    vec3 normal;
    r64 pen;
    if (!epa(&a->colliders[0], &b->colliders[0], &simplex, &normal, &pen)) return 2;
    out[0] = normal.x; out[1] = normal.y; out[2] = normal.z; out[3] = pen;
    return 1;
}

// The reference's OBJ reader (obj_parse, src/render/obj.cpp:7-80): the face-corner positions it
// emits, 3 floats each, in its order; returns their number (only the first `cap` are written).
uint32_t orc_obj_parse(const char* path, float* out, uint32_t cap) {
    Vertex* vertices = nullptr;
    u32* indices = nullptr;
    obj_parse(path, &vertices, &indices);
    const uint32_t n = (uint32_t)array_length(vertices);
    for (uint32_t i = 0; i < n && i < cap; ++i) {
        out[3 * i + 0] = vertices[i].position.x;
        out[3 * i + 1] = vertices[i].position.y;
        out[3 * i + 2] = vertices[i].position.z;
    }
    array_free(vertices);
    array_free(indices);
    return n;
}

}  // extern "C"
