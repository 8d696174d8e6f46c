/*
 * Drop-in boundary for existing raw-physics callers (C++ only).
 *
 * raw-physics is compiled as C++, so its step entry points are C++-mangled:
 *   void pbd_simulate(r64 dt, Entity** entities, u32 num_substeps, u32 num_pos_iters, boolean enable_collisions);
 *   void pbd_simulate_with_constraints(r64 dt, Entity** entities, Constraint* external_constraints,
 *                                      u32 num_substeps, u32 num_pos_iters, boolean enable_collisions);
 *   (src/physics/pbd.h:93-94)
 * librawphys_gb300.so exports both symbols with the same mangled names, so a caller that links it in
 * place of src/physics/pbd.cpp runs every step on the GPU unchanged.
 *
 * The struct layouts below restate the reference's Entity (src/entity.h:17-47, 504 bytes),
 * Collider (src/physics/collider.h:5-44, 64 bytes), Physics_Force (entity.h:11-15) and Constraint
 * (src/physics/pbd.h:22-91, 144 bytes), with the reference's packed FP64 vectors
 * (include/gm.h:10-136); only the names Entity and Constraint take part in the mangled signatures.
 * Arrays are the reference's light_arrays: a {size_t capacity; size_t length;} header directly in
 * front of the first element (include/light_array.h:68-71).
 *
 * Contract (as the reference's): the caller owns the entities; dt <= 0 is a no-op; every Entity
 * field the reference writes (pose, velocities, previous pose and velocities, active,
 * deactivation_time) is written back, and so are the colliders' transformed vertices and normals.
 * The external constraints are read only. Errors the reference would assert on are reported on
 * stderr and leave the entities untouched.
 * Transformed geometry: every entity's is written at its final pose (colliders_update computed on
 * the device in FP64), which is what the callers' own colliders_update before the next call computes
 * (src/examples/stack.cpp:88-91). The reference leaves it at the last substep's predicted pose, and
 * only for the bodies of that substep's live pairs (pbd.cpp:598-599); nothing in its step reads it
 * before recomputing it. RP_SHIM_COLLIDERS=none skips the refresh.
 * Transfers: the entities' state is uploaded only when the caller changed it since the last call
 * wrote it back, and forces that are exactly the examples' gravity (0, -g / inverse_mass, 0) at the
 * origin stay on the device as the world's gravity; everything else is uploaded per call.
 * Environment: RP_SHIM_PRECISION=fp64 selects the all-FP64 kernels (default fp32), RP_SHIM_DEVICE
 * the CUDA device (default 0).
 */
#ifndef RP_GB300_COMPAT_H
#define RP_GB300_COMPAT_H
#include <stddef.h>
#include <stdint.h>

#pragma pack(push, 1)
typedef struct { double x, y, z; } rpc_vec3;
typedef struct { double x, y, z, w; } rpc_vec4;
typedef struct { double data[3][3]; } rpc_mat3;
#pragma pack(pop)
typedef struct { double x, y, z, w; } rpc_quat;
typedef struct { uint32_t VAO, VBO, EBO, num_indices; } rpc_mesh;

typedef struct {
    rpc_vec3 position;
    rpc_vec3 force;
    int32_t local_coords;
} rpc_force;

typedef struct {
    uint32_t* elements;
    rpc_vec3 normal;
} rpc_hull_face;

typedef struct {
    rpc_vec3* vertices;
    rpc_vec3* transformed_vertices;
    rpc_hull_face* faces;
    rpc_hull_face* transformed_faces;
    uint32_t** vertex_to_faces;
    uint32_t** vertex_to_neighbors;
    uint32_t** face_to_neighbors;
} rpc_hull;

typedef struct {
    float radius;
    rpc_vec3 center;
} rpc_sphere;

typedef struct {
    int32_t type;   /* 0 sphere, 1 convex hull */
    union {
        rpc_hull convex_hull;
        rpc_sphere sphere;
    };
} rpc_collider;

typedef struct {
    uint64_t id;
    rpc_mesh mesh;
    rpc_vec3 world_position;
    rpc_quat world_rotation;
    rpc_vec3 world_scale;
    rpc_vec4 color;
    rpc_collider* colliders;
    double bounding_sphere_radius;
    rpc_force* forces;
    double inverse_mass;
    rpc_mat3 inertia_tensor;
    rpc_mat3 inverse_inertia_tensor;
    rpc_vec3 angular_velocity;
    rpc_vec3 linear_velocity;
    int32_t fixed;
    int32_t active;
    double deactivation_time;
    double static_friction_coefficient;
    double dynamic_friction_coefficient;
    double restitution_coefficient;
    rpc_vec3 previous_world_position;
    rpc_quat previous_world_rotation;
    rpc_vec3 previous_linear_velocity;
    rpc_vec3 previous_angular_velocity;
} Entity;

typedef struct {
    int32_t type;    /* Constraint_Type: 0 positional, 1 collision, 2 mutual orientation, 3 hinge, 4 spherical */
    uint64_t e1_id;
    uint64_t e2_id;
    union {
        struct { rpc_vec3 r1_lc, r2_lc; double compliance, lambda; rpc_vec3 distance; } positional_constraint;
        struct { rpc_vec3 r1_lc, r2_lc, normal; double lambda_t, lambda_n; } collision_constraint;
        struct { double compliance, lambda; } mutual_orientation_constraint;
        struct {
            rpc_vec3 r1_lc, r2_lc;
            double compliance, lambda_pos;
            int32_t e1_aligned_axis, e2_aligned_axis;
            double lambda_aligned_axes;
            int32_t limited;
            double upper_limit, lower_limit;
            int32_t e1_limit_axis, e2_limit_axis;
            double lambda_limit_axes;
        } hinge_joint_constraint;
        struct {
            rpc_vec3 r1_lc, r2_lc;
            double lambda_pos, lambda_swing, swing_upper_limit, swing_lower_limit;
            int32_t e1_swing_axis, e2_swing_axis;
            double lambda_twist, twist_upper_limit, twist_lower_limit;
            int32_t e1_twist_axis, e2_twist_axis;
        } spherical_joint_constraint;
    };
} Constraint;

#ifdef __cplusplus
static_assert(sizeof(Entity) == 504, "Entity layout must match src/entity.h");
static_assert(sizeof(rpc_collider) == 64, "Collider layout must match src/physics/collider.h");
static_assert(sizeof(Constraint) == 144, "Constraint layout must match src/physics/pbd.h");
static_assert(offsetof(Entity, world_rotation) == 48 && offsetof(Entity, fixed) == 360 &&
              offsetof(Entity, previous_angular_velocity) == 480, "Entity field offsets");

void pbd_simulate(double dt, Entity** entities, uint32_t num_substeps, uint32_t num_pos_iters, int32_t enable_collisions);
void pbd_simulate_with_constraints(double dt, Entity** entities, Constraint* external_constraints, uint32_t num_substeps,
                                   uint32_t num_pos_iters, int32_t enable_collisions);

extern "C" {
/* Releases the drop-in's device world (it is rebuilt on the next call). */
void rp_compat_reset(void);
/* The drop-in's device world (NULL before the first call), for diagnostics through include/rp.h
 * (rp_transfer_bytes, rp_counters, ...). */
struct rp_world* rp_compat_world(void);
}
#endif
#endif
