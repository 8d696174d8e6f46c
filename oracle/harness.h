/*
 * Oracle harness interface — TEST INFRASTRUCTURE ONLY.
 *
 * Two libraries export this same C interface:
 *   oracle/_ref/libref_harness.so  the reference's own physics sources (src/physics/*.cpp,
 *                                  src/entity.cpp, src/quaternion.cpp, src/util.cpp) compiled
 *                                  headless by oracle/Makefile, driven by oracle/ref_harness.cpp;
 *   oracle/_build/liboracle.so     oracle/port/oracle.c, a plain-C FP64 restatement of the same
 *                                  path that keeps the reference's operation order.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load either library, and
 * only as the checker: the product path never links or calls anything under oracle/.
 *
 * The calls mirror what the reference's example scenes do around pbd_simulate
 * (src/examples/stack.cpp:86-104): colliders_update on every entity, a gravity force of
 * -g/inverse_mass per entity, pbd_simulate_with_constraints, then entity_clear_forces.
 * Entities are addressed by their index in creation order (the reference's entity_get_all()
 * order, src/entity.cpp:88, as long as no entity is destroyed).
 */
#ifndef RP_ORACLE_HARNESS_H
#define RP_ORACLE_HARNESS_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Number of doubles per entity in orc_get_state / orc_set_state:
 * pos[3] rot[4](x,y,z,w) v[3] w[3] prev_pos[3] prev_rot[4] prev_v[3] prev_w[3] active deactivation_time */
#define ORC_STATE_DOUBLES 28
/* Number of doubles per contact in orc_contacts: p1[3] p2[3] normal[3] */
#define ORC_CONTACT_DOUBLES 9

void     orc_reset(void);
/* Registers a de-indexed triangle mesh as the reference's OBJ loader produces it
 * (src/render/obj.cpp:45-106): float positions, indices. Returns a mesh handle. */
int      orc_mesh_add(const float* positions, uint32_t num_vertices, const uint32_t* indices, uint32_t num_indices);
/* Pending collider list for the next orc_entity_create (a compound body takes several). */
void     orc_colliders_begin(void);
/* Hull from mesh vertices pre-scaled in FP64 as examples_util.cpp:5-24 does. */
int      orc_colliders_add_hull(int mesh, const double scale[3]);
int      orc_colliders_add_sphere(float radius);
/* entity_create / entity_create_fixed (src/entity.h:52-55). Returns the entity index. */
int      orc_entity_create(const double pos[3], const double rot[4], double mass, int fixed,
                           double static_friction, double dynamic_friction, double restitution);
void     orc_entity_set_velocity(int entity, const double v[3], const double w[3]);
/* Extra force for the next orc_step only (entity_add_force, src/entity.cpp:176). */
void     orc_entity_add_force(int entity, const double position[3], const double force[3], int local_coords);
double   orc_entity_get_inverse_mass(int entity);
void     orc_entity_get_inertia(int entity, double inertia[9], double inverse_inertia[9]);
double   orc_entity_get_radius(int entity);

/* Topology of collider k of an entity (convex hulls): which = 0 face loops, 1 vertex->faces,
 * 2 vertex->neighbours, 3 face->neighbours, as CSR (start gets rows+1 entries; data up to cap).
 * Returns the number of rows; *ndata receives the number of entries. */
int      orc_hull_topology(int entity, int k, int which, int32_t* start, int32_t* data, int32_t cap, int32_t* ndata);
/* Unique vertices (3 each) and face normals (3 each) of collider k; returns nv, *nf receives nf. */
int      orc_hull_geometry(int entity, int k, double* verts, double* normals, int32_t cap_vertices, int32_t cap_faces, int32_t* nf);

/* Constraint initialisers (src/physics/pbd.h:96-102). Axis values follow PBD_Axis_Type. */
int orc_constraint_positional(int e1, int e2, const double r1[3], const double r2[3], double compliance, const double distance[3]);
int orc_constraint_mutual_orientation(int e1, int e2, double compliance);
int orc_constraint_hinge(int e1, int e2, const double r1[3], const double r2[3], double compliance,
                         int e1_axis, int e2_axis, int limited, int e1_limit_axis, int e2_limit_axis,
                         double lower, double upper);
int orc_constraint_spherical(int e1, int e2, const double r1[3], const double r2[3],
                             int e1_swing_axis, int e2_swing_axis, int e1_twist_axis, int e2_twist_axis,
                             double swing_lower, double swing_upper, double twist_lower, double twist_upper);

/* One frame: colliders_update(all), gravity force, pbd_simulate_with_constraints, clear forces.
 * gravity is the magnitude g of a force (0, -g/inverse_mass, 0) added to every entity. */
void     orc_step(double dt, uint32_t num_substeps, uint32_t num_pos_iters, int enable_collisions, double gravity);

/* Port only: the collision constraints of the last substep of the last orc_step, in constraint
 * order: entity pairs (2 each) and r1_lc[3] r2_lc[3] normal[3] lambda_n lambda_t (11 each). */
uint32_t orc_last_contacts(int32_t* pairs, double* out, uint32_t cap);
uint32_t orc_num_entities(void);
/* Port only: which of the reference's assert conditions the steps since orc_reset met (0: none);
 * bits 2 EPA face normal vanishes (epa.cpp:41), 4 EPA polytope coplanar with the origin (epa.cpp:72),
 * 8 parallel skew lines (clipping.cpp:279), 1 any other. */
int      orc_last_error(void);
void     orc_get_state(double* out);
void     orc_set_state(const double* in);

/* broad_get_collision_pairs on the current state; writes entity-index pairs, returns the count
 * (which may exceed cap; only cap pairs are written). */
uint32_t orc_broad_pairs(uint32_t* out_pairs, uint32_t cap);
/* colliders_update on both entities, then colliders_get_contacts (src/physics/collider.cpp:560). */
uint32_t orc_contacts(int e1, int e2, double* out, uint32_t cap);
/* gjk_collides + epa on the first collider of each entity (src/physics/gjk.cpp:350, epa.cpp:118).
 * Returns 0 = no collision, 1 = collision and EPA converged, 2 = collision and EPA failed.
 * out = normal[3], penetration. */
int      orc_gjk_epa(int e1, int e2, double* out);
/* colliders_update on both entities, then clipping_get_contact_manifold (src/physics/clipping.cpp:
 * 343-370) of their first colliders for a given normal (pointing from e1 to e2) and penetration:
 * the manifold the reference builds once EPA has returned that normal. out: ORC_CONTACT_DOUBLES per
 * contact; returns the count. */
uint32_t orc_manifold(int e1, int e2, const double* normal, double penetration, double* out, uint32_t cap);

#ifdef __cplusplus
}
#endif
#endif
