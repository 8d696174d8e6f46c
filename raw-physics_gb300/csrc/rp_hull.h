// Host-side set-up of raw-physics colliders and entities: convex-hull topology, bounding radius,
// point-mass inertia. Runs once per hull / entity, in FP64, keeping the reference's operation order
// (compiled with -ffp-contract=off) so that the device starts from the reference's exact constants.
#pragma once
#include <stdint.h>
#include <string>
#include <vector>

namespace rp {

struct Hull {
    std::vector<double> verts;                 // 3 * nv unique vertices, first-occurrence order
    std::vector<double> normals;               // 3 * nf face normals
    std::vector<std::vector<int>> faces;       // boundary loop of every polygon face
    std::vector<std::vector<int>> v2f;         // vertex -> faces (one entry per incident triangle)
    std::vector<std::vector<int>> v2n;         // vertex -> neighbour vertices
    std::vector<std::vector<int>> f2n;         // face -> faces sharing at least one vertex
    int nv() const { return (int)(verts.size() / 3); }
    int nf() const { return (int)faces.size(); }
};

// collider_convex_hull_create (src/physics/collider.cpp:194-364). Returns "" or an error message
// (where the reference would fail an assert).
std::string build_hull(const double* vertices, uint32_t num_vertices, const uint32_t* indices, uint32_t num_indices,
                       Hull& out);

struct ColliderDesc {
    int type;          // 0 sphere, 1 hull
    const Hull* hull;
    float radius;
};

// colliders_get_bounding_sphere_radius (collider.cpp:178-189, 510-520)
double bounding_radius(const std::vector<ColliderDesc>& cols);
// colliders_get_default_inertia_tensor (collider.cpp:448-494) and gm_mat3_inverse (include/gm.h:380).
// Returns "" or an error message.
std::string inertia(const std::vector<ColliderDesc>& cols, double mass, double I[9], double Iinv[9]);

}  // namespace rp
