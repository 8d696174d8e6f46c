// Convex-hull topology and entity mass properties (see rp_hull.h).
//
// The order of every list matters downstream: vertex order fixes support-point tie-breaks
// (support.cpp:10), face order and the order inside vertex->faces, vertex->neighbours and
// face->neighbours fix the clipping's reference-face, edge and clip-plane choices
// (clipping.cpp:121-200). Each list is therefore produced in the order the reference builds it.
#include "rp_hull.h"
#include <array>
#include <cfloat>
#include <cmath>
#include <map>

namespace rp {
namespace {

struct P3 { double x, y, z; };
inline P3 sub(P3 a, P3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline P3 cross(P3 a, P3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline double dot(P3 a, P3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline P3 normalize(P3 v) {
    if (!(v.x != 0.0 || v.y != 0.0 || v.z != 0.0)) return {0.0, 0.0, 0.0};
    double l = std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z);
    return {v.x / l, v.y / l, v.z / l};
}

struct Tri { int a, b, c; };

struct Builder {
    std::vector<P3> pts;
    std::vector<Tri> tris;
    std::vector<std::vector<int>> tri_nbr;
    std::vector<char> done;
    std::string err;

    P3 tri_normal(int t) const {
        const Tri& r = tris[(size_t)t];
        return normalize(cross(sub(pts[(size_t)r.b], pts[(size_t)r.a]), sub(pts[(size_t)r.c], pts[(size_t)r.a])));
    }

    // Depth-first collection of the triangles coplanar with `target` (collider.cpp:47-77): a
    // triangle joins when its normal is within 1e-6 of the target's; neighbours are visited in
    // neighbour-list order, so the collected order is the reference's.
    void collect(int t, P3 target, std::vector<int>& out) {
        P3 n = tri_normal(t);
        if (done[(size_t)t]) return;
        double p = dot(n, target);
        if ((p - 1.0) > -0.000001 && (p - 1.0) < 0.000001) {
            out.push_back(t);
            done[(size_t)t] = 1;
            for (int nb : tri_nbr[(size_t)t]) collect(nb, target, out);
        }
    }

    // Boundary loop of a set of coplanar triangles (collider.cpp:93-166): edges shared by two
    // triangles cancel (an unordered removal moves the last edge into the hole), then the loop is
    // chained by swapping each successor into place.
    std::vector<int> boundary(const std::vector<int>& planar) {
        std::vector<std::array<int, 2>> e;
        for (int t : planar) {
            const Tri& r = tris[(size_t)t];
            const std::array<int, 2> cand[3] = {{r.a, r.b}, {r.b, r.c}, {r.c, r.a}};
            for (const auto& c : cand) {
                int hit = -1;
                for (size_t j = 0; j < e.size(); ++j)
                    if ((e[j][0] == c[0] && e[j][1] == c[1]) || (e[j][0] == c[1] && e[j][1] == c[0])) { hit = (int)j; break; }
                if (hit >= 0) {
                    e[(size_t)hit] = e.back();
                    e.pop_back();
                } else {
                    e.push_back(c);
                }
            }
        }
        for (size_t i = 0; i < e.size(); ++i) {
            const std::array<int, 2> cur = e[i];
            for (size_t j = i + 1; j < e.size(); ++j) {
                std::array<int, 2> c = e[j];
                if (cur[1] != c[0] && cur[1] != c[1]) continue;
                if (cur[1] == c[1]) std::swap(c[0], c[1]);
                std::array<int, 2> tmp = e[i + 1];
                e[i + 1] = c;
                e[j] = tmp;
            }
        }
        if (e.empty() || e[0][0] != e.back()[1]) err = "hull face boundary is not a closed loop";
        std::vector<int> loop;
        for (const auto& x : e) loop.push_back(x[0]);
        return loop;
    }
};

bool contains(const std::vector<int>& v, int x) {
    for (int y : v)
        if (y == x) return true;
    return false;
}

}  // namespace

std::string build_hull(const double* vertices, uint32_t nv, const uint32_t* indices, uint32_t ni, Hull& out) {
    if (ni % 3 != 0 || ni == 0 || nv == 0) return "hull needs at least one triangle";
    for (uint32_t i = 0; i < ni; ++i)
        if (indices[i] >= nv) return "hull index out of range";
    Builder B;
    // unique vertices by exact FP64 value, first occurrence first (collider.cpp:200-209)
    std::map<std::array<double, 3>, int> seen;
    std::vector<int> remap(nv);
    for (uint32_t i = 0; i < nv; ++i) {
        std::array<double, 3> key = {vertices[3 * i], vertices[3 * i + 1], vertices[3 * i + 2]};
        if (!(std::isfinite(key[0]) && std::isfinite(key[1]) && std::isfinite(key[2]))) return "hull vertex is not finite";
        auto it = seen.find(key);
        if (it == seen.end()) {
            int id = (int)B.pts.size();
            seen.emplace(key, id);
            B.pts.push_back({key[0], key[1], key[2]});
            remap[i] = id;
        } else {
            remap[i] = it->second;
        }
    }
    for (uint32_t t = 0; t < ni / 3; ++t) B.tris.push_back({remap[indices[3 * t]], remap[indices[3 * t + 1]], remap[indices[3 * t + 2]]});
    const size_t nt = B.tris.size(), np = B.pts.size();
    out = Hull();
    out.v2f.assign(np, {});
    out.v2n.assign(np, {});
    B.tri_nbr.assign(nt, {});
    for (size_t i = 0; i < nt; ++i) {
        const Tri a = B.tris[i];
        for (size_t j = 0; j < nt; ++j) {
            if (i == j) continue;
            const Tri b = B.tris[j];
            bool share = a.a == b.a || a.a == b.b || a.a == b.c || a.b == b.a || a.b == b.b || a.b == b.c ||
                         a.c == b.a || a.c == b.b || a.c == b.c;
            if (share) B.tri_nbr[i].push_back((int)j);
        }
        const int order[6][2] = {{a.a, a.b}, {a.a, a.c}, {a.b, a.a}, {a.b, a.c}, {a.c, a.a}, {a.c, a.b}};
        for (const auto& o : order)
            if (!contains(out.v2n[(size_t)o[0]], o[1])) out.v2n[(size_t)o[0]].push_back(o[1]);
    }
    B.done.assign(nt, 0);
    for (size_t i = 0; i < nt; ++i) {
        if (B.done[i]) continue;
        P3 n = B.tri_normal((int)i);
        std::vector<int> planar;
        B.collect((int)i, n, planar);
        std::vector<int> loop = B.boundary(planar);
        int fi = (int)out.faces.size();
        out.faces.push_back(loop);
        out.normals.push_back(n.x);
        out.normals.push_back(n.y);
        out.normals.push_back(n.z);
        for (int t : planar) {
            out.v2f[(size_t)B.tris[(size_t)t].a].push_back(fi);
            out.v2f[(size_t)B.tris[(size_t)t].b].push_back(fi);
            out.v2f[(size_t)B.tris[(size_t)t].c].push_back(fi);
        }
    }
    if (!B.err.empty()) return B.err;
    const size_t nf = out.faces.size();
    out.f2n.assign(nf, {});
    for (size_t i = 0; i < nf; ++i)
        for (size_t j = 0; j < nf; ++j) {
            if (i == j) continue;
            bool share = false;
            for (int x : out.faces[i]) {
                for (int y : out.faces[j])
                    if (x == y) { share = true; break; }
                if (share) break;
            }
            if (share) out.f2n[i].push_back((int)j);
        }
    for (const P3& p : B.pts) {
        out.verts.push_back(p.x);
        out.verts.push_back(p.y);
        out.verts.push_back(p.z);
    }
    return "";
}

double bounding_radius(const std::vector<ColliderDesc>& cols) {
    double mx = -DBL_MAX;
    for (const ColliderDesc& c : cols) {
        double r;
        if (c.type == 1) {
            r = 0.0;
            for (int i = 0; i < c.hull->nv(); ++i) {
                const double* v = &c.hull->verts[(size_t)(3 * i)];
                double d = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
                if (d > r) r = d;
            }
        } else {
            r = c.radius;
        }
        if (r > mx) mx = r;
    }
    return mx;
}

std::string inertia(const std::vector<ColliderDesc>& cols, double mass, double I[9], double Iinv[9]) {
    for (int k = 0; k < 9; ++k) I[k] = Iinv[k] = 0.0;
    if (cols.size() == 1 && cols[0].type == 0) {
        double v = (2.0 / 5.0) * mass * cols[0].radius * cols[0].radius;
        I[0] = v; I[4] = v; I[8] = v;
    } else {
        unsigned total = 0;
        for (const ColliderDesc& c : cols) {
            if (c.type != 1) return "a compound body may only hold convex hulls (the reference asserts this)";
            total += (unsigned)c.hull->nv();
        }
        double mpv = mass / total;
        for (const ColliderDesc& c : cols)
            for (int j = 0; j < c.hull->nv(); ++j) {
                const double x = c.hull->verts[(size_t)(3 * j)], y = c.hull->verts[(size_t)(3 * j + 1)],
                             z = c.hull->verts[(size_t)(3 * j + 2)];
                I[0] += mpv * (y * y + z * z);
                I[1] += mpv * x * y;
                I[2] += mpv * x * z;
                I[3] += mpv * x * y;
                I[4] += mpv * (x * x + z * z);
                I[5] += mpv * y * z;
                I[6] += mpv * x * z;
                I[7] += mpv * y * z;
                I[8] += mpv * (x * x + y * y);
            }
    }
    // gm_mat3_inverse (include/gm.h:380-405), row-major m[r][c] = I[3r+c]
    const double* m = I;
    double det = m[0] * (m[4] * m[8] - m[7] * m[5]) - m[1] * (m[3] * m[8] - m[5] * m[6]) + m[2] * (m[3] * m[7] - m[4] * m[6]);
    if (det == 0.0) return "inertia tensor is singular";
    double inv = 1 / det;
    Iinv[0] = (m[4] * m[8] - m[7] * m[5]) * inv;
    Iinv[1] = (m[2] * m[7] - m[1] * m[8]) * inv;
    Iinv[2] = (m[1] * m[5] - m[2] * m[4]) * inv;
    Iinv[3] = (m[5] * m[6] - m[3] * m[8]) * inv;
    Iinv[4] = (m[0] * m[8] - m[2] * m[6]) * inv;
    Iinv[5] = (m[3] * m[2] - m[0] * m[5]) * inv;
    Iinv[6] = (m[3] * m[7] - m[6] * m[4]) * inv;
    Iinv[7] = (m[6] * m[1] - m[0] * m[7]) * inv;
    Iinv[8] = (m[0] * m[4] - m[3] * m[1]) * inv;
    return "";
}

}  // namespace rp
