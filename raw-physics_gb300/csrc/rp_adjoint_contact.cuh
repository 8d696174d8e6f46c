// The collision half of the adjoint substep (rp_adjoint.cuh): broad phase and islands of a frame,
// hull transforms, GJK, EPA, contact-manifold clipping, the contact constraint solve and the
// velocity solver, for one scene on one thread.
//
// Every function is written once for both passes. The scalar pass (S = double) repeats the all-FP64
// step's arithmetic operation for operation, so its trajectory is the FP64 step's. The taped pass
// (S = AVar) computes the same values and records the derivatives of the continuous quantities:
// transformed vertices and face normals, the EPA normal, the clipped contact points, the constraint
// offsets, the solves. Every discrete choice (support vertex, simplex case, EPA face, reference face,
// inside/outside tests, contact acting or not) is taken on values only, identically in both passes.
// GJK and EPA run on values only and keep, for every polytope point, the pair of hull vertices it is
// the difference of; the taped pass rebuilds the returned face's normal from those vertices.
//
// References (raw-physics): broad.cpp:6-116, pbd.cpp:107-154,408-424,477-532,583-611,646-711,
// collider.cpp:409-446,523-571, support.cpp:5-39, gjk.cpp:7-379, epa.cpp:8-237, clipping.cpp:12-341.
#pragma once
#include <float.h>
#include "rp_narrow.cuh"
#include "rp_adjoint.cuh"
#include "rp_launch.h"

namespace rp {

// ---------------------------------------------------------------------------------------------
// Frame start: broad phase (broad.cpp:6-28) and islands with sleeping (broad.cpp:31-116,
// pbd.cpp:477-506), on the scalar state. Pairs are scene-local body indices in the reference order.
__device__ inline bool g_broad_hit(const double* xi, const double* xj, double ri, double rj) {
    const double dx = __dsub_rn(xi[0], xj[0]), dy = __dsub_rn(xi[1], xj[1]), dz = __dsub_rn(xi[2], xj[2]);
    const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
    return __dsqrt_rn(d2) <= __dadd_rn(__dadd_rn(ri, rj), 0.1);
}

__device__ inline int g_broad(const AdjointScene& sc, const AdjGeom& G, const double* st, int2* pairs) {
    int n = 0;
    for (int i = 0; i < sc.nb; ++i)
        for (int j = i + 1; j < sc.nb; ++j) {
            if (!g_broad_hit(st + 13 * i, st + 13 * j, G.radius[sc.body0 + i], G.radius[sc.body0 + j])) continue;
            if (n < sc.pair_cap) pairs[n] = make_int2(i, j);
            else sc.status[0] |= ADJ_ST_PAIRS;
            ++n;
        }
    return min(n, sc.pair_cap);
}

__device__ inline int g_find(int* parent, int x) {
    while (parent[x] != x) x = parent[x];
    return x;
}

__device__ inline void g_islands(const AdjointScene& sc, const double* st, const int2* pairs, int np, double dt) {
    const int nb = sc.nb;
    for (int b = 0; b < nb; ++b) { sc.uf[b] = b; sc.awake[b] = 0; }
    auto unite = [&](int a, int c) {
        if (sc.fixed[a] || sc.fixed[c]) return;
        const int ra = g_find(sc.uf, a), rc = g_find(sc.uf, c);
        if (ra != rc) sc.uf[max(ra, rc)] = min(ra, rc);
    };
    for (int k = 0; k < np; ++k) unite(pairs[k].x, pairs[k].y);
    for (int e = 0; e < sc.ne; ++e) unite(sc.ext[e].e1 - sc.body0, sc.ext[e].e2 - sc.body0);
    for (int b = 0; b < nb; ++b) {
        if (sc.fixed[b]) continue;
        const double* o = st + 13 * b;
        const double lv = vlen(v3<double>(o[7], o[8], o[9])), av = vlen(v3<double>(o[10], o[11], o[12]));
        double d = sc.deact[b];
        if (lv < 0.10 && av < 0.10) d += dt;
        else d = 0.0;
        sc.deact[b] = d;
        if (d < 1.0) sc.awake[g_find(sc.uf, b)] = 1;
    }
    for (int b = 0; b < nb; ++b)
        if (!sc.fixed[b]) sc.active[b] = sc.awake[g_find(sc.uf, b)];
}

// ---------------------------------------------------------------------------------------------
// Per-substep views of the scene's transformed hulls and contacts
template <typename S>
struct GCon {                 // a COLLISION_CONSTRAINT (clipping_contact_to_collision_constraint)
    V3<S> r1, r2, n;
    S ln, lt;
    int a, b;                 // scene-local bodies
};

template <typename S>
struct GClip {                // Sutherland-Hodgman ping-pong buffers and the clip planes
    V3<S> buf[2][CLIP_MAX];
    V3<S> pn[CLIP_MAX], pp[CLIP_MAX];
};

struct GEpa {                 // EPA polytope; every point is tv1[pix.x] - tv2[pix.y]
    V3<double> poly[EPA_MAXV];
    int2 pix[EPA_MAXV];
    uchar4 f[EPA_MAXF];
    V3<double> fn[EPA_MAXF];
    double fd[EPA_MAXF];
    int ex[EPA_MAXE], ey[EPA_MAXE];
};

template <typename S>
struct GScene {
    V3<S>* tv;                // the scene's transformed vertices / normals (scene-relative offsets)
    V3<S>* tn;
    V3<double>* tvv;          // their values
    V3<double>* tnv;
    GCon<S>* con;
    int ncon;
    GClip<S>* clip;
    GEpa* epa;
    int* stamp;               // substep counter shared by both passes (bodies transformed in a substep carry its number)
};

template <typename S>
struct GHull {
    Shape sh;
    const V3<S>* tv;
    const V3<S>* tn;
    const V3<double>* tvv;
    const V3<double>* tnv;
};

// collider_update (collider.cpp:409-446) for every hull of body i. The model matrix is translation
// times rotation with a (0 0 0 1) last row, so the reference's 4x4 product and divide by w reduce,
// operation for operation, to (v.x R00 + v.y R01) + v.z R02 + x and (R00 n.x + R01 n.y) + R02 n.z.
template <typename S>
__device__ __noinline__ void g_transform(const AdjointScene& sc, const AdjGeom& G, const GBody<S>& B, int i, GScene<S>& X) {
    const M3<S> R = qmat3(B.q);
    const int slot = sc.body0 + i;
    for (int c = G.col_start[slot]; c < G.col_start[slot + 1]; ++c) {
        const Collider col = G.colliders[c];
        if (col.type != COL_HULL) continue;
        const Shape sh = G.shapes[col.shape];
        const int tv = col.tv_off - sc.tv0, tn = col.tn_off - sc.tn0;
        for (int k = 0; k < sh.nv; ++k) {
            const double* v = G.shape_verts + 3 * (sh.vert_off + k);
            const S vx = S(v[0]), vy = S(v[1]), vz = S(v[2]);
            const V3<S> t = v3<S>(vx * R.d[0][0] + vy * R.d[0][1] + vz * R.d[0][2] + B.x.x,
                                  vx * R.d[1][0] + vy * R.d[1][1] + vz * R.d[1][2] + B.x.y,
                                  vx * R.d[2][0] + vy * R.d[2][1] + vz * R.d[2][2] + B.x.z);
            X.tv[tv + k] = t;
            X.tvv[tv + k] = vval(t);
        }
        for (int k = 0; k < sh.nf; ++k) {
            const double* nn = G.face_normal + 3 * (sh.face_off + k);
            const S nx = S(nn[0]), ny = S(nn[1]), nz = S(nn[2]);
            const V3<S> t = vnorm(v3<S>(R.d[0][0] * nx + R.d[0][1] * ny + R.d[0][2] * nz,
                                        R.d[1][0] * nx + R.d[1][1] * ny + R.d[1][2] * nz,
                                        R.d[2][0] * nx + R.d[2][1] * ny + R.d[2][2] * nz));
            X.tn[tn + k] = t;
            X.tnv[tn + k] = vval(t);
        }
    }
}

// support_point_get_index (support.cpp:5-14): strict >, the first maximum wins
__device__ inline int g_support(const V3<double>* tv, int nv, V3<double> d) {
    double best = -DBL_MAX;
    int bi = 0;
    for (int k = 0; k < nv; ++k) {
        const double dot = vdot(tv[k], d);
        if (dot > best) { best = dot; bi = k; }
    }
    return bi;
}

template <typename S>
__device__ inline V3<double> g_mink(const GHull<S>& a, const GHull<S>& b, V3<double> d, int2& ix) {
    const int i = g_support(a.tvv, a.sh.nv, d), j = g_support(b.tvv, b.sh.nv, vscale(-1.0, d));
    ix = make_int2(i, j);
    return vsub(a.tvv[i], b.tvv[j]);
}

// gjk_collides (gjk.cpp:350-379) on values; ix: the vertex pair of each simplex point
template <typename S>
__device__ __noinline__ bool g_gjk(const GHull<S>& c1, const GHull<S>& c2, Simplex<double>& s, int2 (&ix)[4]) {
    int2 id;
    s.a = g_mink(c1, c2, v3<double>(0, 0, 1), id);
    ix[0] = id;
    s.b = s.c = s.d = v3<double>(0, 0, 0);
    ix[1] = ix[2] = ix[3] = make_int2(0, 0);
    s.num = 1;
    V3<double> dir = vscale(-1.0, s.a);
    for (int it = 0; it < 100; ++it) {
        const V3<double> p = g_mink(c1, c2, dir, id);
        if (vdot(p, dir) < 0.0) return false;
        if (s.num == 1) { s.b = s.a; ix[1] = ix[0]; }
        else if (s.num == 2) { s.c = s.b; s.b = s.a; ix[2] = ix[1]; ix[1] = ix[0]; }
        else { s.d = s.c; s.c = s.b; s.b = s.a; ix[3] = ix[2]; ix[2] = ix[1]; ix[1] = ix[0]; }
        s.a = p;
        ix[0] = id;
        s.num++;
        const V3<double> old[4] = {s.a, s.b, s.c, s.d};
        const int2 oix[4] = {ix[0], ix[1], ix[2], ix[3]};
        const bool hit = do_simplex(s, dir);
        // do_simplex keeps a subset of the points, reordered: carry their vertex pairs along
        const V3<double> now[4] = {s.a, s.b, s.c, s.d};
        for (int k = 0; k < 4; ++k)
            for (int m = 0; m < 4; ++m)
                if (veq(now[k], old[m])) { ix[k] = oix[m]; break; }
        if (hit) return true;
    }
    return false;
}

// get_face_normal_and_distance_to_origin (epa.cpp:32-77)
__device__ inline void g_epa_face(GEpa& E, int fi, int npoly) {
    const uchar4 f = E.f[fi];
    const V3<double> a = E.poly[f.x], b = E.poly[f.y], c = E.poly[f.z];
    V3<double> n = vnorm(vcross(vsub(b, a), vsub(c, a)));
    double d = vdot(n, a);
    if (d < -0.0) {
        n = vinv(n);
        d = -d;
    } else if (d >= -0.0 && d <= 0.0) {
        for (int i = 0; i < npoly; ++i) {
            const double ad = vdot(n, E.poly[i]);
            if (ad < -0.0 || ad > 0.0) {
                n = ad < -0.0 ? n : vinv(n);
                break;
            }
        }
    }
    E.fn[fi] = n;
    E.fd[fi] = d;
}

// add_edge (epa.cpp:79-110): remove the first equal edge (by index or by endpoint position, either
// orientation), moving the last edge into its slot; otherwise append
__device__ inline bool g_epa_edge(GEpa& E, int& ne, int x, int y) {
    const V3<double> px = E.poly[x], py = E.poly[y];
    for (int k = 0; k < ne; ++k) {
        const int a = E.ex[k], b = E.ey[k];
        if ((a == x && b == y) || (a == y && b == x) || (veq(E.poly[a], px) && veq(E.poly[b], py)) ||
            (veq(E.poly[a], py) && veq(E.poly[b], px))) {
            E.ex[k] = E.ex[ne - 1];
            E.ey[k] = E.ey[ne - 1];
            --ne;
            return true;
        }
    }
    if (ne >= EPA_MAXE) return false;
    E.ex[ne] = x;
    E.ey[ne] = y;
    ++ne;
    return true;
}

// epa (epa.cpp:118-237) on values. Returns true when converged, with the face whose normal is the
// result; false when it did not converge (the pair then has no contacts) or outgrew its storage.
template <typename S>
__device__ __noinline__ bool g_epa(GEpa& E, const GHull<S>& c1, const GHull<S>& c2, const Simplex<double>& s, const int2 (&ix)[4],
                      uchar4& face, int& npoly, bool& overflow) {
    overflow = false;
    E.poly[0] = s.a; E.poly[1] = s.b; E.poly[2] = s.c; E.poly[3] = s.d;
    for (int k = 0; k < 4; ++k) E.pix[k] = ix[k];
    E.f[0] = make_uchar4(0, 1, 2, 0);
    E.f[1] = make_uchar4(0, 2, 3, 0);
    E.f[2] = make_uchar4(0, 3, 1, 0);
    E.f[3] = make_uchar4(1, 2, 3, 0);
    int nf = 4;
    npoly = 4;
    for (int k = 0; k < 4; ++k) g_epa_face(E, k, 4);
    double md = DBL_MAX;
    int mi = -1;
    for (int i = 0; i < nf; ++i)
        if (E.fd[i] < md) { md = E.fd[i]; mi = i; }
    V3<double> min_n = mi < 0 ? v3<double>(0, 0, 0) : E.fn[mi];
    uchar4 min_f = mi < 0 ? E.f[0] : E.f[mi];
    double min_d = md;
    for (int it = 0; it < 100; ++it) {
        int2 id;
        const V3<double> sp = g_mink(c1, c2, min_n, id);
        const double d = vdot(min_n, sp);
        if (fabs(d - min_d) < 0.0001) {
            face = min_f;
            return true;
        }
        const int np = npoly;
        if (np >= EPA_MAXV) { overflow = true; return false; }
        E.poly[np] = sp;
        E.pix[np] = id;
        npoly = np + 1;
        for (int i = 0; i < nf; ++i) {
            uchar4 f = E.f[i];
            V3<double> cen = vadd(vadd(E.poly[f.y], E.poly[f.z]), E.poly[f.x]);
            cen = vscale(1.0 / 3.0, cen);
            f.w = vdot(E.fn[i], vsub(sp, cen)) > 0.0 ? 1 : 0;
            E.f[i] = f;
        }
        int ne = 0;
        bool ok = true;
        for (int i = 0; i < nf;) {
            const uchar4 f = E.f[i];
            if (f.w) {
                ok = g_epa_edge(E, ne, f.x, f.y) && ok;
                ok = g_epa_edge(E, ne, f.y, f.z) && ok;
                ok = g_epa_edge(E, ne, f.z, f.x) && ok;
                --nf;
                E.f[i] = E.f[nf];
                E.fd[i] = E.fd[nf];
                E.fn[i] = E.fn[nf];
            } else {
                ++i;
            }
        }
        if (!ok || nf + ne > EPA_MAXF) { overflow = true; return false; }
        for (int k = 0; k < ne; ++k) {
            E.f[nf + k] = make_uchar4((unsigned char)E.ex[k], (unsigned char)E.ey[k], (unsigned char)np, 0);
            g_epa_face(E, nf + k, np + 1);
        }
        nf += ne;
        md = DBL_MAX;
        mi = -1;
        for (int i = 0; i < nf; ++i)
            if (E.fd[i] < md) { md = E.fd[i]; mi = i; }
        min_d = md;
        if (mi >= 0) { min_n = E.fn[mi]; min_f = E.f[mi]; }
    }
    return false;
}

// The EPA normal of face f, rebuilt from its hull vertices (the taped pass records its derivatives)
template <typename S>
__device__ __noinline__ V3<S> g_epa_normal(const GEpa& E, uchar4 f, int npoly, const GHull<S>& c1, const GHull<S>& c2) {
    auto P = [&](int k) { return vsub(c1.tv[E.pix[k].x], c2.tv[E.pix[k].y]); };
    const V3<S> a = P(f.x), b = P(f.y), c = P(f.z);
    V3<S> n = vnorm(vcross(vsub(b, a), vsub(c, a)));
    const double d = val(vdot(n, a));
    if (d < -0.0) {
        n = vinv(n);
    } else if (d >= -0.0 && d <= 0.0) {
        const V3<double> nv = vval(n);
        for (int i = 0; i < npoly; ++i) {
            const double ad = vdot(nv, E.poly[i]);
            if (ad < -0.0 || ad > 0.0) {
                if (!(ad < -0.0)) n = vinv(n);
                break;
            }
        }
    }
    return n;
}

// ---------------------------------------------------------------------------------------------
// Clipping (clipping.cpp:12-113), the float roundings kept
template <typename S>
__device__ __forceinline__ bool g_in_plane(const V3<S>& pn, const V3<S>& pp, const V3<S>& pos) {
    const V3<double> n = vval(pn);
    const float distance = -vdot(n, vval(pp));
    return !(vdot(vval(pos), n) + (double)distance < 0.0);
}

template <typename S>
__device__ __forceinline__ bool g_plane_edge(const V3<S>& pn, const V3<S>& pp, const V3<S>& start, const V3<S>& end, V3<S>& out) {
    const V3<S> ab = vsub(end, start);
    const S ab_p = g_f32(vdot(pn, ab));
    if ((double)fabsf((float)val(ab_p)) > 0.000001) {
        const S distance = g_f32(-vdot(pn, pp));
        const V3<S> p_co = vscale(-distance, pn);
        S fac = g_f32(-vdot(pn, vsub(start, p_co)) / ab_p);
        const S mx = (val(fac) > 0.0) ? fac : S(0.0);
        fac = g_f32((val(mx) < 1.0) ? mx : S(1.0));
        out = vadd(start, vscale(fac, ab));
        return true;
    }
    return false;
}

// One Sutherland-Hodgman pass; -1 when every vertex is inside (the input stays as it is)
template <typename S>
__device__ __noinline__ int g_sh_pass(const V3<S>* in, int n, V3<S>* out, const V3<S>& pn, const V3<S>& pp, bool remove_only, bool& overflow) {
    bool all_in = true;
    for (int j = 0; j < n; ++j) all_in = all_in && g_in_plane(pn, pp, in[j]);
    if (all_in) return -1;
    int m = 0;
    auto emit = [&](const V3<S>& p) {
        if (m < CLIP_MAX) out[m++] = p;
        else overflow = true;
    };
    for (int j = 0; j < n; ++j) {
        const V3<S> end = in[j], start = in[j == 0 ? n - 1 : j - 1];
        const bool si = g_in_plane(pn, pp, start), ei = g_in_plane(pn, pp, end);
        V3<S> t;
        if (remove_only) {
            if (ei) emit(end);
        } else if (si && ei) {
            emit(end);
        } else if (si && !ei) {
            if (g_plane_edge(pn, pp, start, end, t)) emit(t);
        } else if (!si && ei) {
            if (g_plane_edge(pn, pp, start, end, t)) emit(t);
            emit(end);
        }
    }
    return m;
}

template <typename S>
__device__ void g_push_contact(const AdjointScene& sc, GScene<S>& X, const GBody<S>& A, const GBody<S>& B, int ia, int ib,
                               const V3<S>& p1, const V3<S>& p2, const V3<S>& n, int& npair) {
    // clipping_contact_to_collision_constraint (pbd.cpp:408-424); at most CMAX per body pair
    if (npair >= CMAX) { sc.status[0] |= ADJ_ST_CONTACTS; return; }
    if (X.ncon >= sc.contact_cap) { sc.status[0] |= ADJ_ST_CONTACTS; return; }
    GCon<S>& c = X.con[X.ncon++];
    ++npair;
    c.r1 = qrotate(qinverse(A.q), vsub(p1, A.x));
    c.r2 = qrotate(qinverse(B.q), vsub(p2, B.x));
    c.n = n;
    c.ln = S(0.0);
    c.lt = S(0.0);
    c.a = ia;
    c.b = ib;
}

__device__ __forceinline__ int g_csr_len(const int32_t* start, int row) { return start[row + 1] - start[row]; }

// convex_convex_contact_manifold (clipping.cpp:249-341)
template <typename S>
__device__ __noinline__ void g_manifold(const AdjointScene& sc, const AdjGeom& G, GScene<S>& X, const GHull<S>& h1, const GHull<S>& h2,
                           const V3<S>& normal, const GBody<S>& A, const GBody<S>& B, int ia, int ib, int& npair) {
    const V3<S> inv_n = vinv(normal);
    const V3<double> nd = vval(normal), ind = vval(inv_n);
    const int s1 = g_support(h1.tvv, h1.sh.nv, nd), s2 = g_support(h2.tvv, h2.sh.nv, ind);
    const int32_t* cs = G.csr_start;
    const int32_t* cd = G.csr_data;
    // get_face_with_most_fitting_normal over vertex -> faces (first maximum wins)
    auto best_face = [&](const GHull<S>& h, int v2f, V3<double> dir) {
        double best = -DBL_MAX;
        int bk = 0;
        for (int k = 0; k < g_csr_len(cs, v2f); ++k) {
            const double p = vdot(h.tnv[cd[cs[v2f] + k]], dir);
            if (p > best) { best = p; bk = k; }
        }
        return cd[cs[v2f] + bk];
    };
    const int f1 = best_face(h1, h1.sh.v2f_off + s1, nd), f2 = best_face(h2, h2.sh.v2f_off + s2, ind);
    // get_edge_with_most_fitting_normal: candidates in (i, j, normal / inverted) order
    const int v2n1 = h1.sh.v2n_off + s1, v2n2 = h2.sh.v2n_off + s2;
    const int nn1 = g_csr_len(cs, v2n1), nn2 = g_csr_len(cs, v2n2);
    const V3<double> sp1v = h1.tvv[s1], sp2v = h2.tvv[s2];
    double bestE = -DBL_MAX;
    int bestK = -1;
    for (int k = 0; k < nn1 * nn2; ++k) {
        const int i = k / nn2, j = k % nn2;
        const V3<double> e1 = vsub(sp1v, h1.tvv[cd[cs[v2n1] + i]]);
        const V3<double> e2 = vsub(sp2v, h2.tvv[cd[cs[v2n2] + j]]);
        const V3<double> cn = vnorm(vcross(e1, e2));
        const V3<double> ci = vinv(cn);
        const double d0 = vdot(cn, nd);
        if (d0 > bestE) { bestE = d0; bestK = 2 * k; }
        const double d1 = vdot(ci, nd);
        if (d1 > bestE) { bestE = d1; bestK = 2 * k + 1; }
    }
    V3<S> edge_normal = v3<S>(S(0.0), S(0.0), S(0.0));
    int ei = 0, ej = 0;
    if (bestK >= 0) {
        const int k = bestK >> 1;
        ei = cd[cs[v2n1] + k / nn2];
        ej = cd[cs[v2n2] + k % nn2];
        const V3<S> e1 = vsub(h1.tv[s1], h1.tv[ei]);
        const V3<S> e2 = vsub(h2.tv[s2], h2.tv[ej]);
        edge_normal = vnorm(vcross(e1, e2));
        if (bestK & 1) edge_normal = vinv(edge_normal);
    }
    const double d1 = vdot(h1.tnv[f1], nd), d2 = vdot(h2.tnv[f2], ind), de = vdot(vval(edge_normal), nd);
    if (de > d1 + 0.0001 && de > d2 + 0.0001) {
        // collision_distance_between_skew_lines (clipping.cpp:210-239)
        const V3<S> p1 = h1.tv[s1], dd1 = vsub(h1.tv[ei], p1);
        const V3<S> p2 = h2.tv[s2], dd2 = vsub(h2.tv[ej], p2);
        const S nA = dd1.x * dd2.x + dd1.y * dd2.y + dd1.z * dd2.z;
        const S nB = dd2.x * dd2.x + dd2.y * dd2.y + dd2.z * dd2.z;
        const S mA = -dd1.x * dd1.x - dd1.y * dd1.y - dd1.z * dd1.z;
        const S mB = -dd2.x * dd1.x - dd2.y * dd1.y - dd2.z * dd1.z;
        const S rA = -dd1.x * p2.x + dd1.x * p1.x - dd1.y * p2.y + dd1.y * p1.y - dd1.z * p2.z + dd1.z * p1.z;
        const S rB = -dd2.x * p2.x + dd2.x * p1.x - dd2.y * p2.y + dd2.y * p1.y - dd2.z * p2.z + dd2.z * p1.z;
        const S den = (nA * mB) - (nB * mA);
        if (val(den) == 0.0) { sc.status[0] |= ADJ_ST_NARROW; return; }
        const S nn = ((rA * mB) - (rB * mA)) / den;
        const S mm = ((nA * rB) - (nB * rA)) / den;
        const V3<S> l1 = vadd(p1, vscale(mm, dd1));
        const V3<S> l2 = vadd(p2, vscale(nn, dd2));
        g_push_contact(sc, X, A, B, ia, ib, l1, l2, normal, npair);
        return;
    }
    const bool ref1 = d1 > d2;
    const GHull<S>& rh = ref1 ? h1 : h2;
    const GHull<S>& ih = ref1 ? h2 : h1;
    const int rf = ref1 ? f1 : f2, inf = ref1 ? f2 : f1;
    const int32_t* fes = G.face_elem_start;
    GClip<S>& C = *X.clip;
    bool overflow = false;
    // incident polygon and boundary planes (build_boundary_planes, clipping.cpp:121-134)
    const int fs_i = fes[ih.sh.elem_off + inf];
    int ninc = fes[ih.sh.elem_off + inf + 1] - fs_i;
    if (ninc > CLIP_MAX) { overflow = true; ninc = CLIP_MAX; }
    for (int k = 0; k < ninc; ++k) C.buf[0][k] = ih.tv[G.face_elem[fs_i + k]];
    const int f2n_row = rh.sh.f2n_off + rf;
    int npl = g_csr_len(cs, f2n_row);
    if (npl > CLIP_MAX) { overflow = true; npl = CLIP_MAX; }
    for (int k = 0; k < npl; ++k) {
        const int nf = cd[cs[f2n_row] + k];
        C.pp[k] = rh.tv[G.face_elem[fes[rh.sh.elem_off + nf]]];
        C.pn[k] = vinv(rh.tn[nf]);
    }
    int n = ninc, cur = 0;
    for (int p = 0; p < npl; ++p) {
        if (n == 0) break;
        const int m = g_sh_pass(C.buf[cur], n, C.buf[cur ^ 1], C.pn[p], C.pp[p], false, overflow);
        if (m >= 0) { n = m; cur ^= 1; }
    }
    const V3<S> ref_n = vinv(rh.tn[rf]);
    const V3<S> ref_p = rh.tv[G.face_elem[fes[rh.sh.elem_off + rf]]];
    if (n > 0) {
        const int m = g_sh_pass(C.buf[cur], n, C.buf[cur ^ 1], ref_n, ref_p, true, overflow);
        if (m >= 0) { n = m; cur ^= 1; }
    }
    if (overflow) sc.status[0] |= ADJ_ST_NARROW;
    // contacts from the kept points (clipping.cpp:302-327)
    for (int k = 0; k < n; ++k) {
        const V3<S> pt = C.buf[cur][k];
        const S dd = vdot(vscale(S(-1.0), ref_n), ref_p);
        const V3<S> cp = vsub(pt, vscale(vdot(ref_n, pt) + dd, ref_n));
        const V3<S> diff = vsub(pt, cp);
        S pen;
        V3<S> c1, c2;
        if (ref1) {
            pen = vdot(diff, normal);
            c1 = vsub(pt, vscale(pen, normal));
            c2 = pt;
        } else {
            pen = -vdot(diff, normal);
            c1 = pt;
            c2 = vadd(pt, vscale(pen, normal));
        }
        if (val(pen) < 0.0) g_push_contact(sc, X, A, B, ia, ib, c1, c2, normal, npair);
    }
}

// The contacts of one broad-phase pair (colliders_get_contacts, collider.cpp:523-571; hulls only)
template <typename S>
__device__ __noinline__ void g_pair_contacts(const AdjointScene& sc, const AdjGeom& G, GScene<S>& X, const GBody<S>* B, int ia, int ib) {
    const int sa = sc.body0 + ia, sb = sc.body0 + ib;
    int npair = 0;
    for (int ca = G.col_start[sa]; ca < G.col_start[sa + 1]; ++ca)
        for (int cb = G.col_start[sb]; cb < G.col_start[sb + 1]; ++cb) {
            const Collider c1 = G.colliders[ca], c2 = G.colliders[cb];
            if (c1.type != COL_HULL || c2.type != COL_HULL) { sc.status[0] |= ADJ_ST_UNSUPPORTED; continue; }
            GHull<S> h1, h2;
            h1.sh = G.shapes[c1.shape];
            h2.sh = G.shapes[c2.shape];
            h1.tv = X.tv + (c1.tv_off - sc.tv0); h1.tn = X.tn + (c1.tn_off - sc.tn0);
            h1.tvv = X.tvv + (c1.tv_off - sc.tv0); h1.tnv = X.tnv + (c1.tn_off - sc.tn0);
            h2.tv = X.tv + (c2.tv_off - sc.tv0); h2.tn = X.tn + (c2.tn_off - sc.tn0);
            h2.tvv = X.tvv + (c2.tv_off - sc.tv0); h2.tnv = X.tnv + (c2.tn_off - sc.tn0);
            Simplex<double> s;
            int2 ix[4];
            if (!g_gjk(h1, h2, s, ix)) continue;
            uchar4 face;
            int npoly = 0;
            bool overflow = false;
            if (!g_epa(*X.epa, h1, h2, s, ix, face, npoly, overflow)) {
                if (overflow) sc.status[0] |= ADJ_ST_NARROW;
                continue;
            }
            const V3<S> normal = g_epa_normal(*X.epa, face, npoly, h1, h2);
            g_manifold(sc, G, X, h1, h2, normal, B[ia], B[ib], ia, ib, npair);
        }
}

// ---------------------------------------------------------------------------------------------
// collision_constraint_solve (pbd.cpp:107-154)
template <typename S>
__device__ __noinline__ void g_collision_solve(GBody<S>& a, GBody<S>& b, GCon<S>& c, double h) {
    GPcpd<S> p = g_pcpd(a, b, c.r1, c.r2);
    const S d = vdot(vsub(vadd(a.x, p.r1), vadd(b.x, p.r2)), c.n);
    if (!(val(d) > 0.0)) return;
    const V3<S> dx = vscale(d, c.n);
    S dl = g_pos_dlambda(a, b, p, h, 0.0, c.ln, dx);
    g_pos_apply(a, b, p, dl, dx);
    c.ln = c.ln + dl;
    p = g_pcpd(a, b, c.r1, c.r2);
    const V3<S> p1 = vadd(a.x, p.r1), p2 = vadd(b.x, p.r2);
    dl = g_pos_dlambda(a, b, p, h, 0.0, c.lt, dx);
    const double mus = (val(a.mus) + val(b.mus)) / 2.0;
    if (val(c.lt) + val(dl) > mus * val(c.ln)) {
        const V3<S> t1 = vadd(a.px, qrotate(a.pq, c.r1)), t2 = vadd(b.px, qrotate(b.pq, c.r2));
        const V3<S> dp = vsub(vsub(p1, t1), vsub(p2, t2));
        const V3<S> dpt = vsub(dp, vscale(vdot(dp, c.n), c.n));
        g_pos_apply(a, b, p, dl, dpt);
        c.lt = c.lt + dl;
    }
}

// The velocity solver for one contact (pbd.cpp:646-711)
template <typename S>
__device__ __noinline__ void g_contact_velocity(GBody<S>& a, GBody<S>& b, const GCon<S>& c, double h) {
    const V3<S> r1 = qrotate(a.q, c.r1), r2 = qrotate(b.q, c.r2);
    const M3<S> I1 = world_tensor(a.q, a.Iinv), I2 = world_tensor(b.q, b.Iinv);
    const V3<S> v = vsub(vadd(a.v, vcross(a.w, r1)), vadd(b.v, vcross(b.w, r2)));
    const S vn = vdot(c.n, v);
    const V3<S> vt = vsub(v, vscale(vn, c.n));
    V3<S> dv = v3<S>(S(0.0), S(0.0), S(0.0));
    const S mud = (a.mud + b.mud) / S(2.0);
    const S fn = c.ln / S(h);
    const S x1 = mud * fabs(fn), x2 = vlen(vt);
    S fact = (val(x1) < val(x2)) ? x1 : x2;
    dv = vadd(dv, vscale(-fact, vnorm(vt)));
    const V3<S> vtil = vsub(vadd(a.pv, vcross(a.pw, r1)), vadd(b.pv, vcross(b.pw, r2)));
    const S vntil = vdot(c.n, vtil);
    const S e = a.rest * b.rest;
    const S m = -e * vntil;
    fact = -vn + ((val(m) < 0.0) ? m : S(0.0));
    dv = vadd(dv, vscale(fact, c.n));
    const S w1 = a.invm + vdot(vcross(r1, c.n), mmulv(I1, vcross(r1, c.n)));
    const S w2 = b.invm + vdot(vcross(r2, c.n), mmulv(I2, vcross(r2, c.n)));
    const V3<S> P = vscale(S(1.0) / (w1 + w2), dv);
    if (!a.fixed) {
        a.v = vadd(a.v, vscale(a.invm, P));
        a.w = vadd(a.w, mmulv(I1, vcross(r1, P)));
    }
    if (!b.fixed) {
        b.v = vadd(b.v, vinv(vscale(b.invm, P)));
        b.w = vadd(b.w, vinv(mmulv(I2, vcross(r2, P))));
    }
}

}  // namespace rp
