/*
 * Oracle port — TEST INFRASTRUCTURE ONLY. A plain-C FP64 restatement of raw-physics'
 * rigid-body step (pbd_simulate_with_constraints, src/physics/pbd.cpp:468-747) and of the
 * set-up it depends on (collider_convex_hull_create, entity_create_ex). It keeps the reference's
 * operation order so that, built with -O2 -ffp-contract=off (oracle/Makefile), it reproduces the
 * reference build bit for bit; tests/test_oracle.py pins it against fixtures generated from the
 * reference's own sources (tests/golden/make_golden.py) and, where the reference checkout exists,
 * against oracle/_ref/libref_harness.so directly.
 *
 * It implements oracle/harness.h. Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline load it; the product path never does.
 *
 * Where the reference aborts on an assert (degenerate EPA face, parallel skew lines, singular
 * inertia) the port records an error in g_error instead; such inputs are outside what the
 * reference can simulate, so no comparison uses them.
 */
#include <stdlib.h>
#include <string.h>
#include <float.h>
#include <stdio.h>
#include "oracle_math.h"
#include "../harness.h"

/* ------------------------------------------------------------------------------------------ */
/* Growable int arrays with the reference's light_array semantics: push at the end, unordered
 * remove that moves the last element into the hole (include/light_array.h:116,146). */
typedef struct { int n, cap; int* a; } ivec;
static void iv_push(ivec* v, int x) {
    if (v->n == v->cap) { v->cap = v->cap ? 2 * v->cap : 8; v->a = (int*)realloc(v->a, sizeof(int) * (size_t)v->cap); }
    v->a[v->n++] = x;
}
static void iv_free(ivec* v) { free(v->a); v->a = NULL; v->n = v->cap = 0; }

typedef struct { int x, y; } i2;
typedef struct { int x, y, z; } i3;

static int g_error = 0;   /* bits: 1 other assert, 2 EPA face normal vanishes (epa.cpp:41),
                           * 4 EPA polytope coplanar with the origin (epa.cpp:72), 8 parallel skew
                           * lines (clipping.cpp:279) */

/* ------------------------------------------------------------------------------------------ */
/* Colliders (src/physics/collider.h:5-44) */
typedef struct {
    ivec elements;
    v3 normal;
} face_t;

typedef struct {
    int type;  /* 0 sphere, 1 convex hull (Collider_Type order) */
    float radius;
    v3 center;
    int nv;
    v3* v;
    v3* tv;
    int nf;
    face_t* f;
    v3* tn;          /* transformed face normals */
    ivec* v2f;       /* vertex -> faces */
    ivec* v2n;       /* vertex -> neighbour vertices */
    ivec* f2n;       /* face -> faces sharing a vertex */
} collider_t;

static int tri_share(i3 a, i3 b) {
    return a.x == b.x || a.x == b.y || a.x == b.z || a.y == b.x || a.y == b.y || a.y == b.z ||
           a.z == b.x || a.z == b.y || a.z == b.z;
}
static int faces_share(const ivec* a, const ivec* b) {
    for (int i = 0; i < a->n; ++i)
        for (int j = 0; j < b->n; ++j)
            if (a->a[i] == b->a[j]) return 1;
    return 0;
}
static int iv_contains(const ivec* v, int x) {
    for (int i = 0; i < v->n; ++i)
        if (v->a[i] == x) return 1;
    return 0;
}

typedef struct { int n, cap; i3* a; } tvec;
static void tv_push(tvec* v, i3 x) {
    if (v->n == v->cap) { v->cap = v->cap ? 2 * v->cap : 8; v->a = (i3*)realloc(v->a, sizeof(i3) * (size_t)v->cap); }
    v->a[v->n++] = x;
}

/* collect_faces_planar_to (src/physics/collider.cpp:47-77) */
static void collect_planar(const v3* hull, const i3* tris, ivec* tri_nbrs, int* processed, int idx, v3 target, tvec* out) {
    const double EPS = 0.000001;
    i3 t = tris[idx];
    v3 n = v_norm(v_cross(v_sub(hull[t.y], hull[t.x]), v_sub(hull[t.z], hull[t.x])));
    if (processed[idx]) return;
    double p = v_dot(n, target);
    if ((p - 1.0) > -EPS && (p - 1.0) < EPS) {
        tv_push(out, t);
        processed[idx] = 1;
        for (int i = 0; i < tri_nbrs[idx].n; ++i) collect_planar(hull, tris, tri_nbrs, processed, tri_nbrs[idx].a[i], target, out);
    }
}

/* create_convex_hull_face (src/physics/collider.cpp:93-166) */
static face_t make_face(const tvec* tris, v3 normal) {
    int n = 0, cap = 16;
    i2* e = (i2*)malloc(sizeof(i2) * (size_t)cap);
    for (int i = 0; i < tris->n; ++i) {
        i3 t = tris->a[i];
        i2 cand[3] = {{t.x, t.y}, {t.y, t.z}, {t.z, t.x}};
        for (int k = 0; k < 3; ++k) {
            int found = -1;
            for (int j = 0; j < n; ++j) {
                if ((e[j].x == cand[k].x && e[j].y == cand[k].y) || (e[j].x == cand[k].y && e[j].y == cand[k].x)) {
                    found = j;
                    break;
                }
            }
            if (found >= 0) {
                n--;
                e[found] = e[n];
            } else {
                if (n == cap) { cap *= 2; e = (i2*)realloc(e, sizeof(i2) * (size_t)cap); }
                e[n++] = cand[k];
            }
        }
    }
    for (int i = 0; i < n; ++i) {
        i2 cur = e[i];
        for (int j = i + 1; j < n; ++j) {
            i2 c = e[j];
            if (cur.y != c.x && cur.y != c.y) continue;
            if (cur.y == c.y) { int tmp = c.x; c.x = c.y; c.y = tmp; }
            i2 tmp = e[i + 1];
            e[i + 1] = c;
            e[j] = tmp;
        }
    }
    if (n == 0 || e[0].x != e[n - 1].y) g_error |= 1;
    face_t f;
    memset(&f, 0, sizeof(f));
    for (int i = 0; i < n; ++i) iv_push(&f.elements, e[i].x);
    f.normal = normal;
    free(e);
    return f;
}

/* collider_convex_hull_create (src/physics/collider.cpp:194-364) */
static collider_t hull_create(const v3* verts, int nverts, const unsigned* idx, int nidx) {
    collider_t c;
    memset(&c, 0, sizeof(c));
    c.type = 1;
    /* unique vertices in first-occurrence order (exact FP64 equality, collider.cpp:200-209) */
    v3* hull = (v3*)malloc(sizeof(v3) * (size_t)(nverts > 0 ? nverts : 1));
    int* remap = (int*)malloc(sizeof(int) * (size_t)(nverts > 0 ? nverts : 1));
    int nh = 0;
    for (int i = 0; i < nverts; ++i) {
        int found = -1;
        for (int j = 0; j < nh; ++j)
            if (v_eq(hull[j], verts[i])) { found = j; break; }
        if (found < 0) { hull[nh] = verts[i]; found = nh++; }
        remap[i] = found;
    }
    int nt = nidx / 3;
    i3* tris = (i3*)malloc(sizeof(i3) * (size_t)(nt > 0 ? nt : 1));
    for (int i = 0; i < nt; ++i) {
        /* the reference looks the position up again, so duplicates map to the first occurrence */
        i3 t = {remap[idx[3 * i]], remap[idx[3 * i + 1]], remap[idx[3 * i + 2]]};
        tris[i] = t;
    }
    ivec* v2f = (ivec*)calloc((size_t)nh, sizeof(ivec));
    ivec* v2n = (ivec*)calloc((size_t)nh, sizeof(ivec));
    ivec* tn = (ivec*)calloc((size_t)(nt > 0 ? nt : 1), sizeof(ivec));
    for (int i = 0; i < nt; ++i) {
        i3 t = tris[i];
        for (int j = 0; j < nt; ++j) {
            if (i == j) continue;
            if (tri_share(t, tris[j])) iv_push(&tn[i], j);
        }
        if (!iv_contains(&v2n[t.x], t.y)) iv_push(&v2n[t.x], t.y);
        if (!iv_contains(&v2n[t.x], t.z)) iv_push(&v2n[t.x], t.z);
        if (!iv_contains(&v2n[t.y], t.x)) iv_push(&v2n[t.y], t.x);
        if (!iv_contains(&v2n[t.y], t.z)) iv_push(&v2n[t.y], t.z);
        if (!iv_contains(&v2n[t.z], t.x)) iv_push(&v2n[t.z], t.x);
        if (!iv_contains(&v2n[t.z], t.y)) iv_push(&v2n[t.z], t.y);
    }
    int nf = 0, fcap = 8;
    face_t* faces = (face_t*)malloc(sizeof(face_t) * (size_t)fcap);
    int* processed = (int*)calloc((size_t)(nt > 0 ? nt : 1), sizeof(int));
    for (int i = 0; i < nt; ++i) {
        if (processed[i]) continue;
        i3 t = tris[i];
        v3 normal = v_norm(v_cross(v_sub(hull[t.y], hull[t.x]), v_sub(hull[t.z], hull[t.x])));
        tvec planar = {0, 0, NULL};
        collect_planar(hull, tris, tn, processed, i, normal, &planar);
        face_t f = make_face(&planar, normal);
        if (nf == fcap) { fcap *= 2; faces = (face_t*)realloc(faces, sizeof(face_t) * (size_t)fcap); }
        int fi = nf;
        faces[nf++] = f;
        for (int j = 0; j < planar.n; ++j) {
            iv_push(&v2f[planar.a[j].x], fi);
            iv_push(&v2f[planar.a[j].y], fi);
            iv_push(&v2f[planar.a[j].z], fi);
        }
        free(planar.a);
    }
    ivec* f2n = (ivec*)calloc((size_t)(nf > 0 ? nf : 1), sizeof(ivec));
    for (int i = 0; i < nf; ++i)
        for (int j = 0; j < nf; ++j) {
            if (i == j) continue;
            if (faces_share(&faces[i].elements, &faces[j].elements)) iv_push(&f2n[i], j);
        }
    for (int i = 0; i < nt; ++i) iv_free(&tn[i]);
    free(tn);
    free(processed);
    free(tris);
    free(remap);
    c.nv = nh;
    c.v = hull;
    c.tv = (v3*)malloc(sizeof(v3) * (size_t)(nh > 0 ? nh : 1));
    memcpy(c.tv, hull, sizeof(v3) * (size_t)nh);
    c.nf = nf;
    c.f = faces;
    c.tn = (v3*)malloc(sizeof(v3) * (size_t)(nf > 0 ? nf : 1));
    for (int i = 0; i < nf; ++i) c.tn[i] = faces[i].normal;
    c.v2f = v2f;
    c.v2n = v2n;
    c.f2n = f2n;
    return c;
}

static void collider_free(collider_t* c) {
    if (c->type != 1) return;
    for (int i = 0; i < c->nv; ++i) { iv_free(&c->v2f[i]); iv_free(&c->v2n[i]); }
    for (int i = 0; i < c->nf; ++i) { iv_free(&c->f2n[i]); iv_free(&c->f[i].elements); }
    free(c->v2f); free(c->v2n); free(c->f2n); free(c->f); free(c->v); free(c->tv); free(c->tn);
}

/* collider_update (src/physics/collider.cpp:409-438) */
static void collider_update(collider_t* c, v3 t, qt q) {
    if (c->type == 1) {
        m4 m = model_matrix_no_scale(q, t);
        for (int i = 0; i < c->nv; ++i) c->tv[i] = m4_transform_point(m, c->v[i]);
        for (int i = 0; i < c->nf; ++i) c->tn[i] = v_norm(m4_transform_dir(m, c->f[i].normal));
    } else {
        c->center = t;
    }
}

/* ------------------------------------------------------------------------------------------ */
/* Entities (src/entity.h:17-47) */
typedef struct { v3 position, force; int local; } force_t;

typedef struct {
    v3 pos; qt rot; v3 v, w;
    v3 ppos; qt prot; v3 pv, pw;
    double radius, invm;
    m3 I, Iinv;
    int fixed, active;
    double deact, mus, mud, rest;
    int ncol;
    collider_t* col;
    int nf, fcap;
    force_t* forces;
} body_t;

typedef struct {
    float* pos;
    unsigned nv;
    unsigned* idx;
    unsigned ni;
} mesh_t;

enum { C_POS = 0, C_COL = 1, C_MO = 2, C_HINGE = 3, C_SPH = 4 };
typedef struct {
    int type, e1, e2;
    v3 r1, r2;
    double compliance;
    v3 distance;            /* positional */
    v3 normal;              /* collision */
    double lambda, lambda_t, lambda_n, lambda_pos, lambda_aligned, lambda_limit, lambda_swing, lambda_twist;
    int a1, a2, limited, l1, l2;   /* hinge axes */
    double lower, upper;
    int s1, s2, t1, t2;            /* spherical axes */
    double slo, shi, tlo, thi;
} constraint_t;

static body_t* g_bodies = NULL;
static int g_nb = 0, g_bcap = 0;
static mesh_t* g_meshes = NULL;
static int g_nm = 0;
static collider_t* g_pending = NULL;
static int g_np = 0, g_pcap = 0;
static constraint_t* g_cons = NULL;
static int g_nc = 0, g_ccap = 0;
static constraint_t* g_last = NULL;   /* collision constraints of the last substep */
static int g_nlast = 0, g_lastcap = 0;

void orc_reset(void) {
    for (int i = 0; i < g_nb; ++i) {
        for (int k = 0; k < g_bodies[i].ncol; ++k) collider_free(&g_bodies[i].col[k]);
        free(g_bodies[i].col);
        free(g_bodies[i].forces);
    }
    free(g_bodies); g_bodies = NULL; g_nb = g_bcap = 0;
    for (int i = 0; i < g_nm; ++i) { free(g_meshes[i].pos); free(g_meshes[i].idx); }
    free(g_meshes); g_meshes = NULL; g_nm = 0;
    for (int i = 0; i < g_np; ++i) collider_free(&g_pending[i]);
    free(g_pending); g_pending = NULL; g_np = g_pcap = 0;
    free(g_cons); g_cons = NULL; g_nc = g_ccap = 0;
    g_error = 0;
}

int orc_mesh_add(const float* positions, uint32_t nv, const uint32_t* indices, uint32_t ni) {
    g_meshes = (mesh_t*)realloc(g_meshes, sizeof(mesh_t) * (size_t)(g_nm + 1));
    mesh_t* m = &g_meshes[g_nm];
    m->pos = (float*)malloc(sizeof(float) * 3 * (size_t)nv);
    memcpy(m->pos, positions, sizeof(float) * 3 * (size_t)nv);
    m->nv = nv;
    m->idx = (unsigned*)malloc(sizeof(unsigned) * (size_t)(ni ? ni : 1));
    memcpy(m->idx, indices, sizeof(unsigned) * (size_t)ni);
    m->ni = ni;
    return g_nm++;
}

void orc_colliders_begin(void) {
    for (int i = 0; i < g_np; ++i) collider_free(&g_pending[i]);
    g_np = 0;
}

static void pending_push(collider_t c) {
    if (g_np == g_pcap) { g_pcap = g_pcap ? 2 * g_pcap : 4; g_pending = (collider_t*)realloc(g_pending, sizeof(collider_t) * (size_t)g_pcap); }
    g_pending[g_np++] = c;
}

int orc_colliders_add_hull(int mesh, const double s[3]) {
    mesh_t* m = &g_meshes[mesh];
    v3* verts = (v3*)malloc(sizeof(v3) * (size_t)(m->nv ? m->nv : 1));
    for (unsigned i = 0; i < m->nv; ++i) {
        v3 p = V3((double)m->pos[3 * i], (double)m->pos[3 * i + 1], (double)m->pos[3 * i + 2]);
        p.x *= s[0];
        p.y *= s[1];
        p.z *= s[2];
        verts[i] = p;
    }
    pending_push(hull_create(verts, (int)m->nv, m->idx, (int)m->ni));
    free(verts);
    return g_np - 1;
}

int orc_colliders_add_sphere(float radius) {
    collider_t c;
    memset(&c, 0, sizeof(c));
    c.type = 0;
    c.radius = radius;
    c.center = V3(0.0, 0.0, 0.0);
    pending_push(c);
    return g_np - 1;
}

/* colliders_get_default_inertia_tensor (src/physics/collider.cpp:448-494) */
static m3 default_inertia(const collider_t* cs, int n, double mass) {
    m3 r;
    memset(&r, 0, sizeof(r));
    if (n == 1 && cs[0].type == 0) {
        double I = (2.0 / 5.0) * mass * cs[0].radius * cs[0].radius;
        r.d[0][0] = I; r.d[1][1] = I; r.d[2][2] = I;
        return r;
    }
    unsigned total = 0;
    for (int i = 0; i < n; ++i) {
        if (cs[i].type != 1) { g_error |= 1; return r; }
        total += (unsigned)cs[i].nv;
    }
    double mpv = mass / total;
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < cs[i].nv; ++j) {
            v3 v = cs[i].v[j];
            r.d[0][0] += mpv * (v.y * v.y + v.z * v.z);
            r.d[0][1] += mpv * v.x * v.y;
            r.d[0][2] += mpv * v.x * v.z;
            r.d[1][0] += mpv * v.x * v.y;
            r.d[1][1] += mpv * (v.x * v.x + v.z * v.z);
            r.d[1][2] += mpv * v.y * v.z;
            r.d[2][0] += mpv * v.x * v.z;
            r.d[2][1] += mpv * v.y * v.z;
            r.d[2][2] += mpv * (v.x * v.x + v.y * v.y);
        }
    return r;
}

/* colliders_get_bounding_sphere_radius (src/physics/collider.cpp:178-189, 510-520) */
static double bounding_radius(const collider_t* cs, int n) {
    double mx = -DBL_MAX;
    for (int i = 0; i < n; ++i) {
        double r;
        if (cs[i].type == 1) {
            r = 0.0;
            for (int j = 0; j < cs[i].nv; ++j) {
                double d = v_len(cs[i].v[j]);
                if (d > r) r = d;
            }
        } else {
            r = cs[i].radius;
        }
        if (r > mx) mx = r;
    }
    return mx;
}

/* entity_create_ex (src/entity.cpp:24-65) */
int orc_entity_create(const double pos[3], const double rot[4], double mass, int fixed, double mus, double mud, double rest) {
    if (g_nb == g_bcap) { g_bcap = g_bcap ? 2 * g_bcap : 16; g_bodies = (body_t*)realloc(g_bodies, sizeof(body_t) * (size_t)g_bcap); }
    body_t* b = &g_bodies[g_nb];
    memset(b, 0, sizeof(*b));
    b->pos = V3(pos[0], pos[1], pos[2]);
    b->rot = Q(rot[0], rot[1], rot[2], rot[3]);
    b->ncol = g_np;
    b->col = (collider_t*)malloc(sizeof(collider_t) * (size_t)(g_np ? g_np : 1));
    memcpy(b->col, g_pending, sizeof(collider_t) * (size_t)g_np);
    g_np = 0;
    b->radius = bounding_radius(b->col, b->ncol);
    if (fixed) {
        b->invm = 0.0;
    } else {
        b->invm = 1.0 / mass;
        b->I = default_inertia(b->col, b->ncol, mass);
        if (!m3_inverse(b->I, &b->Iinv)) g_error |= 1;
    }
    b->fixed = fixed;
    b->active = 1;
    b->deact = 0.0;
    b->mus = mus;
    b->mud = mud;
    b->rest = rest;
    return g_nb++;
}

void orc_entity_set_velocity(int i, const double v[3], const double w[3]) {
    g_bodies[i].v = V3(v[0], v[1], v[2]);
    g_bodies[i].w = V3(w[0], w[1], w[2]);
}

/* entity_add_force (src/entity.cpp:176-191) */
static void add_force(body_t* b, v3 position, v3 force, int local) {
    if (local) {
        force = q_rotate(b->rot, force);
        /* model matrix without translation with unit scale: rotation * I */
        m4 rm = q_mat4(b->rot);
        m4 sc;
        for (int r = 0; r < 4; ++r)
            for (int c = 0; c < 4; ++c) sc.d[r][c] = (r == c) ? 1.0 : 0.0;
        m4 m = m4_mul(rm, sc);
        position = V3(m.d[0][0] * position.x + m.d[0][1] * position.y + m.d[0][2] * position.z + m.d[0][3] * 1.0,
                      m.d[1][0] * position.x + m.d[1][1] * position.y + m.d[1][2] * position.z + m.d[1][3] * 1.0,
                      m.d[2][0] * position.x + m.d[2][1] * position.y + m.d[2][2] * position.z + m.d[2][3] * 1.0);
    }
    if (b->nf == b->fcap) { b->fcap = b->fcap ? 2 * b->fcap : 4; b->forces = (force_t*)realloc(b->forces, sizeof(force_t) * (size_t)b->fcap); }
    b->forces[b->nf].position = position;
    b->forces[b->nf].force = force;
    b->forces[b->nf].local = local;
    b->nf++;
}

void orc_entity_add_force(int i, const double p[3], const double f[3], int local) {
    add_force(&g_bodies[i], V3(p[0], p[1], p[2]), V3(f[0], f[1], f[2]), local);
}

double orc_entity_get_inverse_mass(int i) { return g_bodies[i].invm; }
void orc_entity_get_inertia(int i, double I[9], double Iinv[9]) {
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) { I[3 * r + c] = g_bodies[i].I.d[r][c]; Iinv[3 * r + c] = g_bodies[i].Iinv.d[r][c]; }
}
double orc_entity_get_radius(int i) { return g_bodies[i].radius; }

int orc_hull_topology(int i, int k, int which, int32_t* start, int32_t* data, int32_t cap, int32_t* ndata) {
    const collider_t* c = &g_bodies[i].col[k];
    int rows = (which == 0 || which == 3) ? c->nf : c->nv;
    int32_t n = 0;
    for (int r = 0; r < rows; ++r) {
        const ivec* row = which == 0 ? &c->f[r].elements : which == 1 ? &c->v2f[r] : which == 2 ? &c->v2n[r] : &c->f2n[r];
        if (start) start[r] = n;
        for (int q = 0; q < row->n; ++q) {
            if (data && n < cap) data[n] = row->a[q];
            ++n;
        }
    }
    if (start) start[rows] = n;
    if (ndata) *ndata = n;
    return rows;
}

int orc_hull_geometry(int i, int k, double* verts, double* normals, int32_t capv, int32_t capf, int32_t* nf) {
    const collider_t* c = &g_bodies[i].col[k];
    for (int v = 0; v < c->nv && v < capv; ++v) { verts[3 * v] = c->v[v].x; verts[3 * v + 1] = c->v[v].y; verts[3 * v + 2] = c->v[v].z; }
    for (int j = 0; j < c->nf && j < capf; ++j) { normals[3 * j] = c->f[j].normal.x; normals[3 * j + 1] = c->f[j].normal.y; normals[3 * j + 2] = c->f[j].normal.z; }
    if (nf) *nf = c->nf;
    return c->nv;
}

static constraint_t* new_constraint(int type, int e1, int e2) {
    if (g_nc == g_ccap) { g_ccap = g_ccap ? 2 * g_ccap : 8; g_cons = (constraint_t*)realloc(g_cons, sizeof(constraint_t) * (size_t)g_ccap); }
    constraint_t* c = &g_cons[g_nc++];
    memset(c, 0, sizeof(*c));
    c->type = type;
    c->e1 = e1;
    c->e2 = e2;
    return c;
}

int orc_constraint_positional(int e1, int e2, const double r1[3], const double r2[3], double compliance, const double d[3]) {
    constraint_t* c = new_constraint(C_POS, e1, e2);
    c->r1 = V3(r1[0], r1[1], r1[2]); c->r2 = V3(r2[0], r2[1], r2[2]);
    c->compliance = compliance;
    c->distance = V3(d[0], d[1], d[2]);
    return g_nc - 1;
}
int orc_constraint_mutual_orientation(int e1, int e2, double compliance) {
    constraint_t* c = new_constraint(C_MO, e1, e2);
    c->compliance = compliance;
    return g_nc - 1;
}
int orc_constraint_hinge(int e1, int e2, const double r1[3], const double r2[3], double compliance, int a1, int a2,
                         int limited, int l1, int l2, double lower, double upper) {
    constraint_t* c = new_constraint(C_HINGE, e1, e2);
    c->r1 = V3(r1[0], r1[1], r1[2]); c->r2 = V3(r2[0], r2[1], r2[2]);
    c->compliance = compliance;
    c->a1 = a1; c->a2 = a2; c->limited = limited;
    if (limited) { c->l1 = l1; c->l2 = l2; c->lower = lower; c->upper = upper; }
    return g_nc - 1;
}
int orc_constraint_spherical(int e1, int e2, const double r1[3], const double r2[3], int s1, int s2, int t1, int t2,
                             double slo, double shi, double tlo, double thi) {
    constraint_t* c = new_constraint(C_SPH, e1, e2);
    c->r1 = V3(r1[0], r1[1], r1[2]); c->r2 = V3(r2[0], r2[1], r2[2]);
    c->s1 = s1; c->s2 = s2; c->t1 = t1; c->t2 = t2;
    c->slo = slo; c->shi = shi; c->tlo = tlo; c->thi = thi;
    return g_nc - 1;
}

/* ------------------------------------------------------------------------------------------ */
/* Support mapping (src/physics/support.cpp:5-39) */
static int support_index(const collider_t* c, v3 d) {
    int sel = 0;
    double mx = -DBL_MAX;
    for (int i = 0; i < c->nv; ++i) {
        double dot = v_dot(c->tv[i], d);
        if (dot > mx) { sel = i; mx = dot; }
    }
    return sel;
}
static v3 support(const collider_t* c, v3 d) {
    if (c->type == 1) return c->tv[support_index(c, d)];
    return v_add(c->center, v_scale(c->radius, v_norm(d)));
}
static v3 support_mink(const collider_t* a, const collider_t* b, v3 d) {
    v3 s1 = support(a, d);
    v3 s2 = support(b, v_scale(-1.0, d));
    return v_sub(s1, s2);
}

/* GJK (src/physics/gjk.cpp) */
typedef struct { v3 a, b, c, d; int num; } simplex_t;

static v3 triple_cross(v3 a, v3 b, v3 c) { return v_cross(v_cross(a, b), c); }

static void simplex_add(simplex_t* s, v3 p) {
    switch (s->num) {
    case 1: s->b = s->a; s->a = p; break;
    case 2: s->c = s->b; s->b = s->a; s->a = p; break;
    case 3: s->d = s->c; s->c = s->b; s->b = s->a; s->a = p; break;
    default: g_error |= 1; break;
    }
    s->num++;
}

static int do_simplex_2(simplex_t* s, v3* dir) {
    v3 a = s->a, b = s->b;
    v3 ao = v_inv(a), ab = v_sub(b, a);
    if (v_dot(ab, ao) >= 0.0) { s->a = a; s->b = b; s->num = 2; *dir = triple_cross(ab, ao, ab); }
    else { s->a = a; s->num = 1; *dir = ao; }
    return 0;
}

static int do_simplex_3(simplex_t* s, v3* dir) {
    v3 a = s->a, b = s->b, c = s->c;
    v3 ao = v_inv(a), ab = v_sub(b, a), ac = v_sub(c, a), abc = v_cross(ab, ac);
    if (v_dot(v_cross(abc, ac), ao) >= 0.0) {
        if (v_dot(ac, ao) >= 0.0) { s->a = a; s->b = c; s->num = 2; *dir = triple_cross(ac, ao, ac); }
        else if (v_dot(ab, ao) >= 0.0) { s->a = a; s->b = b; s->num = 2; *dir = triple_cross(ab, ao, ab); }
        else { s->a = a; *dir = ao; }
    } else {
        if (v_dot(v_cross(ab, abc), ao) >= 0.0) {
            if (v_dot(ab, ao) >= 0.0) { s->a = a; s->b = b; s->num = 2; *dir = triple_cross(ab, ao, ab); }
            else { s->a = a; *dir = ao; }
        } else {
            if (v_dot(abc, ao) >= 0.0) { s->a = a; s->b = b; s->c = c; s->num = 3; *dir = abc; }
            else { s->a = a; s->b = c; s->c = b; s->num = 3; *dir = v_inv(abc); }
        }
    }
    return 0;
}

static int do_simplex_4(simplex_t* s, v3* dir) {
    v3 a = s->a, b = s->b, c = s->c, d = s->d;
    v3 ao = v_inv(a), ab = v_sub(b, a), ac = v_sub(c, a), ad = v_sub(d, a);
    v3 abc = v_cross(ab, ac), acd = v_cross(ac, ad), adb = v_cross(ad, ab);
    int info = 0;
    if (v_dot(abc, ao) >= 0.0) info |= 1;
    if (v_dot(acd, ao) >= 0.0) info |= 2;
    if (v_dot(adb, ao) >= 0.0) info |= 4;
    switch (info) {
    case 0: return 1;
    case 1:
        if (v_dot(v_cross(abc, ac), ao) >= 0.0) {
            if (v_dot(ac, ao) >= 0.0) { s->a = a; s->b = c; s->num = 2; *dir = triple_cross(ac, ao, ac); }
            else if (v_dot(ab, ao) >= 0.0) { s->a = a; s->b = b; s->num = 2; *dir = triple_cross(ab, ao, ab); }
            else { s->a = a; *dir = ao; }
        } else {
            if (v_dot(v_cross(ab, abc), ao) >= 0.0) {
                if (v_dot(ab, ao) >= 0.0) { s->a = a; s->b = b; s->num = 2; *dir = triple_cross(ab, ao, ab); }
                else { s->a = a; *dir = ao; }
            } else { s->a = a; s->b = b; s->c = c; s->num = 3; *dir = abc; }
        }
        break;
    case 2:
        if (v_dot(v_cross(acd, ad), ao) >= 0.0) {
            if (v_dot(ad, ao) >= 0.0) { s->a = a; s->b = d; s->num = 2; *dir = triple_cross(ad, ao, ad); }
            else if (v_dot(ac, ao) >= 0.0) {
                /* the reference pairs the AC simplex with the AB direction here (gjk.cpp:213) */
                s->a = a; s->b = c; s->num = 2; *dir = triple_cross(ab, ao, ab);
            } else { s->a = a; *dir = ao; }
        } else {
            if (v_dot(v_cross(ac, acd), ao) >= 0.0) {
                if (v_dot(ac, ao) >= 0.0) { s->a = a; s->b = c; s->num = 2; *dir = triple_cross(ac, ao, ac); }
                else { s->a = a; *dir = ao; }
            } else { s->a = a; s->b = c; s->c = d; s->num = 3; *dir = acd; }
        }
        break;
    case 3:
        if (v_dot(ac, ao) >= 0.0) { s->a = a; s->b = c; s->num = 2; *dir = triple_cross(ac, ao, ac); }
        else { s->a = a; s->num = 1; *dir = ao; }
        break;
    case 4:
        if (v_dot(v_cross(adb, ab), ao) >= 0.0) {
            if (v_dot(ab, ao) >= 0.0) { s->a = a; s->b = b; s->num = 2; *dir = triple_cross(ab, ao, ab); }
            else if (v_dot(ad, ao) >= 0.0) { s->a = a; s->b = d; s->num = 2; *dir = triple_cross(ad, ao, ad); }
            else { s->a = a; *dir = ao; }
        } else {
            if (v_dot(v_cross(ad, adb), ao) >= 0.0) {
                if (v_dot(ad, ao) >= 0.0) { s->a = a; s->b = d; s->num = 2; *dir = triple_cross(ad, ao, ad); }
                else { s->a = a; *dir = ao; }
            } else { s->a = a; s->b = d; s->c = b; s->num = 3; *dir = adb; }
        }
        break;
    case 5:
        if (v_dot(ab, ao) >= 0.0) { s->a = a; s->b = b; s->num = 2; *dir = triple_cross(ab, ao, ab); }
        else { s->a = a; s->num = 1; *dir = ao; }
        break;
    case 6:
        if (v_dot(ad, ao) >= 0.0) { s->a = a; s->b = d; s->num = 2; *dir = triple_cross(ad, ao, ad); }
        else { s->a = a; s->num = 1; *dir = ao; }
        break;
    case 7: s->a = a; s->num = 1; *dir = ao; break;
    }
    return 0;
}

static int gjk(const collider_t* c1, const collider_t* c2, simplex_t* out) {
    simplex_t s;
    memset(&s, 0, sizeof(s));
    s.a = support_mink(c1, c2, V3(0.0, 0.0, 1.0));
    s.num = 1;
    v3 dir = v_scale(-1.0, s.a);
    for (int i = 0; i < 100; ++i) {
        v3 p = support_mink(c1, c2, dir);
        if (v_dot(p, dir) < 0.0) return 0;
        simplex_add(&s, p);
        int hit = 0;
        switch (s.num) {
        case 2: hit = do_simplex_2(&s, &dir); break;
        case 3: hit = do_simplex_3(&s, &dir); break;
        case 4: hit = do_simplex_4(&s, &dir); break;
        default: g_error |= 1; return 0;
        }
        if (hit) { *out = s; return 1; }
    }
    return 0;
}

/* EPA (src/physics/epa.cpp) */
typedef struct { int n, cap; v3* a; } v3vec;
static void vv_push(v3vec* v, v3 x) {
    if (v->n == v->cap) { v->cap = v->cap ? 2 * v->cap : 16; v->a = (v3*)realloc(v->a, sizeof(v3) * (size_t)v->cap); }
    v->a[v->n++] = x;
}

static void face_normal_distance(i3 f, const v3* poly, int npoly, v3* out_n, double* out_d) {
    v3 a = poly[f.x], b = poly[f.y], c = poly[f.z];
    v3 n = v_norm(v_cross(v_sub(b, a), v_sub(c, a)));
    if (!(n.x != 0.0 || n.y != 0.0 || n.z != 0.0)) g_error |= 2;
    const double TOL = 0.0;
    double d = v_dot(n, a);
    if (d < -TOL) {
        n = v_inv(n);
        d = -d;
    } else if (d >= -TOL && d <= TOL) {
        int ok = 0;
        for (int i = 0; i < npoly; ++i) {
            double ad = v_dot(n, poly[i]);
            if (ad < -TOL || ad > TOL) {
                n = ad < -TOL ? n : v_inv(n);
                ok = 1;
                break;
            }
        }
        if (!ok) g_error |= 4;
    }
    *out_n = n;
    *out_d = d;
}

static void epa_add_edge(i2* edges, int* ne, i2 e, const v3* poly) {
    for (int i = 0; i < *ne; ++i) {
        i2 cur = edges[i];
        if ((e.x == cur.x && e.y == cur.y) || (e.x == cur.y && e.y == cur.x)) { (*ne)--; edges[i] = edges[*ne]; return; }
        v3 c1 = poly[cur.x], c2 = poly[cur.y], e1 = poly[e.x], e2 = poly[e.y];
        if (v_eq(c1, e1) && v_eq(c2, e2)) { (*ne)--; edges[i] = edges[*ne]; return; }
        if (v_eq(c1, e2) && v_eq(c2, e1)) { (*ne)--; edges[i] = edges[*ne]; return; }
    }
    edges[(*ne)++] = e;
}

static int epa(const collider_t* c1, const collider_t* c2, const simplex_t* s, v3* out_n, double* out_pen) {
    const double EPS = 0.0001;
    v3vec poly = {0, 0, NULL};
    vv_push(&poly, s->a); vv_push(&poly, s->b); vv_push(&poly, s->c); vv_push(&poly, s->d);
    int nf = 4, fcap = 64;
    i3* faces = (i3*)malloc(sizeof(i3) * (size_t)fcap);
    v3* normals = (v3*)malloc(sizeof(v3) * (size_t)fcap);
    double* dists = (double*)malloc(sizeof(double) * (size_t)fcap);
    i3 f0 = {0, 1, 2}, f1 = {0, 2, 3}, f2 = {0, 3, 1}, f3 = {1, 2, 3};
    faces[0] = f0; faces[1] = f1; faces[2] = f2; faces[3] = f3;
    v3 min_n = V3(0.0, 0.0, 0.0);
    double min_d = DBL_MAX;
    for (int i = 0; i < nf; ++i) {
        face_normal_distance(faces[i], poly.a, poly.n, &normals[i], &dists[i]);
        if (dists[i] < min_d) { min_d = dists[i]; min_n = normals[i]; }
    }
    int ecap = 3 * fcap + 16;
    i2* edges = (i2*)malloc(sizeof(i2) * (size_t)ecap);
    int converged = 0;
    for (int it = 0; it < 100; ++it) {
        v3 sp = support_mink(c1, c2, min_n);
        double d = v_dot(min_n, sp);
        if (fabs(d - min_d) < EPS) { *out_n = min_n; *out_pen = min_d; converged = 1; break; }
        int np = poly.n;
        vv_push(&poly, sp);
        int ne = 0;
        if (ecap < 3 * nf + 16) { ecap = 3 * nf + 16; edges = (i2*)realloc(edges, sizeof(i2) * (size_t)ecap); }
        for (int i = 0; i < nf; ++i) {
            v3 normal = normals[i];
            i3 f = faces[i];
            v3 cen = v_add(v_add(poly.a[f.y], poly.a[f.z]), poly.a[f.x]);
            cen = v_scale(1.0 / 3.0, cen);
            if (v_dot(normal, v_sub(sp, cen)) > 0.0) {
                i2 e1 = {f.x, f.y}, e2 = {f.y, f.z}, e3 = {f.z, f.x};
                epa_add_edge(edges, &ne, e1, poly.a);
                epa_add_edge(edges, &ne, e2, poly.a);
                epa_add_edge(edges, &ne, e3, poly.a);
                nf--;
                faces[i] = faces[nf];
                dists[i] = dists[nf];
                normals[i] = normals[nf];
                --i;
            }
        }
        if (nf + ne > fcap) {
            while (nf + ne > fcap) fcap *= 2;
            faces = (i3*)realloc(faces, sizeof(i3) * (size_t)fcap);
            normals = (v3*)realloc(normals, sizeof(v3) * (size_t)fcap);
            dists = (double*)realloc(dists, sizeof(double) * (size_t)fcap);
        }
        for (int i = 0; i < ne; ++i) {
            i3 nfc = {edges[i].x, edges[i].y, np};
            faces[nf] = nfc;
            face_normal_distance(nfc, poly.a, poly.n, &normals[nf], &dists[nf]);
            nf++;
        }
        min_d = DBL_MAX;
        for (int i = 0; i < nf; ++i)
            if (dists[i] < min_d) { min_d = dists[i]; min_n = normals[i]; }
    }
    free(faces); free(normals); free(dists); free(edges); free(poly.a);
    return converged;
}

/* Clipping (src/physics/clipping.cpp) */
typedef struct { v3 normal, point; } plane_t;

static int point_in_plane(const plane_t* p, v3 pos) {
    float distance = -v_dot(p->normal, p->point);
    if (v_dot(pos, p->normal) + distance < 0.0) return 0;
    return 1;
}

static int plane_edge(const plane_t* p, v3 start, v3 end, v3* out) {
    const double EPS = 0.000001;
    v3 ab = v_sub(end, start);
    float ab_p = v_dot(p->normal, ab);
    if (fabsf(ab_p) > EPS) {
        float distance = -v_dot(p->normal, p->point);
        v3 p_co = v_scale(-distance, p->normal);
        float fac = -v_dot(p->normal, v_sub(start, p_co)) / ab_p;
        double mx = ((fac) > (0.0)) ? (fac) : (0.0);
        fac = (mx < 1.0) ? mx : 1.0;
        *out = v_add(start, v_scale(fac, ab));
        return 1;
    }
    return 0;
}

static void sutherland_hodgman(const v3vec* in_poly, int nplanes, const plane_t* planes, v3vec* out, int remove_only) {
    v3vec input = {0, 0, NULL}, output = {0, 0, NULL};
    for (int i = 0; i < in_poly->n; ++i) vv_push(&input, in_poly->a[i]);
    for (int i = 0; i < nplanes; ++i) {
        if (input.n == 0) break;
        const plane_t* pl = &planes[i];
        v3 tmp, start = input.a[input.n - 1];
        for (int j = 0; j < input.n; ++j) {
            v3 end = input.a[j];
            int si = point_in_plane(pl, start), ei = point_in_plane(pl, end);
            if (remove_only) {
                if (ei) vv_push(&output, end);
            } else {
                if (si && ei) vv_push(&output, end);
                else if (si && !ei) { if (plane_edge(pl, start, end, &tmp)) vv_push(&output, tmp); }
                else if (!si && ei) { if (plane_edge(pl, start, end, &tmp)) vv_push(&output, tmp); vv_push(&output, end); }
            }
            start = end;
        }
        v3vec t = input; input = output; output = t;
        output.n = 0;
    }
    *out = input;
    free(output.a);
}

static v3 closest_on_plane(v3 pos, const plane_t* ref) {
    double d = v_dot(v_scale(-1.0, ref->normal), ref->point);
    return v_sub(pos, v_scale(v_dot(ref->normal, pos) + d, ref->normal));
}

static int face_most_fitting(int sidx, const collider_t* h, v3 normal) {
    double mx = -DBL_MAX;
    int sel = 0;
    for (int i = 0; i < h->v2f[sidx].n; ++i) {
        int fi = h->v2f[sidx].a[i];
        double p = v_dot(h->tn[fi], normal);
        if (p > mx) { mx = p; sel = fi; }
    }
    return sel;
}

static void edge_most_fitting(int s1, int s2, const collider_t* h1, const collider_t* h2, v3 normal, int sel[4], v3* edge_normal) {
    v3 sp1 = h1->tv[s1], sp2 = h2->tv[s2];
    double mx = -DBL_MAX;
    for (int i = 0; i < h1->v2n[s1].n; ++i) {
        v3 e1 = v_sub(sp1, h1->tv[h1->v2n[s1].a[i]]);
        for (int j = 0; j < h2->v2n[s2].n; ++j) {
            v3 e2 = v_sub(sp2, h2->tv[h2->v2n[s2].a[j]]);
            v3 cn = v_norm(v_cross(e1, e2));
            v3 ci = v_inv(cn);
            double dot = v_dot(cn, normal);
            if (dot > mx) { mx = dot; sel[0] = s1; sel[1] = h1->v2n[s1].a[i]; sel[2] = s2; sel[3] = h2->v2n[s2].a[j]; *edge_normal = cn; }
            dot = v_dot(ci, normal);
            if (dot > mx) { mx = dot; sel[0] = s1; sel[1] = h1->v2n[s1].a[i]; sel[2] = s2; sel[3] = h2->v2n[s2].a[j]; *edge_normal = ci; }
        }
    }
}

static int skew_lines(v3 p1, v3 d1, v3 p2, v3 d2, v3* l1, v3* l2) {
    double n1 = d1.x * d2.x + d1.y * d2.y + d1.z * d2.z;
    double n2 = d2.x * d2.x + d2.y * d2.y + d2.z * d2.z;
    double m1 = -d1.x * d1.x - d1.y * d1.y - d1.z * d1.z;
    double m2 = -d2.x * d1.x - d2.y * d1.y - d2.z * d1.z;
    double r1 = -d1.x * p2.x + d1.x * p1.x - d1.y * p2.y + d1.y * p1.y - d1.z * p2.z + d1.z * p1.z;
    double r2 = -d2.x * p2.x + d2.x * p1.x - d2.y * p2.y + d2.y * p1.y - d2.z * p2.z + d2.z * p1.z;
    if ((n1 * m2) - (n2 * m1) == 0) return 0;
    double n = ((r1 * m2) - (r2 * m1)) / ((n1 * m2) - (n2 * m1));
    double m = ((n1 * r2) - (n2 * r1)) / ((n1 * m2) - (n2 * m1));
    *l1 = v_add(p1, v_scale(m, d1));
    *l2 = v_add(p2, v_scale(n, d2));
    return 1;
}

typedef struct { v3 p1, p2, n; } contact_t;
typedef struct { int n, cap; contact_t* a; } cvec;
static void cv_push(cvec* v, contact_t c) {
    if (v->n == v->cap) { v->cap = v->cap ? 2 * v->cap : 16; v->a = (contact_t*)realloc(v->a, sizeof(contact_t) * (size_t)v->cap); }
    v->a[v->n++] = c;
}

static void face_vertices(const collider_t* h, int fi, v3vec* out) {
    for (int i = 0; i < h->f[fi].elements.n; ++i) vv_push(out, h->tv[h->f[fi].elements.a[i]]);
}

static void convex_convex_manifold(const collider_t* h1, const collider_t* h2, v3 normal, cvec* contacts) {
    const double EPS = 0.0001;
    v3 inv_n = v_inv(normal);
    v3 edge_normal = V3(0.0, 0.0, 0.0);
    int s1 = support_index(h1, normal);
    int s2 = support_index(h2, inv_n);
    int f1 = face_most_fitting(s1, h1, normal);
    int f2 = face_most_fitting(s2, h2, inv_n);
    v3 n1 = h1->tn[f1], n2 = h2->tn[f2];
    int e[4] = {0, 0, 0, 0};
    edge_most_fitting(s1, s2, h1, h2, normal, e, &edge_normal);
    double d1 = v_dot(n1, normal), d2 = v_dot(n2, inv_n), de = v_dot(edge_normal, normal);
    if (de > d1 + EPS && de > d2 + EPS) {
        v3 l1, l2;
        v3 p1 = h1->tv[e[0]];
        v3 dd1 = v_sub(h1->tv[e[1]], p1);
        v3 p2 = h2->tv[e[2]];
        v3 dd2 = v_sub(h2->tv[e[3]], p2);
        if (!skew_lines(p1, dd1, p2, dd2, &l1, &l2)) { g_error |= 8; return; }
        contact_t c = {l1, l2, normal};
        cv_push(contacts, c);
    } else {
        int ref1 = d1 > d2;
        v3vec refv = {0, 0, NULL}, inc = {0, 0, NULL};
        if (ref1) { face_vertices(h1, f1, &refv); face_vertices(h2, f2, &inc); }
        else { face_vertices(h2, f2, &refv); face_vertices(h1, f1, &inc); }
        const collider_t* rh = ref1 ? h1 : h2;
        int rf = ref1 ? f1 : f2;
        int npl = rh->f2n[rf].n;
        plane_t* planes = (plane_t*)malloc(sizeof(plane_t) * (size_t)(npl ? npl : 1));
        for (int i = 0; i < npl; ++i) {
            int nf = rh->f2n[rf].a[i];
            planes[i].point = rh->tv[rh->f[nf].elements.a[0]];
            planes[i].normal = v_inv(rh->tn[nf]);
        }
        v3vec clipped, final_pts;
        sutherland_hodgman(&inc, npl, planes, &clipped, 0);
        plane_t refp;
        refp.normal = ref1 ? v_inv(n1) : v_inv(n2);
        refp.point = refv.a[0];
        sutherland_hodgman(&clipped, 1, &refp, &final_pts, 1);
        for (int i = 0; i < final_pts.n; ++i) {
            v3 pt = final_pts.a[i];
            v3 cp = closest_on_plane(pt, &refp);
            v3 diff = v_sub(pt, cp);
            double pen;
            contact_t c;
            if (ref1) {
                pen = v_dot(diff, normal);
                c.p1 = v_sub(pt, v_scale(pen, normal));
                c.p2 = pt;
            } else {
                pen = -v_dot(diff, normal);
                c.p1 = pt;
                c.p2 = v_add(pt, v_scale(pen, normal));
            }
            c.n = normal;
            if (pen < 0.0) cv_push(contacts, c);
        }
        free(refv.a); free(inc.a); free(planes); free(clipped.a); free(final_pts.a);
    }
}

static void contact_manifold(const collider_t* c1, const collider_t* c2, v3 normal, double pen, cvec* contacts) {
    if (c1->type == 0) {
        v3 sp = support(c1, normal);
        contact_t c = {sp, v_sub(sp, v_scale(pen, normal)), normal};
        cv_push(contacts, c);
    } else if (c2->type == 0) {
        v3 in = v_inv(normal);
        v3 sp = support(c2, in);
        contact_t c = {v_add(sp, v_scale(pen, normal)), sp, normal};
        cv_push(contacts, c);
    } else {
        convex_convex_manifold(c1, c2, normal, contacts);
    }
}

/* collider_get_contacts (src/physics/collider.cpp:523-558) */
static void collider_contacts(collider_t* c1, collider_t* c2, cvec* contacts) {
    if (c1->type == 0 && c2->type == 0) {
        v3 dv = v_sub(c1->center, c2->center);
        float dsq = v_dot(dv, dv);
        float mind = c1->radius + c2->radius;
        if (dsq < (mind * mind)) {
            v3 normal = v_norm(v_sub(c2->center, c1->center));
            double pen = (float)(mind - sqrtf(dsq));
            contact_manifold(c1, c2, normal, pen, contacts);
        }
        return;
    }
    simplex_t s;
    if (gjk(c1, c2, &s)) {
        v3 normal;
        double pen;
        if (!epa(c1, c2, &s, &normal, &pen)) return;
        contact_manifold(c1, c2, normal, pen, contacts);
    }
}

static void body_colliders_update(body_t* b) {
    for (int k = 0; k < b->ncol; ++k) collider_update(&b->col[k], b->pos, b->rot);
}

static void body_contacts(body_t* a, body_t* b, cvec* out) {
    for (int i = 0; i < a->ncol; ++i)
        for (int j = 0; j < b->ncol; ++j) collider_contacts(&a->col[i], &b->col[j], out);
}

/* ------------------------------------------------------------------------------------------ */
/* XPBD primitives (src/physics/pbd_base_constraints.cpp, src/physics/physics_util.cpp) */
static m3 dyn_inertia(const body_t* e, int inverse) {
    m3 r = q_mat3(e->rot);
    m3 rt = m3_transpose(r);
    m3 aux = m3_mul(r, inverse ? e->Iinv : e->I);
    return m3_mul(aux, rt);
}

typedef struct { body_t *e1, *e2; v3 r1, r2; m3 I1, I2; } pcpd_t;
typedef struct { body_t *e1, *e2; m3 I1, I2; } acpd_t;

static void pos_pre(body_t* e1, body_t* e2, v3 r1, v3 r2, pcpd_t* p) {
    p->e1 = e1; p->e2 = e2;
    p->r1 = q_rotate(e1->rot, r1);
    p->r2 = q_rotate(e2->rot, r2);
    p->I1 = dyn_inertia(e1, 1);
    p->I2 = dyn_inertia(e2, 1);
}

static double pos_dlambda(const pcpd_t* p, double h, double compliance, double lambda, v3 dx) {
    double c = v_len(dx);
    if (c <= 1e-50) return 0.0;
    v3 n = V3(dx.x / c, dx.y / c, dx.z / c);
    double w1 = p->e1->invm + v_dot(v_cross(p->r1, n), m3_mulv(p->I1, v_cross(p->r1, n)));
    double w2 = p->e2->invm + v_dot(v_cross(p->r2, n), m3_mulv(p->I2, v_cross(p->r2, n)));
    if (!(w1 + w2 != 0.0)) g_error |= 1;
    double til = compliance / (h * h);
    return (-c - til * lambda) / (w1 + w2 + til);
}

static void pos_apply(const pcpd_t* p, double dl, v3 dx) {
    double c = v_len(dx);
    if (c <= 1e-50) return;
    body_t *e1 = p->e1, *e2 = p->e2;
    v3 n = V3(dx.x / c, dx.y / c, dx.z / c);
    v3 imp = v_scale(dl, n);
    if (!e1->fixed) e1->pos = v_add(e1->pos, v_scale(e1->invm, imp));
    if (!e2->fixed) e2->pos = v_add(e2->pos, v_scale(-e2->invm, imp));
    v3 a1 = m3_mulv(p->I1, v_cross(p->r1, imp));
    v3 a2 = m3_mulv(p->I2, v_cross(p->r2, imp));
    qt q1 = q_mul(Q(a1.x, a1.y, a1.z, 0.0), e1->rot);
    qt q2 = q_mul(Q(a2.x, a2.y, a2.z, 0.0), e2->rot);
    if (!e1->fixed) {
        e1->rot.x = e1->rot.x + 0.5 * q1.x; e1->rot.y = e1->rot.y + 0.5 * q1.y;
        e1->rot.z = e1->rot.z + 0.5 * q1.z; e1->rot.w = e1->rot.w + 0.5 * q1.w;
        e1->rot = q_normalize(e1->rot);
    }
    if (!e2->fixed) {
        e2->rot.x = e2->rot.x - 0.5 * q2.x; e2->rot.y = e2->rot.y - 0.5 * q2.y;
        e2->rot.z = e2->rot.z - 0.5 * q2.z; e2->rot.w = e2->rot.w - 0.5 * q2.w;
        e2->rot = q_normalize(e2->rot);
    }
}

static void ang_pre(body_t* e1, body_t* e2, acpd_t* a) {
    a->e1 = e1; a->e2 = e2;
    a->I1 = dyn_inertia(e1, 1);
    a->I2 = dyn_inertia(e2, 1);
}

static double ang_dlambda(const acpd_t* a, double h, double compliance, double lambda, v3 dq) {
    double th = v_len(dq);
    if (th <= 1e-50) return 0.0;
    v3 n = V3(dq.x / th, dq.y / th, dq.z / th);
    double w1 = v_dot(n, m3_mulv(a->I1, n));
    double w2 = v_dot(n, m3_mulv(a->I2, n));
    if (!(w1 + w2 != 0.0)) g_error |= 1;
    double til = compliance / (h * h);
    return (-th - til * lambda) / (w1 + w2 + til);
}

static void ang_apply(const acpd_t* a, double dl, v3 dq) {
    double th = v_len(dq);
    if (th <= 1e-50) return;
    body_t *e1 = a->e1, *e2 = a->e2;
    v3 n = V3(dq.x / th, dq.y / th, dq.z / th);
    v3 imp = v_scale(-dl, n);
    v3 a1 = m3_mulv(a->I1, imp);
    v3 a2 = m3_mulv(a->I2, imp);
    qt q1 = q_mul(Q(a1.x, a1.y, a1.z, 0.0), e1->rot);
    qt q2 = q_mul(Q(a2.x, a2.y, a2.z, 0.0), e2->rot);
    if (!e1->fixed) {
        e1->rot.x = e1->rot.x + 0.5 * q1.x; e1->rot.y = e1->rot.y + 0.5 * q1.y;
        e1->rot.z = e1->rot.z + 0.5 * q1.z; e1->rot.w = e1->rot.w + 0.5 * q1.w;
        e1->rot = q_normalize(e1->rot);
    }
    if (!e2->fixed) {
        e2->rot.x = e2->rot.x - 0.5 * q2.x; e2->rot.y = e2->rot.y - 0.5 * q2.y;
        e2->rot.z = e2->rot.z - 0.5 * q2.z; e2->rot.w = e2->rot.w - 0.5 * q2.w;
        e2->rot = q_normalize(e2->rot);
    }
}

/* ------------------------------------------------------------------------------------------ */
/* Constraint solves (src/physics/pbd.cpp:81-406) */
#define PI_F 3.14159265358979

static void solve_positional(constraint_t* c, double h) {
    body_t *e1 = &g_bodies[c->e1], *e2 = &g_bodies[c->e2];
    v3 ad = v_sub(e1->pos, e2->pos);
    v3 dx = v_sub(ad, c->distance);
    pcpd_t p;
    pos_pre(e1, e2, c->r1, c->r2, &p);
    double dl = pos_dlambda(&p, h, c->compliance, c->lambda, dx);
    pos_apply(&p, dl, dx);
    c->lambda += dl;
}

static void solve_collision(constraint_t* c, double h) {
    body_t *e1 = &g_bodies[c->e1], *e2 = &g_bodies[c->e2];
    pcpd_t p;
    pos_pre(e1, e2, c->r1, c->r2, &p);
    v3 p1 = v_add(e1->pos, p.r1);
    v3 p2 = v_add(e2->pos, p.r2);
    double d = v_dot(v_sub(p1, p2), c->normal);
    if (d > 0.0) {
        v3 dx = v_scale(d, c->normal);
        double dl = pos_dlambda(&p, h, 0.0, c->lambda_n, dx);
        pos_apply(&p, dl, dx);
        c->lambda_n += dl;
        pos_pre(e1, e2, c->r1, c->r2, &p);
        p1 = v_add(e1->pos, p.r1);
        p2 = v_add(e2->pos, p.r2);
        dl = pos_dlambda(&p, h, 0.0, c->lambda_t, dx);
        const double mus = (e1->mus + e2->mus) / 2.0f;
        double ln = c->lambda_n;
        double lt = c->lambda_t + dl;
        if (lt > mus * ln) {
            v3 p1t = v_add(e1->ppos, q_rotate(e1->prot, c->r1));
            v3 p2t = v_add(e2->ppos, q_rotate(e2->prot, c->r2));
            v3 dp = v_sub(v_sub(p1, p1t), v_sub(p2, p2t));
            v3 dpt = v_sub(dp, v_scale(v_dot(dp, c->normal), c->normal));
            pos_apply(&p, dl, dpt);
            c->lambda_t += dl;
        }
    }
}

static void solve_mutual_orientation(constraint_t* c, double h) {
    body_t *e1 = &g_bodies[c->e1], *e2 = &g_bodies[c->e2];
    acpd_t a;
    ang_pre(e1, e2, &a);
    qt q2i = q_inverse(e2->rot);
    qt aux = q_mul(e1->rot, q2i);
    v3 dq = V3(2.0 * aux.x, 2.0 * aux.y, 2.0 * aux.z);
    double dl = ang_dlambda(&a, h, c->compliance, c->lambda, dq);
    ang_apply(&a, dl, dq);
    c->lambda += dl;
}

static int limit_angle(v3 n, v3 n1, v3 n2, double alpha, double beta, v3* dq) {
    double phi = asin(v_dot(v_cross(n1, n2), n));
    if (v_dot(n1, n2) < 0.0) phi = PI_F - phi;
    if (phi > PI_F) phi = phi - 2.0 * PI_F;
    if (phi < -PI_F) phi = phi + 2.0 * PI_F;
    if (phi < alpha || phi > beta) {
        phi = ((phi) > (beta)) ? (beta) : (((phi) < (alpha)) ? (alpha) : (phi));
        qt rot = q_from_axis_angle(n, phi);
        n1 = q_rotate(rot, n1);
        *dq = v_cross(n1, n2);
        return 1;
    }
    return 0;
}

static void solve_hinge(constraint_t* c, double h) {
    body_t *e1 = &g_bodies[c->e1], *e2 = &g_bodies[c->e2];
    acpd_t a;
    ang_pre(e1, e2, &a);
    v3 a1 = q_axis(e1->rot, c->a1), a2 = q_axis(e2->rot, c->a2);
    v3 dq = v_cross(a1, a2);
    double dl = ang_dlambda(&a, h, c->compliance, c->lambda_aligned, dq);
    ang_apply(&a, dl, dq);
    c->lambda_aligned += dl;
    pcpd_t p;
    pos_pre(e1, e2, c->r1, c->r2, &p);
    v3 p1 = v_add(e1->pos, p.r1), p2 = v_add(e2->pos, p.r2);
    v3 dx = v_sub(p1, p2);
    dl = pos_dlambda(&p, h, 0.0, c->lambda_pos, dx);
    pos_apply(&p, dl, dx);
    c->lambda_pos += dl;
    if (c->limited) {
        v3 n1 = q_axis(e1->rot, c->l1), n2 = q_axis(e2->rot, c->l2), n = q_axis(e1->rot, c->a1);
        if (limit_angle(n, n1, n2, c->lower, c->upper, &dq)) {
            acpd_t b;
            ang_pre(e1, e2, &b);
            double dl2 = ang_dlambda(&b, h, 0.0, c->lambda_limit, dq);
            ang_apply(&b, dl2, dq);
            c->lambda_limit += dl2;
        }
    }
}

static void solve_spherical(constraint_t* c, double h) {
    const double EPS = 1e-50;
    body_t *e1 = &g_bodies[c->e1], *e2 = &g_bodies[c->e2];
    pcpd_t p;
    pos_pre(e1, e2, c->r1, c->r2, &p);
    v3 p1 = v_add(e1->pos, p.r1), p2 = v_add(e2->pos, p.r2);
    v3 dx = v_sub(p1, p2);
    double dl = pos_dlambda(&p, h, 0.0, c->lambda_pos, dx);
    pos_apply(&p, dl, dx);
    c->lambda_pos += dl;
    v3 n1 = q_axis(e1->rot, c->s1), n2 = q_axis(e2->rot, c->s2);
    v3 n = v_cross(n1, n2);
    double nl = v_len(n);
    if (nl > EPS) {
        n = V3(n.x / nl, n.y / nl, n.z / nl);
        v3 dq;
        if (limit_angle(n, n1, n2, c->slo, c->shi, &dq)) {
            acpd_t a;
            ang_pre(e1, e2, &a);
            double d2 = ang_dlambda(&a, h, 0.0, c->lambda_swing, dq);
            ang_apply(&a, d2, dq);
            c->lambda_swing += d2;
        }
    }
    v3 a1 = q_axis(e1->rot, c->s1), b1 = q_axis(e1->rot, c->t1);
    v3 a2 = q_axis(e2->rot, c->s2), b2 = q_axis(e2->rot, c->t2);
    n = v_add(a1, a2);
    nl = v_len(n);
    if (nl > EPS) {
        n = V3(n.x / nl, n.y / nl, n.z / nl);
        n1 = v_sub(b1, v_scale(v_dot(n, b1), n));
        n2 = v_sub(b2, v_scale(v_dot(n, b2), n));
        double l1 = v_len(n1), l2 = v_len(n2);
        if (l1 > EPS && l2 > EPS) {
            n1 = V3(n1.x / l1, n1.y / l1, n1.z / l1);
            n2 = V3(n2.x / l2, n2.y / l2, n2.z / l2);
            v3 dq;
            if (limit_angle(n, n1, n2, c->tlo, c->thi, &dq)) {
                acpd_t a;
                ang_pre(e1, e2, &a);
                double d2 = ang_dlambda(&a, h, 0.0, c->lambda_twist, dq);
                ang_apply(&a, d2, dq);
                c->lambda_twist += d2;
            }
        }
    }
}

static void solve_constraint(constraint_t* c, double h) {
    switch (c->type) {
    case C_POS: solve_positional(c, h); break;
    case C_COL: solve_collision(c, h); break;
    case C_MO: solve_mutual_orientation(c, h); break;
    case C_HINGE: solve_hinge(c, h); break;
    case C_SPH: solve_spherical(c, h); break;
    default: g_error |= 1; break;
    }
}

/* ------------------------------------------------------------------------------------------ */
/* Broad phase and islands (src/physics/broad.cpp) */
typedef struct { int a, b; } pair_t;

static pair_t* broad_pairs(int* out_n) {
    int n = 0, cap = 32;
    pair_t* p = (pair_t*)malloc(sizeof(pair_t) * (size_t)cap);
    for (int i = 0; i < g_nb; ++i) {
        body_t* e1 = &g_bodies[i];
        for (int j = i + 1; j < g_nb; ++j) {
            body_t* e2 = &g_bodies[j];
            double dist = v_len(v_sub(e1->pos, e2->pos));
            double mx = e1->radius + e2->radius + 0.1;
            if (dist <= mx) {
                if (n == cap) { cap *= 2; p = (pair_t*)realloc(p, sizeof(pair_t) * (size_t)cap); }
                p[n].a = i;
                p[n].b = j;
                n++;
            }
        }
    }
    *out_n = n;
    return p;
}

static int uf_find(int* parent, int x) {
    while (parent[x] != x) x = parent[x];
    return x;
}

/* broad_collect_simulation_islands + the sleeping update (src/physics/pbd.cpp:477-506) */
static void islands_and_sleep(const pair_t* pairs, int np, const constraint_t* cons, int nc, double dt) {
    int* parent = (int*)malloc(sizeof(int) * (size_t)(g_nb ? g_nb : 1));
    for (int i = 0; i < g_nb; ++i) parent[i] = i;
    for (int k = 0; k < np; ++k) {
        int a = pairs[k].a, b = pairs[k].b;
        if (!g_bodies[a].fixed && !g_bodies[b].fixed) { int ry = uf_find(parent, b), rx = uf_find(parent, a); parent[ry] = rx; }
    }
    for (int k = 0; k < nc; ++k) {
        int a = cons[k].e1, b = cons[k].e2;
        if (!g_bodies[a].fixed && !g_bodies[b].fixed) { int ry = uf_find(parent, b), rx = uf_find(parent, a); parent[ry] = rx; }
    }
    int* all_inactive = (int*)malloc(sizeof(int) * (size_t)(g_nb ? g_nb : 1));
    for (int i = 0; i < g_nb; ++i) all_inactive[i] = 1;
    for (int i = 0; i < g_nb; ++i) {
        body_t* e = &g_bodies[i];
        if (e->fixed) continue;
        double lv = v_len(e->v), av = v_len(e->w);
        if (lv < 0.10 && av < 0.10) e->deact += dt;
        else e->deact = 0.0;
        if (e->deact < 1.0) all_inactive[uf_find(parent, i)] = 0;
    }
    for (int i = 0; i < g_nb; ++i) {
        body_t* e = &g_bodies[i];
        if (e->fixed) continue;
        e->active = !all_inactive[uf_find(parent, i)];
    }
    free(parent);
    free(all_inactive);
}

/* ------------------------------------------------------------------------------------------ */
/* pbd_simulate_with_constraints (src/physics/pbd.cpp:468-747) */
static void clip_to_constraint(int i1, int i2, const contact_t* ct, constraint_t* c) {
    memset(c, 0, sizeof(*c));
    body_t *e1 = &g_bodies[i1], *e2 = &g_bodies[i2];
    c->type = C_COL;
    c->e1 = i1;
    c->e2 = i2;
    c->normal = ct->n;
    v3 r1 = v_sub(ct->p1, e1->pos), r2 = v_sub(ct->p2, e2->pos);
    c->r1 = q_rotate(q_inverse(e1->rot), r1);
    c->r2 = q_rotate(q_inverse(e2->rot), r2);
}

static void simulate(double dt, unsigned substeps, unsigned iters, int collisions) {
    if (dt <= 0.0) return;
    double h = dt / substeps;
    int np = 0;
    pair_t* pairs = broad_pairs(&np);
    islands_and_sleep(pairs, np, g_cons, g_nc, dt);
    int ccap = g_nc + 64;
    constraint_t* cons = (constraint_t*)malloc(sizeof(constraint_t) * (size_t)ccap);
    cvec contacts = {0, 0, NULL};
    for (unsigned s = 0; s < substeps; ++s) {
        for (int j = 0; j < g_nb; ++j) {
            body_t* e = &g_bodies[j];
            e->ppos = e->pos;
            e->prot = e->rot;
            if (e->fixed) continue;
            if (!e->active) continue;
            v3 F = V3(0.0, 0.0, 0.0), T = V3(0.0, 0.0, 0.0);
            for (int k = 0; k < e->nf; ++k) F = v_add(F, e->forces[k].force);
            for (int k = 0; k < e->nf; ++k) {
                v3 dist = v_sub(e->forces[k].position, V3(0.0, 0.0, 0.0));
                T = v_add(T, v_cross(dist, e->forces[k].force));
            }
            e->v = v_add(e->v, v_scale(h * e->invm, F));
            e->pos = v_add(e->pos, v_scale(h, e->v));
            m3 Iinv = dyn_inertia(e, 1), I = dyn_inertia(e, 0);
            e->w = v_add(e->w, v_scale(h, m3_mulv(Iinv, v_sub(T, v_cross(e->w, m3_mulv(I, e->w))))));
            qt q = q_mul(Q(e->w.x, e->w.y, e->w.z, 0.0), e->rot);
            e->rot.x = e->rot.x + h * 0.5 * q.x;
            e->rot.y = e->rot.y + h * 0.5 * q.y;
            e->rot.z = e->rot.z + h * 0.5 * q.z;
            e->rot.w = e->rot.w + h * 0.5 * q.w;
            e->rot = q_normalize(e->rot);
        }
        int nc = g_nc;
        for (int k = 0; k < g_nc; ++k) {
            cons[k] = g_cons[k];
            cons[k].lambda = cons[k].lambda_t = cons[k].lambda_n = 0.0;
            cons[k].lambda_pos = cons[k].lambda_aligned = cons[k].lambda_limit = 0.0;
            cons[k].lambda_swing = cons[k].lambda_twist = 0.0;
        }
        if (collisions) {
            for (int j = 0; j < np; ++j) {
                body_t *e1 = &g_bodies[pairs[j].a], *e2 = &g_bodies[pairs[j].b];
                if ((e1->fixed || !e1->active) && (e2->fixed || !e2->active)) continue;
                body_colliders_update(e1);
                body_colliders_update(e2);
                contacts.n = 0;
                body_contacts(e1, e2, &contacts);
                for (int l = 0; l < contacts.n; ++l) {
                    if (nc == ccap) { ccap *= 2; cons = (constraint_t*)realloc(cons, sizeof(constraint_t) * (size_t)ccap); }
                    clip_to_constraint(pairs[j].a, pairs[j].b, &contacts.a[l], &cons[nc++]);
                }
            }
        }
        for (unsigned it = 0; it < iters; ++it)
            for (int k = 0; k < nc; ++k) solve_constraint(&cons[k], h);
        for (int j = 0; j < g_nb; ++j) {
            body_t* e = &g_bodies[j];
            if (e->fixed) continue;
            if (!e->active) continue;
            e->pv = e->v;
            e->pw = e->w;
            e->v = v_scale(1.0 / h, v_sub(e->pos, e->ppos));
            qt inv = q_inverse(e->prot);
            qt dq = q_mul(e->rot, inv);
            if (dq.w >= 0.0) e->w = v_scale(2.0 / h, V3(dq.x, dq.y, dq.z));
            else e->w = v_scale(-2.0 / h, V3(dq.x, dq.y, dq.z));
        }
        for (int k = 0; k < nc; ++k) {
            constraint_t* c = &cons[k];
            if (c->type != C_COL) continue;
            body_t *e1 = &g_bodies[c->e1], *e2 = &g_bodies[c->e2];
            v3 n = c->normal;
            double ln = c->lambda_n;
            pcpd_t p;
            pos_pre(e1, e2, c->r1, c->r2, &p);
            v3 v1 = e1->v, w1 = e1->w, v2 = e2->v, w2 = e2->w;
            v3 v = v_sub(v_add(v1, v_cross(w1, p.r1)), v_add(v2, v_cross(w2, p.r2)));
            double vn = v_dot(n, v);
            v3 vt = v_sub(v, v_scale(vn, n));
            v3 dv = V3(0.0, 0.0, 0.0);
            const double mud = (e1->mud + e2->mud) / 2.0f;
            double fn = ln / h;
            double a = mud * fabs(fn), b = v_len(vt);
            double fact = (a < b) ? a : b;
            dv = v_add(dv, v_scale(-fact, v_norm(vt)));
            v3 ov1 = e1->pv, ow1 = e1->pw, ov2 = e2->pv, ow2 = e2->pw;
            v3 vtil = v_sub(v_add(ov1, v_cross(ow1, p.r1)), v_add(ov2, v_cross(ow2, p.r2)));
            double vntil = v_dot(n, vtil);
            double e = e1->rest * e2->rest;
            double m = -e * vntil;
            fact = -vn + ((m < 0.0) ? m : 0.0);
            dv = v_add(dv, v_scale(fact, n));
            double W1 = e1->invm + v_dot(v_cross(p.r1, n), m3_mulv(p.I1, v_cross(p.r1, n)));
            double W2 = e2->invm + v_dot(v_cross(p.r2, n), m3_mulv(p.I2, v_cross(p.r2, n)));
            v3 P = v_scale(1.0 / (W1 + W2), dv);
            if (!e1->fixed) {
                e1->v = v_add(e1->v, v_scale(e1->invm, P));
                e1->w = v_add(e1->w, m3_mulv(p.I1, v_cross(p.r1, P)));
            }
            if (!e2->fixed) {
                e2->v = v_add(e2->v, v_inv(v_scale(e2->invm, P)));
                e2->w = v_add(e2->w, v_inv(m3_mulv(p.I2, v_cross(p.r2, P))));
            }
        }
        if (s + 1 == substeps) {
            /* keep the last substep's collision constraints for orc_last_contacts */
            g_nlast = 0;
            for (int k = 0; k < nc; ++k)
                if (cons[k].type == C_COL) {
                    if (g_nlast == g_lastcap) { g_lastcap = g_lastcap ? 2 * g_lastcap : 64; g_last = (constraint_t*)realloc(g_last, sizeof(constraint_t) * (size_t)g_lastcap); }
                    g_last[g_nlast++] = cons[k];
                }
        }
    }
    free(contacts.a);
    free(cons);
    free(pairs);
}

uint32_t orc_last_contacts(int32_t* pairs, double* out, uint32_t cap) {
    for (int k = 0; k < g_nlast && (uint32_t)k < cap; ++k) {
        const constraint_t* c = &g_last[k];
        pairs[2 * k] = c->e1;
        pairs[2 * k + 1] = c->e2;
        double v[11] = {c->r1.x, c->r1.y, c->r1.z, c->r2.x, c->r2.y, c->r2.z, c->normal.x, c->normal.y, c->normal.z,
                        c->lambda_n, c->lambda_t};
        for (int j = 0; j < 11; ++j) out[11 * k + j] = v[j];
    }
    return (uint32_t)g_nlast;
}

void orc_step(double dt, uint32_t substeps, uint32_t iters, int collisions, double gravity) {
    for (int i = 0; i < g_nb; ++i) body_colliders_update(&g_bodies[i]);
    for (int i = 0; i < g_nb; ++i) add_force(&g_bodies[i], V3(0.0, 0.0, 0.0), V3(0.0, -gravity * 1.0 / g_bodies[i].invm, 0.0), 0);
    simulate(dt, substeps, iters, collisions);
    for (int i = 0; i < g_nb; ++i) g_bodies[i].nf = 0;
}

uint32_t orc_num_entities(void) { return (uint32_t)g_nb; }

void orc_get_state(double* out) {
    for (int i = 0; i < g_nb; ++i) {
        body_t* e = &g_bodies[i];
        double* o = out + (size_t)i * ORC_STATE_DOUBLES;
        o[0] = e->pos.x; o[1] = e->pos.y; o[2] = e->pos.z;
        o[3] = e->rot.x; o[4] = e->rot.y; o[5] = e->rot.z; o[6] = e->rot.w;
        o[7] = e->v.x; o[8] = e->v.y; o[9] = e->v.z;
        o[10] = e->w.x; o[11] = e->w.y; o[12] = e->w.z;
        o[13] = e->ppos.x; o[14] = e->ppos.y; o[15] = e->ppos.z;
        o[16] = e->prot.x; o[17] = e->prot.y; o[18] = e->prot.z; o[19] = e->prot.w;
        o[20] = e->pv.x; o[21] = e->pv.y; o[22] = e->pv.z;
        o[23] = e->pw.x; o[24] = e->pw.y; o[25] = e->pw.z;
        o[26] = e->active ? 1.0 : 0.0;
        o[27] = e->deact;
    }
}

void orc_set_state(const double* in) {
    for (int i = 0; i < g_nb; ++i) {
        body_t* e = &g_bodies[i];
        const double* o = in + (size_t)i * ORC_STATE_DOUBLES;
        e->pos = V3(o[0], o[1], o[2]);
        e->rot = Q(o[3], o[4], o[5], o[6]);
        e->v = V3(o[7], o[8], o[9]);
        e->w = V3(o[10], o[11], o[12]);
        e->ppos = V3(o[13], o[14], o[15]);
        e->prot = Q(o[16], o[17], o[18], o[19]);
        e->pv = V3(o[20], o[21], o[22]);
        e->pw = V3(o[23], o[24], o[25]);
        e->active = o[26] != 0.0;
        e->deact = o[27];
    }
}

uint32_t orc_broad_pairs(uint32_t* out, uint32_t cap) {
    int n = 0;
    pair_t* p = broad_pairs(&n);
    for (int k = 0; k < n && (uint32_t)k < cap; ++k) { out[2 * k] = (uint32_t)p[k].a; out[2 * k + 1] = (uint32_t)p[k].b; }
    free(p);
    return (uint32_t)n;
}

uint32_t orc_contacts(int e1, int e2, double* out, uint32_t cap) {
    body_colliders_update(&g_bodies[e1]);
    body_colliders_update(&g_bodies[e2]);
    cvec c = {0, 0, NULL};
    body_contacts(&g_bodies[e1], &g_bodies[e2], &c);
    for (int k = 0; k < c.n && (uint32_t)k < cap; ++k) {
        double* o = out + (size_t)k * ORC_CONTACT_DOUBLES;
        o[0] = c.a[k].p1.x; o[1] = c.a[k].p1.y; o[2] = c.a[k].p1.z;
        o[3] = c.a[k].p2.x; o[4] = c.a[k].p2.y; o[5] = c.a[k].p2.z;
        o[6] = c.a[k].n.x; o[7] = c.a[k].n.y; o[8] = c.a[k].n.z;
    }
    uint32_t n = (uint32_t)c.n;
    free(c.a);
    return n;
}

int orc_gjk_epa(int e1, int e2, double* out) {
    body_colliders_update(&g_bodies[e1]);
    body_colliders_update(&g_bodies[e2]);
    simplex_t s;
    if (!gjk(&g_bodies[e1].col[0], &g_bodies[e2].col[0], &s)) return 0;
    v3 n;
    double pen;
    if (!epa(&g_bodies[e1].col[0], &g_bodies[e2].col[0], &s, &n, &pen)) return 2;
    out[0] = n.x; out[1] = n.y; out[2] = n.z; out[3] = pen;
    return 1;
}

uint32_t orc_manifold(int e1, int e2, const double* normal, double penetration, double* out, uint32_t cap) {
    body_colliders_update(&g_bodies[e1]);
    body_colliders_update(&g_bodies[e2]);
    cvec c = {0, 0, NULL};
    v3 n = {normal[0], normal[1], normal[2]};
    contact_manifold(&g_bodies[e1].col[0], &g_bodies[e2].col[0], n, penetration, &c);
    for (int k = 0; k < c.n && (uint32_t)k < cap; ++k) {
        double* o = out + (size_t)k * ORC_CONTACT_DOUBLES;
        o[0] = c.a[k].p1.x; o[1] = c.a[k].p1.y; o[2] = c.a[k].p1.z;
        o[3] = c.a[k].p2.x; o[4] = c.a[k].p2.y; o[5] = c.a[k].p2.z;
        o[6] = c.a[k].n.x; o[7] = c.a[k].n.y; o[8] = c.a[k].n.z;
    }
    uint32_t cnt = (uint32_t)c.n;
    free(c.a);
    return cnt;
}

int orc_last_error(void) { return g_error; }
