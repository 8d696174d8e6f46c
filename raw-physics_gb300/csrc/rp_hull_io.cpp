// Hull preprocessing: OBJ input and a binary topology cache (include/rp.h: rp_hull_from_obj,
// rp_hull_save, rp_hull_load).
//
// The reference builds every hull at start-up from its OBJ file: obj_parse (src/render/obj.cpp:7-80)
// reads it with tinyobj, emits one vertex per face corner in face order with indices 0, 1, 2, ...,
// the caller scales the FP32 positions in FP64 (examples_util.cpp:5-24), and
// collider_convex_hull_create (collider.cpp:194-364) derives the topology. rp_hull_from_obj does the
// same from the file's `v` and `f` lines; rp_hull_save writes a built hull's topology so that
// rp_hull_load can restore it without the construction. Everything here goes through the public
// C ABI (rp_hull_create, rp_hull_topology, rp_hull_geometry, rp_hull_create_from_topology).
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <cstddef>
#include <string>
#include <vector>

#include "rp.h"

namespace rp {
rp_status report_error(rp_status code, const char* msg);   // rp_host.cpp: sets rp_last_error
}

namespace {

using rp::report_error;

// File layout (little-endian): magic, version, six counts, then the arrays in this order, then an
// FNV-1a 64-bit hash of every preceding byte.
const char kMagic[8] = {'R', 'P', 'H', 'U', 'L', 'L', 0, 1};
const uint32_t kVersion = 1;
const int32_t kMaxElems = 1 << 24;

uint64_t fnv1a(const unsigned char* p, size_t n) {
    uint64_t h = 1469598103934665603ull;
    for (size_t i = 0; i < n; ++i) {
        h ^= p[i];
        h *= 1099511628211ull;
    }
    return h;
}

bool little_endian() {
    const uint32_t x = 1;
    unsigned char c;
    memcpy(&c, &x, 1);
    return c == 1;
}

template <typename T>
void put(std::vector<unsigned char>& out, const T* p, size_t n) {
    const unsigned char* b = reinterpret_cast<const unsigned char*>(p);
    out.insert(out.end(), b, b + n * sizeof(T));
}

template <typename T>
bool get(const std::vector<unsigned char>& in, size_t& off, T* p, size_t n) {
    const size_t bytes = n * sizeof(T);
    if (off + bytes > in.size()) return false;
    if (bytes) memcpy(p, in.data() + off, bytes);
    off += bytes;
    return true;
}

// One CSR table of a built hull (which: 0 faces, 1 vertex->faces, 2 vertex->neighbours, 3 face->neighbours)
rp_status table(rp_world* w, int32_t hull, int32_t which, std::vector<int32_t>& start, std::vector<int32_t>& data) {
    int32_t rows = 0, n = 0;
    rp_status s = rp_hull_topology(w, hull, which, nullptr, nullptr, 0, &rows, &n);
    if (s != RP_OK) return s;
    start.assign((size_t)rows + 1, 0);
    data.assign((size_t)(n > 0 ? n : 1), 0);
    return rp_hull_topology(w, hull, which, start.data(), data.data(), n, &rows, &n);
}

// "12", "12/3", "12/3/4", "12//4", "-1": the position index, 0-based; false when malformed
bool obj_index(const char* tok, int32_t nverts, int32_t& out) {
    char* end = nullptr;
    const long v = strtol(tok, &end, 10);
    if (end == tok || (*end != '\0' && *end != '/')) return false;
    long i = v > 0 ? v - 1 : (v < 0 ? (long)nverts + v : -1);
    if (i < 0 || i >= nverts) return false;
    out = (int32_t)i;
    return true;
}

// Crossing-number point-in-triangle test on the projected coordinates (the even-odd rule)
bool inside_tri(const float* xs, const float* ys, float tx, float ty) {
    bool in = false;
    for (int i = 0, j = 2; i < 3; j = i++) {
        if (((ys[i] > ty) != (ys[j] > ty)) && (tx < (xs[j] - xs[i]) * (ty - ys[i]) / (ys[j] - ys[i]) + xs[i])) in = !in;
    }
    return in;
}

// Triangles of one polygon face, as the OBJ loader the reference uses produces them (ear clipping on
// the polygon projected onto the two axes its first non-degenerate corner spans most; an ear is a
// corner turning with the polygon's orientation whose triangle holds none of the other remaining
// corners). Arithmetic in FP32, the loader's number type. A triangle face comes out as it is.
void triangulate(const std::vector<float>& pos, const std::vector<int32_t>& poly, std::vector<int32_t>& tris) {
    const size_t n = poly.size();
    auto P = [&](int32_t v, int a) { return pos[3 * (size_t)v + (size_t)a]; };
    int ax0 = 1, ax1 = 2;
    for (size_t k = 0; k < n; ++k) {
        const int32_t a = poly[k], b = poly[(k + 1) % n], c = poly[(k + 2) % n];
        const float e0x = P(b, 0) - P(a, 0), e0y = P(b, 1) - P(a, 1), e0z = P(b, 2) - P(a, 2);
        const float e1x = P(c, 0) - P(b, 0), e1y = P(c, 1) - P(b, 1), e1z = P(c, 2) - P(b, 2);
        const float cx = fabsf(e0y * e1z - e0z * e1y), cy = fabsf(e0z * e1x - e0x * e1z), cz = fabsf(e0x * e1y - e0y * e1x);
        const float eps = FLT_EPSILON;
        if (cx > eps || cy > eps || cz > eps) {
            if (!(cx > cy && cx > cz)) {
                ax0 = 0;
                if (cz > cx && cz > cy) ax1 = 1;
            }
            break;
        }
    }
    float area = 0.0f;
    for (size_t k = 0; k < n; ++k) {
        const int32_t a = poly[k], b = poly[(k + 1) % n];
        area += (P(a, ax0) * P(b, ax1) - P(a, ax1) * P(b, ax0)) * 0.5f;
    }
    std::vector<int32_t> rest = poly;
    size_t guess = 0, budget = n, last_size = n;
    while (rest.size() > 3 && budget > 0) {
        const size_t m = rest.size();
        if (guess >= m) guess -= m;
        if (last_size != m) {
            last_size = m;
            budget = m;
        } else {
            --budget;
        }
        int32_t c3[3];
        float xs[3], ys[3];
        for (int k = 0; k < 3; ++k) {
            c3[k] = rest[(guess + (size_t)k) % m];
            xs[k] = P(c3[k], ax0);
            ys[k] = P(c3[k], ax1);
        }
        const float turn = (xs[1] - xs[0]) * (ys[2] - ys[1]) - (ys[1] - ys[0]) * (xs[2] - xs[1]);
        if (turn * area < 0.0f) { ++guess; continue; }
        bool covers = false;
        for (size_t o = 3; o < m && !covers; ++o) {
            const int32_t t = rest[(guess + o) % m];
            covers = inside_tri(xs, ys, P(t, ax0), P(t, ax1));
        }
        if (covers) { ++guess; continue; }
        tris.insert(tris.end(), c3, c3 + 3);
        rest.erase(rest.begin() + (std::ptrdiff_t)((guess + 1) % m));
    }
    if (rest.size() == 3) tris.insert(tris.end(), rest.begin(), rest.end());
}

}  // namespace

extern "C" {

rp_status rp_hull_save(rp_world* w, int32_t hull, const char* path) {
    if (!w || !path) return report_error(RP_ERR_INVALID, "null argument");
    if (!little_endian()) return report_error(RP_ERR_INVALID, "the hull cache format is little-endian");
    int32_t nv = 0, nf = 0;
    rp_status s = rp_hull_info(w, hull, &nv, &nf);
    if (s != RP_OK) return s;
    std::vector<double> verts(3 * (size_t)nv), normals(3 * (size_t)nf);
    if ((s = rp_hull_geometry(w, hull, verts.data(), normals.data())) != RP_OK) return s;
    std::vector<int32_t> st[4], dt[4];
    for (int k = 0; k < 4; ++k)
        if ((s = table(w, hull, k, st[k], dt[k])) != RP_OK) return s;
    std::vector<unsigned char> out;
    put(out, kMagic, 8);
    put(out, &kVersion, 1);
    int32_t counts[6] = {nv, nf, st[0].back(), st[1].back(), st[2].back(), st[3].back()};
    put(out, counts, 6);
    put(out, verts.data(), verts.size());
    put(out, normals.data(), normals.size());
    for (int k = 0; k < 4; ++k) {
        put(out, st[k].data(), st[k].size());
        put(out, dt[k].data(), (size_t)st[k].back());
    }
    const uint64_t h = fnv1a(out.data(), out.size());
    put(out, &h, 1);
    FILE* f = fopen(path, "wb");
    if (!f) return report_error(RP_ERR_INVALID, "cannot open the hull cache for writing");
    const bool ok = fwrite(out.data(), 1, out.size(), f) == out.size();
    return (fclose(f) == 0 && ok) ? RP_OK : report_error(RP_ERR_INVALID, "cannot write the hull cache");
}

rp_status rp_hull_load(rp_world* w, const char* path, int32_t* out_hull) {
    if (!w || !path || !out_hull) return report_error(RP_ERR_INVALID, "null argument");
    if (!little_endian()) return report_error(RP_ERR_INVALID, "the hull cache format is little-endian");
    FILE* f = fopen(path, "rb");
    if (!f) return report_error(RP_ERR_INVALID, "cannot open the hull cache");
    std::vector<unsigned char> in;
    unsigned char buf[1 << 16];
    size_t got;
    while ((got = fread(buf, 1, sizeof(buf), f)) > 0) in.insert(in.end(), buf, buf + got);
    fclose(f);
    if (in.size() < 8 + 4 + 24 + 8) return report_error(RP_ERR_INVALID, "hull cache too short");
    uint64_t h = 0;
    memcpy(&h, in.data() + in.size() - 8, 8);
    if (h != fnv1a(in.data(), in.size() - 8)) return report_error(RP_ERR_INVALID, "hull cache checksum mismatch");
    in.resize(in.size() - 8);
    size_t off = 0;
    char magic[8];
    uint32_t version = 0;
    int32_t c[6];
    if (!get(in, off, magic, 8) || memcmp(magic, kMagic, 8) != 0) return report_error(RP_ERR_INVALID, "not a hull cache");
    if (!get(in, off, &version, 1) || version != kVersion) return report_error(RP_ERR_INVALID, "unknown hull cache version");
    if (!get(in, off, c, 6)) return report_error(RP_ERR_INVALID, "hull cache truncated");
    for (int k = 0; k < 6; ++k)
        if (c[k] < 0 || c[k] > kMaxElems) return report_error(RP_ERR_INVALID, "hull cache counts out of range");
    const int32_t nv = c[0], nf = c[1];
    if (nv <= 0 || nf <= 0) return report_error(RP_ERR_INVALID, "hull cache counts out of range");
    std::vector<double> verts(3 * (size_t)nv), normals(3 * (size_t)nf);
    if (!get(in, off, verts.data(), verts.size()) || !get(in, off, normals.data(), normals.size()))
        return report_error(RP_ERR_INVALID, "hull cache truncated");
    const int32_t rows[4] = {nf, nv, nv, nf};
    std::vector<int32_t> st[4], dt[4];
    for (int k = 0; k < 4; ++k) {
        st[k].resize((size_t)rows[k] + 1);
        dt[k].resize((size_t)(c[2 + k] > 0 ? c[2 + k] : 1));
        if (!get(in, off, st[k].data(), st[k].size()) || !get(in, off, dt[k].data(), (size_t)c[2 + k]))
            return report_error(RP_ERR_INVALID, "hull cache truncated");
        if (st[k][0] != 0 || st[k].back() != c[2 + k]) return report_error(RP_ERR_INVALID, "hull cache table inconsistent");
    }
    if (off != in.size()) return report_error(RP_ERR_INVALID, "hull cache has trailing bytes");
    // index ranges and row monotonicity are checked by rp_hull_create_from_topology
    return rp_hull_create_from_topology(w, verts.data(), nv, normals.data(), nf, st[0].data(), dt[0].data(), st[1].data(),
                                        dt[1].data(), st[2].data(), dt[2].data(), st[3].data(), dt[3].data(), out_hull);
}

rp_status rp_hull_from_obj(rp_world* w, const char* path, const double scale[3], int32_t* out_hull) {
    if (!w || !path || !scale || !out_hull) return report_error(RP_ERR_INVALID, "null argument");
    FILE* f = fopen(path, "rb");
    if (!f) return report_error(RP_ERR_INVALID, "cannot open the OBJ file");
    std::vector<float> pos;            // the file's positions, as tinyobj stores them (FP32)
    std::vector<double> corners;       // one vertex per face corner, in face order (obj.cpp:45-80)
    std::string line;
    char buf[4096];
    bool bad = false;
    while (!bad && fgets(buf, sizeof(buf), f)) {
        line.assign(buf);
        while (!line.empty() && (line.back() == '\n' || line.back() == '\r')) line.pop_back();
        if (line.size() >= 2 && line[0] == 'v' && (line[1] == ' ' || line[1] == '\t')) {
            // parsed to double, stored as float (tinyobj's real_t)
            double x, y, z;
            if (sscanf(line.c_str() + 2, "%lf %lf %lf", &x, &y, &z) != 3) { bad = true; break; }
            pos.push_back((float)x);
            pos.push_back((float)y);
            pos.push_back((float)z);
        } else if (line.size() >= 2 && line[0] == 'f' && (line[1] == ' ' || line[1] == '\t')) {
            std::vector<int32_t> poly;
            char* save = nullptr;
            std::vector<char> tmp(line.begin() + 2, line.end());
            tmp.push_back('\0');
            for (char* tok = strtok_r(tmp.data(), " \t", &save); tok; tok = strtok_r(nullptr, " \t", &save)) {
                int32_t i;
                if (!obj_index(tok, (int32_t)(pos.size() / 3), i)) { bad = true; break; }
                poly.push_back(i);
            }
            if (bad) break;
            if (poly.size() < 3) continue;   // the loader skips faces of fewer than three corners
            std::vector<int32_t> tris;
            triangulate(pos, poly, tris);
            for (int32_t v : tris)
                for (int a = 0; a < 3; ++a) corners.push_back((double)pos[3 * (size_t)v + (size_t)a] * scale[a]);
        }
    }
    fclose(f);
    if (bad) return report_error(RP_ERR_INVALID, "malformed OBJ: a v line without three numbers or a bad face index");
    if (corners.empty()) return report_error(RP_ERR_INVALID, "OBJ file without faces");
    const uint32_t n = (uint32_t)(corners.size() / 3);
    std::vector<uint32_t> idx(n);
    for (uint32_t i = 0; i < n; ++i) idx[i] = i;
    return rp_hull_create(w, corners.data(), n, idx.data(), n, out_hull);
}

}  // extern "C"
