// t3d_oracle.cpp -- TEST INFRASTRUCTURE ONLY (parity checker and CPU baseline).
//
// A CPU restatement of Tetra3D's software vertex stage, following the Go
// reference function by function. Every routine cites the reference file:line it
// restates. Compile with -ffp-contract=off and without -ffast-math: the parity
// convention is unfused IEEE binary32 (the Go compiler may fuse x*y+z on arm64;
// on amd64 it does not).
//
// PARITY UNPINNED by reference tests: the reference has no golden vectors for
// this path and its Go sources cannot be compiled here. See t3d_oracle.h.

#include "t3d_oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <limits>
#include <memory>
#include <thread>
#include <functional>
#include <vector>

namespace {

// ---------------------------------------------------------------- math32 ----
// math32/math32.go: Sqrt/Tan/Cos/Atan/Round/Abs go through float64.
template <typename R> inline R m_sqrt(R x) { return (R)std::sqrt((double)x); }   // math32.go:126
template <typename R> inline R m_tan(R x) { return (R)std::tan((double)x); }     // math32.go:476
template <typename R> inline R m_cos(R x) { return (R)std::cos((double)x); }     // math32.go:147
template <typename R> inline R m_atan(R x) { return (R)std::atan((double)x); }   // math32.go:177
template <typename R> inline R m_round(R x) { return (R)std::round((double)x); } // math32.go:114
template <typename R> inline R m_abs(R x) { return (R)std::fabs((double)x); }    // math32.go:227
template <typename R> inline R m_clamp(R v, R lo, R hi) {                         // math32.go:39-47
    if (v < lo) return lo;
    else if (v > hi) return hi;
    return v;
}
template <typename R> inline R k(double v) { return (R)v; }
template <typename R> inline R maxf() { return (R)std::numeric_limits<float>::max(); }

// Go's int(float) for the light-volume cell index: values that cannot be a
// cell index map to -1 (no cell).
template <typename R> inline long long to_index(R v) {
    if (!(v > (R)-2147483648.0 && v < (R)2147483647.0)) return -1;
    return (long long)v;
}

template <typename R> struct V3 { R x, y, z; };
template <typename R> struct V4 { R x, y, z, w; };
template <typename R> struct M4 { R m[4][4]; };
template <typename R> struct C4 { R r, g, b, a; };

template <typename R> inline V3<R> v3(R x, R y, R z) { return V3<R>{x, y, z}; }
template <typename R> inline V3<R> add(V3<R> a, V3<R> b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }  // vector.go:86
template <typename R> inline V3<R> sub(V3<R> a, V3<R> b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }  // vector.go:112
template <typename R> inline V3<R> hmul(V3<R> a, V3<R> b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); } // vector.go Mult
template <typename R> inline R dot(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }      // vector.go:526
template <typename R> inline R magnitude(V3<R> a) { return m_sqrt<R>(a.x * a.x + a.y * a.y + a.z * a.z); } // vector.go:191
template <typename R> inline R dist2(V3<R> a, V3<R> b) {                                                  // vector.go:242
    R x = a.x - b.x, y = a.y - b.y, z = a.z - b.z;
    return x * x + y * y + z * z;
}
template <typename R> inline V3<R> unit(V3<R> a) {                                                        // vector.go:258-266
    R l = magnitude(a);
    if (l < k<R>(1e-8) || l == (R)1) return a;
    return v3(a.x / l, a.y / l, a.z / l);
}
template <typename R> inline V4<R> unit4(V4<R> a) {                                                       // vector.go:1869-1877
    R l = m_sqrt<R>(a.x * a.x + a.y * a.y + a.z * a.z);
    if (l < k<R>(1e-8) || l == (R)1) return a;
    return V4<R>{a.x / l, a.y / l, a.z / l, a.w};
}

template <typename R> inline M4<R> identity() {                                                           // matrix.go:13-23
    M4<R> r;
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) r.m[i][j] = (i == j) ? (R)1 : (R)0;
    return r;
}
template <typename R> inline M4<R> load_m(const float* p) {
    M4<R> r;
    for (int i = 0; i < 16; i++) r.m[i / 4][i % 4] = (R)p[i];
    return r;
}
// matrix_none.go:6-32 (and matrix_amd64.s, same order, no fusion)
template <typename R> inline M4<R> mult(const M4<R>& a, const M4<R>& b) {
    M4<R> n = identity<R>();
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++)
            n.m[i][j] = a.m[i][0] * b.m[0][j] + a.m[i][1] * b.m[1][j] + a.m[i][2] * b.m[2][j] + a.m[i][3] * b.m[3][j];
    return n;
}
template <typename R> inline M4<R> transposed(const M4<R>& a) {                                          // matrix.go:218-230
    M4<R> n = identity<R>();
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) n.m[i][j] = a.m[j][i];
    return n;
}
template <typename R> inline V3<R> mult_vec(const M4<R>& m, V3<R> v) {                                   // matrix.go:619-627
    return v3(m.m[0][0] * v.x + m.m[1][0] * v.y + m.m[2][0] * v.z + m.m[3][0],
              m.m[0][1] * v.x + m.m[1][1] * v.y + m.m[2][1] * v.z + m.m[3][1],
              m.m[0][2] * v.x + m.m[1][2] * v.y + m.m[2][2] * v.z + m.m[3][2]);
}
template <typename R> inline V4<R> mult_vec_w(const M4<R>& m, V3<R> v) {                                 // matrix.go:630-636, model.go:808-811
    return V4<R>{m.m[0][0] * v.x + m.m[1][0] * v.y + m.m[2][0] * v.z + m.m[3][0],
                 m.m[0][1] * v.x + m.m[1][1] * v.y + m.m[2][1] * v.z + m.m[3][1],
                 m.m[0][2] * v.x + m.m[1][2] * v.y + m.m[2][2] * v.z + m.m[3][2],
                 m.m[0][3] * v.x + m.m[1][3] * v.y + m.m[2][3] * v.z + m.m[3][3]};
}
template <typename R> inline M4<R> translate(R x, R y, R z) {                                            // matrix.go:82-88
    M4<R> r = identity<R>();
    r.m[3][0] = x; r.m[3][1] = y; r.m[3][2] = z;
    return r;
}
template <typename R> inline M4<R> scale_m(R x, R y, R z) {                                              // matrix.go:91-97
    M4<R> r = identity<R>();
    r.m[0][0] = x; r.m[1][1] = y; r.m[2][2] = z;
    return r;
}
// matrix.go:255-307
template <typename R> M4<R> inverted(const M4<R>& M) {
    const R(&m)[4][4] = M.m;
    R A2323 = m[2][2] * m[3][3] - m[2][3] * m[3][2];
    R A1323 = m[2][1] * m[3][3] - m[2][3] * m[3][1];
    R A1223 = m[2][1] * m[3][2] - m[2][2] * m[3][1];
    R A0323 = m[2][0] * m[3][3] - m[2][3] * m[3][0];
    R A0223 = m[2][0] * m[3][2] - m[2][2] * m[3][0];
    R A0123 = m[2][0] * m[3][1] - m[2][1] * m[3][0];
    R A2313 = m[1][2] * m[3][3] - m[1][3] * m[3][2];
    R A1313 = m[1][1] * m[3][3] - m[1][3] * m[3][1];
    R A1213 = m[1][1] * m[3][2] - m[1][2] * m[3][1];
    R A2312 = m[1][2] * m[2][3] - m[1][3] * m[2][2];
    R A1312 = m[1][1] * m[2][3] - m[1][3] * m[2][1];
    R A1212 = m[1][1] * m[2][2] - m[1][2] * m[2][1];
    R A0313 = m[1][0] * m[3][3] - m[1][3] * m[3][0];
    R A0213 = m[1][0] * m[3][2] - m[1][2] * m[3][0];
    R A0312 = m[1][0] * m[2][3] - m[1][3] * m[2][0];
    R A0212 = m[1][0] * m[2][2] - m[1][2] * m[2][0];
    R A0113 = m[1][0] * m[3][1] - m[1][1] * m[3][0];
    R A0112 = m[1][0] * m[2][1] - m[1][1] * m[2][0];
    R det = m[0][0] * (m[1][1] * A2323 - m[1][2] * A1323 + m[1][3] * A1223) -
            m[0][1] * (m[1][0] * A2323 - m[1][2] * A0323 + m[1][3] * A0223) +
            m[0][2] * (m[1][0] * A1323 - m[1][1] * A0323 + m[1][3] * A0123) -
            m[0][3] * (m[1][0] * A1223 - m[1][1] * A0223 + m[1][2] * A0123);
    det = (R)1 / det;
    M4<R> r = identity<R>();
    r.m[0][0] = det * (m[1][1] * A2323 - m[1][2] * A1323 + m[1][3] * A1223);
    r.m[0][1] = det * -(m[0][1] * A2323 - m[0][2] * A1323 + m[0][3] * A1223);
    r.m[0][2] = det * (m[0][1] * A2313 - m[0][2] * A1313 + m[0][3] * A1213);
    r.m[0][3] = det * -(m[0][1] * A2312 - m[0][2] * A1312 + m[0][3] * A1212);
    r.m[1][0] = det * -(m[1][0] * A2323 - m[1][2] * A0323 + m[1][3] * A0223);
    r.m[1][1] = det * (m[0][0] * A2323 - m[0][2] * A0323 + m[0][3] * A0223);
    r.m[1][2] = det * -(m[0][0] * A2313 - m[0][2] * A0313 + m[0][3] * A0213);
    r.m[1][3] = det * (m[0][0] * A2312 - m[0][2] * A0312 + m[0][3] * A0212);
    r.m[2][0] = det * (m[1][0] * A1323 - m[1][1] * A0323 + m[1][3] * A0123);
    r.m[2][1] = det * -(m[0][0] * A1323 - m[0][1] * A0323 + m[0][3] * A0123);
    r.m[2][2] = det * (m[0][0] * A1313 - m[0][1] * A0313 + m[0][3] * A0113);
    r.m[2][3] = det * -(m[0][0] * A1312 - m[0][1] * A0312 + m[0][3] * A0112);
    r.m[3][0] = det * -(m[1][0] * A1223 - m[1][1] * A0223 + m[1][2] * A0123);
    r.m[3][1] = det * (m[0][0] * A1223 - m[0][1] * A0223 + m[0][2] * A0123);
    r.m[3][2] = det * -(m[0][0] * A1213 - m[0][1] * A0213 + m[0][2] * A0113);
    r.m[3][3] = det * (m[0][0] * A1212 - m[0][1] * A0212 + m[0][2] * A0112);
    return r;
}
// matrix.go:181-196
template <typename R> void decompose(const M4<R>& M, V3<R>& pos, V3<R>& scl, M4<R>& rot) {
    pos = v3(M.m[3][0], M.m[3][1], M.m[3][2]);
    rot = identity<R>();
    for (int i = 0; i < 3; i++) {
        V4<R> row = unit4(V4<R>{M.m[i][0], M.m[i][1], M.m[i][2], M.m[i][3]});
        rot.m[i][0] = row.x; rot.m[i][1] = row.y; rot.m[i][2] = row.z; rot.m[i][3] = row.w;
    }
    M4<R> in = mult(M, transposed(rot));
    scl = v3(magnitude(v3(in.m[0][0], in.m[0][1], in.m[0][2])),
             magnitude(v3(in.m[1][0], in.m[1][1], in.m[1][2])),
             magnitude(v3(in.m[2][0], in.m[2][1], in.m[2][2])));
}
template <typename R> inline V3<R> row3(const M4<R>& M, int i) { return v3(M.m[i][0], M.m[i][1], M.m[i][2]); }
template <typename R> inline V3<R> forward(const M4<R>& M) { return unit(row3(M, 2)); }  // matrix.go:169-175
template <typename R> inline V3<R> right(const M4<R>& M) { return unit(row3(M, 0)); }    // matrix.go:151-157
template <typename R> inline V3<R> up(const M4<R>& M) { return unit(row3(M, 1)); }       // matrix.go:160-166

// ----------------------------------------------------------------- scene ----
struct Dims { float mn[3], mx[3]; };

template <typename R> struct Camera {
    const t3d_camera_desc* d;
    M4<R> vp;
    V3<R> pos, fwd, rgt, upv;
    R sphere_tang, sphere_y, sphere_x, aspect;
    R near_, far_, W, H, halfW, halfH, margin, spread;
};

template <typename R> struct LightPrep {  // per frame (beginRender, light.go:110-113, :318-320)
    int type;
    V3<R> color;
    R energy, range, range2;
    V3<R> wpos;        // WorldPosition
    V3<R> amb;         // ambient premultiplied result
    V3<R> fwd;         // directional workingForward
    const t3d_light_desc* d;
};

template <typename R> struct ModelState {
    M4<R> transform, world_rot;
};

// One render pair: model index + part index + draw-order slot.
struct Pair { uint32_t model, part; float depth; int32_t order; bool batch = false; uint32_t draw = 0, draw_transparent = 0; };

// Mesh.SetAutoSubdivide (mesh.go:447-490) restated: every part triangle,
// then the triangles of its subdivision levels (forEachTri order,
// mesh.go:2238-2256); new vertices appended; per listed triangle its centre
// and, for handleSubdivision, the base's Normal, MaxSpan and level count.
struct SubMesh {
    std::vector<float> pos, nrm, uv, col;
    std::vector<uint32_t> idx;
    std::vector<float> ctr;
    std::vector<float> bnormal, bspan;  // per listed triangle: its base triangle's Normal (3) and MaxSpan
    std::vector<int> level, nlevels, base;  // level (-1: the base), the base's level count, the base's entry
    std::vector<t3d_part_desc> parts;
    t3d_mesh_desc desc;
};

struct Subdivision {  // Triangle.performSubdivision (mesh.go:1758-1864)
    SubMesh& M;
    bool colors;
    float intended;
    int max_count;
    struct T { uint32_t a, b, c; float span; float ctr[3]; };
    std::vector<std::vector<T>> lv;
    void lerp3(std::vector<float>& v, int n, uint32_t i, uint32_t j) {  // Lerp(.., 0.5)
        for (int k = 0; k < n; k++) {
            float a = v[n * (size_t)i + k], b = v[n * (size_t)j + k];
            v.push_back(a + ((b - a) * 0.5f));
        }
    }
    T make(uint32_t a, uint32_t b, uint32_t c, float span) {
        T t{a, b, c, span, {0, 0, 0}};
        const float* P = M.pos.data();
        for (int k = 0; k < 3; k++)  // Add(..).Add(..).Scale(1.0 / 3.0)
            t.ctr[k] = ((P[3 * (size_t)a + k] + P[3 * (size_t)b + k]) + P[3 * (size_t)c + k]) * (float)(1.0 / 3.0);
        return t;
    }
    void run(int level, T t) {
        if (level == max_count || t.span <= intended) return;
        const uint32_t s = (uint32_t)(M.pos.size() / 3);
        const uint32_t e[3][2] = {{t.a, t.b}, {t.b, t.c}, {t.c, t.a}};
        for (auto& q : e) lerp3(M.pos, 3, q[0], q[1]);
        for (auto& q : e) lerp3(M.nrm, 3, q[0], q[1]);
        for (auto& q : e) lerp3(M.uv, 2, q[0], q[1]);
        if (colors)
            for (auto& q : e) lerp3(M.col, 4, q[0], q[1]);
        T A = make(t.a, s, s + 2, t.span / 2), B = make(s, t.b, s + 1, t.span / 2);
        T C = make(s + 1, t.c, s + 2, t.span / 2), D = make(s, s + 1, s + 2, t.span / 2);
        lv[level].insert(lv[level].end(), {A, B, C, D});
        run(level + 1, A);
        run(level + 1, B);
        run(level + 1, C);
        run(level + 1, D);
    }
};

void build_submesh(const t3d_mesh_desc& me, const float* levels, uint32_t nlev, int max_count, SubMesh& M) {
    M.pos.assign(me.positions, me.positions + 3 * (size_t)me.num_vertices);
    M.nrm.assign(me.normals, me.normals + 3 * (size_t)me.num_vertices);
    M.uv.assign(me.uvs, me.uvs + 2 * (size_t)me.num_vertices);
    if (me.colors) M.col.assign(me.colors, me.colors + 4 * (size_t)me.num_vertices);
    float smallest = std::numeric_limits<float>::max();
    for (uint32_t i = 0; i < nlev; i++) smallest = std::min(smallest, levels[2 * i + 1]);
    Subdivision div{M, me.colors != nullptr, smallest, max_count, {}};
    auto cross3 = [](V3<float> a, V3<float> b) {  // Vector3.Cross, vector.go:164-175
        return v3<float>(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
    };
    for (uint32_t p = 0; p < me.num_parts; p++) {
        t3d_part_desc part = me.parts[p];
        uint32_t first = (uint32_t)(M.idx.size() / 3);
        for (uint32_t t = me.parts[p].tri_start; t < me.parts[p].tri_start + me.parts[p].tri_count; t++) {
            uint32_t a = me.indices[3 * (size_t)t], b = me.indices[3 * (size_t)t + 1], c = me.indices[3 * (size_t)t + 2];
            V3<float> pa = v3<float>(M.pos[3 * (size_t)a], M.pos[3 * (size_t)a + 1], M.pos[3 * (size_t)a + 2]);
            V3<float> pb = v3<float>(M.pos[3 * (size_t)b], M.pos[3 * (size_t)b + 1], M.pos[3 * (size_t)b + 2]);
            V3<float> pc = v3<float>(M.pos[3 * (size_t)c], M.pos[3 * (size_t)c + 1], M.pos[3 * (size_t)c + 2]);
            // MaxSpan = max of the edge lengths (mesh.go:2020-2024), Normal (mesh.go:2030-2037, :2171-2179)
            float e0 = magnitude(sub(pa, pb)), e1 = magnitude(sub(pb, pc)), e2 = magnitude(sub(pc, pa));
            float span = (std::isnan(e0) || std::isnan(e1) || std::isnan(e2)) ? NAN : std::max(std::max(e0, e1), e2);
            V3<float> n = unit(cross3(sub(pb, pa), sub(pc, pb)));
            if (!(std::fabs(n.x) > 1e-4f || std::fabs(n.y) > 1e-4f || std::fabs(n.z) > 1e-4f))
                n = v3<float>(me.normals[3 * (size_t)a], me.normals[3 * (size_t)a + 1], me.normals[3 * (size_t)a + 2]);
            int nl = span <= smallest ? 0 : max_count;
            div.lv.assign(nl, {});
            if (nl) div.run(0, Subdivision::T{a, b, c, span, {0, 0, 0}});
            int baseEntry = (int)(M.idx.size() / 3);
            auto push = [&](uint32_t x, uint32_t y, uint32_t z, const float* ctr, int level) {
                M.idx.insert(M.idx.end(), {x, y, z});
                M.ctr.insert(M.ctr.end(), {ctr[0], ctr[1], ctr[2]});
                M.bnormal.insert(M.bnormal.end(), {n.x, n.y, n.z});
                M.bspan.push_back(span);
                M.level.push_back(level);
                M.nlevels.push_back(nl);
                M.base.push_back(baseEntry);
            };
            float c0[3] = {(pa.x + pb.x + pc.x) / 3.0f, (pa.y + pb.y + pc.y) / 3.0f, (pa.z + pb.z + pc.z) / 3.0f};
            push(a, b, c, c0, -1);
            for (int L = 0; L < nl; L++)
                for (auto& st : div.lv[L]) push(st.a, st.b, st.c, st.ctr, L);
        }
        part.tri_start = first;
        part.tri_count = (uint32_t)(M.idx.size() / 3) - first;
        M.parts.push_back(part);
    }
    M.desc = me;
    M.desc.positions = M.pos.data();
    M.desc.normals = M.nrm.data();
    M.desc.uvs = M.uv.data();
    M.desc.colors = me.colors ? M.col.data() : nullptr;
    M.desc.indices = M.idx.data();
    M.desc.parts = M.parts.data();
    M.desc.num_vertices = (uint32_t)(M.pos.size() / 3);
    M.desc.num_triangles = (uint32_t)(M.idx.size() / 3);
}

// closestPointOnTri (colliderTriangles.go:177-281)
template <typename R> V3<R> closest_on_line(V3<R> point, V3<R> start, V3<R> end) {
    V3<R> diff = sub(end, start);
    R d = dot(sub(point, start), diff) / dot(diff, diff);
    if (d > 1) d = 1;
    else if (d < 0) d = 0;
    return add(start, v3<R>(diff.x * d, diff.y * d, diff.z * d));
}
template <typename R> V3<R> closest_on_tri(V3<R> point, V3<R> v0, V3<R> v1, V3<R> v2, V3<R> normal) {
    R distance = dot(normal, v0);
    R dist = dot(normal, point) - distance;
    V3<R> planePoint = sub(point, v3<R>(normal.x * dist, normal.y * dist, normal.z * dist));
    V3<R> ca = sub(v2, v0), ba = sub(v1, v0), pa = sub(planePoint, v0);
    R dot00 = dot(ca, ca), dot01 = dot(ca, ba), dot02 = dot(ca, pa), dot11 = dot(ba, ba), dot12 = dot(ba, pa);
    R invDenom = (R)1 / ((dot00 * dot11) - (dot01 * dot01));
    R u = ((dot11 * dot02) - (dot01 * dot12)) * invDenom;
    R v = ((dot00 * dot12) - (dot01 * dot02)) * invDenom;
    if (u >= 0 && v >= 0 && u + v < 1) return planePoint;
    V3<R> ab = closest_on_line(point, v0, v1), bc = closest_on_line(point, v1, v2), cap = closest_on_line(point, v2, v0);
    V3<R> closest = ab;
    R closestDist = dist2(point, ab), bcDist = dist2(point, bc), caDist = dist2(point, cap);
    if (bcDist < closestDist) { closest = bc; closestDist = bcDist; }
    if (caDist < closestDist) closest = cap;
    return closest;
}

// Triangle.handleSubdivision (mesh.go:1877-1949) for listed triangle t: is it
// the base (level -1) or on the level that the base triangle picks?
template <typename R> bool subdiv_active(const t3d_scene_desc* sc, const SubMesh& M, uint32_t t, V3<R> camPos) {
    const int nl = M.nlevels[t], level = M.level[t];
    if (nl == 0) return level < 0;
    const uint32_t b = (uint32_t)M.base[t];
    V3<R> v[3];
    for (int i = 0; i < 3; i++) {
        const uint32_t k = M.idx[3 * (size_t)b + i];
        v[i] = v3<R>((R)M.pos[3 * (size_t)k], (R)M.pos[3 * (size_t)k + 1], (R)M.pos[3 * (size_t)k + 2]);
    }
    V3<R> n = v3<R>((R)M.bnormal[3 * (size_t)t], (R)M.bnormal[3 * (size_t)t + 1], (R)M.bnormal[3 * (size_t)t + 2]);
    R dist = dist2(camPos, closest_on_tri(camPos, v[0], v[1], v[2], n));
    int active = -1;
    R closestDistance = maxf<R>();
    for (uint32_t i = 0; i < sc->num_subdivision_levels; i++) {
        R d2 = (R)sc->subdivision_levels[2 * i];
        if (dist < d2 && d2 < closestDistance) { closestDistance = d2; active = (int)i; }
    }
    if (active == -1) return level < 0;
    R ms = (R)M.bspan[t];
    int subIndex = -1;
    while (ms > (R)sc->subdivision_levels[2 * active + 1]) { ms /= 2; subIndex++; }
    if (subIndex >= nl) subIndex = nl - 1;
    return subIndex >= 0 ? level == subIndex : level < 0;
}

template <typename R> struct Frame {
    const t3d_scene_desc* sc;
    std::vector<std::unique_ptr<SubMesh>> sub;  // auto-subdivided meshes
    std::vector<const t3d_mesh_desc*> mesh;     // the mesh each model draws (subdivided or as given)
    Camera<R> cam;
    std::vector<LightPrep<R>> lights;
    std::vector<ModelState<R>> models;
    std::vector<Dims> dims;
    const uint64_t* mask;
    std::vector<uint32_t> scene_lights;  // list 0 after the light mask and Camera.MaxLightCount
};

inline bool light_enabled(const uint64_t* mask, uint32_t i) {
    if (!mask) return true;
    if (i >= 128) return false;
    return (mask[i >> 6] >> (i & 63)) & 1ull;
}

// sort.SliceStable of Go's standard library (sort/zsortfunc.go): insertionSort over
// 20-element blocks, then symMerge of doubling runs (Kim & Kutzner's SymMerge with
// rotations by block swaps). Camera.Render (camera.go:1482-1495) sorts the scene lights
// with it under a comparator that is not a strict weak order, so its exact steps matter.
struct GoSort {
    std::vector<uint32_t>& v;
    std::function<bool(uint32_t, uint32_t)> less;
    bool lt(int i, int j) const { return less(v[i], v[j]); }
    void sw(int i, int j) { std::swap(v[i], v[j]); }
    void insertion_sort(int a, int b) {
        for (int i = a + 1; i < b; i++)
            for (int j = i; j > a && lt(j, j - 1); j--) sw(j, j - 1);
    }
    void swap_range(int a, int b, int n) {
        for (int i = 0; i < n; i++) sw(a + i, b + i);
    }
    void rotate(int a, int m, int b) {
        int i = m - a, j = b - m;
        while (i != j) {
            if (i > j) { swap_range(m - i, m, j); i -= j; }
            else { swap_range(m - i, m + j - i, i); j -= i; }
        }
        swap_range(m - i, m, i);
    }
    void sym_merge(int a, int m, int b) {
        if (m - a == 1) {  // insert v[a] into v[m:b]
            int i = m, j = b;
            while (i < j) { int h = (int)((unsigned)(i + j) >> 1); if (lt(h, a)) i = h + 1; else j = h; }
            for (int k = a; k < i - 1; k++) sw(k, k + 1);
            return;
        }
        if (b - m == 1) {  // insert v[m] into v[a:m]
            int i = a, j = m;
            while (i < j) { int h = (int)((unsigned)(i + j) >> 1); if (!lt(m, h)) i = h + 1; else j = h; }
            for (int k = m; k > i; k--) sw(k, k - 1);
            return;
        }
        int mid = (int)((unsigned)(a + b) >> 1), n = mid + m, start, r;
        if (m > mid) { start = n - b; r = mid; } else { start = a; r = m; }
        int p = n - 1;
        while (start < r) { int c = (int)((unsigned)(start + r) >> 1); if (!lt(p - c, c)) start = c + 1; else r = c; }
        int end = n - start;
        if (start < m && m < end) rotate(start, m, end);
        if (a < start && start < mid) sym_merge(a, start, mid);
        if (mid < end && end < b) sym_merge(mid, end, b);
    }
    void run() {
        int n = (int)v.size(), bs = 20, a = 0, b = bs;
        for (; b <= n; a = b, b += bs) insertion_sort(a, b);
        insertion_sort(a, n);
        for (; bs < n; bs *= 2) {
            a = 0; b = 2 * bs;
            for (; b <= n; a = b, b += 2 * bs) sym_merge(a, a + bs, b);
            if (a + bs < n) sym_merge(a, a + bs, n);
        }
    }
};

// Mesh.UpdateDimensions (mesh.go:713-748)
Dims mesh_dims(const t3d_mesh_desc& me) {
    Dims d;
    if (me.has_dimensions) {
        for (int c = 0; c < 3; c++) { d.mn[c] = me.dim_min[c]; d.mx[c] = me.dim_max[c]; }
        return d;
    }
    for (int c = 0; c < 3; c++) { d.mn[c] = std::numeric_limits<float>::max(); d.mx[c] = -std::numeric_limits<float>::max(); }
    for (uint32_t v = 0; v < me.num_vertices; v++)
        for (int c = 0; c < 3; c++) {
            float p = me.positions[3 * v + c];
            if (d.mn[c] > p) d.mn[c] = p;
            if (d.mx[c] < p) d.mx[c] = p;
        }
    return d;
}

// Model.isTransparent (model.go:1274-1282)
bool is_transparent(const t3d_model_desc& m, const t3d_part_desc& p) {
    const t3d_material& mat = p.mat;
    if (mat.present) {
        bool matT = mat.transparency_mode == T3D_TRANSPARENCY_TRANSPARENT || !mat.blend_source_over ||
                    (mat.transparency_mode == T3D_TRANSPARENCY_AUTO && mat.color[3] < 0.999f);
        bool modelT = mat.transparency_mode != T3D_TRANSPARENCY_OPAQUE && m.color[3] < 0.999f;
        return matT || modelT;
    }
    return m.color[3] < 0.999f;
}

// Camera.ViewMatrix / Projection / Clear basis (camera.go:638-679, :1085-1088)
template <typename R> void setup_camera(Camera<R>& c, const t3d_camera_desc* d) {
    c.d = d;
    M4<R> ct = load_m<R>(d->transform);
    M4<R> cr = load_m<R>(d->world_rotation);
    c.pos = row3(ct, 3);
    M4<R> view = mult(translate<R>(-c.pos.x, -c.pos.y, -c.pos.z), transposed(cr));
    R fov = (R)d->fov_y, nr = (R)d->near_plane, fr = (R)d->far_plane;
    R W = (R)d->width, H = (R)d->height;
    c.aspect = W / H;  // AspectRatio, camera.go:992-995
    R angle = fov * k<R>(3.1415) / (R)360;
    c.sphere_tang = m_tan<R>(angle);
    c.sphere_y = (R)1 / m_cos<R>(angle);
    c.sphere_x = (R)1 / m_cos<R>(m_atan<R>(c.sphere_tang * c.aspect));
    M4<R> proj;
    if (d->perspective) {  // matrix.go:588-604
        R aspect = W / H;
        R t = m_tan<R>(fov * (R)(float)M_PI / (R)360);
        R b = -t, r = t * aspect, l = -r;
        proj = identity<R>();
        proj.m[0][0] = ((R)2 * nr) / (r - l); proj.m[0][1] = 0; proj.m[0][2] = (r + l) / (r - l); proj.m[0][3] = 0;
        proj.m[1][0] = 0; proj.m[1][1] = ((R)2 * nr) / (t - b); proj.m[1][2] = (t + b) / (t - b); proj.m[1][3] = 0;
        proj.m[2][0] = 0; proj.m[2][1] = 0; proj.m[2][2] = -((fr + nr) / (fr - nr)); proj.m[2][3] = -(((R)2 * fr * nr) / (fr - nr));
        proj.m[3][0] = 0; proj.m[3][1] = 0; proj.m[3][2] = -1; proj.m[3][3] = 0;
    } else {  // camera.go:670-675, matrix.go:609-616
        R asr = H / W;
        R os = (R)d->ortho_scale;
        R right_ = (R)1 * os, left_ = (R)-1 * os, top = asr * os, bottom = -asr * os;
        proj = identity<R>();
        proj.m[0][0] = (R)2 / (right_ - left_);
        proj.m[1][1] = (R)2 / (top - bottom);
        proj.m[2][2] = (R)-2 / (fr - nr);
        proj.m[3][3] = 1;
    }
    c.vp = mult(view, proj);
    c.fwd = forward(cr); c.rgt = right(cr); c.upv = up(cr);
    c.near_ = nr; c.far_ = fr; c.W = W; c.H = H;
    c.halfW = W / (R)2; c.halfH = H / (R)2;
    c.margin = (fr - nr) * (R)d->depth_margin;      // camera.go:1339
    c.spread = fr - nr + (c.margin * (R)2);         // camera.go:1341
}

// Camera.SphereInFrustum (camera.go:933-983)
template <typename R> bool sphere_in_frustum(const Camera<R>& c, V3<R> position, R radius) {
    V3<R> diff = sub(position, c.pos);
    V3<R> fi = v3(-c.fwd.x, -c.fwd.y, -c.fwd.z);
    R pcZ = dot(diff, fi);
    if (pcZ > c.far_ + radius || pcZ < c.near_ - radius) return false;
    if (c.d->perspective) {
        R d = c.sphere_y * radius;
        pcZ *= c.sphere_tang;
        R pcY = dot(diff, c.upv);
        if (pcY > pcZ + d || pcY < -pcZ - d) return false;
        pcZ *= c.aspect;
        d = c.sphere_x * radius;
        R pcX = dot(diff, c.rgt);
        if (pcX > pcZ + d || pcX < -pcZ - d) return false;
    } else {
        R width = (R)c.d->ortho_scale;
        R height = width / c.aspect;
        R pcY = dot(diff, c.upv);
        if (-height / (R)2 - radius > pcY || pcY > height / (R)2 + radius) return false;
        R pcX = dot(diff, c.rgt);
        if (-width / (R)2 - radius > pcX || pcX > width / (R)2 + radius) return false;
    }
    return true;
}

// Model.onTransformUpdate (model.go:142-182) + ModelInFrustum (camera.go:986-989);
// a skinned model's sphere has no mesh-centre offset (model.go:158-161)
template <typename R> bool model_in_frustum(const Camera<R>& c, const M4<R>& transform, const Dims& dm, bool skinned) {
    V3<R> position, scale; M4<R> rotation;
    decompose(transform, position, scale, rotation);
    V3<R> center = v3<R>(0, 0, 0);
    if (!skinned)
        center = v3<R>(((R)dm.mx[0] + (R)dm.mn[0]) / (R)2, ((R)dm.mx[1] + (R)dm.mn[1]) / (R)2,
                       ((R)dm.mx[2] + (R)dm.mn[2]) / (R)2);
    center = mult_vec(rotation, center);
    position.x += center.x * scale.x;
    position.y += center.y * scale.y;
    position.z += center.z * scale.z;
    V3<R> mn = v3<R>((R)dm.mn[0] * scale.x, (R)dm.mn[1] * scale.y, (R)dm.mn[2] * scale.z);
    V3<R> mx = v3<R>((R)dm.mx[0] * scale.x, (R)dm.mx[1] * scale.y, (R)dm.mx[2] * scale.z);
    R radius = magnitude(sub(mx, mn)) / (R)2;
    return sphere_in_frustum(c, position, radius);
}

// ---------------------------------------------------------- billboards ----
template <typename R> inline bool vequals(V3<R> a, V3<R> b) {  // Vector3.Equals, vector.go:415-425
    const R eps = k<R>(1e-4);
    return !(m_abs<R>(a.x - b.x) > eps || m_abs<R>(a.y - b.y) > eps || m_abs<R>(a.z - b.z) > eps);
}
template <typename R> inline V3<R> cross(V3<R> a, V3<R> b) {  // Vector3.Cross, vector.go:164-175
    R z = a.x * b.y - b.x * a.y;
    R y = a.z * b.x - b.z * a.x;
    R x = a.y * b.z - b.y * a.z;
    return v3(x, y, z);
}
template <typename R> M4<R> look_at(V3<R> from, V3<R> to, V3<R> up) {  // NewMatrix4LookAt, matrix.go:788-815
    if (vequals(from, to)) return identity<R>();
    V3<R> z = unit(sub(to, from));
    up = unit(up);
    if (vequals(z, up) || vequals(z, v3<R>(-up.x, -up.y, -up.z))) {
        if (!vequals(up, v3<R>(1, 0, 0))) up = v3<R>(1, 0, 0);
        else up = v3<R>(0, 0, 1);
    }
    V3<R> x = unit(cross(up, z));
    V3<R> y = cross(z, x);
    M4<R> m = identity<R>();
    m.m[0][0] = x.x; m.m[0][1] = x.y; m.m[0][2] = x.z; m.m[0][3] = 0;
    m.m[1][0] = y.x; m.m[1][1] = y.y; m.m[1][2] = y.z; m.m[1][3] = 0;
    m.m[2][0] = z.x; m.m[2][1] = z.y; m.m[2][2] = z.z; m.m[2][3] = 0;
    return m;
}
template <typename R> inline V4<R> row4(const M4<R>& m, int i) { return V4<R>{m.m[i][0], m.m[i][1], m.m[i][2], m.m[i][3]}; }
template <typename R> inline void set_row(M4<R>& m, int i, V4<R> v) {  // Matrix4.SetRow, matrix.go:564-569
    m.m[i][0] = v.x; m.m[i][1] = v.y; m.m[i][2] = v.z; m.m[i][3] = v.w;
}
// The billboarded `base` of ProcessVertices (model.go:634-688).
template <typename R>
M4<R> billboard_base(const M4<R>& modelTransform, const Camera<R>& cam, const t3d_material& mat) {
    V3<R> up = v3<R>(0, 1, 0);  // WorldUp
    if (mat.billboard_up == T3D_BILLBOARD_UP_CAMERA_Y) up = cam.upv;
    M4<R> lookat = look_at(row3(modelTransform, 3), cam.pos, up);
    if (mat.billboard_lock[0]) {
        set_row(lookat, 0, V4<R>{1, 0, 0, 0});
        V4<R> row = row4(lookat, 1); row.x = 0; set_row(lookat, 1, unit4(row));
        row = row4(lookat, 2); row.x = 0; set_row(lookat, 2, unit4(row));
    }
    if (mat.billboard_lock[1]) {
        set_row(lookat, 1, V4<R>{0, 1, 0, 0});
        V4<R> row = row4(lookat, 0); row.y = 0; set_row(lookat, 0, unit4(row));
        row = row4(lookat, 2); row.y = 0; set_row(lookat, 2, unit4(row));
    }
    if (mat.billboard_lock[2]) {
        set_row(lookat, 2, V4<R>{0, 0, 1, 0});
        V4<R> row = row4(lookat, 0); row.z = 0; set_row(lookat, 0, unit4(row));
        row = row4(lookat, 1); row.z = 0; set_row(lookat, 1, unit4(row));
    }
    V3<R> p, s; M4<R> r;
    decompose(modelTransform, p, s, r);
    M4<R> base = mult(mult(r, scale_m<R>(s.x, s.y, s.z)), lookat);
    set_row(base, 3, V4<R>{p.x, p.y, p.z, 1});
    return base;
}

// ------------------------------------------------------ per-pair render ----
template <typename R> struct Scratch {
    std::vector<V4<R>> clip;               // globalVertexTransforms
    std::vector<V3<R>> apos, anrm;         // globalMeshAlteredVertexPositions / Normals
    std::vector<R> udepth;                 // globalVertexDepthUnbillboarded
    std::vector<C4<R>> vlight;             // mesh.vertexLights
    std::vector<std::vector<std::pair<uint32_t, R>>> bins;
    std::vector<std::pair<uint32_t, R>> unset;
    Scratch() : bins(512) {}
};

template <typename R> struct ModelLight {  // beginModel results for one model
    const LightPrep<R>* l;
    V3<R> working;          // point workingPosition
    bool skip;              // model-level point-range skip (camera.go:1625-1629)
    const std::vector<ModelLight<R>>* nested = nullptr;  // every scene light after beginModel (cell useLights)
};

// LightVolume helpers (light.go:717-741, :1267-1272)
template <typename R> bool lv_cell(const t3d_light_desc* d, V3<R> p, long long& idx) {
    R csx = (R)d->cell_size[0], csy = (R)d->cell_size[1], csz = (R)d->cell_size[2];
    long long x = to_index<R>(m_round<R>(((p.x - (R)d->offset[0] - (R)d->vol_min[0] - (csx / (R)2)) / csx)));
    long long y = to_index<R>(m_round<R>(((p.y - (R)d->offset[1] - (R)d->vol_min[1] - (csy / (R)2)) / csy)));
    long long z = to_index<R>(m_round<R>(((p.z - (R)d->offset[2] - (R)d->vol_min[2] - (csz / (R)2)) / csz)));
    if (x < 0 || y < 0 || z < 0 || x >= d->cell_count[0] || y >= d->cell_count[1] || z >= d->cell_count[2]) return false;
    idx = x + (y * d->cell_count[0]) + (z * d->cell_count[0] * d->cell_count[1]);
    return true;
}

// vpos / vnrm: the altered vertex (model space, or world space when skinned).
template <typename R>
void vertex_light(const Frame<R>& F, const ModelLight<R>& ml, const t3d_part_desc& part, bool skinned,
                  const M4<R>& transform, const M4<R>& dir_rot, V3<R> vpos, V3<R> vnrm, C4<R>& tgt) {
    const LightPrep<R>& L = *ml.l;
    const t3d_material& mat = part.mat;
    switch (L.type) {
    case T3D_LIGHT_AMBIENT:  // light.go:115-120
        tgt.r += L.amb.x; tgt.g += L.amb.y; tgt.b += L.amb.z;
        break;
    case T3D_LIGHT_POINT: {  // light.go:191-258
        R distance = dist2(ml.working, vpos);
        if (L.range > 0) {
            if (distance > L.range2) return;
        } else {
            if ((R)1 / distance * L.energy < k<R>(0.001)) return;
        }
        V3<R> lightVec = unit(sub(ml.working, vpos));
        V3<R> n = vnrm;
        if (mat.present && mat.lighting_mode == T3D_LIGHTING_FIXED_NORMALS) n = lightVec;
        R diffuse = dot(n, lightVec);
        if (mat.present && mat.lighting_mode == T3D_LIGHTING_DOUBLE_SIDED) diffuse = m_abs<R>(diffuse);
        if (diffuse > 0) {
            R diffuseFactor = diffuse * ((R)1 / ((R)1 + (k<R>(0.1) * distance))) * (R)2;
            if (L.range2 > 0) {
                R distClamp = m_clamp<R>((L.range2 - distance) / distance, 0, 1);
                diffuseFactor *= distClamp;
            }
            tgt.r += L.color.x * diffuseFactor * L.energy;
            tgt.g += L.color.y * diffuseFactor * L.energy;
            tgt.b += L.color.z * diffuseFactor * L.energy;
        }
        break;
    }
    case T3D_LIGHT_DIRECTIONAL: {  // light.go:332-360
        V3<R> normal;
        if (mat.present && mat.lighting_mode == T3D_LIGHTING_FIXED_NORMALS) normal = L.fwd;
        else if (skinned) normal = vnrm;
        else normal = mult_vec(dir_rot, vnrm);
        R diffuseFactor = dot(normal, L.fwd);
        if (mat.present && mat.lighting_mode == T3D_LIGHTING_DOUBLE_SIDED) diffuseFactor = m_abs<R>(diffuseFactor);
        if (diffuseFactor <= 0) return;
        tgt.r += L.color.x * diffuseFactor * L.energy;
        tgt.g += L.color.y * diffuseFactor * L.energy;
        tgt.b += L.color.z * diffuseFactor * L.energy;
        break;
    }
    case T3D_LIGHT_VOLUME: {  // light.go:583-663 (+ Light :667-678)
        if (mat.present && mat.lv_shading_mode == T3D_LV_OFF) return;
        const t3d_light_desc* d = L.d;
        int mode = mat.present ? mat.lv_shading_mode : 0;
        C4<R> cellColor{0, 0, 0, 1};
        V3<R> cellSize = v3<R>((R)d->cell_size[0] / (R)2, (R)d->cell_size[1] / (R)2, (R)d->cell_size[2] / (R)2);
        V3<R> bias = v3<R>((R)d->bias[0], (R)d->bias[1], (R)d->bias[2]);
        long long idx;
        if (mat.present && mode == T3D_LV_PER_OBJECT) {
            if (lv_cell(d, row3(transform, 3), idx)) {
                const float* cc = F.sc->volume_cells + 4 * (size_t)(d->cell_first + idx);
                cellColor.r = (R)cc[0]; cellColor.g = (R)cc[1]; cellColor.b = (R)cc[2];
            }
        } else {
            V3<R> vertPos = v3<R>(0, 0, 0), vertPosWithNormal = v3<R>(0, 0, 0);
            if (skinned) {  // light.go:613-620
                if (mode == T3D_LV_PER_VERTEX_WITH_NORMAL) vertPosWithNormal = add(add(vertPos, hmul(vnrm, cellSize)), bias);
                else vertPos = add(vpos, bias);
            } else if (mode == T3D_LV_PER_VERTEX_WITH_NORMAL) {
                vertPosWithNormal = add(mult_vec(transform, add(vpos, hmul(vnrm, cellSize))), bias);
            } else {
                vertPos = add(mult_vec(transform, vpos), bias);
            }
            // Dimensions.Contains (mesh.go:82-84)
            if (!(vertPos.x >= (R)d->vol_min[0] && vertPos.y >= (R)d->vol_min[1] && vertPos.z >= (R)d->vol_min[2] &&
                  vertPos.x <= (R)d->vol_max[0] && vertPos.y <= (R)d->vol_max[1] && vertPos.z <= (R)d->vol_max[2]))
                return;
            cellColor.r = 0; cellColor.g = 0; cellColor.b = 0;
            if (lv_cell(d, mode == T3D_LV_PER_VERTEX_WITH_NORMAL ? vertPosWithNormal : vertPos, idx)) {
                const float* cc = F.sc->volume_cells + 4 * (size_t)(d->cell_first + idx);
                cellColor.r = (R)cc[0]; cellColor.g = (R)cc[1]; cellColor.b = (R)cc[2]; cellColor.a = (R)cc[3];
                if (F.sc->cell_use_offsets && ml.nested) {  // cell.useLights (light.go:652-654)
                    const size_t c = (size_t)d->cell_first + (size_t)idx;
                    for (uint32_t u = F.sc->cell_use_offsets[c]; u < F.sc->cell_use_offsets[c + 1]; u++)
                        vertex_light<R>(F, (*ml.nested)[F.sc->cell_use_items[u]], part, skinned, transform, dir_rot, vpos,
                                        vnrm, tgt);
                }
            }
        }
        tgt.r += L.color.x * cellColor.r * L.energy;
        tgt.g += L.color.y * cellColor.g * L.energy;
        tgt.b += L.color.z * cellColor.b * L.energy;
        break;
    }
    default:
        break;
    }
}

// Mesh.VertexPositionWithShapeKeys / VertexNormalWithShapeKeys (mesh.go:796-822)
// and, for a skinned model, Model.skinVertex (model.go:559-594).
template <typename R>
void altered_vertex(const t3d_scene_desc* sc, const t3d_model_desc& md, const t3d_mesh_desc& me, uint32_t v,
                    V3<R>& pos, V3<R>& nrm) {
    pos = v3<R>((R)me.positions[3 * v], (R)me.positions[3 * v + 1], (R)me.positions[3 * v + 2]);
    nrm = v3<R>((R)me.normals[3 * v], (R)me.normals[3 * v + 1], (R)me.normals[3 * v + 2]);
    for (uint32_t key = 0; key < me.num_shape_keys; key++) {
        const R w = (R)me.shape_weights[key];
        const size_t e = 3 * ((size_t)key * me.num_vertices + v);
        pos.x += (R)me.shape_positions[e] * w;
        pos.y += (R)me.shape_positions[e + 1] * w;
        pos.z += (R)me.shape_positions[e + 2] * w;
        nrm.x += (R)me.shape_normals[e] * w;
        nrm.y += (R)me.shape_normals[e + 1] * w;
        nrm.z += (R)me.shape_normals[e + 2] * w;
    }
    if (!md.skinned) return;
    M4<R> skin;
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++) skin.m[r][c] = 0;  // Matrix4.Clear
    for (int i = 0; i < 4; i++) {
        const R w = (R)me.weights[4 * (size_t)v + i];
        if (w == 0) continue;
        const float* bone = sc->bones + 16 * ((size_t)md.bone_first + me.joints[4 * (size_t)v + i]);
        if (w == 1) {
            skin = load_m<R>(bone);
            break;
        }
        for (int q = 0; q < 16; q++) skin.m[q / 4][q % 4] = skin.m[q / 4][q % 4] + (R)bone[q] * w;  // Add(Scale(w))
    }
    pos = mult_vec(skin, pos);
    skin.m[3][0] = 0; skin.m[3][1] = 0; skin.m[3][2] = 0; skin.m[3][3] = 1;
    nrm = mult_vec(skin, nrm);
}

// The render closure (camera.go:1507-1827) with Model.ProcessVertices
// (model.go:600-995) and the bucket sort (sortingTriangles.go:38-125) for one
// render pair. Writes up to part.tri_count triangles from `slot`.
template <typename R, typename OutT>
uint32_t render_pair(const Frame<R>& F, Scratch<R>& S, const Pair& rp, uint32_t slot, t3d_oracle_out* out) {
    const t3d_scene_desc* sc = F.sc;
    const t3d_model_desc& md = sc->models[rp.model];
    const t3d_mesh_desc& me = *F.mesh[md.mesh];
    const SubMesh* subm = F.sub[md.mesh].get();
    const t3d_part_desc& part = me.parts[rp.part];
    const t3d_material& mat = part.mat;
    const Camera<R>& cam = F.cam;
    const t3d_camera_desc* cd = cam.d;

    // ---- Model.ProcessVertices ----
    S.unset.clear();
    for (auto& b : S.bins) b.clear();
    if ((md.color[3] == 0 && is_transparent(md, part)) || !md.visible) return 0;  // model.go:604-606

    const M4<R>& modelTransform = F.models[rp.model].transform;
    V3<R> camPos = cam.pos;
    V3<R> p, s; M4<R> r;
    decompose(inverted(modelTransform), p, s, r);  // model.go:629
    V3<R> invertedCamPos = add(mult_vec(r, camPos), hmul(p, v3<R>((R)1 / s.x, (R)1 / s.y, (R)1 / s.z)));  // :630
    const bool skinned = md.skinned != 0;
    // skinned vertices are in world space: VP alone (model.go:760-770)
    const bool billboard = mat.present && mat.billboard && !skinned;
    const bool unbillboarded = billboard && mat.billboard_depth == T3D_DEPTH_UNBILLBOARDED;
    M4<R> base = billboard ? billboard_base(modelTransform, cam, mat) : modelTransform;
    M4<R> mvp = skinned ? cam.vp : mult(base, cam.vp);  // model.go:695
    M4<R> unalteredMVP = mult(modelTransform, cam.vp);   // model.go:700-703

    R minDepth = maxf<R>();   // model.go:710-711
    R maxDepth = -maxf<R>();
    R camNear = cam.near_, camFar = cam.far_;

    if (S.clip.size() < me.num_vertices) {
        S.clip.resize(me.num_vertices);
        S.apos.resize(me.num_vertices);
        S.anrm.resize(me.num_vertices);
        S.udepth.resize(me.num_vertices);
    }
    uint32_t t_end = part.tri_start + part.tri_count;
    for (uint32_t t = part.tri_start; t < t_end; t++) {  // model.go:751-979
        // auto-subdivision: only the triangles of the level handleSubdivision picked (model.go:753-755)
        if (subm && !subdiv_active<R>(sc, *subm, t, invertedCamPos)) continue;
        uint32_t vidx[3] = {me.indices[3 * t], me.indices[3 * t + 1], me.indices[3 * t + 2]};
        for (int vi = 0; vi < 3; vi++) {
            uint32_t v = vidx[vi];
            altered_vertex<R>(sc, md, me, v, S.apos[v], S.anrm[v]);
            S.clip[v] = mult_vec_w(mvp, S.apos[v]);  // model.go:808-811
            if (cd->vertex_snapping > 0) {  // model.go:813-818
                const R snap = (R)cd->vertex_snapping;
                S.clip[v].x = m_round<R>(S.clip[v].x * snap) / snap;
                S.clip[v].y = m_round<R>(S.clip[v].y * snap) / snap;
                S.clip[v].z = m_round<R>(S.clip[v].z * snap) / snap;
            }
            if (unbillboarded) S.udepth[v] = mult_vec_w(unalteredMVP, S.apos[v]).z;  // model.go:800-801
        }
        bool outOfBounds = true;  // model.go:855-886
        V3<R> tv[3];
        for (int i = 0; i < 3; i++) {
            const V4<R>& c = S.clip[vidx[i]];
            R w = c.w;
            if (w < 0) w = k<R>(0.000001);
            tv[i].x = c.x / w;
            tv[i].y = c.y / w;
            if (c.z + (R)1 >= camNear && c.z < camFar) outOfBounds = false;
        }
        if (outOfBounds) continue;
        if ((tv[0].x < k<R>(-0.5) && tv[1].x < k<R>(-0.5) && tv[2].x < k<R>(-0.5)) ||  // model.go:890-898
            (tv[0].x > k<R>(0.5) && tv[1].x > k<R>(0.5) && tv[2].x > k<R>(0.5)) ||
            (tv[0].y < k<R>(-0.5) && tv[1].y < k<R>(-0.5) && tv[2].y < k<R>(-0.5)) ||
            (tv[0].y > k<R>(0.5) && tv[1].y > k<R>(0.5) && tv[2].y > k<R>(0.5)))
            continue;
        if (mat.present && mat.backface_culling) {  // model.go:902-925
            R n0x = tv[0].x - tv[1].x, n0y = tv[0].y - tv[1].y;
            R n1x = tv[1].x - tv[2].x, n1y = tv[1].y - tv[2].y;
            R nor = (n0x * n1y) - (n1x * n0y);
            if (nor < 0) continue;
        }
        // tri.Center (mesh.go:1980-1982)
        const float* pa = me.positions + 3 * (size_t)vidx[0];
        const float* pb = me.positions + 3 * (size_t)vidx[1];
        const float* pc = me.positions + 3 * (size_t)vidx[2];
        V3<R> center = v3<R>(((R)pa[0] + (R)pb[0] + (R)pc[0]) / (R)3, ((R)pa[1] + (R)pb[1] + (R)pc[1]) / (R)3,
                             ((R)pa[2] + (R)pb[2] + (R)pc[2]) / (R)3);
        if (subm)  // subdivided triangles' centres come from the subdivision (mesh.go:1821-1845)
            center = v3<R>((R)subm->ctr[3 * (size_t)t], (R)subm->ctr[3 * (size_t)t + 1], (R)subm->ctr[3 * (size_t)t + 2]);
        V3<R> from = invertedCamPos;
        if (skinned) {  // the skinned centre from the world camera (model.go:840-863, :941-946)
            const V3<R>& a = S.apos[vidx[0]];
            const V3<R>& b = S.apos[vidx[1]];
            const V3<R>& c = S.apos[vidx[2]];
            center = v3<R>((((R)0 + a.x) + b.x + c.x) / (R)3, (((R)0 + a.y) + b.y + c.y) / (R)3,
                           (((R)0 + a.z) + b.z + c.z) / (R)3);
            from = camPos;
        }
        R dx = from.x - center.x, dy = from.y - center.y, dz = from.z - center.z;
        R depth = dx * dx + dy * dy + dz * dz;  // model.go:950-953
        if (std::isnan(depth) || std::isinf(depth)) continue;
        if (depth < minDepth) minDepth = depth;
        if (depth > maxDepth) maxDepth = depth;
        S.unset.push_back({t, depth});  // AddTriangle
    }
    if (S.unset.empty()) return 0;  // camera.go:1555-1557

    // ---- sortingTriangleBucket.Sort (sortingTriangles.go:38-64) ----
    int sortMode = mat.present ? mat.sort_mode : T3D_SORT_BACK_TO_FRONT;  // camera.go:1540-1543
    const int binCount = 512;
    R minRange = minDepth, maxRange = maxDepth;
    R rangeDiff = maxRange - minRange;
    if (rangeDiff == 0) { maxRange += k<R>(0.001); rangeDiff += k<R>(0.001); }
    for (auto& e : S.unset) {
        int targetBin = 0;
        if (sortMode != T3D_SORT_NONE) {
            R depth = (e.second - minRange) / rangeDiff * (R)binCount;
            R t = m_clamp<R>(depth, 0, (R)(binCount - 1));
            targetBin = (int)t;
        }
        S.bins[targetBin].push_back(e);
    }
    std::vector<uint32_t> order;
    order.reserve(S.unset.size());
    if (sortMode == T3D_SORT_BACK_TO_FRONT) {  // ForEach, sortingTriangles.go:93-125
        for (int b = binCount - 1; b >= 0; b--) for (auto& e : S.bins[b]) order.push_back(e.first);
    } else {
        for (int b = 0; b < binCount; b++) for (auto& e : S.bins[b]) order.push_back(e.first);
    }

    // ---- lighting (camera.go:1521-1528, :1576-1644) ----
    bool lighting = cd->lighting_on && !(mat.present && mat.shadeless) && !md.shadeless;
    std::vector<ModelLight<R>> mlights;
    std::vector<ModelLight<R>> nested_ml;  // beginModel of the lights light-volume cells use
    M4<R> dir_rot = identity<R>();
    if (lighting) {
        uint32_t list = md.light_list < 0 ? 0u : (uint32_t)md.light_list;
        if (list < sc->num_lists) {
            V3<R> ip, is; M4<R> ir;
            decompose(inverted(modelTransform), ip, is, ir);  // light.go:177
            dir_rot = transposed(inverted(F.models[rp.model].world_rot));  // light.go:328
            Dims dm = F.dims[md.mesh];
            R maxSpan = magnitude(v3<R>((R)dm.mx[0] - (R)dm.mn[0], (R)dm.mx[1] - (R)dm.mn[1], (R)dm.mx[2] - (R)dm.mn[2]));
            V3<R> modelPos = row3(modelTransform, 3);
            std::vector<uint32_t> items;
            if (list == 0) items = F.scene_lights;
            else for (uint32_t q = sc->list_offsets[list]; q < sc->list_offsets[list + 1]; q++) items.push_back(sc->list_items[q]);
            if (sc->cell_use_offsets) {
                nested_ml.resize(F.lights.size());
                for (uint32_t li = 0; li < F.lights.size(); li++) {
                    ModelLight<R>& nm = nested_ml[li];
                    nm.l = &F.lights[li];
                    nm.skip = false;
                    nm.working = v3<R>(0, 0, 0);
                    if (nm.l->type == T3D_LIGHT_POINT)
                        nm.working = skinned ? nm.l->wpos
                                             : add(mult_vec(ir, nm.l->wpos), hmul(ip, v3<R>((R)1 / is.x, (R)1 / is.y, (R)1 / is.z)));
                }
            }
            for (uint32_t li : items) {
                if (li >= F.lights.size() || !light_enabled(F.mask, li)) continue;
                ModelLight<R> ml;
                ml.nested = nested_ml.empty() ? nullptr : &nested_ml;
                ml.l = &F.lights[li];
                ml.working = v3<R>(0, 0, 0);
                ml.skip = false;
                if (ml.l->type == T3D_LIGHT_POINT) {
                    if (skinned) ml.working = ml.l->wpos;  // light.go:183-184
                    else ml.working = add(mult_vec(ir, ml.l->wpos), hmul(ip, v3<R>((R)1 / is.x, (R)1 / is.y, (R)1 / is.z)));  // light.go:186
                    if (ml.l->range > 0) {
                        R dist = maxSpan + ml.l->range;
                        if (dist2(modelPos, ml.l->wpos) > dist * dist) ml.skip = true;
                    }
                }
                mlights.push_back(ml);
            }
        }
    }
    if (lighting) {
        if (S.vlight.size() < me.num_vertices) S.vlight.resize(me.num_vertices);
        for (uint32_t t : order) {  // camera.go:1613-1641
            uint32_t vidx[3] = {me.indices[3 * t], me.indices[3 * t + 1], me.indices[3 * t + 2]};
            for (int i = 0; i < 3; i++) S.vlight[vidx[i]] = C4<R>{0, 0, 0, 1};
            for (auto& ml : mlights) {
                if (ml.skip) continue;
                for (int i = 0; i < 3; i++)
                    vertex_light<R>(F, ml, part, skinned, modelTransform, dir_rot, S.apos[vidx[i]], S.anrm[vidx[i]],
                                    S.vlight[vidx[i]]);
            }
        }
    }

    // ---- emit (camera.go:1646-1820) ----
    C4<R> mp{(R)md.color[0], (R)md.color[1], (R)md.color[2], (R)md.color[3]};
    if (mat.present) { mp.r *= (R)mat.color[0]; mp.g *= (R)mat.color[1]; mp.b *= (R)mat.color[2]; mp.a *= (R)mat.color[3]; }
    R srcW = mat.present ? (R)mat.tex_w : (R)0, srcH = mat.present ? (R)mat.tex_h : (R)0;
    OutT* oxyuv = (OutT*)out->xyuv;
    OutT* orgba = (OutT*)out->rgba;
    OutT* odepth = (OutT*)out->depth;
    OutT* ocustom = cd->perspective_corrected ? (OutT*)out->custom0 : nullptr;
    uint32_t n = 0;
    for (uint32_t t : order) {
        size_t s_ = (size_t)slot + n;
        out->tri_index[s_] = t;
        for (int vi = 0; vi < 3; vi++) {
            uint32_t v = me.indices[3 * t + vi];
            const V4<R>& c = S.clip[v];
            R w = c.w;
            if (!cd->perspective) w = (R)1;
            if (w < 0) w = k<R>(0.001);
            R dx = (c.x / w) * cam.W + cam.halfW;
            R dy = (c.y / -w) * cam.H + cam.halfH;
            R U = (R)me.uvs[2 * v], V = (R)me.uvs[2 * v + 1];
            R uvU, uvV;
            if (cd->perspective_corrected) { uvU = (U / w) * srcW; uvV = (((R)1 - V) / w) * srcH; }
            else { uvU = U * srcW; uvV = ((R)1 - V) * srcH; }
            C4<R> col;
            if (me.colors) {
                const float* vc = me.colors + 4 * (size_t)v;
                col = C4<R>{(R)vc[0] * mp.r, (R)vc[1] * mp.g, (R)vc[2] * mp.b, (R)vc[3] * mp.a};
            } else {
                col = mp;
            }
            if (lighting) { col.r *= S.vlight[v].r; col.g *= S.vlight[v].g; col.b *= S.vlight[v].b; }
            R depthOut = 0;
            if (cd->render_depth || cd->fog_on) {
                // camera.go:1760-1765 (RenderDepth) and :1785 (fog)
                R vz = (cd->render_depth && unbillboarded) ? S.udepth[v] : c.z;
                R depth = (vz + cam.margin) / cam.spread;
                if (depth < 0) depth = 0;
                else if (depth > 1) depth = 1;
                depthOut = depth;
                if (!cd->render_depth) {  // fog branch, camera.go:1783-1812
                    R f0 = (R)cd->fog_range[0], f1 = (R)cd->fog_range[1];
                    R fd = f0 + ((f1 - f0) * (R)1 - depth);
                    if (cd->fog_mode == T3D_FOG_ADD) {
                        col.r += (R)cd->fog_color[0] * fd; col.g += (R)cd->fog_color[1] * fd; col.b += (R)cd->fog_color[2] * fd;
                    } else if (cd->fog_mode == T3D_FOG_SUB) {
                        col.r *= (R)cd->fog_color[0] * fd; col.g *= (R)cd->fog_color[1] * fd; col.b *= (R)cd->fog_color[2] * fd;
                    }
                }
            }
            size_t ci = s_ * 3 + vi;
            oxyuv[4 * ci] = (OutT)dx; oxyuv[4 * ci + 1] = (OutT)dy; oxyuv[4 * ci + 2] = (OutT)uvU; oxyuv[4 * ci + 3] = (OutT)uvV;
            orgba[4 * ci] = (OutT)col.r; orgba[4 * ci + 1] = (OutT)col.g; orgba[4 * ci + 2] = (OutT)col.b; orgba[4 * ci + 3] = (OutT)col.a;
            odepth[ci] = (OutT)depthOut;
            if (ocustom) ocustom[ci] = (OutT)((R)1 / w);  // Custom0 (camera.go:1700-1704)
        }
        n++;
    }
    return n;
}

template <typename R, typename OutT>
int render(const t3d_scene_desc* sc, const t3d_camera_desc* cd, const uint64_t* mask, uint32_t animate_frames,
           uint32_t threads, t3d_oracle_out* out) {
    if (!sc || !cd || !out) return T3D_E_INVAL;
    Frame<R> F;
    F.sc = sc;
    F.mask = mask;
    const uint32_t nlev = sc->subdivision_levels ? sc->num_subdivision_levels : 0u;
    F.sub.resize(sc->num_meshes);
    F.mesh.resize(sc->num_meshes);
    for (uint32_t m = 0; m < sc->num_meshes; m++) {
        F.mesh[m] = &sc->meshes[m];
        if (sc->meshes[m].auto_subdivide && nlev) {
            F.sub[m] = std::make_unique<SubMesh>();
            build_submesh(sc->meshes[m], sc->subdivision_levels, nlev,
                          sc->max_subdivisions ? (int)sc->max_subdivisions : 3, *F.sub[m]);
            F.mesh[m] = &F.sub[m]->desc;
        }
    }
    // the scene light list after the mask, then Camera.MaxLightCount (camera.go:1474-1497)
    if (sc->num_lists > 0)
        for (uint32_t q = sc->list_offsets[0]; q < sc->list_offsets[1]; q++)
            if (sc->list_items[q] < sc->num_lights && light_enabled(mask, sc->list_items[q]))
                F.scene_lights.push_back(sc->list_items[q]);
    if (cd->max_light_count > 0) {
        const float fx = cd->focus_set ? cd->focus[0] : cd->transform[12];
        const float fy = cd->focus_set ? cd->focus[1] : cd->transform[13];
        const float fz = cd->focus_set ? cd->focus[2] : cd->transform[14];
        auto dist2_to = [&](uint32_t li) {  // Vector3.DistanceSquaredTo, vector.go:242-247
            const float* t = sc->lights[li].transform;
            float x = fx - t[12], y = fy - t[13], z = fz - t[14];
            return x * x + y * y + z * z;
        };
        GoSort gs{F.scene_lights, [&](uint32_t i, uint32_t j) {
                      const int a = sc->lights[i].type, b = sc->lights[j].type;
                      if (a == T3D_LIGHT_AMBIENT) return true;
                      if (b == T3D_LIGHT_AMBIENT) return false;
                      if (a == T3D_LIGHT_DIRECTIONAL) return true;
                      if (b == T3D_LIGHT_DIRECTIONAL) return false;
                      return dist2_to(i) < dist2_to(j);
                  }};
        gs.run();
        if (F.scene_lights.size() > (size_t)cd->max_light_count) F.scene_lights.resize((size_t)cd->max_light_count);
    }
    setup_camera(F.cam, cd);

    // models: Node.Transform (node.go:572-608) with optional animation steps
    F.models.resize(sc->num_models);
    for (uint32_t i = 0; i < sc->num_models; i++) {
        const t3d_model_desc& md = sc->models[i];
        if (md.mesh >= sc->num_meshes) return T3D_E_INVAL;
        if (md.use_trs) {
            M4<R> rot = load_m<R>(md.rotation);
            M4<R> step = load_m<R>(md.rotate_step);
            for (uint32_t f = 0; f < animate_frames; f++) rot = mult(step, rot);  // Matrix4.Rotated, matrix.go:583-585
            M4<R> tr = scale_m<R>((R)md.scale[0], (R)md.scale[1], (R)md.scale[2]);
            tr = mult(tr, rot);
            tr = mult(tr, translate<R>((R)md.position[0], (R)md.position[1], (R)md.position[2]));
            F.models[i].transform = tr;
            F.models[i].world_rot = rot;
        } else {
            F.models[i].transform = load_m<R>(md.transform);
            F.models[i].world_rot = load_m<R>(md.world_rotation);
        }
    }
    F.dims.resize(sc->num_meshes);
    for (uint32_t m = 0; m < sc->num_meshes; m++) F.dims[m] = mesh_dims(sc->meshes[m]);

    // lights: beginRender (light.go:110-113, :318-320)
    F.lights.resize(sc->num_lights);
    for (uint32_t i = 0; i < sc->num_lights; i++) {
        const t3d_light_desc& d = sc->lights[i];
        LightPrep<R>& L = F.lights[i];
        L.d = &d;
        L.type = d.type;
        L.color = v3<R>((R)d.color[0], (R)d.color[1], (R)d.color[2]);
        L.energy = (R)d.energy;
        L.range = (R)d.range;
        L.range2 = L.range * L.range;  // PointLight.SetRange, light.go:270-273
        M4<R> lt = load_m<R>(d.transform);
        L.wpos = row3(lt, 3);
        L.amb = v3<R>(L.color.x * L.energy, L.color.y * L.energy, L.color.z * L.energy);
        L.fwd = forward(load_m<R>(d.world_rotation));
    }

    // Render pairs (camera.go:1343-1457, :2050-2109). Frustum-culled models
    // never become pairs in the reference; their removal does not change the
    // relative draw order of the others (the sorts are stable), so the segment
    // table keeps them, with zero triangles, to line up with the device layout.
    std::vector<char> is_culled(sc->num_models, 0);
    uint32_t culled = 0;
    std::vector<Pair> solids, transparents;
    // Model.DynamicBatchModels: owner -> (owner part -> members in model order)
    std::vector<std::vector<std::pair<uint32_t, std::vector<uint32_t>>>> batch_of(sc->num_models);
    for (uint32_t i = 0; i < sc->num_models; i++) {
        const t3d_model_desc& md = sc->models[i];
        if (!md.batched) continue;
        auto& parts = batch_of[md.batch_owner];
        auto it = std::find_if(parts.begin(), parts.end(), [&](const auto& e) { return e.first == md.batch_part; });
        if (it == parts.end()) {
            parts.push_back({md.batch_part, {}});
            it = parts.end() - 1;
        }
        it->second.push_back(i);
    }
    for (auto& parts : batch_of)  // the owner's batch parts in ascending part order
        std::sort(parts.begin(), parts.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
    for (uint32_t i = 0; i < sc->num_models; i++) {
        const t3d_model_desc& md = sc->models[i];
        if (!md.visible) continue;
        // frustum culling of a batch member happens when its batch draws (camera.go:2083-2088)
        if (md.frustum_culling && !model_in_frustum(F.cam, F.models[i].transform, F.dims[md.mesh], md.skinned != 0)) {
            is_culled[i] = 1;
            culled++;
        }
        if (md.batched) continue;  // camera.go:1346
        const t3d_mesh_desc& me = *F.mesh[md.mesh];
        V3<R> mpos = row3(F.models[i].transform, 3);
        if (!batch_of[i].empty()) {  // a dynamic batcher: one pair per batch part (camera.go:1397-1451)
            bool transparent = false;
            for (const auto& bp : batch_of[i]) {
                const t3d_material& bm = me.parts[bp.first].mat;
                if (bm.present && !bm.visible) continue;
                for (uint32_t c : bp.second) {
                    const t3d_model_desc& cm = sc->models[c];
                    if (!cm.visible || transparent) continue;
                    const t3d_mesh_desc& cme = *F.mesh[cm.mesh];
                    for (uint32_t q = 0; q < cme.num_parts && !transparent; q++)
                        if (!(cme.parts[q].mat.present && !cme.parts[q].mat.visible) && is_transparent(cm, cme.parts[q]))
                            transparent = true;
                }
                Pair rp{i, bp.first, 0.0f, bm.present ? bm.render_order : 0, true};
                if (transparent || !cd->render_depth) rp.depth = (float)dist2(F.cam.pos, mpos);
                if (transparent) transparents.push_back(rp);
                else solids.push_back(rp);
            }
            continue;
        }
        for (uint32_t p = 0; p < me.num_parts; p++) {
            const t3d_part_desc& part = me.parts[p];
            if (part.mat.present && !part.mat.visible) continue;  // MeshPart.isVisible, mesh.go:2402-2407
            Pair rp{i, p, (float)dist2(F.cam.pos, mpos), part.mat.present ? part.mat.render_order : 0};
            if (is_transparent(md, part)) transparents.push_back(rp);
            else solids.push_back(rp);
        }
    }
    auto stable_by = [](std::vector<Pair>& v, auto less) {
        // bottom-up stable merge sort (any stable sort orders a strict weak ordering identically)
        std::vector<Pair> tmp(v.size());
        for (size_t width = 1; width < v.size(); width *= 2) {
            for (size_t lo = 0; lo < v.size(); lo += 2 * width) {
                size_t mid = std::min(lo + width, v.size()), hi = std::min(lo + 2 * width, v.size());
                size_t a = lo, b = mid, o = lo;
                while (a < mid && b < hi) tmp[o++] = less(v[b], v[a]) ? v[b++] : v[a++];
                while (a < mid) tmp[o++] = v[a++];
                while (b < hi) tmp[o++] = v[b++];
            }
            v.swap(tmp);
        }
    };
    auto by_order_then_far = [](const Pair& a, const Pair& b) {
        return a.order != b.order ? a.order < b.order : a.depth > b.depth;
    };
    if (!cd->render_depth) stable_by(solids, by_order_then_far);  // camera.go:1461-1470
    stable_by(transparents, by_order_then_far);                   // camera.go:2050-2055
    std::vector<Pair> ordered(solids);
    ordered.insert(ordered.end(), transparents.begin(), transparents.end());
    // every pair is one flush; a batch draws its visible members far to near from the
    // camera (camera.go:2072-2093; equal distances keep model order), all their parts
    std::vector<Pair> segs;
    for (size_t q = 0; q < ordered.size(); q++) {
        Pair rp = ordered[q];
        rp.draw = (uint32_t)q;
        rp.draw_transparent = q >= solids.size() ? 1u : 0u;
        if (!rp.batch) {
            segs.push_back(rp);
            continue;
        }
        std::vector<std::pair<R, uint32_t>> members;
        for (const auto& bp : batch_of[rp.model])
            if (bp.first == rp.part)
                for (uint32_t c : bp.second)
                    if (sc->models[c].visible) members.push_back({dist2(F.cam.pos, row3(F.models[c].transform, 3)), c});
        std::stable_sort(members.begin(), members.end(),
                         [](const std::pair<R, uint32_t>& a, const std::pair<R, uint32_t>& b) { return a.first > b.first; });
        for (const auto& mc : members)
            for (uint32_t p = 0; p < F.mesh[sc->models[mc.second].mesh]->num_parts; p++) {
                Pair m{mc.second, p, 0.0f, 0, false, rp.draw, rp.draw_transparent};
                segs.push_back(m);
            }
    }

    if (segs.size() > out->max_segments) return T3D_E_INVAL;
    uint64_t base = 0;
    for (size_t s = 0; s < segs.size(); s++) {
        const t3d_mesh_desc& me = *F.mesh[sc->models[segs[s].model].mesh];
        out->seg_model[s] = segs[s].model;
        if (out->seg_draw) out->seg_draw[s] = segs[s].draw;
        if (out->seg_draw_transparent) out->seg_draw_transparent[s] = segs[s].draw_transparent;
        out->seg_part[s] = segs[s].part;
        out->seg_base[s] = (uint32_t)base;
        out->seg_capacity[s] = me.parts[segs[s].part].tri_count;
        out->seg_count[s] = 0;
        base += me.parts[segs[s].part].tri_count;
    }
    out->num_segments = (uint32_t)segs.size();
    out->total_slots = base;
    out->culled_models = culled;
    if (base > out->max_tris) return T3D_E_INVAL;

    std::atomic<size_t> next{0};
    auto worker = [&]() {
        Scratch<R> S;
        for (;;) {
            size_t s = next.fetch_add(1);
            if (s >= segs.size()) break;
            if (is_culled[segs[s].model]) continue;
            out->seg_count[s] = render_pair<R, OutT>(F, S, segs[s], out->seg_base[s], out);
        }
    };
    if (threads <= 1) {
        worker();
    } else {
        std::vector<std::thread> pool;
        for (uint32_t t = 0; t < threads; t++) pool.emplace_back(worker);
        for (auto& th : pool) th.join();
    }
    uint64_t vis = 0;
    for (size_t s = 0; s < segs.size(); s++) vis += out->seg_count[s];
    out->visible_tris = vis;
    return T3D_OK;
}

}  // namespace

extern "C" {

int t3d_oracle_render_f32(const t3d_scene_desc* scene, const t3d_camera_desc* cam, const uint64_t* light_mask,
                          uint32_t animate_frames, uint32_t threads, t3d_oracle_out* out) {
    return render<float, float>(scene, cam, light_mask, animate_frames, threads, out);
}
int t3d_oracle_render_f64(const t3d_scene_desc* scene, const t3d_camera_desc* cam, const uint64_t* light_mask,
                          uint32_t animate_frames, uint32_t threads, t3d_oracle_out* out) {
    return render<double, double>(scene, cam, light_mask, animate_frames, threads, out);
}

void t3d_oracle_mat_mult(const float* a, const float* b, float* out) {
    M4<float> r = mult(load_m<float>(a), load_m<float>(b));
    for (int i = 0; i < 16; i++) out[i] = r.m[i / 4][i % 4];
}
void t3d_oracle_mat_inverted(const float* m, float* out) {
    M4<float> r = inverted(load_m<float>(m));
    for (int i = 0; i < 16; i++) out[i] = r.m[i / 4][i % 4];
}
// NewMatrix4Rotate (matrix.go:101-128); Sin/Cos through float64 (math32.go:137-150)
void t3d_oracle_mat_rotate(float x, float y, float z, float angle, float* out) {
    if (x == 0 && y == 0 && z == 0) y = 1;
    M4<float> mat = identity<float>();
    V3<float> v = unit(v3<float>(x, y, z));
    float s = (float)std::sin((double)angle);
    float c = (float)std::cos((double)angle);
    float m = 1 - c;
    mat.m[0][0] = m * v.x * v.x + c;
    mat.m[0][1] = m * v.x * v.y + v.z * s;
    mat.m[0][2] = m * v.z * v.x - v.y * s;
    mat.m[1][0] = m * v.x * v.y - v.z * s;
    mat.m[1][1] = m * v.y * v.y + c;
    mat.m[1][2] = m * v.y * v.z + v.x * s;
    mat.m[2][0] = m * v.z * v.x + v.y * s;
    mat.m[2][1] = m * v.y * v.z - v.x * s;
    mat.m[2][2] = m * v.z * v.z + c;
    for (int i = 0; i < 16; i++) out[i] = mat.m[i / 4][i % 4];
}
void t3d_oracle_mat_decompose(const float* m, float* pos3, float* scale3, float* rot16) {
    V3<float> p, s; M4<float> r;
    decompose(load_m<float>(m), p, s, r);
    pos3[0] = p.x; pos3[1] = p.y; pos3[2] = p.z;
    scale3[0] = s.x; scale3[1] = s.y; scale3[2] = s.z;
    for (int i = 0; i < 16; i++) rot16[i] = r.m[i / 4][i % 4];
}
// Quaternion.ToMatrix4 (quaternion.go:135-182)
void t3d_oracle_quat_to_mat(float x, float y, float z, float w, float* out) {
    M4<float> m1 = identity<float>(), m2 = identity<float>();
    m1.m[0][0] = w;  m1.m[0][1] = z;  m1.m[0][2] = -y; m1.m[0][3] = x;
    m1.m[1][0] = -z; m1.m[1][1] = w;  m1.m[1][2] = x;  m1.m[1][3] = y;
    m1.m[2][0] = y;  m1.m[2][1] = -x; m1.m[2][2] = w;  m1.m[2][3] = z;
    m1.m[3][0] = -x; m1.m[3][1] = -y; m1.m[3][2] = -z; m1.m[3][3] = w;
    m2.m[0][0] = w;  m2.m[0][1] = z;  m2.m[0][2] = -y; m2.m[0][3] = -x;
    m2.m[1][0] = -z; m2.m[1][1] = w;  m2.m[1][2] = x;  m2.m[1][3] = -y;
    m2.m[2][0] = y;  m2.m[2][1] = -x; m2.m[2][2] = w;  m2.m[2][3] = -z;
    m2.m[3][0] = x;  m2.m[3][1] = y;  m2.m[3][2] = z;  m2.m[3][3] = w;
    M4<float> r = mult(m1, m2);
    for (int i = 0; i < 16; i++) out[i] = r.m[i / 4][i % 4];
}
void t3d_oracle_vec_unit(const float* v, float* o) {
    V3<float> r = unit(v3<float>(v[0], v[1], v[2]));
    o[0] = r.x; o[1] = r.y; o[2] = r.z;
}

}  // extern "C"
