// t3d_runtime.cu -- host side of the C ABI declared in include/t3d.h.
//
// Owns resident scenes in HBM, builds the per-frame job / instance / segment /
// work-item tables (the part of Camera.Render that decides what to draw and in
// which order, camera.go:1269-1503 and :2050-2109), launches the persistent
// frame kernel (one launch for all models, or one launch per render pair) and
// reads back the per-segment visible counts.

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "t3d_device.cuh"
#include "t3d_runtime.h"

extern "C" const void* t3d_frame_kernel_ptr();
extern "C" const void* t3d_frame_kernel_mesh_ptr();
extern "C" const void* t3d_phase_kernel_ptr(int mesh, int k);
extern "C" cudaError_t t3d_fill_keyed(cudaStream_t st, unsigned char* pool, const void* fills, uint32_t nfills,
                                      const uint32_t* vmap, const float4* va, const float4* vb, uint32_t colors);
extern "C" cudaError_t t3d_bake_shapes(cudaStream_t st, const float4* va, const float4* vb, const float4* sa,
                                       const float2* sb, const float* sw, uint32_t nverts, uint32_t nkeys, float4* oa,
                                       float4* ob);
extern "C" size_t t3d_frame_smem_bytes(uint32_t tile_tris, uint32_t block_threads);

namespace t3d {

// ------------------------------------------------------------ utilities ----
// A kernel's dynamic shared-memory limit is one process-wide attribute shared by
// every context and the allocation-free entry: it is only ever raised, so a
// launch configured for more shared memory never fails after another caller
// configured less.
cudaError_t raise_smem_limit(const void* fn, size_t bytes) {
    static std::mutex mu;
    std::lock_guard<std::mutex> g(mu);
    cudaFuncAttributes fa;
    cudaError_t e = cudaFuncGetAttributes(&fa, fn);
    if (e != cudaSuccess) return e;
    if ((size_t)fa.maxDynamicSharedSizeBytes >= bytes) return cudaSuccess;
    return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

void set_err(t3d_ctx* c, const char* fmt, ...) {
    if (!c) return;
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    c->err = buf;
}

#define CK(call)                                                                        \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess) {                                                        \
            set_err(ctx, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
            return e_ == cudaErrorMemoryAllocation ? T3D_E_OOM : T3D_E_CUDA;            \
        }                                                                               \
    } while (0)

int DevBuf::ensure(t3d_ctx* ctx, size_t bytes) {
    if (bytes <= cap) return T3D_OK;
    release();
    size_t want = std::max(bytes, (size_t)256);
    want = want + want / 4;
    cudaError_t e = ctx->pool ? cudaMallocFromPoolAsync(&ptr, want, ctx->pool, ctx->stream) : cudaMalloc(&ptr, want);
    if (e != cudaSuccess) {
        ptr = nullptr;
        set_err(ctx, "device allocation of %zu bytes failed: %s", want, cudaGetErrorString(e));
        return T3D_E_OOM;
    }
    pooled = ctx->pool ? ctx->stream : nullptr;
    cap = want;
    return T3D_OK;
}
void DevBuf::release() {
    if (ptr) {
        if (pooled) cudaFreeAsync(ptr, pooled);  // after the work already queued on the stream
        else cudaFree(ptr);
    }
    ptr = nullptr;
    cap = 0;
    pooled = nullptr;
}

int HostBuf::ensure(size_t bytes) {
    if (bytes <= cap) return T3D_OK;
    if (ptr) cudaFreeHost(ptr);
    ptr = nullptr;
    cap = 0;
    size_t want = std::max(bytes, (size_t)256);
    want = want + want / 4;
    if (cudaMallocHost(&ptr, want) != cudaSuccess) {
        ptr = nullptr;
        return T3D_E_OOM;
    }
    cap = want;
    return T3D_OK;
}
void HostBuf::release() {
    if (ptr) cudaFreeHost(ptr);
    ptr = nullptr;
    cap = 0;
}

static bool light_enabled(const uint64_t* mask, uint32_t i) {
    if (i >= 128) return false;
    return (mask[i >> 6] >> (i & 63)) & 1ull;
}

// Model.isTransparent (model.go:1274-1282)
// Go's sort.SliceStable (sort/zsortfunc.go: insertion sort of 20-element blocks, then
// SymMerge passes, Kim & Kutzner), restated because Camera.Render sorts the scene lights
// with a comparator that is not a strict weak order (two ambient or two directional
// lights are each "less" than the other): the order it produces is the algorithm's.
namespace gosort {
template <typename Less> void insertion(std::vector<uint32_t>& d, int a, int b, Less less) {
    for (int i = a + 1; i < b; i++)
        for (int j = i; j > a && less(d[j], d[j - 1]); j--) std::swap(d[j], d[j - 1]);
}
inline void swap_range(std::vector<uint32_t>& d, int a, int b, int n) {
    for (int i = 0; i < n; i++) std::swap(d[a + i], d[b + i]);
}
inline void rotate(std::vector<uint32_t>& d, int a, int m, int b) {
    int i = m - a, j = b - m;
    while (i != j) {
        if (i > j) {
            swap_range(d, m - i, m, j);
            i -= j;
        } else {
            swap_range(d, m - i, m + j - i, i);
            j -= i;
        }
    }
    swap_range(d, m - i, m, i);
}
template <typename Less> void sym_merge(std::vector<uint32_t>& d, int a, int m, int b, Less less) {
    if (m - a == 1) {
        int i = m, j = b;
        while (i < j) {
            const int h = (int)((unsigned)(i + j) >> 1);
            if (less(d[h], d[a])) i = h + 1;
            else j = h;
        }
        for (int k = a; k < i - 1; k++) std::swap(d[k], d[k + 1]);
        return;
    }
    if (b - m == 1) {
        int i = a, j = m;
        while (i < j) {
            const int h = (int)((unsigned)(i + j) >> 1);
            if (!less(d[m], d[h])) i = h + 1;
            else j = h;
        }
        for (int k = m; k > i; k--) std::swap(d[k], d[k - 1]);
        return;
    }
    const int mid = (int)((unsigned)(a + b) >> 1), n = mid + m;
    int start, r;
    if (m > mid) {
        start = n - b;
        r = mid;
    } else {
        start = a;
        r = m;
    }
    const int p = n - 1;
    while (start < r) {
        const int c = (int)((unsigned)(start + r) >> 1);
        if (!less(d[p - c], d[c])) start = c + 1;
        else r = c;
    }
    const int end = n - start;
    if (start < m && m < end) rotate(d, start, m, end);
    if (a < start && start < mid) sym_merge(d, a, start, mid, less);
    if (mid < end && end < b) sym_merge(d, mid, end, b, less);
}
template <typename Less> void stable(std::vector<uint32_t>& d, Less less) {
    const int n = (int)d.size();
    int block = 20, a = 0, b = block;
    while (b <= n) {
        insertion(d, a, b, less);
        a = b;
        b += block;
    }
    insertion(d, a, n, less);
    while (block < n) {
        a = 0;
        b = 2 * block;
        while (b <= n) {
            sym_merge(d, a, a + block, b, less);
            a = b;
            b += 2 * block;
        }
        if (a + block < n) sym_merge(d, a, a + block, n, less);
        block *= 2;
    }
}
}  // namespace gosort

// Camera.MaxLightCount (camera.go:1474-1497) over the job's scene light list.
static std::vector<uint32_t> culled_scene_lights(const Scene* sc, const t3d_job_desc& job) {
    std::vector<uint32_t> l;
    for (uint32_t li : sc->lists[0])
        if (light_enabled(job.light_mask, li)) l.push_back(li);
    const t3d_camera_desc& cd = job.camera;
    if (cd.max_light_count <= 0) return l;
    const float px = cd.focus_set ? cd.focus[0] : cd.transform[12];
    const float py = cd.focus_set ? cd.focus[1] : cd.transform[13];
    const float pz = cd.focus_set ? cd.focus[2] : cd.transform[14];
    auto d2 = [&](uint32_t li) {  // Vector3.DistanceSquaredTo (vector.go:242-247)
        const float* t = sc->lights[li].transform;
        const float x = px - t[12], y = py - t[13], z = pz - t[14];
        return x * x + y * y + z * z;
    };
    auto less = [&](uint32_t i, uint32_t j) {
        const int ti = sc->lights[i].type, tj = sc->lights[j].type;
        if (ti == T3D_LIGHT_AMBIENT) return true;
        if (tj == T3D_LIGHT_AMBIENT) return false;
        if (ti == T3D_LIGHT_DIRECTIONAL) return true;
        if (tj == T3D_LIGHT_DIRECTIONAL) return false;
        return d2(i) < d2(j);
    };
    gosort::stable(l, less);
    if (l.size() > (size_t)cd.max_light_count) l.resize((size_t)cd.max_light_count);
    return l;
}

static bool is_transparent(const float* model_color, const t3d_material& mat) {
    if (mat.present) {
        bool matT = mat.transparency_mode == T3D_TRANSPARENCY_TRANSPARENT || !mat.blend_source_over ||
                    (mat.transparency_mode == T3D_TRANSPARENCY_AUTO && mat.color[3] < 0.999f);
        bool modelT = mat.transparency_mode != T3D_TRANSPARENCY_OPAQUE && model_color[3] < 0.999f;
        return matT || modelT;
    }
    return model_color[3] < 0.999f;
}

// Camera.ViewMatrix, Projection, sphere factors, Clear basis and the depth
// margin (camera.go:638-679, :1085-1088, :1337-1341; matrix.go:588-616).
void build_camera(const t3d_camera_desc& d, JobCam& c) {
    memset(&c, 0, sizeof c);
    m4 ct = load16(d.transform), cr = load16(d.world_rotation);
    f3 pos = row3(ct, 3);
    m4 view = mult(translate(-pos.x, -pos.y, -pos.z), transposed(cr));
    float fov = d.fov_y, nr = d.near_plane, fr = d.far_plane;
    float W = (float)d.width, H = (float)d.height;
    float aspect = W / H;
    float angle = fov * 3.1415f / 360.0f;
    c.sphere_tang = (float)std::tan((double)angle);
    c.sphere_y = 1.0f / (float)std::cos((double)angle);
    c.sphere_x = 1.0f / (float)std::cos((double)(float)std::atan((double)(c.sphere_tang * aspect)));
    c.aspect = aspect;
    m4 proj = ident();
    if (d.perspective) {
        float t = (float)std::tan((double)(fov * (float)M_PI / 360.0f));
        float b = -t, r = t * aspect, l = -r;
        proj.m[0][0] = (2.0f * nr) / (r - l); proj.m[0][1] = 0; proj.m[0][2] = (r + l) / (r - l); proj.m[0][3] = 0;
        proj.m[1][0] = 0; proj.m[1][1] = (2.0f * nr) / (t - b); proj.m[1][2] = (t + b) / (t - b); proj.m[1][3] = 0;
        proj.m[2][0] = 0; proj.m[2][1] = 0; proj.m[2][2] = -((fr + nr) / (fr - nr)); proj.m[2][3] = -((2.0f * fr * nr) / (fr - nr));
        proj.m[3][0] = 0; proj.m[3][1] = 0; proj.m[3][2] = -1; proj.m[3][3] = 0;
    } else {
        float asr = H / W;
        float os = d.ortho_scale;
        float right = 1.0f * os, left = -1.0f * os, top = asr * os, bottom = -asr * os;
        proj.m[0][0] = 2.0f / (right - left);
        proj.m[1][1] = 2.0f / (top - bottom);
        proj.m[2][2] = -2.0f / (fr - nr);
        proj.m[3][3] = 1.0f;
    }
    store16(mult(view, proj), c.vp);
    f3 fw = unit3(row3(cr, 2)), rg = unit3(row3(cr, 0)), upv = unit3(row3(cr, 1));
    c.pos[0] = pos.x; c.pos[1] = pos.y; c.pos[2] = pos.z;
    c.fwd[0] = fw.x; c.fwd[1] = fw.y; c.fwd[2] = fw.z;
    c.rgt[0] = rg.x; c.rgt[1] = rg.y; c.rgt[2] = rg.z;
    c.up[0] = upv.x; c.up[1] = upv.y; c.up[2] = upv.z;
    c.near_ = nr; c.far_ = fr; c.W = W; c.H = H;
    c.halfW = W / 2.0f; c.halfH = H / 2.0f;
    c.margin = (fr - nr) * d.depth_margin;
    c.spread = fr - nr + (c.margin * 2.0f);
    c.ortho_scale = d.ortho_scale;
    c.snap = d.vertex_snapping > 0.0f ? d.vertex_snapping : 0.0f;
    c.fog_range[0] = d.fog_range[0]; c.fog_range[1] = d.fog_range[1];
    for (int i = 0; i < 4; i++) c.fog_color[i] = d.fog_color[i];
    c.perspective = d.perspective; c.render_depth = d.render_depth; c.persp_correct = d.perspective_corrected;
    c.fog_on = d.fog_on; c.fog_mode = d.fog_mode;
}

// beginRender (light.go:110-113, :318-320): per frame, per light.
void build_light(const t3d_light_desc& d, DevLight& L) {
    memset(&L, 0, sizeof L);
    L.type = d.type;
    for (int i = 0; i < 3; i++) {
        L.cnt[i] = d.cell_count[i];
        L.color[i] = d.color[i];
        L.vmin[i] = d.vol_min[i]; L.vmax[i] = d.vol_max[i]; L.cell[i] = d.cell_size[i];
        L.offset[i] = d.offset[i]; L.bias[i] = d.bias[i];
    }
    L.color[3] = d.color[3];
    L.energy = d.energy;
    L.range = d.range;
    L.range2 = d.range * d.range;
    m4 t = load16(d.transform);
    f3 wp = row3(t, 3);
    L.wpos[0] = wp.x; L.wpos[1] = wp.y; L.wpos[2] = wp.z;
    L.amb[0] = d.color[0] * d.energy; L.amb[1] = d.color[1] * d.energy; L.amb[2] = d.color[2] * d.energy;
    f3 fw = unit3(row3(load16(d.world_rotation), 2));
    L.fwd[0] = fw.x; L.fwd[1] = fw.y; L.fwd[2] = fw.z;
    L.cell_first = d.cell_first;
}

// Host mirror of a model's world transform (for draw-order distances).
static m4 host_transform(const SceneModel& m) {
    if (m.d.use_trs)
        return trs(mk3(m.d.position[0], m.d.position[1], m.d.position[2]),
                   mk3(m.d.scale[0], m.d.scale[1], m.d.scale[2]), load16(m.d.rotation));
    return load16(m.d.transform);
}

// ------------------------------------------------------------ scenes ----
// ------------------------------------------------------ auto-subdivision ----
// Mesh.SetAutoSubdivide (mesh.go:447-490) with Triangle.performSubdivision
// (mesh.go:1758-1864), done once at upload: every part lists each of its
// triangles followed by that triangle's subdivision levels (forEachTri with
// subdivisions, mesh.go:2238-2256), the new vertices appended after the mesh's
// own. Per listed triangle: its centre, and for the per-frame level choice the
// base triangle's Normal and MaxSpan, its level (-1: the base itself), the
// base's level count and the distance back to the base's entry.
struct SubdividedMesh {
    std::vector<float> pos, nrm, uv, col;
    std::vector<uint32_t> idx;
    std::vector<float> ctr;
    std::vector<float4> info;
    std::vector<int4> rel;
    std::vector<t3d_part_desc> parts;
    t3d_mesh_desc desc;
};

namespace {
struct SubTri { uint32_t a, b, c; float maxspan; float ctr[3]; };

float edge_len(const float* p, const float* q) {  // Vector3.Sub + Magnitude
    const float x = p[0] - q[0], y = p[1] - q[1], z = p[2] - q[2];
    return sqrtf(x * x + y * y + z * z);
}

struct Subdivider {
    SubdividedMesh& S;
    bool colors;
    float smallest;
    uint32_t maxsub;
    std::vector<std::vector<SubTri>>* levels;

    uint32_t lerp_vertex(uint32_t i, uint32_t j) {  // Vector3/Vector2/Color4 Lerp(.., 0.5): a + ((b - a) * 0.5)
        const uint32_t n = (uint32_t)(S.pos.size() / 3);
        for (int k = 0; k < 3; k++) S.pos.push_back(S.pos[3 * (size_t)i + k] + ((S.pos[3 * (size_t)j + k] - S.pos[3 * (size_t)i + k]) * 0.5f));
        for (int k = 0; k < 3; k++) S.nrm.push_back(S.nrm[3 * (size_t)i + k] + ((S.nrm[3 * (size_t)j + k] - S.nrm[3 * (size_t)i + k]) * 0.5f));
        for (int k = 0; k < 2; k++) S.uv.push_back(S.uv[2 * (size_t)i + k] + ((S.uv[2 * (size_t)j + k] - S.uv[2 * (size_t)i + k]) * 0.5f));
        if (colors)
            for (int k = 0; k < 4; k++)
                S.col.push_back(S.col[4 * (size_t)i + k] + ((S.col[4 * (size_t)j + k] - S.col[4 * (size_t)i + k]) * 0.5f));
        return n;
    }
    SubTri child(uint32_t a, uint32_t b, uint32_t c, float maxspan) {
        SubTri t{a, b, c, maxspan, {0.f, 0.f, 0.f}};
        const float third = (float)(1.0 / 3.0);  // Vector3.Scale(1.0 / 3.0)
        for (int k = 0; k < 3; k++)
            t.ctr[k] = ((S.pos[3 * (size_t)a + k] + S.pos[3 * (size_t)b + k]) + S.pos[3 * (size_t)c + k]) * third;
        return t;
    }
    void perform(uint32_t level, const SubTri& t) {
        if (level == maxsub || t.maxspan <= smallest) return;
        // the three edge midpoints in the order (a, b), (b, c), (c, a)
        const uint32_t s = lerp_vertex(t.a, t.b);
        lerp_vertex(t.b, t.c);
        lerp_vertex(t.c, t.a);
        const float half = t.maxspan / 2.0f;
        const SubTri k[4] = {child(t.a, s, s + 2, half), child(s, t.b, s + 1, half), child(s + 1, t.c, s + 2, half),
                             child(s, s + 1, s + 2, half)};
        for (int q = 0; q < 4; q++) (*levels)[level].push_back(k[q]);
        for (int q = 0; q < 4; q++) perform(level + 1, k[q]);
    }
};
}  // namespace

// Returns false (and stops) once the listed triangles pass `max_tris`.
bool subdivide_mesh(const t3d_mesh_desc& me, const float* lev, uint32_t nlev, uint32_t maxsub, SubdividedMesh& S,
                    uint64_t max_tris) {
    const size_t nv = me.num_vertices;
    S.pos.assign(me.positions, me.positions + 3 * nv);
    S.nrm.assign(me.normals, me.normals + 3 * nv);
    S.uv.assign(me.uvs, me.uvs + 2 * nv);
    if (me.colors) S.col.assign(me.colors, me.colors + 4 * nv);
    float smallest = 3.402823466e38f;
    for (uint32_t i = 0; i < nlev; i++)
        if (lev[2 * i + 1] < smallest) smallest = lev[2 * i + 1];
    std::vector<std::vector<SubTri>> levels;
    Subdivider D{S, me.colors != nullptr, smallest, maxsub, &levels};
    for (uint32_t p = 0; p < me.num_parts; p++) {
        t3d_part_desc part = me.parts[p];
        const uint32_t first = (uint32_t)(S.idx.size() / 3);
        for (uint64_t t = me.parts[p].tri_start; t < (uint64_t)me.parts[p].tri_start + me.parts[p].tri_count; t++) {
            const uint32_t a = me.indices[3 * t], b = me.indices[3 * t + 1], c = me.indices[3 * t + 2];
            const float* pa = me.positions + 3 * (size_t)a;
            const float* pb = me.positions + 3 * (size_t)b;
            const float* pc = me.positions + 3 * (size_t)c;
            // Triangle.RecalculateCenter / MaxSpan (mesh.go:1972-2026): Go's max of the three edges
            const float e0 = edge_len(pa, pb), e1 = edge_len(pb, pc), e2 = edge_len(pc, pa);
            float ms = e0;
            if (e1 > ms) ms = e1;
            if (e2 > ms) ms = e2;
            if (e0 != e0 || e1 != e1 || e2 != e2) ms = NAN;
            // Triangle.RecalculateNormal (mesh.go:2030-2037): Unit(Cross(B - A, C - B)), else A's vertex normal
            const f3 v0 = sub3(mk3(pb[0], pb[1], pb[2]), mk3(pa[0], pa[1], pa[2]));
            const f3 v1 = sub3(mk3(pc[0], pc[1], pc[2]), mk3(pb[0], pb[1], pb[2]));
            f3 n = unit3(cross3(v0, v1));
            if (!(fabsf(n.x) > 1e-4f || fabsf(n.y) > 1e-4f || fabsf(n.z) > 1e-4f))
                n = mk3(me.normals[3 * (size_t)a], me.normals[3 * (size_t)a + 1], me.normals[3 * (size_t)a + 2]);
            const int nl = (ms <= smallest) ? 0 : (int)maxsub;
            levels.assign(nl, std::vector<SubTri>());
            if (nl) D.perform(0, SubTri{a, b, c, ms, {0.f, 0.f, 0.f}});
            const uint32_t base = (uint32_t)(S.idx.size() / 3);
            const float4 info = make_float4(n.x, n.y, n.z, ms);
            S.idx.insert(S.idx.end(), {a, b, c});
            for (int k = 0; k < 3; k++) S.ctr.push_back((pa[k] + pb[k] + pc[k]) / 3.0f);
            S.info.push_back(info);
            S.rel.push_back(make_int4(-1, nl, 0, 0));
            for (int L = 0; L < nl; L++)
                for (const SubTri& st : levels[L]) {
                    const uint32_t e = (uint32_t)(S.idx.size() / 3);
                    S.idx.insert(S.idx.end(), {st.a, st.b, st.c});
                    S.ctr.insert(S.ctr.end(), {st.ctr[0], st.ctr[1], st.ctr[2]});
                    S.info.push_back(info);
                    S.rel.push_back(make_int4(L, nl, (int)(e - base), 0));
                }
            if (S.idx.size() / 3 > max_tris || S.pos.size() / 3 > max_tris) return false;
        }
        part.tri_start = first;
        part.tri_count = (uint32_t)(S.idx.size() / 3) - first;
        S.parts.push_back(part);
    }
    S.desc = me;
    S.desc.positions = S.pos.data();
    S.desc.normals = S.nrm.data();
    S.desc.uvs = S.uv.data();
    S.desc.colors = me.colors ? S.col.data() : nullptr;
    S.desc.indices = S.idx.data();
    S.desc.parts = S.parts.data();
    S.desc.num_vertices = (uint32_t)(S.pos.size() / 3);
    S.desc.num_triangles = (uint32_t)(S.idx.size() / 3);
    if (!me.has_dimensions) {  // Dimensions stay those of the mesh before subdividing
        S.desc.has_dimensions = 1;
        for (int c = 0; c < 3; c++) { S.desc.dim_min[c] = 3.402823466e38f; S.desc.dim_max[c] = -3.402823466e38f; }
        for (size_t v = 0; v < nv; v++)
            for (int c = 0; c < 3; c++) {
                const float p = me.positions[3 * v + c];
                if (S.desc.dim_min[c] > p) S.desc.dim_min[c] = p;
                if (S.desc.dim_max[c] < p) S.desc.dim_max[c] = p;
            }
    }
    return true;
}

// The keyed streams of shape-keyed mesh m for its current weights, queued on the
// context's stream (the caller synchronises before the next frame reads them).
int bake_shapes(t3d_ctx* ctx, Scene* sc, uint32_t m) {
    const SceneMesh& sm = sc->meshes[m];
    const cudaError_t e =
        t3d_bake_shapes(ctx->stream, (const float4*)sc->va.ptr + sm.vbase, (const float4*)sc->vb.ptr + sm.vbase,
                        (const float4*)sc->shape_a.ptr + sm.shape_first, (const float2*)sc->shape_b.ptr + sm.shape_first,
                        (const float*)sc->shape_w.ptr + sm.weight_first, sm.nverts, sm.nkeys,
                        (float4*)sc->vaS.ptr + sm.sbase, (float4*)sc->vbS.ptr + sm.sbase);
    if (e != cudaSuccess) {
        set_err(ctx, "shape key bake: %s", cudaGetErrorString(e));
        return T3D_E_CUDA;
    }
    return T3D_OK;
}

// ------------------------------------------------------------ meshlets ----
// Cuts triangles [t0, t1) of a mesh into runs of consecutive triangles with at
// most T triangles and at most U distinct vertices (a run ends before the
// triangle that would exceed either). `stamp` marks the vertices of the run.
static void cut_meshlets(const uint32_t* idx, uint32_t t0, uint32_t t1, uint32_t T, uint32_t U,
                         std::vector<uint32_t>& stamp, uint32_t& gen, std::vector<Meshlet>& out) {
    uint32_t t = t0;
    while (t < t1) {
        if (++gen == 0) { std::fill(stamp.begin(), stamp.end(), 0u); gen = 1; }
        const uint32_t s = t;
        uint32_t nu = 0;
        while (t < t1 && t - s < T) {
            const uint32_t a = idx[3 * (size_t)t], b = idx[3 * (size_t)t + 1], c = idx[3 * (size_t)t + 2];
            const uint32_t add = (stamp[a] != gen) + (stamp[b] != gen && b != a) + (stamp[c] != gen && c != a && c != b);
            if (nu + add > U) break;
            stamp[a] = stamp[b] = stamp[c] = gen;
            nu += add;
            t++;
        }
        out.push_back({s, t - s, nu, 0u});
    }
}

// Writes one meshlet (layout in t3d_device.cuh): slots in order of first use.
static void fill_meshlet(const Meshlet& ml, const uint32_t* idx, const float4* va, const float4* vb, const float4* vc,
                         bool colors, std::vector<uint32_t>& stamp, std::vector<uint32_t>& slot, uint32_t& gen,
                         std::vector<uint32_t>& verts, unsigned char* dst) {
    if (++gen == 0) { std::fill(stamp.begin(), stamp.end(), 0u); gen = 1; }
    verts.clear();
    uint16_t* li = reinterpret_cast<uint16_t*>(dst);
    for (uint32_t t = 0; t < ml.nt; t++)
        for (int k = 0; k < 3; k++) {
            const uint32_t v = idx[3 * ((size_t)ml.t0 + t) + k];
            if (stamp[v] != gen) {
                stamp[v] = gen;
                slot[v] = (uint32_t)verts.size();
                verts.push_back(v);
            }
            li[3 * t + k] = (uint16_t)slot[v];
        }
    memset(dst + 6ull * ml.nt, 0, mlet_lidx_bytes(ml.nt) - 6ull * ml.nt);
    const uint32_t U4 = mlet_slots4(ml.nu);
    float* pos = reinterpret_cast<float*>(dst + mlet_lidx_bytes(ml.nt));
    float* aos = pos + 3ull * U4;
    const uint32_t af = mlet_aos_stride(colors) / 4;
    memset(pos, 0, (12ull + 4 * af) * U4);
    for (uint32_t q = 0; q < (uint32_t)verts.size(); q++) {
        const float4 a = va[verts[q]], b = vb[verts[q]];
        pos[3 * q] = a.x; pos[3 * q + 1] = a.y; pos[3 * q + 2] = a.z;
        float* r = aos + (size_t)af * q;
        r[0] = a.x; r[1] = a.y; r[2] = a.z; r[3] = a.w;
        r[4] = b.x; r[5] = b.y; r[6] = b.z; r[7] = b.w;
        if (colors) {
            const float4 c = vc[verts[q]];
            r[8] = c.x; r[9] = c.y; r[10] = c.z; r[11] = c.w;
        }
    }
}

// Cuts every part of the scene's meshes into meshlets for a triangle budget T
// and a vertex budget U and stores them in the scene's meshlet pool, from the
// resident vertex and index streams. Meshes with shape keys are cut from their
// keyed streams (baked for the current weights), and each of their meshlets keeps
// its slot -> vertex map so that fill_keyed_meshlets refills it when the weights
// change. Auto-subdivided meshes get none: their pairs take the per-vertex record
// path.
int build_meshlets(t3d_ctx* ctx, Scene* sc, uint32_t T, uint32_t U) {
    sc->mlet.release();
    sc->mlet_kfill.release();
    sc->mlet_vmap.release();
    sc->mlet_T = sc->mlet_U = 0;
    for (SceneMesh& me : sc->meshes) {
        me.mparts.assign(me.parts.size(), {});
        me.kfill_first = me.kfill_count = 0;
    }
    if (U < 3 || U > 65535u) return T3D_OK;
    std::vector<uint32_t> stamp, slot, verts, idx;
    uint32_t gen = 0;
    uint64_t total16 = 0;
    // pass 1: the cuts and their offsets
    for (SceneMesh& me : sc->meshes) {
        if (me.subdiv || me.ntris == 0) continue;
        idx.resize(3ull * me.ntris);
        CK(cudaMemcpy(idx.data(), (const uint32_t*)sc->idx.ptr + 3ull * me.tbase, 12ull * me.ntris, cudaMemcpyDeviceToHost));
        stamp.assign(me.nverts, 0u);
        gen = 0;
        for (size_t p = 0; p < me.parts.size(); p++) {
            const t3d_part_desc& pd = me.parts[p].d;
            cut_meshlets(idx.data(), pd.tri_start, pd.tri_start + pd.tri_count, T, U, stamp, gen, me.mparts[p]);
            for (Meshlet& ml : me.mparts[p]) {
                ml.off16 = (uint32_t)total16;
                total16 += mlet_bytes(ml.nt, ml.nu, me.colors) / 16;
                if (total16 > 0xFFFFFFF0ull) {
                    set_err(ctx, "meshlet pool beyond 64 GB");
                    return T3D_E_INVAL;
                }
            }
        }
    }
    if (total16 == 0) {
        sc->mlet_T = T;
        sc->mlet_U = U;
        return T3D_OK;
    }
    int rc;
    if ((rc = sc->mlet.ensure(ctx, 16ull * total16))) return rc;
    // pass 2: the data, one mesh at a time (shape-keyed meshes from their keyed streams)
    std::vector<float4> va, vb, vc;
    std::vector<unsigned char> data;
    std::vector<MletFill> kfill;
    std::vector<uint32_t> vmap;
    for (SceneMesh& me : sc->meshes) {
        bool any = false;
        for (const auto& v : me.mparts) any |= !v.empty();
        if (!any) continue;
        idx.resize(3ull * me.ntris);
        va.resize(me.nverts); vb.resize(me.nverts); vc.resize(me.nverts);
        CK(cudaMemcpy(idx.data(), (const uint32_t*)sc->idx.ptr + 3ull * me.tbase, 12ull * me.ntris, cudaMemcpyDeviceToHost));
        const float4* sa = me.nkeys ? (const float4*)sc->vaS.ptr + me.sbase : (const float4*)sc->va.ptr + me.vbase;
        const float4* sb = me.nkeys ? (const float4*)sc->vbS.ptr + me.sbase : (const float4*)sc->vb.ptr + me.vbase;
        CK(cudaMemcpy(va.data(), sa, 16ull * me.nverts, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(vb.data(), sb, 16ull * me.nverts, cudaMemcpyDeviceToHost));
        if (me.colors) CK(cudaMemcpy(vc.data(), (const float4*)sc->vc.ptr + me.vbase, 16ull * me.nverts, cudaMemcpyDeviceToHost));
        stamp.assign(me.nverts, 0u);
        slot.assign(me.nverts, 0u);
        gen = 0;
        uint64_t lo = UINT64_MAX, hi = 0;
        for (const auto& v : me.mparts)
            for (const Meshlet& ml : v) {
                lo = std::min<uint64_t>(lo, ml.off16);
                hi = std::max<uint64_t>(hi, ml.off16 + mlet_bytes(ml.nt, ml.nu, me.colors) / 16);
            }
        data.assign(16 * (hi - lo), 0);
        if (me.nkeys) me.kfill_first = (uint32_t)kfill.size();
        for (const auto& v : me.mparts)
            for (const Meshlet& ml : v) {
                fill_meshlet(ml, idx.data(), va.data(), vb.data(), vc.data(), me.colors, stamp, slot, gen, verts,
                             data.data() + 16 * (ml.off16 - lo));
                if (me.nkeys) {  // the meshlet's slot -> vertex map, for refills
                    kfill.push_back({ml.off16, ml.nt, ml.nu, (uint32_t)vmap.size()});
                    vmap.insert(vmap.end(), verts.begin(), verts.end());
                }
            }
        if (me.nkeys) me.kfill_count = (uint32_t)kfill.size() - me.kfill_first;
        CK(cudaMemcpy((unsigned char*)sc->mlet.ptr + 16 * lo, data.data(), data.size(), cudaMemcpyHostToDevice));
    }
    if (!kfill.empty()) {
        if ((rc = sc->mlet_kfill.ensure(ctx, sizeof(MletFill) * kfill.size())) ||
            (rc = sc->mlet_vmap.ensure(ctx, 4ull * std::max<size_t>(1, vmap.size()))))
            return rc;
        CK(cudaMemcpy(sc->mlet_kfill.ptr, kfill.data(), sizeof(MletFill) * kfill.size(), cudaMemcpyHostToDevice));
        if (!vmap.empty()) CK(cudaMemcpy(sc->mlet_vmap.ptr, vmap.data(), 4ull * vmap.size(), cudaMemcpyHostToDevice));
    }
    sc->mlet_T = T;
    sc->mlet_U = U;
    return T3D_OK;
}

// Refills the meshlets of shape-keyed mesh m from its keyed streams (after a bake for new weights).
int fill_keyed_meshlets(t3d_ctx* ctx, Scene* sc, uint32_t m) {
    const SceneMesh& me = sc->meshes[m];
    if (!me.kfill_count || !sc->mlet.ptr) return T3D_OK;
    const cudaError_t e = t3d_fill_keyed(ctx->stream, (unsigned char*)sc->mlet.ptr,
                                         (const MletFill*)sc->mlet_kfill.ptr + me.kfill_first, me.kfill_count,
                                         (const uint32_t*)sc->mlet_vmap.ptr, (const float4*)sc->vaS.ptr + me.sbase,
                                         (const float4*)sc->vbS.ptr + me.sbase, me.colors ? 1u : 0u);
    if (e != cudaSuccess) {
        set_err(ctx, "keyed meshlet refill: %s", cudaGetErrorString(e));
        return T3D_E_CUDA;
    }
    return T3D_OK;
}

int scene_upload(t3d_ctx* ctx, const t3d_scene_desc* d, uint32_t* out) {
    if (!d || !out || (d->num_meshes && !d->meshes) || (d->num_models && !d->models) ||
        (d->num_lights && !d->lights) || (d->num_volume_cells && !d->volume_cells)) {
        set_err(ctx, "scene_upload: null array");
        return T3D_E_INVAL;
    }
    if (d->num_lists == 0 || !d->list_offsets || (d->list_offsets[d->num_lists] && !d->list_items)) {
        set_err(ctx, "scene_upload: light list 0 (the scene list) is required");
        return T3D_E_INVAL;
    }
    auto sc = std::make_unique<Scene>();
    uint64_t nv = 0, nt = 0, nshape = 0, nkeys_total = 0, nshaped = 0;
    bool any_skin = false, any_subdiv = false;
    // auto-subdivided meshes are expanded first; the rest of the upload reads eff[m]
    const uint32_t nlev = d->subdivision_levels ? d->num_subdivision_levels : 0u;
    const uint32_t maxsub = d->max_subdivisions ? d->max_subdivisions : 3u;
    if (d->num_subdivision_levels && !d->subdivision_levels) {
        set_err(ctx, "scene_upload: subdivision levels without their array");
        return T3D_E_INVAL;
    }
    for (uint32_t i = 0; i < nlev; i++)
        if (!(d->subdivision_levels[2 * i + 1] > 0.0f)) {  // the level loop halves MaxSpan down to this size
            set_err(ctx, "subdivision level %u: MaximumTriangleSize must be positive", i);
            return T3D_E_INVAL;
        }
    if (maxsub > 8) {
        set_err(ctx, "scene_upload: max_subdivisions %u above 8", maxsub);
        return T3D_E_INVAL;
    }
    std::vector<std::unique_ptr<SubdividedMesh>> subs(d->num_meshes);
    std::vector<const t3d_mesh_desc*> eff(d->num_meshes);
    for (uint32_t m = 0; m < d->num_meshes; m++) {
        const t3d_mesh_desc& me = d->meshes[m];
        eff[m] = &me;
        if (!me.auto_subdivide || nlev == 0) continue;
        if (!me.positions || !me.normals || !me.uvs || !me.indices || (me.num_parts && !me.parts)) {
            set_err(ctx, "mesh %u: null stream", m);
            return T3D_E_INVAL;
        }
        if (me.num_shape_keys) {  // the new vertices have no shape-key deltas in the reference either
            set_err(ctx, "mesh %u: auto-subdivision together with shape keys", m);
            return T3D_E_INVAL;
        }
        for (uint64_t t = 0; t < 3ull * me.num_triangles; t++)
            if (me.indices[t] >= me.num_vertices) {
                set_err(ctx, "mesh %u: index %u out of range (%u vertices)", m, me.indices[t], me.num_vertices);
                return T3D_E_INVAL;
            }
        for (uint32_t p = 0; p < me.num_parts; p++)
            if ((uint64_t)me.parts[p].tri_start + me.parts[p].tri_count > me.num_triangles) {
                set_err(ctx, "mesh %u part %u: triangle range out of bounds", m, p);
                return T3D_E_INVAL;
            }
        subs[m] = std::make_unique<SubdividedMesh>();
        if (!subdivide_mesh(me, d->subdivision_levels, nlev, maxsub, *subs[m], 0x40000000ull)) {
            set_err(ctx, "mesh %u: subdivided mesh too large for 32-bit indexing", m);
            return T3D_E_INVAL;
        }
        subs[m]->desc.joints = nullptr;  // no skinning on subdivided meshes
        subs[m]->desc.weights = nullptr;
        eff[m] = &subs[m]->desc;
        any_subdiv = true;
    }
    for (uint32_t m = 0; m < d->num_meshes; m++) {
        const t3d_mesh_desc& me = *eff[m];
        if (!me.positions || !me.normals || !me.uvs || !me.indices || (me.num_parts && !me.parts)) {
            set_err(ctx, "mesh %u: null stream", m);
            return T3D_E_INVAL;
        }
        SceneMesh sm;
        sm.subdiv = subs[m] != nullptr;
        sm.vbase = (uint32_t)nv;
        sm.tbase = (uint32_t)nt;
        sm.nverts = me.num_vertices;
        sm.ntris = me.num_triangles;
        sm.colors = me.colors != nullptr;
        if (me.num_shape_keys && (!me.shape_positions || !me.shape_normals || !me.shape_weights)) {
            set_err(ctx, "mesh %u: shape keys without position, normal or weight arrays", m);
            return T3D_E_INVAL;
        }
        if ((me.joints != nullptr) != (me.weights != nullptr)) {
            set_err(ctx, "mesh %u: joints and weights must be given together", m);
            return T3D_E_INVAL;
        }
        sm.nkeys = me.num_shape_keys;
        sm.sbase = (uint32_t)nshaped;
        if (me.num_shape_keys) nshaped += me.num_vertices;
        sm.shape_first = (uint32_t)nshape;
        sm.weight_first = (uint32_t)nkeys_total;
        nshape += (uint64_t)me.num_shape_keys * me.num_vertices;
        nkeys_total += me.num_shape_keys;
        if (nshape > 0xFFFFFFF0ull) {
            set_err(ctx, "scene too large: shape key deltas exceed 32-bit indexing");
            return T3D_E_INVAL;
        }
        sm.skin = me.joints != nullptr;
        any_skin |= sm.skin;
        if (sm.skin)
            for (uint64_t q = 0; q < 4ull * me.num_vertices; q++) sm.max_joint = std::max(sm.max_joint, me.joints[q]);
        for (uint32_t t = 0; t < 3ull * me.num_triangles; t++)
            if (me.indices[t] >= me.num_vertices) {
                set_err(ctx, "mesh %u: index %u out of range (%u vertices)", m, me.indices[t], me.num_vertices);
                return T3D_E_INVAL;
            }
        // Mesh.Dimensions (UpdateDimensions, mesh.go:713-748)
        if (me.has_dimensions) {
            for (int c = 0; c < 3; c++) { sm.dmin[c] = me.dim_min[c]; sm.dmax[c] = me.dim_max[c]; }
        } else {
            for (int c = 0; c < 3; c++) { sm.dmin[c] = 3.402823466e38f; sm.dmax[c] = -3.402823466e38f; }
            for (uint32_t v = 0; v < me.num_vertices; v++)
                for (int c = 0; c < 3; c++) {
                    float p = me.positions[3 * (size_t)v + c];
                    if (sm.dmin[c] > p) sm.dmin[c] = p;
                    if (sm.dmax[c] < p) sm.dmax[c] = p;
                }
        }
        for (uint32_t p = 0; p < me.num_parts; p++) {
            const t3d_part_desc& pd = me.parts[p];
            if ((uint64_t)pd.tri_start + pd.tri_count > me.num_triangles) {
                set_err(ctx, "mesh %u part %u: triangle range out of bounds", m, p);
                return T3D_E_INVAL;
            }
            const t3d_material& mt = pd.mat;
            if (mt.present && (mt.sort_mode < 0 || mt.sort_mode > 2 || mt.lighting_mode < 0 || mt.lighting_mode > 2 ||
                               mt.lv_shading_mode < 0 || mt.lv_shading_mode > 3)) {
                set_err(ctx, "mesh %u part %u: bad material enum", m, p);
                return T3D_E_INVAL;
            }
            ScenePart sp;
            sp.d = pd;
            uint32_t vmin = 0xFFFFFFFFu, vmax = 0;
            for (uint64_t t = pd.tri_start; t < (uint64_t)pd.tri_start + pd.tri_count; t++)
                for (int c = 0; c < 3; c++) {
                    uint32_t v = me.indices[3 * t + c];
                    vmin = std::min(vmin, v);
                    vmax = std::max(vmax, v);
                }
            sp.vmin = pd.tri_count ? vmin : 0;
            sp.vcount = pd.tri_count ? vmax - vmin + 1 : 0;
            sm.parts.push_back(sp);
        }
        nv += me.num_vertices;
        nt += me.num_triangles;
        if (nv > 0xFFFFFFF0ull || nt > 0x50000000ull) {
            set_err(ctx, "scene too large for 32-bit vertex/triangle indexing");
            return T3D_E_INVAL;
        }
        sc->meshes.push_back(std::move(sm));
    }
    for (uint32_t i = 0; i < d->num_models; i++) {
        const t3d_model_desc& md = d->models[i];
        if (md.mesh >= d->num_meshes) {
            set_err(ctx, "model %u: mesh %u out of range", i, md.mesh);
            return T3D_E_INVAL;
        }
        if (md.light_list >= (int32_t)d->num_lists) {
            set_err(ctx, "model %u: light list %d out of range", i, md.light_list);
            return T3D_E_INVAL;
        }
        if (md.batched && (md.batch_owner >= d->num_models || md.batch_owner == i ||
                           d->models[md.batch_owner].mesh >= d->num_meshes ||
                           md.batch_part >= d->meshes[d->models[md.batch_owner].mesh].num_parts)) {
            set_err(ctx, "model %u: batch owner %u or its part %u out of range", i, md.batch_owner, md.batch_part);
            return T3D_E_INVAL;
        }
        if (md.skinned && (!sc->meshes[md.mesh].skin || sc->meshes[md.mesh].subdiv ||
                           (uint64_t)md.bone_first + sc->meshes[md.mesh].max_joint >= d->num_bones)) {
            set_err(ctx, "model %u: skinned without joints or with bones beyond the %u scene bones", i, d->num_bones);
            return T3D_E_INVAL;
        }
        SceneModel sm;
        sm.d = md;
        sc->models.push_back(sm);
    }
    for (uint32_t i = 0; i < d->num_lights; i++) {
        const t3d_light_desc& l = d->lights[i];
        if (l.type < 0 || l.type > 3) {
            set_err(ctx, "light %u: bad type %d", i, l.type);
            return T3D_E_INVAL;
        }
        if (l.type == T3D_LIGHT_VOLUME) {
            uint64_t cells = (uint64_t)std::max(0, l.cell_count[0]) * std::max(0, l.cell_count[1]) * std::max(0, l.cell_count[2]);
            if ((uint64_t)l.cell_first + cells > d->num_volume_cells) {
                set_err(ctx, "light %u: volume cells out of range", i);
                return T3D_E_INVAL;
            }
        }
        sc->lights.push_back(l);
    }
    sc->lists.resize(d->num_lists);
    for (uint32_t L = 0; L < d->num_lists; L++) {
        for (uint32_t q = d->list_offsets[L]; q < d->list_offsets[L + 1]; q++) {
            if (d->list_items[q] >= d->num_lights) {
                set_err(ctx, "light list %u: light %u out of range", L, d->list_items[q]);
                return T3D_E_INVAL;
            }
            sc->lists[L].push_back(d->list_items[q]);
        }
    }
    sc->nverts = nv;
    sc->ntris = nt;
    // joints travel as bytes when the scene's largest joint fits one
    bool joint8 = any_skin;
    for (const SceneMesh& sm : sc->meshes)
        if (sm.skin && sm.max_joint > 255u) joint8 = false;
    sc->joint8 = joint8;
    // device pools
    int rc;
    if ((rc = sc->va.ensure(ctx, nv * 16)) || (rc = sc->vb.ensure(ctx, nv * 16)) || (rc = sc->vc.ensure(ctx, nv * 16)) ||
        // 256 bytes of slack: L2 prefetches round their ranges out to 16 bytes
        (rc = sc->idx.ensure(ctx, nt * 12 + 256)) || (rc = sc->centers.ensure(ctx, nt * 12 + 256)) ||
        (rc = sc->dmeshes.ensure(ctx, sizeof(DevMesh) * std::max<size_t>(1, d->num_meshes))) ||
        (rc = sc->dmodels.ensure(ctx, sizeof(DevModel) * std::max<size_t>(1, d->num_models))) ||
        (rc = sc->cells.ensure(ctx, 16 * std::max<size_t>(1, d->num_volume_cells))) ||
        (rc = sc->shape_a.ensure(ctx, 16 * std::max<uint64_t>(1, nshape))) ||
        (rc = sc->shape_b.ensure(ctx, 8 * std::max<uint64_t>(1, nshape))) ||
        (rc = sc->vaS.ensure(ctx, 16 * std::max<uint64_t>(1, nshaped))) ||
        (rc = sc->vbS.ensure(ctx, 16 * std::max<uint64_t>(1, nshaped))) ||
        (rc = sc->shape_w.ensure(ctx, 4 * std::max<uint64_t>(1, nkeys_total))) ||
        (rc = sc->vjoint.ensure(ctx, (joint8 ? 4 : 16) * (any_skin ? std::max<uint64_t>(1, nv) : 1))) ||
        (rc = sc->vweight.ensure(ctx, 16 * (any_skin ? std::max<uint64_t>(1, nv) : 1))) ||
        (rc = sc->bones.ensure(ctx, 64 * std::max<size_t>(1, d->num_bones))) ||
        (rc = sc->sub_info.ensure(ctx, 16 * (any_subdiv ? std::max<uint64_t>(1, nt) : 1))) ||
        (rc = sc->sub_rel.ensure(ctx, 16 * (any_subdiv ? std::max<uint64_t>(1, nt) : 1))) ||
        (rc = sc->sub_levels.ensure(ctx, 8 * std::max<uint32_t>(1, nlev))))
        return rc;
    sc->num_sub_levels = nlev;
    // LightVolumeCell.useLights: offsets per cell, items are scene light indices
    {
        const uint32_t nc = d->num_volume_cells;
        std::vector<uint32_t> off(nc + 1, 0u), items;
        sc->light_uses.assign(d->num_lights, 0);
        sc->light_nested.assign(d->num_lights, 0);
        if (d->cell_use_offsets) {
            if (!d->cell_use_items && d->cell_use_offsets[nc] > d->cell_use_offsets[0]) {
                set_err(ctx, "scene_upload: cell_use_offsets without cell_use_items");
                return T3D_E_INVAL;
            }
            for (uint32_t c = 0; c <= nc; c++) {
                off[c] = d->cell_use_offsets[c] - d->cell_use_offsets[0];
                if (c && off[c] < off[c - 1]) {
                    set_err(ctx, "scene_upload: cell_use_offsets decrease at cell %u", c);
                    return T3D_E_INVAL;
                }
            }
            items.assign(d->cell_use_items + d->cell_use_offsets[0], d->cell_use_items + d->cell_use_offsets[nc]);
            for (uint32_t li : items) {
                if (li >= d->num_lights || d->lights[li].type == T3D_LIGHT_VOLUME) {
                    set_err(ctx, "scene_upload: a cell uses light %u, which is not an ambient, point or directional light", li);
                    return T3D_E_INVAL;
                }
                sc->light_nested[li] = 1;
            }
            for (uint32_t i = 0; i < d->num_lights; i++) {
                const t3d_light_desc& l = d->lights[i];
                if (l.type != T3D_LIGHT_VOLUME) continue;
                const uint64_t cells = (uint64_t)std::max(0, l.cell_count[0]) * std::max(0, l.cell_count[1]) *
                                       std::max(0, l.cell_count[2]);
                sc->light_uses[i] = off[l.cell_first + cells] > off[l.cell_first];
            }
        }
        if ((rc = sc->cell_use_off.ensure(ctx, 4ull * (nc + 1))) ||
            (rc = sc->cell_use_items.ensure(ctx, 4ull * std::max<size_t>(1, items.size()))))
            return rc;
        CK(cudaMemcpy(sc->cell_use_off.ptr, off.data(), 4ull * (nc + 1), cudaMemcpyHostToDevice));
        sc->cell_use_host = off;
        if (!items.empty())
            CK(cudaMemcpy(sc->cell_use_items.ptr, items.data(), 4ull * items.size(), cudaMemcpyHostToDevice));
    }
    if (nlev) CK(cudaMemcpy(sc->sub_levels.ptr, d->subdivision_levels, 8ull * nlev, cudaMemcpyHostToDevice));
    if (d->num_bones && !d->bones) {
        set_err(ctx, "scene_upload: num_bones without bone matrices");
        return T3D_E_INVAL;
    }
    sc->num_bones = d->num_bones;
    sc->num_cells = d->num_volume_cells;
    sc->num_keys = (uint32_t)nkeys_total;
    if (d->num_bones) CK(cudaMemcpy(sc->bones.ptr, d->bones, 64ull * d->num_bones, cudaMemcpyHostToDevice));
    std::vector<float4> a, b, c;
    std::vector<float> ctr;
    for (uint32_t m = 0; m < d->num_meshes; m++) {
        const t3d_mesh_desc& me = *eff[m];
        a.resize(me.num_vertices); b.resize(me.num_vertices); c.resize(me.num_vertices);
        for (uint32_t v = 0; v < me.num_vertices; v++) {
            const float* p = me.positions + 3 * (size_t)v;
            const float* n = me.normals + 3 * (size_t)v;
            const float* u = me.uvs + 2 * (size_t)v;
            a[v] = make_float4(p[0], p[1], p[2], n[0]);
            b[v] = make_float4(n[1], n[2], u[0], u[1]);
            if (me.colors) {
                const float* k = me.colors + 4 * (size_t)v;
                c[v] = make_float4(k[0], k[1], k[2], k[3]);
            } else {
                c[v] = make_float4(1.f, 1.f, 1.f, 1.f);
            }
        }
        size_t off = (size_t)sc->meshes[m].vbase * 16;
        CK(cudaMemcpy((char*)sc->va.ptr + off, a.data(), me.num_vertices * 16ull, cudaMemcpyHostToDevice));
        CK(cudaMemcpy((char*)sc->vb.ptr + off, b.data(), me.num_vertices * 16ull, cudaMemcpyHostToDevice));
        CK(cudaMemcpy((char*)sc->vc.ptr + off, c.data(), me.num_vertices * 16ull, cudaMemcpyHostToDevice));
        CK(cudaMemcpy((char*)sc->idx.ptr + (size_t)sc->meshes[m].tbase * 12, me.indices, me.num_triangles * 12ull,
                      cudaMemcpyHostToDevice));
        // Triangle.RecalculateCenter (mesh.go:1980-1982): ((A + B) + C) / 3 per axis in binary32
        if (subs[m]) {  // subdivided triangles carry their own centres (mesh.go:1821-1845)
            ctr = subs[m]->ctr;
            const size_t tb = sc->meshes[m].tbase;
            CK(cudaMemcpy((float4*)sc->sub_info.ptr + tb, subs[m]->info.data(), 16ull * me.num_triangles,
                          cudaMemcpyHostToDevice));
            CK(cudaMemcpy((int4*)sc->sub_rel.ptr + tb, subs[m]->rel.data(), 16ull * me.num_triangles,
                          cudaMemcpyHostToDevice));
        } else {
            ctr.resize(3ull * me.num_triangles);
            for (uint32_t t = 0; t < me.num_triangles; t++) {
                const float* pa = me.positions + 3 * (size_t)me.indices[3 * (size_t)t];
                const float* pb = me.positions + 3 * (size_t)me.indices[3 * (size_t)t + 1];
                const float* pc = me.positions + 3 * (size_t)me.indices[3 * (size_t)t + 2];
                for (int k = 0; k < 3; k++) ctr[3 * (size_t)t + k] = (pa[k] + pb[k] + pc[k]) / 3.0f;
            }
        }
        CK(cudaMemcpy((char*)sc->centers.ptr + (size_t)sc->meshes[m].tbase * 12, ctr.data(), me.num_triangles * 12ull,
                      cudaMemcpyHostToDevice));
        SceneMesh& smh = sc->meshes[m];
        if (me.num_shape_keys) {  // deltas as (px, py, pz, nx) and (ny, nz)
            const size_t ne = (size_t)me.num_shape_keys * me.num_vertices;
            std::vector<float4> sa(ne);
            std::vector<float2> sb(ne);
            for (size_t q = 0; q < ne; q++) {
                const float* p = me.shape_positions + 3 * q;
                const float* nn = me.shape_normals + 3 * q;
                sa[q] = make_float4(p[0], p[1], p[2], nn[0]);
                sb[q] = make_float2(nn[1], nn[2]);
            }
            CK(cudaMemcpy((float4*)sc->shape_a.ptr + smh.shape_first, sa.data(), 16 * ne, cudaMemcpyHostToDevice));
            CK(cudaMemcpy((float2*)sc->shape_b.ptr + smh.shape_first, sb.data(), 8 * ne, cudaMemcpyHostToDevice));
            CK(cudaMemcpy((float*)sc->shape_w.ptr + smh.weight_first, me.shape_weights, 4ull * me.num_shape_keys,
                          cudaMemcpyHostToDevice));
        }
        if (me.joints && sc->joint8) {
            std::vector<uint32_t> packed(me.num_vertices);
            for (uint32_t v = 0; v < me.num_vertices; v++) {
                const uint32_t* jv = me.joints + 4 * (size_t)v;
                packed[v] = jv[0] | (jv[1] << 8) | (jv[2] << 16) | (jv[3] << 24);
            }
            CK(cudaMemcpy((uint32_t*)sc->vjoint.ptr + smh.vbase, packed.data(), 4ull * me.num_vertices,
                          cudaMemcpyHostToDevice));
        } else if (me.joints) {
            CK(cudaMemcpy((uint4*)sc->vjoint.ptr + smh.vbase, me.joints, 16ull * me.num_vertices, cudaMemcpyHostToDevice));
        }
        if (me.joints) {
            CK(cudaMemcpy((float4*)sc->vweight.ptr + smh.vbase, me.weights, 16ull * me.num_vertices,
                          cudaMemcpyHostToDevice));
        }
        const uint32_t nch = (me.num_triangles + kChunkTris - 1) / kChunkTris;
        smh.chunk_lo.assign(nch, 0xFFFFFFFFu);
        smh.chunk_hi.assign(nch, 0u);
        for (uint32_t t = 0; t < me.num_triangles; t++)
            for (int k = 0; k < 3; k++) {
                const uint32_t v = me.indices[3 * (size_t)t + k];
                smh.chunk_lo[t / kChunkTris] = std::min(smh.chunk_lo[t / kChunkTris], v);
                smh.chunk_hi[t / kChunkTris] = std::max(smh.chunk_hi[t / kChunkTris], v);
            }
    }
    std::vector<DevMesh> dm(d->num_meshes);
    for (uint32_t m = 0; m < d->num_meshes; m++) {
        const SceneMesh& sm = sc->meshes[m];
        dm[m].vbase = sm.vbase; dm[m].tbase = sm.tbase; dm[m].nverts = sm.nverts; dm[m].ntris = sm.ntris;
        dm[m].shape_first = sm.shape_first; dm[m].nkeys = sm.nkeys; dm[m].weight_first = sm.weight_first;
        dm[m].sbase = sm.sbase;
        for (int k = 0; k < 3; k++) { dm[m].dmin[k] = sm.dmin[k]; dm[m].dmax[k] = sm.dmax[k]; }
    }
    if (d->num_meshes) CK(cudaMemcpy(sc->dmeshes.ptr, dm.data(), sizeof(DevMesh) * dm.size(), cudaMemcpyHostToDevice));
    for (uint32_t m = 0; m < d->num_meshes; m++)
        if (sc->meshes[m].nkeys && (rc = bake_shapes(ctx, sc.get(), m))) return rc;
    if (nshaped) CK(cudaStreamSynchronize(ctx->stream));
    if (d->num_volume_cells)
        CK(cudaMemcpy(sc->cells.ptr, d->volume_cells, 16ull * d->num_volume_cells, cudaMemcpyHostToDevice));
    rc = scene_write_models(ctx, sc.get(), 0, d->models, d->num_models);
    if (rc) return rc;
    CK(cudaDeviceSynchronize());
    if (ctx->use_meshlets && ctx->mesh_ucap && (rc = build_meshlets(ctx, sc.get(), ctx->tile_tris, ctx->mesh_ucap))) return rc;
    uint32_t id = ctx->next_scene++;
    *out = id;
    ctx->scenes[id] = std::move(sc);
    return T3D_OK;
}

uint64_t next_version() {
    static std::atomic<uint64_t> v{1};
    return v.fetch_add(1);
}

// Fields of a model that the launch tables are built from, other than its transform.
static bool same_model_structure(const t3d_model_desc& a, const t3d_model_desc& b) {
    return a.mesh == b.mesh && a.visible == b.visible && a.frustum_culling == b.frustum_culling &&
           a.shadeless == b.shadeless && a.light_list == b.light_list && a.use_trs == b.use_trs &&
           a.skinned == b.skinned && a.bone_first == b.bone_first && a.batched == b.batched &&
           a.batch_owner == b.batch_owner && a.batch_part == b.batch_part && memcmp(a.color, b.color, sizeof a.color) == 0;
}

// Model writes are asynchronous: the copy is queued on the stream of the last
// render, behind the frames already issued (which read the previous models),
// and ev_models marks its completion; the next render waits on it on the
// device, and the next write waits on it on the host before reusing the
// pinned staging buffer.
int scene_write_models(t3d_ctx* ctx, Scene* sc, uint32_t first, const t3d_model_desc* models, uint32_t n) {
    if (n == 0) return T3D_OK;
    if (ctx->ev_models) CK(cudaEventSynchronize(ctx->ev_models));
    if (ctx->model_host.ensure(sizeof(DevModel) * n)) {
        set_err(ctx, "pinned model staging alloc failed");
        return T3D_E_OOM;
    }
    DevModel* dv = (DevModel*)ctx->model_host.ptr;
    bool structure = sc->struct_ver == 0;
    for (uint32_t i = 0; i < n; i++) {
        const t3d_model_desc& md = models[i];
        DevModel& m = dv[i];
        memset(&m, 0, sizeof m);
        memcpy(m.transform, md.transform, 64);
        memcpy(m.world_rot, md.world_rotation, 64);
        memcpy(m.position, md.position, 12);
        memcpy(m.scale, md.scale, 12);
        memcpy(m.rotation, md.rotation, 64);
        memcpy(m.rotate_step, md.rotate_step, 64);
        memcpy(m.color, md.color, 16);
        m.mesh = md.mesh;
        m.flags = (md.visible ? MOD_VISIBLE : 0) | (md.frustum_culling ? MOD_FRUSTUM : 0) | (md.shadeless ? MOD_SHADELESS : 0) |
                  (md.use_trs ? MOD_TRS : 0) | (md.skinned ? MOD_SKINNED : 0);
        m.bone_first = md.bone_first;
        if (!structure && !same_model_structure(sc->models[first + i].d, md)) structure = true;
        sc->models[first + i].d = md;
    }
    cudaStream_t st = ctx->last_stream ? ctx->last_stream : ctx->stream;
    CK(cudaMemcpyAsync((char*)sc->dmodels.ptr + sizeof(DevModel) * first, dv, sizeof(DevModel) * n,
                       cudaMemcpyHostToDevice, st));
    if (ctx->ev_models) CK(cudaEventRecord(ctx->ev_models, st));
    else CK(cudaStreamSynchronize(st));
    if (structure) sc->struct_ver = next_version();
    sc->model_ver = next_version();
    return T3D_OK;
}

// ------------------------------------------------------------ frames ----
// Builds the tables of one frame. Instances and segments are laid out per job.
void order_altered_items(t3d_ctx* ctx, FrameTables& F);
void plan_scan(t3d_ctx* ctx, FrameTables& F);

// Segment flags of a part's billboard options; a skinned model's vertices skip
// the model matrix, so billboarding does not apply to it (model.go:760-770).
uint32_t billboard_flags(const t3d_material& mat, bool skinned) {
    if (!mat.present || !mat.billboard || skinned) return 0u;
    uint32_t f = SEG_BILLBOARD;
    if (mat.billboard_lock[0]) f |= SEG_BB_LOCKX;
    if (mat.billboard_lock[1]) f |= SEG_BB_LOCKY;
    if (mat.billboard_lock[2]) f |= SEG_BB_LOCKZ;
    if (mat.billboard_up == T3D_BILLBOARD_UP_CAMERA_Y) f |= SEG_BB_CAMUP;
    if (mat.billboard_depth == T3D_DEPTH_UNBILLBOARDED) f |= SEG_UNBB;
    return f;
}

int build_frame(t3d_ctx* ctx, const t3d_job_desc* jobs, uint32_t njobs, int animate) {
    FrameTables& F = ctx->tables;
    F.clear();
    ctx->tables_ok = false;
    ctx->order_dep = false;
    const uint32_t T = ctx->tile_tris;
    for (uint32_t j = 0; j < njobs; j++) {
        auto it = ctx->scene_map().find(jobs[j].scene);
        if (it == ctx->scene_map().end()) {
            set_err(ctx, "job %u: unknown scene %u", j, jobs[j].scene);
            return T3D_E_NOTFOUND;
        }
        if (jobs[j].camera.width <= 0 || jobs[j].camera.height <= 0) {
            set_err(ctx, "job %u: bad camera size", j);
            return T3D_E_INVAL;
        }
        Scene* sc = it->second.get();
        DevJob dj;
        memset(&dj, 0, sizeof dj);
        build_camera(jobs[j].camera, dj.cam);
        dj.va = (const float4*)sc->va.ptr;
        dj.vb = (const float4*)sc->vb.ptr;
        dj.vc = (const float4*)sc->vc.ptr;
        dj.idx = (const uint32_t*)sc->idx.ptr;
        dj.centers = (const float*)sc->centers.ptr;
        dj.meshes = (const DevMesh*)sc->dmeshes.ptr;
        dj.models = (DevModel*)sc->dmodels.ptr;
        dj.cells = (const float*)sc->cells.ptr;
        dj.shape_a = (const float4*)sc->shape_a.ptr;
        dj.shape_b = (const float2*)sc->shape_b.ptr;
        dj.vaS = (const float4*)sc->vaS.ptr;
        dj.vbS = (const float4*)sc->vbS.ptr;
        dj.shape_w = (const float*)sc->shape_w.ptr;
        dj.vjoint = (const uint4*)sc->vjoint.ptr;
        dj.vjoint8 = sc->joint8 ? (const uint32_t*)sc->vjoint.ptr : nullptr;
        dj.vweight = (const float4*)sc->vweight.ptr;
        dj.bones = (const float4*)sc->bones.ptr;
        dj.sub_info = (const float4*)sc->sub_info.ptr;
        dj.sub_rel = (const int4*)sc->sub_rel.ptr;
        dj.sub_levels = (const float*)sc->sub_levels.ptr;
        dj.nsub_levels = sc->num_sub_levels;
        dj.pad_sub = 0;
        dj.cell_use_off = (const uint32_t*)sc->cell_use_off.ptr;
        dj.cell_use_items = (const uint32_t*)sc->cell_use_items.ptr;
        // meshlets cut for another tuning are rebuilt by the context that owns the scene
        if (ctx->use_meshlets && ctx->mesh_ucap && !ctx->scene_owner && (sc->mlet_T != T || sc->mlet_U != ctx->mesh_ucap)) {
            CK(cudaDeviceSynchronize());
            int rc = build_meshlets(ctx, sc, T, ctx->mesh_ucap);
            if (rc) return rc;
        }
        const bool mlet_ok = ctx->use_meshlets && ctx->mesh_ucap && sc->mlet_T == T && sc->mlet_U == ctx->mesh_ucap;
        const uint32_t light_base = (uint32_t)F.lights.size();
        for (const auto& l : sc->lights) {
            DevLight L;
            build_light(l, L);
            F.lights.push_back(L);
        }
        F.job_light_base.push_back(light_base);
        F.jobs.push_back(dj);
        F.job_scene.push_back(sc);

        const t3d_camera_desc& cd = jobs[j].camera;
        f3 campos = row3(load16(cd.transform), 3);
        struct Pair { uint32_t model, part; float depth; int32_t order; bool batch; };
        std::vector<Pair> solids, transparents;
        std::vector<uint32_t> inst_of(sc->models.size(), 0xFFFFFFFFu);
        // dynamic batches: the members of each (owner, owner part), in model order
        std::map<std::pair<uint32_t, uint32_t>, std::vector<uint32_t>> batches;
        std::vector<char> owner(sc->models.size(), 0);
        std::vector<char> nested(sc->models.size(), 0);  // the model's lights include a volume whose cells use lights
        for (uint32_t mi = 0; mi < sc->models.size(); mi++)
            if (sc->models[mi].d.batched) {
                batches[{sc->models[mi].d.batch_owner, sc->models[mi].d.batch_part}].push_back(mi);
                owner[sc->models[mi].d.batch_owner] = 1;
            }
        const std::vector<uint32_t> scene_lights = culled_scene_lights(sc, jobs[j]);
        for (uint32_t mi = 0; mi < sc->models.size(); mi++) {
            SceneModel& m = sc->models[mi];
            if (!m.d.visible) continue;
            // instance
            DevInst in;
            memset(&in, 0, sizeof in);
            in.job = j;
            in.model = mi;
            in.animate = animate ? 1u : 0u;
            in.light_off = (uint32_t)F.inst_light_idx.size();
            uint32_t list = m.d.light_list < 0 ? 0u : (uint32_t)m.d.light_list;
            uint32_t cnt = 0;
            for (uint32_t li : list == 0 ? scene_lights : sc->lists[list]) {
                if (!light_enabled(jobs[j].light_mask, li)) continue;
                F.inst_light_idx.push_back(li);  // relative to the job's light table (DevJob.lights)
                if (sc->light_uses[li]) nested[mi] = 1;
                cnt++;
            }
            if (cnt > (uint32_t)kMaxLights) {
                set_err(ctx, "model %u: %u lights exceed the per-model maximum %d", mi, cnt, kMaxLights);
                return T3D_E_INVAL;
            }
            in.light_cnt = cnt;
            const SceneMesh& me = sc->meshes[m.d.mesh];
            in.bytes = (uint64_t)(me.colors ? 48 : 32) * me.nverts + 12ull * me.ntris + 64 + 48ull * cnt;
            inst_of[mi] = (uint32_t)F.insts.size();
            F.insts.push_back(in);
            if (animate && m.d.use_trs) {  // host mirror of the device animation step
                m4 rot = mult(load16(m.d.rotate_step), load16(m.d.rotation));
                store16(rot, m.d.rotation);
            }
            m4 M = host_transform(m);
            float depth = dist2(campos, row3(M, 3));  // camera.go:1381
            if (m.d.batched) continue;  // drawn inside its owner's batch (camera.go:1346)
            if (owner[mi]) {
                // one pair per batch part of the owner (camera.go:1397-1451); the
                // transparency found for one part carries over to the later ones there
                F.insts.back().bytes = 0;  // the owner's own mesh is not drawn
                bool transparent = false;
                for (auto it = batches.lower_bound({mi, 0u}); it != batches.end() && it->first.first == mi; ++it) {
                    const t3d_material& bm = me.parts[it->first.second].d.mat;
                    if (bm.present && !bm.visible) continue;
                    for (uint32_t c : it->second) {
                        const SceneModel& cm = sc->models[c];
                        if (!cm.d.visible || transparent) continue;
                        for (const ScenePart& cp : sc->meshes[cm.d.mesh].parts)
                            if (!(cp.d.mat.present && !cp.d.mat.visible) && is_transparent(cm.d.color, cp.d.mat)) {
                                transparent = true;
                                break;
                            }
                    }
                    Pair rp{mi, it->first.second, 0.0f, bm.present ? bm.render_order : 0, true};
                    if (transparent || !cd.render_depth) rp.depth = depth;
                    if (transparent) transparents.push_back(rp);
                    else solids.push_back(rp);
                }
                ctx->order_dep = true;  // members are drawn far to near
                continue;
            }
            for (uint32_t p = 0; p < me.parts.size(); p++) {
                const t3d_material& mat = me.parts[p].d.mat;
                if (mat.present && !mat.visible) continue;
                Pair rp{mi, p, depth, mat.present ? mat.render_order : 0, false};
                if (is_transparent(m.d.color, mat)) transparents.push_back(rp);
                else solids.push_back(rp);
                if (is_transparent(m.d.color, mat) || !cd.render_depth) ctx->order_dep = true;
            }
        }
        auto by_order_then_far = [](const Pair& a, const Pair& b) {
            return a.order != b.order ? a.order < b.order : a.depth > b.depth;
        };
        if (!cd.render_depth) std::stable_sort(solids.begin(), solids.end(), by_order_then_far);
        std::stable_sort(transparents.begin(), transparents.end(), by_order_then_far);
        const size_t nsolid = solids.size();
        solids.insert(solids.end(), transparents.begin(), transparents.end());
        // Draws: a plain pair is one flush; a batch pair draws its visible members far to
        // near from the camera (camera.go:2072-2093; ties keep model order), every part of
        // each, in one flush. Members outside the frustum are culled on the device.
        // fmat: the material of the flush (a batch flushes with its owner's part)
        struct Draw { uint32_t model, part, draw, transparent; const t3d_material* fmat; };
        std::vector<Draw> draws;
        for (size_t q = 0; q < solids.size(); q++) {
            const Pair& rp = solids[q];
            const uint32_t dt = q >= nsolid ? 1u : 0u;
            const t3d_material* fm = &sc->meshes[sc->models[rp.model].d.mesh].parts[rp.part].d.mat;
            if (!rp.batch) {
                draws.push_back({rp.model, rp.part, (uint32_t)q, dt, fm});
                continue;
            }
            std::vector<std::pair<float, uint32_t>> mem;
            for (uint32_t c : batches[{rp.model, rp.part}]) {
                if (!sc->models[c].d.visible) continue;
                mem.push_back({dist2(campos, row3(host_transform(sc->models[c]), 3)), c});
            }
            std::stable_sort(mem.begin(), mem.end(), [](const std::pair<float, uint32_t>& a,
                                                        const std::pair<float, uint32_t>& b) { return a.first > b.first; });
            for (const auto& mc : mem)
                for (uint32_t p = 0; p < sc->meshes[sc->models[mc.second].d.mesh].parts.size(); p++)
                    draws.push_back({mc.second, p, (uint32_t)q, dt, fm});
        }
        for (const Draw& rp : draws) {
            const SceneModel& m = sc->models[rp.model];
            const SceneMesh& me = sc->meshes[m.d.mesh];
            const ScenePart& part = me.parts[rp.part];
            const t3d_material& mat = part.d.mat;
            DevSeg sg;
            memset(&sg, 0, sizeof sg);
            sg.inst = inst_of[rp.model];
            sg.job = j;
            sg.mesh = m.d.mesh;
            sg.tri_start = part.d.tri_start;
            sg.tri_count = part.d.tri_count;
            sg.vmin = part.vmin;
            sg.vcount = part.vcount;
            uint32_t flags = 0;
            if ((m.d.color[3] == 0 && is_transparent(m.d.color, mat)) || part.d.tri_count == 0) flags |= SEG_SKIP;
            bool lit = cd.lighting_on && !(mat.present && mat.shadeless) && !m.d.shadeless;
            if (lit) flags |= SEG_LIT;
            if (lit && nested[rp.model]) flags |= SEG_NESTED;
            if (mat.present && mat.backface_culling) flags |= SEG_BACKFACE;
            if (me.colors) flags |= SEG_COLORS;
            if (mat.present) flags |= SEG_MAT;
            if (part.vcount > kLocalVerts) flags |= SEG_WIDE;
            if (is_transparent(m.d.color, mat)) flags |= SEG_TRANSPARENT;
            if (m.d.skinned) { flags |= SEG_SKINNED; F.any_skinned = true; }
            if (me.nkeys) flags |= SEG_SHAPES;
            if (me.subdiv) flags |= SEG_SUBDIV;
            flags |= billboard_flags(mat, m.d.skinned != 0);
            if (cd.vertex_snapping > 0.0f) flags |= SEG_SNAP;
            if (cd.perspective_corrected) { flags |= SEG_PCORRECT; F.any_pcorrect = true; }
            if (flags & (SEG_ALTERED | SEG_ALT_TILES)) F.any_altered = true;
            // pairs that need no more than the plain vertex loop take their part's meshlets
            const std::vector<Meshlet>* mls = nullptr;
            if (mlet_ok && !(flags & (SEG_ALTERED | SEG_ALT_TILES | SEG_SKIP)) &&
                rp.part < me.mparts.size() && !me.mparts[rp.part].empty())
                mls = &me.mparts[rp.part];
            if (mls) { flags |= SEG_MESHLET; F.any_mesh = true; }
            uint32_t sort_mode = mat.present ? (uint32_t)mat.sort_mode : 0u;
            flags |= sort_mode << 8;
            flags |= (uint32_t)(mat.present ? mat.lighting_mode : 0) << 10;
            flags |= (uint32_t)(mat.present ? mat.lv_shading_mode : 0) << 12;
            sg.mp[0] = m.d.color[0]; sg.mp[1] = m.d.color[1]; sg.mp[2] = m.d.color[2]; sg.mp[3] = m.d.color[3];
            if (mat.present) {
                sg.mp[0] *= mat.color[0]; sg.mp[1] *= mat.color[1]; sg.mp[2] *= mat.color[2]; sg.mp[3] *= mat.color[3];
                sg.tex_w = mat.tex_w; sg.tex_h = mat.tex_h;
            }
            sg.vscratch = (uint32_t)F.nscratch;
            F.seg_vitem_first.push_back((uint32_t)F.vitem_seg.size());
            if (!mls) {  // per-vertex records and vertex work items: record path only
                F.nscratch += sg.vcount;
                const uint32_t nch = (sg.vcount + ctx->vchunk - 1) / ctx->vchunk;
                for (uint32_t c = 0; c < nch; c++) { F.vitem_seg.push_back((uint32_t)F.segs.size()); F.vitem_chunk.push_back(c); }
            }
            sg.out_base = (uint32_t)F.nslots;
            F.nslots += sg.tri_count;
            uint32_t ntiles = mls ? (uint32_t)mls->size() : (sg.tri_count + T - 1) / T;
            if (ntiles == 0) ntiles = 1;
            sg.tile_first = (uint32_t)F.tiles.size();
            sg.ntiles = ntiles;
            const uint32_t s = (uint32_t)F.segs.size();
            if (ntiles > 1 || mls) {  // every meshlet pair takes the multi-tile route
                flags |= SEG_MULTI;
                sg.mt_first = (uint32_t)F.mt_desc.size();
                if (mls && ntiles == 1) flags |= SEG_SINGLE;  // ranked alone: no cross-tile scan
            }
            sg.flags = flags;
            if (mls) {
                for (uint32_t t = 0; t < ntiles; t++) {
                    const Meshlet& ml = (*mls)[t];
                    TileDesc td;
                    memset(&td, 0, sizeof td);
                    td.seg = s; td.inst = sg.inst; td.job = j; td.flags = flags;
                    td.t0 = ml.t0; td.t1 = ml.t0 + ml.nt;
                    td.tbase = me.tbase;
                    td.vmin = ml.nu; td.vlo = ml.off16; td.out_base = sg.out_base;
                    const uint64_t addr = (uint64_t)(uintptr_t)sc->mlet.ptr + 16ull * ml.off16;  // read by the kernel
                    td.vhi = (uint32_t)addr;
                    td.pad1 = (uint32_t)(addr >> 32);
                    td.mt = sg.mt_first + t;
                    td.nearp = dj.cam.near_; td.farp = dj.cam.far_;
                    F.tiles.push_back(td);
                    F.mt_desc.push_back(td);
                }
            }
            for (uint32_t t = 0; t < (mls ? 0u : ntiles); t++) {
                TileDesc td;
                memset(&td, 0, sizeof td);
                td.seg = s; td.inst = sg.inst; td.job = j; td.flags = flags;
                td.t0 = sg.tri_start + t * T;
                td.t1 = std::min(sg.tri_start + sg.tri_count, td.t0 + T);
                td.tbase = me.tbase;
                td.vmin = sg.vmin; td.vscratch = sg.vscratch; td.out_base = sg.out_base;
                td.mt = ntiles > 1 ? sg.mt_first + t : 0u;
                td.nearp = dj.cam.near_; td.farp = dj.cam.far_;
                if (td.t1 > td.t0 && sg.vcount) {  // vertex range of the tile from the chunk table
                    uint32_t lo = 0xFFFFFFFFu, hi = 0u;
                    for (uint32_t c = td.t0 / kChunkTris; c <= (td.t1 - 1) / kChunkTris; c++) {
                        lo = std::min(lo, me.chunk_lo[c]);
                        hi = std::max(hi, me.chunk_hi[c]);
                    }
                    lo = std::max(lo, sg.vmin);
                    hi = std::min(hi, sg.vmin + sg.vcount - 1);
                    if (hi >= lo) { td.vlo = sg.vscratch + (lo - sg.vmin); td.vhi = sg.vscratch + (hi - sg.vmin) + 1; }
                }
                F.tiles.push_back(td);
                if (flags & SEG_MULTI) F.mt_desc.push_back(td);
            }

            sg.pad[0] = rp.draw | (rp.transparent << 31);  // flush and its pass, for the rasteriser
            if (rp.fmat->present) {  // the flush's texture state (camera.go:1840-1876)
                sg.pad[1] = rp.fmat->texture;
                sg.pad[2] = (rp.fmat->texture_filter ? 1u : 0u) | (rp.fmat->texture_map_mode == 1 ? 2u : 0u) |
                            (rp.fmat->transparency_mode == T3D_TRANSPARENCY_ALPHA_CLIP ? 4u : 0u);
                sg.pad2[0] = rp.fmat->texture_map_scale[0];
                sg.pad2[1] = rp.fmat->texture_map_scale[1];
            }
            F.segs.push_back(sg);
            t3d_segment_info si;
            si.job = j; si.model = rp.model; si.part = rp.part; si.base = sg.out_base; si.capacity = sg.tri_count; si.count = 0;
            si.draw = rp.draw; si.draw_transparent = rp.transparent;
            F.seg_info.push_back(si);
            F.seg_mt_seg.push_back(0xFFFFFFFFu);  // the pair's first scan item (plan_scan)
        }
        F.job_seg_end.push_back((uint32_t)F.segs.size());
    }
    if (F.nslots > 0xFFFFFFF0ull || F.nscratch > 0xFFFFFFF0ull) {
        set_err(ctx, "frame too large for 32-bit slots");
        return T3D_E_INVAL;
    }
    F.tile_alt = F.tile_mesh = (uint32_t)F.tiles.size();
    F.vitem_alt = (uint32_t)F.vitem_seg.size();
    F.mt_mesh = (uint32_t)F.mt_desc.size();
    if (F.any_altered || F.any_mesh) order_altered_items(ctx, F);
    plan_scan(ctx, F);
    // point the jobs at their light tables (device address known after upload)
    return T3D_OK;
}

// Vertex items of parts with shape keys or skinning, and tiles of skinned
// parts, move behind the others: the kernel runs them in loops of their own
// (queues 5 and 7), so the loops of plain parts carry none of their code.
// Meshlet tiles go last (tiles: plain | altered | meshlet) and their multi-tile
// numbers after the record path's (mt_desc: record path | meshlet); each part's
// items stay contiguous and in order.
void order_altered_items(t3d_ctx* ctx, FrameTables& F) {
    std::vector<TileDesc> tiles;
    std::vector<uint32_t> vseg, vch;
    tiles.reserve(F.tiles.size());
    vseg.reserve(F.vitem_seg.size());
    vch.reserve(F.vitem_chunk.size());
    const uint32_t nseg = (uint32_t)F.segs.size();
    std::vector<uint32_t> new_tile(nseg), new_vitem(nseg);
    auto tile_class = [](uint32_t f) { return (f & SEG_MESHLET) ? 2 : (f & SEG_ALT_TILES) ? 1 : 0; };
    for (int pass = 0; pass < 3; pass++) {
        for (uint32_t s = 0; s < nseg; s++) {
            const DevSeg& sg = F.segs[s];
            if (tile_class(sg.flags) == pass) {
                new_tile[s] = (uint32_t)tiles.size();
                tiles.insert(tiles.end(), F.tiles.begin() + sg.tile_first, F.tiles.begin() + sg.tile_first + sg.ntiles);
            }
            if (pass < 2 && ((sg.flags & SEG_ALTERED) != 0) == (pass == 1)) {
                const uint32_t nch = (sg.flags & SEG_MESHLET) ? 0u : (sg.vcount + ctx->vchunk - 1) / ctx->vchunk;
                const uint32_t f = F.seg_vitem_first[s];
                new_vitem[s] = (uint32_t)vseg.size();
                vseg.insert(vseg.end(), F.vitem_seg.begin() + f, F.vitem_seg.begin() + f + nch);
                vch.insert(vch.end(), F.vitem_chunk.begin() + f, F.vitem_chunk.begin() + f + nch);
            }
        }
        if (pass == 0) {
            F.tile_alt = (uint32_t)tiles.size();
            F.vitem_alt = (uint32_t)vseg.size();
        } else if (pass == 1) {
            F.tile_mesh = (uint32_t)tiles.size();
        }
    }
    for (uint32_t s = 0; s < nseg; s++) {
        F.segs[s].tile_first = new_tile[s];
        F.seg_vitem_first[s] = new_vitem[s];
    }
    F.tiles.swap(tiles);
    F.vitem_seg.swap(vseg);
    F.vitem_chunk.swap(vch);
    // multi-tile numbers: the record path's first, then the meshlet pairs'
    std::vector<TileDesc> mt;
    mt.reserve(F.mt_desc.size());
    for (int pass = 0; pass < 2; pass++) {
        for (uint32_t s = 0; s < nseg; s++) {
            DevSeg& sg = F.segs[s];
            if (!(sg.flags & SEG_MULTI) || ((sg.flags & SEG_MESHLET) != 0) != (pass == 1)) continue;
            const uint32_t first = (uint32_t)mt.size();
            for (uint32_t t = 0; t < sg.ntiles; t++) {
                TileDesc td = F.mt_desc[sg.mt_first + t];
                td.mt = first + t;
                F.tiles[sg.tile_first + t].mt = first + t;
                mt.push_back(td);
            }
            sg.mt_first = first;
        }
        if (pass == 0) F.mt_mesh = (uint32_t)mt.size();
    }
    F.mt_desc.swap(mt);
}

// The cross-tile scan's work items, in pair order: one per pair of several tiles, or, for a
// pair whose scan would run long beside the rest of the phase -- more than kScanSplit tiles
// and more than four times the frame's multi-tile tiles per block of the scan phase -- one
// per chunk of kScanChunk tiles (the histogram phase then sums each chunk's counts).
void plan_scan(t3d_ctx* ctx, FrameTables& F) {
    F.mt_scan.clear();
    F.mt_chunk.assign(F.mt_desc.size(), kNoChunk);
    F.nchunks = 0;
    const uint64_t blocks = std::max<uint64_t>(1, 2ull * (uint64_t)ctx->num_sms);
    const uint64_t split = std::max<uint64_t>(kScanSplit, 4ull * F.mt_desc.size() / blocks);
    for (uint32_t s = 0; s < (uint32_t)F.segs.size(); s++) {
        const DevSeg& sg = F.segs[s];
        F.seg_mt_seg[s] = 0xFFFFFFFFu;
        if (!(sg.flags & SEG_MULTI) || (sg.flags & SEG_SINGLE)) continue;
        F.seg_mt_seg[s] = (uint32_t)F.mt_scan.size();
        uint32_t nc = 1, cf = kNoChunk;
        if (sg.ntiles > split) {
            nc = (sg.ntiles + kScanChunk - 1) / kScanChunk;
            cf = F.nchunks;
            F.nchunks += nc;
            for (uint32_t t = 0; t < sg.ntiles; t++) F.mt_chunk[sg.mt_first + t] = cf + t / kScanChunk;
        }
        for (uint32_t c = 0; c < nc; c++) F.mt_scan.push_back(make_uint4(s, cf, c, nc));
    }
}

template <typename T> static size_t bytes_of(const std::vector<T>& v) { return v.size() * sizeof(T); }

// Uploads the tables into one device arena and the scratch buffers.
int upload_frame(t3d_ctx* ctx, cudaStream_t st) {
    FrameTables& F = ctx->tables;
    struct Piece { const void* src; size_t bytes; size_t off; };
    std::vector<Piece> pieces;
    size_t off = 0;
    auto add = [&](const void* p, size_t b) {
        size_t o = (off + 255) & ~(size_t)255;
        pieces.push_back({p, b, o});
        off = o + b;
        return o;
    };
    size_t o_lights = add(F.lights.data(), bytes_of(F.lights));
    // jobs reference the light table: patch after we know the arena base
    size_t o_jobs = add(F.jobs.data(), bytes_of(F.jobs));
    size_t o_insts = add(F.insts.data(), bytes_of(F.insts));
    size_t o_ili = add(F.inst_light_idx.data(), bytes_of(F.inst_light_idx));
    size_t o_segs = add(F.segs.data(), bytes_of(F.segs));
    size_t o_ts = add(F.tiles.data(), bytes_of(F.tiles));
    size_t o_mtt = add(F.mt_desc.data(), bytes_of(F.mt_desc));
    size_t o_mts = add(F.mt_scan.data(), bytes_of(F.mt_scan));
    size_t o_mtc = add(F.mt_chunk.data(), bytes_of(F.mt_chunk));
    size_t o_vs = add(F.vitem_seg.data(), bytes_of(F.vitem_seg));
    size_t o_vc = add(F.vitem_chunk.data(), bytes_of(F.vitem_chunk));

    std::vector<DevInst> noanim(F.insts);
    for (auto& in : noanim) in.animate = 0;
    size_t o_noanim = add(noanim.data(), bytes_of(noanim));
    int rc;
    // the previous upload must have left the staging buffer before it is rewritten
    if (ctx->ev_upload) CK(cudaEventSynchronize(ctx->ev_upload));
    if ((rc = ctx->table_host.ensure(off + 256))) { set_err(ctx, "pinned table alloc failed"); return rc; }
    if ((rc = ctx->table_dev.ensure(ctx, off + 256))) return rc;
    char* hb = (char*)ctx->table_host.ptr;
    char* db = (char*)ctx->table_dev.ptr;
    for (auto& p : pieces)
        if (p.bytes) memcpy(hb + p.off, p.src, p.bytes);
    DevJob* hj = (DevJob*)(hb + o_jobs);
    for (size_t j = 0; j < F.jobs.size(); j++) hj[j].lights = (const DevLight*)(db + o_lights) + F.job_light_base[j];
    ctx->last_h2d = off;
    if (off) {
        cudaError_t e = cudaMemcpyAsync(db, hb, off, cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) { set_err(ctx, "table upload: %s", cudaGetErrorString(e)); return T3D_E_CUDA; }
        if (ctx->ev_upload) CK(cudaEventRecord(ctx->ev_upload, st));
    }
    FrameParams& P = ctx->params;
    memset(&P, 0, sizeof P);
    P.jobs = (const DevJob*)(db + o_jobs);
    P.insts = (const DevInst*)(db + o_insts);
    P.inst_light_idx = (const uint32_t*)(db + o_ili);
    P.segs = (const DevSeg*)(db + o_segs);
    P.tiles = (const TileDesc*)(db + o_ts);
    P.mt_desc = (const TileDesc*)(db + o_mtt);
    P.mt_segs = nullptr;
    P.mt_scan = (const uint4*)(db + o_mts);
    P.mt_chunk = F.nchunks ? (const uint32_t*)(db + o_mtc) : nullptr;  // no chunk: no look-ups
    P.vitem_seg = (const uint32_t*)(db + o_vs);
    P.vitem_chunk = (const uint32_t*)(db + o_vc);

    ctx->insts_noanim = (const DevInst*)(db + o_noanim);
    // scratch
    const size_t ninst = std::max<size_t>(1, F.insts.size()), nseg = std::max<size_t>(1, F.segs.size());
    const size_t nmt = std::max<size_t>(1, F.mt_desc.size());
    const size_t nsc = std::max<uint64_t>(1, F.nscratch);
    const size_t nslots = std::max<uint64_t>(1, F.nslots);
    if ((rc = ctx->preps.ensure(ctx, sizeof(DevPrep) * ninst)) ||
(rc = ctx->vcull.ensure(ctx, 16 * nsc)) || (rc = ctx->valt.ensure(ctx, 16 * (F.any_skinned ? nsc : 1))) ||
        (rc = ctx->vxyuv.ensure(ctx, 16 * nsc)) || (rc = ctx->vrgba.ensure(ctx, 16 * nsc)) ||
        (rc = ctx->vis_idx.ensure(ctx, 2ull * nmt * ctx->tile_tris)) ||
        (rc = ctx->vis_depth.ensure(ctx, 4ull * nmt * ctx->tile_tris)) ||
        (rc = ctx->vis_vloc.ensure(ctx, 6ull * nmt * ctx->tile_tris)) || (rc = ctx->tile_count.ensure(ctx, 4 * nmt)) ||
        (rc = ctx->tile_wcnt.ensure(ctx, 4ull * kMaxWarps * nmt)) ||
        (rc = ctx->tile_hist.ensure(ctx, 4ull * kBins * nmt)) ||
        (rc = ctx->chunk_hist.ensure(ctx, 4ull * kBins * std::max<uint32_t>(1u, F.nchunks))) ||
        (rc = ctx->seg_minmax.ensure(ctx, 8 * nseg)) ||
        (rc = ctx->seg_count.ensure(ctx, 4 * nseg)) || (rc = ctx->out_xyuv.ensure(ctx, 48 * nslots)) ||
        (rc = ctx->out_rgba.ensure(ctx, 48 * nslots)) || (rc = ctx->out_depth.ensure(ctx, 12 * nslots)))
        return rc;
    P.preps = (DevPrep*)ctx->preps.ptr;
    P.job_bytes = nullptr;
    if (ctx->want_job_bytes) {
        if ((rc = ctx->job_bytes.ensure(ctx, 8ull * std::max<size_t>(1, F.jobs.size())))) return rc;
        P.job_bytes = (unsigned long long*)ctx->job_bytes.ptr;
    }
    P.inst_lights = nullptr;
    P.vis_rank = nullptr;
    P.live_tiles = nullptr;
    if (F.any_mesh) {  // the instances' staged light lists, the meshlet tiles' rank lists and live list
        if ((rc = ctx->inst_lights.ensure(ctx, 56ull * kMaxLights * ninst + 16)) ||
            (rc = ctx->vis_rank.ensure(ctx, 4ull * nmt * ctx->tile_tris)) || (rc = ctx->live_tiles.ensure(ctx, 4 * nmt)))
            return rc;
        P.inst_lights = (float4*)ctx->inst_lights.ptr;
        P.vis_rank = (uint32_t*)ctx->vis_rank.ptr;
        P.live_tiles = (uint32_t*)ctx->live_tiles.ptr;
    }

    P.vinvw = nullptr;
    P.out_invw = nullptr;
    if (F.any_pcorrect) {  // Custom0: 1 / w per record and per emitted corner
        if ((rc = ctx->vinvw.ensure(ctx, 4 * nsc)) || (rc = ctx->out_invw.ensure(ctx, 12 * nslots))) return rc;
        P.vinvw = (float*)ctx->vinvw.ptr;
        P.out_invw = (float*)ctx->out_invw.ptr;
    }
    P.vcull = (float4*)ctx->vcull.ptr;
    P.valt = (float4*)ctx->valt.ptr;
    P.vxyuv = (float4*)ctx->vxyuv.ptr;
    P.vrgba = (float4*)ctx->vrgba.ptr;
    P.vis_idx = (uint16_t*)ctx->vis_idx.ptr;
    P.vis_depth = (float*)ctx->vis_depth.ptr;
    P.vis_vloc = (uint16_t*)ctx->vis_vloc.ptr;
    P.tile_wcnt = (uint32_t*)ctx->tile_wcnt.ptr;
    P.tile_count = (uint32_t*)ctx->tile_count.ptr;
    P.tile_hist = (uint32_t*)ctx->tile_hist.ptr;
    P.chunk_hist = (uint32_t*)ctx->chunk_hist.ptr;
    P.seg_minmax = (uint32_t*)ctx->seg_minmax.ptr;
    P.seg_count = (uint32_t*)ctx->seg_count.ptr;
    P.out_xyuv = (float4*)ctx->out_xyuv.ptr;
    P.out_rgba = (float4*)ctx->out_rgba.ptr;
    P.out_depth = (float*)ctx->out_depth.ptr;
    P.accum = (unsigned long long*)ctx->accum.ptr;
    P.tile_tris = ctx->tile_tris;
    P.vchunk = ctx->vchunk;
    P.mesh_ucap = ctx->mesh_ucap;
    P.spin_limit = ctx->spin_limit;
    return T3D_OK;
}

static int launch_one(t3d_ctx* ctx, FrameParams P, Ctl* ctl, uint32_t max_items, cudaStream_t st) {
    P.ctl = ctl;
    // frames with meshlet tiles run the instantiation that has their phases
    const bool mesh = P.mesh_begin < P.mesh_end;
    // a launch of one phase runs that phase's own kernel (when split launches are on)
    const uint32_t ph = P.phases;
    const int pk = (ph && !(ph & (ph - 1))) ? __builtin_ctz(ph) : -1;
    const bool one = pk >= 0 && pk < 6 && ctx->split_phases && ctx->phase_grid[mesh][pk];
    const uint32_t cap = std::max(1u, (one ? ctx->phase_grid[mesh][pk] : mesh ? ctx->max_grid_mesh : ctx->max_grid) /
                                          ctx->grid_share);
    const size_t smem = one ? ctx->phase_smem[mesh][pk] : mesh ? ctx->smem_mesh : ctx->smem_bytes;
    uint32_t grid = std::max(1u, std::min(cap, max_items));
    const void* fn = one ? t3d_phase_kernel_ptr(mesh, pk) : mesh ? t3d_frame_kernel_mesh_ptr() : t3d_frame_kernel_ptr();
    void* args[] = {&P};
    cudaLaunchConfig_t cfg;
    memset(&cfg, 0, sizeof cfg);
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(ctx->block_threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    // grid barriers need every block resident: a cooperative launch when more than one block
    // runs more than one phase (one block, or one phase per launch, needs none)
    const bool coop = grid > 1 && (P.phases == 0 || (P.phases & (P.phases - 1)) != 0);
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = coop ? attr : nullptr;
    cfg.numAttrs = coop ? 1 : 0;
    cudaError_t e = cudaLaunchKernelExC(&cfg, fn, args);
    if (e != cudaSuccess) {
        set_err(ctx, "frame kernel launch failed: %s (grid %u, block %u, smem %zu)", cudaGetErrorString(e), grid,
                ctx->block_threads, smem);
        return T3D_E_CUDA;
    }
    ctx->launches++;
    ctx->last_grid = grid;
    for (int k = 0; k < 6; k++)
        if (one ? k == pk : (ph == 0 || (ph >> k) & 1u)) ctx->phase_grid_used[k] = grid;
    return T3D_OK;
}

int launch_frame(t3d_ctx* ctx, int mode, cudaStream_t st) {
    FrameTables& F = ctx->tables;
    const FrameParams& P0 = ctx->params;
    ctx->launches = 0;
    const size_t nlaunch = (mode == T3D_MODE_BATCHED) ? 1 : std::max<size_t>(1, F.segs.size());
    int rc;
    if ((rc = ctx->ctl.ensure(ctx, sizeof(Ctl) * nlaunch))) return rc;
    cudaError_t e = cudaMemsetAsync(ctx->ctl.ptr, 0, sizeof(Ctl) * nlaunch, st);
    if (e != cudaSuccess) { set_err(ctx, "ctl memset: %s", cudaGetErrorString(e)); return T3D_E_CUDA; }
    if (P0.job_bytes && (e = cudaMemsetAsync(ctx->job_bytes.ptr, 0, 8ull * std::max<size_t>(1, F.jobs.size()), st)) != cudaSuccess) {
        set_err(ctx, "job bytes memset: %s", cudaGetErrorString(e));
        return T3D_E_CUDA;
    }
    Ctl* ctl = (Ctl*)ctx->ctl.ptr;
    ctx->nctl = (uint32_t)nlaunch;
    if (F.segs.empty() && F.insts.empty()) return T3D_OK;
    if (mode == T3D_MODE_BATCHED) {
        FrameParams P = P0;
        P.inst_begin = 0; P.inst_end = (uint32_t)F.insts.size();
        P.seg_begin = 0; P.seg_end = (uint32_t)F.segs.size();
        P.tile_begin = 0; P.tile_end = F.tile_mesh;
        P.mesh_begin = F.tile_mesh; P.mesh_end = (uint32_t)F.tiles.size();
        P.mt_tile_begin = 0; P.mt_tile_end = F.mt_mesh;
        P.mt_mesh_begin = F.mt_mesh; P.mt_mesh_end = (uint32_t)F.mt_desc.size();
        P.mt_seg_begin = 0; P.mt_seg_end = (uint32_t)F.mt_scan.size();
        P.chunk_zero_begin = 0; P.chunk_zero_end = F.nchunks;

        P.vitem_begin = 0; P.vitem_end = (uint32_t)F.vitem_seg.size();
        P.tile_alt = F.tile_alt; P.vitem_alt = F.vitem_alt;
        P.has_multi = F.mt_desc.empty() ? 0u : 1u;
        const uint32_t inst_blocks = (uint32_t)((F.insts.size() + ctx->block_threads - 1) / ctx->block_threads);
        if (!ctx->split_phases) {
            uint32_t items = (uint32_t)std::max({F.tiles.size(), F.mt_desc.size(), F.vitem_seg.size(), (size_t)inst_blocks});
            return launch_one(ctx, P, ctl, items, st);
        }
        // one launch per phase, each sized to its own work (the prep phase spreads its models
        // one per block over every SM; the histogram phase ranks one tile per warp); phases
        // with no work are left out
        const uint32_t nmt = (uint32_t)F.mt_desc.size(), warps = ctx->block_threads / 32;
        const uint32_t seq[6][2] = {{1u, std::max<uint32_t>(1u, (uint32_t)std::max(F.insts.size(), F.segs.size()))},
                                    {2u, (uint32_t)F.vitem_seg.size()},
                                    {4u, (uint32_t)F.tiles.size()},
                                    {8u, (nmt + warps - 1) / warps},
                                    {16u, (uint32_t)F.mt_scan.size()},
                                    {32u, nmt}};
        for (const auto& q : seq) {
            if (q[1] == 0 || (q[0] >= 8u && !P.has_multi)) continue;
            P.phases = q[0];
            if ((rc = launch_one(ctx, P, ctl, q[1], st))) return rc;
        }
        return T3D_OK;
    }
    // Plain: render pairs one after another, in draw order (render + flush per pair,
    // camera.go:2061-2106). A pair of one tile is one launch of one block (its phases
    // separated by block barriers); a pair of several tiles is a sequence of launches of
    // one phase each (prep, vertex records, triangles, histogram, scan, rank + emit), so
    // no launch waits on a grid barrier. A model's prep (and animation step) runs with
    // its first pair; its later pairs recompute the same prep without animating.
    std::vector<char> animated(F.insts.size(), 0);
    for (size_t s = 0; s < F.segs.size(); s++) {
        const DevSeg& sg = F.segs[s];
        FrameParams P = P0;
        P.inst_begin = sg.inst; P.inst_end = sg.inst + 1;
        P.seg_begin = (uint32_t)s; P.seg_end = (uint32_t)s + 1;
        const bool mesh = sg.flags & SEG_MESHLET;
        if (mesh) {
            P.tile_begin = P.tile_alt = P.tile_end = 0;
            P.mesh_begin = sg.tile_first; P.mesh_end = sg.tile_first + sg.ntiles;
            P.vitem_begin = P.vitem_alt = P.vitem_end = 0;
        } else {
            P.tile_begin = sg.tile_first; P.tile_end = sg.tile_first + sg.ntiles;
            P.mesh_begin = P.mesh_end = 0;
            P.vitem_begin = F.seg_vitem_first[s];
            P.vitem_end = P.vitem_begin + (sg.vcount + ctx->vchunk - 1) / ctx->vchunk;
            P.tile_alt = (sg.flags & SEG_ALT_TILES) ? P.tile_begin : P.tile_end;
            P.vitem_alt = (sg.flags & SEG_ALTERED) ? P.vitem_begin : P.vitem_end;
        }
        P.mt_tile_begin = P.mt_tile_end = 0; P.mt_mesh_begin = P.mt_mesh_end = 0;
        P.mt_seg_begin = P.mt_seg_end = 0; P.has_multi = 0;
        if (sg.flags & SEG_MULTI) {
            if (mesh) { P.mt_mesh_begin = sg.mt_first; P.mt_mesh_end = sg.mt_first + sg.ntiles; }
            else { P.mt_tile_begin = sg.mt_first; P.mt_tile_end = sg.mt_first + sg.ntiles; }
            if (!(sg.flags & SEG_SINGLE)) {  // the pair's scan items, and its chunks' counts zeroed by its prep
                const uint4 it = F.mt_scan[F.seg_mt_seg[s]];
                P.mt_seg_begin = F.seg_mt_seg[s];
                P.mt_seg_end = P.mt_seg_begin + it.w;
                if (it.w > 1) { P.chunk_zero_begin = it.y; P.chunk_zero_end = it.y + it.w; }
            }
            P.has_multi = 1;
        }
        // animation must be applied once: host tables carry the flag on the instance,
        // so later pairs of the same model use a copy without it.
        if (F.insts[sg.inst].animate && animated[sg.inst]) {
            // re-point the instance range to the no-animate shadow copy
            P.insts = ctx->insts_noanim;
        }
        animated[sg.inst] = 1;
        if (sg.ntiles <= 1) {
            P.phases = 0;
            if ((rc = launch_one(ctx, P, ctl + s, 1u, st))) return rc;
            continue;
        }
        const uint32_t vitems = P.vitem_end - P.vitem_begin;
        const bool scan = P.mt_seg_begin < P.mt_seg_end;
        const uint32_t seq[6][2] = {{1u, 1u}, {2u, vitems}, {4u, sg.ntiles}, {8u, sg.ntiles},
                                    {16u, P.mt_seg_end - P.mt_seg_begin}, {32u, sg.ntiles}};
        for (const auto& q : seq) {
            if ((q[0] == 2u && vitems == 0) || (q[0] >= 8u && !P.has_multi) || (q[0] == 16u && !scan)) continue;
            P.phases = q[0];
            if ((rc = launch_one(ctx, P, ctl + s, q[1], st))) return rc;
        }
    }
    return T3D_OK;
}

}  // namespace t3d
