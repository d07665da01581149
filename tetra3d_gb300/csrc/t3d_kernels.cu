// t3d_kernels.cu -- the GB300 vertex stage: one persistent kernel with phases.
//
//   P0 model prep   per (job, model): Node.Transform (+ animation step), MVP,
//                   model-space camera, SphereInFrustum, light beginModel.
//   P1 vertex       per (segment, vertex chunk): MultVecW, the cull record,
//                   per-vertex lighting and the emitted corner attributes.
//   P2 triangle     per (segment, tile): near/far, +-0.5 and backface rejection,
//                   the depth key, a stable in-tile compaction and, for
//                   single-tile segments, the whole bucket sort + emit.
//   P3..P5          multi-tile segments only: tile histograms, cross-tile bin
//                   scan, stable rank + emit.
// Phases are separated by a bounded software grid barrier; the grid is sized so
// that every block is co-resident (cooperative launch), and work items are
// pulled from per-phase atomic queues so uneven models balance across SMs.
//
// Parity: compiled with -fmad=false and IEEE div/sqrt, every value follows the
// reference's unfused binary32 operation order (see t3d_math.cuh).

#include "t3d_device.cuh"

namespace t3d {

constexpr uint32_t kSpinLimit = 1u << 25;  // ~3-6 s of polling before a barrier gives up

__device__ __forceinline__ uint32_t vload(const uint32_t* p) { return *(const volatile uint32_t*)p; }
__device__ __forceinline__ int32_t vload(const int32_t* p) { return *(const volatile int32_t*)p; }

// Sense-by-generation grid barrier with a bounded wait. On timeout it records
// ERR_BARRIER_TIMEOUT; every block then leaves the kernel at its next barrier.
__device__ bool grid_barrier(Ctl* ctl) {
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t gen = vload(&ctl->bar_gen);
        __threadfence();
        uint32_t arrived = atomicAdd(&ctl->bar_count, 1u) + 1u;
        if (arrived == gridDim.x) {
            atomicExch(&ctl->bar_count, 0u);
            __threadfence();
            atomicAdd(&ctl->bar_gen, 1u);
        } else {
            uint32_t spins = 0;
            while (vload(&ctl->bar_gen) == gen) {
                if (vload(&ctl->err) != 0) break;
                if (++spins > kSpinLimit) {
                    atomicCAS(&ctl->err, 0, ERR_BARRIER_TIMEOUT);
                    break;
                }
                __nanosleep(128);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return vload(&ctl->err) == 0;
}

__device__ __forceinline__ uint32_t next_item(Ctl* ctl, int q, uint32_t* s_item) {
    __syncthreads();
    if (threadIdx.x == 0) *s_item = atomicAdd(&ctl->queue[q], 1u);
    __syncthreads();
    return *s_item;
}

__device__ __forceinline__ float clampf(float v, float lo, float hi) {  // math32.Clamp, math32.go:39-47
    if (v < lo) return lo;
    else if (v > hi) return hi;
    return v;
}

// ------------------------------------------------------------------ P0 ----
// Camera.SphereInFrustum (camera.go:933-983) on the frustum sphere that
// Model.onTransformUpdate derives from the transform (model.go:142-182).
__device__ bool model_in_frustum(const JobCam& c, const m4& M, const DevMesh& me) {
    f3 position, scale;
    m4 rotation;
    decompose(M, position, scale, rotation);
    f3 center = mk3((me.dmax[0] + me.dmin[0]) / 2.0f, (me.dmax[1] + me.dmin[1]) / 2.0f, (me.dmax[2] + me.dmin[2]) / 2.0f);
    center = mult_vec(rotation, center);
    position.x += center.x * scale.x;
    position.y += center.y * scale.y;
    position.z += center.z * scale.z;
    f3 mn = mk3(me.dmin[0] * scale.x, me.dmin[1] * scale.y, me.dmin[2] * scale.z);
    f3 mx = mk3(me.dmax[0] * scale.x, me.dmax[1] * scale.y, me.dmax[2] * scale.z);
    float radius = mag3(sub3(mx, mn)) / 2.0f;

    f3 cpos = mk3(c.pos[0], c.pos[1], c.pos[2]);
    f3 diff = sub3(position, cpos);
    float pcZ = dot3(diff, mk3(-c.fwd[0], -c.fwd[1], -c.fwd[2]));
    if (pcZ > c.far_ + radius || pcZ < c.near_ - radius) return false;
    f3 up = mk3(c.up[0], c.up[1], c.up[2]);
    f3 rgt = mk3(c.rgt[0], c.rgt[1], c.rgt[2]);
    if (c.perspective) {
        float d = c.sphere_y * radius;
        pcZ *= c.sphere_tang;
        float pcY = dot3(diff, up);
        if (pcY > pcZ + d || pcY < -pcZ - d) return false;
        pcZ *= c.aspect;
        d = c.sphere_x * radius;
        float pcX = dot3(diff, rgt);
        if (pcX > pcZ + d || pcX < -pcZ - d) return false;
    } else {
        float width = c.ortho_scale;
        float height = width / c.aspect;
        float pcY = dot3(diff, up);
        if (-height / 2.0f - radius > pcY || pcY > height / 2.0f + radius) return false;
        float pcX = dot3(diff, rgt);
        if (-width / 2.0f - radius > pcX || pcX > width / 2.0f + radius) return false;
    }
    return true;
}

__device__ void phase_prep(const FrameParams& P) {
    const uint32_t n = P.inst_end - P.inst_begin;
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    for (uint32_t k = g; k < n; k += stride) {
        const uint32_t i = P.inst_begin + k;
        const DevInst in = P.insts[i];
        const DevJob& J = P.jobs[in.job];
        DevModel* md = J.models + in.model;
        const DevMesh me = J.meshes[md->mesh];
        m4 M, WR;
        if (md->flags & MOD_TRS) {
            m4 rot = load16(md->rotation);
            if (in.animate) {  // Node.Rotate -> Matrix4.Rotated (node.go:1039-1047, matrix.go:583-585)
                rot = mult(load16(md->rotate_step), rot);
                store16(rot, md->rotation);
            }
            M = trs(mk3(md->position[0], md->position[1], md->position[2]),
                    mk3(md->scale[0], md->scale[1], md->scale[2]), rot);
            WR = rot;
            if (in.animate) {
                store16(M, md->transform);
                store16(rot, md->world_rot);
            }
        } else {
            M = load16(md->transform);
            WR = load16(md->world_rot);
        }
        DevPrep& pr = P.preps[i];
        const JobCam& cam = J.cam;
        m4 vp = load16(cam.vp);
        store16(mult(M, vp), pr.mvp);  // model.go:695
        store16(M, pr.M);
        InvFrame inv = inv_frame(M);   // model.go:629
        f3 ic = to_model_space(inv, mk3(cam.pos[0], cam.pos[1], cam.pos[2]));  // model.go:630
        pr.invcam[0] = ic.x; pr.invcam[1] = ic.y; pr.invcam[2] = ic.z; pr.invcam[3] = 0.0f;
        store16(transposed(inverted(WR)), pr.dirrot);  // light.go:326-330
        bool culled = (md->flags & MOD_FRUSTUM) && !model_in_frustum(cam, M, me);
        pr.culled = culled ? 1u : 0u;
        if (culled) {
            atomicAdd(&P.ctl->culled, 1u);
        } else {
            atomicAdd(&P.ctl->bytes, (unsigned long long)in.bytes);
            atomicAdd(&P.accum[1], (unsigned long long)in.bytes);
        }
        // PointLight.beginModel (light.go:175-189) and the model-level range skip (camera.go:1625-1629)
        f3 dspan = mk3(me.dmax[0] - me.dmin[0], me.dmax[1] - me.dmin[1], me.dmax[2] - me.dmin[2]);
        float maxSpan = mag3(dspan);
        f3 modelPos = row3(M, 3);
        for (uint32_t s = 0; s < in.light_cnt; s++) {
            const uint32_t li = P.inst_light_idx[in.light_off + s];
            const DevLight& L = J.lights[li];
            float4 w = make_float4(0.f, 0.f, 0.f, 0.f);
            if (L.type == T3D_LIGHT_POINT) {
                f3 lp = mk3(L.wpos[0], L.wpos[1], L.wpos[2]);
                f3 wp = to_model_space(inv, lp);
                w.x = wp.x; w.y = wp.y; w.z = wp.z;
                if (L.range > 0.0f) {
                    float dist = maxSpan + L.range;
                    if (dist2(modelPos, lp) > dist * dist) w.w = 1.0f;
                }
            }
            P.inst_light_work[in.light_off + s] = w;
        }
    }
    const uint32_t ns = P.seg_end - P.seg_begin;
    for (uint32_t k = g; k < ns; k += stride) {
        const uint32_t s = P.seg_begin + k;
        P.seg_minmax[2 * s] = 0xFFFFFFFFu;
        P.seg_minmax[2 * s + 1] = 0u;
        P.seg_count[s] = 0u;
    }
}

// ------------------------------------------------------------------ P1 ----
struct SLight {
    int32_t type, skip;
    int32_t cnt[3];
    uint32_t cell_first;
    float cr, cg, cb, energy, range, range2;
    float wx, wy, wz;    // point: model-space workingPosition
    float ax, ay, az;    // ambient result
    float fx, fy, fz;    // directional workingForward
    float vmin[3], vmax[3], cell[3], off[3], bias[3];
};

struct VertexSmem {
    SLight lights[kMaxLights];
    float mvp[16];
    float M[16];
    float dirrot[16];
    uint32_t nlights;
    uint32_t item;
};

// LightVolume.convertToXYZIndices + getLightCell (light.go:717-741, :1267-1272)
__device__ __forceinline__ int lv_index(float v) {
    if (!(v > -2147483648.0f && v < 2147483647.0f)) return -1;
    return (int)v;
}
__device__ bool lv_cell(const SLight& L, f3 p, uint32_t& idx) {
    float csx = L.cell[0], csy = L.cell[1], csz = L.cell[2];
    int x = lv_index(roundf(((p.x - L.off[0] - L.vmin[0] - (csx / 2.0f)) / csx)));
    int y = lv_index(roundf(((p.y - L.off[1] - L.vmin[1] - (csy / 2.0f)) / csy)));
    int z = lv_index(roundf(((p.z - L.off[2] - L.vmin[2] - (csz / 2.0f)) / csz)));
    if (x < 0 || y < 0 || z < 0 || x >= L.cnt[0] || y >= L.cnt[1] || z >= L.cnt[2]) return false;
    idx = (uint32_t)(x + (y * L.cnt[0]) + (z * L.cnt[0] * L.cnt[1]));
    return true;
}

// One light's contribution to one vertex (ILight.VertexLight, light.go:115-663).
__device__ __forceinline__ void light_vertex(const SLight& L, uint32_t flags, f3 vpos, f3 vnrm, const m4& M,
                                             const m4& dirrot, const float* __restrict__ cells, float& r, float& g,
                                             float& b) {
    const bool mat = flags & SEG_MAT;
    const uint32_t lmode = seg_light_mode(flags);
    switch (L.type) {
    case T3D_LIGHT_AMBIENT:
        r += L.ax; g += L.ay; b += L.az;
        break;
    case T3D_LIGHT_POINT: {
        f3 work = mk3(L.wx, L.wy, L.wz);
        float distance = dist2(work, vpos);
        if (L.range > 0.0f) {
            if (distance > L.range2) return;
        } else {
            if (1.0f / distance * L.energy < 0.001f) return;
        }
        f3 lightVec = unit3(sub3(work, vpos));
        f3 n = (mat && lmode == T3D_LIGHTING_FIXED_NORMALS) ? lightVec : vnrm;
        float diffuse = dot3(n, lightVec);
        if (mat && lmode == T3D_LIGHTING_DOUBLE_SIDED) diffuse = fabsf(diffuse);
        if (diffuse > 0.0f) {
            float df = diffuse * (1.0f / (1.0f + (0.1f * distance))) * 2.0f;
            if (L.range2 > 0.0f) {
                float dc = clampf((L.range2 - distance) / distance, 0.0f, 1.0f);
                df *= dc;
            }
            r += L.cr * df * L.energy;
            g += L.cg * df * L.energy;
            b += L.cb * df * L.energy;
        }
        break;
    }
    case T3D_LIGHT_DIRECTIONAL: {
        f3 fwd = mk3(L.fx, L.fy, L.fz);
        f3 normal = (mat && lmode == T3D_LIGHTING_FIXED_NORMALS) ? fwd : mult_vec(dirrot, vnrm);
        float df = dot3(normal, fwd);
        if (mat && lmode == T3D_LIGHTING_DOUBLE_SIDED) df = fabsf(df);
        if (df <= 0.0f) return;
        r += L.cr * df * L.energy;
        g += L.cg * df * L.energy;
        b += L.cb * df * L.energy;
        break;
    }
    case T3D_LIGHT_VOLUME: {
        const uint32_t mode = mat ? seg_lv_mode(flags) : 0u;
        if (mat && mode == T3D_LV_OFF) return;
        float cr = 0.0f, cg = 0.0f, cb = 0.0f;
        uint32_t idx;
        if (mat && mode == T3D_LV_PER_OBJECT) {
            if (lv_cell(L, row3(M, 3), idx)) {
                const float* c = cells + 4 * (size_t)(L.cell_first + idx);
                cr = c[0]; cg = c[1]; cb = c[2];
            }
        } else {
            f3 cs = mk3(L.cell[0] / 2.0f, L.cell[1] / 2.0f, L.cell[2] / 2.0f);
            f3 bias = mk3(L.bias[0], L.bias[1], L.bias[2]);
            f3 vertPos = mk3(0.f, 0.f, 0.f), vertPosN = mk3(0.f, 0.f, 0.f);
            if (mode == T3D_LV_PER_VERTEX_WITH_NORMAL) vertPosN = add3(mult_vec(M, add3(vpos, hmul3(vnrm, cs))), bias);
            else vertPos = add3(mult_vec(M, vpos), bias);
            if (!(vertPos.x >= L.vmin[0] && vertPos.y >= L.vmin[1] && vertPos.z >= L.vmin[2] && vertPos.x <= L.vmax[0] &&
                  vertPos.y <= L.vmax[1] && vertPos.z <= L.vmax[2]))
                return;
            if (lv_cell(L, mode == T3D_LV_PER_VERTEX_WITH_NORMAL ? vertPosN : vertPos, idx)) {
                const float* c = cells + 4 * (size_t)(L.cell_first + idx);
                cr = c[0]; cg = c[1]; cb = c[2];
            }
        }
        r += L.cr * cr * L.energy;
        g += L.cg * cg * L.energy;
        b += L.cb * cb * L.energy;
        break;
    }
    default:
        break;
    }
}

__device__ void phase_vertex(const FrameParams& P, unsigned char* smem_raw) {
    VertexSmem& sm = *reinterpret_cast<VertexSmem*>(smem_raw);
    for (;;) {
        const uint32_t item = P.vitem_begin + next_item(P.ctl, 1, &sm.item);
        if (item >= P.vitem_end) break;
        const uint32_t s = P.vitem_seg[item];
        const DevSeg seg = P.segs[s];
        if (seg.flags & SEG_SKIP) continue;
        const DevPrep& pr = P.preps[seg.inst];
        if (pr.culled) continue;
        const DevJob& J = P.jobs[seg.job];
        const DevInst& in = P.insts[seg.inst];
        const bool lit = seg.flags & SEG_LIT;
        // stage the model's matrices and light list
        for (uint32_t k = threadIdx.x; k < 48; k += blockDim.x) {
            if (k < 16) sm.mvp[k] = pr.mvp[k];
            else if (k < 32) sm.M[k - 16] = pr.M[k - 16];
            else sm.dirrot[k - 32] = pr.dirrot[k - 32];
        }
        const uint32_t nl = lit ? min(in.light_cnt, (uint32_t)kMaxLights) : 0u;
        for (uint32_t k = threadIdx.x; k < nl; k += blockDim.x) {
            const DevLight& L = J.lights[P.inst_light_idx[in.light_off + k]];
            const float4 w = P.inst_light_work[in.light_off + k];
            SLight& d = sm.lights[k];
            d.type = L.type;
            d.skip = (L.type == T3D_LIGHT_POINT && w.w != 0.0f) ? 1 : 0;
            d.cnt[0] = L.cnt[0]; d.cnt[1] = L.cnt[1]; d.cnt[2] = L.cnt[2];
            d.cell_first = L.cell_first;
            d.cr = L.color[0]; d.cg = L.color[1]; d.cb = L.color[2];
            d.energy = L.energy; d.range = L.range; d.range2 = L.range2;
            d.wx = w.x; d.wy = w.y; d.wz = w.z;
            d.ax = L.amb[0]; d.ay = L.amb[1]; d.az = L.amb[2];
            d.fx = L.fwd[0]; d.fy = L.fwd[1]; d.fz = L.fwd[2];
            for (int c = 0; c < 3; c++) {
                d.vmin[c] = L.vmin[c]; d.vmax[c] = L.vmax[c]; d.cell[c] = L.cell[c];
                d.off[c] = L.offset[c]; d.bias[c] = L.bias[c];
            }
        }
        __syncthreads();
        const m4 mvp = load16(sm.mvp);
        const m4 M = load16(sm.M);
        const m4 dirrot = load16(sm.dirrot);
        const JobCam& cam = J.cam;
        const float nearp = cam.near_;
        (void)nearp;
        const float W = cam.W, H = cam.H, halfW = cam.halfW, halfH = cam.halfH;
        const bool persp = cam.perspective != 0, pc = cam.persp_correct != 0;
        const bool want_depth = cam.render_depth || cam.fog_on;
        const uint32_t vbase = J.meshes[seg.mesh].vbase;
        const uint32_t v0 = P.vitem_chunk[item] * P.vchunk;
        const uint32_t v1 = min(seg.vcount, v0 + P.vchunk);
        for (uint32_t lv = v0 + threadIdx.x; lv < v1; lv += blockDim.x) {
            const uint32_t gv = vbase + seg.vmin + lv;
            const float4 a = J.va[gv];
            const float4 b = J.vb[gv];
            const f3 vert = mk3(a.x, a.y, a.z);
            // MultVecW (model.go:808-811)
            const float X = mvp.m[0][0] * vert.x + mvp.m[1][0] * vert.y + mvp.m[2][0] * vert.z + mvp.m[3][0];
            const float Y = mvp.m[0][1] * vert.x + mvp.m[1][1] * vert.y + mvp.m[2][1] * vert.z + mvp.m[3][1];
            const float Z = mvp.m[0][2] * vert.x + mvp.m[1][2] * vert.y + mvp.m[2][2] * vert.z + mvp.m[3][2];
            const float Wc = mvp.m[0][3] * vert.x + mvp.m[1][3] * vert.y + mvp.m[2][3] * vert.z + mvp.m[3][3];
            // cull record (model.go:862-873)
            float w1 = Wc;
            if (w1 < 0.0f) w1 = 0.000001f;
            const float cx = X / w1, cy = Y / w1;
            // emit (camera.go:1655-1742)
            float w = Wc;
            if (!persp) w = 1.0f;
            if (w < 0.0f) w = 0.001f;
            const float dx = (X / w) * W + halfW;
            const float dy = (Y / -w) * H + halfH;
            const float U = b.z, Vv = b.w;
            float uvU, uvV;
            if (pc) { uvU = (U / w) * seg.tex_w; uvV = ((1.0f - Vv) / w) * seg.tex_h; }
            else { uvU = U * seg.tex_w; uvV = (1.0f - Vv) * seg.tex_h; }
            float cr, cg, cb, ca;
            if (seg.flags & SEG_COLORS) {
                const float4 c = J.vc[gv];
                cr = c.x * seg.mp[0]; cg = c.y * seg.mp[1]; cb = c.z * seg.mp[2]; ca = c.w * seg.mp[3];
            } else {
                cr = seg.mp[0]; cg = seg.mp[1]; cb = seg.mp[2]; ca = seg.mp[3];
            }
            if (lit) {
                const f3 vnrm = mk3(a.w, b.x, b.y);
                float lr = 0.0f, lg = 0.0f, lb = 0.0f;
                for (uint32_t k = 0; k < nl; k++) {
                    const SLight& L = sm.lights[k];
                    if (L.skip) continue;
                    light_vertex(L, seg.flags, vert, vnrm, M, dirrot, J.cells, lr, lg, lb);
                }
                cr *= lr; cg *= lg; cb *= lb;
            }
            float depth = 0.0f;
            if (want_depth) {  // camera.go:1744-1812
                depth = (Z + cam.margin) / cam.spread;
                if (depth < 0.0f) depth = 0.0f;
                else if (depth > 1.0f) depth = 1.0f;
                if (!cam.render_depth) {
                    const float fd = cam.fog_range[0] + ((cam.fog_range[1] - cam.fog_range[0]) * 1.0f - depth);
                    if (cam.fog_mode == T3D_FOG_ADD) {
                        cr += cam.fog_color[0] * fd; cg += cam.fog_color[1] * fd; cb += cam.fog_color[2] * fd;
                    } else if (cam.fog_mode == T3D_FOG_SUB) {
                        cr *= cam.fog_color[0] * fd; cg *= cam.fog_color[1] * fd; cb *= cam.fog_color[2] * fd;
                    }
                }
            }
            const uint32_t o = seg.vscratch + lv;
            P.vcull[o] = make_float4(cx, cy, Z, depth);
            P.vxyuv[o] = make_float4(dx, dy, uvU, uvV);
            P.vrgba[o] = make_float4(cr, cg, cb, ca);
        }
    }
}

// --------------------------------------------------------- P2 .. P5 ----
struct TileSmem {
    uint32_t item, nvis, warp_tot[kMaxWarps], scan_tmp[kMaxWarps];
    float wmin[kMaxWarps], wmax[kMaxWarps];
    uint32_t bins_walk[kBins];     // per-bin counts / bases in walk order
    uint32_t whist[kMaxWarps * kBins];
    // followed by: uint16 lidx[tile], float depth[tile], uint16 bin[tile]
};

__device__ __forceinline__ uint16_t* tile_lidx(unsigned char* smem) { return (uint16_t*)(smem + sizeof(TileSmem)); }
__device__ __forceinline__ float* tile_depth(unsigned char* smem, uint32_t tile) {
    return (float*)(smem + sizeof(TileSmem) + 2 * (size_t)tile);
}
__device__ __forceinline__ uint16_t* tile_bin(unsigned char* smem, uint32_t tile) {
    return (uint16_t*)(smem + sizeof(TileSmem) + 6 * (size_t)tile);
}

__device__ __forceinline__ uint32_t walk_pos(uint32_t b, uint32_t sort_mode) {
    return sort_mode == T3D_SORT_BACK_TO_FRONT ? (uint32_t)(kBins - 1) - b : b;
}

// sortingTriangleBucket.Sort bin (sortingTriangles.go:42-58)
__device__ __forceinline__ uint32_t bin_of(float d, float mn, float range, uint32_t sort_mode) {
    if (sort_mode == T3D_SORT_NONE) return 0u;
    float x = (d - mn) / range * (float)kBins;
    float t = clampf(x, 0.0f, (float)(kBins - 1));
    return (uint32_t)(int)t;
}
__device__ __forceinline__ float range_of(float mn, float mx) {
    float r = mx - mn;
    if (r == 0.0f) r += 0.001f;
    return r;
}

// In-place exclusive scan of bins_walk[0..kBins) by the whole block.
__device__ void scan_bins(TileSmem& sm) {
    __syncthreads();
    const uint32_t per = (kBins + blockDim.x - 1) / blockDim.x;
    const uint32_t lo = threadIdx.x * per, hi = min((uint32_t)kBins, lo + per);
    uint32_t sum = 0;
    for (uint32_t i = lo; i < hi; i++) sum += sm.bins_walk[i];
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t incl = sum;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (uint32_t)o) incl += v;
    }
    if (lane == 31) sm.scan_tmp[wid] = incl;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t run = 0;
        for (uint32_t w = 0; w < blockDim.x / 32; w++) { uint32_t t = sm.scan_tmp[w]; sm.scan_tmp[w] = run; run += t; }
    }
    __syncthreads();
    uint32_t run = sm.scan_tmp[wid] + incl - sum;
    for (uint32_t i = lo; i < hi; i++) { uint32_t t = sm.bins_walk[i]; sm.bins_walk[i] = run; run += t; }
    __syncthreads();
}

// Stable placement of a tile's n visible triangles (in triangle order in smem)
// and their emission. bins_walk holds, in walk order, the first output
// position of each bin for this tile (within the segment).
__device__ void rank_and_emit(const FrameParams& P, const DevSeg& seg, const DevJob& J, unsigned char* smem,
                              uint32_t tile_tris, uint32_t t0, uint32_t n, uint32_t sort_mode) {
    TileSmem& sm = *reinterpret_cast<TileSmem*>(smem);
    const uint16_t* lidx = tile_lidx(smem);
    const uint16_t* bins = tile_bin(smem, tile_tris);
    const uint32_t nw = blockDim.x >> 5, wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t chunk = (n + nw - 1) / nw;
    const uint32_t lo = min(n, wid * chunk), hi = min(n, lo + chunk);
    for (uint32_t i = threadIdx.x; i < nw * kBins; i += blockDim.x) sm.whist[i] = 0u;
    __syncthreads();
    for (uint32_t j = lo + lane; j < hi; j += 32) atomicAdd(&sm.whist[wid * kBins + bins[j]], 1u);
    __syncthreads();
    for (uint32_t b = threadIdx.x; b < kBins; b += blockDim.x) {
        uint32_t run = sm.bins_walk[walk_pos(b, sort_mode)];
        for (uint32_t w = 0; w < nw; w++) {
            uint32_t t = sm.whist[w * kBins + b];
            sm.whist[w * kBins + b] = run;
            run += t;
        }
    }
    __syncthreads();
    const uint32_t mesh_tbase = J.meshes[seg.mesh].tbase;
    const uint32_t lt = (1u << lane) - 1u;
    for (uint32_t j0 = lo; j0 < hi; j0 += 32) {
        const uint32_t j = j0 + lane;
        const bool active = j < hi;
        const uint32_t mask = __ballot_sync(0xffffffffu, active);
        uint32_t b = 0, peers = 0, pos = 0;
        if (active) {
            b = bins[j];
            peers = __match_any_sync(mask, b);
            pos = sm.whist[wid * kBins + b] + __popc(peers & lt);
        }
        __syncwarp();
        if (active && lane == (uint32_t)(__ffs(peers) - 1)) sm.whist[wid * kBins + b] += __popc(peers);
        __syncwarp();
        if (active) {
            const uint32_t t = t0 + lidx[j];  // mesh-absolute triangle
            const uint32_t* ip = J.idx + 3 * (size_t)(mesh_tbase + t);
            const size_t slot = (size_t)seg.out_base + pos;
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const uint32_t o = seg.vscratch + (ip[c] - seg.vmin);
                P.out_xyuv[3 * slot + c] = P.vxyuv[o];
                P.out_rgba[3 * slot + c] = P.vrgba[o];
                P.out_depth[3 * slot + c] = P.vcull[o].w;
            }
        }
    }
}

__device__ void phase_triangles(const FrameParams& P, unsigned char* smem) {
    TileSmem& sm = *reinterpret_cast<TileSmem*>(smem);
    const uint32_t T = P.tile_tris;
    uint16_t* lidx = tile_lidx(smem);
    float* dep = tile_depth(smem, T);
    uint16_t* bins = tile_bin(smem, T);
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (;;) {
        const uint32_t item = P.tile_begin + next_item(P.ctl, 2, &sm.item);
        if (item >= P.tile_end) break;
        const uint32_t s = P.tile_seg[item];
        const DevSeg seg = P.segs[s];
        const uint32_t tile = item - seg.tile_first;
        const bool multi = seg.flags & SEG_MULTI;
        const uint32_t mt = seg.mt_first + tile;
        const DevPrep& pr = P.preps[seg.inst];
        if ((seg.flags & SEG_SKIP) || pr.culled) {
            if (multi && threadIdx.x == 0) P.tile_count[mt] = 0u;
            continue;
        }
        const DevJob& J = P.jobs[seg.job];
        const JobCam& cam = J.cam;
        const float nearp = cam.near_, farp = cam.far_;
        const bool backface = seg.flags & SEG_BACKFACE;
        const f3 ic = mk3(pr.invcam[0], pr.invcam[1], pr.invcam[2]);
        const DevMesh me = J.meshes[seg.mesh];
        const uint32_t t0 = seg.tri_start + tile * T;
        const uint32_t t1 = min(seg.tri_start + seg.tri_count, t0 + T);
        if (threadIdx.x == 0) sm.nvis = 0u;
        float lmin = 3.402823466e38f, lmax = 0.0f;
        __syncthreads();
        for (uint32_t base = t0; base < t1; base += blockDim.x) {
            const uint32_t t = base + threadIdx.x;
            bool vis = false;
            float depth = 0.0f;
            if (t < t1) {
                const uint32_t* ip = J.idx + 3 * (size_t)(me.tbase + t);
                const uint32_t i0 = ip[0], i1 = ip[1], i2 = ip[2];
                const float4 c0 = P.vcull[seg.vscratch + (i0 - seg.vmin)];
                const float4 c1 = P.vcull[seg.vscratch + (i1 - seg.vmin)];
                const float4 c2 = P.vcull[seg.vscratch + (i2 - seg.vmin)];
                // model.go:857-925
                const bool inb = (c0.z + 1.0f >= nearp && c0.z < farp) || (c1.z + 1.0f >= nearp && c1.z < farp) ||
                                 (c2.z + 1.0f >= nearp && c2.z < farp);
                vis = inb;
                if (vis && ((c0.x < -0.5f && c1.x < -0.5f && c2.x < -0.5f) || (c0.x > 0.5f && c1.x > 0.5f && c2.x > 0.5f) ||
                            (c0.y < -0.5f && c1.y < -0.5f && c2.y < -0.5f) || (c0.y > 0.5f && c1.y > 0.5f && c2.y > 0.5f)))
                    vis = false;
                if (vis && backface) {
                    const float n0x = c0.x - c1.x, n0y = c0.y - c1.y;
                    const float n1x = c1.x - c2.x, n1y = c1.y - c2.y;
                    const float nor = (n0x * n1y) - (n1x * n0y);
                    if (nor < 0.0f) vis = false;
                }
                if (vis) {  // tri.Center (mesh.go:1980-1982) and the depth key (model.go:950-953)
                    const float4 pa = J.va[me.vbase + i0];
                    const float4 pb = J.va[me.vbase + i1];
                    const float4 pc = J.va[me.vbase + i2];
                    const float cxx = (pa.x + pb.x + pc.x) / 3.0f;
                    const float cyy = (pa.y + pb.y + pc.y) / 3.0f;
                    const float czz = (pa.z + pb.z + pc.z) / 3.0f;
                    const float ddx = ic.x - cxx, ddy = ic.y - cyy, ddz = ic.z - czz;
                    depth = ddx * ddx + ddy * ddy + ddz * ddz;
                    if (isnan(depth) || isinf(depth)) vis = false;
                }
            }
            // stable compaction in triangle order
            const uint32_t bal = __ballot_sync(0xffffffffu, vis);
            if (lane == 0) sm.warp_tot[wid] = __popc(bal);
            __syncthreads();
            if (threadIdx.x == 0) {
                uint32_t run = sm.nvis;
                for (uint32_t w = 0; w < nw; w++) { uint32_t c = sm.warp_tot[w]; sm.scan_tmp[w] = run; run += c; }
                sm.nvis = run;
            }
            __syncthreads();
            if (vis) {
                const uint32_t p = sm.scan_tmp[wid] + __popc(bal & ((1u << lane) - 1u));
                lidx[p] = (uint16_t)(t - t0);
                dep[p] = depth;
                lmin = fminf(lmin, depth);
                lmax = fmaxf(lmax, depth);
            }
        }
        // block min / max of the visible depths
        for (int o = 16; o > 0; o >>= 1) {
            lmin = fminf(lmin, __shfl_xor_sync(0xffffffffu, lmin, o));
            lmax = fmaxf(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
        }
        if (lane == 0) { sm.wmin[wid] = lmin; sm.wmax[wid] = lmax; }
        __syncthreads();
        const uint32_t n = sm.nvis;
        float mn = sm.wmin[0], mx = sm.wmax[0];
        for (uint32_t w = 1; w < nw; w++) { mn = fminf(mn, sm.wmin[w]); mx = fmaxf(mx, sm.wmax[w]); }
        const uint32_t sort_mode = seg_sort_mode(seg.flags);
        if (!multi) {
            if (n > 0) {
                const float range = range_of(mn, mx);
                for (uint32_t b = threadIdx.x; b < kBins; b += blockDim.x) sm.bins_walk[b] = 0u;
                __syncthreads();
                for (uint32_t j = threadIdx.x; j < n; j += blockDim.x) {
                    const uint32_t b = bin_of(dep[j], mn, range, sort_mode);
                    bins[j] = (uint16_t)b;
                    atomicAdd(&sm.bins_walk[walk_pos(b, sort_mode)], 1u);
                }
                scan_bins(sm);
                rank_and_emit(P, seg, J, smem, T, t0, n, sort_mode);
            }
            if (threadIdx.x == 0) {
                P.seg_count[s] = n;
                if (n) atomicAdd(&P.accum[0], (unsigned long long)n);
            }
        } else {
            uint32_t* gi = P.vis_idx + (size_t)mt * T;
            float* gd = P.vis_depth + (size_t)mt * T;
            for (uint32_t j = threadIdx.x; j < n; j += blockDim.x) { gi[j] = lidx[j]; gd[j] = dep[j]; }
            if (threadIdx.x == 0) {
                P.tile_count[mt] = n;
                if (n > 0) {
                    atomicMin(&P.seg_minmax[2 * s], __float_as_uint(mn));
                    atomicMax(&P.seg_minmax[2 * s + 1], __float_as_uint(mx));
                    atomicAdd(&P.seg_count[s], n);
                    atomicAdd(&P.accum[0], (unsigned long long)n);
                }
            }
        }
        __syncthreads();
    }
}

__device__ void phase_hist(const FrameParams& P, unsigned char* smem) {
    TileSmem& sm = *reinterpret_cast<TileSmem*>(smem);
    const uint32_t T = P.tile_tris;
    for (;;) {
        const uint32_t i = P.mt_tile_begin + next_item(P.ctl, 3, &sm.item);
        if (i >= P.mt_tile_end) break;
        const uint32_t g = P.mt_tiles[i];
        const uint32_t s = P.tile_seg[g];
        const DevSeg seg = P.segs[s];
        const uint32_t n = __ldcg(&P.tile_count[i]);
        for (uint32_t b = threadIdx.x; b < kBins; b += blockDim.x) sm.bins_walk[b] = 0u;
        __syncthreads();
        if (n > 0) {
            const float mn = __uint_as_float(__ldcg(&P.seg_minmax[2 * s]));
            const float mx = __uint_as_float(__ldcg(&P.seg_minmax[2 * s + 1]));
            const float range = range_of(mn, mx);
            const uint32_t sort_mode = seg_sort_mode(seg.flags);
            const float* gd = P.vis_depth + (size_t)i * T;
            for (uint32_t j = threadIdx.x; j < n; j += blockDim.x)
                atomicAdd(&sm.bins_walk[bin_of(__ldcg(&gd[j]), mn, range, sort_mode)], 1u);
        }
        __syncthreads();
        for (uint32_t b = threadIdx.x; b < kBins; b += blockDim.x) P.tile_hist[(size_t)i * kBins + b] = sm.bins_walk[b];
    }
}

__device__ void phase_scan(const FrameParams& P, unsigned char* smem) {
    TileSmem& sm = *reinterpret_cast<TileSmem*>(smem);
    for (;;) {
        const uint32_t k = P.mt_seg_begin + next_item(P.ctl, 4, &sm.item);
        if (k >= P.mt_seg_end) break;
        const uint32_t s = P.mt_segs[k];
        const DevSeg seg = P.segs[s];
        const uint32_t sort_mode = seg_sort_mode(seg.flags);
        for (uint32_t b = threadIdx.x; b < kBins; b += blockDim.x) {
            uint32_t tot = 0;
            for (uint32_t t = 0; t < seg.ntiles; t++) tot += __ldcg(&P.tile_hist[(size_t)(seg.mt_first + t) * kBins + b]);
            sm.bins_walk[walk_pos(b, sort_mode)] = tot;
        }
        scan_bins(sm);
        for (uint32_t b = threadIdx.x; b < kBins; b += blockDim.x) {
            uint32_t run = sm.bins_walk[walk_pos(b, sort_mode)];
            for (uint32_t t = 0; t < seg.ntiles; t++) {
                uint32_t* h = &P.tile_hist[(size_t)(seg.mt_first + t) * kBins + b];
                uint32_t c = __ldcg(h);
                *h = run;
                run += c;
            }
        }
    }
}

__device__ void phase_emit_multi(const FrameParams& P, unsigned char* smem) {
    TileSmem& sm = *reinterpret_cast<TileSmem*>(smem);
    const uint32_t T = P.tile_tris;
    uint16_t* lidx = tile_lidx(smem);
    uint16_t* bins = tile_bin(smem, T);
    for (;;) {
        const uint32_t i = P.mt_tile_begin + next_item(P.ctl, 5, &sm.item);
        if (i >= P.mt_tile_end) break;
        const uint32_t g = P.mt_tiles[i];
        const uint32_t s = P.tile_seg[g];
        const DevSeg seg = P.segs[s];
        const uint32_t n = __ldcg(&P.tile_count[i]);
        if (n == 0) continue;
        const DevJob& J = P.jobs[seg.job];
        const float mn = __uint_as_float(__ldcg(&P.seg_minmax[2 * s]));
        const float mx = __uint_as_float(__ldcg(&P.seg_minmax[2 * s + 1]));
        const float range = range_of(mn, mx);
        const uint32_t sort_mode = seg_sort_mode(seg.flags);
        const uint32_t* gi = P.vis_idx + (size_t)i * T;
        const float* gd = P.vis_depth + (size_t)i * T;
        for (uint32_t j = threadIdx.x; j < n; j += blockDim.x) {
            lidx[j] = (uint16_t)__ldcg(&gi[j]);
            bins[j] = (uint16_t)bin_of(__ldcg(&gd[j]), mn, range, sort_mode);
        }
        for (uint32_t b = threadIdx.x; b < kBins; b += blockDim.x)
            sm.bins_walk[walk_pos(b, sort_mode)] = __ldcg(&P.tile_hist[(size_t)i * kBins + b]);
        __syncthreads();
        const uint32_t tile = g - seg.tile_first;
        rank_and_emit(P, seg, J, smem, T, seg.tri_start + tile * T, n, sort_mode);
    }
}

__global__ void __launch_bounds__(512) t3d_frame_kernel(const FrameParams P) {
    extern __shared__ __align__(16) unsigned char smem[];
    phase_prep(P);
    if (!grid_barrier(P.ctl)) return;
    phase_vertex(P, smem);
    if (!grid_barrier(P.ctl)) return;
    phase_triangles(P, smem);
    if (!P.has_multi) return;
    if (!grid_barrier(P.ctl)) return;
    phase_hist(P, smem);
    if (!grid_barrier(P.ctl)) return;
    phase_scan(P, smem);
    if (!grid_barrier(P.ctl)) return;
    phase_emit_multi(P, smem);
}

size_t tile_smem_bytes(uint32_t tile_tris) { return sizeof(TileSmem) + 8 * (size_t)tile_tris; }
size_t vertex_smem_bytes() { return sizeof(VertexSmem); }

}  // namespace t3d

// Launch entry used by the runtime (same translation-unit linkage).
extern "C" const void* t3d_frame_kernel_ptr() { return (const void*)&t3d::t3d_frame_kernel; }
extern "C" size_t t3d_frame_smem_bytes(uint32_t tile_tris) {
    size_t a = t3d::tile_smem_bytes(tile_tris), b = t3d::vertex_smem_bytes();
    return a > b ? a : b;
}
