// t3d_kernels.cu -- the GB300 vertex stage: persistent kernels, one per phase.
//
//   prep            per (job, model): Node.Transform (+ animation step), MVP,
//                   model-space camera, SphereInFrustum, light beginModel.
//   vertex          per-vertex route only, per (segment, vertex chunk): MultVecW,
//                   the cull record, lighting and the emitted corner attributes.
//   triangles       per tile (a meshlet, or a run of the per-vertex route): near/far,
//                   +-0.5 and backface rejection, the depth key, a stable in-tile
//                   compaction (per-vertex single-tile segments: the whole sort + emit).
//   histogram, scan, rank + emit: tile histograms and stable ranking, cross-tile
//                   bin scan, emission of the corners in output order.
// Each phase is a persistent kernel over its own atomic work queue (uneven models
// balance across SMs), compiled with its own register budget and shared memory;
// the launch boundary orders the phases. The same phases also run as one
// cooperative launch with a bounded software grid barrier between them.
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
__device__ __forceinline__ uint32_t spin_limit(const FrameParams& P) { return P.spin_limit ? P.spin_limit : kSpinLimit; }
__device__ bool grid_barrier(Ctl* ctl, uint32_t limit) {
    __threadfence();
    __syncthreads();
    if (gridDim.x == 1) return vload(&ctl->err) == 0;  // one block: the block barrier is the grid barrier
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
                if (++spins > limit) {
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

// ---- bulk copies into shared memory (cp.async.bulk completing on an mbarrier) ----
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long* b, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
// orders this thread's earlier shared-memory accesses before later bulk copies into the same bytes
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* b, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes) : "memory");
}
// global -> shared, `bytes` a multiple of 16, both addresses 16-byte aligned
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, unsigned long long* b) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(b)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* b, uint32_t parity) {
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok) : "r"(smem_u32(b)), "r"(parity) : "memory");
    return ok != 0;
}
__device__ __forceinline__ void mbar_inval(unsigned long long* b) {
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(b)) : "memory");
}
// Waits for phase `parity` of barrier b with a bounded number of polls. On
// timeout it records ERR_COPY_TIMEOUT and waits once more, with the default
// bound, for the copy in flight, so that no copy lands in shared memory after
// the block has moved on.
__device__ __noinline__ bool mbar_wait(unsigned long long* b, uint32_t parity, Ctl* ctl, uint32_t limit) {
    for (uint32_t i = 0; i < limit; i++)
        if (mbar_try_wait(b, parity)) return true;
    atomicCAS(&ctl->err, 0, ERR_COPY_TIMEOUT);
    for (uint32_t i = 0; i < kSpinLimit; i++)
        if (mbar_try_wait(b, parity)) break;
    return false;
}

// Loads of per-vertex records. The records are written only in the vertex
// phase, before the first grid barrier, and every read comes after it; no SM
// can hold a stale L1 line of them (L1 starts empty each launch), so the reads
// may use L1, where the corners of one tile find their shared vertices.
#ifndef T3D_REC_L1
#define T3D_REC_L1 1
#endif
template <typename V>
__device__ __forceinline__ V rec_load(const V* p) {
#if T3D_REC_L1
    return *p;
#else
    return __ldcg(p);
#endif
}

// Asynchronous L2 prefetch of a byte range (cp.async.bulk.prefetch.L2): the
// start is rounded down and the end up to 16 bytes (the pools carry slack for
// that), and ranges above kPrefetchMax are left to demand loads.
constexpr uint32_t kPrefetchMax = 256u << 10;

__device__ __forceinline__ void l2_prefetch(const void* p, size_t bytes) {
    const uintptr_t a = (uintptr_t)p & ~(uintptr_t)15;
    const uintptr_t e = ((uintptr_t)p + bytes + 15) & ~(uintptr_t)15;
    if (e > a && e - a <= kPrefetchMax)
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(a), "r"((uint32_t)(e - a)) : "memory");
}

// The k-th meshlet tile the histogram and emit phases take: the k-th entry of the list of
// tiles with visible triangles, or the k-th tile of the range when there is no list.
__device__ __forceinline__ uint32_t mesh_tile_at(const FrameParams& P, uint32_t k) {
    return P.live_tiles ? __ldcg(&P.live_tiles[P.mt_mesh_begin + k]) : P.mt_mesh_begin + k;
}
__device__ __forceinline__ uint32_t mesh_tile_count(const FrameParams& P) {
    return P.live_tiles ? vload(&P.ctl->live) : P.mt_mesh_end - P.mt_mesh_begin;
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
// Model.onTransformUpdate derives from the transform (model.go:142-182); a
// skinned model's sphere is centred on its position (model.go:158-161).
__device__ bool model_in_frustum(const JobCam& c, const m4& M, const DevMesh& me, bool skinned) {
    f3 position, scale;
    m4 rotation;
    decompose(M, position, scale, rotation);
    f3 center = mk3(0.0f, 0.0f, 0.0f);
    if (!skinned)
        center = mk3((me.dmax[0] + me.dmin[0]) / 2.0f, (me.dmax[1] + me.dmin[1]) / 2.0f, (me.dmax[2] + me.dmin[2]) / 2.0f);
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

// One light of the model's list as the emit loop reads it (56 bytes).
// x, y, z: point = model-space workingPosition, ambient = result,
// directional = workingForward. Volume geometry is read from `vol`.
struct SLight {
    int32_t type, skip;
    float cr, cg, cb, energy, range, range2;
    float x, y, z;
    const DevLight* vol;
};
static_assert(sizeof(SLight) == 56, "staged light records are 56 bytes");
// Bytes of a bulk copy of n staged lights (rounded up to 16; the regions hold kMaxLights records).
__device__ __forceinline__ uint32_t slight_copy_bytes(uint32_t n) { return (56u * n + 15u) & ~15u; }

// Model.ProcessVertices' light set-up for one light of an unskinned model as the
// vertex loop reads it: ILight.beginModel (light.go:175-189, :326-330) and the
// model-level point-light range skip (camera.go:1625-1629). r = the model's
// Decompose(Inverted(M)) rows, M its transform, maxspan Mesh.Dimensions.MaxSpan.
// (stage_model does the same per work item for the record path.)
__device__ __forceinline__ SLight light_for_model(const DevLight& L, const float* r, const float* M, float maxspan) {
    float4 w = make_float4(0.f, 0.f, 0.f, 0.f);
    if (L.type == T3D_LIGHT_POINT) {
        const f3 lp = mk3(L.wpos[0], L.wpos[1], L.wpos[2]);
        // Decompose(Inverted(M)): r.MultVec(lp) + p * (1/s)
        const f3 q = mk3(r[0] * lp.x + r[4] * lp.y + r[8] * lp.z + r[12], r[1] * lp.x + r[5] * lp.y + r[9] * lp.z + r[13],
                         r[2] * lp.x + r[6] * lp.y + r[10] * lp.z + r[14]);
        w.x = q.x + r[3]; w.y = q.y + r[7]; w.z = q.z + r[11];
        if (L.range > 0.0f) {
            const float dist = maxspan + L.range;
            if (dist2(mk3(M[12], M[13], M[14]), lp) > dist * dist) w.w = 1.0f;
        }
    }
    SLight d;
    d.type = L.type;
    d.skip = (L.type == T3D_LIGHT_POINT && w.w != 0.0f) ? 1 : 0;
    d.cr = L.color[0]; d.cg = L.color[1]; d.cb = L.color[2];
    d.energy = L.energy; d.range = L.range; d.range2 = L.range2;
    if (L.type == T3D_LIGHT_POINT) { d.x = w.x; d.y = w.y; d.z = w.z; }
    else if (L.type == T3D_LIGHT_AMBIENT) { d.x = L.amb[0]; d.y = L.amb[1]; d.z = L.amb[2]; }
    else { d.x = L.fwd[0]; d.y = L.fwd[1]; d.z = L.fwd[2]; }
    d.vol = &L;
    return d;
}

template <int kV>
__device__ __noinline__ void phase_prep(const FrameParams& P) {
    const uint32_t n = P.inst_end - P.inst_begin;
    const uint32_t stride = gridDim.x * blockDim.x;
    {  // the scan chunks' counts start from zero (the histogram phase adds to them)
        uint4* z = reinterpret_cast<uint4*>(P.chunk_hist + (size_t)P.chunk_zero_begin * kBins);
        const size_t nz = (size_t)(P.chunk_zero_end - P.chunk_zero_begin) * (kBins / 4);
        for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < nz; q += stride)
            z[q] = make_uint4(0u, 0u, 0u, 0u);
    }
    // model k runs on block k % grid: the serial per-model chains spread over every SM
    for (uint32_t k = blockIdx.x + gridDim.x * threadIdx.x; k < n; k += stride) {
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
        const bool skinned = md->flags & MOD_SKINNED;
        m4 vp = load16(cam.vp);
        // skinned vertices are already in world space: VP alone, and the depth
        // key is measured from the world camera position (model.go:760-770, :941-946)
        store16(skinned ? vp : mult(M, vp), pr.mvp);  // model.go:695
        store16(M, pr.M);
        InvFrame inv = inv_frame(M);   // model.go:629
        f3 ic = skinned ? mk3(cam.pos[0], cam.pos[1], cam.pos[2])
                        : to_model_space(inv, mk3(cam.pos[0], cam.pos[1], cam.pos[2]));  // model.go:630
        pr.invcam[0] = ic.x; pr.invcam[1] = ic.y; pr.invcam[2] = ic.z; pr.invcam[3] = 0.0f;
        for (int r = 0; r < 4; r++)
            for (int c = 0; c < 3; c++) pr.inv_r[4 * r + c] = inv.r.m[r][c];
        const f3 off = hmul3(inv.p, inv.inv_s);
        pr.inv_r[3] = off.x; pr.inv_r[7] = off.y; pr.inv_r[11] = off.z; pr.inv_r[15] = 0.0f;
        store16(transposed(inverted(WR)), pr.dirrot);  // light.go:326-330
        bool culled = (md->flags & MOD_FRUSTUM) && !model_in_frustum(cam, M, me, skinned);
        pr.culled = culled ? 1u : 0u;
        if (culled) {
            atomicAdd(&P.ctl->culled, 1u);
        } else {
            atomicAdd(&P.ctl->bytes, (unsigned long long)in.bytes);
            atomicAdd(&P.accum[1], (unsigned long long)in.bytes);
            if (P.job_bytes) atomicAdd(&P.job_bytes[in.job], (unsigned long long)in.bytes);
        }
        // Mesh.Dimensions.MaxSpan for the model-level point-light skip (camera.go:1625-1629)
        pr.maxspan = mag3(mk3(me.dmax[0] - me.dmin[0], me.dmax[1] - me.dmin[1], me.dmax[2] - me.dmin[2]));
    }
    // meshlet frames: each model's light list as its render pairs' vertex loops read it, staged
    // once, by one warp per model of this block (the models k = blockIdx.x + gridDim.x * t whose
    // prep records this block's threads just wrote): lane l stages lights l, l + 32, ..., and
    // the kept ones (not skipped by the model-level range test) go out in list order
    if ((kV & 1) && P.inst_lights) {
        __syncthreads();
        const uint32_t lane = threadIdx.x & 31, lt = (1u << lane) - 1u;
        for (uint32_t t = threadIdx.x >> 5;; t += blockDim.x >> 5) {
            const uint32_t k = blockIdx.x + gridDim.x * t;
            if (k >= n) break;
            const uint32_t i = P.inst_begin + k;
            const DevInst in = P.insts[i];
            DevPrep& pr = P.preps[i];
            const DevJob& J = P.jobs[in.job];
            if (pr.culled || (J.models[in.model].flags & MOD_SKINNED)) continue;
            SLight* out = reinterpret_cast<SLight*>(P.inst_lights) + (size_t)i * kMaxLights;
            const uint32_t nl = min(in.light_cnt, (uint32_t)kMaxLights);
            uint32_t o = 0;
            for (uint32_t k0 = 0; k0 < nl; k0 += 32) {
                SLight d;
                bool keep = false;
                if (k0 + lane < nl) {
                    d = light_for_model(J.lights[P.inst_light_idx[in.light_off + k0 + lane]], pr.inv_r, pr.M, pr.maxspan);
                    keep = !d.skip;
                }
                const uint32_t bal = __ballot_sync(0xffffffffu, keep);
                if (keep) out[o + __popc(bal & lt)] = d;
                o += __popc(bal);
            }
            if (lane == 0) pr.nl = o;
        }
    }
    const uint32_t ns = P.seg_end - P.seg_begin;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < ns; k += stride) {
        const uint32_t s = P.seg_begin + k;
        P.seg_minmax[2 * s] = 0xFFFFFFFFu;
        P.seg_minmax[2 * s + 1] = 0u;
        P.seg_count[s] = 0u;
    }
}

// LightVolume.convertToXYZIndices + getLightCell (light.go:717-741, :1267-1272)
__device__ __forceinline__ int lv_index(float v) {
    if (!(v > -2147483648.0f && v < 2147483647.0f)) return -1;
    return (int)v;
}
__device__ bool lv_cell(const DevLight& L, f3 p, uint32_t& idx) {
    float csx = L.cell[0], csy = L.cell[1], csz = L.cell[2];
    int x = lv_index(roundf(((p.x - L.offset[0] - L.vmin[0] - (csx / 2.0f)) / csx)));
    int y = lv_index(roundf(((p.y - L.offset[1] - L.vmin[1] - (csy / 2.0f)) / csy)));
    int z = lv_index(roundf(((p.z - L.offset[2] - L.vmin[2] - (csz / 2.0f)) / csz)));
    if (x < 0 || y < 0 || z < 0 || x >= L.cnt[0] || y >= L.cnt[1] || z >= L.cnt[2]) return false;
    idx = (uint32_t)(x + (y * L.cnt[0]) + (z * L.cnt[0] * L.cnt[1]));
    return true;
}

// Matrix4.MultVec with the matrix read from shared memory (row-major 16 floats).
__device__ __forceinline__ f3 mult_vec_s(const float* m, f3 v) {
    return mk3(m[0] * v.x + m[4] * v.y + m[8] * v.z + m[12], m[1] * v.x + m[5] * v.y + m[9] * v.z + m[13],
               m[2] * v.x + m[6] * v.y + m[10] * v.z + m[14]);
}

// What the lights used by light-volume cells need (LightVolumeCell.useLights).
struct NestedSrc {
    const DevLight* lights;   // the job's light table
    const uint32_t* off;      // cell c uses items [off[c], off[c + 1])
    const uint32_t* items;
    const float* inv_r;       // the model's Decompose(Inverted(M)) rows, for point-light positions
};

// A light used by a light-volume cell, lit at the vertex that fell into that cell
// (light.go:652-654): its VertexLight as after its beginModel (light.go:175-189,
// :326-330), without the model-level range skip of the scene's lights. Returns
// the vertex's light sums (r, g, b) with this light added.
__device__ __noinline__ float3 nested_light(const DevLight& N, uint32_t flags, f3 vpos, f3 vnrm, const float* dirrot,
                                            const float* __restrict__ r_, float r, float g, float b) {
    const bool mat = flags & SEG_MAT;
    const uint32_t lmode = seg_light_mode(flags);
    const bool skinned = flags & SEG_SKINNED;
    if (N.type == T3D_LIGHT_AMBIENT) {
        r += N.amb[0]; g += N.amb[1]; b += N.amb[2];
        return make_float3(r, g, b);
    } else if (N.type == T3D_LIGHT_POINT) {
        const f3 lp = mk3(N.wpos[0], N.wpos[1], N.wpos[2]);
        f3 work = lp;
        if (!skinned) {  // the same model-space position as stage_model computes
            const f3 q = mk3(r_[0] * lp.x + r_[4] * lp.y + r_[8] * lp.z + r_[12],
                             r_[1] * lp.x + r_[5] * lp.y + r_[9] * lp.z + r_[13],
                             r_[2] * lp.x + r_[6] * lp.y + r_[10] * lp.z + r_[14]);
            work = mk3(q.x + r_[3], q.y + r_[7], q.z + r_[11]);
        }
        const float distance = dist2(work, vpos);
        if (N.range > 0.0f) {
            if (distance > N.range2) return make_float3(r, g, b);
        } else {
            if (1.0f / distance * N.energy < 0.001f) return make_float3(r, g, b);
        }
        const f3 lightVec = unit3(sub3(work, vpos));
        const f3 n = (mat && lmode == T3D_LIGHTING_FIXED_NORMALS) ? lightVec : vnrm;
        float diffuse = dot3(n, lightVec);
        if (mat && lmode == T3D_LIGHTING_DOUBLE_SIDED) diffuse = fabsf(diffuse);
        if (diffuse > 0.0f) {
            float df = diffuse * (1.0f / (1.0f + (0.1f * distance))) * 2.0f;
            if (N.range2 > 0.0f) df *= clampf((N.range2 - distance) / distance, 0.0f, 1.0f);
            r += N.color[0] * df * N.energy;
            g += N.color[1] * df * N.energy;
            b += N.color[2] * df * N.energy;
        }
    } else if (N.type == T3D_LIGHT_DIRECTIONAL) {
        const f3 fwd = mk3(N.fwd[0], N.fwd[1], N.fwd[2]);
        const f3 normal = (mat && lmode == T3D_LIGHTING_FIXED_NORMALS) ? fwd : skinned ? vnrm : mult_vec_s(dirrot, vnrm);
        float df = dot3(normal, fwd);
        if (mat && lmode == T3D_LIGHTING_DOUBLE_SIDED) df = fabsf(df);
        if (df <= 0.0f) return make_float3(r, g, b);
        r += N.color[0] * df * N.energy;
        g += N.color[1] * df * N.energy;
        b += N.color[2] * df * N.energy;
    }
    return make_float3(r, g, b);
}

// One light's contribution to one vertex (ILight.VertexLight, light.go:115-663).
// M (model transform) and dirrot (workingModelRotation) live in shared memory.
// For a skinned model vpos and vnrm are already in world space (light.go:334-343, :613-620).
template <bool kSkin>
__device__ __forceinline__ void light_vertex(const SLight& L, uint32_t flags, f3 vpos, f3 vnrm, const float* M,
                                             const float* dirrot, const float* __restrict__ cells, const NestedSrc& ns,
                                             float& r, float& g, float& b) {
    const bool mat = flags & SEG_MAT;
    const uint32_t lmode = seg_light_mode(flags);
    switch (L.type) {
    case T3D_LIGHT_AMBIENT:
        r += L.x; g += L.y; b += L.z;
        break;
    case T3D_LIGHT_POINT: {
        f3 work = mk3(L.x, L.y, L.z);
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
        f3 fwd = mk3(L.x, L.y, L.z);
        f3 normal = (mat && lmode == T3D_LIGHTING_FIXED_NORMALS) ? fwd
                    : (kSkin && (flags & SEG_SKINNED))             ? vnrm
                                                                   : mult_vec_s(dirrot, vnrm);
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
        const DevLight& G = *L.vol;
        float cr = 0.0f, cg = 0.0f, cb = 0.0f;
        uint32_t idx;
        if (mat && mode == T3D_LV_PER_OBJECT) {
            if (lv_cell(G, mk3(M[12], M[13], M[14]), idx)) {
                const float* c = cells + 4 * (size_t)(G.cell_first + idx);
                cr = c[0]; cg = c[1]; cb = c[2];
            }
        } else {
            f3 cs = mk3(G.cell[0] / 2.0f, G.cell[1] / 2.0f, G.cell[2] / 2.0f);
            f3 bias = mk3(G.bias[0], G.bias[1], G.bias[2]);
            f3 vertPos = mk3(0.f, 0.f, 0.f), vertPosN = mk3(0.f, 0.f, 0.f);
            if (kSkin && (flags & SEG_SKINNED)) {  // the zero vertPos plus the scaled normal (light.go:614-619)
                if (mode == T3D_LV_PER_VERTEX_WITH_NORMAL) vertPosN = add3(add3(vertPos, hmul3(vnrm, cs)), bias);
                else vertPos = add3(vpos, bias);
            } else if (mode == T3D_LV_PER_VERTEX_WITH_NORMAL) {
                vertPosN = add3(mult_vec_s(M, add3(vpos, hmul3(vnrm, cs))), bias);
            } else {
                vertPos = add3(mult_vec_s(M, vpos), bias);
            }
            if (!(vertPos.x >= G.vmin[0] && vertPos.y >= G.vmin[1] && vertPos.z >= G.vmin[2] && vertPos.x <= G.vmax[0] &&
                  vertPos.y <= G.vmax[1] && vertPos.z <= G.vmax[2]))
                return;
            if (lv_cell(G, mode == T3D_LV_PER_VERTEX_WITH_NORMAL ? vertPosN : vertPos, idx)) {
                const float* c = cells + 4 * (size_t)(G.cell_first + idx);
                cr = c[0]; cg = c[1]; cb = c[2];
                if (kSkin && (flags & SEG_NESTED)) {  // the cell's useLights, before its colour (light.go:650-656)
                    const uint32_t cc = G.cell_first + idx;
                    for (uint32_t u = ns.off[cc]; u < ns.off[cc + 1]; u++)
                    {
                        const float3 o = nested_light(ns.lights[ns.items[u]], flags, vpos, vnrm, dirrot, ns.inv_r, r, g, b);
                        r = o.x; g = o.y; b = o.z;
                    }
                }
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

// ------------------------------------------------------- tile phases ----
// Shared memory of one block while it works on a tile:
//   ModelSmem | TileSmem | whist[nwarps][kBinsPadded] | lidx u16[T] | depth f32[T] | bin u16[T]
// Per work item constants of the emit path (camera, segment and stream bases).
enum : uint32_t { EC_PERSP = 1, EC_PCORRECT = 2, EC_DEPTH = 4, EC_RDEPTH = 8, EC_FOG_ADD = 16, EC_FOG_SUB = 32,
                  EC_LIT = 64, EC_COLORS = 128, EC_UNBB = 256, EC_SNAP = 512 };
struct EmitConst {
    float W, H, halfW, halfH;
    float margin, spread, tex_w, tex_h;
    float mp[4];
    float fog0, fogspan, fog_r, fog_g;
    float fog_b;
    uint32_t flags, seg_flags, pad;
    float uz[4];             // EC_UNBB: depth row of the unbillboarded MVP (model.go:700-803)
    float snap, pad2[3];     // EC_SNAP: Camera.VertexSnapping
    const float4* va;        // vertex streams of the mesh (mesh vertex 0)
    const float4* vb;
    const float4* vc;
    const uint32_t* idx;     // triangle 0 of the mesh
    const float* cells;
};

struct ModelSmem {
    SLight lights[kMaxLights];  // active lights only (model-level skips removed), in list order
    float4 mvpc[4];   // MVP columns: clip.x = dot(mvpc[0], (x, y, z, 1)) in the reference's order
    float M[16];
    float dirrot[16];
    EmitConst ec;
    uint32_t nl;
    uint32_t pad[3];
    NestedSrc nested;  // SEG_NESTED: lights used by light-volume cells
};

struct TileSmem {
    uint32_t item, nvis, warp_tot[kMaxWarps], scan_tmp[kMaxWarps];
    uint32_t wlo[kMaxWarps], whi[kMaxWarps];  // per-warp range of the visible list
    float wmin[kMaxWarps], wmax[kMaxWarps];
    uint32_t bins_walk[kBins];  // per-bin first output position of this tile in the segment (walk order)
    uint32_t loc_walk[kBins];   // per-bin first position within this tile's own output order (walk order)
};

// Per-warp bin counter regions hold kBinsPadded words: the meshlet ranking keeps counter b
// at pad_bin(b) (one padding word after every 16), the per-vertex route's at b.
constexpr uint32_t kBinsPadded = kBins + kBins / 16;
__device__ __forceinline__ uint32_t pad_bin(uint32_t b) { return b + (b >> 4); }

struct SmemLayout {
    TileSmem* ts;
    uint32_t* whist;
    uint16_t* lidx;
    float* depth;
    uint16_t* bin;
    uint16_t* perm;   // list entry of each output position of the tile
    uint16_t* vloc;   // rank phase: 3 vertex offsets per list entry (aliases depth + lidx, unused there)
};

__device__ __forceinline__ SmemLayout smem_layout(unsigned char* smem, uint32_t tile) {
    SmemLayout L;
    size_t o = 0;
    L.ts = (TileSmem*)(smem + o);
    o += (sizeof(TileSmem) + 15) & ~(size_t)15;  // 16-byte alignment for the vector accesses below
    L.whist = (uint32_t*)(smem + o);
    o += sizeof(uint32_t) * (blockDim.x >> 5) * kBinsPadded;
    L.depth = (float*)(smem + o);
    o += 4 * (size_t)tile;
    L.lidx = (uint16_t*)(smem + o);
    o += 2 * (size_t)tile;
    L.bin = (uint16_t*)(smem + o);
    o += 2 * (size_t)tile;
    L.perm = (uint16_t*)(smem + o);
    L.vloc = (uint16_t*)L.depth;  // 6 bytes per entry = the depth (4) and lidx (2) arrays
    return L;
}

// Stages the model's matrices and (if lit) its light list in shared memory;
// each thread runs ILight.beginModel for one light (light.go:175-189) and the
// model-level point-range skip (camera.go:1625-1629).
// The per-pair constants of the vertex loop: MVP columns (billboarded when the
// material says so), model matrix, directional-light rotation and the emit constants.
// kStreams = false (meshlet tiles): the vertex stream bases are not needed.
template <bool kSkin, bool kStreams = true>
__device__ void stage_model_consts(const DevSeg& seg, const DevJob& J, const DevPrep& pr, ModelSmem& ms) {
    float* mvpc = reinterpret_cast<float*>(ms.mvpc);
    const bool bb = seg.flags & SEG_BILLBOARD;  // either loop: a billboard only changes the MVP
    for (uint32_t k = threadIdx.x; k < 48; k += blockDim.x) {
        if (k < 16) {
            if (!bb) mvpc[4 * (k & 3) + (k >> 2)] = pr.mvp[k];
        }
        else if (k < 32) ms.M[k - 16] = pr.M[k - 16];
        else ms.dirrot[k - 32] = pr.dirrot[k - 32];
    }
    if (threadIdx.x == 0) {
        const JobCam& cam = J.cam;
        EmitConst& e = ms.ec;
        e.W = cam.W; e.H = cam.H; e.halfW = cam.halfW; e.halfH = cam.halfH;
        e.margin = cam.margin; e.spread = cam.spread; e.tex_w = seg.tex_w; e.tex_h = seg.tex_h;
        for (int c = 0; c < 4; c++) e.mp[c] = seg.mp[c];
        e.fog0 = cam.fog_range[0];
        e.fogspan = cam.fog_range[1] - cam.fog_range[0];
        e.fog_r = cam.fog_color[0]; e.fog_g = cam.fog_color[1]; e.fog_b = cam.fog_color[2];
        uint32_t f = 0;
        if (cam.perspective) f |= EC_PERSP;
        if (cam.persp_correct) f |= EC_PCORRECT;
        if (cam.render_depth || cam.fog_on) f |= EC_DEPTH;
        if (cam.render_depth) f |= EC_RDEPTH;
        if (!cam.render_depth && cam.fog_on && cam.fog_mode == T3D_FOG_ADD) f |= EC_FOG_ADD;
        if (!cam.render_depth && cam.fog_on && cam.fog_mode == T3D_FOG_SUB) f |= EC_FOG_SUB;
        if (seg.flags & SEG_LIT) f |= EC_LIT;
        if (seg.flags & SEG_COLORS) f |= EC_COLORS;
        if (kSkin && (seg.flags & SEG_NESTED)) {
            ms.nested.lights = J.lights;
            ms.nested.off = J.cell_use_off;
            ms.nested.items = J.cell_use_items;
            ms.nested.inv_r = pr.inv_r;
        }
        if (kSkin && (seg.flags & SEG_SNAP)) {
            f |= EC_SNAP;
            e.snap = cam.snap;
        }
        if (bb) {  // billboarded MVP of this part (model.go:634-695)
            const m4 base = billboard_base(load16(pr.M), mk3(cam.pos[0], cam.pos[1], cam.pos[2]),
                                           (seg.flags & SEG_BB_CAMUP) ? mk3(cam.up[0], cam.up[1], cam.up[2])
                                                                      : mk3(0.f, 1.f, 0.f),
                                           seg.flags & SEG_BB_LOCKX, seg.flags & SEG_BB_LOCKY, seg.flags & SEG_BB_LOCKZ);
            const m4 mvp = mult(base, load16(cam.vp));
            for (int r = 0; r < 4; r++)
                for (int c = 0; c < 4; c++) mvpc[4 * c + r] = mvp.m[r][c];
            if ((seg.flags & SEG_UNBB) && cam.render_depth) {
                f |= EC_UNBB;
                for (int r = 0; r < 4; r++) e.uz[r] = pr.mvp[4 * r + 2];
            }
        }
        e.flags = f;
        e.seg_flags = seg.flags;
        if (kStreams) {  // shape-keyed meshes read their keyed streams (baked once per weight set)
            const DevMesh& me = J.meshes[seg.mesh];
            e.va = me.nkeys ? J.vaS + me.sbase : J.va + me.vbase;
            e.vb = me.nkeys ? J.vbS + me.sbase : J.vb + me.vbase;
            e.vc = J.vc + me.vbase;
            e.idx = J.idx + 3 * (size_t)me.tbase;
        }
        e.cells = J.cells;
    }
}

template <bool kSkin>
__device__ void stage_model(const FrameParams& P, const DevSeg& seg, const DevJob& J, ModelSmem& ms) {
    const DevPrep& pr = P.preps[seg.inst];
    const DevInst& in = P.insts[seg.inst];
    stage_model_consts<kSkin>(seg, J, pr, ms);
    const uint32_t nl = (seg.flags & SEG_LIT) ? min(in.light_cnt, (uint32_t)kMaxLights) : 0u;
    for (uint32_t k = threadIdx.x; k < nl; k += blockDim.x) {
        const DevLight& L = J.lights[P.inst_light_idx[in.light_off + k]];
        float4 w = make_float4(0.f, 0.f, 0.f, 0.f);
        if (L.type == T3D_LIGHT_POINT) {
            const f3 lp = mk3(L.wpos[0], L.wpos[1], L.wpos[2]);
            const float* r = pr.inv_r;
            // Decompose(Inverted(M)): r.MultVec(lp) + p * (1/s)
            const f3 q = mk3(r[0] * lp.x + r[4] * lp.y + r[8] * lp.z + r[12], r[1] * lp.x + r[5] * lp.y + r[9] * lp.z + r[13],
                             r[2] * lp.x + r[6] * lp.y + r[10] * lp.z + r[14]);
            w.x = q.x + r[3]; w.y = q.y + r[7]; w.z = q.z + r[11];
            if (kSkin && (seg.flags & SEG_SKINNED)) { w.x = lp.x; w.y = lp.y; w.z = lp.z; }  // light.go:183-184
            if (L.range > 0.0f) {
                const float dist = pr.maxspan + L.range;
                if (dist2(mk3(pr.M[12], pr.M[13], pr.M[14]), lp) > dist * dist) w.w = 1.0f;
            }
        }
        SLight& d = ms.lights[k];
        d.type = L.type;
        d.skip = (L.type == T3D_LIGHT_POINT && w.w != 0.0f) ? 1 : 0;
        d.cr = L.color[0]; d.cg = L.color[1]; d.cb = L.color[2];
        d.energy = L.energy; d.range = L.range; d.range2 = L.range2;
        if (L.type == T3D_LIGHT_POINT) { d.x = w.x; d.y = w.y; d.z = w.z; }
        else if (L.type == T3D_LIGHT_AMBIENT) { d.x = L.amb[0]; d.y = L.amb[1]; d.z = L.amb[2]; }
        else { d.x = L.fwd[0]; d.y = L.fwd[1]; d.z = L.fwd[2]; }
        d.vol = &L;
    }
    // drop model-level skipped point lights, keeping list order (the per-vertex
    // sums run over the remaining lights in the same sequence)
    __syncthreads();
    if (threadIdx.x < 32) {
        const uint32_t lane = threadIdx.x;
        uint32_t out = 0;
        for (uint32_t k0 = 0; k0 < nl; k0 += 32) {
            const uint32_t k = k0 + lane;
            SLight rec;
            bool keep = false;
            if (k < nl) {
                rec = ms.lights[k];
                keep = !rec.skip;
            }
            const uint32_t bal = __ballot_sync(0xffffffffu, keep);
            __syncwarp();
            if (keep) ms.lights[out + __popc(bal & ((1u << lane) - 1u))] = rec;
            out += __popc(bal);
            __syncwarp();
        }
        if (lane == 0) ms.nl = out;
    }
}

// MultVecW (model.go:808-811) of one model-space vertex by the staged MVP columns.
__device__ __forceinline__ float4 clip_of(const float4* mc, float x, float y, float z) {
    float4 c;
    const float4 a = mc[0], b = mc[1], d = mc[2], e = mc[3];
    c.x = a.x * x + a.y * y + a.z * z + a.w;
    c.y = b.x * x + b.y * y + b.z * z + b.w;
    c.z = d.x * x + d.y * y + d.z * z + d.w;
    c.w = e.x * x + e.y * y + e.z * z + e.w;
    return c;
}

// The emitted corner of one vertex (camera.go:1655-1812): screen position,
// UV, colour (vertex colour * model/material colour * light) and depth.
// The per-vertex results of one (model, mesh part) for mesh vertex v with
// a = (px, py, pz, nx), b = (ny, nz, u, v):
//   cull  = (X/w, Y/w, Z, depth) with w<0 -> 1e-6 (model.go:862-873) and the
//           depth vertex colour (camera.go:1744-1779)
//   xyuv  = screen position and texture coordinate with w<0 -> 0.001 (camera.go:1655-1708)
//   rgba  = vertex colour * model/material colour * light (camera.go:1726-1742)
// Every value depends only on the vertex, the model, the part and the camera, so
// computing it once per vertex gives the reference's per-corner values bit for bit.
template <bool kSkin>
__device__ __forceinline__ void vertex_record(const ModelSmem& ms, const float4 a, const float4 b, const float4 k,
                                              float4& cull, float4& xyuv, float4& rgba) {
    const EmitConst& e = ms.ec;
    const uint32_t f = e.flags;
    float4 c = clip_of(ms.mvpc, a.x, a.y, a.z);
    if (kSkin && (f & EC_SNAP)) {  // VertexSnapping (model.go:813-818): math32.Round = round half away from zero
        c.x = roundf(c.x * e.snap) / e.snap;
        c.y = roundf(c.y * e.snap) / e.snap;
        c.z = roundf(c.z * e.snap) / e.snap;
    }
    const float w1 = c.w < 0.0f ? 0.000001f : c.w;
    const float cx = c.x / w1, cy = c.y / w1;
    float w = c.w;
    if (!(f & EC_PERSP)) w = 1.0f;
    if (w < 0.0f) w = 0.001f;
    float qx, qy;
    if (w == w1) {  // same divisor: RN(Y / -w) == -RN(Y / w)
        qx = cx;
        qy = -cy;
    } else {
        qx = c.x / w;
        qy = c.y / -w;
    }
    xyuv.x = qx * e.W + e.halfW;
    xyuv.y = qy * e.H + e.halfH;
    if (f & EC_PCORRECT) {
        xyuv.z = (b.z / w) * e.tex_w;
        xyuv.w = ((1.0f - b.w) / w) * e.tex_h;
    } else {
        xyuv.z = b.z * e.tex_w;
        xyuv.w = (1.0f - b.w) * e.tex_h;
    }
    float cr, cg, cb, ca;
    if (f & EC_COLORS) {
        cr = k.x * e.mp[0]; cg = k.y * e.mp[1]; cb = k.z * e.mp[2]; ca = k.w * e.mp[3];
    } else {
        cr = e.mp[0]; cg = e.mp[1]; cb = e.mp[2]; ca = e.mp[3];
    }
    if (f & EC_LIT) {
        const f3 vert = mk3(a.x, a.y, a.z);
        const f3 vnrm = mk3(a.w, b.x, b.y);
        float lr = 0.0f, lg = 0.0f, lb = 0.0f;
        const uint32_t nl = ms.nl;
        for (uint32_t k = 0; k < nl; k++)
            light_vertex<kSkin>(ms.lights[k], e.seg_flags, vert, vnrm, ms.M, ms.dirrot, e.cells, ms.nested, lr, lg, lb);
        cr *= lr; cg *= lg; cb *= lb;
    }
    float depth = 0.0f;
    if (f & EC_DEPTH) {
        float vz = c.z;
        if (kSkin && (f & EC_UNBB)) vz = e.uz[0] * a.x + e.uz[1] * a.y + e.uz[2] * a.z + e.uz[3];
        depth = (vz + e.margin) / e.spread;
        if (depth < 0.0f) depth = 0.0f;
        else if (depth > 1.0f) depth = 1.0f;
        if (f & (EC_FOG_ADD | EC_FOG_SUB)) {
            const float fd = e.fog0 + (e.fogspan * 1.0f - depth);
            if (f & EC_FOG_ADD) {
                cr += e.fog_r * fd; cg += e.fog_g * fd; cb += e.fog_b * fd;
            } else {
                cr *= e.fog_r * fd; cg *= e.fog_g * fd; cb *= e.fog_b * fd;
            }
        }
    }
    cull = make_float4(cx, cy, c.z, depth);
    rgba = make_float4(cr, cg, cb, ca);
}

// Custom0 of a corner under perspective-corrected texture mapping (camera.go:1669-1704):
// 1 / w with the emit loop's w (1 for an orthographic camera, 0.001 when negative).
__device__ __forceinline__ float corner_invw(const ModelSmem& ms, const float4 a) {
    float w = clip_of(ms.mvpc, a.x, a.y, a.z).w;
    if (!(ms.ec.flags & EC_PERSP)) w = 1.0f;
    if (w < 0.0f) w = 0.001f;
    return 1.0f / w;
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

// In-place exclusive scan of arr[0..kBins) by the whole block.
__device__ void scan_bins(TileSmem& sm, uint32_t* arr) {
    __syncthreads();
    const uint32_t per = (kBins + blockDim.x - 1) / blockDim.x;
    const uint32_t lo = threadIdx.x * per, hi = min((uint32_t)kBins, lo + per);
    uint32_t sum = 0;
    for (uint32_t i = lo; i < hi; i++) sum += arr[i];
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
    for (uint32_t i = lo; i < hi; i++) { uint32_t t = arr[i]; arr[i] = run; run += t; }
    __syncthreads();
}

// Stable ranking of a tile's visible list (bins computed, entries in triangle
// order). Warp w owns entries [ts.wlo[w], ts.whi[w]); the ranges follow each
// other in triangle order. Produces the tile's own output order:
// perm[r] = list entry of the tile's r-th output triangle, and loc_walk[] =
// first local rank of each bin (walk order). The tile's output triangles of a
// bin are contiguous in the segment: local ranks loc_walk[w] .. map to
// positions bins_walk[w] ..
__device__ void rank_tile(const SmemLayout& L, uint32_t sort_mode) {
    TileSmem& sm = *L.ts;
    const uint32_t nw = blockDim.x >> 5, wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t lo = sm.wlo[wid], hi = sm.whi[wid];
    for (uint32_t i = threadIdx.x; i < nw * kBins; i += blockDim.x) L.whist[i] = 0u;
    __syncthreads();
    for (uint32_t j = lo + lane; j < hi; j += 32) atomicAdd(&L.whist[wid * kBins + L.bin[j]], 1u);
    __syncthreads();
    for (uint32_t b = threadIdx.x; b < kBins; b += blockDim.x) {
        uint32_t tot = 0;
        for (uint32_t w = 0; w < nw; w++) tot += L.whist[w * kBins + b];
        sm.loc_walk[walk_pos(b, sort_mode)] = tot;
    }
    scan_bins(sm, sm.loc_walk);
    for (uint32_t b = threadIdx.x; b < kBins; b += blockDim.x) {
        uint32_t run = sm.loc_walk[walk_pos(b, sort_mode)];
        for (uint32_t w = 0; w < nw; w++) {
            uint32_t t = L.whist[w * kBins + b];
            L.whist[w * kBins + b] = run;
            run += t;
        }
    }
    __syncthreads();
    const uint32_t lt = (1u << lane) - 1u;
    for (uint32_t j0 = lo; j0 < hi; j0 += 32) {
        const uint32_t j = j0 + lane;
        const bool active = j < hi;
        const uint32_t mask = __ballot_sync(0xffffffffu, active);
        uint32_t b = 0, peers = 0, r = 0;
        if (active) {
            b = L.bin[j];
            peers = __match_any_sync(mask, b);
            r = L.whist[wid * kBins + b] + __popc(peers & lt);
        }
        __syncwarp();
        if (active && lane == (uint32_t)(__ffs(peers) - 1)) L.whist[wid * kBins + b] += __popc(peers);
        __syncwarp();
        if (active) L.perm[r] = (uint16_t)j;
    }
    __syncthreads();
}

// Emits a ranked tile by copying per-vertex records: one thread per output
// corner in the tile's output order, so consecutive threads read vertices of
// the same tile and write consecutive corners of one bin run. Each thread keeps
// kEmitILP corners in flight: their record addresses first, then all loads,
// then all stores.
#ifndef T3D_STREAM_STORES
#define T3D_STREAM_STORES 0  // write-back stores: a tile writes short bin runs that L2 merges into full lines
#endif
#ifndef T3D_EMIT_ILP
#define T3D_EMIT_ILP 1
#endif
constexpr int kEmitILP = T3D_EMIT_ILP;
#ifndef T3D_EMIT_ILP_SINGLE
#define T3D_EMIT_ILP_SINGLE 1  // single-tile segments, emitted inside the register-heavy triangle phase
#endif
constexpr int kEmitILPSingle = T3D_EMIT_ILP_SINGLE;
template <int kILP>
__device__ void tile_emit(const FrameParams& P, const TileDesc& td, const SmemLayout& L, const uint32_t* __restrict__ midx,
                          uint32_t n, uint32_t sort_mode, bool single, bool use_vloc) {
    const TileSmem& sm = *L.ts;
    float4* __restrict__ oxyuv = P.out_xyuv + 3 * (size_t)td.out_base;
    float4* __restrict__ orgba = P.out_rgba + 3 * (size_t)td.out_base;
    float* __restrict__ odepth = P.out_depth + 3 * (size_t)td.out_base;
    const bool pcorrect = td.flags & SEG_PCORRECT;
    const uint32_t vs = td.vscratch, vm = td.vmin, t0 = td.t0;
    const uint32_t total = 3 * n, B = blockDim.x;
    for (uint32_t q0 = threadIdx.x; q0 < total; q0 += kILP * B) {
        uint32_t o[kILP], oc[kILP];
        bool ok[kILP];
#pragma unroll
        for (int u = 0; u < kILP; u++) {
            const uint32_t q = q0 + u * B;
            ok[u] = q < total;
            o[u] = vs;
            oc[u] = 0;
            if (ok[u]) {
                const uint32_t r = q / 3u, c = q - 3u * r;
                const uint32_t j = L.perm[r];
                uint32_t pos = r;
                if (!single) {
                    const uint32_t w = walk_pos(L.bin[j], sort_mode);
                    pos = sm.bins_walk[w] + (r - sm.loc_walk[w]);
                }
                o[u] = vs + (use_vloc ? (uint32_t)L.vloc[3 * j + c] : midx[3 * (t0 + L.lidx[j]) + c] - vm);
                oc[u] = 3 * pos + c;
            }
        }
        float4 x[kILP], k[kILP];
        float d[kILP];
#pragma unroll
        for (int u = 0; u < kILP; u++) {
            if (ok[u]) {
                x[u] = rec_load(&P.vxyuv[o[u]]);
                k[u] = rec_load(&P.vrgba[o[u]]);
                d[u] = rec_load(&P.vcull[o[u]].w);
            }
        }
#pragma unroll
        for (int u = 0; u < kILP; u++) {
            if (ok[u]) {
#if T3D_STREAM_STORES
                __stcs(&oxyuv[oc[u]], x[u]);
                __stcs(&orgba[oc[u]], k[u]);
                __stcs(&odepth[oc[u]], d[u]);
#else
                oxyuv[oc[u]] = x[u];
                orgba[oc[u]] = k[u];
                odepth[oc[u]] = d[u];
#endif
                if (pcorrect) P.out_invw[3 * (size_t)td.out_base + oc[u]] = rec_load(&P.vinvw[o[u]]);
            }
        }
    }
}

// ProcessVertices' rejection tests and depth key for one triangle from its
// corners' cull records (cx, cy, Z) and its model-space centre (model.go:855-969).
__device__ __forceinline__ bool tri_visible(float nearp, float farp, bool backface, f3 ic, float4 c0, float4 c1,
                                            float4 c2, f3 ctr, float& depth) {
    // near/far: some corner with Z + 1 >= near && Z < far (model.go:855-886)
    if (!((c0.z + 1.0f >= nearp && c0.z < farp) || (c1.z + 1.0f >= nearp && c1.z < farp) ||
          (c2.z + 1.0f >= nearp && c2.z < farp)))
        return false;
    const float x0 = c0.x, y0 = c0.y, x1 = c1.x, y1 = c1.y, x2 = c2.x, y2 = c2.y;
    // wholly off one side of the screen (model.go:890-898)
    if ((x0 < -0.5f && x1 < -0.5f && x2 < -0.5f) || (x0 > 0.5f && x1 > 0.5f && x2 > 0.5f) ||
        (y0 < -0.5f && y1 < -0.5f && y2 < -0.5f) || (y0 > 0.5f && y1 > 0.5f && y2 > 0.5f))
        return false;
    if (backface) {  // 2D cross product (model.go:902-925)
        const float n0x = x0 - x1, n0y = y0 - y1;
        const float n1x = x1 - x2, n1y = y1 - y2;
        const float nor = (n0x * n1y) - (n1x * n0y);
        if (nor < 0.0f) return false;
    }
    // squared distance from the model-space camera to tri.Center (model.go:950-953),
    // or from the world camera to the skinned centre (model.go:941-946)
    const float ddx = ic.x - ctr.x, ddy = ic.y - ctr.y, ddz = ic.z - ctr.z;
    depth = ddx * ddx + ddy * ddy + ddz * ddz;
    return !(isnan(depth) || isinf(depth));
}

// tri_visible for corners whose per-corner test outcomes are bits in .w (1 inside near/far,
// 2 / 4 / 8 / 16 off the left / right / bottom / top of the screen): some corner inside
// near/far, not all three off one side, the backface test and the depth key as there.
__device__ __forceinline__ bool tri_visible_bits(bool backface, f3 ic, float4 c0, float4 c1, float4 c2, f3 ctr,
                                                 float& depth) {
    const uint32_t f0 = __float_as_uint(c0.w), f1 = __float_as_uint(c1.w), f2 = __float_as_uint(c2.w);
    if (!((f0 | f1 | f2) & 1u) || (f0 & f1 & f2 & 30u)) return false;
    if (backface) {
        const float n0x = c0.x - c1.x, n0y = c0.y - c1.y;
        const float n1x = c1.x - c2.x, n1y = c1.y - c2.y;
        if ((n0x * n1y) - (n1x * n0y) < 0.0f) return false;
    }
    const float ddx = ic.x - ctr.x, ddy = ic.y - ctr.y, ddz = ic.z - ctr.z;
    depth = ddx * ddx + ddy * ddy + ddz * ddz;
    return !(isnan(depth) || isinf(depth));
}

// Model.skinVertex (model.go:559-594) for vertex v counted from the part's first
// vertex (its shape keys are already in the streams); a = (px, py, pz, nx),
// b = (ny, nz, u, v).
struct AlterSrc {
    const uint4* vj;      // joints of vertex v
    const uint32_t* vj8;  // or the same as bytes (null when not packed)
    const float4* vw;     // their weights
    const float4* bones;  // the model's bone 0 (4 rows each)
};

// Mesh.VertexPositionWithShapeKeys / VertexNormalWithShapeKeys (mesh.go:796-822):
// a mesh's keyed streams, key by key in order, for one weight set. Every model of
// the mesh reads them (the weights belong to the mesh).
__global__ void k_bake_shapes(const float4* __restrict__ va, const float4* __restrict__ vb,
                              const float4* __restrict__ sa, const float2* __restrict__ sb,
                              const float* __restrict__ sw, uint32_t nverts, uint32_t nkeys, float4* oa, float4* ob) {
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nverts) return;
    float4 a = va[v], b = vb[v];
    for (uint32_t k = 0; k < nkeys; k++) {
        const float w = sw[k];
        const float4 da = sa[(size_t)k * nverts + v];  // position delta xyz, normal delta x
        const float2 db = sb[(size_t)k * nverts + v];  // normal delta y, z
        a.x += da.x * w; a.y += da.y * w; a.z += da.z * w;
        a.w += da.w * w; b.x += db.x * w; b.y += db.y * w;
    }
    oa[v] = a;
    ob[v] = b;
}

__device__ __forceinline__ void alter_vertex(const AlterSrc& ms, uint32_t flags, uint32_t v, float4& a, float4& b) {
    if (flags & SEG_SKINNED) {
        uint4 jv;
        if (ms.vj8) {
            const uint32_t p = ms.vj8[v];
            jv = make_uint4(p & 255u, (p >> 8) & 255u, (p >> 16) & 255u, p >> 24);
        } else {
            jv = ms.vj[v];
        }
        const float4 wv = ms.vw[v];
        const uint32_t js[4] = {jv.x, jv.y, jv.z, jv.w};
        const float ws[4] = {wv.x, wv.y, wv.z, wv.w};
        float4 s0 = make_float4(0.f, 0.f, 0.f, 0.f), s1 = s0, s2 = s0, s3 = s0;  // skinMatrix.Clear()
        for (int i = 0; i < 4; i++) {
            const float w = ws[i];
            if (w == 0.0f) continue;
            const float4* B = ms.bones + 4 * (size_t)js[i];
            const float4 b0 = B[0], b1 = B[1], b2 = B[2], b3 = B[3];
            if (w == 1.0f) {
                s0 = b0; s1 = b1; s2 = b2; s3 = b3;
                break;
            }
            // skinMatrix.Add(boneInfluence.Scale(w)), element by element
            s0.x = s0.x + b0.x * w; s0.y = s0.y + b0.y * w; s0.z = s0.z + b0.z * w; s0.w = s0.w + b0.w * w;
            s1.x = s1.x + b1.x * w; s1.y = s1.y + b1.y * w; s1.z = s1.z + b1.z * w; s1.w = s1.w + b1.w * w;
            s2.x = s2.x + b2.x * w; s2.y = s2.y + b2.y * w; s2.z = s2.z + b2.z * w; s2.w = s2.w + b2.w * w;
            s3.x = s3.x + b3.x * w; s3.y = s3.y + b3.y * w; s3.z = s3.z + b3.z * w; s3.w = s3.w + b3.w * w;
        }
        const float px = a.x, py = a.y, pz = a.z, nx = a.w, ny = b.x, nz = b.y;
        a.x = s0.x * px + s1.x * py + s2.x * pz + s3.x;
        a.y = s0.y * px + s1.y * py + s2.y * pz + s3.y;
        a.z = s0.z * px + s1.z * py + s2.z * pz + s3.z;
        // the normal goes through the same matrix with its last row set to (0, 0, 0, 1)
        a.w = s0.x * nx + s1.x * ny + s2.x * nz + 0.0f;
        b.x = s0.y * nx + s1.y * ny + s2.y * nz + 0.0f;
        b.y = s0.z * nx + s1.z * ny + s2.z * nz + 0.0f;
    }
}

// The vertex records of a part whose mesh has shape keys or whose model is
// skinned; a skinned part also leaves its world-space positions in valt for
// the triangles' depth keys.
__device__ __forceinline__ void vertex_chunk_altered(const FrameParams& P, const ModelSmem& ms, const DevSeg& seg,
                                                     uint32_t v0, uint32_t v1) {
    const float4* __restrict__ va = ms.ec.va + seg.vmin;
    const float4* __restrict__ vb = ms.ec.vb + seg.vmin;
    const float4* __restrict__ vc = ms.ec.vc + seg.vmin;
    const bool colors = ms.ec.flags & EC_COLORS;
    const bool skinned = seg.flags & SEG_SKINNED;
    const DevJob& J = P.jobs[seg.job];
    const DevMesh& me = J.meshes[seg.mesh];
    AlterSrc src;
    src.vj = J.vjoint + me.vbase + seg.vmin;
    src.vj8 = J.vjoint8 ? J.vjoint8 + me.vbase + seg.vmin : nullptr;
    src.vw = J.vweight + me.vbase + seg.vmin;
    src.bones = J.bones + 4 * (size_t)J.models[P.insts[seg.inst].model].bone_first;
    for (uint32_t lv = v0 + threadIdx.x; lv < v1; lv += blockDim.x) {
        float4 a = va[lv], b = vb[lv], k = make_float4(0.f, 0.f, 0.f, 0.f);
        if (colors) k = vc[lv];
        alter_vertex(src, seg.flags, lv, a, b);
        float4 cull, xyuv, rgba;
        vertex_record<true>(ms, a, b, k, cull, xyuv, rgba);
        const uint32_t o = seg.vscratch + lv;
        P.vcull[o] = cull;
        P.vxyuv[o] = xyuv;
        P.vrgba[o] = rgba;
        if (skinned) P.valt[o] = make_float4(a.x, a.y, a.z, 0.0f);
        if (seg.flags & SEG_PCORRECT) P.vinvw[o] = corner_invw(ms, a);
    }
}

// ------------------------------------------------- auto-subdivision ----
// closestPointOnTri with its plane and line helpers (colliderTriangles.go:177-182,
// :206-281), in the model space of the camera position.
__device__ __forceinline__ f3 closest_on_line(f3 point, f3 start, f3 end) {
    const f3 diff = sub3(end, start);
    float d = dot3(sub3(point, start), diff) / dot3(diff, diff);
    if (d > 1.0f) d = 1.0f;
    else if (d < 0.0f) d = 0.0f;
    return add3(start, mk3(diff.x * d, diff.y * d, diff.z * d));
}
__device__ __forceinline__ f3 closest_on_tri(f3 point, f3 v0, f3 v1, f3 v2, f3 normal) {
    const float dist = dot3(normal, point) - dot3(normal, v0);
    const f3 pp = sub3(point, mk3(normal.x * dist, normal.y * dist, normal.z * dist));
    // isPointInsideTriangle (colliderTriangles.go:240-265)
    const f3 ca = sub3(v2, v0), ba = sub3(v1, v0), pa = sub3(pp, v0);
    const float dot00 = dot3(ca, ca), dot01 = dot3(ca, ba), dot02 = dot3(ca, pa);
    const float dot11 = dot3(ba, ba), dot12 = dot3(ba, pa);
    const float inv = 1.0f / ((dot00 * dot11) - (dot01 * dot01));
    const float u = ((dot11 * dot02) - (dot01 * dot12)) * inv;
    const float v = ((dot00 * dot12) - (dot01 * dot02)) * inv;
    if (u >= 0.0f && v >= 0.0f && u + v < 1.0f) return pp;
    const f3 ab = closest_on_line(point, v0, v1);
    const f3 bc = closest_on_line(point, v1, v2);
    const f3 cl = closest_on_line(point, v2, v0);
    f3 closest = ab;
    float cd = dist2(point, ab);
    const float bcd = dist2(point, bc), cad = dist2(point, cl);
    if (bcd < cd) { closest = bc; cd = bcd; }
    if (cad < cd) closest = cl;
    return closest;
}
// Whether pool triangle t of an auto-subdivided part is drawn this frame:
// Triangle.handleSubdivision (mesh.go:1877-1949) of its base triangle picks
// the base itself or one subdivision level.
__device__ __forceinline__ bool subdiv_active(const DevJob& J, const float4* __restrict__ va, uint32_t t, f3 ic) {
    const int4 r = J.sub_rel[t];
    if (r.y == 0) return r.x < 0;
    const float4 inf = J.sub_info[t];
    const uint32_t tb = t - (uint32_t)r.z;
    const float4 A = va[J.idx[3 * (size_t)tb]], B = va[J.idx[3 * (size_t)tb + 1]], C = va[J.idx[3 * (size_t)tb + 2]];
    const f3 cp = closest_on_tri(ic, mk3(A.x, A.y, A.z), mk3(B.x, B.y, B.z), mk3(C.x, C.y, C.z), mk3(inf.x, inf.y, inf.z));
    const float dist = dist2(ic, cp);
    int act = -1;
    float closest = 3.402823466e38f;
    for (uint32_t i = 0; i < J.nsub_levels; i++) {
        const float d2 = J.sub_levels[2 * i];
        if (dist < d2 && d2 < closest) { closest = d2; act = (int)i; }
    }
    if (act < 0) return r.x < 0;
    const float size = J.sub_levels[2 * act + 1];
    float ms = inf.w;
    int sub = -1;
    for (int it = 0; ms > size && it < 400; it++) {  // sizes are positive, so this ends within ~280 halvings
        ms /= 2.0f;
        sub++;
    }
    if (sub >= r.y) sub = r.y - 1;
    return sub >= 0 ? r.x == sub : r.x < 0;
}

// The skinned triangle centre, summed from zero over the corners' skinned
// positions and divided by 3 (model.go:840-863, :941-946).
__device__ __forceinline__ f3 skinned_centre(const float4* __restrict__ valt, uint32_t i0, uint32_t i1, uint32_t i2) {
    const float4 p0 = rec_load(&valt[i0]), p1 = rec_load(&valt[i1]), p2 = rec_load(&valt[i2]);
    return mk3((((0.0f + p0.x) + p1.x) + p2.x) / 3.0f, (((0.0f + p0.y) + p1.y) + p2.y) / 3.0f,
               (((0.0f + p0.z) + p1.z) + p2.z) / 3.0f);
}

// PV: per (segment, vertex chunk) the vertex records of every vertex the
// part's triangles use.
template <int kV>
__device__ __noinline__ void phase_vertex(const FrameParams& P, unsigned char* smem) {
    ModelSmem& ms = *reinterpret_cast<ModelSmem*>(smem);
    uint32_t* s_item = reinterpret_cast<uint32_t*>(smem + sizeof(ModelSmem));
    uint32_t item = P.vitem_begin + next_item(P.ctl, 6, s_item);
    while (item < P.vitem_alt) {
        const uint32_t s = P.vitem_seg[item];
        const DevSeg seg = P.segs[s];
        if (!((seg.flags & SEG_SKIP) || P.preps[seg.inst].culled)) {
        const DevJob& J = P.jobs[seg.job];
        stage_model<false>(P, seg, J, ms);
        __syncthreads();
        const uint32_t v0 = P.vitem_chunk[item] * P.vchunk;
        const uint32_t v1 = min(seg.vcount, v0 + P.vchunk);
        const float4* __restrict__ va = ms.ec.va + seg.vmin;
        const float4* __restrict__ vb = ms.ec.vb + seg.vmin;
        const float4* __restrict__ vc = ms.ec.vc + seg.vmin;
        const bool colors = ms.ec.flags & EC_COLORS;
        // software pipeline: the next vertex's streams load while this one computes
        uint32_t lv = v0 + threadIdx.x;
        const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
        float4 a = zero, b = zero, k = zero;
        if (lv < v1) {
            a = va[lv];
            b = vb[lv];
            if (colors) k = vc[lv];
        }
        while (lv < v1) {
            const uint32_t nlv = lv + blockDim.x;
            float4 na = zero, nb = zero, nk = zero;
            if (nlv < v1) {
                na = va[nlv];
                nb = vb[nlv];
                if (colors) nk = vc[nlv];
            }
            float4 cull, xyuv, rgba;
            vertex_record<false>(ms, a, b, k, cull, xyuv, rgba);
            const uint32_t o = seg.vscratch + lv;
            P.vcull[o] = cull;
            P.vxyuv[o] = xyuv;
            P.vrgba[o] = rgba;
            if (seg.flags & SEG_PCORRECT) P.vinvw[o] = corner_invw(ms, a);
            a = na;
            b = nb;
            k = nk;
            lv = nlv;
        }
        }
        item = P.vitem_begin + next_item(P.ctl, 6, s_item);
    }
}

// PV for the vertex items of parts with shape keys or skinning (queue 5).
template <int kV>
__device__ __noinline__ void phase_vertex_altered(const FrameParams& P, unsigned char* smem) {
    ModelSmem& ms = *reinterpret_cast<ModelSmem*>(smem);
    uint32_t* s_item = reinterpret_cast<uint32_t*>(smem + sizeof(ModelSmem));
    uint32_t item = P.vitem_alt + next_item(P.ctl, 5, s_item);
    while (item < P.vitem_end) {
        const DevSeg seg = P.segs[P.vitem_seg[item]];
        if (!((seg.flags & SEG_SKIP) || P.preps[seg.inst].culled)) {
            stage_model<true>(P, seg, P.jobs[seg.job], ms);
            __syncthreads();
            const uint32_t v0 = P.vitem_chunk[item] * P.vchunk;
            vertex_chunk_altered(P, ms, seg, v0, min(seg.vcount, v0 + P.vchunk));
        }
        item = P.vitem_alt + next_item(P.ctl, 5, s_item);
    }
}

// The triangle phase works one grid-width ahead in L2: when a block starts
// item i, one lane asks L2 for what item i + gridDim.x will read (the item some
// block is likely to take next), so its loads hit L2 instead of HBM. (The same
// for the rank phase measured slower: the issuing warp's descriptor loads delay
// its block more than the prefetch saves.)
__device__ __noinline__ void prefetch_triangle_tile(const FrameParams& P, uint32_t item) {
    const TileDesc td = P.tiles[item];
    if ((td.flags & SEG_SKIP) || P.preps[td.inst].culled) return;
    const DevJob& J = P.jobs[td.job];
    const size_t t0 = (size_t)td.tbase + td.t0, nt = td.t1 - td.t0;
    l2_prefetch(J.idx + 3 * t0, 12 * nt);
    l2_prefetch(J.centers + 3 * t0, 12 * nt);
    if (td.vhi > td.vlo) {
        l2_prefetch(P.vcull + td.vlo, 16ull * (td.vhi - td.vlo));
        // skinned parts take their depth keys from the skinned positions
        if (td.flags & SEG_SKINNED) l2_prefetch(P.valt + td.vlo, 16ull * (td.vhi - td.vlo));
    }
}
// P1: visibility and depth keys per tile; single-tile segments are sorted and
// emitted right here, multi-tile segments leave their visible list in HBM.
// Tiles [first, end) from queue q; kSkinned: the tiles of skinned parts, whose
// depth keys come from the skinned positions.
template <bool kSkinned>
__device__ __forceinline__ void triangle_tiles(const FrameParams& P, unsigned char* smem) {
    // item ranges read from the launch parameters where they are used (no registers held)
#define T3D_TILE_FIRST (kSkinned ? P.tile_alt : P.tile_begin)
#define T3D_TILE_END (kSkinned ? P.tile_end : P.tile_alt)
    constexpr int q = kSkinned ? 7 : 1;
    const uint32_t T = P.tile_tris;
    const SmemLayout L = smem_layout(smem, T);
    TileSmem& sm = *L.ts;
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    uint32_t item = T3D_TILE_FIRST + next_item(P.ctl, q, &sm.item);
    while (item < T3D_TILE_END) {
        if (threadIdx.x == blockDim.x - 32 && item + gridDim.x < T3D_TILE_END) prefetch_triangle_tile(P, item + gridDim.x);
        const TileDesc td = P.tiles[item];
        const uint32_t s = td.seg;
        const bool multi = td.flags & SEG_MULTI;
        const uint32_t mt = td.mt;
        const DevPrep& pr = P.preps[td.inst];
        // multi-tile segments: entries go straight to the tile's list in HBM, each warp into its own region
        uint16_t* __restrict__ gi = P.vis_idx + (size_t)mt * T;
        float* __restrict__ gd = P.vis_depth + (size_t)mt * T;
        uint16_t* __restrict__ gv = P.vis_vloc + (size_t)mt * 3 * T;
        if (!((td.flags & SEG_SKIP) || pr.culled)) {
        const DevJob& J = P.jobs[td.job];
        const float nearp = td.nearp, farp = td.farp;
        const bool backface = td.flags & SEG_BACKFACE;
        const f3 ic = mk3(pr.invcam[0], pr.invcam[1], pr.invcam[2]);
        const uint32_t* __restrict__ midx = J.idx + 3 * (size_t)td.tbase;
        const float* __restrict__ mctr = J.centers + 3 * (size_t)td.tbase;
        const float4* __restrict__ vcull = P.vcull + td.vscratch;
        const float4* __restrict__ valt = P.valt + td.vscratch;
        const bool skinned = kSkinned && (td.flags & SEG_SKINNED);
        const bool subdiv = kSkinned && (td.flags & SEG_SUBDIV);
        const float4* __restrict__ sva = J.va + (subdiv ? J.meshes[P.segs[td.seg].mesh].vbase : 0u);
        const uint32_t vm = td.vmin;
        const bool wide = td.flags & SEG_WIDE;
        const uint32_t t0 = td.t0;
        const uint32_t t1 = td.t1;
        float lmin = 3.402823466e38f, lmax = 0.0f;
        // each warp compacts its own contiguous quarter/eighth of the tile
        const uint32_t per = T / nw;
        const uint32_t wt0 = t0 + wid * per, wt1 = min(t1, wt0 + per);
        const uint32_t wbase = wid * per;
        uint32_t cnt = 0;
        const uint32_t lt = (1u << lane) - 1u;
        // two triangles per lane per step (t and t + 32): both gathers are in flight together
        for (uint32_t tb = wt0; tb < wt1; tb += 64) {
            const uint32_t ta = tb + lane, tb2 = tb + 32 + lane;
            bool ha = ta < wt1, hb = tb2 < wt1;
            if (subdiv) {  // candidates of a level other than the chosen one are not drawn
                if (ha) ha = subdiv_active(J, sva, td.tbase + ta, ic);
                if (hb) hb = subdiv_active(J, sva, td.tbase + tb2, ic);
            }
            uint32_t ia0 = vm, ia1 = vm, ia2 = vm, ib0 = vm, ib1 = vm, ib2 = vm;
            f3 ca = mk3(0.f, 0.f, 0.f), cb = ca;
            if (ha) {
                ia0 = midx[3 * ta]; ia1 = midx[3 * ta + 1]; ia2 = midx[3 * ta + 2];
                if (!skinned) ca = mk3(mctr[3 * ta], mctr[3 * ta + 1], mctr[3 * ta + 2]);
                else ca = skinned_centre(valt, ia0 - vm, ia1 - vm, ia2 - vm);
            }
            if (hb) {
                ib0 = midx[3 * tb2]; ib1 = midx[3 * tb2 + 1]; ib2 = midx[3 * tb2 + 2];
                if (!skinned) cb = mk3(mctr[3 * tb2], mctr[3 * tb2 + 1], mctr[3 * tb2 + 2]);
                else cb = skinned_centre(valt, ib0 - vm, ib1 - vm, ib2 - vm);
            }
            float4 pa0 = make_float4(0.f, 0.f, 0.f, 0.f), pa1 = pa0, pa2 = pa0, pb0 = pa0, pb1 = pa0, pb2 = pa0;
            if (ha) { pa0 = rec_load(&vcull[ia0 - vm]); pa1 = rec_load(&vcull[ia1 - vm]); pa2 = rec_load(&vcull[ia2 - vm]); }
            if (hb) { pb0 = rec_load(&vcull[ib0 - vm]); pb1 = rec_load(&vcull[ib1 - vm]); pb2 = rec_load(&vcull[ib2 - vm]); }
            float da = 0.0f, db = 0.0f;
            const bool va_ = ha && tri_visible(nearp, farp, backface, ic, pa0, pa1, pa2, ca, da);
            const bool vb_ = hb && tri_visible(nearp, farp, backface, ic, pb0, pb1, pb2, cb, db);
            const uint32_t bala = __ballot_sync(0xffffffffu, va_);
            const uint32_t balb = __ballot_sync(0xffffffffu, vb_);
            if (va_) {
                const uint32_t p = wbase + cnt + __popc(bala & lt);
                if (!multi) {
                    L.lidx[p] = (uint16_t)(ta - t0);
                    L.depth[p] = da;
                } else {
                    gd[p] = da;
                    if (wide) {
                        gi[p] = (uint16_t)(ta - t0);
                    } else {
                        gv[3 * p] = (uint16_t)(ia0 - vm);
                        gv[3 * p + 1] = (uint16_t)(ia1 - vm);
                        gv[3 * p + 2] = (uint16_t)(ia2 - vm);
                    }
                }
                lmin = fminf(lmin, da);
                lmax = fmaxf(lmax, da);
            }
            cnt += __popc(bala);
            if (vb_) {
                const uint32_t p = wbase + cnt + __popc(balb & lt);
                if (!multi) {
                    L.lidx[p] = (uint16_t)(tb2 - t0);
                    L.depth[p] = db;
                } else {
                    gd[p] = db;
                    if (wide) {
                        gi[p] = (uint16_t)(tb2 - t0);
                    } else {
                        gv[3 * p] = (uint16_t)(ib0 - vm);
                        gv[3 * p + 1] = (uint16_t)(ib1 - vm);
                        gv[3 * p + 2] = (uint16_t)(ib2 - vm);
                    }
                }
                lmin = fminf(lmin, db);
                lmax = fmaxf(lmax, db);
            }
            cnt += __popc(balb);
        }
        // block min / max of the visible depths
        for (int o = 16; o > 0; o >>= 1) {
            lmin = fminf(lmin, __shfl_xor_sync(0xffffffffu, lmin, o));
            lmax = fmaxf(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
        }
        if (lane == 0) {
            sm.wmin[wid] = lmin;
            sm.wmax[wid] = lmax;
            sm.wlo[wid] = wbase;
            sm.whi[wid] = wbase + cnt;
            sm.warp_tot[wid] = cnt;
            if (multi) P.tile_wcnt[(size_t)mt * kMaxWarps + wid] = cnt;
        }
        __syncthreads();
        uint32_t n = 0;
        for (uint32_t w = 0; w < nw; w++) n += sm.warp_tot[w];
        float mn = sm.wmin[0], mx = sm.wmax[0];
        for (uint32_t w = 1; w < nw; w++) { mn = fminf(mn, sm.wmin[w]); mx = fmaxf(mx, sm.wmax[w]); }
        const uint32_t sort_mode = seg_sort_mode(td.flags);
        if (!multi) {
            if (n > 0) {
                const float range = range_of(mn, mx);
                for (uint32_t j = wbase + lane; j < wbase + cnt; j += 32)
                    L.bin[j] = (uint16_t)bin_of(L.depth[j], mn, range, sort_mode);
                rank_tile(L, sort_mode);
                tile_emit<kEmitILPSingle>(P, td, L, midx, n, sort_mode, true, false);
            }
            if (threadIdx.x == 0) {
                P.seg_count[s] = n;
                if (n) atomicAdd(&P.accum[0], (unsigned long long)n);
            }
        } else {
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
        } else if (multi && threadIdx.x == 0) {
            P.tile_count[mt] = 0u;
        }
        item = T3D_TILE_FIRST + next_item(P.ctl, q, &sm.item);
    }
#undef T3D_TILE_FIRST
#undef T3D_TILE_END
}
template <int kV>
__device__ __noinline__ void phase_triangles(const FrameParams& P, unsigned char* smem) { triangle_tiles<false>(P, smem); }
template <int kV>
__device__ __noinline__ void phase_triangles_skinned(const FrameParams& P, unsigned char* smem) {
    triangle_tiles<true>(P, smem);
}

// bin_of for keys in [mn, mn + range] without a divide per key: the quotient is
// (d - mn) * RN(1 / range) with one Markstein correction, within one ulp of the
// division's; its bin can differ only when 512 q lies within an ulp or two of an
// integer, and such keys (|512 q - nearest integer| <= 2^-13, at least two ulps
// for 512 q <= 512) take the exact division, as does every key of a range whose
// reciprocal is passed as NaN.
__device__ __noinline__ uint32_t bin_exact(float d, float mn, float range, uint32_t sort_mode) {
    return bin_of(d, mn, range, sort_mode);
}
__device__ __forceinline__ uint32_t bin_fast(float d, float mn, float range, float rinv, uint32_t sort_mode) {
    if (sort_mode == T3D_SORT_NONE) return 0u;
    const float a = d - mn;
    const float q0 = a * rinv;
    const float q = __fmaf_rn(__fmaf_rn(-range, q0, a), rinv, q0);
    const float x = q * (float)kBins;
    if (!(fabsf(x - rintf(x)) > 0.0001220703125f) || !(x >= 0.0f && x <= (float)kBins)) return bin_exact(d, mn, range, sort_mode);
    return (uint32_t)(int)clampf(x, 0.0f, (float)(kBins - 1));
}

// P2 for one meshlet tile, by one warp: the tile's stable ranking and bin counts.
// One pass over the dense list (entries in triangle order, 32 at a time) bins
// each entry and gives it its index among the earlier entries of its bin (equal
// bins ranked by lane with match_any; one lane per distinct bin advances that
// bin's count), keeping bin and index in shared memory. The counts go out for the
// cross-tile scan (unless the pair has one tile); their exclusive scan in the
// pair's walk order gives each bin's first local rank, and a second pass writes
// entry j of bin b with index w to position first(b) + w of the tile's rank list
// as j | b << 11 | w << 20. cnt: kBins counters, counter b at pad_bin(b) (a padding word
// after every 16, so the lanes' 16-bin runs of the scan fall in distinct banks); sb, sw: a
// bin and an index per entry.
__device__ __noinline__ void hist_rank_meshlet(const FrameParams& P, uint32_t i, const TileDesc& td, uint32_t* cnt,
                                               uint16_t* sb, uint16_t* sw) {
    const uint32_t lane = threadIdx.x & 31, T = P.tile_tris;
    const uint32_t n = __ldcg(&P.tile_count[i]);
    const uint32_t s = td.seg;
    for (uint32_t b = lane; b < kBinsPadded; b += 32) cnt[b] = 0u;
    const float mn = __uint_as_float(__ldcg(&P.seg_minmax[2 * s]));
    const float mx = __uint_as_float(__ldcg(&P.seg_minmax[2 * s + 1]));
    const float range = range_of(mn, mx);
    // ranges outside [2^-60, 2^60] (never met by depth keys) take the exact bins: a NaN reciprocal
    const float rinv = (range >= 0x1p-60f && range <= 0x1p60f) ? 1.0f / range : __int_as_float(0x7fc00000);
    const uint32_t sort_mode = seg_sort_mode(td.flags);
    const float* dep = P.vis_depth + (size_t)i * T;
    const uint32_t lt = (1u << lane) - 1u;
    __syncwarp();
    // pass 1: bins and indices within bins, the next four keys in flight per lane
    float nxt[4];
#pragma unroll
    for (int u = 0; u < 4; u++) nxt[u] = (32u * u + lane < n) ? __ldcg(&dep[32u * u + lane]) : 0.0f;
    for (uint32_t j0 = 0; j0 < n; j0 += 128) {
        float cur[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            cur[u] = nxt[u];
            const uint32_t jn = j0 + 128u + 32u * u + lane;
            nxt[u] = jn < n ? __ldcg(&dep[jn]) : 0.0f;
        }
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const uint32_t j = j0 + 32u * u + lane;
            const bool active = j < n;
            const uint32_t mask = __ballot_sync(0xffffffffu, active);
            if (active) {
                const uint32_t bn = bin_fast(cur[u], mn, range, rinv, sort_mode);
                const uint32_t peers = __match_any_sync(mask, bn);
                const uint32_t w = cnt[pad_bin(bn)] + __popc(peers & lt);
                sb[j] = (uint16_t)bn;
                sw[j] = (uint16_t)w;
                __syncwarp(mask);
                if (lane == (uint32_t)(__ffs(peers) - 1)) cnt[pad_bin(bn)] += __popc(peers);
            }
            __syncwarp();
        }
    }
    if (!(td.flags & SEG_SINGLE)) {
        uint32_t* out = P.tile_hist + (size_t)i * kBins;
        for (uint32_t b = lane; b < kBins; b += 32) out[b] = cnt[pad_bin(b)];
    }
    // exclusive scan in walk order: lane l owns walk positions [16 l, 16 l + 16)
    {
        constexpr uint32_t kPer = kBins / 32;
        uint32_t c[kPer], sum = 0;
#pragma unroll
        for (uint32_t u = 0; u < kPer; u++) {
            c[u] = cnt[pad_bin(walk_pos(lane * kPer + u, sort_mode))];  // walk_pos maps walk positions to bins too
            sum += c[u];
        }
        uint32_t incl = sum;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= (uint32_t)o) incl += v;
        }
        uint32_t base = incl - sum;
        __syncwarp();
#pragma unroll
        for (uint32_t u = 0; u < kPer; u++) {
            cnt[pad_bin(walk_pos(lane * kPer + u, sort_mode))] = base;
            base += c[u];
        }
    }
    __syncwarp();
    // pass 2: each entry to its rank
    uint32_t* rk = P.vis_rank + (size_t)i * T;
    for (uint32_t j = lane; j < n; j += 32) {
        const uint32_t bn = sb[j], w = sw[j];
        rk[cnt[pad_bin(bn)] + w] = j | (bn << 11) | (w << 20);
    }
}

// A tile of a pair whose scan runs in chunks adds its bin counts (just written to tile_hist by
// the same lanes) to its chunk's sums. Kept out of the ranking code, whose schedule it
// slowed even in frames without chunks.
__device__ __noinline__ void add_chunk_counts(const FrameParams& P, uint32_t i) {
    const uint32_t ch = __ldg(&P.mt_chunk[i]);
    if (ch == kNoChunk) return;
    const uint32_t* h = P.tile_hist + (size_t)i * kBins;
    for (uint32_t b = threadIdx.x & 31; b < kBins; b += 32) {
        const uint32_t c = h[b];
        if (c) atomicAdd(&P.chunk_hist[(size_t)ch * kBins + b], c);
    }
}

// P2: bin histograms of the tiles of multi-tile segments, one warp per tile
// (each warp pulls its own tiles and owns a kBins-counter region of shared
// memory). Queue slots run over the record-path tiles [mt_tile_begin,
// mt_tile_end), then the meshlet tiles [mt_mesh_begin, mt_mesh_end), whose
// lists are dense.
template <int kV>
__device__ __noinline__ void phase_hist(const FrameParams& P, unsigned char* smem) {
    const uint32_t T = P.tile_tris;
    const SmemLayout L = smem_layout(smem, T);
    const uint32_t nw = blockDim.x >> 5, wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t per = T / nw;
    const uint32_t n_rec = P.mt_tile_end - P.mt_tile_begin;
    const uint32_t n_all = n_rec + (P.mt_mesh_begin < P.mt_mesh_end ? mesh_tile_count(P) : 0u);
    uint32_t* wh = L.whist + wid * kBinsPadded;
    uint32_t k = 0;
    if (lane == 0) k = atomicAdd(&P.ctl->queue[2], 1u);
    k = __shfl_sync(0xffffffffu, k, 0);
    while (k < n_all) {
        const uint32_t i = k < n_rec ? P.mt_tile_begin + k : mesh_tile_at(P, k - n_rec);
        const TileDesc& td = P.mt_desc[i];
        const uint32_t s = td.seg;
        if (td.flags & SEG_MESHLET) {  // counts, cross-tile counts and the tile's stable ranking
            uint16_t* sb = reinterpret_cast<uint16_t*>(L.whist + (size_t)nw * kBinsPadded) + 2 * (size_t)wid * T;
            hist_rank_meshlet(P, i, td, wh, sb, sb + T);
            if (P.mt_chunk && !(td.flags & SEG_SINGLE)) add_chunk_counts(P, i);
            uint32_t nx = 0;
            if (lane == 0) nx = atomicAdd(&P.ctl->queue[2], 1u);
            k = __shfl_sync(0xffffffffu, nx, 0);
            continue;
        }
        const uint32_t n = __ldcg(&P.tile_count[i]);
        for (uint32_t b = lane; b < kBins; b += 32) wh[b] = 0u;
        __syncwarp();
        if (n > 0) {
            const float mn = __uint_as_float(__ldcg(&P.seg_minmax[2 * s]));
            const float mx = __uint_as_float(__ldcg(&P.seg_minmax[2 * s + 1]));
            const float range = range_of(mn, mx);
            const uint32_t sort_mode = seg_sort_mode(td.flags);
            // the tile's list regions (one per warp of the triangle phase), 4 keys per load
            for (uint32_t w = 0; w < nw; w++) {
                const uint32_t c = __ldcg(&P.tile_wcnt[(size_t)i * kMaxWarps + w]);
                const float4* rd = reinterpret_cast<const float4*>(P.vis_depth + (size_t)i * T + w * per);
                for (uint32_t q = lane; 4 * q < c; q += 32) {
                    const float4 v = __ldcg(&rd[q]);
                    const uint32_t j = 4 * q;
                    atomicAdd(&wh[bin_of(v.x, mn, range, sort_mode)], 1u);
                    if (j + 1 < c) atomicAdd(&wh[bin_of(v.y, mn, range, sort_mode)], 1u);
                    if (j + 2 < c) atomicAdd(&wh[bin_of(v.z, mn, range, sort_mode)], 1u);
                    if (j + 3 < c) atomicAdd(&wh[bin_of(v.w, mn, range, sort_mode)], 1u);
                }
            }
        }
        __syncwarp();
        uint32_t* out = P.tile_hist + (size_t)i * kBins;
        for (uint32_t b = lane; b < kBins; b += 32) out[b] = wh[b];
        if (P.mt_chunk) add_chunk_counts(P, i);
        __syncwarp();
        uint32_t nx = 0;
        if (lane == 0) nx = atomicAdd(&P.ctl->queue[2], 1u);
        k = __shfl_sync(0xffffffffu, nx, 0);
    }
}

// P3: per multi-tile segment, turn tile histograms into per-tile bin bases. A pair of
// several scan chunks is several work items, one per chunk: each takes the pair's bin
// totals and the counts of the chunks before its own from the chunk sums, then runs
// through its own chunk's tiles.
template <int kV>
__device__ __noinline__ void phase_scan(const FrameParams& P, unsigned char* smem) {
    const SmemLayout L = smem_layout(smem, P.tile_tris);
    TileSmem& sm = *L.ts;
    for (;;) {
        const uint32_t k = P.mt_seg_begin + next_item(P.ctl, 3, &sm.item);
        if (k >= P.mt_seg_end) break;
        const uint4 it = P.mt_scan ? P.mt_scan[k] : make_uint4(P.mt_segs[k], kNoChunk, 0u, 1u);
        const uint32_t s = it.x;
        const DevSeg seg = P.segs[s];
        const uint32_t sort_mode = seg_sort_mode(seg.flags);
        if (it.w > 1) {
            const uint32_t c = it.z, nc = it.w;
            const uint32_t* chb = P.chunk_hist + (size_t)it.y * kBins;
            uint32_t* pre = L.whist;  // per bin: the counts of the chunks before this one
            for (uint32_t b = threadIdx.x; b < kBins; b += blockDim.x) {
                uint32_t tot = 0, pb = 0, q = 0;
                for (; q + 8 <= nc; q += 8) {
                    uint32_t v[8];
#pragma unroll
                    for (int u = 0; u < 8; u++) v[u] = __ldcg(&chb[(size_t)(q + u) * kBins + b]);
#pragma unroll
                    for (int u = 0; u < 8; u++) {
                        if (q + u == c) pb = tot;
                        tot += v[u];
                    }
                }
                for (; q < nc; q++) {
                    if (q == c) pb = tot;
                    tot += __ldcg(&chb[(size_t)q * kBins + b]);
                }
                pre[b] = pb;
                sm.bins_walk[walk_pos(b, sort_mode)] = tot;
            }
            scan_bins(sm, sm.bins_walk);
            const uint32_t t0 = c * kScanChunk, nt = min(seg.ntiles, t0 + kScanChunk) - t0;
            for (uint32_t b = threadIdx.x; b < kBins; b += blockDim.x) {
                uint32_t run = sm.bins_walk[walk_pos(b, sort_mode)] + pre[b];
                uint32_t* h = P.tile_hist + (size_t)(seg.mt_first + t0) * kBins + b;
                uint32_t t = 0;
                for (; t + 8 <= nt; t += 8) {
                    uint32_t v[8];
#pragma unroll
                    for (int u = 0; u < 8; u++) v[u] = __ldcg(&h[(size_t)(t + u) * kBins]);
#pragma unroll
                    for (int u = 0; u < 8; u++) { h[(size_t)(t + u) * kBins] = run; run += v[u]; }
                }
                for (; t < nt; t++) {
                    const uint32_t cnt = __ldcg(&h[(size_t)t * kBins]);
                    h[(size_t)t * kBins] = run;
                    run += cnt;
                }
            }
            continue;
        }
        const uint32_t* hbase = P.tile_hist + (size_t)seg.mt_first * kBins;
        for (uint32_t b = threadIdx.x; b < kBins; b += blockDim.x) {
            uint32_t tot = 0;
            uint32_t t = 0;
            for (; t + 8 <= seg.ntiles; t += 8) {  // 8 independent loads in flight
                uint32_t v[8];
#pragma unroll
                for (int u = 0; u < 8; u++) v[u] = __ldcg(&hbase[(size_t)(t + u) * kBins + b]);
#pragma unroll
                for (int u = 0; u < 8; u++) tot += v[u];
            }
            for (; t < seg.ntiles; t++) tot += __ldcg(&hbase[(size_t)t * kBins + b]);
            sm.bins_walk[walk_pos(b, sort_mode)] = tot;
        }
        scan_bins(sm, sm.bins_walk);
        for (uint32_t b = threadIdx.x; b < kBins; b += blockDim.x) {
            uint32_t run = sm.bins_walk[walk_pos(b, sort_mode)];
            uint32_t t = 0;
            uint32_t* h = P.tile_hist + (size_t)seg.mt_first * kBins + b;
            for (; t + 8 <= seg.ntiles; t += 8) {
                uint32_t v[8];
#pragma unroll
                for (int u = 0; u < 8; u++) v[u] = __ldcg(&h[(size_t)(t + u) * kBins]);
#pragma unroll
                for (int u = 0; u < 8; u++) { h[(size_t)(t + u) * kBins] = run; run += v[u]; }
            }
            for (; t < seg.ntiles; t++) {
                const uint32_t c = __ldcg(&h[(size_t)t * kBins]);
                h[(size_t)t * kBins] = run;
                run += c;
            }
        }
    }
}

// P4: stable rank and emission of the tiles of multi-tile segments.
template <int kV>
__device__ __noinline__ void phase_rank_multi(const FrameParams& P, unsigned char* smem) {
    const uint32_t T = P.tile_tris;
    const SmemLayout L = smem_layout(smem, T);
    TileSmem& sm = *L.ts;
    const uint32_t nw = blockDim.x >> 5, wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t per = T / nw, r0 = wid * per;
    uint32_t i = P.mt_tile_begin + next_item(P.ctl, 4, &sm.item);
    while (i < P.mt_tile_end) {
        const TileDesc td = P.mt_desc[i];
        const uint32_t n = __ldcg(&P.tile_count[i]);
        if (n > 0) {
        const uint32_t s = td.seg;
        const uint32_t c = __ldcg(&P.tile_wcnt[(size_t)i * kMaxWarps + wid]);
        const float mn = __uint_as_float(__ldcg(&P.seg_minmax[2 * s]));
        const float mx = __uint_as_float(__ldcg(&P.seg_minmax[2 * s + 1]));
        const float range = range_of(mn, mx);
        const uint32_t sort_mode = seg_sort_mode(td.flags);
        const bool wide = td.flags & SEG_WIDE;
        // each warp loads the list region its namesake warp wrote in the triangle phase
        // (same block size), with 16-byte loads all in flight together
        {
            const float4* rd = reinterpret_cast<const float4*>(P.vis_depth + (size_t)i * T + r0);
            for (uint32_t k = lane; 4 * k < c; k += 32) {
                const float4 v = __ldcg(&rd[k]);
                const uint32_t j = r0 + 4 * k;
                L.bin[j] = (uint16_t)bin_of(v.x, mn, range, sort_mode);
                L.bin[j + 1] = (uint16_t)bin_of(v.y, mn, range, sort_mode);
                L.bin[j + 2] = (uint16_t)bin_of(v.z, mn, range, sort_mode);
                L.bin[j + 3] = (uint16_t)bin_of(v.w, mn, range, sort_mode);
            }
            if (!wide) {  // 3 offsets per entry, 8 per load
                const uint4* rv = reinterpret_cast<const uint4*>(P.vis_vloc + (size_t)i * 3 * T + 3 * r0);
                uint4* sv = reinterpret_cast<uint4*>(L.vloc + 3 * r0);
                for (uint32_t k = lane; 8 * k < 3 * c; k += 32) sv[k] = __ldcg(&rv[k]);
            } else {  // 8 triangle numbers per load
                const uint4* ri = reinterpret_cast<const uint4*>(P.vis_idx + (size_t)i * T + r0);
                uint4* si = reinterpret_cast<uint4*>(L.lidx + r0);
                for (uint32_t k = lane; 8 * k < c; k += 32) si[k] = __ldcg(&ri[k]);
            }
        }
        if (lane == 0) {
            sm.wlo[wid] = r0;
            sm.whi[wid] = r0 + c;
        }
        for (uint32_t b = threadIdx.x; b < kBins; b += blockDim.x)
            sm.bins_walk[walk_pos(b, sort_mode)] = __ldcg(&P.tile_hist[(size_t)i * kBins + b]);
        __syncthreads();
        rank_tile(L, sort_mode);
        const uint32_t* __restrict__ midx = P.jobs[td.job].idx + 3 * (size_t)td.tbase;
        tile_emit<kEmitILP>(P, td, L, midx, n, sort_mode, false, !wide);
        }
        i = P.mt_tile_begin + next_item(P.ctl, 4, &sm.item);  // its barriers also fence the shared arrays
    }
}

// ------------------------------------------------------- meshlet tiles ----
// Render pairs whose parts have meshlets (SEG_MESHLET) keep no per-vertex
// records in HBM. The triangle phase bulk-copies a meshlet's local indices and
// positions into shared memory (the next tile's copy in flight while this one
// is processed), computes the clip values of its slots there, tests the
// triangles and writes the tile's dense visible list; the rank phase copies the
// meshlet's interleaved vertices, computes every slot's emitted corner
// (transform, lighting, depth) in shared memory, ranks the visible list and
// emits from shared memory. Every meshlet tile takes the multi-tile route
// (histogram, cross-tile scan, rank), also when its pair has one tile.

struct MeshHdr {
    unsigned long long bar[4];   // mbarriers: triangle phase 0, 1 = copy buffers; rank phase
                                 // 0 = list + bases, 1 = vertex block, 3 = lights
    uint32_t item[2];            // work item whose copy is in buffer b
    uint32_t copied[2];          // buffer b holds a copy in flight
    uint32_t pad[4];
    TileDesc td[2];              // descriptor of the tile in buffer b
};
static_assert(sizeof(MeshHdr) % 16 == 0, "MeshHdr keeps 16-byte alignment");
// Device address of a meshlet tile's data (the host keeps it in the descriptor's vhi / pad1).
__device__ __forceinline__ const unsigned char* mlet_addr(const TileDesc& td) {
    return reinterpret_cast<const unsigned char*>(((uint64_t)td.pad1 << 32) | td.vhi);
}

__host__ __device__ __forceinline__ size_t al16(size_t x) { return (x + 15) & ~(size_t)15; }
// The head of a DevPrep record the triangle phase copies: mvp, M, dirrot, invcam.
constexpr uint32_t kPrepHead = 208;
static_assert(offsetof(DevPrep, invcam) + 16 == kPrepHead && sizeof(DevPrep) % 16 == 0, "DevPrep head layout");
// Triangle phase: MeshHdr | per-round warp counts (two rounds' worth) and per-warp depth
// range | buf (the model's prep record up to the model-space camera, then lidx + pos of one
// meshlet); each slot's 12 bytes of position become its clip record (X/w, Y/w, test bits)
struct MeshTriWarp {
    uint32_t cnt[2][kMaxWarps];
    float mn[kMaxWarps], mx[kMaxWarps];
};
struct MeshTriLayout { size_t wc, buf, total; };
__host__ __device__ __forceinline__ MeshTriLayout mesh_tri_layout(uint32_t T, uint32_t U) {
    MeshTriLayout L;
    size_t o = sizeof(MeshHdr);
    L.wc = o; o += al16(sizeof(MeshTriWarp));
    const size_t buf = kPrepHead + (size_t)mlet_lidx_bytes(T) + 12ull * U;
    L.buf = o; o += al16(buf);
    L.total = o;
    return L;
}
// Rank phase: MeshHdr | TileSmem | ModelSmem | bases u32[kBins] | ranks u32[T] | vloc u16[3T] |
// staged records | records: 48 bytes per slot (xyuv float4, rgba float4, depth float),
// computed in place over the copied vertex block
struct MeshRankLayout { size_t ts, ms, hist, rk, vloc, stg, rec, total; };
constexpr uint32_t kRecBytes = 48;
constexpr uint32_t kMeshStageBytes = 768;  // sizeof(MeshStage)
__host__ __device__ __forceinline__ MeshRankLayout mesh_rank_layout(uint32_t T, uint32_t U, uint32_t warps) {
    MeshRankLayout L;
    size_t o = sizeof(MeshHdr);
    L.ts = o; o += al16(sizeof(TileSmem));
    L.ms = o; o += al16(sizeof(ModelSmem));
    L.hist = o; o += 4ull * kBins;
    L.rk = o; o += al16(4ull * T);
    L.vloc = o; o += al16(6ull * T);
    L.stg = o; o += kMeshStageBytes;
    L.rec = o; o += (size_t)kRecBytes * U;
    L.total = o;
    (void)warps;
    return L;
}

// Thread 0: records the descriptor of the tile going into buf and starts the copy of
// its model's prep head, local indices and positions (nothing for skipped pairs
// and culled models).
__device__ __forceinline__ uint32_t mesh_issue_tri(const FrameParams& P, const TileDesc& td, bool culled,
                                                   unsigned char* buf, unsigned long long* bar, TileDesc* slot) {
    *slot = td;
    if ((td.flags & SEG_SKIP) || culled) return 0u;
    const uint32_t bytes = mlet_lidx_bytes(td.t1 - td.t0) + 12u * mlet_slots4(td.vmin);
    fence_proxy_async();
    mbar_expect_tx(bar, kPrepHead + bytes);
    bulk_g2s(buf, &P.preps[td.inst], kPrepHead, bar);
    bulk_g2s(buf + kPrepHead, mlet_addr(td), bytes, bar);
    return 1u;
}

// x / 3 rounded to nearest even without a divide instruction: q0 = x * RN(1/3),
// then one correction with the exact residual x - 3 q0 (Markstein's correction,
// P. Markstein, "Computation of elementary functions on the IBM RISC System/6000
// processor", IBM J. Res. Dev. 34(1), 1990). Inputs whose quotient is tiny or not
// finite take the division itself. t3d_check_div3 compares it with IEEE division
// for every float.
__device__ __noinline__ float div3_slow(float x) { return x / 3.0f; }
__device__ __forceinline__ float div3(float x) {
    const float c = 0.3333333432674408f;  // RN(1/3)
    const float q = x * c;
    const float r = __fmaf_rn(-3.0f, q, x);  // exact
    const float y = __fmaf_rn(r, c, q);
    // tiny or non-finite quotients (never met by finite vertex positions) take the division
    return (fabsf(q) >= 1.1754944e-36f && fabsf(q) <= 3.0e38f) ? y : div3_slow(x);
}

// MultVecW (model.go:808-811) by MVP rows m (row-major), in the reference's order.
__device__ __forceinline__ float4 clip_rows(const float* m, float x, float y, float z) {
    float4 c;
    c.x = m[0] * x + m[4] * y + m[8] * z + m[12];
    c.y = m[1] * x + m[5] * y + m[9] * z + m[13];
    c.z = m[2] * x + m[6] * y + m[10] * z + m[14];
    c.w = m[3] * x + m[7] * y + m[11] * z + m[15];
    return c;
}

// Thread 0 also reads, between the steps of a tile, what the copy of the block's
// tile after next needs: the descriptor of queue slot `kn` (after the clip values)
// and its model's culling flag (after the triangles), so their latency hides
// behind work.
struct NextTile {
    uint32_t kn;       // queue slot taken for the tile after next
    TileDesc td;
    uint32_t culled;
};
__device__ __forceinline__ void next_desc(const FrameParams& P, NextTile& nx) {
    if (threadIdx.x == 0 && nx.kn < P.mesh_end - P.mesh_begin) nx.td = P.tiles[P.mesh_begin + nx.kn];
}
__device__ __forceinline__ void next_culled(const FrameParams& P, NextTile& nx) {
    if (threadIdx.x == 0 && nx.kn < P.mesh_end - P.mesh_begin) nx.culled = P.preps[nx.td.inst].culled;
}

// A meshlet tile with no visible triangle: its counts in the pair's cross-tile scan are
// zeros (the histogram phase takes only the tiles with visible triangles).
__device__ __forceinline__ void zero_tile_hist(const FrameParams& P, uint32_t mt) {
    uint4* h = reinterpret_cast<uint4*>(P.tile_hist + (size_t)mt * kBins);
    for (uint32_t b = threadIdx.x; b < kBins / 4; b += blockDim.x) h[b] = make_uint4(0u, 0u, 0u, 0u);
}

// Triangle steps of 32 that a warp holds in registers per round (a round covers
// blockDim / 32 * kTriSteps * 32 triangles of the tile).
constexpr uint32_t kTriSteps = 4;

// One meshlet tile of the triangle phase, its prep head + lidx + pos block in buf. The
// tile's triangles go in rounds; in a round each warp tests 32 * kTriSteps consecutive
// triangles and keeps its visible ones in registers, the warps exchange their counts,
// and every lane writes its entries straight to their places in the tile's dense list
// (triangle order). After the last round's reads of buf, thread 0 starts the copy of
// the block's next tile into it (nx: its queue slot, descriptor and culling flag).
__device__ __forceinline__ void mesh_tile_tri(const FrameParams& P, const TileDesc td, unsigned char* buf,
                                              MeshTriWarp& wc, NextTile& nx, MeshHdr& H, uint32_t nitems) {
    const uint32_t mt = td.mt;
    const DevPrep& pr = *reinterpret_cast<const DevPrep*>(buf);  // its head: mvp, M, dirrot, invcam
    float* mrow = reinterpret_cast<float*>(buf);
    if (td.flags & SEG_BILLBOARD) {  // the part turns to the camera (model.go:634-695)
        if (threadIdx.x == 0) {
            const JobCam& cam = P.jobs[td.job].cam;
            const m4 base = billboard_base(load16(pr.M), mk3(cam.pos[0], cam.pos[1], cam.pos[2]),
                                           (td.flags & SEG_BB_CAMUP) ? mk3(cam.up[0], cam.up[1], cam.up[2])
                                                                     : mk3(0.f, 1.f, 0.f),
                                           td.flags & SEG_BB_LOCKX, td.flags & SEG_BB_LOCKY, td.flags & SEG_BB_LOCKZ);
            store16(mult(base, load16(cam.vp)), mrow);
        }
        __syncthreads();
    }
    const uint32_t U = td.vmin, nt = td.t1 - td.t0;
    const uint16_t* __restrict__ lidx = reinterpret_cast<const uint16_t*>(buf + kPrepHead);
    // a slot's position (x, y, z), then, written over it by the same thread, its clip record
    float* slot = reinterpret_cast<float*>(buf + kPrepHead + mlet_lidx_bytes(nt));
    // Triangle.RecalculateCenter (mesh.go:1980-1982), ((A + B) + C) / 3 per axis, is a constant of
    // the mesh: the scene keeps it per triangle (computed at upload in the same binary32
    // operations); the tile's run is asked into L2 now and read by the triangle loop
    const float* __restrict__ cen = P.jobs[td.job].centers + 3ull * ((size_t)td.tbase + td.t0);
    if (threadIdx.x == 0) l2_prefetch(cen, 12ull * nt);
    const float nearp = td.nearp, farp = td.farp;
    for (uint32_t v = threadIdx.x; v < U; v += blockDim.x) {
        // MultVecW and the x/y divide of the rejection tests (model.go:808-873), and the
        // per-corner outcomes of those tests as bits: 1 inside near/far, 2 / 4 left / right of
        // the screen (X/w < -0.5 / > 0.5), 8 / 16 below / above it
        float* cl = slot + 3 * v;
        const float4 c = clip_rows(mrow, cl[0], cl[1], cl[2]);
        const float w1 = c.w < 0.0f ? 0.000001f : c.w;
        const float sx = c.x / w1, sy = c.y / w1;
        const uint32_t f = ((c.z + 1.0f >= nearp && c.z < farp) ? 1u : 0u) | (sx < -0.5f ? 2u : 0u) |
                           (sx > 0.5f ? 4u : 0u) | (sy < -0.5f ? 8u : 0u) | (sy > 0.5f ? 16u : 0u);
        cl[0] = sx;
        cl[1] = sy;
        cl[2] = __uint_as_float(f);
    }
    next_desc(P, nx);
    const f3 ic = mk3(pr.invcam[0], pr.invcam[1], pr.invcam[2]);
    __syncthreads();
    const uint32_t T = P.tile_tris;
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    float* __restrict__ gd = P.vis_depth + (size_t)mt * T;
    uint16_t* __restrict__ gv = P.vis_vloc + (size_t)mt * 3 * T;
    const bool backface = td.flags & SEG_BACKFACE;
    float lmin = 3.402823466e38f, lmax = 0.0f;
    const uint32_t lt = (1u << lane) - 1u;
    const uint32_t span = nw * 32u * kTriSteps;
    const uint32_t rounds = (nt + span - 1) / span;
    uint32_t base = 0;  // entries of the earlier rounds
    for (uint32_t r = 0; r < rounds; r++) {
        float d[kTriSteps];
        uint32_t s01[kTriSteps], s2[kTriSteps];
        uint32_t vm = 0, wcnt = 0;
#pragma unroll
        for (uint32_t it = 0; it < kTriSteps; it++) {
            const uint32_t t = r * span + (wid * kTriSteps + it) * 32u + lane;
            bool vis = false;
            d[it] = 0.0f;
            s01[it] = 0u;
            s2[it] = 0u;
            if (t < nt) {
                const uint32_t i0 = lidx[3 * t], i1 = lidx[3 * t + 1], i2 = lidx[3 * t + 2];
                const float4 c0 = make_float4(slot[3 * i0], slot[3 * i0 + 1], 0.f, slot[3 * i0 + 2]);
                const float4 c1 = make_float4(slot[3 * i1], slot[3 * i1 + 1], 0.f, slot[3 * i1 + 2]);
                const float4 c2 = make_float4(slot[3 * i2], slot[3 * i2 + 1], 0.f, slot[3 * i2 + 2]);
                const f3 ctr = mk3(__ldg(&cen[3 * t]), __ldg(&cen[3 * t + 1]), __ldg(&cen[3 * t + 2]));
                vis = tri_visible_bits(backface, ic, c0, c1, c2, ctr, d[it]);
                s01[it] = i0 | (i1 << 16);
                s2[it] = i2;
            }
            if (vis) {
                vm |= 1u << it;
                lmin = fminf(lmin, d[it]);
                lmax = fmaxf(lmax, d[it]);
            }
            wcnt += __popc(__ballot_sync(0xffffffffu, vis));
        }
        if (r == 0) next_culled(P, nx);
        const bool last = r + 1 == rounds;
        if (last) {
            for (int o = 16; o > 0; o >>= 1) {
                lmin = fminf(lmin, __shfl_xor_sync(0xffffffffu, lmin, o));
                lmax = fmaxf(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
            }
        }
        uint32_t* cnt = wc.cnt[r & 1u];
        if (lane == 0) {
            cnt[wid] = wcnt;
            if (last) {
                wc.mn[wid] = lmin;
                wc.mx[wid] = lmax;
            }
        }
        __syncthreads();  // the round's counts are in; after the last round buf is no longer read
        if (last && threadIdx.x == 0) {
            H.item[0] = nx.kn;
            H.copied[0] = nx.kn < nitems ? mesh_issue_tri(P, nx.td, nx.culled != 0, buf, &H.bar[0], &H.td[0]) : 0u;
        }
        uint32_t p = base, tot = 0;
        for (uint32_t w = 0; w < nw; w++) {
            const uint32_t c = cnt[w];
            p += w < wid ? c : 0u;
            tot += c;
        }
#pragma unroll
        for (uint32_t it = 0; it < kTriSteps; it++) {
            const bool vis = (vm >> it) & 1u;
            const uint32_t bal = __ballot_sync(0xffffffffu, vis);
            if (vis) {
                const uint32_t q = p + __popc(bal & lt);
                gd[q] = d[it];
                gv[3 * q] = (uint16_t)(s01[it] & 0xFFFFu);
                gv[3 * q + 1] = (uint16_t)(s01[it] >> 16);
                gv[3 * q + 2] = (uint16_t)s2[it];
            }
            p += __popc(bal);
        }
        base += tot;
    }
    if (base == 0 && !(td.flags & SEG_SINGLE)) zero_tile_hist(P, mt);
    if (threadIdx.x == 0) {
        P.tile_count[mt] = base;
        if (base > 0) {
            if (P.live_tiles) P.live_tiles[P.mt_mesh_begin + atomicAdd(&P.ctl->live, 1u)] = mt;
            float mn = wc.mn[0], mx = wc.mx[0];
            for (uint32_t w = 1; w < nw; w++) { mn = fminf(mn, wc.mn[w]); mx = fmaxf(mx, wc.mx[w]); }
            atomicMin(&P.seg_minmax[2 * td.seg], __float_as_uint(mn));
            atomicMax(&P.seg_minmax[2 * td.seg + 1], __float_as_uint(mx));
            atomicAdd(&P.seg_count[td.seg], base);
            atomicAdd(&P.accum[0], (unsigned long long)base);
        }
    }
}

// Triangle phase over meshlet tiles (queue 0). One copy buffer: a tile's copy is started
// as soon as the previous tile's triangles have been read (its list writes overlap the
// copy), and the blocks on an SM cover each other's waits; thread 0 spreads the queue
// slot, descriptor and culling reads for the next tile over the current tile's work.
template <int kV>
__device__ __noinline__ void phase_triangles_meshlet(const FrameParams& P, unsigned char* smem) {
    MeshHdr& H = *reinterpret_cast<MeshHdr*>(smem);
    const MeshTriLayout L = mesh_tri_layout(P.tile_tris, P.mesh_ucap);
    MeshTriWarp& wc = *reinterpret_cast<MeshTriWarp*>(smem + L.wc);
    unsigned char* buf = smem + L.buf;
    const uint32_t n = P.mesh_end - P.mesh_begin, limit = spin_limit(P);
    uint32_t ph0 = 0;
    // the barrier lives in bytes that other phases use: set up here, invalidated at the end
    if (threadIdx.x == 0) {
        mbar_init(&H.bar[0], 1);
        fence_mbar_init();
        const uint32_t k = atomicAdd(&P.ctl->queue[0], 1u);
        H.item[0] = k;
        H.copied[0] = 0u;
        if (k < n) {
            const TileDesc td = P.tiles[P.mesh_begin + k];
            H.copied[0] = mesh_issue_tri(P, td, P.preps[td.inst].culled != 0, buf, &H.bar[0], &H.td[0]);
        }
    }
    __syncthreads();
    for (;;) {
        const uint32_t k = H.item[0];
        if (k >= n) break;
        NextTile nx;
        nx.kn = 0xFFFFFFFFu;
        nx.culled = 1u;
        if (threadIdx.x == 0) nx.kn = atomicAdd(&P.ctl->queue[0], 1u);  // read after the clip values
        const bool copied = H.copied[0] != 0u;
        bool ok = true;
        if (copied) {
            ok = mbar_wait(&H.bar[0], ph0, P.ctl, limit);  // on giving up it has let the copy land
            ph0 ^= 1u;
        }
        if (!__syncthreads_and(ok)) break;
        const TileDesc td = H.td[0];
        if (copied) {
            mesh_tile_tri(P, td, buf, wc, nx, H, n);
        } else {  // skipped pair or culled model
            next_desc(P, nx);
            next_culled(P, nx);
            if (!(td.flags & SEG_SINGLE)) zero_tile_hist(P, td.mt);
            if (threadIdx.x == 0) {
                P.tile_count[td.mt] = 0u;
                H.item[0] = nx.kn;
                H.copied[0] = nx.kn < n ? mesh_issue_tri(P, nx.td, nx.culled != 0, buf, &H.bar[0], &H.td[0]) : 0u;
            }
        }
        __syncthreads();  // the next tile's slot, descriptor and copy state are in place
    }
    __syncthreads();
    // every copy issued was waited for (a queue slot past the end issues none)
    if (threadIdx.x == 0) mbar_inval(&H.bar[0]);
    __syncthreads();
}

// The records a meshlet tile's rank phase starts from, staged in shared memory
// by bulk copies while the block's previous tile is processed.
struct MeshStage {
    TileDesc td;
    DevSeg seg;
    DevPrep pr;
    unsigned char job[304];  // DevJob up to and including `cells`: the camera and the cell table
    uint32_t n;              // visible entries of the tile
    uint32_t pad[3];
};
static_assert(sizeof(MeshStage) == kMeshStageBytes, "MeshStage size");
static_assert(sizeof(DevSeg) % 16 == 0 && sizeof(DevJob) % 16 == 0 && offsetof(DevJob, cells) + 8 <= 304 &&
              offsetof(MeshStage, seg) % 16 == 0 && offsetof(MeshStage, pr) % 16 == 0 &&
              offsetof(MeshStage, job) % 16 == 0 && sizeof(MeshStage) % 16 == 0, "MeshStage layout");

// Thread 0: stages meshlet tile i (its descriptor and count read already) for the
// block's next round: the pair, prep and job records travel by bulk copy.
__device__ __forceinline__ void mesh_stage_tile(const FrameParams& P, const TileDesc& td, uint32_t n, MeshStage& S,
                                                unsigned long long* bar) {
    S.td = td;
    S.n = n;
    if (n == 0) return;
    fence_proxy_async();
    mbar_expect_tx(bar, (uint32_t)(sizeof(DevSeg) + sizeof(DevPrep) + 304));
    bulk_g2s(&S.seg, &P.segs[td.seg], sizeof(DevSeg), bar);
    bulk_g2s(&S.pr, &P.preps[td.inst], sizeof(DevPrep), bar);
    bulk_g2s(S.job, &P.jobs[td.job], 304, bar);
}

// Rank phase over meshlet tiles (queue 9): the emit of tiles the histogram phase
// has ranked. A tile's descriptor, pair, prep and job records are staged during
// the block's previous tile; at its start thread 0 starts every copy at once:
// the tile's rank list, visible corners' slots and bin bases (barrier 0), the
// meshlet's interleaved vertex block (barrier 1) and the model's staged lights
// (barrier 3). The block stages the pair's constants from shared memory, turns
// the vertex block into emitted corners in place and writes the corners in
// output order, one per thread. The next tile is taken at the start of a tile,
// its data asked into L2 and its records staged halfway through.
template <int kV>
__device__ __noinline__ void phase_rank_meshlet(const FrameParams& P, unsigned char* smem) {
    MeshHdr& H = *reinterpret_cast<MeshHdr*>(smem);
    const uint32_t T = P.tile_tris, nw = blockDim.x >> 5;
    const MeshRankLayout ML = mesh_rank_layout(T, P.mesh_ucap, nw);
    ModelSmem& ms = *reinterpret_cast<ModelSmem*>(smem + ML.ms);
    MeshStage& S = *reinterpret_cast<MeshStage*>(smem + ML.stg);
    const uint32_t* hist = reinterpret_cast<const uint32_t*>(smem + ML.hist);
    uint32_t* rk = reinterpret_cast<uint32_t*>(smem + ML.rk);
    uint16_t* vloc = reinterpret_cast<uint16_t*>(smem + ML.vloc);
    unsigned char* rec = smem + ML.rec;
    const uint32_t limit = spin_limit(P);
    uint32_t ph0 = 0, ph1 = 0, ph2 = 0, ph3 = 0;  // mbarrier phases
    const uint32_t nmt = mesh_tile_count(P);
    if (threadIdx.x == 0) {
        for (int b = 0; b < 4; b++) mbar_init(&H.bar[b], 1);
        fence_mbar_init();
        const uint32_t k0 = atomicAdd(&P.ctl->queue[9], 1u);
        H.item[0] = k0;
        if (k0 < nmt) {
            const uint32_t i0 = mesh_tile_at(P, k0);
            mesh_stage_tile(P, P.mt_desc[i0], __ldcg(&P.tile_count[i0]), S, &H.bar[2]);
        }
    }
    __syncthreads();
    for (;;) {
        const uint32_t k = H.item[0];
        if (k >= nmt) break;
        const uint32_t i = mesh_tile_at(P, k);
        const TileDesc td = S.td;
        const uint32_t n = S.n;
        uint32_t kn = 0xFFFFFFFFu;
        if (threadIdx.x == 0) kn = atomicAdd(&P.ctl->queue[9], 1u);
        bool ok = true;
        if (n > 0) {
        const uint32_t U = td.vmin, U4 = mlet_slots4(U), nt = td.t1 - td.t0;
        const bool colors = td.flags & SEG_COLORS;
        const bool single = td.flags & SEG_SINGLE;
        const bool pcorrect = td.flags & SEG_PCORRECT;
        const uint32_t as = mlet_aos_stride(colors);
        // the vertex block lands at the end of the record area: a slot's 48-byte record then
        // only ever covers input bytes of its own or earlier slots
        unsigned char* vin = rec + (size_t)(kRecBytes - as) * U4;
        ok = mbar_wait(&H.bar[2], ph2, P.ctl, limit);  // the staged records
        ph2 ^= 1u;
        const uint32_t nl = (td.flags & SEG_LIT) ? S.pr.nl : 0u;
        if (threadIdx.x == 0) {
            const uint32_t rb = (4u * n + 15u) & ~15u, vb = (6u * n + 15u) & ~15u;
            const uint32_t hb = single ? 0u : 4u * kBins;
            fence_proxy_async();
            mbar_expect_tx(&H.bar[0], hb + rb + vb);
            if (hb) bulk_g2s(smem + ML.hist, P.tile_hist + (size_t)i * kBins, hb, &H.bar[0]);
            bulk_g2s(rk, P.vis_rank + (size_t)i * T, rb, &H.bar[0]);
            bulk_g2s(vloc, P.vis_vloc + (size_t)i * 3 * T, vb, &H.bar[0]);
            mbar_expect_tx(&H.bar[1], as * U4);
            bulk_g2s(vin, mlet_addr(td) + mlet_lidx_bytes(nt) + 12ull * U4, as * U4, &H.bar[1]);
            if (nl) {
                const unsigned char* src = reinterpret_cast<const unsigned char*>(P.inst_lights) +
                                           (size_t)td.inst * kMaxLights * sizeof(SLight);
                mbar_expect_tx(&H.bar[3], slight_copy_bytes(nl));
                bulk_g2s(ms.lights, src, slight_copy_bytes(nl), &H.bar[3]);
            }
            ms.nl = nl;
        }
        stage_model_consts<false, false>(S.seg, *reinterpret_cast<const DevJob*>(S.job), S.pr, ms);
        uint32_t nn = 0, in_ = 0;
        TileDesc tn;
        if (threadIdx.x == 0 && kn < nmt) {  // read now, used after the records
            in_ = mesh_tile_at(P, kn);
            nn = __ldcg(&P.tile_count[in_]);
            tn = P.mt_desc[in_];
        }
        if (nl) {
            ok = mbar_wait(&H.bar[3], ph3, P.ctl, limit) && ok;
            ph3 ^= 1u;
        }
        ok = mbar_wait(&H.bar[1], ph1, P.ctl, limit) && ok;
        ph1 ^= 1u;
        __syncthreads();  // the constants are in place
        // a tile with fewer visible corners than slots computes each corner where it is written
        // (from the vertex block, same function, same bits); the others compute every slot's
        // emitted corner once, in place: a round of two slots per thread reads its inputs, then
        // (after a barrier) writes its records; a record covers only input bytes of its own or
        // earlier slots, all read by the end of the round
        const bool sparse = 3u * n < U;
        for (uint32_t v0 = 0; !sparse && v0 < U; v0 += 2 * blockDim.x) {
            float4 a[2], bb[2], kc[2];
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const uint32_t v = v0 + h * blockDim.x + threadIdx.x;
                a[h] = make_float4(0.f, 0.f, 0.f, 0.f); bb[h] = a[h]; kc[h] = a[h];
                if (v < U) {
                    const float4* in = reinterpret_cast<const float4*>(vin + (size_t)as * v);
                    a[h] = in[0];
                    bb[h] = in[1];
                    if (colors) kc[h] = in[2];
                }
            }
            __syncthreads();
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const uint32_t v = v0 + h * blockDim.x + threadIdx.x;
                if (v < U) {
                    float4 cull, xyuv, rgba;
                    vertex_record<false>(ms, a[h], bb[h], kc[h], cull, xyuv, rgba);
                    float4* out = reinterpret_cast<float4*>(rec + (size_t)kRecBytes * v);
                    out[0] = xyuv;
                    out[1] = rgba;
                    out[2] = make_float4(cull.w, pcorrect ? corner_invw(ms, a[h]) : 0.f, 0.f, 0.f);
                }
            }
        }
        if (threadIdx.x == 0) {
            if (nn > 0) {  // the next tile's vertex block, lists and bases into L2
                const uint32_t u4n = mlet_slots4(tn.vmin), ntn = tn.t1 - tn.t0;
                l2_prefetch(mlet_addr(tn) + mlet_lidx_bytes(ntn) + 12ull * u4n,
                            (size_t)mlet_aos_stride(tn.flags & SEG_COLORS) * u4n);
                l2_prefetch(P.vis_rank + (size_t)in_ * T, 4ull * nn);
                l2_prefetch(P.vis_vloc + (size_t)in_ * 3 * T, 6ull * nn);
                if (!(tn.flags & SEG_SINGLE)) l2_prefetch(P.tile_hist + (size_t)in_ * kBins, 4ull * kBins);
            }
            if (kn < nmt) mesh_stage_tile(P, tn, nn, S, &H.bar[2]);  // the staged records are no longer read
        }
        ok = mbar_wait(&H.bar[0], ph0, P.ctl, limit) && ok;  // ranks, slots, bases (landed long ago)
        ph0 ^= 1u;
        if (__syncthreads_and(ok)) {
            float4* __restrict__ oxyuv = P.out_xyuv + 3 * (size_t)td.out_base;
            float4* __restrict__ orgba = P.out_rgba + 3 * (size_t)td.out_base;
            float* __restrict__ odepth = P.out_depth + 3 * (size_t)td.out_base;
            for (uint32_t q = threadIdx.x; sparse && q < 3 * n; q += blockDim.x) {  // corners computed here
                const uint32_t r = q / 3u, cc = q - 3u * r;
                const uint32_t w = rk[r];
                const uint32_t j = w & 2047u, bn = (w >> 11) & 511u;
                const uint32_t pos = single ? r : hist[bn] + (w >> 20);
                const float4* in = reinterpret_cast<const float4*>(vin + (size_t)as * vloc[3 * j + cc]);
                const float4 a = in[0], b = in[1];
                const float4 kc = colors ? in[2] : make_float4(0.f, 0.f, 0.f, 0.f);
                float4 cull, xyuv, rgba;
                vertex_record<false>(ms, a, b, kc, cull, xyuv, rgba);
                oxyuv[3 * pos + cc] = xyuv;
                orgba[3 * pos + cc] = rgba;
                odepth[3 * pos + cc] = cull.w;
                if (pcorrect) P.out_invw[3 * ((size_t)td.out_base + pos) + cc] = corner_invw(ms, a);
            }
            for (uint32_t q = threadIdx.x; !sparse && q < 3 * n; q += blockDim.x) {  // one corner per thread, output order
                const uint32_t r = q / 3u, cc = q - 3u * r;
                const uint32_t w = rk[r];
                const uint32_t j = w & 2047u, bn = (w >> 11) & 511u;
                const uint32_t pos = single ? r : hist[bn] + (w >> 20);
                const float4* rc = reinterpret_cast<const float4*>(rec + (size_t)kRecBytes * vloc[3 * j + cc]);
                oxyuv[3 * pos + cc] = rc[0];
                orgba[3 * pos + cc] = rc[1];
                odepth[3 * pos + cc] = reinterpret_cast<const float*>(rc + 2)[0];
                if (pcorrect) P.out_invw[3 * ((size_t)td.out_base + pos) + cc] = reinterpret_cast<const float*>(rc + 2)[1];
            }
        }
        } else if (threadIdx.x == 0 && kn < nmt) {  // an empty tile: stage the next one now
            const uint32_t in2 = mesh_tile_at(P, kn);
            mesh_stage_tile(P, P.mt_desc[in2], __ldcg(&P.tile_count[in2]), S, &H.bar[2]);
        }
        __syncthreads();  // the shared arrays are free; the slot taken above becomes the current tile
        if (threadIdx.x == 0) H.item[0] = kn;
        __syncthreads();
        if (!ok) {  // gave up: every issued copy was waited for; leave (the staged copy too)
            if (threadIdx.x == 0 && kn < nmt && S.n > 0) mbar_wait(&H.bar[2], ph2, P.ctl, kSpinLimit);
            break;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {  // every copy of the last tile was waited for
        for (int b = 0; b < 4; b++) mbar_inval(&H.bar[b]);
    }
    __syncthreads();
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Records when the last block finished phase k (kernel start in slot 7) and the
// time this block spent inside the phase (from `since`).
__device__ __forceinline__ void phase_done(Ctl* ctl, int k, unsigned long long& since) {
    if (threadIdx.x == 0) {
        const unsigned long long now = global_ns();
        atomicMax(&ctl->t_end[k], now);
        atomicAdd(&ctl->busy[k], now - since);
    }
}
__device__ __forceinline__ void phase_start(unsigned long long& since) {
    if (threadIdx.x == 0) since = global_ns();
}

#ifndef T3D_MIN_BLOCKS
#define T3D_MIN_BLOCKS 4  // resident blocks of 256 threads per SM the record-path kernel's registers are sized for
#endif
#ifndef T3D_MESH_BLOCKS
#define T3D_MESH_BLOCKS 2  // the same for the kernel with meshlet tiles (its shared memory allows 2 per SM)
#endif
// Blocks of 256 threads per SM that the one-phase kernels are compiled for (registers:
// 65536 / (256 blocks)), per phase: prep, vertex records, triangles, histogram, scan,
// rank + emit; for frames with meshlet tiles and for the others.
#ifndef T3D_PHASE_BLOCKS_MESH
#define T3D_PHASE_BLOCKS_MESH 2, 2, 4, 2, 2, 2
#endif
#ifndef T3D_PHASE_BLOCKS_REC
#define T3D_PHASE_BLOCKS_REC 4, 4, 4, 4, 4, 4
#endif
constexpr int kPhaseBlocks[2][6] = {{T3D_PHASE_BLOCKS_REC}, {T3D_PHASE_BLOCKS_MESH}};
// The phases of one launch (ph: bit 0 prep, 1 vertex records, 2 triangles, 3 histogram,
// 4 scan, 5 rank + emit), with a grid barrier between two phases of the same launch.
// kV & 1: the frame has meshlet tiles; the other bits tell the instantiations apart, so
// every kernel below compiles its own copy of its phases under its own register budget.
// A launch of a single phase after an earlier one has failed does nothing.
template <int kV>
__device__ __forceinline__ void frame_body(const FrameParams& P, unsigned char* smem, const uint32_t ph) {
    constexpr bool kM = kV & 1;
    unsigned long long since = 0;
    const uint32_t limit = spin_limit(P);
    // a grid barrier after phase bit b when this launch also runs a later phase
    auto barrier_after = [&](uint32_t b) { return !(ph & b) || !(ph & ~(2u * b - 1u)) || grid_barrier(P.ctl, limit); };
    if (!(ph & 1u) && vload(&P.ctl->err) != 0) return;
    if (blockIdx.x == 0 && threadIdx.x == 0 && (ph & 1u)) P.ctl->t_end[7] = global_ns();
    if (ph & 1u) {
        phase_start(since);
        phase_prep<kV>(P);
        phase_done(P.ctl, 0, since);
    }
    if (!barrier_after(1u)) return;
    if (ph & 2u) {
        phase_start(since);
        if (P.vitem_begin < P.vitem_alt) phase_vertex<kV>(P, smem);
        if (P.vitem_alt < P.vitem_end) phase_vertex_altered<kV>(P, smem);
        phase_done(P.ctl, 6, since);
    }
    if (!barrier_after(2u)) return;
    if (ph & 4u) {
        phase_start(since);
        if (kM && P.mesh_begin < P.mesh_end) phase_triangles_meshlet<kV>(P, smem);
        if (P.tile_begin < P.tile_alt) phase_triangles<kV>(P, smem);
        if (P.tile_alt < P.tile_end) phase_triangles_skinned<kV>(P, smem);
        phase_done(P.ctl, 1, since);
    }
    if (!P.has_multi) return;
    if (!barrier_after(4u)) return;
    if (ph & 8u) {
        phase_start(since);
        phase_hist<kV>(P, smem);
        phase_done(P.ctl, 2, since);
    }
    if (!barrier_after(8u)) return;
    if (ph & 16u) {
        phase_start(since);
        phase_scan<kV>(P, smem);
        phase_done(P.ctl, 3, since);
    }
    if (!barrier_after(16u)) return;
    if (ph & 32u) {
        phase_start(since);
        if (P.mt_tile_begin < P.mt_tile_end) phase_rank_multi<kV>(P, smem);
        if (kM && P.mt_mesh_begin < P.mt_mesh_end) phase_rank_meshlet<kV>(P, smem);
        phase_done(P.ctl, 4, since);
    }
}

// The whole frame in one cooperative launch (every block resident, phases separated by
// grid barriers), or the phases P.phases names. kM: the frame has meshlet tiles. Both
// instantiations run the record path for the pairs that need it (skinning, shape keys,
// subdivision, snapping, ...).
template <bool kM>
__global__ void __launch_bounds__(256, kM ? T3D_MESH_BLOCKS : T3D_MIN_BLOCKS) t3d_frame_kernel(const __grid_constant__ FrameParams P) {
    extern __shared__ __align__(16) unsigned char smem[];
    frame_body<kM ? 1 : 0>(P, smem, P.phases ? P.phases : 0x3Fu);
}

// One phase per launch (kPh one phase bit): a frame is a sequence of these launches, no
// block waits on another, and each phase runs under its own register budget and
// blocks per SM (kBlocks).
template <int kV, uint32_t kPh, int kBlocks>
__global__ void __launch_bounds__(256, kBlocks) t3d_phase_kernel(const __grid_constant__ FrameParams P) {
    extern __shared__ __align__(16) unsigned char smem[];
    frame_body<kV>(P, smem, kPh);
}

}  // namespace t3d

// Launch entry used by the runtime (same translation-unit linkage).
extern "C" const void* t3d_frame_kernel_ptr() { return (const void*)&t3d::t3d_frame_kernel<false>; }
// The instantiation for frames with meshlet tiles.
extern "C" const void* t3d_frame_kernel_mesh_ptr() { return (const void*)&t3d::t3d_frame_kernel<true>; }
namespace t3d {
template <int kM>
const void* phase_kernel_ptr(int k) {
    switch (k) {
        case 0: return (const void*)&t3d_phase_kernel<kM | 2, 1u, kPhaseBlocks[kM][0]>;
        case 1: return (const void*)&t3d_phase_kernel<kM | 4, 2u, kPhaseBlocks[kM][1]>;
        case 2: return (const void*)&t3d_phase_kernel<kM | 6, 4u, kPhaseBlocks[kM][2]>;
        case 3: return (const void*)&t3d_phase_kernel<kM | 8, 8u, kPhaseBlocks[kM][3]>;
        case 4: return (const void*)&t3d_phase_kernel<kM | 10, 16u, kPhaseBlocks[kM][4]>;
        case 5: return (const void*)&t3d_phase_kernel<kM | 12, 32u, kPhaseBlocks[kM][5]>;
        default: return nullptr;
    }
}
}  // namespace t3d
// The one-phase kernel of phase k (0 prep .. 5 rank + emit), for frames with meshlet tiles
// (mesh != 0) or without; and the blocks per SM it is compiled for.
extern "C" const void* t3d_phase_kernel_ptr(int mesh, int k) {
    return mesh ? t3d::phase_kernel_ptr<1>(k) : t3d::phase_kernel_ptr<0>(k);
}
extern "C" int t3d_phase_kernel_blocks(int mesh, int k) { return (k >= 0 && k < 6) ? t3d::kPhaseBlocks[mesh ? 1 : 0][k] : 0; }
// The vertex data of a shape-keyed mesh's meshlets from its keyed streams (one block per
// meshlet, one thread per slot): positions and the interleaved records' position, normal and
// UV (a mesh's colours are not keyed, so the colour part stays as cut).
__global__ void k_fill_keyed(unsigned char* __restrict__ pool, const t3d::MletFillDev* __restrict__ fills,
                             const uint32_t* __restrict__ vmap, const float4* __restrict__ va, const float4* __restrict__ vb,
                             uint32_t colors) {
    const t3d::MletFillDev f = fills[blockIdx.x];
    float* pos = reinterpret_cast<float*>(pool + 16ull * f.off16 + t3d::mlet_lidx_bytes(f.nt));
    const uint32_t U4 = t3d::mlet_slots4(f.nu), af = t3d::mlet_aos_stride(colors != 0) / 4;
    float* aos = pos + 3ull * U4;
    for (uint32_t s = threadIdx.x; s < f.nu; s += blockDim.x) {
        const uint32_t v = vmap[f.vmap_off + s];
        const float4 a = va[v], b = vb[v];
        pos[3 * s] = a.x; pos[3 * s + 1] = a.y; pos[3 * s + 2] = a.z;
        float* r = aos + (size_t)af * s;
        r[0] = a.x; r[1] = a.y; r[2] = a.z; r[3] = a.w;
        r[4] = b.x; r[5] = b.y; r[6] = b.z; r[7] = b.w;
    }
}
extern "C" cudaError_t t3d_fill_keyed(cudaStream_t st, unsigned char* pool, const void* fills, uint32_t nfills,
                                      const uint32_t* vmap, const float4* va, const float4* vb, uint32_t colors) {
    if (nfills == 0) return cudaSuccess;
    k_fill_keyed<<<nfills, 256, 0, st>>>(pool, (const t3d::MletFillDev*)fills, vmap, va, vb, colors);
    return cudaGetLastError();
}
// The keyed streams of one mesh (k_bake_shapes) on stream st.
extern "C" cudaError_t t3d_bake_shapes(cudaStream_t st, const float4* va, const float4* vb, const float4* sa,
                                       const float2* sb, const float* sw, uint32_t nverts, uint32_t nkeys, float4* oa,
                                       float4* ob) {
    if (nverts == 0) return cudaSuccess;
    t3d::k_bake_shapes<<<(nverts + 255) / 256, 256, 0, st>>>(va, vb, sa, sb, sw, nverts, nkeys, oa, ob);
    return cudaGetLastError();
}
extern "C" size_t t3d_frame_smem_bytes(uint32_t tile_tris, uint32_t block_threads) {
    const size_t tiles = ((sizeof(t3d::TileSmem) + 15) & ~(size_t)15) + 4ull * (block_threads / 32) * t3d::kBinsPadded +
                         10ull * tile_tris + 16;
    const size_t verts = sizeof(t3d::ModelSmem) + 16;
    return tiles > verts ? tiles : verts;
}
// Shared memory of the meshlet kernel: the record-path layouts and both meshlet phases.
extern "C" size_t t3d_frame_smem_bytes_mesh(uint32_t tile_tris, uint32_t block_threads, uint32_t mesh_ucap) {
    const size_t a = t3d_frame_smem_bytes(tile_tris, block_threads);
    const size_t b = t3d::mesh_tri_layout(tile_tris, mesh_ucap).total;
    const size_t c = t3d::mesh_rank_layout(tile_tris, mesh_ucap, block_threads / 32).total;
    // the histogram phase's meshlet ranking: per warp kBins counters and a bin and an index per entry
    const size_t d = ((sizeof(t3d::TileSmem) + 15) & ~(size_t)15) + (block_threads / 32) * (4ull * t3d::kBinsPadded + 4ull * tile_tris);
    size_t m = a > b ? a : b;
    m = m > c ? m : c;
    return m > d ? m : d;
}

// Shared memory of the one-phase kernel of phase k (0 prep .. 5 rank + emit): the
// record-path layout of that phase and, for frames with meshlet tiles, the meshlet one.
extern "C" size_t t3d_phase_smem_bytes(int mesh, int k, uint32_t tile_tris, uint32_t block_threads, uint32_t mesh_ucap) {
    if (k == 0) return 0;
    const size_t a = t3d_frame_smem_bytes(tile_tris, block_threads);
    if (!mesh) return a;
    size_t b = 0;
    if (k == 2) b = t3d::mesh_tri_layout(tile_tris, mesh_ucap).total;
    if (k == 3)
        b = ((sizeof(t3d::TileSmem) + 15) & ~(size_t)15) +
            (block_threads / 32) * (4ull * t3d::kBinsPadded + 4ull * tile_tris);
    if (k == 5) b = t3d::mesh_rank_layout(tile_tris, mesh_ucap, block_threads / 32).total;
    return a > b ? a : b;
}

// Compares div3 with IEEE division for every 32-bit pattern (NaNs match NaNs):
// the number of differences and the first differing pattern found.
__global__ void k_check_div3(unsigned long long* bad, unsigned int* first) {
    for (unsigned long long k = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; k < (1ull << 32);
         k += (unsigned long long)gridDim.x * blockDim.x) {
        const float x = __uint_as_float((unsigned int)k);
        const float a = t3d::div3(x), b = x / 3.0f;
        if (!(__float_as_uint(a) == __float_as_uint(b) || (isnan(a) && isnan(b)))) {
            atomicAdd(bad, 1ull);
            atomicMin(first, (unsigned int)k);
        }
    }
}
extern "C" int t3d_check_div3(unsigned long long* mismatches, unsigned int* first_pattern) {
    unsigned long long* d = nullptr;
    if (cudaMalloc(&d, 16) != cudaSuccess) return -1;
    cudaMemset(d, 0, 8);
    cudaMemset((char*)d + 8, 0xFF, 4);
    k_check_div3<<<4096, 256>>>(d, (unsigned int*)((char*)d + 8));
    cudaError_t e = cudaDeviceSynchronize();
    unsigned long long h[2] = {0, 0};
    if (e == cudaSuccess) e = cudaMemcpy(h, d, 16, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return -1;
    *mismatches = h[0];
    *first_pattern = (unsigned int)h[1];
    return 0;
}

namespace t3d {
// Compares bin_fast with bin_of on n keys per range for 4096 ranges from a seeded
// generator (range magnitudes 1e-3 .. 1e6, keys spread over the range and placed
// next to bin edges): the number of differing bins.
__global__ void k_check_bins(unsigned long long seed, uint32_t n, unsigned long long* bad) {
    const uint32_t g = blockIdx.x;  // one range per block
    unsigned long long h = seed ^ (0x9E3779B97F4A7C15ull * (g + 1));
    auto next = [&h]() { h ^= h << 13; h ^= h >> 7; h ^= h << 17; return (uint32_t)(h >> 32); };
    const float mn = (float)(next() % 2000000u) * 0.37f - 3.0e5f;
    const float range = range_of(0.0f, __powf(10.0f, -3.0f + 9.0f * (float)(next() % 100000u) / 100000.0f));
    const float rinv = (range >= 0x1p-60f && range <= 0x1p60f) ? 1.0f / range : __int_as_float(0x7fc00000);
    for (uint32_t k = threadIdx.x; k < n; k += blockDim.x) {
        unsigned long long hk = h + 0xD1B54A32D192ED03ull * (k + 1);
        hk ^= hk >> 29; hk *= 0xBF58476D1CE4E5B9ull; hk ^= hk >> 32;
        float d;
        if (k & 1) {  // next to the edge of bin b (a few ulps either side)
            const float e = mn + range * ((float)(uint32_t)(hk % 513u) / 512.0f);
            d = __uint_as_float(__float_as_uint(e) + (int)((hk >> 20) % 9u) - 4);
        } else {
            d = mn + range * ((float)(uint32_t)(hk >> 40) / 16777216.0f);
        }
        if (!(d >= mn) || !(d <= mn + range)) continue;
        for (uint32_t m = 0; m < 2; m++)
            if (bin_fast(d, mn, range, rinv, m) != bin_of(d, mn, range, m)) atomicAdd(bad, 1ull);
    }
}
}  // namespace t3d
extern "C" int t3d_check_bins(unsigned long long seed, unsigned int keys_per_range, unsigned long long* mismatches) {
    unsigned long long* d = nullptr;
    if (cudaMalloc(&d, 8) != cudaSuccess) return -1;
    cudaMemset(d, 0, 8);
    t3d::k_check_bins<<<4096, 256>>>(seed, keys_per_range, d);
    cudaError_t e = cudaDeviceSynchronize();
    unsigned long long h = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&h, d, 8, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return -1;
    *mismatches = h;
    return 0;
}
