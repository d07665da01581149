// t3d_noalloc.cu -- t3d_render_part_noalloc: the vertex stage for one render
// pair without any allocation.
//
// Some callers cannot allocate device memory while they render: an engine or
// rasteriser that owns the whole device memory budget through its own
// allocator, a real-time render thread where cudaMalloc / cudaFree would
// synchronise the device and stall the frame, or code already short of memory.
// This entry point takes the mesh and output buffers from the caller and keeps
// every intermediate (packed vertex streams, per-vertex records, visible lists,
// bin histograms, launch tables and the control block) in one file-scope
// __device__ array of fixed size, kNoallocScratchBytes (16 MiB). The array is
// reserved on every GPU that loads the library, for the life of the process.
//
// Limits per call: kNaMaxV vertices, kNaMaxT triangles, T3D_MAX_LIGHTS_PER_MODEL
// lights; larger requests are rejected with T3D_E_INVAL and a message.
//
// All calls share the one array (and one static host staging area), so calls
// that overlap on the GPU -- on different streams or from different host
// threads -- race and corrupt each other; serialise them. The first call on a
// device performs the set-up (symbol address, kernel attributes, occupancy);
// make that first call before any stream capture. The call waits for its own
// stream before returning so that it can report the kernel's status.

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "t3d_runtime.h"

extern "C" const void* t3d_frame_kernel_ptr();
extern "C" size_t t3d_frame_smem_bytes(uint32_t tile_tris, uint32_t block_threads);

using namespace t3d;

namespace {

constexpr uint32_t kNaMaxV = 65536;    // vertices per call
constexpr uint32_t kNaMaxT = 131072;   // triangles per call (mesh)
constexpr uint32_t kNaTile = 2048;     // triangles per tile
constexpr uint32_t kNaChunk = 1024;    // vertices per vertex work item
constexpr uint32_t kNaBlock = 256;
constexpr uint32_t kNaMaxTiles = kNaMaxT / kNaTile;
constexpr uint32_t kNaMaxChunks = kNaMaxV / kNaChunk;
constexpr uint32_t kNaMaxL = T3D_MAX_LIGHTS_PER_MODEL;
constexpr size_t kNoallocScratchBytes = 16u << 20;

constexpr size_t al(size_t x) { return (x + 255) & ~(size_t)255; }

// byte offsets of the regions of the scratch array
constexpr size_t O_VA = 0;
constexpr size_t O_VB = O_VA + al(16ull * kNaMaxV);
constexpr size_t O_VC = O_VB + al(16ull * kNaMaxV);
constexpr size_t O_IDX = O_VC + al(16ull * kNaMaxV);
constexpr size_t O_CTR = O_IDX + al(12ull * kNaMaxT);
constexpr size_t O_VCULL = O_CTR + al(12ull * kNaMaxT);
constexpr size_t O_VXYUV = O_VCULL + al(16ull * kNaMaxV);
constexpr size_t O_VRGBA = O_VXYUV + al(16ull * kNaMaxV);
constexpr size_t O_VISI = O_VRGBA + al(16ull * kNaMaxV);
constexpr size_t O_VISD = O_VISI + al(2ull * kNaMaxT);
constexpr size_t O_VISV = O_VISD + al(4ull * kNaMaxT);
constexpr size_t O_TCNT = O_VISV + al(6ull * kNaMaxT);
constexpr size_t O_TWC = O_TCNT + al(4ull * kNaMaxTiles);
constexpr size_t O_THIST = O_TWC + al(4ull * kMaxWarps * kNaMaxTiles);
constexpr size_t O_MINMAX = O_THIST + al(4ull * kBins * kNaMaxTiles);
constexpr size_t O_PREP = O_MINMAX + al(8);
constexpr size_t O_ACCUM = O_PREP + al(sizeof(DevPrep));
constexpr size_t O_CTL = O_ACCUM + al(16);
constexpr size_t O_ERR = O_CTL + al(sizeof(Ctl));
constexpr size_t O_TABLES = O_ERR + al(4);
// launch tables (uploaded from the static host staging area)
constexpr size_t T_JOB = 0;
constexpr size_t T_INST = T_JOB + al(sizeof(DevJob));
constexpr size_t T_SEG = T_INST + al(sizeof(DevInst));
constexpr size_t T_MESH = T_SEG + al(sizeof(DevSeg));
constexpr size_t T_MODEL = T_MESH + al(sizeof(DevMesh));
constexpr size_t T_LIGHTS = T_MODEL + al(sizeof(DevModel));
constexpr size_t T_LIDX = T_LIGHTS + al(sizeof(DevLight) * kNaMaxL);
constexpr size_t T_TILES = T_LIDX + al(4ull * kNaMaxL);
constexpr size_t T_MTD = T_TILES + al(sizeof(TileDesc) * kNaMaxTiles);
constexpr size_t T_MTS = T_MTD + al(sizeof(TileDesc) * kNaMaxTiles);
constexpr size_t T_VSEG = T_MTS + al(4);
constexpr size_t T_VCH = T_VSEG + al(4ull * kNaMaxChunks);
constexpr size_t T_END = T_VCH + al(4ull * kNaMaxChunks);
constexpr size_t O_END = O_TABLES + T_END;
static_assert(O_END <= kNoallocScratchBytes, "no-alloc scratch layout exceeds the array");

// Host staging for the launch tables (no allocation per call).
static unsigned char g_host_tables[T_END];
static std::mutex g_mu;

struct NaDevice {
    bool ready = false;
    unsigned char* scratch = nullptr;  // device address of g_noalloc_scratch on this device
    uint32_t max_grid = 0;
    size_t smem = 0;
};
static NaDevice g_dev[64];

void fail(t3d_noalloc_args* a, const char* fmt, const char* detail = "") {
    if (a) snprintf(a->error, sizeof a->error, fmt, detail);
}

}  // namespace

// The scratch array. Host code must not use its name as an address; the device
// address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

// Packs the caller's SoA streams into the kernel's 16-byte vertex records,
// copies the indices (replacing out-of-range ones by 0 and flagging them) and
// computes Triangle.RecalculateCenter, ((A + B) + C) / 3 in binary32 (mesh.go:1980-1982).
__global__ void t3d_noalloc_pack(const float* __restrict__ pos, const float* __restrict__ nrm,
                                 const float* __restrict__ uv, const float* __restrict__ col,
                                 const uint32_t* __restrict__ idx, uint32_t nv, uint32_t nt) {
    float4* va = reinterpret_cast<float4*>(g_noalloc_scratch + O_VA);
    float4* vb = reinterpret_cast<float4*>(g_noalloc_scratch + O_VB);
    float4* vc = reinterpret_cast<float4*>(g_noalloc_scratch + O_VC);
    uint32_t* io = reinterpret_cast<uint32_t*>(g_noalloc_scratch + O_IDX);
    float* ctr = reinterpret_cast<float*>(g_noalloc_scratch + O_CTR);
    uint32_t* err = reinterpret_cast<uint32_t*>(g_noalloc_scratch + O_ERR);
    const uint32_t n = nv > nt ? nv : nt;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        if (k < nv) {
            va[k] = make_float4(pos[3 * k], pos[3 * k + 1], pos[3 * k + 2], nrm[3 * k]);
            vb[k] = make_float4(nrm[3 * k + 1], nrm[3 * k + 2], uv[2 * k], uv[2 * k + 1]);
            vc[k] = col ? make_float4(col[4 * k], col[4 * k + 1], col[4 * k + 2], col[4 * k + 3])
                        : make_float4(1.f, 1.f, 1.f, 1.f);
        }
        if (k < nt) {
            uint32_t i[3] = {idx[3 * k], idx[3 * k + 1], idx[3 * k + 2]};
            for (int c = 0; c < 3; c++)
                if (i[c] >= nv) {
                    atomicOr(err, 1u);
                    i[c] = 0;
                }
            for (int c = 0; c < 3; c++) io[3 * k + c] = i[c];
            for (int a = 0; a < 3; a++)
                ctr[3 * k + a] = (pos[3 * i[0] + a] + pos[3 * i[1] + a] + pos[3 * i[2] + a]) / 3.0f;
        }
    }
}

static int na_setup(int device, t3d_noalloc_args* a) {
    NaDevice& d = g_dev[device];
    if (d.ready) return T3D_OK;
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr) {
        fail(a, "cudaGetSymbolAddress(scratch) failed: %s", cudaGetErrorString(e));
        return T3D_E_CUDA;
    }
    d.smem = t3d_frame_smem_bytes(kNaTile, kNaBlock);
    const void* fn = t3d_frame_kernel_ptr();
    if ((e = raise_smem_limit(fn, d.smem)) != cudaSuccess) {
        fail(a, "kernel attribute: %s", cudaGetErrorString(e));
        return T3D_E_CUDA;
    }
    int per_sm = 0, sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, (int)kNaBlock, d.smem)) != cudaSuccess ||
        per_sm < 1) {
        fail(a, "occupancy query failed: %s", cudaGetErrorString(e));
        return T3D_E_CUDA;
    }
    d.scratch = (unsigned char*)ptr;
    d.max_grid = (uint32_t)(per_sm * sms);
    d.ready = true;
    return T3D_OK;
}

// Model.isTransparent (model.go:1274-1282)
static bool na_transparent(const float* mc, const t3d_material& mat) {
    if (mat.present) {
        bool matT = mat.transparency_mode == T3D_TRANSPARENCY_TRANSPARENT || !mat.blend_source_over ||
                    (mat.transparency_mode == T3D_TRANSPARENCY_AUTO && mat.color[3] < 0.999f);
        bool modelT = mat.transparency_mode != T3D_TRANSPARENCY_OPAQUE && mc[3] < 0.999f;
        return matT || modelT;
    }
    return mc[3] < 0.999f;
}

#define NA_CK(call)                                                        \
    do {                                                                   \
        cudaError_t e_ = (call);                                           \
        if (e_ != cudaSuccess) {                                           \
            fail(a, #call " failed: %s", cudaGetErrorString(e_));          \
            return T3D_E_CUDA;                                             \
        }                                                                  \
    } while (0)

extern "C" int t3d_render_part_noalloc(int device, t3d_noalloc_args* a, void* stream) {
    if (!a) return T3D_E_INVAL;
    a->error[0] = '\0';
    if (!a->model || !a->camera || (a->num_lights && !a->lights) || !a->positions || !a->normals || !a->uvs ||
        !a->indices || !a->out_xyuv || !a->out_rgba || !a->out_depth || !a->out_count) {
        fail(a, "null argument%s");
        return T3D_E_INVAL;
    }
    if (a->num_vertices == 0) {
        fail(a, "empty mesh: num_vertices is 0%s");
        return T3D_E_INVAL;
    }
    if (a->num_vertices > kNaMaxV || a->num_triangles > kNaMaxT || a->num_lights > kNaMaxL) {
        snprintf(a->error, sizeof a->error,
                 "size beyond the no-alloc limits: %u vertices (max %u), %u triangles (max %u), %u lights (max %u)",
                 a->num_vertices, kNaMaxV, a->num_triangles, kNaMaxT, a->num_lights, kNaMaxL);
        return T3D_E_INVAL;
    }
    if ((uint64_t)a->tri_start + a->tri_count > a->num_triangles) {
        snprintf(a->error, sizeof a->error, "part [%u, %u + %u) lies outside the mesh's %u triangles", a->tri_start,
                 a->tri_start, a->tri_count, a->num_triangles);
        return T3D_E_INVAL;
    }
    if (a->camera->width <= 0 || a->camera->height <= 0) {
        fail(a, "bad camera size%s");
        return T3D_E_INVAL;
    }
    if (a->model->skinned) {  // the part's vertices come without joints, weights or bones
        fail(a, "skinned models need the scene path (t3d_scene_upload)%s");
        return T3D_E_INVAL;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev || device >= 64) {
        fail(a, "bad device%s");
        return T3D_E_INVAL;
    }
    std::lock_guard<std::mutex> guard(g_mu);
    // the caller's current device is restored on every return
    struct DeviceGuard {
        int prev = -1;
        ~DeviceGuard() { if (prev >= 0) cudaSetDevice(prev); }
    } dev_guard;
    NA_CK(cudaGetDevice(&dev_guard.prev));
    NA_CK(cudaSetDevice(device));
    int rc = na_setup(device, a);
    if (rc) return rc;
    NaDevice& d = g_dev[device];
    cudaStream_t st = (cudaStream_t)stream;
    unsigned char* S = d.scratch;
    const t3d_model_desc& md = *a->model;
    const t3d_material& mat = a->mat;

    // A pair the reference never draws, or that ProcessVertices empties
    // (camera.go:1343-1380, model.go:604-606), emits nothing.
    const bool drawn = md.visible && !(mat.present && !mat.visible) && a->tri_count > 0 &&
                       !(md.color[3] == 0 && na_transparent(md.color, mat));
    if (!drawn) {
        NA_CK(cudaMemsetAsync(a->out_count, 0, 4, st));
        NA_CK(cudaStreamSynchronize(st));
        return T3D_OK;
    }

    // ---- launch tables in the static host staging area ----
    unsigned char* H = g_host_tables;
    memset(H, 0, T_END);
    DevJob& job = *reinterpret_cast<DevJob*>(H + T_JOB);
    build_camera(*a->camera, job.cam);
    job.va = (const float4*)(S + O_VA);
    job.vb = (const float4*)(S + O_VB);
    job.vc = (const float4*)(S + O_VC);
    job.idx = (const uint32_t*)(S + O_IDX);
    job.centers = (const float*)(S + O_CTR);
    job.meshes = (const DevMesh*)(S + O_TABLES + T_MESH);
    job.models = (DevModel*)(S + O_TABLES + T_MODEL);
    job.cells = a->volume_cells;
    job.lights = (const DevLight*)(S + O_TABLES + T_LIGHTS);

    DevMesh& me = *reinterpret_cast<DevMesh*>(H + T_MESH);
    me.vbase = 0;
    me.tbase = 0;
    me.nverts = a->num_vertices;
    me.ntris = a->num_triangles;
    for (int k = 0; k < 3; k++) { me.dmin[k] = a->dim_min[k]; me.dmax[k] = a->dim_max[k]; }

    DevModel& m = *reinterpret_cast<DevModel*>(H + T_MODEL);
    memcpy(m.transform, md.transform, 64);
    memcpy(m.world_rot, md.world_rotation, 64);
    memcpy(m.position, md.position, 12);
    memcpy(m.scale, md.scale, 12);
    memcpy(m.rotation, md.rotation, 64);
    memcpy(m.rotate_step, md.rotate_step, 64);
    memcpy(m.color, md.color, 16);
    m.mesh = 0;
    m.flags = MOD_VISIBLE | (md.frustum_culling ? MOD_FRUSTUM : 0) | (md.shadeless ? MOD_SHADELESS : 0) |
              (md.use_trs ? MOD_TRS : 0);

    DevLight* lights = reinterpret_cast<DevLight*>(H + T_LIGHTS);
    uint32_t* lidx = reinterpret_cast<uint32_t*>(H + T_LIDX);
    for (uint32_t i = 0; i < a->num_lights; i++) {
        if (a->lights[i].type < 0 || a->lights[i].type > 3 || (a->lights[i].type == T3D_LIGHT_VOLUME && !a->volume_cells)) {
            fail(a, "bad light (type, or a volume light without cells)%s");
            return T3D_E_INVAL;
        }
        build_light(a->lights[i], lights[i]);
        lidx[i] = i;
    }

    DevInst& in = *reinterpret_cast<DevInst*>(H + T_INST);
    in.job = 0;
    in.model = 0;
    in.light_off = 0;
    in.light_cnt = a->num_lights;
    in.animate = 0;
    in.bytes = 0;

    const uint32_t ntiles = (a->tri_count + kNaTile - 1) / kNaTile;
    const uint32_t nchunks = (a->num_vertices + kNaChunk - 1) / kNaChunk;
    DevSeg& sg = *reinterpret_cast<DevSeg*>(H + T_SEG);
    sg.inst = 0;
    sg.job = 0;
    sg.mesh = 0;
    sg.tri_start = a->tri_start;
    sg.tri_count = a->tri_count;
    sg.vmin = 0;
    sg.vcount = a->num_vertices;
    sg.vscratch = 0;
    sg.out_base = 0;
    sg.tile_first = 0;
    sg.ntiles = ntiles;
    sg.mt_first = 0;
    uint32_t flags = 0;
    if (a->camera->lighting_on && !(mat.present && mat.shadeless) && !md.shadeless) flags |= SEG_LIT;
    if (mat.present && mat.backface_culling) flags |= SEG_BACKFACE;
    if (a->colors) flags |= SEG_COLORS;
    if (mat.present) flags |= SEG_MAT;
    if (ntiles > 1) flags |= SEG_MULTI;
    flags |= (uint32_t)(mat.present ? mat.sort_mode & 3 : 0) << 8;
    flags |= (uint32_t)(mat.present ? mat.lighting_mode & 3 : 0) << 10;
    flags |= (uint32_t)(mat.present ? mat.lv_shading_mode & 3 : 0) << 12;
    flags |= billboard_flags(mat, false);
    if (a->camera->vertex_snapping > 0.0f) flags |= SEG_SNAP;
    sg.flags = flags;
    for (int k = 0; k < 4; k++) sg.mp[k] = mat.present ? md.color[k] * mat.color[k] : md.color[k];
    sg.tex_w = mat.present ? mat.tex_w : 0.0f;
    sg.tex_h = mat.present ? mat.tex_h : 0.0f;
    TileDesc* tds = reinterpret_cast<TileDesc*>(H + T_TILES);
    TileDesc* mtd = reinterpret_cast<TileDesc*>(H + T_MTD);
    uint32_t* vseg = reinterpret_cast<uint32_t*>(H + T_VSEG);
    uint32_t* vch = reinterpret_cast<uint32_t*>(H + T_VCH);
    for (uint32_t t = 0; t < ntiles; t++) {
        TileDesc& td = tds[t];
        td.seg = 0; td.inst = 0; td.job = 0; td.flags = flags;
        td.t0 = a->tri_start + t * kNaTile;
        td.t1 = std::min(a->tri_start + a->tri_count, td.t0 + kNaTile);
        td.tbase = 0; td.vmin = 0; td.vscratch = 0; td.out_base = 0;
        td.mt = ntiles > 1 ? t : 0u;
        td.nearp = job.cam.near_; td.farp = job.cam.far_;
        mtd[t] = td;
    }
    for (uint32_t c = 0; c < nchunks; c++) { vseg[c] = 0; vch[c] = c; }

    // ---- uploads (no allocation: plain copies into the static array) ----
    NA_CK(cudaMemcpyAsync(S + O_TABLES, H, T_END, cudaMemcpyHostToDevice, st));
    NA_CK(cudaMemsetAsync(S + O_CTL, 0, sizeof(Ctl), st));
    NA_CK(cudaMemsetAsync(S + O_ERR, 0, 4, st));
    NA_CK(cudaMemsetAsync(S + O_ACCUM, 0, 16, st));
    t3d_noalloc_pack<<<std::max(1u, std::min(1024u, (std::max(a->num_vertices, a->num_triangles) + 255) / 256)), 256, 0,
                       st>>>(a->positions, a->normals, a->uvs, a->colors, a->indices, a->num_vertices,
                             a->num_triangles);
    NA_CK(cudaGetLastError());

    FrameParams P;
    memset(&P, 0, sizeof P);
    P.jobs = (const DevJob*)(S + O_TABLES + T_JOB);
    P.insts = (const DevInst*)(S + O_TABLES + T_INST);
    P.preps = (DevPrep*)(S + O_PREP);
    P.inst_light_idx = (const uint32_t*)(S + O_TABLES + T_LIDX);
    P.segs = (const DevSeg*)(S + O_TABLES + T_SEG);
    P.tiles = (const TileDesc*)(S + O_TABLES + T_TILES);
    P.mt_desc = (const TileDesc*)(S + O_TABLES + T_MTD);
    P.mt_segs = (const uint32_t*)(S + O_TABLES + T_MTS);
    P.vitem_seg = (const uint32_t*)(S + O_TABLES + T_VSEG);
    P.vitem_chunk = (const uint32_t*)(S + O_TABLES + T_VCH);
    P.vcull = (float4*)(S + O_VCULL);
    P.vxyuv = (float4*)(S + O_VXYUV);
    P.vrgba = (float4*)(S + O_VRGBA);
    P.vis_idx = (uint16_t*)(S + O_VISI);
    P.vis_depth = (float*)(S + O_VISD);
    P.vis_vloc = (uint16_t*)(S + O_VISV);
    P.tile_count = (uint32_t*)(S + O_TCNT);
    P.tile_wcnt = (uint32_t*)(S + O_TWC);
    P.tile_hist = (uint32_t*)(S + O_THIST);
    P.seg_minmax = (uint32_t*)(S + O_MINMAX);
    P.seg_count = a->out_count;
    P.out_xyuv = (float4*)a->out_xyuv;
    P.out_rgba = (float4*)a->out_rgba;
    P.out_depth = a->out_depth;
    P.ctl = (Ctl*)(S + O_CTL);
    P.accum = (unsigned long long*)(S + O_ACCUM);
    P.inst_begin = 0; P.inst_end = 1;
    P.seg_begin = 0; P.seg_end = 1;
    P.tile_begin = 0; P.tile_end = ntiles; P.tile_alt = ntiles;
    P.vitem_begin = 0; P.vitem_end = nchunks; P.vitem_alt = (flags & SEG_ALTERED) ? 0u : nchunks;
    P.mt_tile_begin = 0; P.mt_tile_end = ntiles > 1 ? ntiles : 0;
    P.mt_seg_begin = 0; P.mt_seg_end = ntiles > 1 ? 1 : 0;
    P.tile_tris = kNaTile;
    P.vchunk = kNaChunk;
    P.has_multi = ntiles > 1 ? 1u : 0u;

    const void* fn = t3d_frame_kernel_ptr();
    NA_CK(raise_smem_limit(fn, d.smem));  // never lowers what a context configured
    uint32_t grid = std::max(1u, std::min(d.max_grid, std::max(ntiles, nchunks)));
    void* args[] = {&P};
    cudaLaunchConfig_t cfg;
    memset(&cfg, 0, sizeof cfg);
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kNaBlock);
    cfg.dynamicSmemBytes = d.smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    NA_CK(cudaLaunchKernelExC(&cfg, fn, args));

    // ---- status ----
    Ctl ctl;
    uint32_t perr = 0;
    NA_CK(cudaMemcpyAsync(&ctl, S + O_CTL, sizeof ctl, cudaMemcpyDeviceToHost, st));
    NA_CK(cudaMemcpyAsync(&perr, S + O_ERR, 4, cudaMemcpyDeviceToHost, st));
    NA_CK(cudaStreamSynchronize(st));
    if (perr) {
        fail(a, "an index is out of range of num_vertices (replaced by 0; output not valid)%s");
        return T3D_E_INVAL;
    }
    if (ctl.err) {
        fail(a, "frame kernel reported error %s", ctl.err == ERR_BARRIER_TIMEOUT ? "barrier timeout" : "internal");
        return ctl.err == ERR_BARRIER_TIMEOUT ? T3D_E_TIMEOUT : T3D_E_CUDA;
    }
    return T3D_OK;
}
