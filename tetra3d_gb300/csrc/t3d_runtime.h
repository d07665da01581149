// t3d_runtime.h -- host-side state behind the C ABI (include/t3d.h).
#pragma once

#include <cuda_runtime.h>

#include <map>
#include <memory>
#include <string>
#include <vector>

#include "t3d_device.cuh"

namespace t3d {

// Grow-only device buffer.
// Grow-only device buffer. In a context with a memory pool (serving slots) it grows by
// stream-ordered allocation on the context's stream, which does not synchronize the
// device the way cudaMalloc / cudaFree do.
struct DevBuf {
    void* ptr = nullptr;
    size_t cap = 0;
    cudaStream_t pooled = nullptr;  // stream of the stream-ordered allocation (null: cudaMalloc)
    int ensure(t3d_ctx* ctx, size_t bytes);
    void release();
};
// Grow-only pinned host buffer.
struct HostBuf {
    void* ptr = nullptr;
    size_t cap = 0;
    int ensure(size_t bytes);
    void release();
};

struct ScenePart {
    t3d_part_desc d;
    uint32_t vmin = 0, vcount = 0;  // vertex range referenced by the part's triangles
};
// One meshlet of a part (t3d_device.cuh): triangles [t0, t0 + nt) of the mesh with
// nu distinct vertices, stored at byte 16 * off16 of the scene's meshlet pool.
struct Meshlet {
    uint32_t t0, nt, nu, off16;
};
// A meshlet of a shape-keyed mesh, for refilling its vertex data from the keyed streams when
// the weights change (the record the refill kernel reads).
using MletFill = MletFillDev;
struct SceneMesh {
    uint32_t vbase = 0, tbase = 0, nverts = 0, ntris = 0;
    bool colors = false;
    float dmin[3], dmax[3];
    std::vector<ScenePart> parts;
    // per kChunkTris triangles: smallest and largest vertex index they use (prefetch ranges)
    std::vector<uint32_t> chunk_lo, chunk_hi;
    uint32_t nkeys = 0, shape_first = 0, weight_first = 0;  // shape keys
    uint32_t sbase = 0;                                     // first vertex of the keyed streams
    bool skin = false;                                      // joints and weights present
    uint32_t max_joint = 0;
    bool subdiv = false;  // auto-subdivided: parts list each triangle followed by its subdivision levels
    std::vector<std::vector<Meshlet>> mparts;  // per part: its meshlets (empty: the part has none)
    uint32_t kfill_first = 0, kfill_count = 0;  // shape-keyed mesh: its MletFill records in the scene's list
};
struct SceneModel {
    t3d_model_desc d;  // host mirror (rotation advanced with every animated frame)
};
struct Scene {
    std::vector<SceneMesh> meshes;
    std::vector<SceneModel> models;
    std::vector<t3d_light_desc> lights;
    std::vector<std::vector<uint32_t>> lists;
    uint64_t nverts = 0, ntris = 0;
    // versions (unique across scenes): struct_ver changes with anything the launch
    // tables are built from except transforms; model_ver with any model write
    uint64_t struct_ver = 0, model_ver = 0;
    DevBuf va, vb, vc, idx, centers, dmeshes, dmodels, cells;
    DevBuf shape_a, shape_b, shape_w, vjoint, vweight, bones;
    DevBuf vaS, vbS;  // keyed streams of the shape-keyed meshes (baked per weight set)
    bool joint8 = false;  // vjoint holds four 8-bit joints per vertex (every joint below 256)
    DevBuf sub_info, sub_rel, sub_levels, cell_use_off, cell_use_items;
    DevBuf mlet;                         // meshlet pool
    DevBuf mlet_kfill, mlet_vmap;        // shape-keyed meshes' meshlets: MletFill records, slot -> vertex maps
    uint32_t mlet_T = 0, mlet_U = 0;     // triangle and vertex budgets the meshlets were cut for (0: none)
    std::vector<char> light_uses;    // per light: a volume whose cells use lights
    std::vector<char> light_nested;  // per light: used by some cell (cannot become a volume)
    std::vector<uint32_t> cell_use_host;  // host copy of the cell use offsets
    bool cell_uses_between(uint64_t c0, uint64_t c1) const {
        return c1 < cell_use_host.size() && cell_use_host[c1] > cell_use_host[c0];
    }
    uint32_t num_bones = 0, num_keys = 0, num_sub_levels = 0, num_cells = 0;
    uint64_t device_bytes() const {
        return va.cap + vb.cap + vc.cap + idx.cap + centers.cap + dmeshes.cap + dmodels.cap + cells.cap + shape_a.cap + vaS.cap + vbS.cap +
               shape_b.cap + shape_w.cap + vjoint.cap + vweight.cap + bones.cap + sub_info.cap + sub_rel.cap +
               sub_levels.cap + cell_use_off.cap + cell_use_items.cap + mlet.cap + mlet_kfill.cap + mlet_vmap.cap;
    }
    void release() {
        mlet.release(); mlet_kfill.release(); mlet_vmap.release(); mlet_T = mlet_U = 0;
        sub_info.release(); sub_rel.release(); sub_levels.release(); cell_use_off.release(); cell_use_items.release();
        shape_a.release(); shape_b.release(); vaS.release(); vbS.release(); shape_w.release(); vjoint.release(); vweight.release(); bones.release();
        va.release(); vb.release(); vc.release(); idx.release(); centers.release();
        dmeshes.release(); dmodels.release(); cells.release();
    }
};

// Tables of one frame (host side).
struct FrameTables {
    std::vector<DevJob> jobs;
    std::vector<Scene*> job_scene;
    std::vector<uint32_t> job_light_base, job_seg_end;
    std::vector<DevLight> lights;
    std::vector<DevInst> insts;
    std::vector<uint32_t> inst_light_idx;
    std::vector<DevSeg> segs;
    std::vector<t3d_segment_info> seg_info;
    std::vector<uint32_t> seg_mt_seg;
    std::vector<TileDesc> tiles, mt_desc;
    // cross-tile scan work items (segment, first chunk, chunk, chunks) and each multi-tile
    // tile's scan chunk (kNoChunk in pairs of one chunk); chunks numbered [0, nchunks)
    std::vector<uint4> mt_scan;
    std::vector<uint32_t> mt_chunk;
    uint32_t nchunks = 0;
    std::vector<uint32_t> vitem_seg, vitem_chunk, seg_vitem_first;
    uint64_t nscratch = 0, nslots = 0;
    bool any_skinned = false, any_altered = false, any_mesh = false;
    bool any_pcorrect = false;             // a job's camera uses perspective-corrected texture mapping
    uint32_t tile_alt = 0, vitem_alt = 0;  // first tile of a skinned part / vertex item of an altered part
    uint32_t tile_mesh = 0;                // first meshlet tile (tiles: record-path plain | record-path altered | meshlet)
    uint32_t mt_mesh = 0;                  // first meshlet multi-tile number (mt_desc: record path | meshlet)
    void clear() {
        jobs.clear(); job_scene.clear(); job_light_base.clear(); job_seg_end.clear(); lights.clear();
        insts.clear(); inst_light_idx.clear(); segs.clear(); seg_info.clear();
        seg_mt_seg.clear(); tiles.clear(); mt_desc.clear(); mt_scan.clear(); mt_chunk.clear(); nchunks = 0;
        vitem_seg.clear(); vitem_chunk.clear(); seg_vitem_first.clear();
        nscratch = 0; nslots = 0; any_skinned = false; any_altered = false; any_mesh = false; any_pcorrect = false;
        tile_alt = 0; vitem_alt = 0;
        tile_mesh = 0; mt_mesh = 0;
    }
};

}  // namespace t3d

struct t3d_raster_state;
void t3d_raster_release(struct t3d_ctx* ctx);

struct t3d_ctx {
    int device = 0;
    std::string err;
    cudaStream_t stream = nullptr;
    cudaStream_t last_stream = nullptr;
    int num_sms = 0;
    uint32_t tile_tris = 2048, vchunk = 4096, block_threads = 256;
    uint32_t max_grid = 0;   // co-resident blocks for the current tuning
    size_t smem_bytes = 0;
    // the kernel instantiation for frames with meshlet tiles
    uint32_t mesh_ucap = 0;       // distinct vertices per meshlet (0: meshlets off)
    uint32_t max_grid_mesh = 0;
    size_t smem_mesh = 0;
    bool use_meshlets = true;     // t3d_set_meshlets: 0 sends every pair through the per-vertex record path
    // batched frames as one launch per phase (t3d_set_split_phases); per phase kernel
    // ([0] frames without meshlet tiles, [1] with; phases prep .. rank + emit): its shared
    // memory and its co-resident blocks
    bool split_phases = true;
    size_t phase_smem[2][6] = {};
    uint32_t phase_grid[2][6] = {};
    uint32_t spin_limit = 0;      // bounded device waits (0: the kernel's default)
    uint32_t next_scene = 1;
    std::map<uint32_t, std::unique_ptr<t3d::Scene>> scenes;
    t3d_ctx* scene_owner = nullptr;  // serving slots render the parent context's scenes
    std::map<uint32_t, std::unique_ptr<t3d::Scene>>& scene_map() { return scene_owner ? scene_owner->scenes : scenes; }
    t3d::FrameTables tables;
    t3d::FrameParams params;
    const t3d::DevInst* insts_noanim = nullptr;  // same instances with animate = 0
    t3d::HostBuf table_host, readback, model_host;
    // deferred read-back of one frame (t3d_frame_readback / t3d_frame_collect): its pinned copy of
    // the per-pair counts and control blocks, the event after the copy, and the frame's sizes
    t3d::HostBuf readback2;
    cudaEvent_t ev_readback = nullptr;
    bool rb2_pending = false;
    size_t rb2_nseg = 0;
    uint32_t rb2_nctl = 0, rb2_launches = 0;
    uint64_t rb2_total = 0, rb2_h2d = 0;
    // launch tables of the last render (reused while nothing they depend on changed)
    std::vector<unsigned char> table_sig;
    std::vector<uint64_t> table_model_vers;
    bool tables_ok = false;
    bool order_dep = true;   // the draw order depends on model transforms (transparents, depth off)
    cudaEvent_t ev_upload = nullptr;  // the last table upload has left the pinned staging buffer
    cudaEvent_t ev_models = nullptr;  // the last model write has reached the device (and left its staging)
    struct t3d_raster_state* raster = nullptr;  // images and scratch of t3d_frame_raster
    t3d::DevBuf valt, inst_lights, job_bytes, vis_rank, vinvw, out_invw, live_tiles;
    bool want_job_bytes = false;  // serving slots: per-job algorithmic bytes (FrameParams.job_bytes)
    std::vector<unsigned long long> job_bytes_host;  // their values, read back by t3d_frame_sync
    uint32_t grid_share = 1;      // serving slots: launches use 1/grid_share of the co-resident blocks
    cudaMemPool_t pool = nullptr; // serving slots: the server's pool for stream-ordered buffer growth
    t3d::DevBuf table_dev, ctl, preps, vcull, vxyuv, vrgba, vis_idx, vis_depth, vis_vloc, tile_count, tile_wcnt, tile_hist,
        chunk_hist, seg_minmax, seg_count, out_xyuv, out_rgba, out_depth, accum;
    uint32_t nctl = 0;
    uint64_t last_h2d = 0;
    uint32_t launches = 0;
    uint32_t last_grid = 0;
    uint32_t phase_grid_used[6] = {};  // blocks of the last launch that ran each phase
    bool frame_pending = false;
    bool frame_valid = false;
    t3d_stats stats{};
    // CUDA graph of one batched frame
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    cudaEvent_t ev_done = nullptr;
};

namespace t3d {
void set_err(t3d_ctx* c, const char* fmt, ...);
cudaError_t raise_smem_limit(const void* fn, size_t bytes);
void build_camera(const t3d_camera_desc& d, JobCam& c);
void build_light(const t3d_light_desc& d, DevLight& L);
int scene_upload(t3d_ctx* ctx, const t3d_scene_desc* d, uint32_t* out);
int scene_write_models(t3d_ctx* ctx, Scene* sc, uint32_t first, const t3d_model_desc* models, uint32_t n);
int build_frame(t3d_ctx* ctx, const t3d_job_desc* jobs, uint32_t njobs, int animate);
uint32_t billboard_flags(const t3d_material& mat, bool skinned);
uint64_t next_version();
int upload_frame(t3d_ctx* ctx, cudaStream_t st);
int launch_frame(t3d_ctx* ctx, int mode, cudaStream_t st);
int configure(t3d_ctx* ctx);
int bake_shapes(t3d_ctx* ctx, Scene* sc, uint32_t mesh);
int build_meshlets(t3d_ctx* ctx, Scene* sc, uint32_t T, uint32_t U);
int fill_keyed_meshlets(t3d_ctx* ctx, Scene* sc, uint32_t m);
}  // namespace t3d
