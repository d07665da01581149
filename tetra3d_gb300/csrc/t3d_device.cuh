// t3d_device.cuh -- layouts shared by the host runtime and the frame kernel.
//
// HBM layout of one resident scene (SoA vertex streams, 16-byte records so a
// warp moves whole 128-bit words):
//   va[v] = (px, py, pz, nx)   vb[v] = (ny, nz, u, v)   vc[v] = (r, g, b, a)
//   idx[3t..3t+2]              mesh-absolute vertex indices per triangle
// Per frame the host builds job / instance / segment / tile tables; the kernel
// writes per-model prep records, one record per (render pair, vertex) with the
// cull and emitted attributes, per-tile visible lists (multi-tile segments
// only) and the resident output stream.
#pragma once

#include <stdint.h>

#include "../../include/t3d.h"
#include "t3d_math.cuh"

namespace t3d {

constexpr int kBins = 512;          // sortingTriangleBucket.Resize(512), sortingTriangles.go:166-168
constexpr int kTileMax = 4096;      // largest triangle tile the kernel supports
constexpr int kMaxLights = 128;     // per model light list
constexpr int kMaxWarps = 8;        // block of at most 256 threads

// segment flags
enum : uint32_t {
    SEG_SKIP = 1u << 0,         // ProcessVertices early-out (model.go:604-606)
    SEG_LIT = 1u << 1,          // lighting on for this pair (camera.go:1521-1528)
    SEG_BACKFACE = 1u << 2,     // Material.BackfaceCulling with a material
    SEG_COLORS = 1u << 3,       // mesh has an active vertex colour channel
    SEG_MAT = 1u << 4,          // MeshPart.Material != nil
    SEG_MULTI = 1u << 5,        // segment spans more than one tile
    SEG_WIDE = 1u << 6,         // vertex range above 65536: local vertex offsets do not fit 16 bits
    SEG_TRANSPARENT = 1u << 7,  // drawn in the transparent pass (no depth composite when rasterised)
    SEG_SKINNED = 1u << 14,     // Model.skinned: world-space skinned vertices (records in valt)
    SEG_SHAPES = 1u << 15,      // the mesh has shape keys
    SEG_BILLBOARD = 1u << 16,   // Material.BillboardEnabled on an unskinned model
    SEG_BB_LOCKX = 1u << 17,    // BillboardLockX
    SEG_BB_LOCKY = 1u << 18,    // BillboardLockY
    SEG_BB_LOCKZ = 1u << 19,    // BillboardLockZ
    SEG_BB_CAMUP = 1u << 20,    // BillboardUpDirection == BillboardYUpCameraY
    SEG_UNBB = 1u << 21,        // BillboardedDepthMode == DepthModeUnbillboarded on a billboard
    SEG_SUBDIV = 1u << 22,      // auto-subdivided mesh: triangles are candidates of a subdivision level
    SEG_SNAP = 1u << 23,        // Camera.VertexSnapping > 0
    SEG_NESTED = 1u << 24,      // a light volume of the pair's list has cells that use lights
    SEG_MESHLET = 1u << 25,     // tiles are meshlets: contiguous vertex blocks with 16-bit local indices
    SEG_SINGLE = 1u << 26,      // a meshlet pair of one tile: its output order is its rank order (no
                                // histogram or cross-tile scan)
    SEG_PCORRECT = 1u << 27,    // Camera.PerspectiveCorrectedTextureMapping: each corner also emits
                                // Custom0 = 1 / w (camera.go:1700-1704)
    // parts whose tiles need more than the plain triangle loop (their own loop, queue 7)
    SEG_ALT_TILES = SEG_SKINNED | SEG_SUBDIV,
    // parts whose vertex records need more than the plain loop (their own loop, queue 5)
    // billboards with DepthModeUnbillboarded need the altered loop; others only a staged MVP
    SEG_ALTERED = SEG_SKINNED | SEG_UNBB | SEG_SNAP | SEG_NESTED,
};
constexpr uint32_t kLocalVerts = 65536;  // vertex range of a segment whose offsets fit uint16
__host__ __device__ inline uint32_t seg_sort_mode(uint32_t f) { return (f >> 8) & 3u; }
__host__ __device__ inline uint32_t seg_light_mode(uint32_t f) { return (f >> 10) & 3u; }
__host__ __device__ inline uint32_t seg_lv_mode(uint32_t f) { return (f >> 12) & 3u; }

// model flags
enum : int32_t { MOD_VISIBLE = 1, MOD_FRUSTUM = 2, MOD_SHADELESS = 4, MOD_TRS = 8, MOD_SKINNED = 16 };

struct DevMesh {
    uint32_t vbase;      // first vertex in the scene pool
    uint32_t tbase;      // first triangle in the scene pool
    uint32_t nverts, ntris;
    float dmin[3], dmax[3];  // Mesh.Dimensions
    uint32_t shape_first;    // key k, vertex v: shape pool entry shape_first + k * nverts + v
    uint32_t nkeys;          // shape keys
    uint32_t weight_first;   // key k's weight: shape_w[weight_first + k]
    uint32_t sbase;          // with shape keys: first vertex of the mesh's keyed streams (vaS / vbS)
};

// Resident, animatable model state.
struct DevModel {
    float transform[16];
    float world_rot[16];
    float position[4];
    float scale[4];
    float rotation[16];
    float rotate_step[16];
    float color[4];
    uint32_t mesh;
    int32_t flags;
    uint32_t bone_first;    // skinned: the mesh's joint j uses bone bone_first + j
    uint32_t pad;
};

// A light as one job sees it: beginRender results plus LightVolume geometry.
struct DevLight {
    int32_t type;
    int32_t cnt[3];
    float color[4];
    float energy, range, range2, pad0;
    float wpos[4];     // WorldPosition
    float amb[4];      // AmbientLight.result (color * energy)
    float fwd[4];      // DirectionalLight.workingForward
    float vmin[4], vmax[4], cell[4], offset[4], bias[4];
    uint32_t cell_first;
    uint32_t pad1[3];
};

// Camera block per job (camera.go:638-679, :933-983, :1085-1088, :1337-1341).
struct JobCam {
    float vp[16];
    float pos[4], fwd[4], rgt[4], up[4];
    float sphere_tang, sphere_y, sphere_x, aspect;
    float near_, far_, W, H;
    float halfW, halfH, margin, spread;
    float ortho_scale, snap;  // snap: Camera.VertexSnapping
    float fog_range[2];
    float fog_color[4];
    int32_t perspective, render_depth, persp_correct, fog_on;
    int32_t fog_mode, pad1[3];
};

struct DevJob {
    JobCam cam;
    const float4* va;
    const float4* vb;
    const float4* vc;
    const uint32_t* idx;
    const float* centers;   // tri.Center per pool triangle (3 floats)
    const DevMesh* meshes;
    DevModel* models;
    const float* cells;
    const DevLight* lights;
    const float4* shape_a;  // per (key, vertex): position delta xyz, normal delta x
    const float2* shape_b;  // per (key, vertex): normal delta y, z
    const float4* vaS;      // shape-keyed meshes: the keyed streams, baked per weight set (as va / vb)
    const float4* vbS;
    const float* shape_w;   // key weights
    const uint4* vjoint;    // per pool vertex: four joints (skinned meshes)
    const uint32_t* vjoint8;  // the same packed one byte each, when every joint of the scene is below 256 (else null)
    const float4* vweight;  // per pool vertex: their weights
    const float4* bones;    // 4 rows per bone: Node.boneInfluence
    const float4* sub_info; // auto-subdivided meshes, per pool triangle: its base triangle's Normal and MaxSpan
    const int4* sub_rel;    // (level or -1 for the base, the base's level count, entries back to the base, 0)
    const float* sub_levels;  // AutoSubdivisionLevel: DistanceSquared, MaximumTriangleSize
    uint32_t nsub_levels;
    uint32_t pad_sub;
    const uint32_t* cell_use_off;    // LightVolumeCell.useLights: cell c uses items [off[c], off[c + 1])
    const uint32_t* cell_use_items;  // light indices of the job's light table
};

// Meshlet tiles (SEG_MESHLET). At upload every mesh part is cut into runs of
// consecutive triangles with at most tile_tris triangles and at most mesh_ucap
// distinct vertices; each run is stored once, contiguous and 16-byte aligned:
//   lidx  uint16 x 3 per triangle: slots of its corners in the run's vertex list
//         (padded to 16 bytes)
//   pos   float x 3 per slot (px, py, pz), slots padded to a multiple of 4 (the
//         triangle phase copies lidx + pos)
//   aos   per slot (px, py, pz, nx, ny, nz, u, v) and, when the mesh has colours,
//         (r, g, b, a): 32 or 48 bytes (the rank phase copies this block)
// A meshlet tile's TileDesc keeps t0/t1 (mesh-absolute triangles), the slot count
// in `vmin`, the run's offset in 16-byte units in `vlo` and its device address in
// `vhi` (low) / `pad1` (high). Only the vertex numbering changes: every emitted
// value depends on vertex values alone, so the output is the same as through
// mesh-absolute indices.
__host__ __device__ inline uint32_t mlet_slots4(uint32_t nu) { return (nu + 3u) & ~3u; }
__host__ __device__ inline uint32_t mlet_lidx_bytes(uint32_t nt) { return (6u * nt + 15u) & ~15u; }
__host__ __device__ inline uint32_t mlet_aos_stride(bool colors) { return colors ? 48u : 32u; }
// A meshlet of a shape-keyed mesh as the refill kernel reads it: its place in the pool (16-byte
// units), triangles, slots, and where its slot -> mesh vertex map starts.
struct MletFillDev {
    uint32_t off16, nt, nu, vmap_off;
};
__host__ __device__ inline uint64_t mlet_bytes(uint32_t nt, uint32_t nu, bool colors) {
    return (uint64_t)mlet_lidx_bytes(nt) + (12ull + mlet_aos_stride(colors)) * mlet_slots4(nu);
}

// One (job, model) pair.
struct DevInst {
    uint32_t job, model;
    uint32_t light_off, light_cnt;  // into inst_light_idx
    uint32_t animate;               // apply rotate_step in this launch
    uint32_t pad;
    uint64_t bytes;                 // algorithmic bytes if the model survives culling
};

// Phase-0 output per instance.
struct DevPrep {
    float mvp[16];
    float M[16];
    float dirrot[16];   // DirectionalLight.workingModelRotation (light.go:328)
    float invcam[4];    // model-space camera position (model.go:630)
    float inv_r[16];    // Decompose(Inverted(M)): rotation rows 0..3 (cols 0..2) and p * (1/s) in column 3
    float maxspan;      // Mesh.Dimensions.MaxSpan()
    uint32_t culled;
    uint32_t nl;        // lights staged for the instance in FrameParams.inst_lights (meshlet frames)
    uint32_t pad;
};

// One render pair (model, mesh part) of one job.
struct DevSeg {
    uint32_t inst, job, mesh, flags;
    uint32_t tri_start, tri_count;   // mesh-absolute
    uint32_t vmin, vcount;           // mesh-absolute vertex range the triangles use
    uint32_t vscratch;               // first per-vertex record of this segment
    uint32_t out_base;               // first output triangle slot
    uint32_t tile_first, ntiles;     // global tile numbers
    uint32_t mt_first;               // first multi-tile tile number (SEG_MULTI)
    uint32_t pad[3];
    float mp[4];                     // Model.Color * Material.Color (camera.go:1597-1601)
    float tex_w, tex_h, pad2[2];
};

// Everything the triangle, histogram and rank phases need about one tile, in
// one 64-byte record so a work item starts after a single dependent load.
struct TileDesc {
    uint32_t seg, inst, job, flags;     // render pair, instance, job, segment flags
    uint32_t t0, t1;                    // mesh-absolute triangle range of the tile
    uint32_t tbase;                     // the mesh's first triangle in the scene pool
    uint32_t vmin, vscratch, out_base;  // segment: first vertex, first record, first output slot
    uint32_t mt;                        // multi-tile tile number (SEG_MULTI), else 0
    uint32_t vlo;                       // records [vlo, vhi) cover every vertex of the tile's triangles
    float nearp, farp;                  // job camera near / far planes
    uint32_t vhi;
    uint32_t pad1;
};
constexpr uint32_t kChunkTris = 256;    // triangles per entry of a mesh's vertex-range table
// A pair whose cross-tile scan would run long beside the rest of the phase (more than
// kScanSplit tiles, and more than four times the frame's multi-tile tiles per block) has it
// split into chunks of kScanChunk tiles (one scan work item each), the chunks' bin counts
// summed by the histogram phase. Other pairs keep one item: where the phase has enough other
// work, the chunk sums cost more than the shorter walk saves.
constexpr uint32_t kScanChunk = 32;
constexpr uint32_t kScanSplit = 64;
constexpr uint32_t kNoChunk = 0xFFFFFFFFu;

// Launch control block (zeroed before every launch).
struct Ctl {
    uint32_t bar_count;
    uint32_t bar_gen;
    uint32_t queue[12];
    int32_t err;
    uint32_t err_info;
    unsigned long long bytes;       // algorithmic bytes of surviving models
    uint32_t culled;
    uint32_t live;                  // meshlet tiles with visible triangles (FrameParams.live_tiles)
    uint32_t pad[2];
    unsigned long long t_end[8];    // globaltimer when the last block finished phase k; [7] = kernel start
    unsigned long long busy[8];     // sum over blocks of the time spent inside phase k (ns)
};

enum : int32_t { ERR_NONE = 0, ERR_BARRIER_TIMEOUT = 1, ERR_BAD_INDEX = 2, ERR_LIGHTS = 3, ERR_COPY_TIMEOUT = 4 };

struct FrameParams {
    const DevJob* jobs;
    const DevInst* insts;
    DevPrep* preps;
    const uint32_t* inst_light_idx;
    const DevSeg* segs;
    const TileDesc* tiles;        // per tile
    const TileDesc* mt_desc;      // per multi-tile tile (a copy of its tile's record)
    const uint32_t* mt_segs;      // multi-tile segments, one scan item each (when mt_scan is null)
    const uint32_t* vitem_seg;    // vertex work item -> segment
    const uint32_t* vitem_chunk;  // vertex work item -> chunk of vchunk vertices
    // scratch
    float4* vcull;                // per-vertex records: (cx, cy, clipZ, depth)
    float4* vxyuv;                // emitted screen position + UV
    float4* vrgba;                // emitted colour
    float4* valt;                 // skinned pairs: world-space skinned position per record (depth key)
    float* vinvw;                 // SEG_PCORRECT pairs: 1 / w per record (Custom0); may be null
    // meshlet tiles: per visible entry in the tile's output order, its list entry j (bits 0-10),
    // bin (11-19) and position among the tile's entries of that bin (20-30), from the histogram phase
    uint32_t* vis_rank;
    // per multi-tile tile, tile_tris entries in blockDim/32 regions (one per warp of the
    // triangle phase, tile_tris/(blockDim/32) entries each, filled from the front)
    uint16_t* vis_idx;            // triangle within the tile (SEG_WIDE only)
    float* vis_depth;             // depth key
    uint16_t* vis_vloc;           // 3 vertex offsets within the segment's range (not SEG_WIDE)
    uint32_t* tile_count;         // visible per multi-tile tile
    uint32_t* tile_wcnt;          // per multi-tile tile, kMaxWarps counts: entries in each warp's list region
    uint32_t* tile_hist;          // per multi-tile tile: kBins counters, then bases
    uint32_t* seg_minmax;         // 2 per segment: min bits, max bits
    uint32_t* seg_count;          // visible per segment (output)
    // output stream
    float4* out_xyuv;
    float4* out_rgba;
    float* out_depth;
    float* out_invw;              // Custom0 per corner, written for SEG_PCORRECT pairs; may be null
    Ctl* ctl;
    unsigned long long* accum;    // [0] visible triangles, [1] model bytes; cumulative across frames
    // ranges processed by this launch
    uint32_t inst_begin, inst_end;
    uint32_t seg_begin, seg_end;
    uint32_t tile_begin, tile_end;
    uint32_t tile_alt;                  // tiles of skinned parts: [tile_alt, tile_end)
    uint32_t mt_tile_begin, mt_tile_end;
    uint32_t mt_seg_begin, mt_seg_end;
    uint32_t vitem_begin, vitem_end;
    uint32_t vitem_alt;                 // vertex items of shape-keyed or skinned parts: [vitem_alt, vitem_end)
    uint32_t tile_tris;           // triangles per tile
    uint32_t vchunk;              // vertices per vertex work item
    uint32_t has_multi;           // any multi-tile segment in range
    uint32_t mesh_ucap;           // largest slot count of a meshlet tile
    // meshlet tiles (SEG_MESHLET): tiles [mesh_begin, mesh_end), their multi-tile
    // numbers [mt_mesh_begin, mt_mesh_end); zero ranges when the frame has none
    uint32_t mesh_begin, mesh_end;
    uint32_t mt_mesh_begin, mt_mesh_end;
    uint32_t spin_limit;          // bounded waits: polls before giving up (0 = the default)
    // phases this launch runs (bit 0 prep, 1 vertex records, 2 triangles, 3 histogram, 4 scan,
    // 5 rank + emit), with grid barriers only between phases of the same launch; 0 = all
    uint32_t phases;
    // meshlet frames: per instance, kMaxLights records of 56 bytes (the light list
    // the vertex loop reads, staged once by the prep phase); null otherwise
    float4* inst_lights;
    // per job: algorithmic bytes of its models that survive frustum culling (serving); may be null
    unsigned long long* job_bytes;
    // meshlet frames: the multi-tile numbers of the meshlet tiles with visible triangles, in the
    // order the triangle phase finished them, from index mt_mesh_begin (Ctl.live of them); the
    // histogram and emit phases take only these. Null: every tile of the range.
    uint32_t* live_tiles;
    // scan work items: per item (segment, first chunk, chunk, chunks); a pair of at most
    // kScanChunk tiles is one item of one chunk (first chunk kNoChunk). Null: one item per
    // segment of mt_segs.
    const uint4* mt_scan;
    // per multi-tile tile: its scan chunk (kNoChunk for pairs of one chunk); null: none
    const uint32_t* mt_chunk;
    // per chunk, kBins counts: the sum of its tiles' histograms (zeroed by the prep phase over
    // chunks [chunk_zero_begin, chunk_zero_end))
    uint32_t* chunk_hist;
    uint32_t chunk_zero_begin, chunk_zero_end;
};
// Dense visible list of a meshlet tile i: depth keys at vis_depth + i * tile_tris,
// 3 slots per entry at vis_vloc + 3 * i * tile_tris, tile_count[i] entries.

}  // namespace t3d
