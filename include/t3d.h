/*
 * t3d.h -- C ABI of the GB300 vertex stage for Tetra3D.
 *
 * This library replaces the software vertex stage that Tetra3D runs inside
 * Camera.Render: per (model, mesh part) it transforms the mesh by the model's
 * MVP, rejects triangles (near/far, screen +-0.5, 2D-cross backface), keys and
 * bucket-sorts the survivors, lights every emitted vertex and writes the
 * per-corner stream that Tetra3D hands to ebiten.DrawTrianglesShader.
 *
 * Reference interface replaced (file:line in SolarLune/tetra3d):
 *   Camera.Render               camera.go:1269-2114  -> t3d_render / t3d_render_jobs
 *   render closure              camera.go:1507-1827  -> device phases (vertex, triangle, emit)
 *   Model.ProcessVertices       model.go:600-995     -> device vertex + triangle phases
 *   sortingTriangleBucket       sortingTriangles.go  -> device segmented 512-bin counting sort
 *   ILight.beginModel / Light   light.go:110-663     -> device model-prep + vertex phases
 *   flush (vertex lists)        camera.go:1829-2048  -> t3d_frame_* (resident device buffers),
 *                                                       t3d_frame_raster (depth + colour passes)
 *   Model.skinVertex, shape keys model.go:559-596,   -> device vertex phase
 *                               mesh.go:796-822
 *   billboarding                model.go:634-703     -> device vertex phase
 *   Mesh.SetAutoSubdivide,      mesh.go:447-490,     -> t3d_scene_upload (subdivision) and
 *   Triangle.handleSubdivision  mesh.go:1877-1949       the device triangle phase (level choice)
 *   Model.DynamicBatchAdd       model.go:210-245,    -> t3d_model_desc.batched (draw order, flushes)
 *                               camera.go:2068-2093
 *
 * Conventions
 *  - Matrices are Tetra3D Matrix4 values: 16 floats, row-major, row vectors
 *    (v' = v * M), translation in row 3 (matrix.go:10, :619-637).
 *  - Every function returns an int status: T3D_OK (0) or a negative T3D_E_*.
 *    t3d_last_error() returns a message for the last failure on that context.
 *    Nothing aborts the process.
 *  - Host arrays passed in are copied during the call; the library keeps no
 *    pointer to caller memory (safe for cgo).
 *  - Device outputs are owned by the context and stay valid until the next
 *    render on that context.
 *  - One context per host thread. Calls on one context are not re-entrant.
 */
#ifndef T3D_H
#define T3D_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define T3D_OK          0
#define T3D_E_INVAL    -1   /* bad argument (index out of range, bad enum, null) */
#define T3D_E_OOM      -2   /* device or host allocation failed */
#define T3D_E_ADMIT    -3   /* serving: request does not fit the HBM budget */
#define T3D_E_TIMEOUT  -4   /* a bounded device wait gave up */
#define T3D_E_CUDA     -5   /* CUDA runtime error */
#define T3D_E_NOTFOUND -6   /* unknown handle */
#define T3D_E_BUSY     -7   /* serving: queue full */

/* ---- enums mirroring material.go / node.go ----------------------------- */
/* material.go:9-13 */
#define T3D_SORT_BACK_TO_FRONT 0
#define T3D_SORT_FRONT_TO_BACK 1
#define T3D_SORT_NONE          2
/* material.go:15-28 */
#define T3D_TRANSPARENCY_AUTO        0
#define T3D_TRANSPARENCY_OPAQUE      1
#define T3D_TRANSPARENCY_ALPHA_CLIP  2
#define T3D_TRANSPARENCY_TRANSPARENT 3
/* material.go:34-38 */
#define T3D_LIGHTING_DEFAULT       0
#define T3D_LIGHTING_FIXED_NORMALS 1
#define T3D_LIGHTING_DOUBLE_SIDED  2
/* material.go:50-55 */
#define T3D_LV_PER_VERTEX              0
#define T3D_LV_PER_VERTEX_WITH_NORMAL  1
#define T3D_LV_PER_OBJECT              2
#define T3D_LV_OFF                     3
/* BillboardUpDirection, material.go:29-32 */
#define T3D_BILLBOARD_UP_GLOBAL_Y 0
#define T3D_BILLBOARD_UP_CAMERA_Y 1
/* BillboardedDepthMode, material.go:45-48 */
#define T3D_DEPTH_DEFAULT        0
#define T3D_DEPTH_UNBILLBOARDED  1
/* light kinds: AmbientLight, PointLight, DirectionalLight, LightVolume (light.go) */
#define T3D_LIGHT_AMBIENT     0
#define T3D_LIGHT_POINT       1
#define T3D_LIGHT_DIRECTIONAL 2
#define T3D_LIGHT_VOLUME      3
/* world.go:7-11 */
#define T3D_FOG_ADD       0
#define T3D_FOG_SUB       1
#define T3D_FOG_OVERWRITE 2

/* render modes */
#define T3D_MODE_PLAIN   0   /* one launch per model (the reference's per-model loop) */
#define T3D_MODE_BATCHED 1   /* all models of all jobs in one frame: a persistent launch per phase */

/* Maximum lights one model may be lit by (length of its light list). */
#define T3D_MAX_LIGHTS_PER_MODEL 128

/* ---- input descriptors -------------------------------------------------- */

/* Material fields read by the vertex stage (material.go:64-125, defaults :146-167).
 * present = 0 stands for MeshPart.Material == nil. */
typedef struct t3d_material {
    float   color[4];          /* Material.Color */
    float   tex_w, tex_h;      /* texture size in px if UseTexture && Texture != nil, else 0 */
    int32_t present;
    int32_t backface_culling;  /* default 1 */
    int32_t sort_mode;         /* T3D_SORT_* */
    int32_t lighting_mode;     /* T3D_LIGHTING_* */
    int32_t lv_shading_mode;   /* T3D_LV_* */
    int32_t shadeless;
    int32_t visible;           /* default 1 */
    int32_t transparency_mode; /* T3D_TRANSPARENCY_* */
    int32_t blend_source_over; /* 1 when Blend == ebiten.BlendSourceOver (default) */
    int32_t render_order;
    /* Billboarding (model.go:634-688): the part turns to face the camera
     * (NewMatrix4LookAt from the model's world position), optionally with
     * axes locked; with T3D_DEPTH_UNBILLBOARDED the depth written when
     * RenderDepth is on is that of the unturned part (model.go:698-803). */
    int32_t billboard;         /* Material.BillboardEnabled */
    int32_t billboard_lock[3]; /* BillboardLockX, BillboardLockY, BillboardLockZ */
    int32_t billboard_up;      /* T3D_BILLBOARD_UP_* */
    int32_t billboard_depth;   /* T3D_DEPTH_* */
    /* Rasteriser only (t3d_frame_raster): the material's texture when UseTexture is set
     * (0 = the default white image, k = texture k - 1 of t3d_raster_set_textures), its
     * TextureFilterMode (0 nearest, 1 bilinear), TextureMapMode (0 UV, 1 screen) and
     * TextureMapScreenSizeMultiplierW/H (the reference's default is 1, 1). */
    uint32_t texture;
    int32_t  texture_filter;
    int32_t  texture_map_mode;
    float    texture_map_scale[2];
    int32_t  reserved_tex;
} t3d_material;

/* A MeshPart (mesh.go:2183-2190): a contiguous triangle range with one material. */
typedef struct t3d_part_desc {
    uint32_t     tri_start;    /* first triangle (mesh-absolute) */
    uint32_t     tri_count;
    t3d_material mat;
} t3d_part_desc;

/* A Mesh (mesh.go:260-302) as SoA vertex streams. Indices are mesh-absolute
 * (Triangle.VertexIndexA/B/C). colors is the active vertex colour channel,
 * NULL when VertexActiveColorChannel < 0. */
typedef struct t3d_mesh_desc {
    const float*         positions;   /* 3 * num_vertices */
    const float*         normals;     /* 3 * num_vertices */
    const float*         uvs;         /* 2 * num_vertices */
    const float*         colors;      /* 4 * num_vertices or NULL */
    const uint32_t*      indices;     /* 3 * num_triangles */
    const t3d_part_desc* parts;
    uint32_t             num_vertices;
    uint32_t             num_triangles;
    uint32_t             num_parts;
    int32_t              has_dimensions; /* 0: Dimensions computed like Mesh.UpdateDimensions */
    float                dim_min[3];     /* Mesh.Dimensions when has_dimensions */
    float                dim_max[3];
    /* Shape keys (Mesh.VertexPositionWithShapeKeys / VertexNormalWithShapeKeys,
     * mesh.go:796-822): per key, a position and a normal delta per vertex, added
     * key by key times the key's weight (t3d_scene_set_shape_weights; initial
     * weights here). NULL / 0 when the mesh has none. */
    const float*         shape_positions; /* 3 * num_vertices * num_shape_keys */
    const float*         shape_normals;   /* 3 * num_vertices * num_shape_keys */
    const float*         shape_weights;   /* num_shape_keys */
    uint32_t             num_shape_keys;
    /* Skinning (Model.skinVertex, model.go:559-596): four joint slots per vertex and
     * their weights (Mesh.VertexWeights); a skinned model maps joint j to scene bone
     * bone_first + j. NULL when no model skins this mesh. */
    /* Mesh.SetAutoSubdivide(true) (mesh.go:447-490): at upload every part triangle
     * longer than the smallest MaximumTriangleSize of the scene's subdivision levels
     * is split into up to max_subdivisions levels of 4-way subdivisions (new vertices
     * appended after num_vertices); each frame a triangle draws the level its
     * distance to the model-space camera selects (Triangle.handleSubdivision,
     * mesh.go:1877-1949). Not with shape keys or on skinned models. */
    int32_t              auto_subdivide;
    const uint32_t*      joints;          /* 4 * num_vertices */
    const float*         weights;         /* 4 * num_vertices */
} t3d_mesh_desc;

/* A Model (model.go:20-61). Either `transform` holds Model.Transform() and
 * `world_rotation` holds Model.WorldRotation() (use_trs = 0), or the library
 * builds the transform itself every frame as Scale * Rotation * Translate
 * from position/scale/rotation (use_trs = 1, a parentless node, node.go:572-608).
 * rotate_step is applied as rotation = rotate_step * rotation before each
 * animated frame (Node.Rotate, node.go:1039-1047); identity when static. */
typedef struct t3d_model_desc {
    uint32_t mesh;             /* index into the scene's mesh array */
    int32_t  visible;
    int32_t  frustum_culling;  /* default 1 */
    int32_t  shadeless;
    int32_t  light_list;       /* -1: the scene light list (list 0); else LightGroup list index */
    int32_t  use_trs;
    float    color[4];         /* Model.Color */
    float    transform[16];
    float    world_rotation[16];
    float    position[3];
    float    scale[3];
    float    rotation[16];
    float    rotate_step[16];
    /* Model.skinned: vertices are skinned by the scene's bone influences (Node.boneInfluence,
     * set with t3d_scene_set_bones) instead of transformed by the model matrix; the model
     * transform still places its frustum sphere and its point-light range test. */
    int32_t  skinned;
    uint32_t bone_first;       /* the mesh's joint j uses scene bone bone_first + j */
    /* Dynamic batching (Model.DynamicBatchAdd, model.go:210-245): batched = 1 makes this
     * model a member of model batch_owner's batch under that model's mesh part
     * batch_part. Members draw only inside the batch: in the owner's place in the draw
     * order, sorted far to near from the camera, each with its own frustum culling and
     * all of its parts, in one flush (camera.go:1343-1457, :2068-2093); an owner draws
     * no mesh of its own. */
    int32_t  batched;
    uint32_t batch_owner;
    uint32_t batch_part;
    uint32_t reserved;
} t3d_model_desc;

/* A light (light.go). transform = the light node's Transform(), world_rotation =
 * its WorldRotation(). Volume fields describe a LightVolume (light.go:377-680):
 * its Dimensions, cell sizes, cell counts (as LightVolumeResize computed them),
 * offset, light bias and the index of its first cell colour (RGBA) in the
 * scene's cell table; the lights its cells use are in the scene desc. */
typedef struct t3d_light_desc {
    int32_t  type;             /* T3D_LIGHT_* */
    int32_t  cell_count[3];
    float    color[4];
    float    energy;
    float    range;            /* PointLight.Range(); 0 = inverse-square falloff */
    float    transform[16];
    float    world_rotation[16];
    float    vol_min[3];
    float    vol_max[3];
    float    cell_size[3];
    float    offset[3];
    float    bias[3];
    uint32_t cell_first;
} t3d_light_desc;

/* Everything the vertex stage reads from a Scene. Light list 0 is the scene
 * light list in Render order: [World.AmbientLight if LightingOn and visible] +
 * visible lights in tree order (camera.go:1275-1303). Lists 1.. are LightGroups
 * (lightGroup.go), used whole when a model names them. */
typedef struct t3d_scene_desc {
    const t3d_mesh_desc*  meshes;
    const t3d_model_desc* models;
    const t3d_light_desc* lights;
    const float*          volume_cells;   /* RGBA per cell */
    const uint32_t*       list_offsets;   /* num_lists + 1 */
    const uint32_t*       list_items;     /* light indices */
    uint32_t              num_meshes;
    uint32_t              num_models;
    uint32_t              num_lights;
    uint32_t              num_volume_cells;
    uint32_t              num_lists;
    uint32_t              num_bones;
    const float*          bones;          /* 16 per bone: initial Node.boneInfluence matrices */
    /* Library.autosubdivisionLevels (library.go:206-209): DistanceSquared and
     * MaximumTriangleSize per level; max_subdivisions = maxAutoSubdivisionCount
     * (0: the library default, 3). */
    const float*          subdivision_levels;     /* 2 * num_subdivision_levels */
    uint32_t              num_subdivision_levels;
    uint32_t              max_subdivisions;
    /* LightVolumeCell.useLights (light.go:1381, :1509-1522): lights applied, in list
     * order, to a vertex that falls into a cell in the per-vertex shading modes, before the
     * cell's own colour (light.go:646-656). Cell c uses cell_use_items[cell_use_offsets[c] ..
     * cell_use_offsets[c + 1]) (ambient, point or directional lights of this scene). NULL:
     * no cell uses lights. Job light masks do not apply to them. */
    const uint32_t*       cell_use_offsets;       /* num_volume_cells + 1 */
    const uint32_t*       cell_use_items;
} t3d_scene_desc;

/* Camera + World settings read by Render (camera.go:256-321, world.go:25-39).
 * Clear() must have run for the reference; here the basis comes from
 * world_rotation directly (camera.go:1085-1088). */
typedef struct t3d_camera_desc {
    float   transform[16];       /* Camera.Transform() */
    float   world_rotation[16];  /* Camera.WorldRotation() */
    int32_t width, height;
    int32_t perspective;         /* default 1 */
    int32_t render_depth;        /* default 1 */
    int32_t perspective_corrected;
    int32_t lighting_on;         /* World.LightingOn (0 also when World == nil) */
    int32_t fog_on;              /* World.FogOn */
    int32_t fog_mode;            /* T3D_FOG_* */
    float   fov_y;               /* degrees, default 60 */
    float   near_plane;          /* default 0.1 */
    float   far_plane;           /* default 100 */
    float   ortho_scale;         /* default 20 */
    float   depth_margin;        /* default 0.04 */
    float   fog_range[2];
    float   fog_color[4];
    /* Camera.MaxLightCount (camera.go:1474-1497): > 0 keeps that many lights of the scene
     * list (list 0) after a stable sort by kind (ambient, directional) then squared
     * distance to the focus point; LightGroups are not affected. 0 = all lights. */
    int32_t max_light_count;
    int32_t focus_set;           /* MaxLightCountFocusPoint != nil */
    float   focus[3];            /* its WorldPosition(); otherwise the camera's is used */
    float   vertex_snapping;     /* Camera.VertexSnapping: > 0 rounds clip X, Y, Z to this grid (model.go:813-818) */
} t3d_camera_desc;

/* One unit of rendering work: one camera over one resident scene, optionally
 * restricted to a subset of the scene's lights (bit i of light_mask keeps
 * light i; the mask filters every light list; all ones = no restriction). */
typedef struct t3d_job_desc {
    uint32_t        scene;
    uint32_t        reserved;
    uint64_t        light_mask[2];   /* lights 0..127 */
    t3d_camera_desc camera;
} t3d_job_desc;

/* ---- outputs ------------------------------------------------------------- */

/* The emitted stream. Per visible triangle, 3 corners in reference emit order;
 * per corner: xyuv = (DstX, DstY, SrcX, SrcY), rgba = colour vertex colour,
 * depth = depth vertex colour (camera.go:1646-1820). Segments are the render
 * pairs (model, mesh part) in Render's draw order: solids then transparents
 * (camera.go:2050-2109). Segment s owns triangles [seg_base[s], seg_base[s] +
 * seg_capacity[s]) of the stream; its seg_count[s] visible triangles are
 * written densely from seg_base[s]. All pointers are device pointers. */
typedef struct t3d_frame_view {
    float*    xyuv;          /* float4 per corner */
    float*    rgba;          /* float4 per corner */
    float*    depth;         /* float per corner */
    uint32_t* seg_base;      /* first triangle slot per segment */
    uint32_t* seg_count;     /* visible triangles per segment (device) */
    uint32_t  num_segments;
    uint32_t  reserved;
    uint64_t  capacity_tris; /* total triangle slots */
} t3d_frame_view;

/* Host-side segment description (same order as the device arrays). */
typedef struct t3d_segment_info {
    uint32_t job;
    uint32_t model;
    uint32_t part;
    uint32_t base;           /* triangle slot */
    uint32_t capacity;       /* triangles in the part */
    uint32_t count;          /* visible triangles (valid after t3d_frame_sync) */
    uint32_t draw;           /* flush this pair belongs to: pairs of one dynamic batch share it */
    uint32_t draw_transparent; /* that flush is in the transparent pass (no depth composite) */
} t3d_segment_info;

typedef struct t3d_stats {
    uint64_t visible_tris;   /* DebugInfo.drawnTris of the last frame */
    uint64_t total_tris;     /* DebugInfo.totalTris */
    uint32_t drawn_parts;    /* segments with at least one visible triangle */
    uint32_t total_parts;
    uint32_t culled_models;  /* models rejected by SphereInFrustum */
    uint32_t launches;       /* kernel launches of the last frame */
    uint64_t algorithmic_bytes; /* 48V+12T of surviving models + 108*visible + 64*models + 48*lights*lit models */
    uint64_t scratch_bytes;  /* device scratch held by the context */
    uint64_t h2d_bytes;      /* host-to-device bytes of the last render call (tables) */
    uint64_t d2h_bytes;      /* device-to-host bytes of the last t3d_frame_sync */
    double   phase_us[7];    /* batched launch: model prep, vertex, triangles, histogram, scan, rank + emit, (unused) */
    double   phase_busy[7];  /* same phases: mean time a block spent working in the phase (us) */
} t3d_stats;

typedef struct t3d_ctx t3d_ctx;

/* ---- context --------------------------------------------------------------- */
int         t3d_create(int device, t3d_ctx** out);
int         t3d_destroy(t3d_ctx* ctx);
const char* t3d_last_error(const t3d_ctx* ctx);
/* Tuning knobs (0 keeps the current value): triangles per tile (power of two,
 * 256..4096), vertices per vertex-phase work item (32..2^20), threads per block
 * (128 or 256). */
int         t3d_set_tuning(t3d_ctx* ctx, uint32_t tile_tris, uint32_t vertex_chunk, uint32_t block_threads);
/* Route of the vertex stage (no reference counterpart: the reference has one CPU
 * path). enable = 1 (the default): render pairs that need nothing beyond the plain
 * vertex loop (no skinning, auto-subdivision, vertex snapping, lights used by volume
 * cells or unbillboarded depth; shape keys allowed) read their part's meshlets --
 * runs of consecutive triangles with their distinct vertices stored contiguously, cut
 * at scene upload (a shape-keyed mesh's from its keyed vertices, refilled when its
 * weights change) -- and keep every per-vertex intermediate in shared memory.
 * enable = 0: every pair writes and reads per-vertex records in device memory. The
 * emitted stream is the same bit for bit either way. */
int         t3d_set_meshlets(t3d_ctx* ctx, int enable);
/* Launch shape of a frame (no reference counterpart: the reference has one CPU
 * path). mode = 1 (the default): one persistent launch per phase (model prep, vertex
 * records, triangles, histogram, scan, rank + emit), each kernel compiled with its
 * own register budget and sized to its own co-resident blocks, the launch boundary
 * ordering the phases. mode = 0: a batched frame in one cooperative persistent
 * launch whose phases are separated by grid barriers. The emitted stream is the same
 * bit for bit either way; the autotuner picks the faster. */
int         t3d_set_split_phases(t3d_ctx* ctx, int mode);
/* Bounded device waits (grid barriers, bulk-copy waits): polls before the frame
 * gives up and t3d_frame_sync returns T3D_E_TIMEOUT (0 = the default, seconds).
 * Meant for tests of the timeout path; the context stays usable and the next
 * frame with the default renders normally. */
int         t3d_set_wait_limit(t3d_ctx* ctx, uint32_t polls);

/* ---- resident scenes --------------------------------------------------------- */
/* Uploads meshes, models and lights to the device. Replaces Tetra3D's
 * per-frame reads of Mesh/Model/Light state. */
int t3d_scene_upload(t3d_ctx* ctx, const t3d_scene_desc* desc, uint32_t* scene_out);
int t3d_scene_release(t3d_ctx* ctx, uint32_t scene);
/* Per-frame model update (Node.Transform changes, visibility, colour, ...): the
 * n model descs of models [first, first+n). The descs are copied during the call;
 * the device copy is queued behind the frames already issued, so the call does
 * not wait for them and the next render sees the new models. */
int t3d_scene_set_models(t3d_ctx* ctx, uint32_t scene, uint32_t first,
                         const t3d_model_desc* models, uint32_t n);
/* Reads back the current (possibly animated) per-model transforms, 16 floats each. */
int t3d_scene_get_transforms(t3d_ctx* ctx, uint32_t scene, float* transforms_out, uint32_t n);
/* Device bytes held by a scene's resident data. */
int t3d_scene_bytes(t3d_ctx* ctx, uint32_t scene, uint64_t* bytes_out);
/* Bone influence matrices [first, first + n) of a scene (16 floats each, Node.boneInfluence,
 * node.go), as an animation player updates them every frame. */
int t3d_scene_set_bones(t3d_ctx* ctx, uint32_t scene, uint32_t first, const float* influences, uint32_t n);
/* Shape-key weights of one mesh of a scene (ShapeKey.weight, mesh.go). The mesh's keyed
 * vertices (shared by all its models) and its meshlets' vertex data are recomputed on the
 * device before this returns. */
int t3d_scene_set_shape_weights(t3d_ctx* ctx, uint32_t scene, uint32_t mesh, const float* weights, uint32_t n);
/* Lights [first, first + n) of a scene: moved, recoloured, re-ranged or of another
 * kind, as Camera.Render reads them anew every frame (camera.go:1269-1300,
 * light.go beginRender). The next render rebuilds its light tables; a
 * captured graph is dropped (capture again). */
int t3d_scene_set_lights(t3d_ctx* ctx, uint32_t scene, uint32_t first, const t3d_light_desc* lights, uint32_t n);

/* ---- rendering --------------------------------------------------------------- */
/* Camera.Render over one scene: enqueue on `stream` (a cudaStream_t, NULL =
 * the context's stream). animate = 1 applies every model's rotate_step first. */
int t3d_render(t3d_ctx* ctx, uint32_t scene, const t3d_camera_desc* cam,
               int mode, int animate, void* stream);
/* Several independent jobs in one frame (serving, multi-view). */
int t3d_render_jobs(t3d_ctx* ctx, const t3d_job_desc* jobs, uint32_t num_jobs,
                    int mode, int animate, void* stream);
/* Waits for the last frame and fills the segment counts. */
int t3d_frame_sync(t3d_ctx* ctx, t3d_stats* stats_out);
/* Deferred read-back for a pipelined render loop (no reference counterpart: the
 * reference renders and flushes frame by frame). t3d_frame_readback enqueues a copy
 * of the last frame's per-pair counts and launch status after it on its stream and
 * returns; the caller may then push the next frame's models and render it, and
 * t3d_frame_collect waits for the copy and returns the read-back frame's stats (the
 * same as t3d_frame_sync would have, without updating the context's per-pair counts,
 * which belong to the latest frame). One read-back can be in flight per context. */
int t3d_frame_readback(t3d_ctx* ctx);
int t3d_frame_collect(t3d_ctx* ctx, t3d_stats* stats_out);
/* Cumulative counters since t3d_create over every frame (graph replays
 * included): visible triangles and the 48V+12T+64+48L bytes of models that
 * survived frustum culling. Waits for the last frame. */
int t3d_frame_counters(t3d_ctx* ctx, uint64_t* visible_total, uint64_t* model_bytes_total);
int t3d_frame_view_get(t3d_ctx* ctx, t3d_frame_view* view_out);
int t3d_frame_segments(t3d_ctx* ctx, t3d_segment_info* segs_out, uint32_t max_segs, uint32_t* num_out);
/* Copies the visible triangles of the last frame to host memory, densely in
 * segment order (3 corners per triangle; xyuv/rgba 4 floats per corner). */
int t3d_frame_download(t3d_ctx* ctx, float* xyuv, float* rgba, float* depth, uint64_t max_tris,
                       uint64_t* tris_out);
/* Copies Custom0 of the last frame's visible corners (one float per corner, same
 * order as t3d_frame_download): 1 / w under perspective-corrected texture mapping
 * (Camera.PerspectiveCorrectedTextureMapping, camera.go:1700-1704; the colour pass
 * divides the interpolated UV by it, shaders/base3d.kage:79-81); 0 for corners of
 * jobs without it. T3D_E_INVAL when no job of the frame uses it. */
int t3d_frame_download_custom0(t3d_ctx* ctx, float* custom0, uint64_t max_tris, uint64_t* tris_out);

/* ---- CUDA graph replay (batched form) ------------------------------------- */
/* Captures the frame of t3d_render(mode=BATCHED, animate) into a CUDA graph. */
int t3d_graph_capture(t3d_ctx* ctx, uint32_t scene, const t3d_camera_desc* cam, int animate);
int t3d_graph_replay(t3d_ctx* ctx, uint32_t frames, void* stream);

/* ---- serving: continuous batching ------------------------------------------- */
typedef struct t3d_server t3d_server;
typedef struct t3d_request {
    t3d_job_desc job;
    uint64_t     id;
    double       arrival_s;   /* replay mode: arrival time relative to start */
} t3d_request;
typedef struct t3d_completion {
    uint64_t id;
    int32_t  status;
    uint32_t batch;           /* requests in the launch that rendered it */
    uint64_t visible_tris;
    double   arrival_s;
    double   admit_s;
    double   done_s;
    uint64_t checksum;        /* order-dependent hash of the emitted stream */
    uint64_t model_bytes;     /* 48V+12T+64+48L bytes of the request's models that survived
                                 frustum culling (with 108 per visible triangle: its algorithmic bytes) */
    double   launch_s;        /* its batch's launch tables built and its kernels queued */
} t3d_completion;

/* hbm_budget_bytes bounds the device bytes of in-flight requests' outputs and
 * scratch; max_batch bounds the jobs per launch; streams = launch slots that
 * run concurrently. With one launch per phase (t3d_set_split_phases, the default)
 * every slot launches full grids and the device interleaves them; a context set to
 * one cooperative launch per frame gives each slot 1/streams of the device's
 * co-resident blocks, so the launches of all slots fit on the device together. The
 * slots render the context's resident scenes: while a server runs, scenes are not
 * uploaded, released or changed (set_models / set_bones / set_shape_weights /
 * set_lights) on that context. */
int t3d_server_create(t3d_ctx* ctx, uint64_t hbm_budget_bytes, uint32_t max_batch,
                      uint32_t streams, t3d_server** out);
int t3d_server_destroy(t3d_server* srv);
/* Thread-safe submit; returns T3D_E_ADMIT if the request can never fit. */
int t3d_server_submit(t3d_server* srv, const t3d_request* req);
/* verify = 1 (default) hashes every request's emitted stream into
 * t3d_completion.checksum (costs a device-to-host copy per request). */
int t3d_server_set_verify(t3d_server* srv, int verify);
/* Bounds the render pairs (visible model parts) of one batch (0 = no bound; default
 * 4096): a batch's launch tables are built on the host in time proportional to its
 * pairs, so the bound keeps one batch of many-model requests from holding its slot
 * (and the requests queued behind it) for milliseconds. A request is admitted alone
 * when it exceeds the bound by itself. */
int t3d_server_set_batch_pairs(t3d_server* srv, uint32_t max_pairs);
/* Non-blocking poll of finished requests. */
int t3d_server_poll(t3d_server* srv, t3d_completion* out, uint32_t max, uint32_t* n_out);
/* Replays requests at their arrival_s offsets from a driver thread and blocks
 * until all complete; completions in id order into out[n]. */
int t3d_server_replay(t3d_server* srv, const t3d_request* reqs, uint32_t n, t3d_completion* out);

/* ---- rasterising the emitted stream ----------------------------------------- */
/* The colour and depth passes of flush (camera.go:1829-2048) over one job of the
 * last rendered frame, on the device: per flush (a render pair, or a dynamic batch) in
 * draw order, the depth pass (camera.go:350-383: encodeDepth into an RGBA8
 * intermediate, tested against the depth texture of the flushes before, composited
 * into it unless the flush is transparent; for TransparencyModeAlphaClip the
 * clip-alpha shader, camera.go:390-480, which drops fragments whose texture alpha is
 * 0.8 or less) and the colour pass (shaders/base3d.kage: texture -- nearest or
 * bilinear, wrapped, UV or screen mapped -- times the vertex colour, alpha
 * premultiplied, fog by the flush's depth with FogCurve and dithering, source-over
 * blending); with RenderDepth off, the plain source-over triangle draw. The camera's
 * fog settings are the World's (FogOn, FogMode, FogRange, FogColor). Images are RGBA8,
 * premultiplied, row-major, camera width x height, cleared to 0 first, like ebiten
 * images. Coverage: pixel centres, top-left fill rule; attributes interpolated linearly
 * in screen space; a texel is the one containing the sample point. Blend modes other
 * than source-over, custom fragment shaders and textures under
 * PerspectiveCorrectedTextureMapping (it needs the 1/w vertex attribute) are not
 * supported. No reference counterpart runs on the device: the reference hands these
 * passes to ebiten. */
/* An RGBA8 texture as ebiten stores it (premultiplied, row-major). */
typedef struct t3d_texture_desc {
    const uint8_t* rgba8;
    int32_t        width, height;
} t3d_texture_desc;
/* Replaces the context's raster texture table (materials refer to entry k as k + 1). */
int t3d_raster_set_textures(t3d_ctx* ctx, const t3d_texture_desc* textures, uint32_t n);
typedef struct t3d_raster_opts {
    int32_t fog_curve;     /* World.FogCurve: 0 linear, 1 out-circ, 2 in-circ */
    float   dither_size;   /* World.DitheredFogSize: > 0 enables Bayer-dithered fog */
    int32_t fogless;       /* Material.Fogless, for every pair */
    /* Tuning: triangles whose pixel box exceeds 32 pixels are shared out to the whole grid in
     * 1024-pixel chunks, up to this many per call (0 = 262144, negative = none); beyond it
     * each warp rasterises its own. The images do not depend on it. */
    int32_t shared_large_tris;
} t3d_raster_opts;
/* Rasterises job `job` (0-based, in the order given to t3d_render_jobs) of the last frame. */
int t3d_frame_raster(t3d_ctx* ctx, uint32_t job, const t3d_raster_opts* opts, void* stream);
/* Copies the last rasterised images (4 * width * height bytes each; either may be NULL). */
int t3d_frame_images(t3d_ctx* ctx, uint8_t* color_rgba8, uint8_t* depth_rgba8, int32_t* width, int32_t* height);

/* ---- rendering without allocation ------------------------------------------ */
/* For callers that cannot allocate device memory while they render -- an engine
 * or rasteriser that owns the device memory budget through its own allocator, a
 * real-time render thread where cudaMalloc/cudaFree would synchronise the device,
 * or code already short of memory. This entry point has no counterpart in the
 * reference: it renders one render pair (one model, one mesh part) from mesh and
 * output buffers the caller owns in device memory, and keeps every intermediate
 * in a fixed 16 MiB __device__ array inside the library (held on every GPU that
 * loads the library until the process exits). It allocates nothing.
 * Limits per call: 65536 vertices, 131072 mesh triangles, T3D_MAX_LIGHTS_PER_MODEL
 * lights; larger requests return T3D_E_INVAL with a message in `error`.
 * All calls share that array: calls that overlap on the GPU race and corrupt each
 * other, so serialise them. The first call on a device sets the library up for it
 * (symbol address, kernel attributes); make it before any stream capture. The call
 * waits for `stream` before returning its status. Output: out_count visible
 * triangles, written densely from slot 0, 3 corners each, in draw order. */
typedef struct t3d_noalloc_args {
    /* mesh streams in device memory, SoA as in t3d_mesh_desc (colors may be NULL) */
    const float*          positions;
    const float*          normals;
    const float*          uvs;
    const float*          colors;
    const uint32_t*       indices;       /* 3 * num_triangles, mesh-absolute */
    const float*          volume_cells;  /* device RGBA cells for volume lights, or NULL; the lights a
                                            cell uses (t3d_scene_desc.cell_use_*) are not carried
                                            here, so cells light with their own colour only */
    /* outputs in device memory, room for tri_count triangles */
    float*                out_xyuv;      /* 3 * 4 floats per triangle */
    float*                out_rgba;      /* 3 * 4 floats per triangle */
    float*                out_depth;     /* 3 floats per triangle */
    uint32_t*             out_count;     /* visible triangles */
    /* host descriptors */
    const t3d_model_desc*  model;        /* `mesh` and `light_list` are ignored */
    const t3d_light_desc*  lights;       /* the model's lights in list order */
    const t3d_camera_desc* camera;
    uint32_t              num_vertices;
    uint32_t              num_triangles;
    uint32_t              tri_start;     /* the part: triangles [tri_start, tri_start + tri_count) */
    uint32_t              tri_count;
    uint32_t              num_lights;
    uint32_t              reserved;
    float                 dim_min[3];    /* Mesh.Dimensions */
    float                 dim_max[3];
    t3d_material          mat;
    char                  error[128];    /* out: message when the call fails */
} t3d_noalloc_args;
int t3d_render_part_noalloc(int device, t3d_noalloc_args* args, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* T3D_H */
