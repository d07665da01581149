/*
 * t3d_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of Tetra3D's software vertex stage (Camera.Render minus the
 * ebiten draw calls) used as the parity checker for the CUDA library and as the
 * timed CPU baseline. Nothing in the product links or calls this library; only
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg do.
 *
 * PARITY UNPINNED: the reference (pure Go) publishes no golden vectors for this
 * path and cannot be compiled here (no Go toolchain). The restatement is pinned
 * only by the reference's one unit test (TestMatrixInversion, matrix_test.go:36-62)
 * and by hand-computed known-answer cases in tests/.
 *
 * Arithmetic convention: unfused IEEE binary32 (-ffp-contract=off), with
 * math32.Sqrt/Tan/Cos/Atan/Round evaluated in binary64 and rounded, as
 * math32/math32.go does. The _f64 twin evaluates everything in binary64 for
 * error reporting.
 */
#ifndef T3D_ORACLE_H
#define T3D_ORACLE_H
#include "../include/t3d.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Output in the same segment layout the GPU library uses: render pairs in draw
 * order, each owning `capacity` triangle slots from `base`; `count` of them are
 * written. Per slot: the mesh-absolute triangle index and 3 corners. */
typedef struct t3d_oracle_out {
    uint32_t  max_segments;
    uint32_t  num_segments;      /* out */
    uint32_t* seg_model;         /* [max_segments] */
    uint32_t* seg_part;
    uint32_t* seg_base;
    uint32_t* seg_capacity;
    uint32_t* seg_count;
    uint64_t  max_tris;          /* slots available */
    uint64_t  total_slots;       /* out: sum of capacities */
    uint64_t  visible_tris;      /* out */
    uint32_t* tri_index;         /* [max_tris] */
    void*     xyuv;              /* [max_tris*3*4] float or double */
    void*     rgba;              /* [max_tris*3*4] */
    void*     depth;             /* [max_tris*3] */
    uint32_t  culled_models;     /* out */
    uint32_t  reserved;
    uint32_t* seg_draw;          /* [max_segments] flush of each pair (a dynamic batch is one); may be NULL */
    uint32_t* seg_draw_transparent; /* that flush is in the transparent pass; may be NULL */
    void*     custom0;           /* [max_tris*3] 1 / w per corner under perspective-corrected texture
                                  * mapping (camera.go:1700-1704); may be NULL */
} t3d_oracle_out;

/* Renders one frame. light_mask may be NULL (all lights). animate_frames
 * applies each model's rotate_step that many times first. threads > 1 splits
 * render pairs over host threads (results identical). */
int t3d_oracle_render_f32(const t3d_scene_desc* scene, const t3d_camera_desc* cam,
                          const uint64_t* light_mask, uint32_t animate_frames,
                          uint32_t threads, t3d_oracle_out* out);
int t3d_oracle_render_f64(const t3d_scene_desc* scene, const t3d_camera_desc* cam,
                          const uint64_t* light_mask, uint32_t animate_frames,
                          uint32_t threads, t3d_oracle_out* out);

/* The texture state of each flush and the texture table, for t3d_oracle_raster. */
typedef struct t3d_oracle_textures {
    const uint32_t* flush_texture;  /* per flush: 0 the white default image, k texture k - 1 */
    const uint32_t* flush_flags;    /* per flush: bit 0 bilinear, bit 1 screen mapped, bit 2 alpha clip */
    const float*    flush_scale;    /* per flush: TextureMapScreenSizeMultiplierW, H */
    uint32_t        ntex;
    const uint32_t* tex_offset;     /* texel k of texture t: texels[tex_offset[t] + k] (RGBA8 premultiplied) */
    const int32_t*  tex_w;
    const int32_t*  tex_h;
    const uint32_t* texels;
} t3d_oracle_textures;

/* Rasterises n triangles of one job in draw order (3 corners each: xyuv, rgba, depth as
 * t3d_frame_download writes them) into RGBA8 colour and depth images of the camera size
 * (pixel = r | g << 8 | b << 16 | a << 24); tri_pair = flush of each triangle,
 * pair_transparent indexed by that id; tex may be NULL (no textures, no alpha clip);
 * custom0 (1 / w per corner) is read when the camera uses perspective-corrected mapping.
 * See t3d_oracle_raster.cpp. */
int t3d_oracle_raster(const t3d_camera_desc* cam, int32_t fog_curve, float dither, int32_t fogless, uint32_t n,
                      const float* xyuv, const float* rgba, const float* depth, const uint32_t* tri_pair,
                      const uint8_t* pair_transparent, const t3d_oracle_textures* tex, uint32_t* color_out,
                      uint32_t* depth_out, const float* custom0);

/* Matrix4 helpers (float32) for pinning against matrix_test.go. */
void t3d_oracle_mat_mult(const float* a, const float* b, float* out);
void t3d_oracle_mat_inverted(const float* m, float* out);
void t3d_oracle_mat_rotate(float x, float y, float z, float angle, float* out);
void t3d_oracle_mat_decompose(const float* m, float* pos3, float* scale3, float* rot16);
void t3d_oracle_quat_to_mat(float x, float y, float z, float w, float* out);
void t3d_oracle_vec_unit(const float* v3, float* out3);

#ifdef __cplusplus
}
#endif
#endif
