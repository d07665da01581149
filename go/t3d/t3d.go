// Package t3d binds Tetra3D's software vertex stage to the GB300 library
// libt3d.so through its C ABI (include/t3d.h).
//
// NOT COMPILED HERE: the machines this repository is built and tested on have
// no Go toolchain, so this file has never been through `go build`. It is the
// cgo shim a Tetra3D maintainer would add; the same entry points are exercised
// through Python ctypes by tests/ and bench.py.
//
// Where it plugs in: Camera.Render (camera.go:1269) keeps collecting models and
// lights; the body from ProcessVertices (model.go:600) to the vertex lists that
// flush (camera.go:1829) hands to ebiten becomes Context.Render, and the lists
// stay in device memory (FrameView) or come back with Download.
package t3d

/*
#cgo CFLAGS: -I${SRCDIR}/../../include
#cgo LDFLAGS: -L${SRCDIR}/../../tetra3d_gb300/_build -lt3d -Wl,-rpath,${SRCDIR}/../../tetra3d_gb300/_build
#include <stdlib.h>
#include "t3d.h"
*/
import "C"

import (
	"errors"
	"fmt"
	"unsafe"

	"github.com/solarlune/tetra3d"
)

// Context owns the device state of one host thread (t3d_ctx).
type Context struct{ h *C.t3d_ctx }

// NewContext creates a context on a CUDA device.
func NewContext(device int) (*Context, error) {
	var h *C.t3d_ctx
	if rc := C.t3d_create(C.int(device), &h); rc != C.T3D_OK {
		return nil, fmt.Errorf("t3d_create(%d) failed: %d", device, int(rc))
	}
	return &Context{h: h}, nil
}

// Close releases the context and everything it holds on the device.
func (c *Context) Close() {
	if c.h != nil {
		C.t3d_destroy(c.h)
		c.h = nil
	}
}

func (c *Context) err(rc C.int) error {
	if rc == C.T3D_OK {
		return nil
	}
	return errors.New(C.GoString(C.t3d_last_error(c.h)))
}

func mat16(m tetra3d.Matrix4) [16]C.float {
	var o [16]C.float
	for i := 0; i < 16; i++ {
		o[i] = C.float(m[i/4][i%4])
	}
	return o
}

func boolInt(b bool) C.int32_t {
	if b {
		return 1
	}
	return 0
}

// UploadScene copies meshes, models and lights to the device. The descriptor is
// filled by walking scene.Root as Camera.RenderNodes does: one t3d_mesh_desc per
// Mesh, one t3d_model_desc per Model in render order, the lights and the light
// lists (list 0: world ambient first if lit, then visible lights in tree order;
// lists 1..: LightGroups). Host arrays are copied before the call returns.
func (c *Context) UploadScene(desc *C.t3d_scene_desc) (uint32, error) {
	var id C.uint32_t
	return uint32(id), c.err(C.t3d_scene_upload(c.h, desc, &id))
}

// FrameReadback queues the read-back of the last frame's counts behind it; FrameCollect
// waits for it and returns that frame's stats (a render loop can queue the next frame in
// between, so the GPU does not wait for the host).
func (c *Context) FrameReadback() error { return c.err(C.t3d_frame_readback(c.h)) }

func (c *Context) FrameCollect() (C.t3d_stats, error) {
	var st C.t3d_stats
	return st, c.err(C.t3d_frame_collect(c.h, &st))
}

// SetSplitPhases picks the launch shape of a frame: 1 (the default) one persistent launch
// per phase, 0 a batched frame as one cooperative launch. The emitted stream is the same.
func (c *Context) SetSplitPhases(mode int) error {
	return c.err(C.t3d_set_split_phases(c.h, C.int(mode)))
}

// SetModels pushes changed model descriptors [first, first+len(models)) (Node.Transform
// changes, visibility, colour). The copy is queued behind frames already issued.
func (c *Context) SetModels(scene uint32, first int, models []C.t3d_model_desc) error {
	if len(models) == 0 {
		return nil
	}
	return c.err(C.t3d_scene_set_models(c.h, C.uint32_t(scene), C.uint32_t(first), &models[0], C.uint32_t(len(models))))
}

// SetLights replaces lights [first, first+len(lights)) after they moved or changed.
func (c *Context) SetLights(scene uint32, first int, lights []C.t3d_light_desc) error {
	if len(lights) == 0 {
		return nil
	}
	return c.err(C.t3d_scene_set_lights(c.h, C.uint32_t(scene), C.uint32_t(first), &lights[0], C.uint32_t(len(lights))))
}

// CameraDesc fills the camera and World fields Camera.Render reads (camera.go:256-321, world.go:25-39).
func CameraDesc(cam *tetra3d.Camera, world *tetra3d.World) C.t3d_camera_desc {
	var d C.t3d_camera_desc
	d.transform = mat16(cam.Transform())
	d.world_rotation = mat16(cam.WorldRotation())
	w, h := cam.Size()
	d.width, d.height = C.int32_t(w), C.int32_t(h)
	d.perspective = boolInt(cam.Perspective())
	d.render_depth = boolInt(cam.RenderDepth)
	d.perspective_corrected = boolInt(cam.PerspectiveCorrectedTextureMapping)
	d.fov_y, d.near_plane, d.far_plane = C.float(cam.FieldOfView()), C.float(cam.Near()), C.float(cam.Far())
	d.ortho_scale, d.depth_margin = C.float(cam.OrthoScale()), C.float(cam.DepthMargin)
	d.max_light_count = C.int32_t(cam.MaxLightCount)
	d.vertex_snapping = C.float(cam.VertexSnapping)
	if world != nil {
		d.lighting_on = boolInt(world.LightingOn)
		d.fog_on = boolInt(world.FogOn)
		d.fog_mode = C.int32_t(world.FogMode)
		d.fog_range = [2]C.float{C.float(world.FogRange[0]), C.float(world.FogRange[1])}
		d.fog_color = [4]C.float{C.float(world.FogColor.R), C.float(world.FogColor.G), C.float(world.FogColor.B), C.float(world.FogColor.A)}
	}
	return d
}

// Render replaces the body of Camera.Render up to flush: all models in one
// batched launch, then waits for the frame and its per-pair visible counts.
func (c *Context) Render(scene uint32, cam *C.t3d_camera_desc) (C.t3d_stats, error) {
	var st C.t3d_stats
	if rc := C.t3d_render(c.h, C.uint32_t(scene), cam, C.T3D_MODE_BATCHED, 0, nil); rc != C.T3D_OK {
		return st, c.err(rc)
	}
	return st, c.err(C.t3d_frame_sync(c.h, &st))
}

// Segments returns the render pairs of the last frame in draw order; pairs of one
// dynamic batch share Draw (one DrawTrianglesShader call).
func (c *Context) Segments() ([]C.t3d_segment_info, error) {
	var n C.uint32_t
	if rc := C.t3d_frame_segments(c.h, nil, 0, &n); rc != C.T3D_OK {
		return nil, c.err(rc)
	}
	if n == 0 {
		return nil, nil
	}
	out := make([]C.t3d_segment_info, int(n))
	return out, c.err(C.t3d_frame_segments(c.h, &out[0], n, &n))
}

// FrameView returns the device buffers of the last frame (they stay valid until
// the next render on this context).
func (c *Context) FrameView() (C.t3d_frame_view, error) {
	var v C.t3d_frame_view
	return v, c.err(C.t3d_frame_view_get(c.h, &v))
}

// Download copies the emitted triangles (3 corners each) for a CPU consumer. The
// per-corner record maps onto ebiten.Vertex as DstX, DstY, SrcX, SrcY = xyuv,
// ColorR..A = rgba for the colour list, ColorR = ColorG = ColorB = depth and
// ColorA = 1 for the depth list (camera.go:1677-1779); indices are 0, 1, 2, ...
func (c *Context) Download(maxTris uint64) (xyuv, rgba, depth []float32, err error) {
	if maxTris == 0 {
		return nil, nil, nil, nil
	}
	xyuv = make([]float32, 12*maxTris)
	rgba = make([]float32, 12*maxTris)
	depth = make([]float32, 3*maxTris)
	var n C.uint64_t
	rc := C.t3d_frame_download(c.h, (*C.float)(unsafe.Pointer(&xyuv[0])), (*C.float)(unsafe.Pointer(&rgba[0])),
		(*C.float)(unsafe.Pointer(&depth[0])), C.uint64_t(maxTris), &n)
	return xyuv[:12*n], rgba[:12*n], depth[:3*n], c.err(rc)
}

// DownloadCustom0 copies ebiten.Vertex.Custom0 of every downloaded corner (same order as
// Download): 1 / w when Camera.PerspectiveCorrectedTextureMapping is on (camera.go:1700-1704).
func (c *Context) DownloadCustom0(maxTris uint64) ([]float32, error) {
	if maxTris == 0 {
		return nil, nil
	}
	out := make([]float32, 3*maxTris)
	var n C.uint64_t
	rc := C.t3d_frame_download_custom0(c.h, (*C.float)(unsafe.Pointer(&out[0])), C.uint64_t(maxTris), &n)
	return out[:3*n], c.err(rc)
}

// UpdateArmature copies the boneInfluence matrices of bones first..first+n.
func (c *Context) UpdateArmature(scene uint32, first int, influences []tetra3d.Matrix4) error {
	if len(influences) == 0 {
		return nil
	}
	buf := make([]C.float, 16*len(influences))
	for i, m := range influences {
		v := mat16(m)
		copy(buf[16*i:16*i+16], v[:])
	}
	return c.err(C.t3d_scene_set_bones(c.h, C.uint32_t(scene), C.uint32_t(first), &buf[0], C.uint32_t(len(influences))))
}

// SetShapeKeyWeights mirrors ShapeKey.SetWeight for every key of one mesh.
func (c *Context) SetShapeKeyWeights(scene, mesh uint32, weights []float32) error {
	if len(weights) == 0 {
		return nil
	}
	return c.err(C.t3d_scene_set_shape_weights(c.h, C.uint32_t(scene), C.uint32_t(mesh),
		(*C.float)(unsafe.Pointer(&weights[0])), C.uint32_t(len(weights))))
}

// Raster runs flush's depth and colour passes on the device and returns the
// premultiplied RGBA8 images (headless callers without an ebiten window).
func (c *Context) Raster(job uint32, opts C.t3d_raster_opts, w, h int) (color, depth []byte, err error) {
	if rc := C.t3d_frame_raster(c.h, C.uint32_t(job), &opts, nil); rc != C.T3D_OK {
		return nil, nil, c.err(rc)
	}
	color, depth = make([]byte, 4*w*h), make([]byte, 4*w*h)
	var cw, ch C.int32_t
	rc := C.t3d_frame_images(c.h, (*C.uint8_t)(&color[0]), (*C.uint8_t)(&depth[0]), &cw, &ch)
	return color, depth, c.err(rc)
}

// SetTextures replaces the raster texture table with premultiplied RGBA8 images
// (ebiten's ReadPixels); material texture k names entry k - 1.
func (c *Context) SetTextures(pixels [][]byte, sizes [][2]int) error {
	descs := make([]C.t3d_texture_desc, len(pixels))
	for i, px := range pixels {
		cpx := C.CBytes(px) // C memory: the array handed to C holds no Go pointers
		defer C.free(cpx)
		descs[i] = C.t3d_texture_desc{rgba8: (*C.uint8_t)(cpx), width: C.int32_t(sizes[i][0]), height: C.int32_t(sizes[i][1])}
	}
	var p *C.t3d_texture_desc
	if len(descs) > 0 {
		p = &descs[0]
	}
	return c.err(C.t3d_raster_set_textures(c.h, p, C.uint32_t(len(descs))))
}

// Server is the continuous-batching render server over a context's resident scenes.
type Server struct {
	c *Context
	h *C.t3d_server
}

// NewServer admits requests within hbmBudget device bytes, at most maxBatch per
// launch, on `streams` concurrent launch slots.
func (c *Context) NewServer(hbmBudget uint64, maxBatch, streams uint32) (*Server, error) {
	var h *C.t3d_server
	if rc := C.t3d_server_create(c.h, C.uint64_t(hbmBudget), C.uint32_t(maxBatch), C.uint32_t(streams), &h); rc != C.T3D_OK {
		return nil, c.err(rc)
	}
	return &Server{c: c, h: h}, nil
}

// SetBatchPairs bounds the render pairs of one batch (0: no bound; the default is 4096).
func (s *Server) SetBatchPairs(maxPairs uint32) error {
	if rc := C.t3d_server_set_batch_pairs(s.h, C.uint32_t(maxPairs)); rc != C.T3D_OK {
		return fmt.Errorf("t3d_server_set_batch_pairs: %d", int(rc))
	}
	return nil
}

// Submit queues one request (thread safe).
func (s *Server) Submit(req *C.t3d_request) error {
	if rc := C.t3d_server_submit(s.h, req); rc != C.T3D_OK {
		return fmt.Errorf("t3d_server_submit: %d", int(rc))
	}
	return nil
}

// Poll returns the requests finished since the last poll.
func (s *Server) Poll(max int) []C.t3d_completion {
	if max <= 0 {
		return nil
	}
	out := make([]C.t3d_completion, max)
	var n C.uint32_t
	C.t3d_server_poll(s.h, &out[0], C.uint32_t(max), &n)
	return out[:int(n)]
}

// Close stops the server's slots.
func (s *Server) Close() {
	if s.h != nil {
		C.t3d_server_destroy(s.h)
		s.h = nil
	}
}
