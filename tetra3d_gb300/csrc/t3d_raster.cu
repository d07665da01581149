// t3d_raster.cu -- rasterising the emitted triangle stream on the device.
//
// Restates the two passes Tetra3D's flush runs per render pair through ebiten
// (camera.go:1829-2048): the depth pass (camera.go:350-383: encodeDepth into an
// RGBA8 intermediate, tested against the depth texture of the pairs drawn
// before, composited into it unless the pair is transparent) and the colour
// pass (shaders/base3d.kage:67-145: vertex colour times the default white
// texture (tetra3d.go:12, :38), alpha premultiplied, fog by the intermediate
// depth with FogCurve and Bayer dithering (camera.go:1257-1262), source-over
// blending); with RenderDepth off, ebiten's plain triangle draw with
// straight-alpha vertex colours. ebiten (v2.9.7) conventions restated: RGBA8
// premultiplied images cleared to 0, fragments at pixel centres, the top-left
// fill rule, attributes interpolated linearly in screen space, unorm8 writes
// rounded to nearest after clamping to [0, 1].
//
// Device work: every visible triangle of the job lists the pixels it covers
// (fragments), a counting sort groups fragments by pixel, and one thread per
// pixel sorts its fragments into draw order (by hit index) and replays them with
// the per-pair depth and colour logic.

#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "t3d_runtime.h"

using namespace t3d;

#define CKR(call)                                                                                       \
    do {                                                                                                \
        cudaError_t e_ = (call);                                                                        \
        if (e_ != cudaSuccess) {                                                                        \
            set_err(ctx, "%s failed: %s", #call, cudaGetErrorString(e_));                              \
            return e_ == cudaErrorMemoryAllocation ? T3D_E_OOM : T3D_E_CUDA;                            \
        }                                                                                               \
    } while (0)

namespace {

constexpr int kScanThreads = 1024;
constexpr int kScanPer = 4;
constexpr int kScanChunk = kScanThreads * kScanPer;
constexpr int kFragThreads = 256;
constexpr uint32_t kUnitTris = 512;        // triangles per warp unit of the fragment passes
constexpr uint32_t kBigChunk = 256;        // pixels per shared (one-warp) work item of a large triangle
constexpr uint32_t kBigTriCap = 1u << 18;  // large triangles the shared list holds
constexpr uint32_t kChunkCap = 1u << 22;   // and their chunks

__constant__ float kBayer[16] = {1.0f / 17.0f,  9.0f / 17.0f, 3.0f / 17.0f,  11.0f / 17.0f,
                                 13.0f / 17.0f, 5.0f / 17.0f, 15.0f / 17.0f, 7.0f / 17.0f,
                                 4.0f / 17.0f,  12.0f / 17.0f, 2.0f / 17.0f,  10.0f / 17.0f,
                                 16.0f / 17.0f, 8.0f / 17.0f, 14.0f / 17.0f, 6.0f / 17.0f};

// One texture of the context's table: texels[offset + y * w + x], RGBA8 premultiplied.
struct RasterTex {
    uint32_t offset;
    int32_t w, h, pad;
};

struct RasterJob {
    const RasterTex* texs;      // texture k + 1 of a flush (DevSeg.pad[1]) is texs[k]
    const uint32_t* texels;
    const float4* xyuv;
    const float4* rgba;
    const float* depth;
    const float* custom0;       // 1 / w per corner (perspective-corrected texture mapping), else null
    const uint32_t* cbase;      // exclusive prefix of the job's per-pair visible counts (nseg + 1)
    uint32_t seg_lo, nseg;      // the job's render pairs: segs[seg_lo, seg_lo + nseg)
    uint32_t big_cap;           // large triangles the shared list takes (<= kBigTriCap)
    const DevSeg* segs;
    int32_t W, H;
    int32_t render_depth;
    int32_t fog_mode;           // -1 off, 0 add, 1 sub, 2 overwrite
    float fog_r, fog_g, fog_b, fog0, fog1;
    int32_t fog_curve, fogless;
    float dither;
};

// ---- fragments ---------------------------------------------------------------
struct TriScreen {
    float ax, ay, bx, by, cx, cy, area;
    int x0, x1, y0, y1;
    bool ok;
};

__device__ __forceinline__ TriScreen screen_of(const RasterJob& J, const float4 a, const float4 b, const float4 c) {
    TriScreen t;
    t.ax = a.x; t.ay = a.y; t.bx = b.x; t.by = b.y; t.cx = c.x; t.cy = c.y;
    t.area = (t.bx - t.ax) * (t.cy - t.ay) - (t.by - t.ay) * (t.cx - t.ax);
    t.ok = t.area != 0.0f && isfinite(t.area);
    const float mnx = fminf(fminf(t.ax, t.bx), t.cx), mxx = fmaxf(fmaxf(t.ax, t.bx), t.cx);
    const float mny = fminf(fminf(t.ay, t.by), t.cy), mxy = fmaxf(fmaxf(t.ay, t.by), t.cy);
    // pixels whose centre (x + 0.5) lies in [mn, mx]
    t.x0 = (int)fminf(fmaxf(0.0f, ceilf(mnx - 0.5f)), (float)J.W);
    t.x1 = (int)fmaxf(fminf((float)J.W - 1.0f, floorf(mxx - 0.5f)), -1.0f);
    t.y0 = (int)fminf(fmaxf(0.0f, ceilf(mny - 0.5f)), (float)J.H);
    t.y1 = (int)fmaxf(fminf((float)J.H - 1.0f, floorf(mxy - 0.5f)), -1.0f);
    if (!(mnx == mnx) || !(mny == mny) || !(mxx == mxx) || !(mxy == mxy)) t.ok = false;
    return t;
}
__device__ __forceinline__ TriScreen tri_screen(const RasterJob& J, uint32_t slot) {
    return screen_of(J, J.xyuv[3 * (size_t)slot], J.xyuv[3 * (size_t)slot + 1], J.xyuv[3 * (size_t)slot + 2]);
}

// Edge weights of pixel centre (x, y): w_c for edge a->b, w_a for b->c, w_b for c->a.
// Inside: every weight of the positively oriented triangle > 0, or == 0 on a top-left edge.
__device__ __forceinline__ bool tl_edge(float dx, float dy) { return dy < 0.0f || (dy == 0.0f && dx > 0.0f); }
__device__ __forceinline__ bool covers(const TriScreen& t, float x, float y, float& wa, float& wb, float& wc) {
    wc = (t.bx - t.ax) * (y - t.ay) - (t.by - t.ay) * (x - t.ax);
    wa = (t.cx - t.bx) * (y - t.by) - (t.cy - t.by) * (x - t.bx);
    wb = (t.ax - t.cx) * (y - t.cy) - (t.ay - t.cy) * (x - t.cx);
    const float s = t.area > 0.0f ? 1.0f : -1.0f;
    const float ea = s * wa, eb = s * wb, ec = s * wc;
    const bool ia = ea > 0.0f || (ea == 0.0f && tl_edge(s * (t.cx - t.bx), s * (t.cy - t.by)));
    const bool ib = eb > 0.0f || (eb == 0.0f && tl_edge(s * (t.ax - t.cx), s * (t.ay - t.cy)));
    const bool ic = ec > 0.0f || (ec == 0.0f && tl_edge(s * (t.bx - t.ax), s * (t.by - t.ay)));
    return ia && ib && ic;
}

__global__ void k_seg_bases(const uint32_t* __restrict__ seg_count, uint32_t seg_lo, uint32_t nseg, uint32_t* cbase) {
    // one block: exclusive prefix of the job's per-pair visible counts, cbase[nseg] = total
    __shared__ uint32_t warp_sum[32];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (uint32_t base = 0; base < nseg; base += blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const uint32_t v = i < nseg ? seg_count[seg_lo + i] : 0u;
        uint32_t incl = v;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t u = __shfl_up_sync(0xffffffffu, incl, o);
            if ((threadIdx.x & 31) >= (uint32_t)o) incl += u;
        }
        if ((threadIdx.x & 31) == 31) warp_sum[threadIdx.x >> 5] = incl;
        __syncthreads();
        if (threadIdx.x < 32) {
            const uint32_t nw = blockDim.x >> 5;
            uint32_t w = threadIdx.x < nw ? warp_sum[threadIdx.x] : 0u, wi = w;
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t u = __shfl_up_sync(0xffffffffu, wi, o);
                if (threadIdx.x >= (uint32_t)o) wi += u;
            }
            if (threadIdx.x < nw) warp_sum[threadIdx.x] = wi - w;
        }
        __syncthreads();
        if (i < nseg) cbase[i] = carry + warp_sum[threadIdx.x >> 5] + incl - v;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry += warp_sum[threadIdx.x >> 5] + incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) cbase[nseg] = carry;
}

// The render pair holding visible triangle c of the job (draw order), searched forward
// from pair `from` (cbase[from] <= c): gallop to a pair past c, then bisect. Pairs with no
// visible triangle share their successor's prefix and are never returned.
__device__ __forceinline__ uint32_t find_pair(const RasterJob& J, uint32_t c, uint32_t from) {
    uint32_t lo = from, hi = from + 1, step = 1;
    while (hi < J.nseg && __ldg(&J.cbase[hi]) <= c) {  // cbase[nseg] = n > c
        lo = hi;
        step <<= 1;
        hi = lo + step;
    }
    if (hi > J.nseg) hi = J.nseg;
    while (hi - lo > 1) {  // cbase[lo] <= c < cbase[hi]
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(&J.cbase[mid]) <= c) lo = mid;
        else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ uint32_t tri_fragments(const TriScreen& t) {
    uint32_t k = 0;
    for (int y = t.y0; y <= t.y1; y++)
        for (int x = t.x0; x <= t.x1; x++) {
            float wa, wb, wc;
            if (covers(t, (float)x + 0.5f, (float)y + 0.5f, wa, wb, wc)) k++;
        }
    return k;
}

// Bounding-box pixels of a triangle (0 when it covers no pixel centre's row or column).
__device__ __forceinline__ uint32_t bbox_pixels(const TriScreen& t) {
    if (!t.ok || t.x1 < t.x0 || t.y1 < t.y0) return 0u;
    return (uint32_t)(t.x1 - t.x0 + 1) * (uint32_t)(t.y1 - t.y0 + 1);
}
// Triangles with larger pixel boxes are shared out to the whole grid in kBigChunk-pixel
// chunks (or, when the shared list is full, tested by their warp together); smaller ones are
// tested by their own thread.
constexpr uint32_t kBigBox = 8;

// A large triangle shared by the grid: its pixel box (row-major) is cut into kBigChunk-pixel
// chunks [chunk0, chunk0 + ceil(box / kBigChunk)); `hit` is its entry in the hit list and
// `cursor` the next free fragment of its range (set by the write pass).
struct BigTri {
    uint32_t slot, hit, unit, chunk0, cursor, pad0, pad1, pad2;
};

__device__ __forceinline__ uint32_t warp_exclusive(uint32_t v, uint32_t lane, uint32_t& total) {
    uint32_t incl = v;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t u = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (uint32_t)o) incl += u;
    }
    total = __shfl_sync(0xffffffffu, incl, 31);
    return incl - v;
}

// A warp's count of the pixel centres triangle t covers (lanes stride the box row-major).
__device__ __forceinline__ uint32_t warp_fragments(const TriScreen& t, uint32_t lane) {
    const uint32_t bw = (uint32_t)(t.x1 - t.x0 + 1), area = bbox_pixels(t);
    uint32_t k = 0;
    for (uint32_t i = lane; i < area; i += 32) {
        float wa, wb, wc;
        if (covers(t, (float)(t.x0 + (int)(i % bw)) + 0.5f, (float)(t.y0 + (int)(i / bw)) + 0.5f, wa, wb, wc)) k++;
    }
    for (int o = 16; o > 0; o >>= 1) k += __shfl_xor_sync(0xffffffffu, k, o);
    return k;
}

// A fragment's attributes at pixel centre (x, y): depth, colour and SrcX/SrcY interpolated
// linearly in screen space with the edge weights of `covers`.
struct Frag {
    float d, r, g, b, a, u, v;
    float c;  // Custom0 (perspective-corrected texture mapping only)
};
struct TriAttr {
    float4 ka, kb, kc;  // colour of the corners
    float da, db, dc;   // depth
    float ua, ub, uc, va, vb, vc;  // SrcX, SrcY
    float ca, cb, cc;   // Custom0
};
__device__ __forceinline__ TriAttr tri_attr(const RasterJob& J, uint32_t slot) {
    TriAttr A;
    A.ka = J.rgba[3 * (size_t)slot]; A.kb = J.rgba[3 * (size_t)slot + 1]; A.kc = J.rgba[3 * (size_t)slot + 2];
    A.da = J.depth[3 * (size_t)slot]; A.db = J.depth[3 * (size_t)slot + 1]; A.dc = J.depth[3 * (size_t)slot + 2];
    const float4 pa = J.xyuv[3 * (size_t)slot], pb = J.xyuv[3 * (size_t)slot + 1], pc = J.xyuv[3 * (size_t)slot + 2];
    A.ua = pa.z; A.ub = pb.z; A.uc = pc.z; A.va = pa.w; A.vb = pb.w; A.vc = pc.w;
    A.ca = A.cb = A.cc = 0.0f;
    if (J.custom0) {
        A.ca = J.custom0[3 * (size_t)slot]; A.cb = J.custom0[3 * (size_t)slot + 1]; A.cc = J.custom0[3 * (size_t)slot + 2];
    }
    return A;
}
__device__ __forceinline__ Frag interp(const TriAttr& A, float area, float wa, float wb, float wc) {
    Frag f;
    f.c = ((wa * A.ca + wb * A.cb) + wc * A.cc) / area;
    f.d = ((wa * A.da + wb * A.db) + wc * A.dc) / area;
    f.r = ((wa * A.ka.x + wb * A.kb.x) + wc * A.kc.x) / area;
    f.g = ((wa * A.ka.y + wb * A.kb.y) + wc * A.kc.y) / area;
    f.b = ((wa * A.ka.z + wb * A.kb.z) + wc * A.kc.z) / area;
    f.a = ((wa * A.ka.w + wb * A.kb.w) + wc * A.kc.w) / area;
    f.u = ((wa * A.ua + wb * A.ub) + wc * A.uc) / area;
    f.v = ((wa * A.va + wb * A.vb) + wc * A.vc) / area;
    return f;
}
// ---- device-wide exclusive scan of uint32 ------------------------------------
__device__ uint32_t block_exclusive(uint32_t v, uint32_t* sh, uint32_t& total) {
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    uint32_t incl = v;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t u = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (uint32_t)o) incl += u;
    }
    if (lane == 31) sh[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        uint32_t w = lane < nw ? sh[lane] : 0u, wi = w;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t u = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= (uint32_t)o) wi += u;
        }
        if (lane < nw) sh[lane] = wi - w;
        if (lane == nw - 1) sh[32] = wi;
    }
    __syncthreads();
    const uint32_t r = sh[wid] + incl - v;
    total = sh[32];
    __syncthreads();
    return r;
}

__global__ void k_scan_local(const uint32_t* __restrict__ in, uint32_t* out, uint32_t n, uint32_t* partial) {
    __shared__ uint32_t sh[33];
    const size_t base = (size_t)blockIdx.x * kScanChunk + (size_t)threadIdx.x * kScanPer;
    uint32_t v[kScanPer], s = 0;
#pragma unroll
    for (int k = 0; k < kScanPer; k++) {
        v[k] = base + k < n ? in[base + k] : 0u;
        s += v[k];
    }
    uint32_t total;
    uint32_t run = block_exclusive(s, sh, total);
#pragma unroll
    for (int k = 0; k < kScanPer; k++) {
        if (base + k < n) out[base + k] = run;
        run += v[k];
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = total;
}

__global__ void k_scan_add(uint32_t* out, uint32_t n, const uint32_t* __restrict__ partial_scanned) {
    const size_t base = (size_t)blockIdx.x * kScanChunk + (size_t)threadIdx.x * kScanPer;
    const uint32_t add = partial_scanned[blockIdx.x];
#pragma unroll
    for (int k = 0; k < kScanPer; k++)
        if (base + k < n) out[base + k] += add;
}

// One warp step of pass 1 over 32 triangles (`valid` lanes): classify each, count the small
// boxes, register the large ones, and append the hits in draw order.
__device__ __forceinline__ void count_step(const RasterJob& J, bool valid, const TriScreen& t, uint32_t slot, uint32_t seg,
                                           uint32_t u, uint32_t base, uint32_t lane, uint4* hits, BigTri* big,
                                           uint32_t* chunk_tri, unsigned long long* ctr, uint32_t& nh, uint32_t& frags) {
    uint32_t k = 0, ref = 0;
    bool hit = false, own_big = false;
    const uint32_t box = valid ? bbox_pixels(t) : 0u;
    const bool large = box > kBigBox;
    const uint32_t lm = __ballot_sync(0xffffffffu, large);
    unsigned long long b = 0, ch0 = 0;
    uint32_t nct = 0;
    if (lm) {  // one pair of atomics per warp for its large triangles
        nct = large ? (box + kBigChunk - 1) / kBigChunk : 0u;
        uint32_t tot;
        const uint32_t before = warp_exclusive(nct, lane, tot);
        unsigned long long b0 = 0, c0 = 0;
        if (lane == 0) {
            b0 = atomicAdd(&ctr[0], (unsigned long long)__popc(lm));
            c0 = atomicAdd(&ctr[1], (unsigned long long)tot);
        }
        b = __shfl_sync(0xffffffffu, b0, 0) + __popc(lm & ((1u << lane) - 1u));
        ch0 = __shfl_sync(0xffffffffu, c0, 0) + before;
    }
    if (large) {
        hit = true;
        own_big = true;
        const bool fits = b < J.big_cap && ch0 + nct <= kChunkCap;
        // the reserved chunks below the cap name their triangle, or none when it did not fit
        for (unsigned long long q = ch0; q < ch0 + nct && q < kChunkCap; q++)
            chunk_tri[q] = fits ? (uint32_t)b : 0xFFFFFFFFu;
        if (fits) {
            own_big = false;
            ref = (uint32_t)b + 1;
            BigTri& B = big[b];
            B.slot = slot;
            B.unit = u;
            B.chunk0 = (uint32_t)ch0;
        }
    } else if (box) {
        k = tri_fragments(t);
        hit = k != 0;
    }
    // large triangles the shared list could not take: the warp counts their pixels
    for (uint32_t m = __ballot_sync(0xffffffffu, own_big); m; m &= m - 1) {
        const int l = __ffs(m) - 1;
        const uint32_t cnt = warp_fragments(tri_screen(J, __shfl_sync(0xffffffffu, slot, l)), lane);
        if (lane == (uint32_t)l) k = cnt;
    }
    frags += k;
    const uint32_t hm = __ballot_sync(0xffffffffu, hit);
    if (hit) {
        const uint32_t pos = base + nh + __popc(hm & ((1u << lane) - 1u));
        hits[pos] = make_uint4(slot, seg, k, ref);
        if (ref) big[ref - 1].hit = pos;
    }
    nh += __popc(hm);
}

// Fragment pass 1, one warp per unit of kUnitTris triangles in draw order: count the pixel
// centres each covers and keep, in draw order, the triangles that may cover any:
// hits[u * kUnitTris + i] = (output slot, render pair, count, shared-list index + 1 or 0),
// uhits[u] of them, ufrags[u] fragments. A triangle whose box exceeds kBigBox pixels goes to
// the shared list (k_big_count adds its count); when the list is full its warp counts it.
// ctr[0] / ctr[1]: large triangles / chunks handed out.
__global__ void __launch_bounds__(kFragThreads, 4) k_frag_count(RasterJob J, uint32_t nunits, uint4* hits, uint32_t* uhits,
                                                             uint32_t* ufrags, BigTri* big, uint32_t* chunk_tri,
                                                             unsigned long long* ctr) {
    const uint32_t lane = threadIdx.x & 31, u = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (u >= nunits) return;  // the whole warp
    const uint32_t n = __ldg(&J.cbase[J.nseg]), base = u * kUnitTris;
    uint32_t nh = 0, frags = 0, pr = 0;
    // 64 triangles a step, two per lane, both loaded before either is classified
    for (uint32_t j = 0; j < kUnitTris && base + j < n; j += 64) {
        const uint32_t c0 = base + j + lane, c1 = c0 + 32;
        uint32_t slot0 = 0, seg0 = 0, slot1 = 0, seg1 = 0;
        float4 a0 = make_float4(0.f, 0.f, 0.f, 0.f), b0 = a0, d0 = a0, a1 = a0, b1 = a0, d1 = a0;
        if (c0 < n) {
            pr = find_pair(J, c0, j ? pr : 0u);
            seg0 = J.seg_lo + pr;
            slot0 = J.segs[seg0].out_base + (c0 - __ldg(&J.cbase[pr]));
            a0 = J.xyuv[3 * (size_t)slot0]; b0 = J.xyuv[3 * (size_t)slot0 + 1]; d0 = J.xyuv[3 * (size_t)slot0 + 2];
        }
        if (c1 < n) {
            pr = find_pair(J, c1, pr);
            seg1 = J.seg_lo + pr;
            slot1 = J.segs[seg1].out_base + (c1 - __ldg(&J.cbase[pr]));
            a1 = J.xyuv[3 * (size_t)slot1]; b1 = J.xyuv[3 * (size_t)slot1 + 1]; d1 = J.xyuv[3 * (size_t)slot1 + 2];
        }
        count_step(J, c0 < n, screen_of(J, a0, b0, d0), slot0, seg0, u, base, lane, hits, big, chunk_tri, ctr, nh, frags);
        count_step(J, c1 < n, screen_of(J, a1, b1, d1), slot1, seg1, u, base, lane, hits, big, chunk_tri, ctr, nh, frags);
    }
    for (int o = 16; o > 0; o >>= 1) frags += __shfl_xor_sync(0xffffffffu, frags, o);
    if (lane == 0) {
        uhits[u] = nh;
        ufrags[u] = frags;
    }
}

__device__ __forceinline__ uint32_t shared_chunks(const unsigned long long* ctr) {
    const unsigned long long c = ctr[1];
    return c < kChunkCap ? (uint32_t)c : kChunkCap;
}

// Counts of the shared large triangles: the grid's warps take kBigChunk-pixel chunks in turn
// and add each chunk's count to its triangle's hit and unit.
__global__ void __launch_bounds__(kFragThreads, 5) k_big_count(RasterJob J, const BigTri* __restrict__ big,
                                                           const uint32_t* __restrict__ chunk_tri,
                                                           const unsigned long long* __restrict__ ctr, uint4* hits,
                                                           uint32_t* ufrags) {
    const uint32_t lane = threadIdx.x & 31, nch = shared_chunks(ctr);
    const uint32_t nw = gridDim.x * (blockDim.x >> 5);
    for (uint32_t ch = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; ch < nch; ch += nw) {
        const uint32_t b = chunk_tri[ch];
        if (b == 0xFFFFFFFFu) continue;  // the same for the whole warp
        const BigTri B = big[b];
        const TriScreen t = tri_screen(J, B.slot);
        const uint32_t bw = (uint32_t)(t.x1 - t.x0 + 1), area = bbox_pixels(t);
        const uint32_t p0 = (ch - B.chunk0) * kBigChunk, p1 = min(p0 + kBigChunk, area);
        uint32_t k = 0;
        for (uint32_t i = p0 + lane; i < p1; i += 32) {
            float wa, wb, wc;
            if (covers(t, (float)(t.x0 + (int)(i % bw)) + 0.5f, (float)(t.y0 + (int)(i / bw)) + 0.5f, wa, wb, wc)) k++;
        }
        for (int o = 16; o > 0; o >>= 1) k += __shfl_xor_sync(0xffffffffu, k, o);
        if (lane == 0 && k) {
            atomicAdd(&hits[B.hit].z, k);
            atomicAdd(&ufrags[B.unit], k);
        }
    }
}

// Fragment pass 2, one warp per unit: the unit's hits write their fragments (key = pixel,
// value = the hit's index, which names its triangle and its place in draw order) from
// ufoff[u] on. A shared large triangle only sets its cursor; k_big_write fills its range.
__global__ void __launch_bounds__(kFragThreads, 4) k_frag_write(RasterJob J, uint32_t nunits, const uint4* __restrict__ hits,
                                                             const uint32_t* __restrict__ uhits,
                                                             const uint32_t* __restrict__ ufoff, BigTri* big,
                                                             uint32_t* keys, uint32_t* vals, const uint32_t* fcount) {
    const uint32_t lane = threadIdx.x & 31, u = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (u >= nunits || fcount[1] == 0u) return;  // the whole warp; nothing when the buffers are too small
    const uint32_t base = u * kUnitTris, nh = uhits[u];
    uint32_t run = ufoff[u];
    for (uint32_t j = 0; j < nh; j += 32) {
        const uint32_t i = j + lane;
        const uint4 h = i < nh ? hits[base + i] : make_uint4(0u, 0u, 0u, 0u);
        uint32_t total;
        const uint32_t o = run + warp_exclusive(h.z, lane, total);
        run += total;
        bool own_big = false;
        if (h.z) {
            if (h.w) {
                big[h.w - 1].cursor = o;
            } else {
                const TriScreen t = tri_screen(J, h.x);
                if (bbox_pixels(t) > kBigBox) {
                    own_big = true;
                } else {
                    uint32_t q = o;
                    for (int y = t.y0; y <= t.y1; y++)
                        for (int x = t.x0; x <= t.x1; x++) {
                            float wa, wb, wc;
                            if (covers(t, (float)x + 0.5f, (float)y + 0.5f, wa, wb, wc)) {
                                keys[q] = (uint32_t)y * (uint32_t)J.W + (uint32_t)x;
                                vals[q] = base + i;
                                q++;
                            }
                        }
                }
            }
        }
        // large triangles outside the shared list: the warp writes them, pixels row-major
        for (uint32_t m = __ballot_sync(0xffffffffu, own_big); m; m &= m - 1) {
            const int l = __ffs(m) - 1;
            const uint32_t slot = __shfl_sync(0xffffffffu, h.x, l), hidx = base + j + (uint32_t)l;
            uint32_t ob = __shfl_sync(0xffffffffu, o, l);
            const TriScreen t = tri_screen(J, slot);
            const uint32_t bw = (uint32_t)(t.x1 - t.x0 + 1), area = bbox_pixels(t);
            for (uint32_t b0 = 0; b0 < area; b0 += 32) {
                const uint32_t pi = b0 + lane;
                const int x = t.x0 + (int)(pi % bw), y = t.y0 + (int)(pi / bw);
                float wa, wb, wc;
                const bool in = pi < area && covers(t, (float)x + 0.5f, (float)y + 0.5f, wa, wb, wc);
                const uint32_t pm = __ballot_sync(0xffffffffu, in);
                if (in) {
                    const uint32_t q = ob + __popc(pm & ((1u << lane) - 1u));
                    keys[q] = (uint32_t)y * (uint32_t)J.W + (uint32_t)x;
                    vals[q] = hidx;
                }
                ob += __popc(pm);
            }
        }
    }
}

// Fragments of the shared large triangles: the grid's warps take chunks in turn; a chunk
// claims its part of the triangle's range with one atomic on the cursor. The order inside a
// triangle's range does not matter: a triangle has at most one fragment per pixel.
__global__ void __launch_bounds__(kFragThreads, 5) k_big_write(RasterJob J, BigTri* big, const uint32_t* __restrict__ chunk_tri,
                                                           const unsigned long long* __restrict__ ctr, uint32_t* keys,
                                                           uint32_t* vals, const uint32_t* fcount) {
    const uint32_t lane = threadIdx.x & 31, nch = fcount[1] ? shared_chunks(ctr) : 0u;
    const uint32_t nw = gridDim.x * (blockDim.x >> 5);
    for (uint32_t ch = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; ch < nch; ch += nw) {
        const uint32_t b = chunk_tri[ch];
        if (b == 0xFFFFFFFFu) continue;  // the same for the whole warp
        const uint32_t slot = big[b].slot, hidx = big[b].hit, chunk0 = big[b].chunk0;
        const TriScreen t = tri_screen(J, slot);
        const uint32_t bw = (uint32_t)(t.x1 - t.x0 + 1), area = bbox_pixels(t);
        const uint32_t p0 = (ch - chunk0) * kBigChunk, p1 = min(p0 + kBigChunk, area);
        uint32_t mask = 0, cnt = 0;  // lane's pixels p0 + lane + 32 q
        for (uint32_t q = 0, i = p0 + lane; q < kBigChunk / 32; q++, i += 32) {
            float wa, wb, wc;
            if (i < p1 && covers(t, (float)(t.x0 + (int)(i % bw)) + 0.5f, (float)(t.y0 + (int)(i / bw)) + 0.5f, wa, wb, wc)) {
                mask |= 1u << q;
                cnt++;
            }
        }
        uint32_t total;
        const uint32_t off = warp_exclusive(cnt, lane, total);
        uint32_t base = 0;
        if (lane == 0 && total) base = atomicAdd(&big[b].cursor, total);
        uint32_t o = __shfl_sync(0xffffffffu, base, 0) + off;
        for (uint32_t q = 0, i = p0 + lane; mask; q++, i += 32) {
            if (!((mask >> q) & 1u)) continue;
            mask &= ~(1u << q);
            keys[o] = (uint32_t)(t.y0 + (int)(i / bw)) * (uint32_t)J.W + (uint32_t)(t.x0 + (int)(i % bw));
            vals[o] = hidx;
            o++;
        }
    }
}

// ---- grouping fragments by pixel ------------------------------------------------
// A counting sort: k_pixel_count counts each pixel's fragments, their exclusive prefix gives
// each pixel its range, and k_pixel_scatter puts every fragment into its pixel's range through
// an atomic cursor. The order inside a range is whatever the atomics gave; k_pixels restores
// draw order by sorting the range by hit index (a triangle has at most one fragment per pixel,
// so the indices of a range are distinct and the sorted order is unique).
__global__ void k_pixel_scatter(const uint32_t* __restrict__ keys, const uint32_t* __restrict__ vals,
                                const uint32_t* __restrict__ fcount, const uint32_t* __restrict__ pstart,
                                uint32_t* cursor, uint32_t* ovals) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= fcount[1]) return;
    const uint32_t p = keys[i];
    ovals[pstart[p] + atomicAdd(&cursor[p], 1u)] = vals[i];
}

// Sorts v[0, n) ascending in place: insertion sort for short ranges, heapsort beyond.
__device__ __forceinline__ void sort_range(uint32_t* v, uint32_t n) {
    if (n <= 32) {
        for (uint32_t i = 1; i < n; i++) {
            const uint32_t x = v[i];
            uint32_t j = i;
            for (; j > 0 && v[j - 1] > x; j--) v[j] = v[j - 1];
            v[j] = x;
        }
        return;
    }
    auto sift = [&](uint32_t root, uint32_t end) {  // max-heap on v[0, end)
        const uint32_t x = v[root];
        uint32_t r = root;
        for (;;) {
            uint32_t c = 2 * r + 1;
            if (c >= end) break;
            if (c + 1 < end && v[c + 1] > v[c]) c++;
            if (v[c] <= x) break;
            v[r] = v[c];
            r = c;
        }
        v[r] = x;
    };
    for (uint32_t i = n / 2; i-- > 0;) sift(i, n);
    for (uint32_t end = n - 1; end > 0; end--) {
        const uint32_t t = v[0];
        v[0] = v[end];
        v[end] = t;
        sift(0, end);
    }
}

// ---- per-pixel replay --------------------------------------------------------
__device__ __forceinline__ float clamp01(float v) { return v < 0.0f ? 0.0f : (v > 1.0f ? 1.0f : v); }
__device__ __forceinline__ uint32_t q8(float v) { return (uint32_t)floorf(clamp01(v) * 255.0f + 0.5f); }
__device__ __forceinline__ float u8f(uint32_t p, int k) { return (float)((p >> (8 * k)) & 255u) / 255.0f; }
__device__ __forceinline__ uint32_t pack(uint32_t r, uint32_t g, uint32_t b, uint32_t a) {
    return r | (g << 8) | (b << 16) | (a << 24);
}
__device__ __forceinline__ float fractf(float v) { return v - floorf(v); }
// encodeDepth (camera.go:356-361) written to RGBA8
__device__ __forceinline__ uint32_t encode_depth(float d) {
    const float r = floorf(d * 255.0f) / 255.0f;
    const float g = floorf(fractf(d * 255.0f) * 255.0f) / 255.0f;
    const float b = fractf(d * 255.0f * 255.0f);
    return pack(q8(r), q8(g), q8(b), 255u);
}
// decodeDepth (camera.go:363-365)
__device__ __forceinline__ float decode_depth(uint32_t p) { return u8f(p, 0) + (u8f(p, 1) / 255.0f) + (u8f(p, 2) / 65025.0f); }
__device__ __forceinline__ float smoothstep(float e0, float e1, float x) {
    const float t = clamp01((x - e0) / (e1 - e0));
    return t * t * (3.0f - 2.0f * t);
}
// source-over onto a premultiplied RGBA8 pixel
__device__ __forceinline__ uint32_t blend_over(uint32_t dst, float r, float g, float b, float a) {
    r = clamp01(r); g = clamp01(g); b = clamp01(b); a = clamp01(a);
    const float k = 1.0f - a;
    return pack(q8(r + u8f(dst, 0) * k), q8(g + u8f(dst, 1) * k), q8(b + u8f(dst, 2) * k), q8(a + u8f(dst, 3) * k));
}

// ---- textures (shaders/base3d.kage:32-58, camera.go:419-478) -------------------
__device__ __forceinline__ float gmod(float x, float y) { return x - y * floorf(x / y); }  // GLSL mod
__device__ __forceinline__ float mixf(float a, float b, float t) { return a * (1.0f - t) + b * t; }  // GLSL mix
// the texel containing (px, py)
__device__ __forceinline__ float4 texel_at(const RasterJob& J, const RasterTex& T, float px, float py) {
    const float fx = floorf(px), fy = floorf(py);  // NaN reads texel 0
    const int ix = !(fx >= 0.0f) ? 0 : (fx >= (float)T.w ? T.w - 1 : (int)fx);
    const int iy = !(fy >= 0.0f) ? 0 : (fy >= (float)T.h ? T.h - 1 : (int)fy);
    const uint32_t p = J.texels[T.offset + (size_t)iy * T.w + ix];
    return make_float4(u8f(p, 0), u8f(p, 1), u8f(p, 2), u8f(p, 3));
}
// nearestFilter / bilinearFilter at texel coordinates (tx, ty)
__device__ float4 tex_sample(const RasterJob& J, const RasterTex& T, bool bilinear, float tx, float ty) {
    if (!bilinear) return texel_at(J, T, tx, ty);
    const float w = (float)T.w, h = (float)T.h;
    const float p0x = gmod(tx - 0.5f, w), p0y = gmod(ty - 0.5f, h);
    const float p1x = gmod(tx + 0.5f, w), p1y = gmod(ty + 0.5f, h);
    const float4 c0 = texel_at(J, T, p0x, p0y), c1 = texel_at(J, T, p1x, p0y);
    const float4 c2 = texel_at(J, T, p0x, p1y), c3 = texel_at(J, T, p1x, p1y);
    const float rx = fractf(p1x), ry = fractf(p1y);
    float4 r;
    r.x = mixf(mixf(c0.x, c1.x, rx), mixf(c2.x, c3.x, rx), ry);
    r.y = mixf(mixf(c0.y, c1.y, rx), mixf(c2.y, c3.y, rx), ry);
    r.z = mixf(mixf(c0.z, c1.z, rx), mixf(c2.z, c3.z, rx), ry);
    r.w = mixf(mixf(c0.w, c1.w, rx), mixf(c2.w, c3.w, rx), ry);
    return r;
}
// The flush's texel for the colour pass (base3d.kage:79-100): UV or screen mapped,
// wrapped with mod; the default white image when the flush has no texture.
__device__ float4 colour_texel(const RasterJob& J, const DevSeg& sg, float x, float y, const Frag& f) {
    if (sg.pad[1] == 0u) return make_float4(1.f, 1.f, 1.f, 1.f);
    const RasterTex T = J.texs[sg.pad[1] - 1];
    float tx = f.u, ty = f.v;
    if (sg.pad[2] & 2u) {
        tx = (x * sg.pad2[0]) + f.u; ty = (y * sg.pad2[1]) + f.v;
    } else if (J.custom0) {  // tx *= 1.0 / custom.x (base3d.kage:79-81)
        const float r = 1.0f / f.c;
        tx = tx * r; ty = ty * r;
    }
    tx = gmod(tx, (float)T.w);
    ty = gmod(ty, (float)T.h);
    return tex_sample(J, T, sg.pad[2] & 1u, tx, ty);
}
// The clip-alpha shader's texture alpha (camera.go:440-474): wrapped with fract.
__device__ float clip_alpha(const RasterJob& J, const DevSeg& sg, float x, float y, const Frag& f) {
    if (sg.pad[1] == 0u) return 1.0f;
    const RasterTex T = J.texs[sg.pad[1] - 1];
    const float w = (float)T.w, h = (float)T.h;
    float tx = f.u, ty = f.v;
    if (sg.pad[2] & 2u) {
        tx = (x * sg.pad2[0]) + f.u; ty = (y * sg.pad2[1]) + f.v;
    } else if (J.custom0) {  // camera.go:454-455
        const float r = 1.0f / f.c;
        tx = tx * r; ty = ty * r;
    }
    tx = fractf(tx / w) * w;
    ty = fractf(ty / h) * h;
    return tex_sample(J, T, sg.pad[2] & 1u, tx, ty).w;
}

// Fragment of the triangle in output slot `slot` at pixel centre (x, y).
__device__ __forceinline__ Frag fragment(const RasterJob& J, uint32_t slot, float x, float y) {
    const TriScreen t = tri_screen(J, slot);
    float wa, wb, wc;
    covers(t, x, y, wa, wb, wc);
    return interp(tri_attr(J, slot), t.area, wa, wb, wc);
}

// One thread per pixel replays the pixel's fragments in draw order (its range of fvals,
// grouped by pixel, sorted here by hit index); fvals[q] is the hit of fragment q's triangle:
// hits[fvals[q]] = (output slot, render pair, ...).
__global__ void __launch_bounds__(256, 5) k_pixels(RasterJob J, const uint32_t* __restrict__ pstart, const uint32_t* fvals,
                         const uint4* __restrict__ hits, uint32_t* color, uint32_t* depth) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= (uint32_t)(J.W * J.H)) return;
    const float x = (float)(p % (uint32_t)J.W) + 0.5f, y = (float)(p / (uint32_t)J.W) + 0.5f;
    uint32_t rc = 0u, rd = 0u;
    const uint32_t f0 = pstart[p], f1 = pstart[p + 1];
    uint32_t* fv = const_cast<uint32_t*>(fvals);  // this thread's own range: draw order first
    if (f1 - f0 > 1) sort_range(fv + f0, f1 - f0);
    uint32_t i = f0;
    while (i < f1) {
        // the fragments of one flush: a render pair, or all pairs of a dynamic batch
        // (pad[0] = flush number | transparent pass << 31)
        const DevSeg& sg = J.segs[hits[fvals[i]].y];  // the flush's state (the same on all its pairs)
        const uint32_t fl = sg.pad[0];
        uint32_t e = i + 1;
        while (e < f1 && J.segs[hits[fvals[e]].y].pad[0] == fl) e++;
        if (J.render_depth) {
            uint32_t inter = 0u;
            const bool clip = sg.pad[2] & 4u;
            for (uint32_t q = i; q < e; q++) {  // depth pass (camera.go:1882-1931)
                const Frag f = fragment(J, hits[fvals[q]].x, x, y);
                if (clip) {  // clip-alpha shader: (encodeDepth.rgb, texture alpha), blended source-over
                    const float ta = clip_alpha(J, sg, x, y, f);
                    if (ta <= 0.8f) continue;
                    if ((rd >> 24) == 0u || decode_depth(rd) > f.d) {
                        const uint32_t enc = encode_depth(f.d);
                        inter = blend_over(inter, u8f(enc, 0), u8f(enc, 1), u8f(enc, 2), ta);
                    }
                } else if ((rd >> 24) == 0u || decode_depth(rd) > f.d) {
                    inter = encode_depth(f.d);
                }
            }
            if ((inter >> 24) != 0u) {
                for (uint32_t q = i; q < e; q++) {  // colour pass (base3d.kage:67-145)
                    const Frag f = fragment(J, hits[fvals[q]].x, x, y);
                    const float4 tc = colour_texel(J, sg, x, y, f);
                    float r = tc.x * f.r, g = tc.y * f.g, b = tc.z * f.b;
                    const float a = tc.w * f.a;
                    r *= f.a; g *= f.a; b *= f.a;
                    if (!J.fogless && J.fog_mode >= 0 && J.fog_mode <= 2) {
                        const float dd = decode_depth(inter);
                        float v = dd;
                        if (J.fog_curve == 1) v = sqrtf(1.0f - (dd - 1.0f) * (dd - 1.0f));
                        else if (J.fog_curve == 2) v = 1.0f - sqrtf(1.0f - dd * dd);
                        float m = smoothstep(J.fog0, J.fog1, v);
                        if (J.dither > 0.0f) {
                            const int yc = (int)(y / J.dither) % 4, xc = (int)(x / J.dither) % 4;
                            m = (m - kBayer[yc * 4 + xc]) < 0.0f ? 0.0f : 1.0f;
                        }
                        if (J.fog_mode == 0) {
                            r += J.fog_r * m * a; g += J.fog_g * m * a; b += J.fog_b * m * a;
                        } else if (J.fog_mode == 1) {
                            r -= J.fog_r * m * a; g -= J.fog_g * m * a; b -= J.fog_b * m * a;
                        } else {
                            r = (r * (1.0f - m) + J.fog_r * m) * a;
                            g = (g * (1.0f - m) + J.fog_g * m) * a;
                            b = (b * (1.0f - m) + J.fog_b * m) * a;
                        }
                    }
                    rc = blend_over(rc, r, g, b, a);
                }
                // depth composite (DrawImage, source-over) unless the flush is transparent
                if (!(fl >> 31)) rd = blend_over(rd, u8f(inter, 0), u8f(inter, 1), u8f(inter, 2), u8f(inter, 3));
            }
        } else {
            for (uint32_t q = i; q < e; q++) {  // plain draw: texel times the premultiplied vertex colour
                const Frag f = fragment(J, hits[fvals[q]].x, x, y);
                const float4 tc = colour_texel(J, sg, x, y, f);
                rc = blend_over(rc, tc.x * (f.r * f.a), tc.y * (f.g * f.a), tc.z * (f.b * f.a), tc.w * f.a);
            }
        }
        i = e;
    }
    color[p] = rc;
    depth[p] = rd;
}

__global__ void k_pixel_count(const uint32_t* __restrict__ keys, const uint32_t* __restrict__ fcount, uint32_t* pcount) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < fcount[1]) atomicAdd(&pcount[keys[i]], 1u);
}

// The job's fragment total from the per-unit offsets: fcount[0] = total, fcount[1] = the total
// when it fits the `cap` entries of the fragment buffers, else 0 (the passes after it then do
// nothing and the host grows the buffers and rasterises again); pstart[npx] = fcount[1].
__global__ void k_frag_total(const uint32_t* __restrict__ ufoff, const uint32_t* __restrict__ ufrags, uint32_t nunits,
                             uint32_t cap, uint32_t* fcount, uint32_t* pstart_end) {
    const uint64_t nf = (uint64_t)ufoff[nunits - 1] + ufrags[nunits - 1];
    const uint32_t fit = nf <= cap ? (uint32_t)nf : 0u;
    fcount[0] = nf > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)nf;
    fcount[1] = fit;
    *pstart_end = fit;
}

struct RasterScratch {
    DevBuf cbase, hits, uhits, ufrags, ufoff, big, chunk_tri, ctr, keys, vals, vals2, partial[3], pstart, pcount,
        color, depth, fcount;
};

}  // namespace

struct t3d_raster_state {
    RasterScratch S;
    uint32_t frag_cap = 1u << 22;  // fragments the sort buffers hold (grow-only)
    int32_t W = 0, H = 0;
    bool valid = false;
    std::vector<RasterTex> tex;  // the texture table (host copy of `texs`)
    DevBuf texs, texels;
};

namespace {

int scan_u32(t3d_ctx* ctx, RasterScratch& S, const uint32_t* in, uint32_t* out, uint32_t n, cudaStream_t st, int level = 0) {
    if (n == 0) return T3D_OK;
    const uint32_t nb = (n + kScanChunk - 1) / kScanChunk;
    if (level > 2) {
        set_err(ctx, "raster: scan too large");
        return T3D_E_INVAL;
    }
    int rc;
    if ((rc = S.partial[level].ensure(ctx, 4ull * (nb + 1)))) return rc;
    uint32_t* part = (uint32_t*)S.partial[level].ptr;
    k_scan_local<<<nb, kScanThreads, 0, st>>>(in, out, n, part);
    if (nb > 1) {
        if ((rc = scan_u32(ctx, S, part, part, nb, st, level + 1))) return rc;
        k_scan_add<<<nb, kScanThreads, 0, st>>>(out, n, part);
    }
    CKR(cudaGetLastError());
    return T3D_OK;
}

}  // namespace

extern "C" {

int t3d_frame_raster(t3d_ctx* ctx, uint32_t job, const t3d_raster_opts* opts, void* stream) {
    if (!ctx) return T3D_E_INVAL;
    FrameTables& F = ctx->tables;
    if ((!ctx->frame_valid && !ctx->frame_pending) || job >= F.jobs.size()) {
        set_err(ctx, "frame_raster: no rendered frame or job %u out of range", job);
        return T3D_E_INVAL;
    }
    cudaSetDevice(ctx->device);
    cudaStream_t st = stream ? (cudaStream_t)stream : (ctx->last_stream ? ctx->last_stream : ctx->stream);
    if (ctx->last_stream && ctx->last_stream != st) CKR(cudaStreamSynchronize(ctx->last_stream));
    if (!ctx->raster) ctx->raster = new t3d_raster_state();
    t3d_raster_state& R = *ctx->raster;
    RasterScratch& S = R.S;
    const uint32_t seg_lo = job ? F.job_seg_end[job - 1] : 0u, seg_hi = F.job_seg_end[job];
    const uint32_t nseg = seg_hi - seg_lo;
    const JobCam& cam = F.jobs[job].cam;
    RasterJob J;
    memset(&J, 0, sizeof J);
    J.W = (int32_t)cam.W;
    J.H = (int32_t)cam.H;
    if (J.W <= 0 || J.H <= 0 || (uint64_t)J.W * J.H >= (1ull << 31)) {
        set_err(ctx, "frame_raster: bad image size %d x %d", J.W, J.H);
        return T3D_E_INVAL;
    }
    J.render_depth = cam.render_depth;
    J.fog_mode = cam.fog_on ? cam.fog_mode : -1;
    J.fog_r = cam.fog_color[0]; J.fog_g = cam.fog_color[1]; J.fog_b = cam.fog_color[2];
    J.fog0 = cam.fog_range[0]; J.fog1 = cam.fog_range[1];
    J.fog_curve = opts ? opts->fog_curve : 0;
    J.fogless = opts ? opts->fogless : 0;
    J.dither = opts ? opts->dither_size : 0.0f;
    {
        const int32_t sl = opts ? opts->shared_large_tris : 0;
        J.big_cap = sl == 0 ? kBigTriCap : (sl < 0 ? 0u : std::min<uint32_t>((uint32_t)sl, kBigTriCap));
    }
    J.xyuv = (const float4*)ctx->out_xyuv.ptr;
    J.rgba = (const float4*)ctx->out_rgba.ptr;
    J.depth = (const float*)ctx->out_depth.ptr;
    J.custom0 = cam.persp_correct ? (const float*)ctx->out_invw.ptr : nullptr;
    J.segs = ctx->params.segs;
    J.texs = (const RasterTex*)R.texs.ptr;
    J.texels = (const uint32_t*)R.texels.ptr;
    uint64_t cap = 0;
    for (uint32_t s = seg_lo; s < seg_hi; s++) {
        const DevSeg& sg = F.segs[s];
        cap += sg.tri_count;
        const uint32_t t = sg.pad[1];
        if (!t) continue;
        if (t > R.tex.size()) {
            set_err(ctx, "frame_raster: texture %u of a material is not in the table of %zu", t, R.tex.size());
            return T3D_E_INVAL;
        }
    }
    const uint64_t npx = (uint64_t)J.W * J.H;
    int rc;
    // the fragment passes run one warp per kUnitTris triangles: of the job's visible count
    // when a frame sync has brought it to the host, else of its capacity (the device's count
    // n = cbase[nseg] bounds the work either way; units past it only record zeros)
    uint64_t span = cap;
    if (ctx->frame_valid && !ctx->frame_pending) {
        span = 0;
        for (uint32_t s = seg_lo; s < seg_hi; s++) span += F.seg_info[s].count;
    }
    const uint32_t nunits = (uint32_t)std::max<uint64_t>(1, (span + kUnitTris - 1) / kUnitTris);
    const uint32_t fblocks = (nunits + kFragThreads / 32 - 1) / (kFragThreads / 32);
    const uint32_t bigblocks = (uint32_t)std::max(1, ctx->num_sms) * 5;  // 5 resident blocks of 256 per SM
    if ((rc = S.cbase.ensure(ctx, 4ull * (nseg + 1))) || (rc = S.hits.ensure(ctx, 16ull * kUnitTris * nunits)) ||
        (rc = S.uhits.ensure(ctx, 4ull * nunits)) || (rc = S.ufrags.ensure(ctx, 4ull * nunits)) ||
        (rc = S.ufoff.ensure(ctx, 4ull * nunits)) || (rc = S.big.ensure(ctx, sizeof(BigTri) * (size_t)kBigTriCap)) ||
        (rc = S.chunk_tri.ensure(ctx, 4ull * kChunkCap)) || (rc = S.ctr.ensure(ctx, 16)) ||
        (rc = S.pstart.ensure(ctx, 4 * (npx + 1))) || (rc = S.pcount.ensure(ctx, 4 * npx)) ||
        (rc = S.color.ensure(ctx, 4 * npx)) || (rc = S.depth.ensure(ctx, 4 * npx)))
        return rc;
    J.cbase = (const uint32_t*)S.cbase.ptr;
    J.seg_lo = seg_lo;
    J.nseg = nseg;
    BigTri* big = (BigTri*)S.big.ptr;
    uint32_t* chunk_tri = (uint32_t*)S.chunk_tri.ptr;
    unsigned long long* ctr = (unsigned long long*)S.ctr.ptr;
    // 1. the job's visible triangles in draw order: per-pair prefix of the visible counts
    k_seg_bases<<<1, 1024, 0, st>>>((const uint32_t*)ctx->seg_count.ptr, seg_lo, nseg, (uint32_t*)S.cbase.ptr);
    // 2. fragments in draw order: count and keep the covering triangles, then write
    CKR(cudaMemsetAsync(ctr, 0, 16, st));
    k_frag_count<<<fblocks, kFragThreads, 0, st>>>(J, nunits, (uint4*)S.hits.ptr, (uint32_t*)S.uhits.ptr,
                                                   (uint32_t*)S.ufrags.ptr, big, chunk_tri, ctr);
    k_big_count<<<bigblocks, kFragThreads, 0, st>>>(J, big, chunk_tri, ctr, (uint4*)S.hits.ptr, (uint32_t*)S.ufrags.ptr);
    if ((rc = scan_u32(ctx, S, (const uint32_t*)S.ufrags.ptr, (uint32_t*)S.ufoff.ptr, nunits, st))) return rc;
    // the fragment total stays on the device: the buffers after this point hold `fcap` fragments
    // (the last raster's total and an eighth more, grow-only); a larger total is found at the
    // end of the call, which then grows them and runs again
    const uint32_t fcap = R.frag_cap;
    if ((rc = S.keys.ensure(ctx, 4ull * fcap)) || (rc = S.vals.ensure(ctx, 4ull * fcap)) ||
        (rc = S.vals2.ensure(ctx, 4ull * fcap)) || (rc = S.fcount.ensure(ctx, 16)))
        return rc;
    uint32_t* fcount = (uint32_t*)S.fcount.ptr;
    k_frag_total<<<1, 1, 0, st>>>((const uint32_t*)S.ufoff.ptr, (const uint32_t*)S.ufrags.ptr, nunits, fcap, fcount,
                                  (uint32_t*)S.pstart.ptr + npx);
    uint32_t *kin = (uint32_t*)S.keys.ptr, *vin = (uint32_t*)S.vals.ptr, *vout = (uint32_t*)S.vals2.ptr;
    k_frag_write<<<fblocks, kFragThreads, 0, st>>>(J, nunits, (const uint4*)S.hits.ptr, (const uint32_t*)S.uhits.ptr,
                                                   (const uint32_t*)S.ufoff.ptr, big, kin, vin, fcount);
    k_big_write<<<bigblocks, kFragThreads, 0, st>>>(J, big, chunk_tri, ctr, kin, vin, fcount);
    // 3. fragments grouped by pixel (pstart[npx], the total, was written by k_frag_total): counts,
    // their prefix, then each fragment into its pixel's range (the counts zeroed again serve as
    // the ranges' cursors)
    CKR(cudaMemsetAsync(S.pcount.ptr, 0, 4 * npx, st));
    k_pixel_count<<<(fcap + 255) / 256, 256, 0, st>>>(kin, fcount, (uint32_t*)S.pcount.ptr);
    if ((rc = scan_u32(ctx, S, (const uint32_t*)S.pcount.ptr, (uint32_t*)S.pstart.ptr, (uint32_t)npx, st))) return rc;
    CKR(cudaMemsetAsync(S.pcount.ptr, 0, 4 * npx, st));
    k_pixel_scatter<<<(fcap + 255) / 256, 256, 0, st>>>(kin, vin, fcount, (const uint32_t*)S.pstart.ptr,
                                                        (uint32_t*)S.pcount.ptr, vout);
    // 4. replay per pixel, each pixel's range sorted into draw order first
    k_pixels<<<(uint32_t)((npx + 255) / 256), 256, 0, st>>>(J, (const uint32_t*)S.pstart.ptr, vout,
                                                           (const uint4*)S.hits.ptr, (uint32_t*)S.color.ptr,
                                                           (uint32_t*)S.depth.ptr);
    CKR(cudaGetLastError());
    uint32_t fc[2] = {0u, 0u};
    CKR(cudaMemcpyAsync(fc, fcount, 8, cudaMemcpyDeviceToHost, st));
    CKR(cudaStreamSynchronize(st));
    if (fc[0] != 0u && fc[1] == 0u) {  // more fragments than the buffers hold: grow them, rasterise again
        if (fc[0] > 0xF0000000u) {
            set_err(ctx, "frame_raster: %u fragments exceed 32-bit fragment indices", fc[0]);
            return T3D_E_INVAL;
        }
        R.frag_cap = fc[0] + fc[0] / 8 + 1024;
        return t3d_frame_raster(ctx, job, opts, stream);
    }
    R.frag_cap = std::max(R.frag_cap, fc[0] + fc[0] / 8);
    R.W = J.W;
    R.H = J.H;
    R.valid = true;
    return T3D_OK;
}

int t3d_raster_set_textures(t3d_ctx* ctx, const t3d_texture_desc* textures, uint32_t n) {
    if (!ctx || (n && !textures)) return T3D_E_INVAL;
    uint64_t total = 0;
    for (uint32_t k = 0; k < n; k++) {
        const t3d_texture_desc& d = textures[k];
        if (!d.rgba8 || d.width <= 0 || d.height <= 0 || d.width > 32768 || d.height > 32768) {
            set_err(ctx, "raster_set_textures: texture %u has no texels or a bad size %d x %d", k, d.width, d.height);
            return T3D_E_INVAL;
        }
        total += (uint64_t)d.width * d.height;
    }
    if (total >= (1ull << 32)) {
        set_err(ctx, "raster_set_textures: %llu texels is more than 32-bit offsets address", (unsigned long long)total);
        return T3D_E_INVAL;
    }
    cudaSetDevice(ctx->device);
    if (ctx->last_stream) CKR(cudaStreamSynchronize(ctx->last_stream));  // a raster in flight reads the table
    if (!ctx->raster) ctx->raster = new t3d_raster_state();
    t3d_raster_state& R = *ctx->raster;
    std::vector<RasterTex> tex(n);
    uint64_t off = 0;
    for (uint32_t k = 0; k < n; k++) {
        tex[k].offset = (uint32_t)off;
        tex[k].w = textures[k].width;
        tex[k].h = textures[k].height;
        tex[k].pad = 0;
        off += (uint64_t)textures[k].width * textures[k].height;
    }
    int rc;
    if ((rc = R.texs.ensure(ctx, sizeof(RasterTex) * std::max(1u, n))) || (rc = R.texels.ensure(ctx, 4 * std::max<uint64_t>(1, total))))
        return rc;
    if (n) CKR(cudaMemcpy(R.texs.ptr, tex.data(), sizeof(RasterTex) * n, cudaMemcpyHostToDevice));
    for (uint32_t k = 0; k < n; k++)
        CKR(cudaMemcpy((uint32_t*)R.texels.ptr + tex[k].offset, textures[k].rgba8,
                       4ull * textures[k].width * textures[k].height, cudaMemcpyHostToDevice));
    R.tex = std::move(tex);
    return T3D_OK;
}

int t3d_frame_images(t3d_ctx* ctx, uint8_t* color_rgba8, uint8_t* depth_rgba8, int32_t* width, int32_t* height) {
    if (!ctx) return T3D_E_INVAL;
    if (!ctx->raster || !ctx->raster->valid) {
        set_err(ctx, "frame_images: nothing rasterised");
        return T3D_E_INVAL;
    }
    t3d_raster_state& R = *ctx->raster;
    if (width) *width = R.W;
    if (height) *height = R.H;
    cudaSetDevice(ctx->device);
    const size_t bytes = 4ull * R.W * R.H;
    if (color_rgba8) CKR(cudaMemcpy(color_rgba8, R.S.color.ptr, bytes, cudaMemcpyDeviceToHost));
    if (depth_rgba8) CKR(cudaMemcpy(depth_rgba8, R.S.depth.ptr, bytes, cudaMemcpyDeviceToHost));
    return T3D_OK;
}

}  // extern "C"

void t3d_raster_release(t3d_ctx* ctx) {
    if (!ctx->raster) return;
    RasterScratch& S = ctx->raster->S;
    for (DevBuf* b : {&S.cbase, &S.hits, &S.uhits, &S.ufrags, &S.ufoff, &S.big, &S.chunk_tri, &S.ctr, &S.keys, &S.vals, &S.vals2,
                      &S.partial[0], &S.partial[1], &S.partial[2], &S.pstart, &S.pcount, &S.color,
                      &S.depth, &S.fcount, &ctx->raster->texs, &ctx->raster->texels})
        b->release();
    delete ctx->raster;
    ctx->raster = nullptr;
}
