// TEST INFRASTRUCTURE ONLY: the oracle of t3d_frame_raster.
//
// A sequential restatement of the colour and depth passes of Tetra3D's flush
// (camera.go:1829-2048) as ebiten would draw them: per render pair in draw order,
// the depth pass of the depth shader (camera.go:350-383) into a cleared RGBA8
// intermediate, tested against the depth texture of the pairs before and
// composited into it unless the pair is transparent; the colour pass of
// shaders/base3d.kage:67-145: the flush material's texture (nearest or bilinear,
// wrapped with mod, UV or screen mapped; the default white image, tetra3d.go:12,
// :38, without one) times the vertex colour, fog curves and Bayer dithering
// (camera.go:1257-1262); for TransparencyModeAlphaClip the clip-alpha shader
// (camera.go:390-480) in the depth pass; with RenderDepth off, ebiten's plain
// draw of the texture times straight-alpha vertex colours. ebiten v2.9.7
// conventions restated: premultiplied RGBA8 images cleared to 0, fragments at
// pixel centres, top-left fill rule, attributes interpolated linearly in
// screen space, unorm8 writes rounded to nearest after clamping to [0, 1].
// PARITY UNPINNED: the rasteriser of the reference is ebiten's GPU pipeline,
// which no machine here can run; this restatement pins the device version.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "t3d_oracle.h"

namespace {

const float kBayer[16] = {1.0f / 17.0f,  9.0f / 17.0f, 3.0f / 17.0f,  11.0f / 17.0f, 13.0f / 17.0f, 5.0f / 17.0f,
                          15.0f / 17.0f, 7.0f / 17.0f, 4.0f / 17.0f,  12.0f / 17.0f, 2.0f / 17.0f,  10.0f / 17.0f,
                          16.0f / 17.0f, 8.0f / 17.0f, 14.0f / 17.0f, 6.0f / 17.0f};

struct Tri {
    float ax, ay, bx, by, cx, cy, area;
    int x0, x1, y0, y1;
    bool ok;
};

Tri tri_of(const float* xyuv, uint32_t c, int W, int H) {
    Tri t;
    const float* p = xyuv + 12 * (size_t)c;
    t.ax = p[0]; t.ay = p[1]; t.bx = p[4]; t.by = p[5]; t.cx = p[8]; t.cy = p[9];
    t.area = (t.bx - t.ax) * (t.cy - t.ay) - (t.by - t.ay) * (t.cx - t.ax);
    t.ok = t.area != 0.0f && std::isfinite(t.area);
    const float mnx = fminf(fminf(t.ax, t.bx), t.cx), mxx = fmaxf(fmaxf(t.ax, t.bx), t.cx);
    const float mny = fminf(fminf(t.ay, t.by), t.cy), mxy = fmaxf(fmaxf(t.ay, t.by), t.cy);
    t.x0 = (int)fminf(fmaxf(0.0f, ceilf(mnx - 0.5f)), (float)W);
    t.x1 = (int)fmaxf(fminf((float)W - 1.0f, floorf(mxx - 0.5f)), -1.0f);
    t.y0 = (int)fminf(fmaxf(0.0f, ceilf(mny - 0.5f)), (float)H);
    t.y1 = (int)fmaxf(fminf((float)H - 1.0f, floorf(mxy - 0.5f)), -1.0f);
    if (!(mnx == mnx) || !(mny == mny) || !(mxx == mxx) || !(mxy == mxy)) t.ok = false;
    return t;
}

bool tl_edge(float dx, float dy) { return dy < 0.0f || (dy == 0.0f && dx > 0.0f); }

bool covers(const Tri& t, float x, float y, float& wa, float& wb, float& wc) {
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

float clamp01(float v) { return v < 0.0f ? 0.0f : (v > 1.0f ? 1.0f : v); }
uint32_t q8(float v) { return (uint32_t)floorf(clamp01(v) * 255.0f + 0.5f); }
float u8f(uint32_t p, int k) { return (float)((p >> (8 * k)) & 255u) / 255.0f; }
uint32_t pack(uint32_t r, uint32_t g, uint32_t b, uint32_t a) { return r | (g << 8) | (b << 16) | (a << 24); }
float fractf(float v) { return v - floorf(v); }
// encodeDepth / decodeDepth (camera.go:356-365)
uint32_t encode_depth(float d) {
    const float r = floorf(d * 255.0f) / 255.0f;
    const float g = floorf(fractf(d * 255.0f) * 255.0f) / 255.0f;
    const float b = fractf(d * 255.0f * 255.0f);
    return pack(q8(r), q8(g), q8(b), 255u);
}
float decode_depth(uint32_t p) { return u8f(p, 0) + (u8f(p, 1) / 255.0f) + (u8f(p, 2) / 65025.0f); }
float smoothstep(float e0, float e1, float x) {
    const float t = clamp01((x - e0) / (e1 - e0));
    return t * t * (3.0f - 2.0f * t);
}
uint32_t blend_over(uint32_t dst, float r, float g, float b, float a) {
    r = clamp01(r); g = clamp01(g); b = clamp01(b); a = clamp01(a);
    const float k = 1.0f - a;
    return pack(q8(r + u8f(dst, 0) * k), q8(g + u8f(dst, 1) * k), q8(b + u8f(dst, 2) * k), q8(a + u8f(dst, 3) * k));
}

// ---- textures (shaders/base3d.kage:32-58 and the clip-alpha shader, camera.go:419-478) ----
float gmod(float x, float y) { return x - y * floorf(x / y); }  // GLSL mod
float mixf(float a, float b, float t) { return a * (1.0f - t) + b * t; }  // GLSL mix
struct Texel {
    float r, g, b, a;
};
// the texel of texture t containing the point (px, py), clamped to the image
Texel texel_at(const t3d_oracle_textures* tx, uint32_t t, float px, float py) {
    const int w = tx->tex_w[t], h = tx->tex_h[t];
    const float fx = floorf(px), fy = floorf(py);  // NaN reads texel 0
    const int ix = !(fx >= 0.0f) ? 0 : (fx >= (float)w ? w - 1 : (int)fx);
    const int iy = !(fy >= 0.0f) ? 0 : (fy >= (float)h ? h - 1 : (int)fy);
    const uint32_t p = tx->texels[tx->tex_offset[t] + (size_t)iy * w + ix];
    return {u8f(p, 0), u8f(p, 1), u8f(p, 2), u8f(p, 3)};
}
// nearestFilter / bilinearFilter
Texel sample(const t3d_oracle_textures* tx, uint32_t t, bool bilinear, float px, float py) {
    if (!bilinear) return texel_at(tx, t, px, py);
    const float w = (float)tx->tex_w[t], h = (float)tx->tex_h[t];
    const float p0x = gmod(px - 0.5f, w), p0y = gmod(py - 0.5f, h);
    const float p1x = gmod(px + 0.5f, w), p1y = gmod(py + 0.5f, h);
    const Texel c0 = texel_at(tx, t, p0x, p0y), c1 = texel_at(tx, t, p1x, p0y);
    const Texel c2 = texel_at(tx, t, p0x, p1y), c3 = texel_at(tx, t, p1x, p1y);
    const float rx = fractf(p1x), ry = fractf(p1y);
    return {mixf(mixf(c0.r, c1.r, rx), mixf(c2.r, c3.r, rx), ry), mixf(mixf(c0.g, c1.g, rx), mixf(c2.g, c3.g, rx), ry),
            mixf(mixf(c0.b, c1.b, rx), mixf(c2.b, c3.b, rx), ry), mixf(mixf(c0.a, c1.a, rx), mixf(c2.a, c3.a, rx), ry)};
}
// the source position of a fragment: SrcX/SrcY, screen mapped (TextureMapMode 1), or
// under perspective correction times 1 / Custom0 (base3d.kage:77-81, camera.go:452-455);
// c is null when the camera does not correct
void src_pos(const t3d_oracle_textures* tx, uint32_t fl, float x, float y, float u, float v, const float* c, float& px,
             float& py) {
    px = u;
    py = v;
    if (tx->flush_flags[fl] & 2u) {
        px = (x * tx->flush_scale[2 * fl]) + u;
        py = (y * tx->flush_scale[2 * fl + 1]) + v;
    } else if (c) {
        const float r = 1.0f / *c;
        px = px * r;
        py = py * r;
    }
}
// the colour pass's texel: wrapped with mod (base3d.kage:86); white without a texture
Texel colour_texel(const t3d_oracle_textures* tx, uint32_t fl, float x, float y, float u, float v, const float* c) {
    if (!tx || tx->flush_texture[fl] == 0u) return {1.0f, 1.0f, 1.0f, 1.0f};
    const uint32_t t = tx->flush_texture[fl] - 1;
    float px, py;
    src_pos(tx, fl, x, y, u, v, c, px, py);
    px = gmod(px, (float)tx->tex_w[t]);
    py = gmod(py, (float)tx->tex_h[t]);
    return sample(tx, t, tx->flush_flags[fl] & 1u, px, py);
}
// the clip-alpha shader's texture alpha: wrapped with fract of the UV (camera.go:458-465)
float clip_alpha(const t3d_oracle_textures* tx, uint32_t fl, float x, float y, float u, float v, const float* c) {
    if (tx->flush_texture[fl] == 0u) return 1.0f;
    const uint32_t t = tx->flush_texture[fl] - 1;
    const float w = (float)tx->tex_w[t], h = (float)tx->tex_h[t];
    float px, py;
    src_pos(tx, fl, x, y, u, v, c, px, py);
    px = fractf(px / w) * w;
    py = fractf(py / h) * h;
    return sample(tx, t, tx->flush_flags[fl] & 1u, px, py).a;
}

}  // namespace

extern "C" int t3d_oracle_raster(const t3d_camera_desc* cam, int32_t fog_curve, float dither, int32_t fogless,
                                 uint32_t n, const float* xyuv, const float* rgba, const float* depth,
                                 const uint32_t* tri_pair, const uint8_t* pair_transparent,
                                 const t3d_oracle_textures* tex, uint32_t* color_out, uint32_t* depth_out,
                                 const float* custom0) {
    const int W = cam->width, H = cam->height;
    if (W <= 0 || H <= 0) return -1;
    const int fog_mode = cam->fog_on ? cam->fog_mode : -1;
    std::vector<std::vector<uint32_t>> lists((size_t)W * H);
    for (uint32_t c = 0; c < n; c++) {  // fragments in draw order
        const Tri t = tri_of(xyuv, c, W, H);
        if (!t.ok) continue;
        for (int y = t.y0; y <= t.y1; y++)
            for (int x = t.x0; x <= t.x1; x++) {
                float wa, wb, wc;
                if (covers(t, (float)x + 0.5f, (float)y + 0.5f, wa, wb, wc)) lists[(size_t)y * W + x].push_back(c);
            }
    }
    for (int py = 0; py < H; py++)
        for (int px = 0; px < W; px++) {
            const float x = (float)px + 0.5f, y = (float)py + 0.5f;
            const std::vector<uint32_t>& L = lists[(size_t)py * W + px];
            const bool pc = cam->perspective_corrected && custom0;
            auto frag = [&](uint32_t c, float* out7) {  // depth, r, g, b, a, SrcX, SrcY, Custom0
                const Tri t = tri_of(xyuv, c, W, H);
                float wa, wb, wc;
                covers(t, x, y, wa, wb, wc);
                const float* k = rgba + 12 * (size_t)c;
                const float* d = depth + 3 * (size_t)c;
                const float* p = xyuv + 12 * (size_t)c;
                out7[0] = ((wa * d[0] + wb * d[1]) + wc * d[2]) / t.area;
                for (int q = 0; q < 4; q++) out7[1 + q] = ((wa * k[q] + wb * k[4 + q]) + wc * k[8 + q]) / t.area;
                for (int q = 0; q < 2; q++) out7[5 + q] = ((wa * p[2 + q] + wb * p[6 + q]) + wc * p[10 + q]) / t.area;
                out7[7] = 0.0f;
                if (pc) {
                    const float* cw = custom0 + 3 * (size_t)c;
                    out7[7] = ((wa * cw[0] + wb * cw[1]) + wc * cw[2]) / t.area;
                }
            };
            uint32_t rc = 0, rd = 0;
            size_t i = 0;
            while (i < L.size()) {
                const uint32_t s = tri_pair[L[i]];
                size_t e = i + 1;
                while (e < L.size() && tri_pair[L[e]] == s) e++;
                float f[8];
                if (cam->render_depth) {
                    uint32_t inter = 0;
                    const bool clip = tex && (tex->flush_flags[s] & 4u);
                    for (size_t q = i; q < e; q++) {
                        frag(L[q], f);
                        if (clip) {  // discard at texture alpha <= 0.8; (encodeDepth.rgb, alpha) over the intermediate
                            const float ta = clip_alpha(tex, s, x, y, f[5], f[6], pc ? &f[7] : nullptr);
                            if (ta <= 0.8f) continue;
                            if ((rd >> 24) == 0u || decode_depth(rd) > f[0]) {
                                const uint32_t enc = encode_depth(f[0]);
                                inter = blend_over(inter, u8f(enc, 0), u8f(enc, 1), u8f(enc, 2), ta);
                            }
                        } else if ((rd >> 24) == 0u || decode_depth(rd) > f[0]) {
                            inter = encode_depth(f[0]);
                        }
                    }
                    if ((inter >> 24) != 0u) {
                        for (size_t q = i; q < e; q++) {
                            frag(L[q], f);
                            const Texel tc = colour_texel(tex, s, x, y, f[5], f[6], pc ? &f[7] : nullptr);
                            float r = tc.r * f[1], g = tc.g * f[2], b = tc.b * f[3];
                            const float a = tc.a * f[4];
                            r *= f[4]; g *= f[4]; b *= f[4];
                            if (!fogless && fog_mode >= 0 && fog_mode <= 2) {
                                const float dd = decode_depth(inter);
                                float v = dd;
                                if (fog_curve == 1) v = sqrtf(1.0f - (dd - 1.0f) * (dd - 1.0f));
                                else if (fog_curve == 2) v = 1.0f - sqrtf(1.0f - dd * dd);
                                float m = smoothstep(cam->fog_range[0], cam->fog_range[1], v);
                                if (dither > 0.0f) {
                                    const int yc = (int)(y / dither) % 4, xc = (int)(x / dither) % 4;
                                    m = (m - kBayer[yc * 4 + xc]) < 0.0f ? 0.0f : 1.0f;
                                }
                                const float fr = cam->fog_color[0], fg = cam->fog_color[1], fb = cam->fog_color[2];
                                if (fog_mode == 0) {
                                    r += fr * m * a; g += fg * m * a; b += fb * m * a;
                                } else if (fog_mode == 1) {
                                    r -= fr * m * a; g -= fg * m * a; b -= fb * m * a;
                                } else {
                                    r = (r * (1.0f - m) + fr * m) * a;
                                    g = (g * (1.0f - m) + fg * m) * a;
                                    b = (b * (1.0f - m) + fb * m) * a;
                                }
                            }
                            rc = blend_over(rc, r, g, b, a);
                        }
                        // DrawImage of the intermediate: source-over
                        if (!pair_transparent[s])
                            rd = blend_over(rd, u8f(inter, 0), u8f(inter, 1), u8f(inter, 2), u8f(inter, 3));
                    }
                } else {
                    for (size_t q = i; q < e; q++) {
                        frag(L[q], f);
                        const Texel tc = colour_texel(tex, s, x, y, f[5], f[6], pc ? &f[7] : nullptr);
                        rc = blend_over(rc, tc.r * (f[1] * f[4]), tc.g * (f[2] * f[4]), tc.b * (f[3] * f[4]), tc.a * f[4]);
                    }
                }
                i = e;
            }
            color_out[(size_t)py * W + px] = rc;
            depth_out[(size_t)py * W + px] = rd;
        }
    return 0;
}
