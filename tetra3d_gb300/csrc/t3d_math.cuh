// t3d_math.cuh -- binary32 Matrix4 / Vector3 arithmetic shared by the host
// runtime and the device kernels.
//
// Every operation keeps Tetra3D's operation order (left-to-right sums, no
// fused multiply-add) so that host and device results are bit-identical to an
// unfused IEEE evaluation of the Go reference. The translation unit must be
// compiled with -fmad=false (device) and -ffp-contract=off (host), with IEEE
// division and square root (nvcc's defaults -prec-div=true -prec-sqrt=true).
#pragma once

#include <math.h>
#include <stdint.h>

#if defined(__CUDACC__)
#define T3D_HD __host__ __device__ __forceinline__
#else
#define T3D_HD inline
#endif

namespace t3d {

struct f3 { float x, y, z; };
struct f4 { float x, y, z, w; };
struct m4 { float m[4][4]; };

T3D_HD f3 mk3(float x, float y, float z) { f3 r; r.x = x; r.y = y; r.z = z; return r; }
T3D_HD f3 add3(f3 a, f3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }   // Vector3.Add, vector.go:86
T3D_HD f3 sub3(f3 a, f3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }   // Vector3.Sub, vector.go:112
T3D_HD f3 hmul3(f3 a, f3 b) { return mk3(a.x * b.x, a.y * b.y, a.z * b.z); }  // Vector3.Mult
T3D_HD f3 neg3(f3 a) { return mk3(-a.x, -a.y, -a.z); }                        // Vector3.Invert
T3D_HD float dot3(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }   // Vector3.Dot, vector.go:526

// math32.Sqrt is float32(math.Sqrt(float64(x))): the correctly rounded binary32
// square root, which is what IEEE sqrtf returns.
T3D_HD float sqrt_rn(float x) { return sqrtf(x); }

T3D_HD float mag3(f3 a) { return sqrt_rn(a.x * a.x + a.y * a.y + a.z * a.z); }  // vector.go:191
T3D_HD float dist2(f3 a, f3 b) {                                                // vector.go:242-247
    float x = a.x - b.x, y = a.y - b.y, z = a.z - b.z;
    return x * x + y * y + z * z;
}
// Vector3.Unit (vector.go:258-266): unchanged when the length is < 1e-8 or exactly 1.
T3D_HD f3 unit3(f3 a) {
    float l = mag3(a);
    if (l < 1e-8f || l == 1.0f) return a;
    return mk3(a.x / l, a.y / l, a.z / l);
}

T3D_HD m4 ident() {
    m4 r;
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) r.m[i][j] = (i == j) ? 1.0f : 0.0f;
    return r;
}
T3D_HD m4 load16(const float* p) {
    m4 r;
    for (int i = 0; i < 16; i++) r.m[i >> 2][i & 3] = p[i];
    return r;
}
T3D_HD void store16(const m4& a, float* p) {
    for (int i = 0; i < 16; i++) p[i] = a.m[i >> 2][i & 3];
}
// Matrix4.Mult (matrix_none.go:6-32; matrix_amd64.s computes the same sums).
T3D_HD m4 mult(const m4& a, const m4& b) {
    m4 n;
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++)
            n.m[i][j] = a.m[i][0] * b.m[0][j] + a.m[i][1] * b.m[1][j] + a.m[i][2] * b.m[2][j] + a.m[i][3] * b.m[3][j];
    return n;
}
T3D_HD m4 transposed(const m4& a) {  // matrix.go:218-230
    m4 n;
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) n.m[i][j] = a.m[j][i];
    return n;
}
// Matrix4.MultVec (matrix.go:619-627): row vector times matrix, translation added last.
T3D_HD f3 mult_vec(const m4& m, f3 v) {
    return mk3(m.m[0][0] * v.x + m.m[1][0] * v.y + m.m[2][0] * v.z + m.m[3][0],
               m.m[0][1] * v.x + m.m[1][1] * v.y + m.m[2][1] * v.z + m.m[3][1],
               m.m[0][2] * v.x + m.m[1][2] * v.y + m.m[2][2] * v.z + m.m[3][2]);
}
T3D_HD m4 translate(float x, float y, float z) {
    m4 r = ident();
    r.m[3][0] = x; r.m[3][1] = y; r.m[3][2] = z;
    return r;
}
T3D_HD m4 scale_m(float x, float y, float z) {
    m4 r = ident();
    r.m[0][0] = x; r.m[1][1] = y; r.m[2][2] = z;
    return r;
}
T3D_HD f3 row3(const m4& a, int i) { return mk3(a.m[i][0], a.m[i][1], a.m[i][2]); }

// Matrix4.Inverted (matrix.go:255-307): cofactor expansion with the 2x2 minors
// grouped as the reference groups them.
T3D_HD m4 inverted(const m4& M) {
    const float(&m)[4][4] = M.m;
    float A2323 = m[2][2] * m[3][3] - m[2][3] * m[3][2];
    float A1323 = m[2][1] * m[3][3] - m[2][3] * m[3][1];
    float A1223 = m[2][1] * m[3][2] - m[2][2] * m[3][1];
    float A0323 = m[2][0] * m[3][3] - m[2][3] * m[3][0];
    float A0223 = m[2][0] * m[3][2] - m[2][2] * m[3][0];
    float A0123 = m[2][0] * m[3][1] - m[2][1] * m[3][0];
    float A2313 = m[1][2] * m[3][3] - m[1][3] * m[3][2];
    float A1313 = m[1][1] * m[3][3] - m[1][3] * m[3][1];
    float A1213 = m[1][1] * m[3][2] - m[1][2] * m[3][1];
    float A2312 = m[1][2] * m[2][3] - m[1][3] * m[2][2];
    float A1312 = m[1][1] * m[2][3] - m[1][3] * m[2][1];
    float A1212 = m[1][1] * m[2][2] - m[1][2] * m[2][1];
    float A0313 = m[1][0] * m[3][3] - m[1][3] * m[3][0];
    float A0213 = m[1][0] * m[3][2] - m[1][2] * m[3][0];
    float A0312 = m[1][0] * m[2][3] - m[1][3] * m[2][0];
    float A0212 = m[1][0] * m[2][2] - m[1][2] * m[2][0];
    float A0113 = m[1][0] * m[3][1] - m[1][1] * m[3][0];
    float A0112 = m[1][0] * m[2][1] - m[1][1] * m[2][0];
    float det = m[0][0] * (m[1][1] * A2323 - m[1][2] * A1323 + m[1][3] * A1223) -
                m[0][1] * (m[1][0] * A2323 - m[1][2] * A0323 + m[1][3] * A0223) +
                m[0][2] * (m[1][0] * A1323 - m[1][1] * A0323 + m[1][3] * A0123) -
                m[0][3] * (m[1][0] * A1223 - m[1][1] * A0223 + m[1][2] * A0123);
    det = 1.0f / det;
    m4 r;
    r.m[0][0] = det * (m[1][1] * A2323 - m[1][2] * A1323 + m[1][3] * A1223);
    r.m[0][1] = det * -(m[0][1] * A2323 - m[0][2] * A1323 + m[0][3] * A1223);
    r.m[0][2] = det * (m[0][1] * A2313 - m[0][2] * A1313 + m[0][3] * A1213);
    r.m[0][3] = det * -(m[0][1] * A2312 - m[0][2] * A1312 + m[0][3] * A1212);
    r.m[1][0] = det * -(m[1][0] * A2323 - m[1][2] * A0323 + m[1][3] * A0223);
    r.m[1][1] = det * (m[0][0] * A2323 - m[0][2] * A0323 + m[0][3] * A0223);
    r.m[1][2] = det * -(m[0][0] * A2313 - m[0][2] * A0313 + m[0][3] * A0213);
    r.m[1][3] = det * (m[0][0] * A2312 - m[0][2] * A0312 + m[0][3] * A0212);
    r.m[2][0] = det * (m[1][0] * A1323 - m[1][1] * A0323 + m[1][3] * A0123);
    r.m[2][1] = det * -(m[0][0] * A1323 - m[0][1] * A0323 + m[0][3] * A0123);
    r.m[2][2] = det * (m[0][0] * A1313 - m[0][1] * A0313 + m[0][3] * A0113);
    r.m[2][3] = det * -(m[0][0] * A1312 - m[0][1] * A0312 + m[0][3] * A0112);
    r.m[3][0] = det * -(m[1][0] * A1223 - m[1][1] * A0223 + m[1][2] * A0123);
    r.m[3][1] = det * (m[0][0] * A1223 - m[0][1] * A0223 + m[0][2] * A0123);
    r.m[3][2] = det * -(m[0][0] * A1213 - m[0][1] * A0213 + m[0][2] * A0113);
    r.m[3][3] = det * (m[0][0] * A1212 - m[0][1] * A0212 + m[0][2] * A0112);
    return r;
}

// Matrix4.Decompose (matrix.go:181-196). Rotation rows are Vector4.Unit of the
// matrix rows (xyz normalised by the xyz length, w kept, vector.go:1869-1877);
// scale is the row lengths of M * rotation^T; position is row 3.
T3D_HD void decompose(const m4& M, f3& pos, f3& scl, m4& rot) {
    pos = row3(M, 3);
    rot = ident();
#pragma unroll
    for (int i = 0; i < 3; i++) {
        float x = M.m[i][0], y = M.m[i][1], z = M.m[i][2], w = M.m[i][3];
        float l = sqrt_rn(x * x + y * y + z * z);
        if (!(l < 1e-8f || l == 1.0f)) { x = x / l; y = y / l; z = z / l; }
        rot.m[i][0] = x; rot.m[i][1] = y; rot.m[i][2] = z; rot.m[i][3] = w;
    }
    m4 in = mult(M, transposed(rot));
    scl = mk3(mag3(row3(in, 0)), mag3(row3(in, 1)), mag3(row3(in, 2)));
}

// Vector3.Equals (vector.go:415-425): every component within 1e-4.
T3D_HD bool equals3(f3 a, f3 b) {
    return !(fabsf(a.x - b.x) > 1e-4f || fabsf(a.y - b.y) > 1e-4f || fabsf(a.z - b.z) > 1e-4f);
}
// Vector3.Cross (vector.go:164-175)
T3D_HD f3 cross3(f3 a, f3 b) { return mk3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y); }

// NewMatrix4LookAt (matrix.go:788-815)
T3D_HD m4 look_at(f3 from, f3 to, f3 up) {
    if (equals3(from, to)) return ident();
    const f3 z = unit3(sub3(to, from));
    up = unit3(up);
    if (equals3(z, up) || equals3(z, neg3(up))) up = !equals3(up, mk3(1.f, 0.f, 0.f)) ? mk3(1.f, 0.f, 0.f) : mk3(0.f, 0.f, 1.f);
    const f3 x = unit3(cross3(up, z));
    const f3 y = cross3(z, x);
    m4 r = ident();
    r.m[0][0] = x.x; r.m[0][1] = x.y; r.m[0][2] = x.z;
    r.m[1][0] = y.x; r.m[1][1] = y.y; r.m[1][2] = y.z;
    r.m[2][0] = z.x; r.m[2][1] = z.y; r.m[2][2] = z.z;
    return r;
}

// Row i replaced by its Vector4.Unit (xyz over the xyz length, w kept; vector.go:1869-1877).
T3D_HD void unit_row(m4& a, int i) {
    const float x = a.m[i][0], y = a.m[i][1], z = a.m[i][2];
    const float l = sqrt_rn(x * x + y * y + z * z);
    if (l < 1e-8f || l == 1.0f) return;
    a.m[i][0] = x / l; a.m[i][1] = y / l; a.m[i][2] = z / l;
}

// The billboarded model transform of ProcessVertices (model.go:634-688): the
// LookAt from the model's world position to the camera, with locked axes, put
// under the model's rotation and scale, at the model's position.
T3D_HD m4 billboard_base(const m4& M, f3 cam_pos, f3 up, bool lock_x, bool lock_y, bool lock_z) {
    m4 L = look_at(row3(M, 3), cam_pos, up);
    if (lock_x) {
        L.m[0][0] = 1.f; L.m[0][1] = 0.f; L.m[0][2] = 0.f; L.m[0][3] = 0.f;
        L.m[1][0] = 0.f; unit_row(L, 1);
        L.m[2][0] = 0.f; unit_row(L, 2);
    }
    if (lock_y) {
        L.m[1][0] = 0.f; L.m[1][1] = 1.f; L.m[1][2] = 0.f; L.m[1][3] = 0.f;
        L.m[0][1] = 0.f; unit_row(L, 0);
        L.m[2][1] = 0.f; unit_row(L, 2);
    }
    if (lock_z) {
        L.m[2][0] = 0.f; L.m[2][1] = 0.f; L.m[2][2] = 1.f; L.m[2][3] = 0.f;
        L.m[0][2] = 0.f; unit_row(L, 0);
        L.m[1][2] = 0.f; unit_row(L, 1);
    }
    f3 p, s;
    m4 r;
    decompose(M, p, s, r);
    m4 base = mult(mult(r, scale_m(s.x, s.y, s.z)), L);
    base.m[3][0] = p.x; base.m[3][1] = p.y; base.m[3][2] = p.z; base.m[3][3] = 1.f;
    return base;
}

// Node.Transform for a parentless node (node.go:583-585): Scale * Rotation * Translate.
T3D_HD m4 trs(f3 pos, f3 scl, const m4& rot) {
    m4 t = scale_m(scl.x, scl.y, scl.z);
    t = mult(t, rot);
    t = mult(t, translate(pos.x, pos.y, pos.z));
    return t;
}

// The model-space camera position ProcessVertices keys triangles against
// (model.go:629-630), also the PointLight.beginModel transform (light.go:177-186):
// (p, s, r) = Decompose(Inverted(M)); r.MultVec(q) + p * (1/s).
struct InvFrame { f3 p, inv_s; m4 r; };
T3D_HD InvFrame inv_frame(const m4& M) {
    InvFrame f;
    f3 s;
    decompose(inverted(M), f.p, s, f.r);
    f.inv_s = mk3(1.0f / s.x, 1.0f / s.y, 1.0f / s.z);
    return f;
}
T3D_HD f3 to_model_space(const InvFrame& f, f3 q) {
    return add3(mult_vec(f.r, q), hmul3(f.p, f.inv_s));
}

}  // namespace t3d
