// rsg_math.cuh -- float 3D math shared by the device tick and the host-side
// mesh builder.
//
// Operation order follows Bullet 3.24 as compiled for x86-64 by the reference
// (scalar btVector3/btMatrix3x3 formulas; btQuaternion and getRotation/
// setRotation in their SSE form).  The library is compiled with -fmad=false so
// no multiply-add is fused, which keeps rounding identical to that build except
// for btVector3::normalize, where the reference uses a hardware rsqrt estimate
// and this code divides exactly.
#pragma once
#include <cfloat>
#include <cmath>
#include <cstdint>

#if defined(__CUDACC__)
#define RSG_HD __host__ __device__ __forceinline__
#else
#define RSG_HD inline
#endif

namespace rsg {

constexpr float BT_LARGE = 1e18f;
constexpr float SIMD_EPS = FLT_EPSILON;
constexpr float PI_F = 3.1415926535897932384626433832795029f;
constexpr float HALF_PI_F = PI_F * 0.5f;
constexpr float TWO_PI_F = 6.283185307179586232f;
constexpr float SQRT12 = 0.7071067811865475244008443621048490f;

struct V3 {
    float x, y, z;
    RSG_HD V3() : x(0), y(0), z(0) {}
    RSG_HD constexpr V3(float a, float b, float c) : x(a), y(b), z(c) {}
    RSG_HD float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    RSG_HD float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

RSG_HD V3 operator+(V3 a, V3 b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
RSG_HD V3 operator-(V3 a, V3 b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
RSG_HD V3 operator-(V3 a) { return V3(-a.x, -a.y, -a.z); }
RSG_HD V3 operator*(V3 a, float s) { return V3(a.x * s, a.y * s, a.z * s); }
RSG_HD V3 operator*(float s, V3 a) { return V3(a.x * s, a.y * s, a.z * s); }
RSG_HD V3 operator*(V3 a, V3 b) { return V3(a.x * b.x, a.y * b.y, a.z * b.z); }
RSG_HD V3 operator/(V3 a, float s) { float r = 1.0f / s; return a * r; }
RSG_HD V3& operator+=(V3& a, V3 b) { a = a + b; return a; }
RSG_HD V3& operator-=(V3& a, V3 b) { a = a - b; return a; }
RSG_HD V3& operator*=(V3& a, float s) { a = a * s; return a; }
RSG_HD bool operator==(V3 a, V3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
RSG_HD bool operator!=(V3 a, V3 b) { return !(a == b); }

RSG_HD float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
RSG_HD V3 cross(V3 a, V3 b) { return V3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
RSG_HD float len2(V3 a) { return dot(a, a); }
RSG_HD float len(V3 a) { return sqrtf(len2(a)); }
RSG_HD V3 normalized(V3 a) { return a / len(a); }
RSG_HD V3 safe_normalized(V3 a) {
    float l2 = len2(a);
    if (l2 >= SIMD_EPS * SIMD_EPS) return a / sqrtf(l2);
    return V3(1, 0, 0);
}
RSG_HD bool is_zero(V3 a) { return a.x == 0 && a.y == 0 && a.z == 0; }
RSG_HD bool fuzzy_zero(V3 a) { return len2(a) < SIMD_EPS * SIMD_EPS; }
RSG_HD V3 vmin(V3 a, V3 b) { return V3(b.x < a.x ? b.x : a.x, b.y < a.y ? b.y : a.y, b.z < a.z ? b.z : a.z); }
RSG_HD V3 vmax(V3 a, V3 b) { return V3(a.x < b.x ? b.x : a.x, a.y < b.y ? b.y : a.y, a.z < b.z ? b.z : a.z); }
RSG_HD V3 lerp(V3 a, V3 b, float t) {
    float s = 1.0f - t;
    return V3(s * a.x + t * b.x, s * a.y + t * b.y, s * a.z + t * b.z);
}
RSG_HD int max_axis(V3 a) { return a.x < a.y ? (a.y < a.z ? 2 : 1) : (a.x < a.z ? 2 : 0); }
RSG_HD int closest_axis4(float a, float b, float c, float d) {
    a = fabsf(a); b = fabsf(b); c = fabsf(c); d = fabsf(d);
    int mi = -1;
    float mv = -BT_LARGE;
    if (a > mv) { mi = 0; mv = a; }
    if (b > mv) { mi = 1; mv = b; }
    if (c > mv) { mi = 2; mv = c; }
    if (d > mv) { mi = 3; }
    return mi;
}
// RocketSim Vec semantics (true division, zero below eps^2)
RSG_HD float rs_len(V3 v) { float l2 = v.x * v.x + v.y * v.y + v.z * v.z; return l2 > 0 ? sqrtf(l2) : 0.f; }
RSG_HD V3 rs_normalized(V3 v) {
    float l = rs_len(v);
    if (l > FLT_EPSILON * FLT_EPSILON) return V3(v.x / l, v.y / l, v.z / l);
    return V3(0, 0, 0);
}
RSG_HD float simd_dot(V3 a, V3 b) { return a.x * b.x + (a.y * b.y + a.z * b.z); }

struct Q {
    float x, y, z, w;
    RSG_HD Q() : x(0), y(0), z(0), w(1) {}
    RSG_HD Q(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
};
RSG_HD Q q_axis_angle(V3 axis, float angle) {
    float d = len(axis);
    float s = sinf(angle * 0.5f) / d;
    return Q(axis.x * s, axis.y * s, axis.z * s, cosf(angle * 0.5f));
}
RSG_HD Q q_mul(Q a, Q b) {
    float a1x = a.x * b.w, a1y = a.y * b.w, a1z = a.z * b.w, a1w = a.x * b.x;
    float a2x = a.y * b.z, a2y = a.z * b.x, a2z = a.x * b.y, a2w = a.y * b.y;
    float b1x = a.z * b.y, b1y = a.x * b.z, b1z = a.y * b.x, b1w = a.z * b.z;
    float a0x = a.w * b.x, a0y = a.w * b.y, a0z = a.w * b.z, a0w = a.w * b.w;
    a1x = a1x + a2x; a1y = a1y + a2y; a1z = a1z + a2z; a1w = a1w + a2w;
    a0x = a0x - b1x; a0y = a0y - b1y; a0z = a0z - b1z; a0w = a0w - b1w;
    a1w = -a1w;
    return Q(a0x + a1x, a0y + a1y, a0z + a1z, a0w + a1w);
}
RSG_HD float q_len2(Q q) { return (q.x * q.x + q.z * q.z) + (q.y * q.y + q.w * q.w); }
RSG_HD Q q_scale(Q q, float s) { return Q(q.x * s, q.y * s, q.z * s, q.w * s); }
RSG_HD Q q_safe_normalize(Q q) {
    float l2 = q_len2(q);
    if (l2 > SIMD_EPS) return q_scale(q, 1.0f / sqrtf(l2));
    return q;
}
RSG_HD Q q_inverse(Q q) { return Q(-q.x, -q.y, -q.z, q.w); }
RSG_HD V3 q_rotate(Q r, V3 v) {
    Q q((r.w * v.x + r.y * v.z) - r.z * v.y, (r.w * v.y + r.z * v.x) - r.x * v.z, (r.w * v.z + r.x * v.y) - r.y * v.x,
        -(r.x * v.x + r.y * v.y) - r.z * v.z);
    Q o = q_mul(q, q_inverse(r));
    return V3(o.x, o.y, o.z);
}

struct M3 {
    V3 r[3];
    RSG_HD M3() { r[0] = V3(1, 0, 0); r[1] = V3(0, 1, 0); r[2] = V3(0, 0, 1); }
    RSG_HD M3(float a, float b, float c, float d, float e, float f, float g, float h, float i) {
        r[0] = V3(a, b, c); r[1] = V3(d, e, f); r[2] = V3(g, h, i);
    }
    RSG_HD V3 col(int i) const { return V3(r[0][i], r[1][i], r[2][i]); }
};
RSG_HD V3 operator*(const M3& m, V3 v) { return V3(dot(m.r[0], v), dot(m.r[1], v), dot(m.r[2], v)); }
RSG_HD V3 operator*(V3 v, const M3& m) {
    return V3(m.r[0].x * v.x + m.r[1].x * v.y + m.r[2].x * v.z, m.r[0].y * v.x + m.r[1].y * v.y + m.r[2].y * v.z,
              m.r[0].z * v.x + m.r[1].z * v.y + m.r[2].z * v.z);
}
RSG_HD M3 operator*(const M3& a, const M3& b) {
    M3 o;
    for (int i = 0; i < 3; i++) {
        V3 row = a.r[i];
        o.r[i] = V3(b.r[0].x * row.x + b.r[1].x * row.y + b.r[2].x * row.z,
                    b.r[0].y * row.x + b.r[1].y * row.y + b.r[2].y * row.z,
                    b.r[0].z * row.x + b.r[1].z * row.y + b.r[2].z * row.z);
    }
    return o;
}
RSG_HD M3 transpose(const M3& m) {
    return M3(m.r[0].x, m.r[1].x, m.r[2].x, m.r[0].y, m.r[1].y, m.r[2].y, m.r[0].z, m.r[1].z, m.r[2].z);
}
RSG_HD M3 transpose_times(const M3& a, const M3& b) {
    M3 o;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            o.r[i][j] = a.r[0][i] * b.r[0][j] + a.r[1][i] * b.r[1][j] + a.r[2][i] * b.r[2][j];
    return o;
}
RSG_HD M3 scaled(const M3& m, V3 s) {
    return M3(m.r[0].x * s.x, m.r[0].y * s.y, m.r[0].z * s.z, m.r[1].x * s.x, m.r[1].y * s.y, m.r[1].z * s.z,
              m.r[2].x * s.x, m.r[2].y * s.y, m.r[2].z * s.z);
}
RSG_HD M3 absolute(const M3& m) {
    M3 o;
    for (int i = 0; i < 3; i++) o.r[i] = V3(fabsf(m.r[i].x), fabsf(m.r[i].y), fabsf(m.r[i].z));
    return o;
}
RSG_HD float cofac(const M3& m, int r1, int c1, int r2, int c2) {
    return m.r[r1][c1] * m.r[r2][c2] - m.r[r1][c2] * m.r[r2][c1];
}
RSG_HD M3 inverse(const M3& m) {
    V3 co(cofac(m, 1, 1, 2, 2), cofac(m, 1, 2, 2, 0), cofac(m, 1, 0, 2, 1));
    float det = dot(m.r[0], co);
    float s = 1.0f / det;
    return M3(co.x * s, cofac(m, 0, 2, 2, 1) * s, cofac(m, 0, 1, 1, 2) * s, co.y * s, cofac(m, 0, 0, 2, 2) * s,
              cofac(m, 0, 2, 1, 0) * s, co.z * s, cofac(m, 0, 1, 2, 0) * s, cofac(m, 0, 0, 1, 1) * s);
}
RSG_HD M3 m_from_q(Q q) {
    float d = q_len2(q);
    float s = 2.0f / d;
    float x = q.x, y = q.y, z = q.z, w = q.w;
    float r0x = (-y * y + -z * z), r0y = (x * y + -w * z), r0z = (z * x + y * w);
    float r1x = (x * y + z * w), r1y = (-x * x + -z * z), r1z = (y * z + -w * x);
    float r2x = (z * x + -w * y), r2y = (y * z + w * x), r2z = (-x * x + -y * y);
    return M3(r0x * s + 1.0f, r0y * s + 0.0f, r0z * s + 0.0f, r1x * s + 0.0f, r1y * s + 1.0f, r1z * s + 0.0f,
              r2x * s + 0.0f, r2y * s + 0.0f, r2z * s + 1.0f);
}
RSG_HD Q q_from_m(const M3& m) {
    float trace = m.r[0].x + m.r[1].y + m.r[2].z;
    float t[4], x;
    if (trace > 0.0f) {
        x = trace + 1.0f;
        t[0] = m.r[2].y - m.r[1].z;
        t[1] = m.r[0].z - m.r[2].x;
        t[2] = m.r[1].x - m.r[0].y;
        t[3] = x;
    } else {
        int i, j, k;
        if (m.r[0].x < m.r[1].y) {
            if (m.r[1].y < m.r[2].z) { i = 2; j = 0; k = 1; } else { i = 1; j = 2; k = 0; }
        } else {
            if (m.r[0].x < m.r[2].z) { i = 2; j = 0; k = 1; } else { i = 0; j = 1; k = 2; }
        }
        x = m.r[i][i] - m.r[j][j] - m.r[k][k] + 1.0f;
        t[3] = (m.r[k][j] - m.r[j][k]);
        t[j] = (m.r[j][i] + m.r[i][j]);
        t[k] = (m.r[k][i] + m.r[i][k]);
        t[i] = x;
    }
    float s = sqrtf(x);
    s = 0.5f / s;
    return Q(t[0] * s, t[1] * s, t[2] * s, t[3] * s);
}
RSG_HD M3 m_euler_ypr(float yaw, float pitch, float roll) {
    float ci = cosf(roll), cj = cosf(pitch), ch = cosf(yaw);
    float si = sinf(roll), sj = sinf(pitch), sh = sinf(yaw);
    float cc = ci * ch, cs = ci * sh, sc = si * ch, ss = si * sh;
    return M3(cj * ch, sj * sc - cs, sj * cc + ss, cj * sh, sj * ss + cc, sj * cs - sc, -sj, cj * si, cj * ci);
}

struct Xf {
    M3 b;
    V3 o;
};
RSG_HD V3 xf_apply(const Xf& t, V3 v) {
    return V3(dot(t.b.r[0], v) + t.o.x, dot(t.b.r[1], v) + t.o.y, dot(t.b.r[2], v) + t.o.z);
}
RSG_HD V3 xf_inv_apply(const Xf& t, V3 v) { V3 d = v - t.o; return transpose(t.b) * d; }
RSG_HD Xf xf_inverse(const Xf& t) { M3 inv = transpose(t.b); Xf r; r.b = inv; r.o = inv * (-t.o); return r; }
RSG_HD Xf xf_mul(const Xf& a, const Xf& b) { Xf r; r.b = a.b * b.b; r.o = xf_apply(a, b.o); return r; }
RSG_HD Xf xf_identity() { Xf t; t.o = V3(0, 0, 0); return t; }

RSG_HD void transform_aabb(V3 he, float margin, const Xf& t, V3& mn, V3& mx) {
    V3 hm = he + V3(margin, margin, margin);
    M3 ab = absolute(t.b);
    V3 ext(dot(ab.r[0], hm), dot(ab.r[1], hm), dot(ab.r[2], hm));
    mn = t.o - ext;
    mx = t.o + ext;
}
RSG_HD bool aabb_overlap(V3 amin, V3 amax, V3 bmin, V3 bmax) {
    bool o = true;
    o = (amin.x > bmax.x || amax.x < bmin.x) ? false : o;
    o = (amin.z > bmax.z || amax.z < bmin.z) ? false : o;
    o = (amin.y > bmax.y || amax.y < bmin.y) ? false : o;
    return o;
}
RSG_HD void plane_space(V3 n, V3& p, V3& q) {
    if (fabsf(n.z) > SQRT12) {
        float a = n.y * n.y + n.z * n.z;
        float k = 1.0f / sqrtf(a);
        p = V3(0, -n.z * k, n.y * k);
        q = V3(a * k, -n.x * p.z, n.x * p.y);
    } else {
        float a = n.x * n.x + n.y * n.y;
        float k = 1.0f / sqrtf(a);
        p = V3(-n.y * k, n.x * k, 0);
        q = V3(-n.z * p.y, n.z * p.x, a * k);
    }
}

}  // namespace rsg
