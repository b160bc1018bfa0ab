// rsg_adjoint.cuh -- reverse-mode pieces shared by the differentiable rollouts (air and ground).
//
// Each *_bwd function takes the adjoint of a forward function's output and returns (or adds to)
// the adjoints of its inputs, for the forward exactly as written in rsg_math.cuh and in the
// rollout kernels.  Citations are <file>:<line> in the RocketSim tree; B/ is libsrc/bullet3-3.24/.
#pragma once

#include "rsg_consts.cuh"
#include "rsg_math.cuh"

namespace rsg {
namespace adj {

// v -> |v| > m ? v / |v| * m : v  (Car::_FinishPhysicsTick clamps, Car.cpp:176-188)
RSG_HD V3 clamp_len_fwd(V3 v, float m) { return len2(v) > m * m ? normalized(v) * m : v; }
RSG_HD V3 clamp_len_bwd(V3 x, float m, V3 gy) {
    float l2 = len2(x);
    if (!(l2 > m * m)) return gy;
    float l = sqrtf(l2);
    V3 xh = x * (1.f / l);
    return (gy - xh * dot(xh, gy)) * (m / l);
}
// m_from_q (btMatrix3x3::setRotation, B/LinearMath/btMatrix3x3.h:216-246): dM/dq transposed on G
RSG_HD Q m_from_q_bwd(Q q, const M3& G) {
    float x = q.x, y = q.y, z = q.z, w = q.w;
    float d = x * x + y * y + z * z + w * w, s = 2.f / d, ds = -4.f / (d * d);
    float K[3][3] = {{-y * y - z * z, x * y - w * z, z * x + y * w},
                     {x * y + z * w, -x * x - z * z, y * z - w * x},
                     {z * x - w * y, y * z + w * x, -x * x - y * y}};
    float dKx[3][3] = {{0, y, z}, {y, -2 * x, -w}, {z, w, -2 * x}};
    float dKy[3][3] = {{-2 * y, x, w}, {x, 0, z}, {-w, z, -2 * y}};
    float dKz[3][3] = {{-2 * z, -w, x}, {w, -2 * z, y}, {x, y, 0}};
    float dKw[3][3] = {{0, -z, y}, {z, 0, -x}, {-y, x, 0}};
    float gK = 0, gx = 0, gy = 0, gz = 0, gw = 0;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            float g = G.r[i][j];
            gK += g * K[i][j];
            gx += g * dKx[i][j];
            gy += g * dKy[i][j];
            gz += g * dKz[i][j];
            gw += g * dKw[i][j];
        }
    return Q(s * gx + ds * x * gK, s * gy + ds * y * gK, s * gz + ds * z * gK, s * gw + ds * w * gK);
}
// q_from_m (btMatrix3x3::getRotation, btMatrix3x3.h:421-470), the branch the forward took
RSG_HD M3 q_from_m_bwd(const M3& m, Q gq) {
    M3 G;
    for (int i = 0; i < 3; i++) G.r[i] = V3(0, 0, 0);
    float trace = m.r[0].x + m.r[1].y + m.r[2].z;
    float t[4], x;
    int ti = 3, i = 0, j = 1, k = 2;
    if (trace > 0.0f) {
        x = trace + 1.0f;
        t[0] = m.r[2].y - m.r[1].z;
        t[1] = m.r[0].z - m.r[2].x;
        t[2] = m.r[1].x - m.r[0].y;
        t[3] = x;
    } else {
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
        ti = i;
    }
    float sq = sqrtf(x), s = 0.5f / sq, dsdx = -0.25f / (sq * x);
    float g[4] = {gq.x, gq.y, gq.z, gq.w};
    float tg = t[0] * g[0] + t[1] * g[1] + t[2] * g[2] + t[3] * g[3];
    float gt[4] = {s * g[0], s * g[1], s * g[2], s * g[3]};
    float gx = tg * dsdx + gt[ti];
    if (trace > 0.0f) {
        G.r[0].x += gx; G.r[1].y += gx; G.r[2].z += gx;
        G.r[2].y += gt[0]; G.r[1].z -= gt[0];
        G.r[0].z += gt[1]; G.r[2].x -= gt[1];
        G.r[1].x += gt[2]; G.r[0].y -= gt[2];
    } else {
        G.r[i][i] += gx; G.r[j][j] -= gx; G.r[k][k] -= gx;
        G.r[k][j] += gt[3]; G.r[j][k] -= gt[3];
        G.r[j][i] += gt[j]; G.r[i][j] += gt[j];
        G.r[k][i] += gt[k]; G.r[i][k] += gt[k];
    }
    return G;
}
// a (x) b with respect to a and to b
RSG_HD Q qmul_bwd_a(Q b, Q g) {
    return Q(b.w * g.x - b.z * g.y + b.y * g.z - b.x * g.w, b.z * g.x + b.w * g.y - b.x * g.z - b.y * g.w,
             -b.y * g.x + b.x * g.y + b.w * g.z - b.z * g.w, b.x * g.x + b.y * g.y + b.z * g.z + b.w * g.w);
}
RSG_HD Q qmul_bwd_b(Q a, Q g) {
    return Q(a.w * g.x + a.z * g.y - a.y * g.z - a.x * g.w, -a.z * g.x + a.w * g.y + a.x * g.z - a.y * g.w,
             a.y * g.x - a.x * g.y + a.w * g.z - a.z * g.w, a.x * g.x + a.y * g.y + a.z * g.z + a.w * g.w);
}
// v / |v| with respect to v
RSG_HD V3 normalize_bwd(V3 v, V3 g) {
    float l = len(v);
    V3 n = v * (1.f / l);
    return (g - n * dot(n, g)) * (1.f / l);
}
RSG_HD void cross_bwd(V3 a, V3 b, V3 g, V3& ga, V3& gb) {  // c = a x b
    ga += cross(b, g);
    gb += cross(g, a);
}
// LinearPieceCurve::GetOutput (src/Math/Math.cpp:5-35): value and slope in `in`
RSG_HD float curve_slope(const Curve& c, float in) {
    const int n = c.n;
    if (n == 0 || in <= c.x[0]) return 0.f;
    for (int i = 1; i < n; i++)
        if (c.x[i] > in) return (c.y[i] - c.y[i - 1]) / (c.x[i] - c.x[i - 1]);
    return 0.f;
}

// btTransformUtil::integrateTransform (B/LinearMath/btTransformUtil.h:37-80) of the position and
// basis, then the velocity clamps of Car::_FinishPhysicsTick, with the intermediates the reverse
// pass needs.
struct IntTape {
    V3 w1u, v1u;
    Q q0, dq, qm, qn;
    bool ang_clamped, rot_set;
};
RSG_HD void integrate_car(V3& p, M3& B, V3& v, V3& w, V3 v1u, V3 w1u, float dt, IntTape* t) {
    V3 p1 = p + v1u * dt;
    const float ANGULAR_MOTION_THRESHOLD = 0.5f * HALF_PI_F;
    float a2 = len2(w1u);
    float ang = 0;
    if (a2 > SIMD_EPS) ang = sqrtf(a2);
    bool ang_clamped = false;
    if (ang * dt > ANGULAR_MOTION_THRESHOLD) { ang = ANGULAR_MOTION_THRESHOLD / dt; ang_clamped = true; }
    V3 axis;
    if (ang < 0.001f) axis = w1u * (0.5f * dt - (dt * dt * dt) * (0.020833333333f) * ang * ang);
    else axis = w1u * (sinf(0.5f * ang * dt) / ang);
    Q dorn(axis.x, axis.y, axis.z, cosf(ang * dt * 0.5f));
    Q orn0 = q_from_m(B);
    Q qm = q_mul(dorn, orn0);
    Q pred = q_safe_normalize(qm);
    bool rot_set = q_len2(pred) > SIMD_EPS;
    if (t) {
        t->w1u = w1u; t->v1u = v1u;
        t->q0 = orn0; t->dq = dorn; t->qm = qm; t->qn = pred;
        t->ang_clamped = ang_clamped;
        t->rot_set = rot_set;
    }
    if (rot_set) B = m_from_q(pred);
    p = p1;
    v = clamp_len_fwd(v1u, RL::CAR_MAX_SPEED * RL::UU_TO_BT);
    w = clamp_len_fwd(w1u, RL::CAR_MAX_ANG_SPEED);
}
// Reverse of integrate_car: in gp, gB, gv, gw the adjoints after; out: gp (before), gB0 (adjoint of
// the basis before, through the orientation update only), gv1u, gw1u.
RSG_HD void integrate_car_bwd(const M3& B0, const IntTape& t, float dt, V3& gp, const M3& gB, V3 gv, V3 gw, M3& gB0,
                              V3& gv1u, V3& gw1u) {
    gv1u = clamp_len_bwd(t.v1u, RL::CAR_MAX_SPEED * RL::UU_TO_BT, gv) + gp * dt;
    gw1u = clamp_len_bwd(t.w1u, RL::CAR_MAX_ANG_SPEED, gw);
    if (!t.rot_set) {
        gB0 = gB;
        return;
    }
    Q gqn = m_from_q_bwd(t.qn, gB);
    float lm = sqrtf(q_len2(t.qm));
    float pn = t.qn.x * gqn.x + t.qn.y * gqn.y + t.qn.z * gqn.z + t.qn.w * gqn.w;
    Q gqm((gqn.x - t.qn.x * pn) / lm, (gqn.y - t.qn.y * pn) / lm, (gqn.z - t.qn.z * pn) / lm,
          (gqn.w - t.qn.w * pn) / lm);
    Q gq0 = qmul_bwd_b(t.dq, gqm);
    Q gdq = qmul_bwd_a(t.q0, gqm);
    {  // dq(w) = (w * s(|w|), cos(|w| dt / 2))
        V3 w = t.w1u;
        float a2 = len2(w);
        float ang = a2 > SIMD_EPS ? sqrtf(a2) : 0.f;
        if (t.ang_clamped) ang = 0.5f * HALF_PI_F / dt;
        V3 gax(gdq.x, gdq.y, gdq.z);
        float s, dsda;
        if (ang < 0.001f) {
            s = 0.5f * dt - (dt * dt * dt) * 0.020833333333f * ang * ang;
            dsda = -2.f * (dt * dt * dt) * 0.020833333333f * ang;
        } else {
            float h = 0.5f * ang * dt;
            s = sinf(h) / ang;
            dsda = (0.5f * dt * cosf(h) * ang - sinf(h)) / (ang * ang);
        }
        gw1u += gax * s;
        if (ang > 0.f && !t.ang_clamped) {
            V3 wh = w * (1.f / ang);
            gw1u += wh * (dsda * dot(w, gax) - gdq.w * sinf(0.5f * ang * dt) * 0.5f * dt);
        }
    }
    gB0 = q_from_m_bwd(B0, gq0);
}

}  // namespace adj
}  // namespace rsg
