// rsg_air.cu -- contact-free air-phase rollouts of one car and the ball, and their adjoint.
//
// The forward tick is the arena tick restricted to a car with no wheel, body or world contact
// and a ball without contacts: Car::_UpdateAirTorque (src/Sim/Car/Car.cpp:584-669), the boost
// force of Car::_UpdateBoost (Car.cpp:486-533) with the boost input relaxed to [0, 1], gravity,
// the solver's external-impulse write-back (B/BulletDynamics/ConstraintSolver/btSequentialImpulseConstraintSolver.cpp:1878-1904),
// btTransformUtil::integrateTransform (B/LinearMath/btTransformUtil.h:37-80), the clamps of
// Car::_FinishPhysicsTick (Car.cpp:165-193) and, for the ball, btRigidBody::applyDamping
// (B/BulletDynamics/Dynamics/btRigidBody.cpp:153-162) and Ball::_FinishPhysicsTick (Ball.cpp:117-143).  It uses the same
// operations in the same order as rsg_tick_kernel, so for boost inputs of exactly 0 or 1 it
// reproduces the full tick of an airborne car.
//
// The adjoint runs in two launches.  The forward kernel stores the state every `ckpt_every`
// ticks; the tape kernel recomputes every segment from its checkpoint at once (one thread per
// instance and segment) and writes, per tick, what the reverse pass needs (the tick's
// linearisation point) to a caller-provided workspace laid out [tick][word][instance]; the sweep
// kernel (one thread per instance) then walks the ticks backwards through that tape, which it
// prefetches a tick ahead.  The recompute is parallel in time and the serial chain holds only
// the reverse tick.  Citations are <file>:<line> in the RocketSim tree; B/ is
// libsrc/bullet3-3.24/.  The torque path uses
// I_world_inv * inverse(I_world_inv) = identity, so the air-control torque reaches the angular
// velocity as (torque - damping) * CAR_TORQUE_SCALE * dt.
#include <cuda_runtime.h>

#include "../../include/rocketsim_gb300.h"
#include "rsg_consts.cuh"
#include "rsg_kernels.h"
#include "rsg_math.cuh"

namespace rsg {
namespace air {

#define RSG_AD RSG_HD

constexpr int STATE = 24;  // per instance: car pos(3) vel(3) angvel(3) basis rows(9), ball pos(3) vel(3)
constexpr int TAPE_WORDS = 38;  // per instance and tick, see put_tape

struct Cfg {
    V3 iinv;   // car inverse inertia (local)
    float dt;
    float car_damp, ball_damp;  // btRigidBody::applyDamping factors, filled on the device
};

// The damping factors are the same powf calls the arena tick makes every tick; computed once
// per thread they give the same values.
RSG_AD void fill_damping(Cfg& k) {
    k.car_damp = powf(1.f - 0.f, k.dt);
    k.ball_damp = powf(1.f - RL::BALL_DRAG, k.dt);
}

struct St {
    V3 p, v, w;
    M3 B;
    V3 bp, bv;
};

RSG_AD St load_state(const float* s) {
    St x;
    x.p = V3(s[0], s[1], s[2]);
    x.v = V3(s[3], s[4], s[5]);
    x.w = V3(s[6], s[7], s[8]);
    for (int r = 0; r < 3; r++) x.B.r[r] = V3(s[9 + 3 * r], s[10 + 3 * r], s[11 + 3 * r]);
    x.bp = V3(s[18], s[19], s[20]);
    x.bv = V3(s[21], s[22], s[23]);
    return x;
}
RSG_AD void store_state(float* s, const St& x) {
    s[0] = x.p.x; s[1] = x.p.y; s[2] = x.p.z;
    s[3] = x.v.x; s[4] = x.v.y; s[5] = x.v.z;
    s[6] = x.w.x; s[7] = x.w.y; s[8] = x.w.z;
    for (int r = 0; r < 3; r++) {
        s[9 + 3 * r] = x.B.r[r].x;
        s[10 + 3 * r] = x.B.r[r].y;
        s[11 + 3 * r] = x.B.r[r].z;
    }
    s[18] = x.bp.x; s[19] = x.bp.y; s[20] = x.bp.z;
    s[21] = x.bv.x; s[22] = x.bv.y; s[23] = x.bv.z;
}

RSG_AD float clampf(float v, float lo, float hi) { float m = v > lo ? v : lo; return m < hi ? m : hi; }
RSG_AD V3 clamp_len(V3 v, float m) { return len2(v) > m * m ? normalized(v) * m : v; }

// Intermediates of one car tick that the adjoint needs
struct Tape {
    float cp, cy, cr, boost;       // clamped inputs (boost in [0, 1])
    V3 w1u, v1u;                   // velocities before the clamps
    bool ang_clamped;              // integrateTransform's angular motion threshold was hit
    Q q0, dq, qm, qn;              // orientation integration
};

// One tick of the car (and the ball).  Mirrors the air path of rsg_tick_kernel.
RSG_AD void car_tick(St& x, float4 u, const Cfg& k, Tape* tp) {
    const float dt = k.dt;
    const float pitch = clampf(u.x, -1, 1), yaw = clampf(u.y, -1, 1), roll = clampf(u.z, -1, 1);
    const float boost = clampf(u.w, 0, 1);
    const M3 R = x.B;  // CarState::rotMat == basis after the last post-tick
    M3 iw = scaled(x.B, k.iinv) * transpose(x.B);  // btRigidBody::updateInertiaTensor
    // Car::_UpdateAirTorque, not flipping, pitch scale 1
    V3 pitch_right = -R.col(1), yaw_up = R.col(2), roll_fwd = -R.col(0);
    V3 torque(0, 0, 0);
    if (pitch || yaw || roll)
        torque = (pitch * pitch_right * 1.f * RL::AIR_TORQUE_X) + (yaw * yaw_up * RL::AIR_TORQUE_Y) +
                 (roll * roll_fwd * RL::AIR_TORQUE_Z);
    float dp = dot(pitch_right, x.w) * RL::AIR_DAMP_X * (1 - fabsf(pitch * 1.f));
    float dy = dot(yaw_up, x.w) * RL::AIR_DAMP_Y * (1 - fabsf(yaw));
    float dr = dot(roll_fwd, x.w) * RL::AIR_DAMP_Z;
    V3 damping = (yaw_up * dy) + (pitch_right * dp) + (roll_fwd * dr);
    V3 total_torque = V3(0, 0, 0) + inverse(iw) * (torque - damping) * RL::CAR_TORQUE_SCALE;
    // Car::_UpdateBoost in the air, boost input relaxed to [0, 1]
    const float accel = RL::BOOST_ACCEL_AIR * RL::UU_TO_BT;
    V3 total_force = V3(0, 0, 0) + (boost * accel) * R.col(0) * RL::CAR_MASS_BT;
    // applyGravity, predictUnconstraintMotion (no car damping), solver write-back
    const float inv_mass = 1.f / RL::CAR_MASS_BT;
    total_force += V3(0, 0, RL::GRAVITY_Z * RL::UU_TO_BT) * (1.f / inv_mass);
    V3 v = x.v * k.car_damp, w = x.w * k.car_damp;
    V3 ext_f = total_force * inv_mass * dt;
    V3 ext_t = total_torque * iw * dt;
    v = (v + V3(0, 0, 0)) + ext_f;
    w = (w + V3(0, 0, 0)) + ext_t;
    // integrateTransform
    V3 p1 = x.p + v * dt;
    const float ANGULAR_MOTION_THRESHOLD = 0.5f * HALF_PI_F;
    float a2 = len2(w);
    float ang = 0;
    if (a2 > SIMD_EPS) ang = sqrtf(a2);
    bool ang_clamped = false;
    if (ang * dt > ANGULAR_MOTION_THRESHOLD) { ang = ANGULAR_MOTION_THRESHOLD / dt; ang_clamped = true; }
    V3 axis;
    if (ang < 0.001f) axis = w * (0.5f * dt - (dt * dt * dt) * (0.020833333333f) * ang * ang);
    else axis = w * (sinf(0.5f * ang * dt) / ang);
    Q dorn(axis.x, axis.y, axis.z, cosf(ang * dt * 0.5f));
    Q orn0 = q_from_m(x.B);
    Q qm = q_mul(dorn, orn0);
    Q pred = q_safe_normalize(qm);
    if (tp) {
        tp->cp = pitch; tp->cy = yaw; tp->cr = roll; tp->boost = boost;
        tp->w1u = w; tp->v1u = v;
        tp->ang_clamped = ang_clamped;
        tp->q0 = orn0; tp->dq = dorn; tp->qm = qm; tp->qn = pred;
    }
    if (q_len2(pred) > SIMD_EPS) x.B = m_from_q(pred);
    x.p = p1;
    // Car::_FinishPhysicsTick clamps
    x.v = clamp_len(v, RL::CAR_MAX_SPEED * RL::UU_TO_BT);
    x.w = clamp_len(w, RL::CAR_MAX_ANG_SPEED);
}

// One tick of the ball; returns its velocity before the speed clamp (what the adjoint needs).
RSG_AD V3 ball_tick(St& x, const Cfg& k) {
    const float dt = k.dt;
    const float mass = RL::BALL_MASS_BT, inv_mass = 1.f / mass;
    V3 force = V3(0, 0, 0) + V3(0, 0, RL::GRAVITY_Z * RL::UU_TO_BT) * (1.f / inv_mass);
    V3 v = x.bv * k.ball_damp;
    v = (v + V3(0, 0, 0)) + force * inv_mass * dt;
    x.bp = x.bp + v * dt;
    x.bv = clamp_len(v, RL::BALL_MAX_SPEED * RL::UU_TO_BT);
    return v;
}

// ---------------------------------------------------------------- adjoint pieces
RSG_AD V3 clamp_len_bwd(V3 x, float m, V3 gy) {
    float l2 = len2(x);
    if (!(l2 > m * m)) return gy;
    float l = sqrtf(l2);
    V3 xh = x * (1.f / l);
    return (gy - xh * dot(xh, gy)) * (m / l);
}
// d(m_from_q(q)) / dq, transposed, applied to the matrix adjoint G
RSG_AD Q m_from_q_bwd(Q q, const M3& G) {
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
// d(q_from_m(m)) / dm, transposed (same branch as the forward)
RSG_AD M3 q_from_m_bwd(const M3& m, Q gq) {
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
// adjoints of a (x) b with respect to a and b
RSG_AD Q qmul_bwd_a(Q b, Q g) {
    return Q(b.w * g.x - b.z * g.y + b.y * g.z - b.x * g.w, b.z * g.x + b.w * g.y - b.x * g.z - b.y * g.w,
             -b.y * g.x + b.x * g.y + b.w * g.z - b.z * g.w, b.x * g.x + b.y * g.y + b.z * g.z + b.w * g.w);
}
RSG_AD Q qmul_bwd_b(Q a, Q g) {
    return Q(a.w * g.x + a.z * g.y - a.y * g.z - a.x * g.w, -a.z * g.x + a.w * g.y + a.x * g.z - a.y * g.w,
             a.y * g.x - a.x * g.y + a.w * g.z - a.z * g.w, a.x * g.x + a.y * g.y + a.z * g.z + a.w * g.w);
}

struct Adj {
    V3 p, v, w;
    M3 B;
    V3 bp, bv;
};

// Reverse of ball_tick given the ball velocity before the clamp
RSG_AD void ball_tick_bwd(V3 v1u, Adj& g, const Cfg& k) {
    V3 gv1u = clamp_len_bwd(v1u, RL::BALL_MAX_SPEED * RL::UU_TO_BT, g.bv) + g.bp * k.dt;
    g.bv = gv1u * k.ball_damp;
}

// Reverse of car_tick: `g` holds the adjoint of the state after the tick and becomes the adjoint
// of the state before it; returns the adjoint of the four inputs `u`.  Like torch.clamp, an input
// on the boundary of its range passes its gradient; one outside it gets none.
RSG_AD float4 car_tick_bwd(const St& x0, float4 u, const Tape& t, Adj& g, const Cfg& k) {
    const float dt = k.dt;
    V3 gv1u = clamp_len_bwd(t.v1u, RL::CAR_MAX_SPEED * RL::UU_TO_BT, g.v);
    V3 gw1u = clamp_len_bwd(t.w1u, RL::CAR_MAX_ANG_SPEED, g.w);
    V3 gp0 = g.p;
    gv1u += g.p * dt;
    // orientation: B1 = M(qn), qn = qm / |qm|, qm = dq (x) q0, q0 = q_from_m(B0)
    Q gqn = m_from_q_bwd(t.qn, g.B);
    float lm = sqrtf(q_len2(t.qm));
    float pn = t.qn.x * gqn.x + t.qn.y * gqn.y + t.qn.z * gqn.z + t.qn.w * gqn.w;
    Q gqm((gqn.x - t.qn.x * pn) / lm, (gqn.y - t.qn.y * pn) / lm, (gqn.z - t.qn.z * pn) / lm, (gqn.w - t.qn.w * pn) / lm);
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
    M3 gB0 = q_from_m_bwd(x0.B, gq0);
    // velocities before the step (the damping factor is exactly 1 for the car)
    g.v = gv1u * k.car_damp;
    V3 X = gw1u * (RL::CAR_TORQUE_SCALE * dt);  // adjoint of (torque - damping)
    const M3& R = x0.B;
    V3 pr = -R.col(1), yu = R.col(2), rf = -R.col(0), f = R.col(0);
    // boost force: (boost * accel) * f  (mass * inv_mass == 1)
    const float accel = RL::BOOST_ACCEL_AIR * RL::UU_TO_BT;
    float gboost = accel * dt * dot(f, gv1u);
    V3 gf = gv1u * (t.boost * accel * dt);
    // torque = pitch 130 pr + yaw 95 yu + roll 400 rf ; damping = yu dy + pr dp + rf dr
    float cpd = RL::AIR_DAMP_X * (1 - fabsf(t.cp)), cyd = RL::AIR_DAMP_Y * (1 - fabsf(t.cy)), crd = RL::AIR_DAMP_Z;
    float wp = dot(pr, x0.w), wy = dot(yu, x0.w), wr = dot(rf, x0.w);
    V3 gd = -X;
    float gdp = dot(pr, gd), gdy = dot(yu, gd), gdr = dot(rf, gd);
    float gpitch = RL::AIR_TORQUE_X * dot(pr, X) + gdp * wp * RL::AIR_DAMP_X * (t.cp > 0 ? -1.f : (t.cp < 0 ? 1.f : 0.f));
    float gyaw = RL::AIR_TORQUE_Y * dot(yu, X) + gdy * wy * RL::AIR_DAMP_Y * (t.cy > 0 ? -1.f : (t.cy < 0 ? 1.f : 0.f));
    float groll = RL::AIR_TORQUE_Z * dot(rf, X);
    V3 gpr = X * (t.cp * RL::AIR_TORQUE_X) + gd * (wp * cpd) + x0.w * (gdp * cpd);
    V3 gyu = X * (t.cy * RL::AIR_TORQUE_Y) + gd * (wy * cyd) + x0.w * (gdy * cyd);
    V3 grf = X * (t.cr * RL::AIR_TORQUE_Z) + gd * (wr * crd) + x0.w * (gdr * crd);
    g.w = gw1u * k.car_damp + pr * (gdp * cpd) + yu * (gdy * cyd) + rf * (gdr * crd);
    V3 gc0 = gf - grf, gc1 = -gpr, gc2 = gyu;
    for (int r = 0; r < 3; r++) {
        gB0.r[r].x += gc0[r];
        gB0.r[r].y += gc1[r];
        gB0.r[r].z += gc2[r];
    }
    g.B = gB0;
    g.p = gp0;
    // inputs outside the clamp ranges get no gradient
    float4 gu;
    gu.x = (u.x >= -1.f && u.x <= 1.f) ? gpitch : 0.f;
    gu.y = (u.y >= -1.f && u.y <= 1.f) ? gyaw : 0.f;
    gu.z = (u.z >= -1.f && u.z <= 1.f) ? groll : 0.f;
    gu.w = (u.w >= 0.f && u.w <= 1.f) ? gboost : 0.f;
    return gu;
}

// Tape of one tick of one instance, word w at tape[(t * TAPE_WORDS + w) * n + i]: the car basis
// and angular velocity before the tick, its velocities before the clamps, the four orientation
// quaternions of integrateTransform, the ball velocity before its clamp and the angular-clamp flag.
struct TapeRef {
    float* base;
    size_t n;
    RSG_AD float& operator[](int w) const { return base[(size_t)w * n]; }
};
RSG_AD void put_v3(const TapeRef& r, int w, V3 v) { r[w] = v.x; r[w + 1] = v.y; r[w + 2] = v.z; }
RSG_AD void put_q(const TapeRef& r, int w, Q q) { r[w] = q.x; r[w + 1] = q.y; r[w + 2] = q.z; r[w + 3] = q.w; }
RSG_AD V3 get_v3(const float* v, int w) { return V3(v[w], v[w + 1], v[w + 2]); }
RSG_AD Q get_q(const float* v, int w) { return Q(v[w], v[w + 1], v[w + 2], v[w + 3]); }

RSG_AD void put_tape(const TapeRef& r, const St& x0, const Tape& t, V3 ball_v1u) {
    for (int a = 0; a < 3; a++) put_v3(r, 3 * a, x0.B.r[a]);
    put_v3(r, 9, x0.w);
    put_v3(r, 12, t.w1u);
    put_v3(r, 15, t.v1u);
    put_q(r, 18, t.q0);
    put_q(r, 22, t.dq);
    put_q(r, 26, t.qm);
    put_q(r, 30, t.qn);
    put_v3(r, 34, ball_v1u);
    r[37] = t.ang_clamped ? 1.f : 0.f;
}
// Rebuilds the reverse pass's inputs from the tape words `v` and the tick's raw controls `u`.
RSG_AD void get_tape(const float* v, float4 u, St& x0, Tape& t, V3& ball_v1u) {
    for (int a = 0; a < 3; a++) x0.B.r[a] = get_v3(v, 3 * a);
    x0.w = get_v3(v, 9);
    t.w1u = get_v3(v, 12);
    t.v1u = get_v3(v, 15);
    t.q0 = get_q(v, 18);
    t.dq = get_q(v, 22);
    t.qm = get_q(v, 26);
    t.qn = get_q(v, 30);
    ball_v1u = get_v3(v, 34);
    t.ang_clamped = v[37] != 0.f;
    t.cp = clampf(u.x, -1, 1);
    t.cy = clampf(u.y, -1, 1);
    t.cr = clampf(u.z, -1, 1);
    t.boost = clampf(u.w, 0, 1);
}

__global__ void air_forward_kernel(int n, int ticks, const float* __restrict__ state0, const float4* __restrict__ controls,
                                   float* __restrict__ final_state, float* __restrict__ ckpt, int ckpt_every, Cfg k) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    fill_damping(k);
    St x = load_state(state0 + (size_t)i * STATE);
    float4 un = ticks > 0 ? controls[i] : make_float4(0, 0, 0, 0);
    for (int t = 0; t < ticks; t++) {
        const float4 u = un;
        if (t + 1 < ticks) un = controls[(size_t)(t + 1) * n + i];  // a tick ahead
        if (ckpt && t % ckpt_every == 0) store_state(ckpt + ((size_t)(t / ckpt_every) * n + i) * STATE, x);
        car_tick(x, u, k, nullptr);
        ball_tick(x, k);
    }
    store_state(final_state + (size_t)i * STATE, x);
}

// One thread per (segment, instance): recompute the segment from its checkpoint, writing the tape.
__global__ void air_tape_kernel(int n, int ticks, const float4* __restrict__ controls, const float* __restrict__ ckpt,
                                int ckpt_every, int nseg, float* __restrict__ tape, Cfg k) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)nseg * n) return;
    const int sgi = (int)(idx / n), i = (int)(idx % n);
    fill_damping(k);
    const int t0 = sgi * ckpt_every;
    const int t1 = t0 + ckpt_every < ticks ? t0 + ckpt_every : ticks;
    St x = load_state(ckpt + ((size_t)sgi * n + i) * STATE);
    float4 un = controls[(size_t)t0 * n + i];
    for (int t = t0; t < t1; t++) {
        const float4 u = un;
        if (t + 1 < t1) un = controls[(size_t)(t + 1) * n + i];
        const St x0 = x;
        Tape tp;
        car_tick(x, u, k, &tp);
        V3 bv = ball_tick(x, k);
        put_tape(TapeRef{tape + (size_t)t * TAPE_WORDS * n + i, (size_t)n}, x0, tp, bv);
    }
}

// One thread per instance: the reverse pass over all ticks, reading the tape a tick ahead.
__global__ void air_sweep_kernel(int n, int ticks, const float4* __restrict__ controls, const float* __restrict__ tape,
                                 const float* __restrict__ grad_final, float4* __restrict__ grad_controls,
                                 float* __restrict__ grad_state0, Cfg k) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    fill_damping(k);
    Adj g;
    const float* gf = grad_final + (size_t)i * STATE;
    g.p = V3(gf[0], gf[1], gf[2]);
    g.v = V3(gf[3], gf[4], gf[5]);
    g.w = V3(gf[6], gf[7], gf[8]);
    for (int r = 0; r < 3; r++) g.B.r[r] = V3(gf[9 + 3 * r], gf[10 + 3 * r], gf[11 + 3 * r]);
    g.bp = V3(gf[18], gf[19], gf[20]);
    g.bv = V3(gf[21], gf[22], gf[23]);
    float nxt[TAPE_WORDS];
    float4 un = make_float4(0, 0, 0, 0);
    if (ticks > 0) {
        const float* src = tape + (size_t)(ticks - 1) * TAPE_WORDS * n + i;
#pragma unroll
        for (int w = 0; w < TAPE_WORDS; w++) nxt[w] = src[(size_t)w * n];
        un = controls[(size_t)(ticks - 1) * n + i];
    }
    for (int t = ticks - 1; t >= 0; t--) {
        float cur[TAPE_WORDS];
#pragma unroll
        for (int w = 0; w < TAPE_WORDS; w++) cur[w] = nxt[w];
        const float4 u = un;
        if (t > 0) {  // a tick ahead
            const float* src = tape + (size_t)(t - 1) * TAPE_WORDS * n + i;
#pragma unroll
            for (int w = 0; w < TAPE_WORDS; w++) nxt[w] = src[(size_t)w * n];
            un = controls[(size_t)(t - 1) * n + i];
        }
        St x0;
        Tape tp;
        V3 bv;
        get_tape(cur, u, x0, tp, bv);
        ball_tick_bwd(bv, g, k);
        grad_controls[(size_t)t * n + i] = car_tick_bwd(x0, u, tp, g, k);
    }
    if (grad_state0) {
        St gs;
        gs.p = g.p; gs.v = g.v; gs.w = g.w; gs.B = g.B; gs.bp = g.bp; gs.bv = g.bv;
        store_state(grad_state0 + (size_t)i * STATE, gs);
    }
}

static Cfg make_cfg(const rsg_car_config* c, float tick_rate) {
    // inverse inertia of the car box (Car::_BulletSetup, Car.cpp:195-292)
    const float U = RL::UU_TO_BT;
    V3 he = (V3(c->hitbox_size.x, c->hitbox_size.y, c->hitbox_size.z) * U) / 2.f;
    float margin = 0.04f;
    V3 implicit = he - V3(margin, margin, margin);
    int minax = he.x < he.y ? (he.x < he.z ? 0 : 2) : (he.y < he.z ? 1 : 2);
    float safe = 0.1f * he[minax];
    if (safe < margin) margin = safe;
    V3 hm = implicit + V3(margin, margin, margin);
    float lx = 2.f * hm.x, ly = 2.f * hm.y, lz = 2.f * hm.z, m = RL::CAR_MASS_BT;
    V3 inertia(m / 12.f * (ly * ly + lz * lz), m / 12.f * (lx * lx + lz * lz), m / 12.f * (lx * lx + ly * ly));
    Cfg k;
    k.iinv = V3(1.f / inertia.x, 1.f / inertia.y, 1.f / inertia.z);
    k.dt = 1.f / tick_rate;
    k.car_damp = k.ball_damp = 0.f;  // set by fill_damping on the device
    return k;
}

}  // namespace air
}  // namespace rsg

using namespace rsg;

static size_t tape_bytes(int n, int ticks) { return sizeof(float) * air::TAPE_WORDS * (size_t)n * (size_t)ticks; }

extern "C" int rsg_air_forward(const rsg_car_config* car, float tick_rate, int n, int ticks, const float* d_state0,
                               const float* d_controls, float* d_final, float* d_ckpt, int ckpt_every, void* stream) {
    if (!car || n < 0 || ticks < 0 || !d_state0 || !d_controls || !d_final || !(tick_rate > 0.f))
        return report_error(RSG_ERR_ARG, "rsg_air_forward: null pointer, negative size or tick_rate <= 0");
    if (d_ckpt && ckpt_every < 1) return report_error(RSG_ERR_ARG, "rsg_air_forward: ckpt_every must be >= 1");
    if (n == 0) return RSG_OK;
    air::Cfg k = air::make_cfg(car, tick_rate);
    air::air_forward_kernel<<<(n + 63) / 64, 64, 0, (cudaStream_t)stream>>>(
        n, ticks, d_state0, reinterpret_cast<const float4*>(d_controls), d_final, d_ckpt, d_ckpt ? ckpt_every : 1, k);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? RSG_OK : report_error(RSG_ERR_CUDA, cudaGetErrorString(e));
}

extern "C" int rsg_air_backward_workspace_size(int n, int ticks, size_t* bytes) {
    if (n < 0 || ticks < 0 || !bytes)
        return report_error(RSG_ERR_ARG, "rsg_air_backward_workspace_size: negative size or null pointer");
    *bytes = tape_bytes(n, ticks);
    return RSG_OK;
}

extern "C" int rsg_air_backward(const rsg_car_config* car, float tick_rate, int n, int ticks, const float* d_controls,
                                const float* d_ckpt, int ckpt_every, const float* d_grad_final, float* d_grad_controls,
                                float* d_grad_state0, void* d_workspace, size_t workspace_bytes, void* stream) {
    if (!car || n < 0 || ticks < 0 || !d_controls || !d_ckpt || !d_grad_final || !d_grad_controls ||
        !(tick_rate > 0.f))
        return report_error(RSG_ERR_ARG, "rsg_air_backward: null pointer, negative size or tick_rate <= 0");
    if (ckpt_every < 1) return report_error(RSG_ERR_ARG, "rsg_air_backward: ckpt_every must be >= 1");
    if (n == 0) return RSG_OK;
    if (ticks == 0) {  // the gradient passes straight through
        if (d_grad_state0)
            if (cudaMemcpyAsync(d_grad_state0, d_grad_final, sizeof(float) * air::STATE * (size_t)n,
                                cudaMemcpyDeviceToDevice, (cudaStream_t)stream) != cudaSuccess)
                return report_error(RSG_ERR_CUDA, "rsg_air_backward: copy of the gradient failed");
        return RSG_OK;
    }
    if (!d_workspace || workspace_bytes < tape_bytes(n, ticks))
        return report_error(RSG_ERR_ARG, "rsg_air_backward: workspace missing or smaller than "
                                         "rsg_air_backward_workspace_size");
    air::Cfg k = air::make_cfg(car, tick_rate);
    const int nseg = (ticks + ckpt_every - 1) / ckpt_every;
    const long long tape_threads = (long long)nseg * n;
    float* tape = static_cast<float*>(d_workspace);
    air::air_tape_kernel<<<(unsigned)((tape_threads + 127) / 128), 128, 0, (cudaStream_t)stream>>>(
        n, ticks, reinterpret_cast<const float4*>(d_controls), d_ckpt, ckpt_every, nseg, tape, k);
    air::air_sweep_kernel<<<(n + 63) / 64, 64, 0, (cudaStream_t)stream>>>(
        n, ticks, reinterpret_cast<const float4*>(d_controls), tape, d_grad_final,
        reinterpret_cast<float4*>(d_grad_controls), d_grad_state0, k);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? RSG_OK : report_error(RSG_ERR_CUDA, cudaGetErrorString(e));
}
