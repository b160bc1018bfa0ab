// rsg_ground.cuh -- differentiable driving rollouts of one car on the arena floor, and their adjoint:
// the device code shared by rsg_ground.cu (forward and tape kernels, C ABI) and rsg_ground_sweep.cu
// (the reverse sweep).
//
// The forward tick is the arena tick of a car whose four wheels stand on the flat floor (z = 0)
// and whose chassis touches nothing, with a contact-free ball (as in rsg_air.cu):
//   * btVehicleRL::updateWheelTransform and rayCast (src/Sim/btVehicleRL/btVehicleRL.cpp:66-209)
//     with the ray meeting the floor plane, including the persistent extra push-back of a
//     compressed wheel (resolveSingleCollision against the static floor);
//   * btVehicleRL::calcFrictionImpulses (btVehicleRL.cpp:306-380) with the engine force, brake
//     and friction factors of the previous tick;
//   * Car::_UpdateWheels (src/Sim/Car/Car.cpp:339-484) without handbrake: engine, brake and
//     steer angle for the next tick, each wheel's friction curves, the sticky force;
//   * btVehicleRL::updateSuspension and applyFrictionImpulses (btVehicleRL.cpp:270-395);
//   * the ground boost force of Car::_UpdateBoost (Car.cpp:486-533) with the boost input relaxed
//     to [0, 1]; the boost's full throttle becomes throttle + boost * (1 - throttle) (exactly 1
//     at boost 1), the boost amount is not tracked;
//   * gravity, the solver's external-impulse write-back, btTransformUtil::integrateTransform and
//     the clamps of Car::_FinishPhysicsTick (rsg_adjoint.cuh), and the ball of rsg_air.cu.
// Operations and their order follow rsg_tick_kernel, so for boost inputs of exactly 0 or 1 the
// tick is the arena tick of a car driving on the floor, up to the rounding of the hit fraction
// (the arena intersects the ray with the plane's triangles).  A wheel whose ray misses the
// floor or a car tilted past the suspension's 0.1 contact-dot limit leaves the model: the tick
// sets bit 0 or bit 1 of the instance's flags.  Jump, flip, handbrake and auto-roll are not part
// of it.
//
// The adjoint follows rsg_air.cu: the forward keeps a checkpoint every `ckpt_every` ticks; the
// tape kernel recomputes all segments at once and writes each tick's start state to the caller's
// workspace ([tick][word][instance]); the sweep kernel walks the ticks backwards, recomputing
// one tick's intermediates from its tape entry and applying the hand-written reverse tick.
#pragma once
#include <cuda_runtime.h>

#include "../../include/rocketsim_gb300.h"
#include "rsg_adjoint.cuh"
#include "rsg_consts.cuh"
#include "rsg_kernels.h"
#include "rsg_math.cuh"

namespace rsg {
namespace ground {

static __constant__ Curve g_curves[CV_COUNT] = RSG_CURVES_INIT;

// The curve table: constant memory on the device, the constexpr copy on the host.
RSG_HD const Curve& curve(int id) {
#if defined(__CUDA_ARCH__)
    return g_curves[id];
#else
    return CURVES_INIT[id];
#endif
}

// State, [n][STATE] floats (Bullet units): car position, velocity, angular velocity, basis rows,
// front steer angle, engine force, brake force, lateral friction factor per wheel, longitudinal
// friction factor per wheel, extra push-back per wheel, ball position, ball velocity.
// Controls, [ticks][n][4]: throttle, steer, boost, unused.
constexpr int STATE = 39;

struct Cfg {
    V3 iinv;                    // car inverse inertia (local)
    float dt;
    V3 conn[4];                 // wheel connection points (chassis space)
    float rest[2], radius[2];   // suspension rest length, wheel radius (front, back)
    float car_damp, ball_damp;  // btRigidBody::applyDamping factors, filled on the device
};
RSG_HD void fill_damping(Cfg& k) {
    k.car_damp = powf(1.f - 0.f, k.dt);
    k.ball_damp = powf(1.f - RL::BALL_DRAG, k.dt);
}
RSG_HD float suspension_travel() { return ((RL::MAX_SUSPENSION_TRAVEL * RL::UU_TO_BT) * 100) / 100; }
RSG_HD float ray_length(const Cfg& k, int fb) {
    return k.rest[fb] + suspension_travel() + k.radius[fb] - RL::SUSPENSION_SUBTRACTION;
}

struct GS {
    V3 p, v, w;
    M3 B;
    float steer, engine, brake;
    float latf[4], longf[4], push[4];
    V3 bp, bv;
};
template <class In>
RSG_HD GS load_state(In s) {
    GS x;
    x.p = V3(s[0], s[1], s[2]);
    x.v = V3(s[3], s[4], s[5]);
    x.w = V3(s[6], s[7], s[8]);
    for (int r = 0; r < 3; r++) x.B.r[r] = V3(s[9 + 3 * r], s[10 + 3 * r], s[11 + 3 * r]);
    x.steer = s[18];
    x.engine = s[19];
    x.brake = s[20];
    for (int i = 0; i < 4; i++) {
        x.latf[i] = s[21 + i];
        x.longf[i] = s[25 + i];
        x.push[i] = s[29 + i];
    }
    x.bp = V3(s[33], s[34], s[35]);
    x.bv = V3(s[36], s[37], s[38]);
    return x;
}
template <class Out>
RSG_HD void store_state(Out s, const GS& x) {
    s[0] = x.p.x; s[1] = x.p.y; s[2] = x.p.z;
    s[3] = x.v.x; s[4] = x.v.y; s[5] = x.v.z;
    s[6] = x.w.x; s[7] = x.w.y; s[8] = x.w.z;
    for (int r = 0; r < 3; r++) {
        s[9 + 3 * r] = x.B.r[r].x;
        s[10 + 3 * r] = x.B.r[r].y;
        s[11 + 3 * r] = x.B.r[r].z;
    }
    s[18] = x.steer;
    s[19] = x.engine;
    s[20] = x.brake;
    for (int i = 0; i < 4; i++) {
        s[21 + i] = x.latf[i];
        s[25 + i] = x.longf[i];
        s[29 + i] = x.push[i];
    }
    s[33] = x.bp.x; s[34] = x.bp.y; s[35] = x.bp.z;
    s[36] = x.bv.x; s[37] = x.bv.y; s[38] = x.bv.z;
}

RSG_HD float clampf(float v, float lo, float hi) { float m = v > lo ? v : lo; return m < hi ? m : hi; }
RSG_HD int sgnf(float v) { return (v > 0) - (v < 0); }

// One wheel's intermediates: what the reverse tick needs, all functions of the tick's start state,
// its controls and the wheel alone.
struct Wheel {
    V3 hp, dst, cp, lat;   // hard point, ray end, contact point, wheel basis column 1
    Q q;                   // steer rotation (identity for the back wheels)
    M3 sm;
    float frac, trace, sl;
    bool hit, sl_clamped, steep, pushed;
    V3 rel, vac;           // contact point - chassis origin, chassis velocity there
    float inv, srv, cid;   // 1 / contact dot, suspension relative velocity, clipped inverse dot
    // push-back (resolveSingleCollision)
    float pos_err, vel_err, jac, push_imp;
    V3 c0, c0w;
    float push;            // the push-back this tick's suspension impulse uses (and leaves)
    // friction impulse (calcFrictionImpulses)
    V3 axp, axle, fc, fwd, cx, aJ;
    float jinv, dv, side, roll;
    int roll_mode;         // 0 engine, 1 brake unclamped, 2 at -brake, 3 at +brake, 4 none
    bool rv_zeroed, imp_applied;
    V3 imp;
    // friction curves (_UpdateWheels)
    V3 lng, wd, cv;
    float base, q2, in, sb, sq;
    bool in_active;
    float latf_new, longf_new;
    // suspension
    float damp, sf_pre, sf;
    unsigned flags;
};
// The tick's car-wide intermediates
struct Common {
    float thr, str, bst, rt;
    bool rt_one, rt_zero;
    M3 iw;
    float fs, absfs, dss, eng, steer_curve, ns;
    int eng_mode;          // 0: engine from the throttle; 1: engine 0
    float new_engine, new_brake, new_steer;
};

RSG_HD void apply_impulse(V3& v, V3& w, const M3& iw, V3 imp, V3 rel) {  // btRigidBody::applyImpulse
    v += imp * (1.f / RL::CAR_MASS_BT);
    w += iw * cross(rel, imp);
}

// Controls, world inertia and the car part of Car::_UpdateWheels (engine, brake and steer of the
// next tick, four wheels on the floor).
RSG_HD void tick_common(const GS& x, float4 u, const Cfg& k, Common& C) {
    C.thr = clampf(u.x, -1.f, 1.f);
    C.str = clampf(u.y, -1.f, 1.f);
    C.bst = clampf(u.z, 0.f, 1.f);
    C.rt_one = C.bst >= 1.f;
    C.rt = C.rt_one ? 1.f : C.thr + C.bst * (1.f - C.thr);
    C.iw = scaled(x.B, k.iinv) * transpose(x.B);  // btRigidBody::updateInertiaTensor
    C.fs = dot(x.v, x.B.col(0)) * RL::BT_TO_UU;
    C.absfs = fabsf(C.fs);
    C.dss = curve_eval(curve(CV_DRIVE_TORQUE), C.absfs);
    C.eng = C.rt;
    C.eng_mode = 0;
    float real_brake = 0;
    if (fabsf(C.rt) >= RL::THROTTLE_DEADZONE) {
        if (C.absfs > RL::STOPPING_FORWARD_VEL && sgnf(C.rt) != sgnf(C.fs)) {
            real_brake = 1;
            if (C.absfs > RL::BRAKING_NO_THROTTLE_SPEED_THRESH) {
                C.eng = 0;
                C.eng_mode = 1;
            }
        }
    } else {
        C.eng = 0;
        C.eng_mode = 1;
        real_brake = (C.absfs < RL::STOPPING_FORWARD_VEL) ? 1 : RL::COASTING_BRAKE_FACTOR;
    }
    C.new_engine = C.eng * (RL::THROTTLE_TORQUE_AMOUNT * RL::UU_TO_BT) * C.dss;
    C.new_brake = real_brake * (RL::BRAKE_TORQUE_AMOUNT * RL::UU_TO_BT);
    C.steer_curve = curve_eval(curve(CV_STEER), C.absfs);
    C.new_steer = C.steer_curve * C.str;
    C.rt_zero = !(C.rt != 0);
    C.ns = curve_eval(curve(CV_NON_STICKY), 1.f);  // the contact normal's z
}

// Wheel i's part of the tick: transform, ray and push-back (btVehicleRL::updateWheelTransform,
// rayCast), friction impulse from the previous tick's engine, brake and factors
// (calcFrictionImpulses), friction factors of the next tick (_UpdateWheels) and suspension force
// (updateSuspension).
RSG_HD void wheel_forward(const GS& x, const Cfg& k, const Common& C, int i, Wheel& W) {
    const float dt = k.dt;
    const float inv_mass = 1.f / RL::CAR_MASS_BT;
    const V3 n(0, 0, 1);  // the floor's normal
    const M3& R = x.B;
    const V3 p = x.p, v = x.v, w = x.w;
    const V3 x1 = R.col(1), up = R.col(2);
    const float travel = suspension_travel();
    const int fb = i < 2 ? 0 : 1;
    const float rest = k.rest[fb], radius = k.radius[fb];
    Xf xf;
    xf.b = R;
    xf.o = p;
    W.flags = 0;
    W.hp = xf_apply(xf, k.conn[i]);
    const V3 dir = R * V3(0, 0, -1);
    W.q = q_axis_angle(up, i < 2 ? x.steer : 0.f);
    W.sm = m_from_q(W.q);
    W.lat = W.sm * x1;  // (steer rotation * wheel basis) column 1
    W.dst = W.hp + (dir * ray_length(k, fb));
    W.hit = W.hp.z > 0.f && W.dst.z < 0.f;
    W.frac = 1.f;
    W.cp = W.dst;
    W.pushed = false;
    W.imp_applied = false;
    W.in_active = false;
    W.sf = W.sf_pre = 0.f;
    W.imp = V3(0, 0, 0);
    W.latf_new = x.latf[i];
    W.longf_new = x.longf[i];
    if (!W.hit) {  // outside the model
        W.flags = 1u;
        W.push = 0.f;
        return;
    }
    W.frac = W.hp.z / (W.hp.z - W.dst.z);
    W.cp = lerp(W.hp, W.dst, W.frac);
    W.trace = dot(W.hp - W.cp, up);
    const float lo = rest - travel, hi = rest + travel;
    const float sl = W.trace - radius;
    W.sl_clamped = sl < lo || hi < sl;
    W.sl = sl < lo ? lo : (hi < sl ? hi : sl);
    W.rel = W.cp - p;
    W.vac = v + cross(w, W.rel);
    const float denom = up.z;  // contact normal . up
    W.steep = !(denom > 0.1f);
    if (!W.steep) {
        W.inv = 1 / denom;
        W.srv = W.vac.z * W.inv;
        W.cid = W.inv;
    } else {
        W.flags = 2u;
        W.inv = 0;
        W.srv = 0;
        W.cid = 10;
    }
    const float thresh = (rest + radius) - RL::SUSPENSION_SUBTRACTION;
    W.pushed = W.trace < thresh;
    W.push = x.push[i];
    if (W.pushed) {
        const float rel_vel = W.vac.z;
        const float restitution = 0.f * -rel_vel;
        W.pos_err = 0.2f * -(W.trace - thresh) / dt;
        W.vel_err = -(1.0f + restitution) * rel_vel;
        W.c0 = cross(W.rel, n);
        W.c0w = W.c0 * C.iw;
        const float d0 = inv_mass + dot(n, cross(W.c0w, W.rel));
        W.jac = 1.f / (d0 + 0.f);
        W.push_imp = W.pos_err * W.jac + W.vel_err * W.jac;
        W.push = (0.f > W.push_imp ? 0.f : W.push_imp) / 4;
    }
    // friction impulse, resolveSingleBilateral against the static floor (btContactConstraint.cpp:103-150)
    const float fscale = (1.f / inv_mass) / 3;
    W.axp = W.lat - n * dot(W.lat, n);
    W.axle = safe_normalized(W.axp);
    W.fc = cross(n, W.axle);
    W.fwd = safe_normalized(W.fc);
    W.cx = cross(W.rel, W.axle);
    W.aJ = transpose(R) * W.cx;
    const V3 m0 = k.iinv * W.aJ;
    const float diag = inv_mass + dot(m0, W.aJ);
    W.jinv = 1.f / diag;
    W.dv = dot(W.axle, W.vac);
    W.side = -0.2f * W.dv * W.jinv;
    W.rv_zeroed = false;
    if (x.engine == 0) {
        if (x.brake) {
            float rv = dot(W.vac, W.fwd);
            if (dt > (1 / 80.f)) {
                float th = -(1 / (dt * 150.f)) + 0.8f;
                if (fabsf(rv) < th) {
                    rv = 0;
                    W.rv_zeroed = true;
                }
            }
            const float MAGIC = 113.73963f;
            const float xr = -rv * MAGIC;
            const float blo = -x.brake, bhi = x.brake;
            const float r = xr > blo ? xr : blo;
            W.roll_mode = xr > blo ? 1 : 2;
            if (!(r < bhi)) W.roll_mode = 3;
            W.roll = r < bhi ? r : bhi;
        } else {
            W.roll_mode = 4;
            W.roll = 0;
        }
    } else {
        W.roll_mode = 0;
        W.roll = -x.engine / fscale;
    }
    const V3 total = (W.fwd * W.roll * x.longf[i]) + (W.axle * W.side * x.latf[i]);
    W.imp = total * fscale;
    W.imp_applied = !is_zero(W.imp);
    // friction factors of the next tick
    W.lng = cross(W.lat, n);
    W.wd = W.hp - p;
    W.cv = (cross(w, W.wd) + v) * RL::BT_TO_UU;
    const float dl = dot(W.cv, W.lat);
    W.sb = dl < 0 ? -1.f : 1.f;
    W.base = fabsf(dl);
    W.in = 0;
    W.in_active = W.base > 5;
    if (W.in_active) {
        const float dq = dot(W.cv, W.lng);
        W.sq = dq < 0 ? -1.f : 1.f;
        W.q2 = fabsf(dq);
        W.in = W.base / (W.q2 + W.base);
    }
    float latf = curve_eval(curve(CV_LAT_FRIC), W.in);
    float longf = 1;  // no handbrake
    if (C.rt_zero) {
        latf *= C.ns;
        longf *= C.ns;
    }
    W.latf_new = latf;
    W.longf_new = longf;
    // suspension force
    const float force = (rest - W.sl) * RL::SUSPENSION_STIFFNESS * W.cid;
    W.damp = (W.srv < 0) ? RL::WHEELS_DAMPING_COMPRESSION : RL::WHEELS_DAMPING_RELAXATION;
    float sf = force - (W.damp * W.srv);
    sf *= (i < 2) ? RL::SUSPENSION_FORCE_SCALE_FRONT : RL::SUSPENSION_FORCE_SCALE_BACK;
    W.sf_pre = sf;
    W.sf = sf < 0 ? 0 : sf;
}

// One tick of the car.  `it` (optional) receives the integration's intermediates, among them the
// velocities after the solver; returns the flags of the tick.
RSG_HD unsigned car_tick(GS& x, float4 u, const Cfg& k, adj::IntTape* it) {
    const float dt = k.dt;
    const float inv_mass = 1.f / RL::CAR_MASS_BT;
    const V3 n(0, 0, 1);
    Common C;
    tick_common(x, u, k, C);
    const V3 p = x.p, fwd_car = x.B.col(0), up = x.B.col(2);
    V3 rel[4], imp[4];
    float sf[4], push[4], latf[4], longf[4];
    bool applied[4];
    unsigned flags = 0;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        Wheel W;
        wheel_forward(x, k, C, i, W);
        rel[i] = W.rel;
        imp[i] = W.imp;
        applied[i] = W.imp_applied;
        sf[i] = W.sf;
        push[i] = W.push;
        latf[i] = W.latf_new;
        longf[i] = W.longf_new;
        flags |= W.flags;
    }
    // sticky force along the wheels' common contact normal
    const V3 updir(0, 0, 1);
    const bool full = (C.rt != 0) || (C.absfs > RL::STOPPING_FORWARD_VEL);
    float sfs = 0.5f;
    if (full) sfs += 1 - fabsf(updir.z);
    V3 F = V3(0, 0, 0) + updir * sfs * (RL::GRAVITY_Z * RL::UU_TO_BT) * RL::CAR_MASS_BT;
    // the suspension impulses, then the friction impulses, wheel by wheel
    V3 vv = x.v, ww = x.w;
#pragma unroll
    for (int i = 0; i < 4; i++)
        if (sf[i] != 0) apply_impulse(vv, ww, C.iw, n * ((sf[i] * dt) + push[i]), rel[i]);
#pragma unroll
    for (int i = 0; i < 4; i++) {
        if (applied[i]) {
            const float d = dot(up, rel[i]);
            apply_impulse(vv, ww, C.iw, imp[i] * dt, rel[i] - up * d);
        }
    }
    // boost, gravity, damping, the solver's write-back and the integration
    F += ((C.bst * RL::BOOST_ACCEL_GROUND) * RL::UU_TO_BT) * fwd_car * RL::CAR_MASS_BT;
    F += V3(0, 0, RL::GRAVITY_Z * RL::UU_TO_BT) * (1.f / inv_mass);
    vv = vv * k.car_damp;
    ww = ww * k.car_damp;
    const V3 v1u = (vv + V3(0, 0, 0)) + F * inv_mass * dt;
    const V3 w1u = ww;
    adj::integrate_car(x.p, x.B, x.v, x.w, v1u, w1u, dt, it);
    (void)p;
    x.steer = C.new_steer;
    x.engine = C.new_engine;
    x.brake = C.new_brake;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        x.latf[i] = latf[i];
        x.longf[i] = longf[i];
        x.push[i] = push[i];
    }
    return flags;
}

// One tick of the ball; returns its velocity before the speed clamp.
RSG_HD V3 ball_tick(GS& x, const Cfg& k) {
    const float dt = k.dt;
    const float mass = RL::BALL_MASS_BT, inv_mass = 1.f / mass;
    V3 force = V3(0, 0, 0) + V3(0, 0, RL::GRAVITY_Z * RL::UU_TO_BT) * (1.f / inv_mass);
    V3 v = x.bv * k.ball_damp;
    v = (v + V3(0, 0, 0)) + force * inv_mass * dt;
    x.bp = x.bp + v * dt;
    x.bv = adj::clamp_len_fwd(v, RL::BALL_MAX_SPEED * RL::UU_TO_BT);
    return v;
}

// ---------------------------------------------------------------- reverse tick
RSG_HD M3 zero_m3() {
    M3 m;
    for (int r = 0; r < 3; r++) m.r[r] = V3(0, 0, 0);
    return m;
}
RSG_HD void add_col(M3& G, int c, V3 v) {
    G.r[0][c] += v.x;
    G.r[1][c] += v.y;
    G.r[2][c] += v.z;
}
RSG_HD void add_outer(M3& G, V3 a, V3 b) {  // G += a b^T
    for (int r = 0; r < 3; r++) G.r[r] += b * a[r];
}
// Reverse of apply_impulse for the adjoints gv, gw of the velocities after it (which are also
// those before it): adds the adjoints of the impulse J, of its offset rel and of iw.
RSG_HD void apply_impulse_bwd(const M3& iw, V3 J, V3 rel, V3 gv, V3 gw, V3& gJ, V3& grel, M3& giw) {
    gJ += gv * (1.f / RL::CAR_MASS_BT);
    add_outer(giw, gw, cross(rel, J));
    adj::cross_bwd(rel, J, transpose(iw) * gw, grel, gJ);
}

// Adjoint accumulators of the car part of one reverse tick
struct CarAdj {
    V3 p, v, w, col0, col1, up;
    M3 R, iw;
    float steer, engine, brake;
};

// Reverse of wheel i's part of the tick (wheel_forward and the wheel's two impulses): `g` is the
// adjoint of the state after the tick, gvv / gww those of the chassis velocities after the
// impulses; adds to `a` and to o's wheel entries (the adjoint of the state before the tick).
RSG_HD void wheel_bwd(const GS& x0, const Cfg& k, const Common& C, int i, const Wheel& W, const GS& g, V3 gvv,
                      V3 gww, CarAdj& a, GS& o) {
    const float dt = k.dt;
    const float inv_mass = 1.f / RL::CAR_MASS_BT;
    const V3 n(0, 0, 1);
    const M3& R = x0.B;
    const V3 w = x0.w, x1 = R.col(1), up = R.col(2);
    const float fscale = (1.f / inv_mass) / 3;
    const int fb = i < 2 ? 0 : 1;
    if (!W.hit) {  // the factors carry over; the push-back was zeroed
        o.latf[i] += g.latf[i];
        o.longf[i] += g.longf[i];
        return;
    }
    V3 gcp(0, 0, 0), ghp(0, 0, 0), glat(0, 0, 0), gvac(0, 0, 0), grel(0, 0, 0);
    float gpush = g.push[i];  // adjoint of the push-back this tick used (also its output)
    // friction impulse on the chassis: J = imp dt at off - up (up . off), off = rel
    V3 gimp(0, 0, 0);
    if (W.imp_applied) {
        const V3 off = W.rel;
        const float d = dot(up, off);
        V3 gJ(0, 0, 0), gr(0, 0, 0);
        apply_impulse_bwd(C.iw, W.imp * dt, off - up * d, gvv, gww, gJ, gr, a.iw);
        gimp = gJ * dt;
        const float gd = -dot(gr, up);
        a.up += gr * (-d) + off * gd;
        grel += gr + up * gd;
    }
    // suspension impulse: J = n ((sf dt) + push) at rel
    float gsf = 0;
    if (W.sf != 0) {
        const float base = (W.sf * dt) + W.push;
        V3 gJ(0, 0, 0);
        apply_impulse_bwd(C.iw, n * base, W.rel, gvv, gww, gJ, grel, a.iw);
        const float gbase = dot(n, gJ);
        gsf = gbase * dt;
        gpush += gbase;
    }
    // suspension force: sf = max(0, (((rest - sl) K) cid - damp srv) scale)
    float gsl = 0, gcid = 0, gsrv = 0;
    if (W.sf_pre > 0) {
        const float gs = gsf * ((i < 2) ? RL::SUSPENSION_FORCE_SCALE_FRONT : RL::SUSPENSION_FORCE_SCALE_BACK);
        gsrv -= W.damp * gs;
        gsl -= RL::SUSPENSION_STIFFNESS * W.cid * gs;
        gcid += (k.rest[fb] - W.sl) * RL::SUSPENSION_STIFFNESS * gs;
    }
    // lateral friction factor of the next tick: curve(|cv.lat| / (|cv.lng| + |cv.lat|))
    if (W.in_active) {
        float gl = g.latf[i];
        if (C.rt_zero) gl *= C.ns;
        const float gin = adj::curve_slope(curve(CV_LAT_FRIC), W.in) * gl;
        const float s = W.q2 + W.base;
        const float gdl = W.sb * gin * (W.q2 / (s * s));
        const float gdq = -W.sq * gin * (W.base / (s * s));
        V3 gcv = W.lat * gdl + W.lng * gdq;
        glat += W.cv * gdl + cross(n, W.cv * gdq);  // lng = lat x n
        gcv = gcv * RL::BT_TO_UU;
        a.v += gcv;
        V3 gwd(0, 0, 0);
        adj::cross_bwd(w, W.wd, gcv, a.w, gwd);
        ghp += gwd;
        a.p -= gwd;
    }
    // friction impulse: imp = ((fwd roll) longf + (axle side) latf) fscale
    if (W.imp_applied) {
        const V3 gtot = gimp * fscale;
        const V3 gA = gtot * x0.longf[i];
        o.longf[i] += dot(gtot, W.fwd * W.roll);
        V3 gfwd = gA * W.roll;
        const float groll = dot(gA, W.fwd);
        const V3 gBv = gtot * x0.latf[i];
        o.latf[i] += dot(gtot, W.axle * W.side);
        V3 gaxle = gBv * W.side;
        const float gside = dot(gBv, W.axle);
        if (W.roll_mode == 0) {
            a.engine -= groll / fscale;
        } else if (W.roll_mode == 1) {
            if (!W.rv_zeroed) {  // roll = -(vac . fwd) MAGIC
                const float grv = -113.73963f * groll;
                gvac += W.fwd * grv;
                gfwd += W.vac * grv;
            }
        } else if (W.roll_mode == 2) {
            a.brake -= groll;
        } else if (W.roll_mode == 3) {
            a.brake += groll;
        }
        // side = (-0.2 dv) jinv, dv = axle . vac, jinv = 1 / (inv_mass + (iinv aJ) . aJ),
        // aJ = R^T (rel x axle)
        const float gdv = -0.2f * W.jinv * gside;
        const float gjinv = (-0.2f * W.dv) * gside;
        const float gdiag = -W.jinv * W.jinv * gjinv;
        const V3 gaJ = (k.iinv * W.aJ) * (2.f * gdiag);
        add_outer(a.R, W.cx, gaJ);
        adj::cross_bwd(W.rel, W.axle, R * gaJ, grel, gaxle);
        gaxle += W.vac * gdv;
        gvac += W.axle * gdv;
        // fwd = fc / |fc|, fc = n x axle; axle = axp / |axp|, axp = lat - n (lat . n)
        const V3 gfc = adj::normalize_bwd(W.fc, gfwd);
        gaxle += cross(gfc, n);
        const V3 gaxp = adj::normalize_bwd(W.axp, gaxle);
        glat += gaxp - n * dot(n, gaxp);
    }
    // push-back: push = max(0, pos_err jac + vel_err jac) / 4
    float gtrace = 0;
    if (W.pushed) {
        if (W.push_imp > 0) {
            const float gi = gpush * 0.25f;
            const float gjac = (W.pos_err + W.vel_err) * gi;
            gtrace += (-0.2f / dt) * (W.jac * gi);  // pos_err = (0.2 -(trace - thresh)) / dt
            gvac.z -= W.jac * gi;                    // vel_err = -vac.z
            // jac = 1 / d0, d0 = inv_mass + n . (c0w x rel), c0w = c0 iw, c0 = rel x n
            const float gd0 = -W.jac * W.jac * gjac;
            V3 gc0w(0, 0, 0), gn(0, 0, 0);
            adj::cross_bwd(W.c0w, W.rel, n * gd0, gc0w, grel);
            add_outer(a.iw, W.c0, gc0w);
            adj::cross_bwd(W.rel, n, C.iw * gc0w, grel, gn);
        }
    } else {
        o.push[i] += gpush;
    }
    // suspension relative velocity and clipped inverse contact dot: srv = vac.z inv, cid = inv
    if (!W.steep) {
        gvac.z += W.inv * gsrv;
        a.up.z -= W.inv * W.inv * (W.vac.z * gsrv + gcid);
    }
    if (!W.sl_clamped) gtrace += gsl;
    // vac = v + w x rel, rel = cp - p
    a.v += gvac;
    adj::cross_bwd(w, W.rel, gvac, a.w, grel);
    gcp += grel;
    a.p -= grel;
    // trace = (hp - cp) . up
    ghp += up * gtrace;
    gcp -= up * gtrace;
    a.up += (W.hp - W.cp) * gtrace;
    // cp = (1 - frac) hp + frac dst, frac = hp.z / (hp.z - dst.z), dst = hp - up L
    V3 ghs = gcp * (1.0f - W.frac), gdst = gcp * W.frac;
    const float gfrac = dot(gcp, W.dst - W.hp);
    const float den = W.hp.z - W.dst.z;
    ghs.z -= gfrac * W.dst.z / (den * den);
    gdst.z += gfrac * W.hp.z / (den * den);
    ghp += ghs + gdst;
    a.up -= gdst * ray_length(k, fb);
    // hp = R conn + p
    a.p += ghp;
    add_outer(a.R, ghp, k.conn[i]);
    // lat = sm(q(up, steer)) x1
    a.col1 += transpose(W.sm) * glat;
    if (i < 2) {
        M3 gsm;
        for (int r = 0; r < 3; r++) gsm.r[r] = x1 * glat[r];
        const Q gq = adj::m_from_q_bwd(W.q, gsm);
        // q = (up sin(h) / |up|, cos(h)), h = steer / 2
        const float h = x0.steer * 0.5f, d = len(up), sh = sinf(h), ch = cosf(h);
        const V3 gqv(gq.x, gq.y, gq.z);
        const float gs = dot(gqv, up);
        a.up += gqv * (sh / d) - up * (gs * sh / (d * d * d));
        a.steer += gs * (ch * 0.5f / d) - gq.w * sh * 0.5f;
    }
}

// Reverse of ball_tick given the ball velocity before the clamp
RSG_HD void ball_tick_bwd(V3 v1u, GS& g, const Cfg& k) {
    V3 gv1u = adj::clamp_len_bwd(v1u, RL::BALL_MAX_SPEED * RL::UU_TO_BT, g.bv) + g.bp * k.dt;
    g.bv = gv1u * k.ball_damp;
}

// One reverse tick.  x0: the state at the tick's start; v1u, w1u: the chassis velocities after
// the solver (before the clamps).  `g` holds the adjoint of the state after the tick and becomes
// that of the state before it; returns the adjoint of the controls.  Inputs on the boundary of
// their range pass their gradient, inputs outside get none; at boost 1 the boost gets the
// one-sided derivative from inside its range.  Every intermediate is recomputed here: the car-wide
// ones once, each wheel's just before its reverse.
RSG_HD float4 tick_bwd(const GS& x0, float4 u, V3 v1u, V3 w1u, const Cfg& k, GS& g) {
    const float dt = k.dt;
    const float inv_mass = 1.f / RL::CAR_MASS_BT;
    const M3& R = x0.B;
    const V3 v = x0.v;
    const V3 fwd_car = R.col(0);
    // ball
    {
        GS xb = x0;
        const V3 bv1u = ball_tick(xb, k);
        ball_tick_bwd(bv1u, g, k);
    }
    Common C;
    tick_common(x0, u, k, C);
    adj::IntTape it;
    {
        V3 p1 = x0.p, vo, wo;
        M3 B1 = x0.B;
        adj::integrate_car(p1, B1, vo, wo, v1u, w1u, dt, &it);
    }
    GS o;  // adjoint of the state before the tick
    o.bp = g.bp;
    o.bv = g.bv;
    o.steer = o.engine = o.brake = 0;
    for (int i = 0; i < 4; i++) o.latf[i] = o.longf[i] = o.push[i] = 0;
    CarAdj a;
    a.p = a.v = a.w = a.col0 = a.col1 = a.up = V3(0, 0, 0);
    a.iw = zero_m3();
    a.steer = a.engine = a.brake = 0;
    float grt = 0, gbst = 0, gstr = 0;
    // integration and clamps
    V3 gp1 = g.p, gv1u, gw1u;
    adj::integrate_car_bwd(R, it, dt, gp1, g.B, g.v, g.w, a.R, gv1u, gw1u);
    a.p += gp1;
    // v1u = v_imp damp + F inv_mass dt, w1u = w_imp damp; the impulses add to v and w
    const V3 gvv = gv1u * k.car_damp, gww = gw1u * k.car_damp;
    const V3 gF = gv1u * (inv_mass * dt);
    a.v += gvv;
    a.w += gww;
    // boost force ((b A) U) fwd M
    gbst += dot(gF, fwd_car) * (RL::BOOST_ACCEL_GROUND * RL::UU_TO_BT * RL::CAR_MASS_BT);
    a.col0 += gF * (((C.bst * RL::BOOST_ACCEL_GROUND) * RL::UU_TO_BT) * RL::CAR_MASS_BT);
    // each wheel's chain back to the state (the impulses add up, so wheels are independent)
#pragma unroll 1
    for (int i = 0; i < 4; i++) {
        Wheel W;
        wheel_forward(x0, k, C, i, W);
        wheel_bwd(x0, k, C, i, W, g, gvv, gww, a, o);
    }
    // Car::_UpdateWheels: steer = curve(|fs|) steer_input, engine = rt TT curve(|fs|)
    {
        float gabsfs = adj::curve_slope(curve(CV_STEER), C.absfs) * C.str * g.steer;
        gstr += C.steer_curve * g.steer;
        if (C.eng_mode == 0) {
            const float TTU = RL::THROTTLE_TORQUE_AMOUNT * RL::UU_TO_BT;
            grt += TTU * C.dss * g.engine;
            gabsfs += adj::curve_slope(curve(CV_DRIVE_TORQUE), C.absfs) * (C.eng * TTU) * g.engine;
        }
        const float gfs = (C.fs > 0 ? 1.f : (C.fs < 0 ? -1.f : 0.f)) * gabsfs * RL::BT_TO_UU;
        a.v += fwd_car * gfs;
        a.col0 += v * gfs;
    }
    // iw = R diag(iinv) R^T
    {
        M3 S;
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++) S.r[r][c] = a.iw.r[r][c] + a.iw.r[c][r];
        const M3 SR = S * R;
        for (int r = 0; r < 3; r++) a.R.r[r] += SR.r[r] * k.iinv;
    }
    add_col(a.R, 0, a.col0);
    add_col(a.R, 1, a.col1);
    add_col(a.R, 2, a.up);
    o.p = a.p;
    o.v = a.v;
    o.w = a.w;
    o.B = a.R;
    o.steer = a.steer;
    o.engine = a.engine;
    o.brake = a.brake;
    g = o;
    // rt = t + b (1 - t)
    const float gthr = C.rt_one ? 0.f : grt * (1.f - C.bst);
    gbst += grt * (1.f - C.thr);
    float4 gu;
    gu.x = (u.x >= -1.f && u.x <= 1.f) ? gthr : 0.f;
    gu.y = (u.y >= -1.f && u.y <= 1.f) ? gstr : 0.f;
    gu.z = (u.z >= 0.f && u.z <= 1.f) ? gbst : 0.f;
    gu.w = 0.f;
    return gu;
}

struct Strided {  // word w of one instance in a [word][instance] array
    float* base;
    size_t n;
    RSG_HD float& operator[](int w) const { return base[(size_t)w * n]; }
};

// Words per instance and tick on the tape: the tick's start state, then the chassis velocities
// after the solver (what the integration starts from).
constexpr int TAPE_WORDS = STATE + 6;

// Launches the reverse sweep (rsg_ground_sweep.cu): one thread per instance.
cudaError_t launch_ground_sweep(int n, int ticks, const float4* controls, const float* tape, const float* grad_final,
                                float4* grad_controls, float* grad_state0, const Cfg& k, cudaStream_t st);

}  // namespace ground
}  // namespace rsg
