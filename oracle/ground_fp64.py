"""FP64 restatement of the ground-driving tick, and central finite differences of it.

Test infrastructure only: the checker for rsg_ground_forward / rsg_ground_backward and for the
autograd harness over them.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
leg use it.

The tick is the reference arena tick of one car whose four wheels stand on the flat floor
(z = 0) and whose chassis touches nothing, and of a ball that touches nothing, in Bullet units,
vectorised over instances:

* the wheel transforms and suspension rays of btVehicleRL (src/Sim/btVehicleRL/btVehicleRL.cpp:
  66-209): hard point R conn + p, ray down the car's -up of length rest + travel + radius -
  0.05, the floor hit, suspension length clamped to rest -/+ travel, relative velocity and
  clipped inverse contact dot, and the persistent extra push-back of a compressed wheel
  (resolveSingleCollision against the static floor, btVehicleRL.cpp:179-196);
* calcFrictionImpulses (btVehicleRL.cpp:306-380) with the previous tick's engine force, brake
  and friction factors: the side impulse of resolveSingleBilateral
  (libsrc/bullet3-3.24/BulletDynamics/ConstraintSolver/btContactConstraint.cpp:103-150) and the
  rolling impulse;
* Car::_UpdateWheels (src/Sim/Car/Car.cpp:339-484) with no handbrake and four wheels on the
  floor: the next tick's engine force, brake and steer angle, each wheel's lateral friction
  curve, the sticky force;
* updateSuspension and the impulses of btVehicleRL.cpp:270-303 and 383-395, in wheel order;
* the ground boost force of Car::_UpdateBoost (Car.cpp:515-521) with the boost input relaxed to
  [0, 1], whose full throttle becomes throttle + boost (1 - throttle) (1 at boost 1), without
  the boost-amount bookkeeping or the minimum boost time;
* gravity, integrateTransform and the clamps of Car::_FinishPhysicsTick (air_fp64.integrate);
  the ball as in air_fp64.

State layout, [n, 39]: car position (3), velocity (3), angular velocity (3), basis rows (9),
front steer angle, engine force, brake force, lateral friction factor (4), longitudinal friction
factor (4), extra push-back (4), ball position (3), ball velocity (3).  Controls: [ticks, n, 4] =
throttle, steer, boost, unused.  Pinned against the reference itself driving on the soccar
floor (tests/test_ground_oracle.py).
"""
from __future__ import annotations

import numpy as np

from oracle import air_fp64 as A

UU = A.UU_TO_BT
SUSPENSION_TRAVEL = 12.0 * UU
SUSPENSION_SUBTRACTION = 0.05
SUSPENSION_STIFFNESS = 500.0
DAMP_COMPRESSION, DAMP_RELAXATION = 25.0, 40.0
FORCE_SCALE = (36.0 - 0.25, 54.0 + 0.25 + 0.015)
THROTTLE_TORQUE = A.CAR_MASS_BT * 400.0 * UU
BRAKE_TORQUE = A.CAR_MASS_BT * (14.25 + 1.0 / 3.0) * UU
STOPPING_FORWARD_VEL, COASTING_BRAKE_FACTOR = 25.0, 0.15
BRAKING_NO_THROTTLE_SPEED_THRESH, THROTTLE_DEADZONE = 0.01, 0.001
BOOST_ACCEL_GROUND = 2975.0 / 3.0
ROLL_MAGIC = 113.73963
FSCALE = A.CAR_MASS_BT / 3.0

# LinearPieceCurve tables (src/RLConst.h:388-503)
CURVE_STEER = ((0, 500, 1000, 1500, 1750, 3000), (0.53356, 0.31930, 0.18203, 0.10570, 0.08507, 0.03454))
CURVE_DRIVE_TORQUE = ((0, 1400, 1410), (1.0, 0.1, 0.0))
CURVE_NON_STICKY = ((0, 0.7075, 1), (0.1, 0.5, 1.0))
CURVE_LAT_FRIC = ((0, 1), (1.0, 0.2))

OCTANE = dict(hitbox=(120.507, 86.6994, 38.6591), front=(12.50, 38.755, (51.25, 25.90, 20.755)),
              back=(15.00, 37.055, (-33.75, 29.50, 20.755)))

STATE = 39


def curve(c, x):
    """LinearPieceCurve::GetOutput (src/Math/Math.cpp:5-35), vectorised."""
    xs, ys = np.asarray(c[0], np.float64), np.asarray(c[1], np.float64)
    x = np.asarray(x, np.float64)
    out = np.full(x.shape, ys[-1])
    done = x <= xs[0]
    out = np.where(done, ys[0], out)
    for i in range(1, len(xs)):
        sel = ~done & (xs[i] > x)
        f = (x - xs[i - 1]) / (xs[i] - xs[i - 1])
        out = np.where(sel, ys[i - 1] + (ys[i] - ys[i - 1]) * f, out)
        done = done | sel
    return out


def car_geometry(cfg=OCTANE):
    """Inverse inertia, wheel connection points [4, 3], rest lengths and radii (front, back) in
    Bullet units (Car::_BulletSetup, Car.cpp:195-292: the left wheels mirror y; the rest length
    is the configured one minus the travel)."""
    conn = []
    for i in range(4):
        r, rest, c = cfg["front"] if i < 2 else cfg["back"]
        c = np.array(c, np.float64)
        if i % 2:
            c[1] = -c[1]
        conn.append(c * UU)
    rest = np.array([(cfg["front"][1] - 12.0) * UU, (cfg["back"][1] - 12.0) * UU])
    radius = np.array([cfg["front"][0] * UU, cfg["back"][0] * UU])
    return dict(iinv=A.car_inv_inertia(cfg["hitbox"]), conn=np.array(conn), rest=rest, radius=radius)


def _dot(a, b):
    return np.einsum("ni,ni->n", a, b)


def _normalized(a):
    return a / np.sqrt(_dot(a, a))[:, None]


def _axis_angle_matrix(axis, angle):
    """setRotation(btQuaternion(axis, angle)): the rotation by `angle` about `axis`."""
    d = np.sqrt(_dot(axis, axis))
    s = np.sin(angle * 0.5) / d
    q = np.concatenate([axis * s[:, None], np.cos(angle * 0.5)[:, None]], axis=1)
    return A._m_from_q(q)


def car_tick(x: np.ndarray, u: np.ndarray, geo: dict, dt: float, flags: np.ndarray | None = None) -> np.ndarray:
    """One tick of the car part of `x` ([n, 39]) under controls `u` ([n, 4]); ORs 1 into `flags`
    where a wheel misses the floor and 2 where the car tilts past the 0.1 contact-dot limit."""
    n = x.shape[0]
    p, v, w = x[:, 0:3], x[:, 3:6], x[:, 6:9]
    B = x[:, 9:18].reshape(-1, 3, 3)
    steer, engine, brake = x[:, 18], x[:, 19], x[:, 20]
    latf, longf = x[:, 21:25], x[:, 25:29]
    push = x[:, 29:33].copy()
    thr = np.clip(u[:, 0], -1, 1)
    st = np.clip(u[:, 1], -1, 1)
    bst = np.clip(u[:, 2], 0, 1)
    rt = np.where(bst >= 1, 1.0, thr + bst * (1 - thr))
    fwd, x1, up = B[:, :, 0], B[:, :, 1], B[:, :, 2]
    iw = np.einsum("nij,j,nkj->nik", B, geo["iinv"], B)
    nz = np.array([0.0, 0.0, 1.0])
    zero = np.zeros(n)
    hit, cp, lat, hp, sl, srv, cid = [], [], [], [], [], [], []
    fl = np.zeros(n, np.int64)
    for i in range(4):
        fb = 0 if i < 2 else 1
        rest, radius = geo["rest"][fb], geo["radius"][fb]
        h = np.einsum("nij,j->ni", B, geo["conn"][i]) + p
        sm = _axis_angle_matrix(up, steer if i < 2 else zero)
        la = np.einsum("nij,nj->ni", sm, x1)
        L = rest + SUSPENSION_TRAVEL + radius - SUSPENSION_SUBTRACTION
        dst = h - up * L
        ok = (h[:, 2] > 0) & (dst[:, 2] < 0)
        fl |= np.where(ok, 0, 1)
        with np.errstate(divide="ignore", invalid="ignore"):
            frac = np.where(ok, h[:, 2] / (h[:, 2] - dst[:, 2]), 1.0)
        c = (1 - frac)[:, None] * h + frac[:, None] * dst
        trace = _dot(h - c, up)
        s = np.clip(trace - radius, rest - SUSPENSION_TRAVEL, rest + SUSPENSION_TRAVEL)
        rel = c - p
        vac = v + np.cross(w, rel)
        steep = ~(up[:, 2] > 0.1)
        fl |= np.where(ok & steep, 2, 0)
        with np.errstate(divide="ignore", invalid="ignore"):
            inv = np.where(steep, 0.0, 1.0 / up[:, 2])
        srv.append(np.where(steep, 0.0, vac[:, 2] * inv))
        cid.append(np.where(steep, 10.0, inv))
        thresh = rest + radius - SUSPENSION_SUBTRACTION
        pushed = ok & (trace < thresh)
        c0 = np.cross(rel, np.broadcast_to(nz, rel.shape))
        c0w = np.einsum("ni,nij->nj", c0, iw)
        d0 = 1.0 / A.CAR_MASS_BT + np.cross(c0w, rel)[:, 2]
        imp = (0.2 * (thresh - trace) / dt - vac[:, 2]) / d0
        push[:, i] = np.where(pushed, np.maximum(imp, 0.0) / 4, np.where(ok, push[:, i], 0.0))
        hit.append(ok)
        cp.append(c)
        lat.append(la)
        hp.append(h)
        sl.append(s)
    # friction impulses of the previous tick's engine, brake and factors
    fimp = []
    for i in range(4):
        rel = cp[i] - p
        vac = v + np.cross(w, rel)
        axp = lat[i] * np.array([1.0, 1.0, 0.0])
        axle = _normalized(axp)
        fw = _normalized(np.cross(np.broadcast_to(nz, axle.shape), axle))
        aJ = np.einsum("nji,nj->ni", B, np.cross(rel, axle))
        diag = 1.0 / A.CAR_MASS_BT + (geo["iinv"] * aJ * aJ).sum(axis=1)
        side = -0.2 * _dot(axle, vac) / diag
        rv = _dot(vac, fw)
        if dt > 1 / 80.0:
            rv = np.where(np.abs(rv) < -(1 / (dt * 150.0)) + 0.8, 0.0, rv)
        roll_brake = np.minimum(np.maximum(-rv * ROLL_MAGIC, -brake), brake)
        roll = np.where(engine != 0, -engine / FSCALE, np.where(brake != 0, roll_brake, 0.0))
        imp = (fw * (roll * longf[:, i])[:, None] + axle * (side * latf[:, i])[:, None]) * FSCALE
        fimp.append(np.where(hit[i][:, None], imp, 0.0))
    # Car::_UpdateWheels
    fs = _dot(v, fwd) / UU
    absfs = np.abs(fs)
    dss = curve(CURVE_DRIVE_TORQUE, absfs)
    deadzone = np.abs(rt) < THROTTLE_DEADZONE
    opposing = (absfs > STOPPING_FORWARD_VEL) & (np.sign(rt) != np.sign(fs))
    eng = np.where(deadzone | (opposing & (absfs > BRAKING_NO_THROTTLE_SPEED_THRESH)), 0.0, rt)
    real_brake = np.where(deadzone, np.where(absfs < STOPPING_FORWARD_VEL, 1.0, COASTING_BRAKE_FACTOR),
                          np.where(opposing, 1.0, 0.0))
    new_engine = eng * THROTTLE_TORQUE * dss
    new_brake = real_brake * BRAKE_TORQUE
    new_steer = curve(CURVE_STEER, absfs) * st
    ns = curve(CURVE_NON_STICKY, np.ones(n))
    rt_zero = rt == 0
    new_latf, new_longf = latf.copy(), longf.copy()
    for i in range(4):
        lng = np.cross(lat[i], np.broadcast_to(nz, lat[i].shape))
        cv = (np.cross(w, hp[i] - p) + v) / UU
        base = np.abs(_dot(cv, lat[i]))
        with np.errstate(divide="ignore", invalid="ignore"):
            inp = np.where(base > 5, base / (np.abs(_dot(cv, lng)) + base), 0.0)
        lf = curve(CURVE_LAT_FRIC, inp) * np.where(rt_zero, ns, 1.0)
        gf = np.where(rt_zero, ns, 1.0)
        new_latf[:, i] = np.where(hit[i], lf, latf[:, i])
        new_longf[:, i] = np.where(hit[i], gf, longf[:, i])
    F = np.zeros((n, 3))
    F[:, 2] = 0.5 * A.GRAVITY_Z * UU * A.CAR_MASS_BT  # sticky force, the contact normals all point up
    # suspension and friction impulses
    vv, ww = v.copy(), w.copy()
    for i in range(4):
        fb = 0 if i < 2 else 1
        force = (geo["rest"][fb] - sl[i]) * SUSPENSION_STIFFNESS * cid[i]
        damp = np.where(srv[i] < 0, DAMP_COMPRESSION, DAMP_RELAXATION)
        sf = np.maximum((force - damp * srv[i]) * FORCE_SCALE[fb], 0.0)
        sf = np.where(hit[i], sf, 0.0)
        J = np.zeros((n, 3))
        J[:, 2] = sf * dt + push[:, i]
        J = np.where((sf != 0)[:, None], J, 0.0)
        rel = cp[i] - p
        vv = vv + J / A.CAR_MASS_BT
        ww = ww + np.einsum("nij,nj->ni", iw, np.cross(rel, J))
    for i in range(4):
        off = cp[i] - p
        rel = off - up * _dot(up, off)[:, None]
        J = fimp[i] * dt
        vv = vv + J / A.CAR_MASS_BT
        ww = ww + np.einsum("nij,nj->ni", iw, np.cross(rel, J))
    F = F + (bst * BOOST_ACCEL_GROUND * UU * A.CAR_MASS_BT)[:, None] * fwd
    F[:, 2] += A.GRAVITY_Z * UU * A.CAR_MASS_BT
    v1 = vv + F / A.CAR_MASS_BT * dt
    out = x.copy()
    out[:, 0:3], out[:, 3:6], out[:, 6:9], B1 = A.integrate(p, B, v1, ww, dt)
    out[:, 9:18] = B1.reshape(-1, 9)
    out[:, 18] = new_steer
    out[:, 19] = new_engine
    out[:, 20] = new_brake
    out[:, 21:25] = new_latf
    out[:, 25:29] = new_longf
    out[:, 29:33] = push
    if flags is not None:
        flags |= fl
    return out


def ball_tick(x: np.ndarray, dt: float) -> np.ndarray:
    v = x[:, 36:39] * (1.0 - A.BALL_DRAG) ** dt + np.array([0.0, 0.0, A.GRAVITY_Z * UU]) * dt
    out = x.copy()
    out[:, 33:36] = x[:, 33:36] + v * dt
    out[:, 36:39] = A._clamp_len(v, A.BALL_MAX_SPEED * UU)
    return out


def rollout(state0: np.ndarray, controls: np.ndarray, geo: dict, dt: float, trajectory: bool = False,
            flags: np.ndarray | None = None):
    """Runs `controls.shape[0]` ticks from `state0`; returns the final state (and the states
    after every tick when `trajectory`)."""
    x = np.asarray(state0, np.float64)
    traj = []
    for t in range(controls.shape[0]):
        x = ball_tick(car_tick(x, np.asarray(controls[t], np.float64), geo, dt, flags), dt)
        if trajectory:
            traj.append(x)
    return (x, np.stack(traj)) if trajectory else x


# ---------------------------------------------------------------- loss and gradients
def drive_loss(final: np.ndarray, target_xy: np.ndarray, target_dir: np.ndarray) -> np.ndarray:
    """Per-instance loss: squared distance of the final car position to `target_xy` ([n, 2])
    plus the squared distance of its forward axis to the unit vector `target_dir` ([n, 3])."""
    d = final[:, 0:2] - target_xy
    f = final[:, 9:18].reshape(-1, 3, 3)[:, :, 0] - target_dir
    return (d * d).sum(axis=1) + (f * f).sum(axis=1)


def drive_loss_grad(final: np.ndarray, target_xy: np.ndarray, target_dir: np.ndarray) -> np.ndarray:
    """d drive_loss / d final state, [n, 39]."""
    g = np.zeros_like(final)
    g[:, 0:2] = 2.0 * (final[:, 0:2] - target_xy)
    B = final[:, 9:18].reshape(-1, 3, 3)
    gB = np.zeros_like(B)
    gB[:, :, 0] = 2.0 * (B[:, :, 0] - target_dir)
    g[:, 9:18] = gB.reshape(-1, 9)
    return g


# front centre of the Octane hitbox in car space, Bullet units: the hitbox offset plus half its
# length along forward, the offset along up (CarConfig.cpp:20-27)
NOSE = np.array([(13.8757 + 120.507 / 2) * UU, 0.0, 20.755 * UU])


def contact_loss(final: np.ndarray, target_point: np.ndarray, target_vel: np.ndarray,
                 vel_scale: float = 1e-2) -> np.ndarray:
    """Per-instance loss at the end of the horizon: squared distance of the car's nose (the front
    centre of its hitbox, where it would meet a ball) to `target_point` ([n, 3]) plus vel_scale
    times the squared distance of its velocity to `target_vel` ([n, 3])."""
    B = final[:, 9:18].reshape(-1, 3, 3)
    d = final[:, 0:3] + np.einsum("nij,j->ni", B, NOSE) - target_point
    e = final[:, 3:6] - target_vel
    return (d * d).sum(axis=1) + vel_scale * (e * e).sum(axis=1)


def contact_loss_grad(final, target_point, target_vel, vel_scale: float = 1e-2) -> np.ndarray:
    """d contact_loss / d final state, [n, 39]."""
    B = final[:, 9:18].reshape(-1, 3, 3)
    d = final[:, 0:3] + np.einsum("nij,j->ni", B, NOSE) - target_point
    g = np.zeros_like(final)
    g[:, 0:3] = 2.0 * d
    g[:, 3:6] = 2.0 * vel_scale * (final[:, 3:6] - target_vel)
    g[:, 9:18] = (2.0 * d[:, :, None] * NOSE[None, None, :]).reshape(-1, 9)
    return g


def fd_grad(state0, controls, geo, dt, loss_fn, h: float = 1e-4, which=None) -> np.ndarray:
    """Central finite differences of sum(loss_fn(final)) with respect to the controls, in FP64.

    `which` selects the (tick, channel) entries to perturb (default: all three channels of every
    tick); entries not selected are NaN.  Each perturbation moves every instance at once."""
    T, n, _ = controls.shape
    g = np.full(controls.shape, np.nan)
    entries = which if which is not None else [(t, c) for t in range(T) for c in range(3)]
    for t, c in entries:
        cp = np.array(controls, np.float64)
        cm = cp.copy()
        cp[t, :, c] += h
        cm[t, :, c] -= h
        lp = loss_fn(rollout(state0, cp, geo, dt))
        lm = loss_fn(rollout(state0, cm, geo, dt))
        g[t, :, c] = (lp - lm) / (2.0 * h)
    return g
