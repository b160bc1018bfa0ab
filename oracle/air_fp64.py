"""FP64 restatement of the contact-free air tick, and central finite differences of it.

Test infrastructure only: the checker for rsg_air_forward / rsg_air_backward and for the
autograd harness over them.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
leg use it.

The tick is the reference arena tick of a car that touches nothing (no wheel, body or world
contact) and of a ball that touches nothing, in Bullet units, vectorised over instances:

* Car::_UpdateAirTorque, not flipping (src/Sim/Car/Car.cpp:584-669): pitch/yaw/roll torques
  about -right, up and -forward, and the damping about the same axes, scaled by
  CAR_TORQUE_SCALE and applied through the inverse world inertia (Car.cpp:655-668);
* the air boost force of Car::_UpdateBoost (Car.cpp:515-521), boostAccelAir * UU_TO_BT *
  forward * CAR_MASS_BT, with the boost input relaxed from {0, 1} to [0, 1] and without the
  boost-amount bookkeeping or the minimum boost time (Car.cpp:488-507);
* gravity as a force (btRigidBody::applyGravity, libsrc/bullet3-3.24/BulletDynamics/Dynamics/
  btRigidBody.cpp:209-215) and no car damping;
* the solver's external impulses, linear total_force * inv_mass * dt and angular
  total_torque * I_world_inv * dt (btSequentialImpulseConstraintSolver.cpp:458-492, written back
  at :1878-1904);
* btTransformUtil::integrateTransform (libsrc/bullet3-3.24/LinearMath/btTransformUtil.h:37-80)
  with btMatrix3x3::getRotation / setRotation (LinearMath/btMatrix3x3.h:216-246, 421-470);
* the speed clamps of Car::_FinishPhysicsTick (Car.cpp:165-193);
* for the ball, drag through btRigidBody::applyDamping (btRigidBody.cpp:153-162) and the speed
  clamp of Ball::_FinishPhysicsTick (src/Sim/Ball/Ball.cpp:117-143).

State layout, [n, 24] per instance: car position (3), velocity (3), angular velocity (3), basis
rows (9), ball position (3), ball velocity (3).  Controls: [ticks, n, 4] = pitch, yaw, roll,
boost.  Pinned against the reference itself in THE_VOID (tests/test_air_oracle.py).
"""
from __future__ import annotations

import numpy as np

UU_TO_BT = 1.0 / 50.0
GRAVITY_Z = -650.0
CAR_MASS_BT = 180.0
BALL_MASS_BT = 30.0
BALL_DRAG = 0.03
CAR_MAX_SPEED = 2300.0
CAR_MAX_ANG_SPEED = 5.5
BALL_MAX_SPEED = 6000.0
BOOST_ACCEL_AIR = 3175.0 / 3.0
CAR_TORQUE_SCALE = 2.0 * np.pi / (1 << 16) * 1000.0
AIR_TORQUE = np.array([130.0, 95.0, 400.0])
AIR_DAMP = np.array([30.0, 20.0, 50.0])
FLT_EPSILON = float(np.finfo(np.float32).eps)
ANGULAR_MOTION_THRESHOLD = 0.25 * np.pi


def car_inv_inertia(hitbox_size_uu) -> np.ndarray:
    """Local inverse inertia of the car: the hitbox child's own box inertia
    (Car::_BulletSetup, src/Sim/Car/Car.cpp:197-209).

    btBoxShape keeps the default 0.04 margin in its implicit half extents while setSafeMargin
    may shrink the margin itself (libsrc/bullet3-3.24/BulletCollision/CollisionShapes/
    btBoxShape.cpp:17-27); calculateLocalInertia (btBoxShape.cpp:33-44) uses the implicit
    extents plus the margin, m/12 * (b^2 + c^2) per axis."""
    he = np.asarray(hitbox_size_uu, np.float64) * UU_TO_BT / 2.0
    margin = 0.04
    implicit = he - margin
    safe = 0.1 * he.min()
    if safe < margin:
        margin = safe
    L = 2.0 * (implicit + margin)
    m = CAR_MASS_BT
    inertia = m / 12.0 * np.array([L[1] ** 2 + L[2] ** 2, L[0] ** 2 + L[2] ** 2, L[0] ** 2 + L[1] ** 2])
    return 1.0 / inertia


def _q_from_m(B: np.ndarray) -> np.ndarray:
    """btMatrix3x3::getRotation (btMatrix3x3.h:421-470), quaternion (x, y, z, w), batched.

    Positive trace: q = (m21 - m12, m02 - m20, m10 - m01, tr + 1) * 0.5 / sqrt(tr + 1).
    Otherwise the largest diagonal entry i (ties as Bullet breaks them) with j, k the next
    two axes in cyclic order: q[i] = x, q[j] = m_ji + m_ij, q[k] = m_ki + m_ik,
    w = m_kj - m_jk with x = m_ii - m_jj - m_kk + 1, all scaled by 0.5 / sqrt(x)."""
    n = B.shape[0]
    rows = np.arange(n)
    m00, m11, m22 = B[:, 0, 0], B[:, 1, 1], B[:, 2, 2]
    tr = m00 + m11 + m22
    i = np.where(m00 < m11, np.where(m11 < m22, 2, 1), np.where(m00 < m22, 2, 0))
    j = (i + 1) % 3
    k = (i + 2) % 3
    xi = B[rows, i, i] - B[rows, j, j] - B[rows, k, k] + 1.0
    t = np.zeros((n, 4))
    t[rows, i] = xi
    t[rows, j] = B[rows, j, i] + B[rows, i, j]
    t[rows, k] = B[rows, k, i] + B[rows, i, k]
    t[:, 3] = B[rows, k, j] - B[rows, j, k]
    pos = tr > 0.0
    tp = np.stack([B[:, 2, 1] - B[:, 1, 2], B[:, 0, 2] - B[:, 2, 0], B[:, 1, 0] - B[:, 0, 1], tr + 1.0], axis=1)
    x = np.where(pos, tr + 1.0, xi)
    t = np.where(pos[:, None], tp, t)
    return t * (0.5 / np.sqrt(x))[:, None]


def _m_from_q(q: np.ndarray) -> np.ndarray:
    """btMatrix3x3::setRotation (btMatrix3x3.h:216-246), batched (x, y, z, w)."""
    x, y, z, w = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    s = 2.0 / (x * x + y * y + z * z + w * w)
    M = np.empty((q.shape[0], 3, 3))
    M[:, 0, 0] = 1 - s * (y * y + z * z)
    M[:, 0, 1] = s * (x * y - w * z)
    M[:, 0, 2] = s * (x * z + w * y)
    M[:, 1, 0] = s * (x * y + w * z)
    M[:, 1, 1] = 1 - s * (x * x + z * z)
    M[:, 1, 2] = s * (y * z - w * x)
    M[:, 2, 0] = s * (x * z - w * y)
    M[:, 2, 1] = s * (y * z + w * x)
    M[:, 2, 2] = 1 - s * (x * x + y * y)
    return M


def _q_mul(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """btQuaternion::operator*= (LinearMath/btQuaternion.h), Hamilton product, (x, y, z, w)."""
    ax, ay, az, aw = a.T
    bx, by, bz, bw = b.T
    return np.stack([aw * bx + ax * bw + ay * bz - az * by,
                     aw * by + ay * bw + az * bx - ax * bz,
                     aw * bz + az * bw + ax * by - ay * bx,
                     aw * bw - ax * bx - ay * by - az * bz], axis=1)


def _clamp_len(v: np.ndarray, m: float) -> np.ndarray:
    l2 = np.einsum("ni,ni->n", v, v)
    over = l2 > m * m
    out = v.copy()
    out[over] = v[over] / np.sqrt(l2[over])[:, None] * m
    return out


def car_tick(x: np.ndarray, u: np.ndarray, iinv: np.ndarray, dt: float) -> np.ndarray:
    """One tick of the car part of `x` ([n, 24]) under controls `u` ([n, 4])."""
    p, v, w = x[:, 0:3], x[:, 3:6], x[:, 6:9]
    B = x[:, 9:18].reshape(-1, 3, 3)
    pitch = np.clip(u[:, 0], -1, 1)
    yaw = np.clip(u[:, 1], -1, 1)
    roll = np.clip(u[:, 2], -1, 1)
    boost = np.clip(u[:, 3], 0, 1)
    fwd, right, up = B[:, :, 0], B[:, :, 1], B[:, :, 2]
    pr, yu, rf = -right, up, -fwd
    torque = (pitch[:, None] * pr * AIR_TORQUE[0] + yaw[:, None] * yu * AIR_TORQUE[1]
              + roll[:, None] * rf * AIR_TORQUE[2])
    dp = np.einsum("ni,ni->n", pr, w) * AIR_DAMP[0] * (1 - np.abs(pitch))
    dy = np.einsum("ni,ni->n", yu, w) * AIR_DAMP[1] * (1 - np.abs(yaw))
    dr = np.einsum("ni,ni->n", rf, w) * AIR_DAMP[2]
    damping = yu * dy[:, None] + pr * dp[:, None] + rf * dr[:, None]
    # I_world_inv = B diag(iinv) B^T (btRigidBody::updateInertiaTensor)
    iw = np.einsum("nij,j,nkj->nik", B, iinv, B)
    total_torque = np.einsum("nij,nj->ni", np.linalg.inv(iw), torque - damping) * CAR_TORQUE_SCALE
    total_force = (boost * BOOST_ACCEL_AIR * UU_TO_BT)[:, None] * fwd * CAR_MASS_BT
    total_force = total_force + np.array([0.0, 0.0, GRAVITY_Z * UU_TO_BT]) * CAR_MASS_BT
    v1 = v + total_force / CAR_MASS_BT * dt
    w1 = w + np.einsum("nij,nj->ni", iw, total_torque) * dt
    out = x.copy()
    out[:, 0:3], out[:, 3:6], out[:, 6:9], B1 = integrate(p, B, v1, w1, dt)
    out[:, 9:18] = B1.reshape(-1, 9)
    return out


def integrate(p, B, v1, w1, dt):
    """btTransformUtil::integrateTransform of position and basis with the velocities after the
    solver, then the speed clamps of Car::_FinishPhysicsTick; returns p, v, w, B after the tick."""
    p1 = p + v1 * dt
    ang = np.sqrt(np.einsum("ni,ni->n", w1, w1))
    ang = np.where(ang * ang > FLT_EPSILON, ang, 0.0)
    ang = np.minimum(ang, ANGULAR_MOTION_THRESHOLD / dt)
    small = ang < 0.001
    with np.errstate(divide="ignore", invalid="ignore"):
        s = np.where(small, 0.5 * dt - (dt ** 3) * (0.020833333333) * ang * ang,
                     np.sin(0.5 * ang * dt) / np.where(small, 1.0, ang))
    dorn = np.concatenate([w1 * s[:, None], np.cos(ang * dt * 0.5)[:, None]], axis=1)
    q = _q_mul(dorn, _q_from_m(B))
    q = q / np.sqrt(np.einsum("ni,ni->n", q, q))[:, None]
    return (p1, _clamp_len(v1, CAR_MAX_SPEED * UU_TO_BT), _clamp_len(w1, CAR_MAX_ANG_SPEED), _m_from_q(q))


def ball_tick(x: np.ndarray, dt: float) -> np.ndarray:
    v = x[:, 21:24] * (1.0 - BALL_DRAG) ** dt + np.array([0.0, 0.0, GRAVITY_Z * UU_TO_BT]) * dt
    out = x.copy()
    out[:, 18:21] = x[:, 18:21] + v * dt
    out[:, 21:24] = _clamp_len(v, BALL_MAX_SPEED * UU_TO_BT)
    return out


def rollout(state0: np.ndarray, controls: np.ndarray, iinv: np.ndarray, dt: float,
            trajectory: bool = False):
    """Runs `controls.shape[0]` ticks from `state0`; returns the final state (and the states
    after every tick when `trajectory`)."""
    x = np.asarray(state0, np.float64)
    traj = []
    for t in range(controls.shape[0]):
        x = ball_tick(car_tick(x, np.asarray(controls[t], np.float64), iinv, dt), dt)
        if trajectory:
            traj.append(x)
    return (x, np.stack(traj)) if trajectory else x


# ---------------------------------------------------------------- loss and gradients
def aim_loss(final: np.ndarray, target_basis: np.ndarray, dist_scale: float = 1e-2) -> np.ndarray:
    """Per-instance loss: squared Frobenius distance of the final basis to `target_basis`
    ([n, 3, 3]) plus dist_scale * |car position + forward - ball position|^2 (the car's nose
    one Bullet unit ahead of its centre should reach the ball)."""
    B = final[:, 9:18].reshape(-1, 3, 3)
    orient = ((B - target_basis) ** 2).sum(axis=(1, 2))
    nose = final[:, 0:3] + B[:, :, 0]
    d = nose - final[:, 18:21]
    return orient + dist_scale * (d * d).sum(axis=1)


def aim_loss_grad(final: np.ndarray, target_basis: np.ndarray, dist_scale: float = 1e-2) -> np.ndarray:
    """d aim_loss / d final state, [n, 24]."""
    B = final[:, 9:18].reshape(-1, 3, 3)
    g = np.zeros_like(final)
    gB = 2.0 * (B - target_basis)
    d = final[:, 0:3] + B[:, :, 0] - final[:, 18:21]
    gd = 2.0 * dist_scale * d
    g[:, 0:3] = gd
    gB[:, :, 0] += gd
    g[:, 18:21] = -gd
    g[:, 9:18] = gB.reshape(-1, 9)
    return g


def fd_grad(state0, controls, iinv, dt, loss_fn, h: float = 1e-4, which=None) -> np.ndarray:
    """Central finite differences of sum(loss_fn(final)) with respect to the controls, in FP64.

    `which` selects the (tick, channel) entries to perturb (default: all); entries not
    selected are NaN.  Each perturbation moves every instance at once (instances are
    independent, so the per-instance partial derivatives separate)."""
    T, n, _ = controls.shape
    g = np.full(controls.shape, np.nan)
    entries = which if which is not None else [(t, c) for t in range(T) for c in range(4)]
    for t, c in entries:
        cp = np.array(controls, np.float64)
        cm = cp.copy()
        cp[t, :, c] += h
        cm[t, :, c] -= h
        lp = loss_fn(rollout(state0, cp, iinv, dt))
        lm = loss_fn(rollout(state0, cm, iinv, dt))
        g[t, :, c] = (lp - lm) / (2.0 * h)
    return g
