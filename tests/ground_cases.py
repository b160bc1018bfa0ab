"""Shared cases for the ground-rollout tests: the reference golden drives and gradient cases."""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
if REPO not in sys.path:
    sys.path.insert(0, REPO)

from rocketsim_gb300 import abi  # noqa: E402

GOLDEN = os.path.join(HERE, "golden", "ground_rollouts.npz")
DT = 1.0 / 120.0
U = np.float32(1.0 / 50.0)
STATE = 39

# |rollout - reference| bounds after 1, 30 and 120 ticks (uu, uu/s, rad/s, basis entries, and the
# vehicle state relative to each field's largest magnitude, at least 1: the engine force, up to
# 1440, follows the drive-torque curve, whose last segment falls by 1 % per uu/s near 1400 uu/s); the
# golden stores float32 uu, whose conversion alone rounds positions and velocities by ~1e-4, and
# the reference integrates the ball's position in float32 (~1e-4 uu per tick at 1000 uu).
TOL = {1: dict(pos=1e-3, vel=2e-3, ang=1e-5, rot=1e-6, veh=1e-4),
       30: dict(pos=1e-2, vel=5e-3, ang=2e-5, rot=1e-5, veh=5e-4),
       120: dict(pos=3e-2, vel=1e-2, ang=5e-5, rot=2e-5, veh=1e-3)}


def load_golden():
    g = np.load(GOLDEN)
    cars = [abi.CarState.from_buffer_copy(x.tobytes()) for x in g["init_cars"]]
    balls = [abi.BallState.from_buffer_copy(x.tobytes()) for x in g["init_balls"]]
    return cars, balls, g["init_vehicle"], g["controls"], g["traj"], g["vehicle"]


def state_vectors(cars, balls, vehicle) -> np.ndarray:
    """[n, 39] Bullet-unit states (float32 multiply by UU_TO_BT, as Car::SetState does)."""
    out = np.zeros((len(cars), STATE), np.float32)
    for i, (c, b) in enumerate(zip(cars, balls)):
        r = c.rot_mat
        out[i, 0:3] = np.array([c.pos.x, c.pos.y, c.pos.z], np.float32) * U
        out[i, 3:6] = np.array([c.vel.x, c.vel.y, c.vel.z], np.float32) * U
        out[i, 6:9] = [c.ang_vel.x, c.ang_vel.y, c.ang_vel.z]
        out[i, 9:18] = [r.forward.x, r.right.x, r.up.x, r.forward.y, r.right.y, r.up.y,
                        r.forward.z, r.right.z, r.up.z]
        out[i, 18:33] = vehicle[i]
        out[i, 33:36] = np.array([b.pos.x, b.pos.y, b.pos.z], np.float32) * U
        out[i, 36:39] = np.array([b.vel.x, b.vel.y, b.vel.z], np.float32) * U
    return out


def to_reference_layout(x: np.ndarray) -> np.ndarray:
    """Bullet-unit states [..., 39] -> the golden kinematics layout (uu; forward, right, up)."""
    x = np.asarray(x, np.float64)
    B = x[..., 9:18].reshape(x.shape[:-1] + (3, 3))
    return np.concatenate([x[..., 0:6] * 50.0, x[..., 6:9], B[..., :, 0], B[..., :, 1], B[..., :, 2],
                           x[..., 33:39] * 50.0], axis=-1)


def max_errors(states: np.ndarray, traj: np.ndarray, vehicle: np.ndarray) -> dict:
    """Largest |rollout - golden| per quantity for Bullet-unit states [..., 39]."""
    d = np.abs(to_reference_layout(states) - np.asarray(traj, np.float64))
    vg = np.asarray(vehicle, np.float64)
    scale = np.maximum(1.0, np.abs(vg).reshape(-1, 15).max(axis=0))
    v = np.abs(np.asarray(states, np.float64)[..., 18:33] - vg) / scale
    return dict(pos=max(d[..., 0:3].max(), d[..., 18:21].max()),
                vel=max(d[..., 3:6].max(), d[..., 21:24].max()),
                ang=d[..., 6:9].max(), rot=d[..., 9:18].max(), veh=v.max())


def within(errs: dict, tol: dict) -> bool:
    return all(errs[k] <= tol[k] for k in tol)


def smooth(rng, ticks, lo, hi, knots=4):
    xs = np.linspace(0, ticks - 1, knots)
    return np.interp(np.arange(ticks), xs, rng.uniform(lo, hi, knots))


def gradient_case(seed: int, n: int, ticks: int):
    """Start states from the golden's settled cars with smooth controls inside the ranges
    (throttle 0.3..0.9, steer -0.6..0.6, boost 0.2..0.8) and a drive_loss target near where the
    rollout ends: (state0 [n, 39], controls [ticks, n, 4], target_xy [n, 2], target_dir [n, 3])."""
    from oracle import ground_fp64 as G
    cars, balls, veh, _, _, _ = load_golden()
    s_all = state_vectors(cars, balls, veh)
    rng = np.random.default_rng(seed)
    idx = rng.choice(s_all.shape[0], n, replace=n > s_all.shape[0])
    s0 = s_all[idx].copy()
    u = np.zeros((ticks, n, 4), np.float32)
    for i in range(n):
        u[:, i, 0] = smooth(rng, ticks, 0.3, 0.9)
        u[:, i, 1] = smooth(rng, ticks, -0.6, 0.6)
        u[:, i, 2] = smooth(rng, ticks, 0.2, 0.8)
    fin = G.rollout(s0.astype(np.float64), u.astype(np.float64), G.car_geometry(), DT)
    # 50-150 uu from where the rollout ends, so that the float32 rollout's final position (within
    # ~1e-3 uu of the FP64 one) moves the loss gradient by less than 1e-4 of itself
    off_ang = rng.uniform(0, 2 * np.pi, n)
    target_xy = fin[:, 0:2] + np.stack([np.cos(off_ang), np.sin(off_ang)], axis=1) * rng.uniform(1, 3, (n, 1))
    ang = rng.uniform(0, 2 * np.pi, n)
    target_dir = np.stack([np.cos(ang), np.sin(ang), np.zeros(n)], axis=1)
    return s0, u, target_xy, target_dir
