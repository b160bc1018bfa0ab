"""Shared cases for the air-rollout tests: the reference golden rollouts and random gradient cases."""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
if REPO not in sys.path:
    sys.path.insert(0, REPO)

from rocketsim_gb300 import abi  # noqa: E402

GOLDEN = os.path.join(HERE, "golden", "air_rollouts.npz")
OCTANE_HITBOX = (120.507, 86.6994, 38.6591)
DT = 1.0 / 120.0
U = np.float32(1.0 / 50.0)

# |float rollout - reference| bounds (uu, uu/s, rad/s, basis entries) after 1, 8 and 60 ticks;
# the reference golden stores float32, its uu conversion alone rounds pos/vel by ~1e-4.
TOL = {1: dict(pos=1e-3, vel=2e-3, ang=1e-4, rot=1e-5),
       8: dict(pos=1e-2, vel=2e-2, ang=1e-3, rot=1e-4),
       60: dict(pos=5e-2, vel=5e-2, ang=1e-3, rot=1e-3)}


def load_golden():
    g = np.load(GOLDEN)
    cars = [abi.CarState.from_buffer_copy(x.tobytes()) for x in g["init_cars"]]
    balls = [abi.BallState.from_buffer_copy(x.tobytes()) for x in g["init_balls"]]
    return cars, balls, g["controls"], g["traj"]


def state_vectors(cars, balls) -> np.ndarray:
    """[n, 24] Bullet-unit states (float32 multiply by UU_TO_BT, as Car::SetState does)."""
    out = np.zeros((len(cars), 24), np.float32)
    for i, (c, b) in enumerate(zip(cars, balls)):
        r = c.rot_mat
        out[i, 0:3] = np.array([c.pos.x, c.pos.y, c.pos.z], np.float32) * U
        out[i, 3:6] = np.array([c.vel.x, c.vel.y, c.vel.z], np.float32) * U
        out[i, 6:9] = [c.ang_vel.x, c.ang_vel.y, c.ang_vel.z]
        out[i, 9:18] = [r.forward.x, r.right.x, r.up.x, r.forward.y, r.right.y, r.up.y,
                        r.forward.z, r.right.z, r.up.z]
        out[i, 18:21] = np.array([b.pos.x, b.pos.y, b.pos.z], np.float32) * U
        out[i, 21:24] = np.array([b.vel.x, b.vel.y, b.vel.z], np.float32) * U
    return out


def to_reference_layout(x: np.ndarray) -> np.ndarray:
    """Bullet-unit states [..., 24] -> the golden layout (uu; forward, right, up columns)."""
    x = np.asarray(x, np.float64)
    B = x[..., 9:18].reshape(x.shape[:-1] + (3, 3))
    return np.concatenate([x[..., 0:6] * 50.0, x[..., 6:9], B[..., :, 0], B[..., :, 1], B[..., :, 2],
                           x[..., 18:24] * 50.0], axis=-1)


def max_errors(a: np.ndarray, b: np.ndarray) -> dict:
    """Largest |a - b| per quantity, golden layout."""
    d = np.abs(np.asarray(a, np.float64) - np.asarray(b, np.float64))
    return dict(pos=max(d[..., 0:3].max(), d[..., 18:21].max()),
                vel=max(d[..., 3:6].max(), d[..., 21:24].max()),
                ang=d[..., 6:9].max(), rot=d[..., 9:18].max())


def within(errs: dict, tol: dict) -> bool:
    return all(errs[k] <= tol[k] for k in tol)


def random_rotations(rng: np.random.Generator, n: int) -> np.ndarray:
    """[n, 3, 3] rotation matrices from uniform random unit quaternions."""
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    x, y, z, w = q.T
    M = np.empty((n, 3, 3))
    M[:, 0] = np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)], 1)
    M[:, 1] = np.stack([2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)], 1)
    M[:, 2] = np.stack([2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], 1)
    return M


def gradient_case(seed: int, n: int, ticks: int, fast: bool = False):
    """Random airborne states (Bullet units, float32-representable) and controls away from the
    kinks of the tick (|pitch|, |yaw|, |roll| in [0.05, 0.95], boost in [0.05, 0.95]).  With
    `fast`, the car starts at the speed clamps (|v| = 2300 uu/s, |w| = 5.6 rad/s)."""
    rng = np.random.default_rng(seed)
    s = np.zeros((n, 24))
    s[:, 0:3] = rng.uniform(-60, 60, (n, 3))
    v = rng.normal(size=(n, 3))
    w = rng.normal(size=(n, 3))
    if fast:
        s[:, 3:6] = v / np.linalg.norm(v, axis=1, keepdims=True) * 46.0
        s[:, 6:9] = w / np.linalg.norm(w, axis=1, keepdims=True) * 5.6
    else:
        s[:, 3:6] = v * 15.0
        s[:, 6:9] = w * 1.5
    s[:, 9:18] = random_rotations(rng, n).reshape(n, 9)
    s[:, 18:21] = s[:, 0:3] + rng.uniform(-30, 30, (n, 3))
    s[:, 21:24] = rng.normal(size=(n, 3)) * 20.0
    u = rng.uniform(0.05, 0.95, (ticks, n, 4)) * rng.choice([-1.0, 1.0], (ticks, n, 4))
    u[..., 3] = np.abs(u[..., 3])
    target = random_rotations(rng, n)
    return s.astype(np.float32), u.astype(np.float32), target
