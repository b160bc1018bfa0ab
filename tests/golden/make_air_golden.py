"""Writes tests/golden/air_rollouts.npz from the reference RocketSim: airborne cars in THE_VOID.

Run here, where the reference sources exist: ``python tests/golden/make_air_golden.py``.
It builds the reference from its own sources (oracle/Makefile, target ``ref``), places one
airborne car per arena in THE_VOID (nothing to touch, the ball out of reach) with random
orientation, velocity and
angular velocity (some at or above the speed clamps), gives it random pitch / yaw / roll every
tick and a boost input held at 0 or 1 for the whole rollout (the reference keeps boosting for
at least BOOST_MIN_TIME once started, so a held input is the case where the relaxed boost of
the air rollout and the arena agree), and records the car and ball kinematics after every tick.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from scenarios import mesh_bytes, rot_cols, set_rot  # noqa: E402
from rocketsim_gb300 import abi  # noqa: E402

N = 24
TICKS = 60
SEED = 2024
OUT = os.path.join(HERE, "air_rollouts.npz")


def make_instances(seed: int = SEED, n: int = N, ticks: int = TICKS):
    """Initial CarState / BallState per instance and controls [ticks, n, 4] (pitch, yaw, roll, boost)."""
    rng = np.random.default_rng(seed)
    cars, balls = [], []
    for i in range(n):
        s = abi.CarState()
        s.ball_hit_info.tick_count_when_hit = (1 << 64) - 1
        s.ball_hit_info.tick_count_when_extra_impulse_applied = (1 << 64) - 1
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        set_rot(s.rot_mat, rot_cols(q))
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        speed = 2300.0 if i % 6 == 0 else rng.uniform(0, 2300)
        v = d * speed
        w = rng.uniform(-3, 3, 3)
        if i % 6 == 1:
            w *= 5.6 / np.linalg.norm(w)
        s.pos = abi.Vec3(*map(float, rng.uniform(-3000, 3000, 3)))
        s.vel = abi.Vec3(*map(float, v))
        s.ang_vel = abi.Vec3(*map(float, w))
        s.is_on_ground = 0
        s.has_jumped = 1
        s.boost = 100.0
        cars.append(s)
        b = abi.BallState()
        # the ball starts 4500..6000 uu away: closing speeds stay under 8300 uu/s, so in 0.5 s
        # neither the car's body nor its wheel rays can reach it
        off = rng.normal(size=3)
        off *= rng.uniform(4500, 6000) / np.linalg.norm(off)
        b.pos = abi.Vec3(*map(float, np.array([s.pos.x, s.pos.y, s.pos.z]) + off))
        set_rot(b.rot_mat, np.eye(3))
        bd = rng.normal(size=3)
        bd /= np.linalg.norm(bd)
        b.vel = abi.Vec3(*map(float, bd * (6000.0 if i % 6 == 2 else rng.uniform(0, 3000))))
        b.ang_vel = abi.Vec3(*map(float, rng.uniform(-2, 2, 3)))
        balls.append(b)
    controls = rng.uniform(-1, 1, (ticks, n, 4)).astype(np.float32)
    controls[:, :, 3] = (np.arange(n) % 2)[None, :]
    return cars, balls, controls


def kinematics(car: abi.CarState, ball: abi.BallState) -> np.ndarray:
    """pos, vel, ang_vel, forward, right, up of the car, then pos, vel of the ball (uu), 24 floats."""
    r = car.rot_mat
    return np.array([car.pos.x, car.pos.y, car.pos.z, car.vel.x, car.vel.y, car.vel.z,
                     car.ang_vel.x, car.ang_vel.y, car.ang_vel.z,
                     r.forward.x, r.forward.y, r.forward.z, r.right.x, r.right.y, r.right.z,
                     r.up.x, r.up.y, r.up.z,
                     ball.pos.x, ball.pos.y, ball.pos.z, ball.vel.x, ball.vel.y, ball.vel.z], np.float32)


def main():
    from oracle.pyoracle import SimArena, build_ref, CarState as OCarState, BallState as OBallState, \
        CarControls as OCtl
    if build_ref() is None:
        raise SystemExit("reference sources not found")
    cars, balls, controls = make_instances()
    SimArena("ref", mesh_bytes()).close()  # RocketSim::Init, which every arena needs (even THE_VOID)
    traj = np.zeros((TICKS, N, 24), np.float32)
    for i in range(N):
        a = SimArena("ref", None, game_mode=abi.GAMEMODE_THE_VOID)
        cid = a.add_car(0, abi.CAR_OCTANE)
        a.set_car(cid, OCarState.from_buffer_copy(bytes(cars[i])))
        a.set_ball(OBallState.from_buffer_copy(bytes(balls[i])))
        for t in range(TICKS):
            c = OCtl()
            c.pitch, c.yaw, c.roll = (float(x) for x in controls[t, i, :3])
            c.boost = int(controls[t, i, 3])
            a.set_controls(cid, c)
            a.step(1)
            traj[t, i] = kinematics(a.get_car(cid), a.get_ball())
        a.close()
    car_dt, ball_dt = np.dtype(abi.CarState), np.dtype(abi.BallState)
    np.savez_compressed(
        OUT, seed=np.int32(SEED),
        init_cars=np.frombuffer(b"".join(bytes(c) for c in cars), car_dt),
        init_balls=np.frombuffer(b"".join(bytes(b) for b in balls), ball_dt),
        controls=controls, traj=traj)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
