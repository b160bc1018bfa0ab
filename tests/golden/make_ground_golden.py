"""Writes tests/golden/ground_rollouts.npz from the reference RocketSim: cars driving on the floor.

Run here, where the reference sources exist: ``python tests/golden/make_ground_golden.py``.
It builds the reference from its own sources (oracle/Makefile, target ``ref``), puts one Octane
per soccar arena (the seeded stand-in mesh of rocketsim_gb300.arena_mesh) on the floor near the
centre with a random heading and forward speed, lets it settle for SETTLE ticks, then records the
start state (CarState plus the vehicle state CarState leaves out: steer angle, engine force,
brake, friction factors and push-backs; every third car then gets a downward kick of 150-250 uu/s
that compresses its suspension past the push-back threshold) and drives TICKS more ticks under smooth random throttle
and steer with a boost input held at 0 or 1 for the whole rollout.  Throttle patterns cover
forward driving, coasting (throttle 0), braking against the motion and reversing.  The ball
flies far away in the air (with a nonzero velocity: Arena::Step puts a ball at exactly zero
velocity to sleep, Arena.cpp:693-699, which the rollouts' ball does not model).  An instance whose car leaves the flat part of the floor or loses a
wheel contact is redrawn, so every recorded tick is inside the ground-driving model.
"""
from __future__ import annotations

import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from scenarios import mesh_bytes, rot_cols, set_rot  # noqa: E402
from rocketsim_gb300 import abi  # noqa: E402

N = 24
SETTLE = 24
TICKS = 120
SEED = 4242
OUT = os.path.join(HERE, "ground_rollouts.npz")


def smooth(rng, ticks, lo, hi, knots=5):
    """A piecewise-linear random signal in [lo, hi] through `knots` random values."""
    xs = np.linspace(0, ticks - 1, knots)
    return np.interp(np.arange(ticks), xs, rng.uniform(lo, hi, knots))


def controls_for(rng, i, ticks):
    """[ticks, 4]: throttle, steer, boost, 0.  Pattern by instance: forward driving, coasting,
    braking then reversing, full throttle."""
    u = np.zeros((ticks, 4), np.float32)
    kind = i % 4
    if kind == 0:
        u[:, 0] = smooth(rng, ticks, 0.2, 1.0)
    elif kind == 1:
        u[:, 0] = np.where(np.arange(ticks) < ticks // 2, smooth(rng, ticks, 0.3, 1.0), 0.0)
    elif kind == 2:
        u[:, 0] = np.where(np.arange(ticks) < ticks // 3, 0.6, -smooth(rng, ticks, 0.3, 1.0))
    else:
        u[:, 0] = 1.0
    u[:, 1] = smooth(rng, ticks, -1.0, 1.0)
    u[:, 2] = float((i // 2) % 2) if kind != 2 else 0.0
    return u


def kinematics(car, ball) -> np.ndarray:
    """pos, vel, ang_vel, forward, right, up of the car, then pos, vel of the ball (uu), 24 floats."""
    r = car.rot_mat
    return np.array([car.pos.x, car.pos.y, car.pos.z, car.vel.x, car.vel.y, car.vel.z,
                     car.ang_vel.x, car.ang_vel.y, car.ang_vel.z,
                     r.forward.x, r.forward.y, r.forward.z, r.right.x, r.right.y, r.right.z,
                     r.up.x, r.up.y, r.up.z,
                     ball.pos.x, ball.pos.y, ball.pos.z, ball.vel.x, ball.vel.y, ball.vel.z], np.float32)


def run_instance(SimArena, OCarState, OBallState, OCtl, rng, i):
    a = SimArena("ref", mesh_bytes())
    cid = a.add_car(0, abi.CAR_OCTANE)
    s = abi.CarState.from_buffer_copy(bytes(a.get_car(cid)))
    yaw = rng.uniform(0, 2 * math.pi)
    set_rot(s.rot_mat, rot_cols((math.cos(yaw / 2), 0.0, 0.0, math.sin(yaw / 2))))
    speed = rng.uniform(0, 1200) if i % 4 != 2 else rng.uniform(600, 1200)
    s.pos = abi.Vec3(float(rng.uniform(-800, 800)), float(rng.uniform(-800, 800)), 17.0)
    s.vel = abi.Vec3(float(speed * math.cos(yaw)), float(speed * math.sin(yaw)), 0.0)
    s.ang_vel = abi.Vec3(0.0, 0.0, 0.0)
    s.boost = 100.0
    a.set_car(cid, OCarState.from_buffer_copy(bytes(s)))
    b = abi.BallState.from_buffer_copy(bytes(a.get_ball()))
    b.pos = abi.Vec3(2500.0, -3500.0, 1200.0)
    b.vel = abi.Vec3(float(rng.uniform(-300, 300)), float(rng.uniform(-300, 300)), float(rng.uniform(0, 300)))
    b.ang_vel = abi.Vec3(0.0, 0.0, 0.0)
    a.set_ball(OBallState.from_buffer_copy(bytes(b)))
    u = controls_for(rng, i, TICKS)
    c = OCtl()
    c.throttle = float(u[0, 0])
    a.set_controls(cid, c)
    a.step(SETTLE)
    if i % 3 == 2:  # a downward kick that compresses the suspension past the push-back threshold
        s = abi.CarState.from_buffer_copy(bytes(a.get_car(cid)))
        s.vel.z = float(-rng.uniform(150, 250))
        a.set_car(cid, OCarState.from_buffer_copy(bytes(s)))
    car0, ball0 = a.get_car(cid), a.get_ball()
    veh0 = np.array(a.vehicle_state(cid), np.float32)
    ok = all(car0.wheels_with_contact)
    traj = np.zeros((TICKS, 24), np.float32)
    veh = np.zeros((TICKS, 15), np.float32)
    for t in range(TICKS):
        c = OCtl()
        c.throttle, c.steer = float(u[t, 0]), float(u[t, 1])
        c.boost = int(u[t, 2])
        a.set_controls(cid, c)
        a.step(1)
        car = a.get_car(cid)
        traj[t] = kinematics(car, a.get_ball())
        veh[t] = a.vehicle_state(cid)
        ok = ok and all(car.wheels_with_contact) and abs(car.pos.x) < 3500 and abs(car.pos.y) < 4500
    a.close()
    return ok, car0, ball0, veh0, u, traj, veh


def main():
    from oracle.pyoracle import SimArena, build_ref, CarState as OCarState, BallState as OBallState, \
        CarControls as OCtl
    if build_ref() is None:
        raise SystemExit("reference sources not found")
    rng = np.random.default_rng(SEED)
    cars, balls, veh0s, ctls, trajs, vehs = [], [], [], [], [], []
    redrawn = 0
    while len(cars) < N:
        ok, car0, ball0, veh0, u, traj, veh = run_instance(SimArena, OCarState, OBallState, OCtl, rng, len(cars))
        if not ok:
            redrawn += 1
            continue
        cars.append(abi.CarState.from_buffer_copy(bytes(car0)))
        balls.append(abi.BallState.from_buffer_copy(bytes(ball0)))
        veh0s.append(veh0)
        ctls.append(u)
        trajs.append(traj)
        vehs.append(veh)
    car_dt, ball_dt = np.dtype(abi.CarState), np.dtype(abi.BallState)
    np.savez_compressed(
        OUT, seed=np.int32(SEED), settle=np.int32(SETTLE),
        init_cars=np.frombuffer(b"".join(bytes(c) for c in cars), car_dt),
        init_balls=np.frombuffer(b"".join(bytes(b) for b in balls), ball_dt),
        init_vehicle=np.stack(veh0s), controls=np.stack(ctls, axis=1),
        traj=np.stack(trajs, axis=1), vehicle=np.stack(vehs, axis=1))
    print("wrote", OUT, os.path.getsize(OUT), "bytes;", redrawn, "instances redrawn")


if __name__ == "__main__":
    main()
