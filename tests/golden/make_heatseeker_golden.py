"""Writes tests/golden/heatseeker_rollouts.npz from the reference RocketSim in GameMode::HEATSEEKER
(the soccar arena: the procedural mesh, its pads and goals; infinite boost).

Ten arenas, 120 ticks each, played through the reference built from its own sources:

* ``hit``: 4 arenas whose cars drive into a ball at rest; the first touch gives the ball a target net
  (Ball::_OnHit), after which it seeks that net (Ball::_PreTickUpdate);
* ``kickoff``: 4 arenas reset by Arena::ResetToRandomKickoff(seed) before the first tick (heatseeker's
  four kickoff spots, the ball popping up on the side the engine picks), cars at full throttle and
  boost for 60 ticks, then the 2v2 input process;
* ``bounce``: 2 arenas whose ball already seeks a net and flies at the back wall beside it
  (Ball::_OnWorldCollision turns the target around and adds the bounce impulse).

Per arena: the starting state and heatseeker state, the reference's car order, the controls, the
reset seed, the full car / ball state after ticks 1 and 8, after every tick the discrete car state,
the ball-hit record, the pads, the ball state and its heatseeker state, and the goal / bump events.
Run from the repository root: ``python tests/golden/make_heatseeker_golden.py``.
"""
from __future__ import annotations

import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from scenarios import (CONTROLS_DTYPE, _controls_struct, control_sequence, cpu_snapshot, discrete_car,  # noqa: E402
                       discrete_hit, discrete_pads, hit_vec, make_scenario, rot_cols, set_rot, setup_cpu)
from rocketsim_gb300 import abi  # noqa: E402

TICKS = 120
SNAP = (1, 8)
HEATSEEKER = 2
OUT = os.path.join(HERE, "heatseeker_rollouts.npz")


def hit_scenarios():
    out = []
    rng = np.random.default_rng(808)
    for k in range(4):
        sc = make_scenario(900 + k, ncars=2 + 2 * (k % 2), air_frac=0.0, random_order=False)
        bx, by = rng.uniform(-2000, 2000), rng.uniform(-3000, 3000)
        sc.ball.pos = abi.Vec3(float(bx), float(by), 93.15)
        sc.ball.vel = abi.Vec3(0.0, 0.0, 0.0)
        sc.ball.ang_vel = abi.Vec3(0.0, 0.0, 0.0)
        for i, s in enumerate(sc.cars):
            ang = rng.uniform(0, 2 * math.pi)
            d = rng.uniform(300, 900)
            M = rot_cols((math.cos(ang / 2), 0.0, 0.0, math.sin(ang / 2)))
            set_rot(s.rot_mat, M)
            sp = rng.uniform(600, 1600)
            s.pos = abi.Vec3(float(bx - d * math.cos(ang)), float(by - d * math.sin(ang)), 17.0)
            s.vel = abi.Vec3(float(M[0, 0] * sp), float(M[1, 0] * sp), 0.0)
            s.ang_vel = abi.Vec3(0.0, 0.0, 0.0)
            s.boost = 100.0
        sc.controls["throttle"] = 1.0
        sc.controls["steer"] = 0.0
        sc.controls["jump"] = 0
        sc.controls["handbrake"] = 0
        sc.controls["boost"][:40] = 1
        out.append((sc, -1, (0.0, 2900.0, 0.0)))
    return out


def kickoff_scenarios():
    out = []
    for k in range(4):
        n = 2 + 2 * (k % 2)
        sc = make_scenario(950 + k, ncars=n, air_frac=0.0, random_order=False)
        rng = np.random.default_rng(960 + k)
        ctl = control_sequence(rng, TICKS, n)
        ctl["throttle"][:60] = 1.0
        ctl["steer"][:60] = 0.0
        ctl["boost"][:60] = 1
        ctl["jump"][:60] = 0
        ctl["handbrake"][:60] = 0
        sc.controls = ctl
        out.append((sc, 31 + 7 * k, (0.0, 2900.0, 0.0)))
    return out


def bounce_scenarios():
    out = []
    for k, side in enumerate((1.0, -1.0)):
        sc = make_scenario(990 + k, ncars=2, air_frac=0.0, random_order=False)
        sc.ball.pos = abi.Vec3(2500.0 * side, 4300.0 * side, 400.0)
        sc.ball.vel = abi.Vec3(-300.0 * side, 3500.0 * side, 200.0)
        sc.ball.ang_vel = abi.Vec3(0.0, 0.0, 0.0)
        for i, s in enumerate(sc.cars):  # far away on the other half, idle
            s.pos = abi.Vec3(-1500.0 + 3000.0 * i, -3000.0 * side, 17.0)
            s.vel = abi.Vec3(0.0, 0.0, 0.0)
        sc.controls[:] = np.zeros_like(sc.controls)
        out.append((sc, -1, (side, 3500.0, 0.4)))
    return out


def record(items):
    from oracle.pyoracle import CarControls as OCtl
    S = len(items)
    scs = [it[0] for it in items]
    MC = max(len(s.cars) for s in scs)
    car_dt, ball_dt = np.dtype(abi.CarState), np.dtype(abi.BallState)
    z = dict(
        seeds=np.array([s.seed for s in scs]), ncars=np.array([len(s.cars) for s in scs], np.int32),
        presets=np.full((S, MC), -1, np.int32), teams=np.full((S, MC), -1, np.int32),
        order=np.full((S, MC), -1, np.int32), init_cars=np.zeros((S, MC), car_dt), init_ball=np.zeros(S, ball_dt),
        init_hs=np.array([it[2] for it in items], np.float32),
        controls=np.zeros((S, TICKS, MC), CONTROLS_DTYPE),
        reset_seed=np.array([it[1] for it in items], np.int64),
        disc_cars=np.zeros((S, TICKS, MC, 28), np.float32), disc_hit=np.zeros((S, TICKS, MC, 4), np.uint64),
        hit_cont=np.zeros((S, TICKS, MC, 9), np.float32), disc_pads=np.zeros((S, TICKS, 34, 3), np.float32),
        balls=np.zeros((S, TICKS), ball_dt), hs=np.zeros((S, TICKS, 3), np.float32))
    for t in SNAP:
        z[f"cars_t{t}"] = np.zeros((S, MC), car_dt)
        z[f"ball_t{t}"] = np.zeros(S, ball_dt)
    events = []
    for si, (sc, seed, hs) in enumerate(items):
        n = len(sc.cars)
        for i in range(n):
            z["init_cars"][si, i] = np.frombuffer(bytes(sc.cars[i]), car_dt)[0]
        z["init_ball"][si] = np.frombuffer(bytes(sc.ball), ball_dt)[0]
        z["presets"][si, :n] = sc.presets
        z["teams"][si, :n] = sc.teams
        z["controls"][si, :, :n] = sc.controls
        a, ids = setup_cpu("ref", sc, game_mode=HEATSEEKER)
        z["order"][si, :n] = sc.order
        a.set_ball_heatseeker(hs)
        if seed >= 0:
            a.reset_to_random_kickoff(int(seed))
        for t in range(TICKS):
            for i, cid in enumerate(ids):
                a.set_controls(cid, OCtl.from_buffer_copy(bytes(_controls_struct(sc.controls[t, i]))))
            a.step(1)
            cars, ball, pads = cpu_snapshot(a, ids)
            if t + 1 in SNAP:
                z[f"cars_t{t + 1}"][si, :n] = cars
                z[f"ball_t{t + 1}"][si] = ball[0]
            z["disc_cars"][si, t, :n] = discrete_car(cars)
            z["disc_hit"][si, t, :n] = discrete_hit(cars)
            z["hit_cont"][si, t, :n] = hit_vec(cars)
            z["disc_pads"][si, t] = discrete_pads(pads)
            z["balls"][si, t] = ball[0]
            z["hs"][si, t] = a.ball_heatseeker()
            for e in a.pop_events():
                events.append((si,) + e)
        a.close()
    z["events"] = np.array(events, np.uint64).reshape(-1, 6)
    return z


def main():
    from oracle.pyoracle import build_ref
    if build_ref() is None:
        raise SystemExit("reference sources not found")
    items = hit_scenarios() + kickoff_scenarios() + bounce_scenarios()
    z = record(items)
    hs = z["hs"]
    print("arenas", len(items), "events", len(z["events"]),
          "ticks with a target", int((hs[..., 0] != 0).sum()), "target flips",
          int((np.diff(np.sign(hs[..., 0]), axis=1) != 0).sum()))
    z["mesh_seed"] = np.int32(0)
    np.savez_compressed(OUT, **{f"hs_{k}": v for k, v in z.items()})
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
