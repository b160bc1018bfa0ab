"""Writes tests/golden/workload_rollouts.npz from the reference RocketSim.

Three groups of arenas, each played 120 ticks through the reference built from its own
sources (oracle/Makefile, target ``ref``):

* ``bench``: 64 arenas of the batched uniform 2v2 workload that bench.py times (its
  initial_states and ControlProcess for 4096 arenas with the same seeds; every 64th arena);
* ``uneven``: 48 arenas of the uneven workload (bench.uneven_layout: 2, 4 or 6 cars of all six
  hitboxes; initial_states and ControlProcess for 16384 arenas; every 341st arena), every third
  of them reset by Arena::ResetToRandomKickoff(seed) after tick 60;
* ``hits``: 8 arenas whose cars drive into the ball (two of them next to a goal), for the
  ball-hit record, the goal and bump events.

Per arena it stores the starting state, the reference's car update order, the controls, the
resets, the full car / ball state after ticks 1, 8, 61 and 68, the discrete car state, the
ball-hit record and the pads after every tick, and the goal / bump events.  Run from the
repository root: ``python tests/golden/make_workload_golden.py``.
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

from scenarios import (CONTROLS_DTYPE, Scenario, _controls_struct, cpu_snapshot, discrete_car,  # noqa: E402
                       discrete_hit, discrete_pads, hit_vec, make_scenario, rot_cols, set_rot, setup_cpu)
from rocketsim_gb300 import abi  # noqa: E402

TICKS = 120
SNAP = (1, 8, 61, 68)
RESET_AFTER = 60
OUT = os.path.join(HERE, "workload_rollouts.npz")


def _scenarios_from_bench(A: int, mc: int, pick, counts=None, presets=None):
    import bench
    car_dt, ball_dt = np.dtype(abi.CarState), np.dtype(abi.BallState)
    cars, balls = bench.initial_states(A, 1234, car_dt, ball_dt, cars_per_arena=mc)
    proc = bench.ControlProcess(A * mc, 99, CONTROLS_DTYPE)
    ctl = np.stack([proc.tick() for _ in range(TICKS)])  # [T, A * mc]
    out = []
    for a in pick:
        n = mc if counts is None else int(counts[a])
        cs = [abi.CarState.from_buffer_copy(cars[a * mc + i].tobytes()) for i in range(n)]
        ball = abi.BallState.from_buffer_copy(balls[a].tobytes())
        pr = [0] * n if presets is None else [int(p) for p in presets[a][:n]]
        out.append(Scenario(int(a), pr, [i % 2 for i in range(n)], cs, ball, list(range(n)),
                            ctl[:, a * mc:a * mc + n].copy()))
    return out


def bench_group():
    return _scenarios_from_bench(4096, 4, range(0, 4096, 64)), {}


def uneven_group():
    import bench
    counts, presets = bench.uneven_layout(16384, 77)
    pick = list(range(0, 16384, 341))[:48]
    scs = _scenarios_from_bench(16384, 6, pick, counts, presets)
    resets = {k: 1000 + k for k in range(0, len(scs), 3)}
    return scs, resets


def hit_group():
    out = []
    rng = np.random.default_rng(505)
    for k in range(8):
        near_goal = k >= 6
        sc = make_scenario(700 + k, ncars=2 + 2 * (k % 2), air_frac=0.0, random_order=False)
        bx, by = (rng.uniform(-800, 800), 4650.0 if k == 6 else -4650.0) if near_goal else \
            (rng.uniform(-2500, 2500), rng.uniform(-3500, 3500))
        sc.ball.pos = abi.Vec3(float(bx), float(by), 93.15)
        sc.ball.vel = abi.Vec3(0.0, 0.0, 0.0)
        sc.ball.ang_vel = abi.Vec3(0.0, 0.0, 0.0)
        for i, s in enumerate(sc.cars):
            if near_goal:  # behind the ball, towards the goal
                ang = (math.pi / 2 if by > 0 else -math.pi / 2) + rng.uniform(-0.3, 0.3)
                d = 350 + 250 * i
            else:
                ang = rng.uniform(0, 2 * math.pi)
                d = rng.uniform(300, 900)
            x, y = bx - d * math.cos(ang), by - d * math.sin(ang)
            M = rot_cols((math.cos(ang / 2), 0.0, 0.0, math.sin(ang / 2)))
            set_rot(s.rot_mat, M)
            sp = rng.uniform(600, 1600)
            s.pos = abi.Vec3(float(x), float(y), 17.0)
            s.vel = abi.Vec3(float(M[0, 0] * sp), float(M[1, 0] * sp), 0.0)
            s.ang_vel = abi.Vec3(0.0, 0.0, 0.0)
        sc.controls["throttle"] = 1.0
        sc.controls["steer"] = 0.0
        sc.controls["jump"] = 0
        sc.controls["handbrake"] = 0
        sc.controls["boost"][:40] = 1
        out.append(sc)
    return out, {}


def record(scs, resets):
    S, MC = len(scs), max(len(s.cars) for s in scs)
    car_dt, ball_dt = np.dtype(abi.CarState), np.dtype(abi.BallState)
    z = dict(
        seeds=np.array([s.seed for s in scs]), ncars=np.array([len(s.cars) for s in scs], np.int32),
        presets=np.full((S, MC), -1, np.int32), teams=np.full((S, MC), -1, np.int32),
        order=np.full((S, MC), -1, np.int32), init_cars=np.zeros((S, MC), car_dt), init_ball=np.zeros(S, ball_dt),
        controls=np.zeros((S, TICKS, MC), CONTROLS_DTYPE),
        reset_seed=np.array([resets.get(si, -1) for si in range(S)], np.int64),
        disc_cars=np.zeros((S, TICKS, MC, 28), np.float32), disc_hit=np.zeros((S, TICKS, MC, 4), np.uint64),
        hit_cont=np.zeros((S, TICKS, MC, 9), np.float32), disc_pads=np.zeros((S, TICKS, 34, 3), np.float32))
    for t in SNAP:
        z[f"cars_t{t}"] = np.zeros((S, MC), car_dt)
        z[f"ball_t{t}"] = np.zeros(S, ball_dt)
    events = []
    from oracle.pyoracle import CarControls as OCtl
    for si, sc in enumerate(scs):
        n = len(sc.cars)
        for i in range(n):
            z["init_cars"][si, i] = np.frombuffer(bytes(sc.cars[i]), car_dt)[0]
        z["init_ball"][si] = np.frombuffer(bytes(sc.ball), ball_dt)[0]
        z["presets"][si, :n] = sc.presets
        z["teams"][si, :n] = sc.teams
        z["controls"][si, :, :n] = sc.controls
        a, ids = setup_cpu("ref", sc)  # sets sc.order to the reference's own car order
        z["order"][si, :n] = sc.order
        for t in range(TICKS):
            if t == RESET_AFTER and si in resets:
                a.reset_to_random_kickoff(int(resets[si]))
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
            for e in a.pop_events():
                events.append((si,) + e)
        a.close()
    z["events"] = np.array(events, np.uint64).reshape(-1, 6)
    return z


def main():
    from oracle.pyoracle import build_ref
    if build_ref() is None:
        raise SystemExit("reference sources not found")
    out = {}
    for name, (scs, resets) in (("bench", bench_group()), ("uneven", uneven_group()), ("hits", hit_group())):
        z = record(scs, resets)
        hits = int(sum(((z["disc_hit"][si, t, :, 1] == t) & (z["disc_hit"][si, t, :, 0] == 1)).sum()
                       for si in range(len(scs)) for t in range(TICKS)))
        print(f"{name}: {len(scs)} arenas, {len(z['events'])} events, {hits} car-ticks with a ball hit")
        out.update({f"{name}_{k}": v for k, v in z.items()})
    out["mesh_seed"] = np.int32(0)
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
