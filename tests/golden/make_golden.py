"""Writes tests/golden/ref_rollouts.npz from the reference RocketSim.

Run here, where the reference sources exist: ``python tests/golden/make_golden.py``.
It builds the reference from its own sources (oracle/Makefile, target ``ref``),
plays seeded scenarios (tests/scenarios.py) through it and stores, per
scenario, the starting state, update order and controls, the full car / ball
state after 1 and 8 ticks, the discrete state (flags, timers, boost, pads)
after every one of 120 ticks, the ball-hit record (its tick counters bit for bit, its
positions and velocity as floats) and tickCountSinceUpdate after every tick, and the goal /
bump events (kind, tick, car ids, demo flag).  The CPU restatement
is played alongside to record the first tick at which the reference needed
Bullet's EPA penetration solver (a narrow-phase path the restatement does not
cover yet); scenarios without one carry epa_tick = -1.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from scenarios import (CONTROLS_DTYPE, cpu_snapshot, discrete_car, discrete_hit, discrete_pads,  # noqa: E402
                       hit_vec, make_carcar_scenario, make_scenario, run_cpu)
from rocketsim_gb300 import abi  # noqa: E402

TICKS = 120
OUT = os.path.join(HERE, "ref_rollouts.npz")


def scenario_list():
    out = [make_scenario(seed) for seed in range(12)]  # 2v2 Octane
    out.append(make_scenario(100, ncars=2, presets=[1, 2]))  # 1v1 Dominus vs Plank
    out.append(make_scenario(101, ncars=6, presets=[0, 1, 2, 3, 4, 5]))  # 3v3, every hitbox
    out.append(make_scenario(102, ncars=4, presets=[3, 4, 5, 0], air_frac=0.0))  # all on the ground
    out.append(make_scenario(103, ncars=4, air_frac=1.0))  # all airborne
    out += [make_carcar_scenario(s) for s in (0, 3, 6, 8)]  # bumps and demolitions
    return out


def record(scs, mutators=None, epa=True, config=None):
    """Plays the scenarios through the reference (and, with `epa`, the restatement to find the
    first EPA tick) and returns the arrays of the golden file."""
    from oracle.pyoracle import build_ref
    if build_ref() is None:
        raise SystemExit("reference sources not found")
    S, MC = len(scs), max(len(s.cars) for s in scs)
    car_dt, ball_dt = np.dtype(abi.CarState), np.dtype(abi.BallState)
    ncars = np.array([len(s.cars) for s in scs], np.int32)
    presets = np.full((S, MC), -1, np.int32)
    teams = np.full((S, MC), -1, np.int32)
    order = np.full((S, MC), -1, np.int32)
    init_cars = np.zeros((S, MC), car_dt)
    init_ball = np.zeros(S, ball_dt)
    controls = np.zeros((S, TICKS, MC), CONTROLS_DTYPE)
    cars_t = {1: np.zeros((S, MC), car_dt), 8: np.zeros((S, MC), car_dt)}
    ball_t = {1: np.zeros(S, ball_dt), 8: np.zeros(S, ball_dt)}
    disc_cars = np.zeros((S, TICKS, MC, 28), np.float32)
    disc_hit = np.zeros((S, TICKS, MC, 4), np.uint64)
    hit_cont = np.zeros((S, TICKS, MC, 9), np.float32)
    npads = int(config.num_custom_boost_pads) if config is not None and config.use_custom_boost_pads else 34
    disc_pads = np.zeros((S, TICKS, npads, 3), np.float32)
    events = []
    epa_tick = np.full(S, -1, np.int32)
    for si, sc in enumerate(scs):
        n = len(sc.cars)
        for i in range(n):
            init_cars[si, i] = np.frombuffer(bytes(sc.cars[i]), car_dt)[0]
        init_ball[si] = np.frombuffer(bytes(sc.ball), ball_dt)[0]
        presets[si, :n] = sc.presets
        teams[si, :n] = sc.teams
        controls[si, :, :n] = sc.controls

        def rec(t, a, ids):
            cars, ball, pads = cpu_snapshot(a, ids)
            if t + 1 in cars_t:
                cars_t[t + 1][si, :n] = cars
                ball_t[t + 1][si] = ball[0]
            disc_cars[si, t, :n] = discrete_car(cars)
            disc_hit[si, t, :n] = discrete_hit(cars)
            hit_cont[si, t, :n] = hit_vec(cars)
            disc_pads[si, t] = discrete_pads(pads)
            for e in a.pop_events():
                events.append((si,) + e)
        a, ids = run_cpu("ref", sc, TICKS, rec, mutators, config)  # fixes sc.order to the reference's order
        a.close()
        order[si, :n] = sc.order
        if epa:
            def rec_oracle(t, a, ids):
                if epa_tick[si] < 0 and a.counters()[3] > 0:
                    epa_tick[si] = t
            o, _ = run_cpu("oracle", sc, TICKS, rec_oracle)
            o.close()
        print(f"scenario {si}: seed {sc.seed} cars {n} epa_tick {epa_tick[si]}")
    return dict(seeds=np.array([s.seed for s in scs]), ncars=ncars, presets=presets, teams=teams, order=order,
                init_cars=init_cars, init_ball=init_ball, controls=controls, cars_t1=cars_t[1], ball_t1=ball_t[1],
                cars_t8=cars_t[8], ball_t8=ball_t[8], disc_cars=disc_cars, disc_pads=disc_pads,
                disc_hit=disc_hit, hit_cont=hit_cont,
                events=np.array(events, np.uint64).reshape(-1, 6), epa_tick=epa_tick, mesh_seed=np.int32(0))


def main():
    np.savez_compressed(OUT, **record(scenario_list()))
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
