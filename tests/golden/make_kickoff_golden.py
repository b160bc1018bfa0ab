"""Writes tests/golden/kickoff_goal.npz from the reference RocketSim:

* Arena::ResetToRandomKickoff(seed) on soccar arenas with 1 to 8 cars (both teams, uneven teams,
  shuffled update orders), after the cars have driven for 10 ticks: every car state, the ball and
  the pads afterwards;
* Arena::IsBallProbablyGoingIn(maxTime, extraMargin) for 3000 ball states (most of them moving
  towards a goal, some with no y velocity) and three (maxTime, extraMargin) pairs: the answer and
  the goal's team.

Run from the repository root with the reference library built (make -C oracle ref).
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from scenarios import mesh_bytes  # noqa: E402

OUT = os.path.join(HERE, "kickoff_goal.npz")
# (teams in the order the cars are added, seed); the reference's own car order (its hash-set
# order, which decides who takes which kickoff spot) is recorded
CASES = [
    ([0, 1], 0),
    ([0, 1, 0, 1], 1),
    ([0, 0, 1, 1], 7),
    ([0, 1, 0, 1, 0, 1], 42),
    ([0, 0, 0, 1], 123456),
    ([1, 1, 1], 2147483646),
    ([0, 1, 0, 1, 0, 1, 0, 1], 99),
    ([0, 0, 0, 0, 0, 0, 0, 1], 5),
    ([0, 1, 1, 0], -5),
    ([0, 1], 2147483647),
]
PAIRS = [(2.0, 0.0), (0.5, 0.0), (4.0, 100.0)]
N_BALLS = 3000


def ball_states(n: int, dt) -> np.ndarray:
    rng = np.random.default_rng(77)
    b = np.zeros(n, dt)
    b["pos"]["x"] = rng.uniform(-3500, 3500, n)
    b["pos"]["y"] = rng.uniform(-5000, 5000, n)
    b["pos"]["z"] = rng.uniform(93, 1500, n)
    b["vel"]["x"] = rng.uniform(-1500, 1500, n)
    b["vel"]["y"] = rng.uniform(-4000, 4000, n)
    b["vel"]["z"] = rng.uniform(-1500, 1500, n)
    b["vel"]["y"][::50] = 0.0
    b["vel"]["y"][1::50] = 1e-8
    b["rot_mat"]["forward"]["x"] = b["rot_mat"]["right"]["y"] = b["rot_mat"]["up"]["z"] = 1
    return b


def main():
    from oracle.pyoracle import SimArena, build_ref, BallState as OBall
    from rocketsim_gb300 import abi
    build_ref()
    S, MC = len(CASES), 8
    cars = np.zeros((S, MC, abi.C.sizeof(abi.CarState)), np.uint8)
    balls = np.zeros((S, abi.C.sizeof(abi.BallState)), np.uint8)
    pads = np.zeros((S, 34, abi.C.sizeof(abi.PadState)), np.uint8)
    order = np.full((S, MC), -1, np.int32)
    for si, (teams, seed) in enumerate(CASES):
        a = SimArena("ref", mesh_bytes())
        ids = [a.add_car(t, 0) for t in teams]
        order[si, :len(ids)] = a.car_order()
        a.step(10)
        a.reset_to_random_kickoff(seed)
        for k, cid in enumerate(ids):
            cars[si, k] = np.frombuffer(bytes(a.get_car(cid)), np.uint8)
        balls[si] = np.frombuffer(bytes(a.get_ball()), np.uint8)
        for p in range(a.num_pads()):
            pads[si, p] = np.frombuffer(bytes(a.get_pad(p)), np.uint8)
        a.close()
    bs = ball_states(N_BALLS, np.dtype(OBall))
    going, team = np.zeros((len(PAIRS), N_BALLS), np.int32), np.zeros((len(PAIRS), N_BALLS), np.int32)
    a = SimArena("ref", mesh_bytes())
    for i in range(N_BALLS):
        a.set_ball(OBall.from_buffer_copy(bs[i].tobytes()))
        for j, (mt, mg) in enumerate(PAIRS):
            going[j, i], team[j, i] = a.is_ball_probably_going_in(mt, mg)
    a.close()
    print("going in:", going.sum(axis=1), "of", N_BALLS)
    np.savez_compressed(OUT, teams=np.array([c[0] + [-1] * (MC - len(c[0])) for c in CASES], np.int32),
                        order=order, seeds=np.array([c[1] for c in CASES], np.int64), cars=cars, balls=balls, pads=pads,
                        going_balls=bs.view(np.uint8).reshape(N_BALLS, -1), pairs=np.array(PAIRS, np.float32),
                        going=going, team=team)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
