"""Loads tests/golden/ref_rollouts.npz (written by tests/golden/make_golden.py from
the reference RocketSim) and rebuilds the scenarios it holds."""
from __future__ import annotations

import os

import numpy as np

from rocketsim_gb300 import abi
from scenarios import Scenario

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_rollouts.npz")

# Tolerances of the continuous state against the reference (uu, uu/s, rad/s, unitless
# rotation entries).  RocketSim's own "same state" test, BallState::Matches
# (src/Sim/Ball/Ball.h:53), allows 0.8 uu, 0.4 uu/s and 0.02 rad/s; these are 80x to
# 800x tighter.  The reference normalises vectors with the SSE reciprocal square root
# estimate; the restatement and the CUDA code use an exact square root, so the two
# differ by a few float ulps per tick and the bound grows with the tick count.
TOL = {
    1: dict(pos=1e-3, vel=2e-3, ang=1e-4, rot=1e-5),
    8: dict(pos=1e-2, vel=2e-2, ang=1e-3, rot=1e-4),
}


class Golden:
    def __init__(self, z):
        self.z = z
        self.S = len(z["seeds"])
        self.scenarios = []
        for si in range(self.S):
            n = int(z["ncars"][si])
            cars = [abi.CarState.from_buffer_copy(z["init_cars"][si, i].tobytes()) for i in range(n)]
            ball = abi.BallState.from_buffer_copy(z["init_ball"][si].tobytes())
            sc = Scenario(int(z["seeds"][si]), [int(x) for x in z["presets"][si, :n]],
                          [int(x) for x in z["teams"][si, :n]], cars, ball,
                          [int(x) for x in z["order"][si, :n]], z["controls"][si, :, :n].copy())
            self.scenarios.append(sc)

    def ncars(self, si):
        return int(self.z["ncars"][si])

    def cars_at(self, si, t):
        return self.z[f"cars_t{t}"][si, :self.ncars(si)]

    def ball_at(self, si, t):
        return self.z[f"ball_t{t}"][si:si + 1]

    def disc_cars(self, si):
        return self.z["disc_cars"][si, :, :self.ncars(si)]

    def disc_pads(self, si):
        return self.z["disc_pads"][si]

    def epa_tick(self, si):
        return int(self.z["epa_tick"][si])

    def events(self, si):
        ev = self.z["events"]
        return [tuple(int(v) for v in row[1:]) for row in ev if int(row[0]) == si]


def load_golden() -> Golden:
    return Golden(np.load(PATH))


def check_continuous(cars, ball, ref_cars, ref_ball, ticks, what=""):
    """Asserts the continuous state is within TOL[ticks] of the reference."""
    from scenarios import ball_vec, car_vec
    tol = TOL[ticks]
    a, b = car_vec(cars), car_vec(ref_cars)
    d = np.abs(a - b)
    lim = np.array([tol["pos"]] * 3 + [tol["vel"]] * 3 + [tol["ang"]] * 3 + [tol["rot"]] * 9)
    rel = 1e-6 * np.abs(b)
    bad = d > lim + rel
    assert not bad.any(), f"{what}: car state off after {ticks} ticks: max diff {d.max(axis=0)} (limits {lim})"
    a, b = ball_vec(ball), ball_vec(ref_ball)
    d = np.abs(a - b)
    lim = np.array([tol["pos"]] * 3 + [tol["vel"]] * 3 + [tol["ang"]] * 3)
    bad = d > lim + 1e-6 * np.abs(b)
    assert not bad.any(), f"{what}: ball state off after {ticks} ticks: max diff {d.max(axis=0)}"
