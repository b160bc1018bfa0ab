"""The reference's rollouts of the benchmark workloads (tests/golden/workload_rollouts.npz, written by
tests/golden/make_workload_golden.py) and the players that replay them on a checker or on the GPU.

Groups: ``bench`` (64 arenas of the 4096-arena uniform 2v2 workload that bench.py times), ``uneven``
(48 arenas of the uneven workload: 2, 4 or 6 cars of all six hitboxes, every third arena reset to a
random kickoff after tick 60) and ``hits`` (cars driving into the ball, two of them next to a goal).
"""
from __future__ import annotations

import os

import numpy as np

from rocketsim_gb300 import abi
from scenarios import (Scenario, _controls_struct, cpu_snapshot, discrete_car, discrete_hit, discrete_pads,
                       hit_vec, setup_cpu)

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "workload_rollouts.npz")
TICKS = 120
RESET_AFTER = 60
GROUPS = ("bench", "uneven", "hits")
# The ball-hit record's positions and velocity (uu, uu/s) are set at the hit from the contact point
# and the car and ball states of that tick, up to 120 ticks into a rollout.
HIT_TOL = 2e-2


class Workload:
    def __init__(self, z, name: str):
        self.name = name
        g = lambda k: z[f"{name}_{k}"]  # noqa: E731
        self.g = g
        self.S = len(g("seeds"))
        self.scenarios = []
        for si in range(self.S):
            n = int(g("ncars")[si])
            cars = [abi.CarState.from_buffer_copy(g("init_cars")[si, i].tobytes()) for i in range(n)]
            ball = abi.BallState.from_buffer_copy(g("init_ball")[si].tobytes())
            self.scenarios.append(Scenario(int(g("seeds")[si]), [int(x) for x in g("presets")[si, :n]],
                                           [int(x) for x in g("teams")[si, :n]], cars, ball,
                                           [int(x) for x in g("order")[si, :n]], g("controls")[si, :, :n].copy()))
        self.reset_seed = [int(x) for x in g("reset_seed")]

    def ncars(self, si):
        return int(self.g("ncars")[si])

    def cars_at(self, si, t):
        return self.g(f"cars_t{t}")[si, :self.ncars(si)]

    def ball_at(self, si, t):
        return self.g(f"ball_t{t}")[si:si + 1]

    def events(self, si):
        """[(tick, kind, a, b, flag)] in the reference's order."""
        return [(int(r[2]), int(r[1]), int(r[3]), int(r[4]), int(r[5])) for r in self.g("events") if int(r[0]) == si]

    def hit_ticks(self, si):
        """{(tick, car index)} where the reference's ballHitInfo.tickCountWhenHit became that tick."""
        dh = self.g("disc_hit")[si]
        out = set()
        for t in range(TICKS):
            for i in range(self.ncars(si)):
                if dh[t, i, 0] == 1 and dh[t, i, 1] == t:
                    out.add((t, i))
        return out


def load_workload(name: str) -> Workload:
    return Workload(np.load(PATH), name)


def play_cpu(kind: str, wl: Workload, si: int, ticks: int = TICKS):
    """Replays one arena on a checker; the kickoff reset needs the reference, so a checker without it
    stops at the reset.  Returns the per-tick snapshots and the events [(tick, kind, a, b, flag)]."""
    from oracle.pyoracle import CarControls as OCtl
    sc = wl.scenarios[si]
    a, ids = setup_cpu(kind, sc)
    assert ids == list(range(1, len(ids) + 1))
    snaps, events = [], []
    for t in range(ticks):
        if t == RESET_AFTER and wl.reset_seed[si] >= 0:
            if kind != "ref":
                break
            a.reset_to_random_kickoff(wl.reset_seed[si])
        for i, cid in enumerate(ids):
            a.set_controls(cid, OCtl.from_buffer_copy(bytes(_controls_struct(sc.controls[t, i]))))
        a.step(1)
        snaps.append(cpu_snapshot(a, ids))
        events += [(t, int(e[0]), int(e[2]), int(e[3]), int(e[4])) for e in a.pop_events()]
    a.close()
    return snaps, events


def check_arena(wl: Workload, si: int, snaps, events, check_cont, what: str):
    """The replay of arena `si` against the reference: continuous state after 1 and 8 ticks (and 1 and
    8 ticks after a reset) within golden_data.TOL, discrete car state, ball-hit counters,
    tickCountSinceUpdate and pads equal after every tick, the ball-hit positions within HIT_TOL, and
    the goal and bump events equal in tick order."""
    g = wl.g
    n = wl.ncars(si)
    reset = wl.reset_seed[si] >= 0
    for t in (1, 8) + ((RESET_AFTER + 1, RESET_AFTER + 8) if reset else ()):
        if t <= len(snaps):
            cars, ball, _ = snaps[t - 1]
            check_cont(cars, ball, wl.cars_at(si, t), wl.ball_at(si, t), 1 if t in (1, RESET_AFTER + 1) else 8,
                       f"{what} arena {si} tick {t}")
    for t in range(len(snaps)):
        cars, ball, pads = snaps[t]
        np.testing.assert_array_equal(discrete_car(cars).astype(np.float32), g("disc_cars")[si, t, :n],
                                      err_msg=f"{what} arena {si} tick {t + 1}: car discrete state")
        np.testing.assert_array_equal(discrete_hit(cars), g("disc_hit")[si, t, :n],
                                      err_msg=f"{what} arena {si} tick {t + 1}: ball-hit counters")
        np.testing.assert_array_equal(discrete_pads(pads).astype(np.float32), g("disc_pads")[si, t],
                                      err_msg=f"{what} arena {si} tick {t + 1}: pads")
        d = np.abs(hit_vec(cars) - g("hit_cont")[si, t, :n].astype(np.float64))
        assert d.max(initial=0) <= HIT_TOL, f"{what} arena {si} tick {t + 1}: ball-hit record off by {d.max()}"
    ref_ev = [e for e in wl.events(si) if e[0] < len(snaps)]
    assert events == ref_ev, f"{what} arena {si}: events {events} != reference {ref_ev}"
