"""The kickoff fixture (tests/golden/kickoff_goal.npz, from the reference's ResetToRandomKickoff) against
a plain-Python statement of the shuffle the C ABI restates (CPU only): libstdc++'s default engine
(x <- 16807 x mod 2^31 - 1), its uniform_int_distribution (down-scaling with rejection) and its
std::shuffle (positions drawn two at a time), then the spot assignment of Arena.cpp:150-198."""
from __future__ import annotations

import os

import numpy as np

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "kickoff_goal.npz")
SPAWN = [(-2048, -2560), (2048, -2560), (-256, -3840), (256, -3840), (0, -4608)]
RESPAWN = [(-2304, -4608), (-2688, -4608), (2304, -4608), (2688, -4608)]


class MinStd0:
    def __init__(self, seed: int):
        self.x = (seed % (1 << 64)) % 2147483647 or 1

    def __call__(self) -> int:
        self.x = self.x * 16807 % 2147483647
        return self.x


def uniform_upto(g, hi: int) -> int:
    buckets = hi + 1
    scaling = 2147483645 // buckets
    past = buckets * scaling
    while True:
        r = g() - 1
        if r < past:
            return r // scaling


def shuffle(v: list, g) -> None:
    n, i = len(v), 1
    if n % 2 == 0:
        j = uniform_upto(g, 1)
        v[i], v[j] = v[j], v[i]
        i += 1
    while i != n:
        r0 = i + 1
        r1 = r0 + 1
        x = uniform_upto(g, r0 * r1 - 1)
        for j in (x // r1, x % r1):
            v[i], v[j] = v[j], v[i]
            i += 1


def test_shuffle_statement_gives_the_reference_spots():
    z = np.load(PATH)
    cars = z["cars"]
    for a in range(len(z["seeds"])):
        order = list(range(5))
        shuffle(order, MinStd0(int(z["seeds"][a])))
        teams = [int(t) for t in z["teams"][a] if t >= 0]
        upd = [int(i) for i in z["order"][a] if i > 0]  # car ids in the reference's update order
        team_ids = [[i for i in upd if teams[i - 1] == t] for t in (0, 1)]
        at_respawn = [0] * 4
        for i in range(max(len(team_ids[0]), len(team_ids[1]))):
            if i < 5:
                x, y = SPAWN[min(order[i], 4)]
            else:
                r = (i - 5) % 5
                x, y = RESPAWN[r]
                y += 250 * at_respawn[r]
                at_respawn[r] += 1
            for t in (0, 1):
                if i < len(team_ids[t]):
                    cid = team_ids[t][i]
                    rec = cars[a, cid - 1].view(np.float32)
                    want = (x, y) if t == 0 else (-x, -y)
                    # the reference reports positions back from Bullet units: round-off of the conversion
                    assert abs(rec[0] - want[0]) < 1e-2 and abs(rec[1] - want[1]) < 1e-2, (a, cid, rec[:2], want)
