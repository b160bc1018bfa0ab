"""The CUDA tick through the C ABI against the reference's rollouts of the benchmark workloads
(tests/workload_data.py): 64 arenas of the uniform 2v2 workload bench.py times, 48 arenas of the
uneven workload (2, 4 or 6 cars, all six hitboxes, kickoff resets after tick 60) and 8 arenas of
cars driving into the ball.  Continuous state within golden_data.TOL after 1 and 8 ticks (and 1 and 8
ticks after a reset); discrete car state, ball-hit counters, tickCountSinceUpdate and pads equal after
every one of 120 ticks; goal and bump callbacks equal to the reference's events in tick order; the
ball-hit callback firing exactly at the ticks where the reference's ballHitInfo.tickCountWhenHit
moves."""
import numpy as np
import pytest

from golden_data import check_continuous
from scenarios import gpu_controls, gpu_snapshot, setup_gpu
from workload_data import GROUPS, RESET_AFTER, TICKS, check_arena, load_workload

pytestmark = pytest.mark.gpu


def play_gpu(wl):
    scs = wl.scenarios
    batch, ids = setup_gpu(scs)
    pos = [{cid: i for i, cid in enumerate(row)} for row in ids]
    events = [[] for _ in scs]
    hits = [set() for _ in scs]
    cur = {"t": 0}
    batch.set_goal_score_callback(lambda a, team: events[a].append((cur["t"], 1, team, 0, 0)))
    batch.set_car_bump_callback(
        lambda a, x, y, demo: events[a].append((cur["t"], 2, pos[a][x] + 1, pos[a][y] + 1, int(demo))))
    batch.set_ball_hit_callback(lambda a, car, tick: hits[a].add((int(tick), pos[a][car])))
    resets = [si for si in range(wl.S) if wl.reset_seed[si] >= 0]
    snaps = []
    for t in range(TICKS):
        cur["t"] = t
        if t == RESET_AFTER and resets:
            batch.reset_to_random_kickoff_many(np.array(resets, np.uint32),
                                               np.array([wl.reset_seed[si] for si in resets], np.int32))
        batch.set_controls_all(gpu_controls(scs, t, batch.max_cars))
        batch.step(1)
        snaps.append(gpu_snapshot(batch, scs))
    flags = batch.device_flags()
    batch.close()
    return snaps, events, hits, flags


@pytest.mark.parametrize("name", GROUPS)
def test_gpu_follows_the_reference_on_the_workloads(name):
    wl = load_workload(name)
    snaps, events, hits, flags = play_gpu(wl)
    assert not (int(np.bitwise_or.reduce(flags)) & 0xff), flags  # no capacity overflow or NaN
    for si in range(wl.S):
        check_arena(wl, si, [s[si] for s in snaps], events[si], check_continuous, f"gpu {name}")
        assert hits[si] == wl.hit_ticks(si), f"gpu {name} arena {si}: ball-hit callbacks {sorted(hits[si])} " \
                                             f"!= reference {sorted(wl.hit_ticks(si))}"
    if name == "hits":
        assert sum(len(h) for h in hits) > 0
