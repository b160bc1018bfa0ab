"""GameMode::HEATSEEKER through the C ABI against the reference's own rollouts in that mode
(tests/golden/heatseeker_rollouts.npz, written by tests/golden/make_heatseeker_golden.py): cars
touching a ball at rest (the touch gives the ball a target net, after which it seeks it), kickoffs
from Arena::ResetToRandomKickoff (heatseeker's four spots and ball start), and balls that already seek
a net bouncing off the back wall beside it (the target turns around).

Continuous state within golden_data.TOL after 1 and 8 ticks; discrete car state, ball-hit counters,
pads and the ball's heatseeker state (target, target speed, time since the touch) equal after every
one of 120 ticks; the ball within HS_BALL_TOL of the reference's after every tick; the goal and bump
events equal.  The seeking ball turns through atan2 / sin / cos (CUDA's here, the C library's in the
reference), which can differ in the last bit: hence a per-tick ball tolerance rather than the 1- and
8-tick one while it seeks.
"""
import os

import numpy as np
import pytest

from golden_data import check_continuous
from scenarios import ball_vec, discrete_car, discrete_hit, discrete_pads, gpu_controls, gpu_snapshot, setup_gpu
from workload_data import Workload

pytestmark = pytest.mark.gpu

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "heatseeker_rollouts.npz")
TICKS = 120
# uu, uu/s, rad/s: RocketSim's own "same ball state" margins (BallState::Matches, Ball.h:53)
HS_BALL_TOL = np.array([0.8] * 3 + [0.4] * 3 + [0.02] * 3)


def test_heatseeker_follows_the_reference():
    from rocketsim_gb300 import abi
    z = np.load(PATH)
    wl = Workload(z, "hs")
    scs = wl.scenarios
    batch, ids = setup_gpu(scs, game_mode=abi.GAMEMODE_HEATSEEKER)
    assert batch.get_mutator_config().boost_used_per_second == 0  # heatseeker's infinite boost
    pos = [{cid: i for i, cid in enumerate(row)} for row in ids]
    events = [[] for _ in scs]
    cur = {"t": 0}
    batch.set_goal_score_callback(lambda a, team: events[a].append((cur["t"], 1, team, 0, 0)))
    batch.set_car_bump_callback(
        lambda a, x, y, demo: events[a].append((cur["t"], 2, pos[a][x] + 1, pos[a][y] + 1, int(demo))))
    for si in range(wl.S):
        h = abi.HeatseekerInfo(*[float(x) for x in z["hs_init_hs"][si]])
        batch.set_ball_heatseeker(si, h)
    resets = [si for si in range(wl.S) if wl.reset_seed[si] >= 0]
    batch.reset_to_random_kickoff_many(np.array(resets, np.uint32),
                                       np.array([wl.reset_seed[si] for si in resets], np.int32))
    snaps, hs = [], np.zeros((wl.S, TICKS, 3), np.float32)
    for t in range(TICKS):
        cur["t"] = t
        batch.set_controls_all(gpu_controls(scs, t, batch.max_cars))
        batch.step(1)
        snaps.append(gpu_snapshot(batch, scs))
        for si in range(wl.S):
            x = batch.get_ball_heatseeker(si)
            hs[si, t] = (x.y_target_dir, x.cur_target_speed, x.time_since_hit)
    batch.close()
    g = wl.g
    worst = np.zeros(9)
    for si in range(wl.S):
        n = wl.ncars(si)
        for t in (1, 8):
            cars, ball, _ = snaps[t - 1][si]
            check_continuous(cars, ball, wl.cars_at(si, t), wl.ball_at(si, t), t, f"heatseeker arena {si}")
        for t in range(TICKS):
            cars, ball, pads = snaps[t][si]
            what = f"heatseeker arena {si} tick {t + 1}"
            np.testing.assert_array_equal(discrete_car(cars).astype(np.float32), g("disc_cars")[si, t, :n],
                                          err_msg=what + ": car discrete state")
            np.testing.assert_array_equal(discrete_hit(cars), g("disc_hit")[si, t, :n], err_msg=what + ": ball hits")
            np.testing.assert_array_equal(discrete_pads(pads).astype(np.float32), g("disc_pads")[si, t],
                                          err_msg=what + ": pads")
            np.testing.assert_array_equal(hs[si, t], g("hs")[si, t], err_msg=what + ": heatseeker state")
            d = np.abs(ball_vec(ball)[0] - ball_vec(g("balls")[si, t:t + 1])[0])
            worst = np.maximum(worst, d)
            assert (d <= HS_BALL_TOL).all(), f"{what}: ball off by {d}"
        ref_ev = wl.events(si)
        assert events[si] == ref_ev, f"heatseeker arena {si}: events {events[si]} != reference {ref_ev}"
    print("largest ball difference over all ticks:", worst)
    assert (g("hs")[..., 0] != 0).sum() > 300  # the ball sought a net for a good part of the run
