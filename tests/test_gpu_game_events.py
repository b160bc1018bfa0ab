"""GameEventTracker for every arena of a batch (rsg_game_event_tracker_*) against the reference's own
tracker along the scripts of tests/game_event_cases.py (tests/golden/game_events.npz, written by
tests/golden/make_game_event_golden.py): the same shot, goal and save events with the same cars, at
the same updates; no event elsewhere.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

from game_event_cases import SCRIPTS, TEAMS
from golden_data import TOL
from scenarios import mesh_bytes

pytestmark = pytest.mark.gpu

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "game_events.npz")


def run_gpu(auto, script):
    import rocketsim_gb300 as rsg
    from rocketsim_gb300 import abi
    rsg.init_from_mem([mesh_bytes()])
    b = rsg.ArenaBatch(abi.GAMEMODE_SOCCAR, 1, 4, 120.0)
    assert [b.add_car(0, t) for t in TEAMS] == [1, 2, 3, 4]
    cfg = rsg.GameEventTracker.default_config()
    cfg.auto_state_set_detection = 1 if auto else 0
    tr = rsg.GameEventTracker(b, cfg)
    events, balls = [], []
    for op in script:
        if op[0] == "ball":
            s = abi.BallState()
            s.pos.x, s.pos.y, s.pos.z = op[1]
            s.vel.x, s.vel.y, s.vel.z = op[2]
            s.rot_mat.forward.x = s.rot_mat.right.y = s.rot_mat.up.z = 1
            b.set_ball_state(0, s)
        elif op[0] == "hit":
            c = b.get_car_state(0, op[1])
            c.ball_hit_info.is_valid = 1
            c.ball_hit_info.tick_count_when_hit = b.get_tick_count(0) - op[2]
            b.set_car_state(0, op[1], c)
        elif op[0] == "car":
            c = b.get_car_state(0, op[1])
            c.pos.x, c.pos.y, c.pos.z = op[2]
            c.vel.x = c.vel.y = c.vel.z = c.ang_vel.x = c.ang_vel.y = c.ang_vel.z = 0.0
            c.rot_mat.forward.x, c.rot_mat.forward.y, c.rot_mat.forward.z = 0.0, 1.0, 0.0
            c.rot_mat.right.x, c.rot_mat.right.y, c.rot_mat.right.z = -1.0, 0.0, 0.0
            c.rot_mat.up.x, c.rot_mat.up.y, c.rot_mat.up.z = 0.0, 0.0, 1.0
            c.is_on_ground = 1
            b.set_car_state(0, op[1], c)
        elif op[0] == "step":
            b.step(op[1])
        elif op[0] == "update":
            e = tr.update(b)[0]
            events.append([int(e["kind"]), int(e["car_id"]), int(e["other_car_id"])])
            s = b.get_ball_state(0)
            balls.append([s.pos.x, s.pos.y, s.pos.z, s.vel.x, s.vel.y, s.vel.z])
        elif op[0] == "reset":
            tr.reset_persistent_info()
    tr.close()
    b.close()
    return np.array(events, np.int32), np.array(balls, np.float32)


@pytest.mark.parametrize("name", sorted(SCRIPTS))
def test_events_match_the_reference(name):
    z = np.load(PATH)
    auto, script = SCRIPTS[name]
    ev, balls = run_gpu(auto, script)
    ref_ev = z[f"{name}_events"]
    # the ball at every update within the 8-tick tolerance of golden_data.TOL (measured: 1.5e-4 uu,
    # 6.1e-4 uu/s in the longest script), the events equal
    d = np.abs(balls - z[f"{name}_balls"])
    assert d[:, :3].max() <= TOL[8]["pos"] and d[:, 3:].max() <= TOL[8]["vel"], d.max(axis=0)
    np.testing.assert_array_equal(ev, ref_ev, err_msg=name)
    assert (ref_ev[:, 0] != 0).any()  # every script has at least one event
