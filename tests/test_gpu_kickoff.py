"""Kickoff resets and the goal-bound check through the C ABI against the reference's own results
(tests/golden/kickoff_goal.npz, written by tests/golden/make_kickoff_golden.py):

* rsg_reset_to_random_kickoff_many (Arena::ResetToRandomKickoff(seed)): with the reference's car
  update order, every car lands on the spot the reference gives it (the seeded shuffle of
  libstdc++'s default engine), with the reference's state (rotation within 1e-6, the rest bit
  for bit); ball and pads reset;
* rsg_is_ball_probably_going_in (Arena::IsBallProbablyGoingIn): the same answer and goal team for
  3000 ball states and three (maxTime, extraMargin) pairs.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

from scenarios import mesh_bytes

pytestmark = pytest.mark.gpu

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "kickoff_goal.npz")


def test_kickoff_matches_the_reference():
    import rocketsim_gb300 as rsg
    from rocketsim_gb300 import CAR_STATE_DTYPE, BALL_STATE_DTYPE, PAD_STATE_DTYPE, abi
    z = np.load(PATH)
    rsg.init_from_mem([mesh_bytes()])
    S, MC = z["teams"].shape
    b = rsg.ArenaBatch(abi.GAMEMODE_SOCCAR, S, MC, 120.0)
    for a in range(S):
        teams = [int(t) for t in z["teams"][a] if t >= 0]
        ids = [b.add_car(a, t) for t in teams]
        assert ids == list(range(1, len(teams) + 1))
        b.set_car_update_order(a, [int(i) for i in z["order"][a] if i > 0])
    b.step(10)
    b.reset_to_random_kickoff_many(np.arange(S), z["seeds"].astype(np.int32))
    cars, balls, pads = b.get_all_states()
    for a in range(S):
        n = int((z["teams"][a] >= 0).sum())
        got = cars[a * MC:a * MC + n]
        ref = z["cars"][a, :n].copy().view(CAR_STATE_DTYPE).reshape(n)
        for f in CAR_STATE_DTYPE.names:
            if f.startswith("_"):
                continue
            if f == "rot_mat":
                for c in ("forward", "right", "up"):
                    for k in "xyz":
                        assert np.abs(got[f][c][k] - ref[f][c][k]).max() <= 1e-6, (a, f, c, k)
            else:
                assert got[f].tobytes() == ref[f].tobytes(), (a, f)
        assert balls[a:a + 1].tobytes() == z["balls"][a].tobytes(), a
        rp = z["pads"][a].copy().view(PAD_STATE_DTYPE).reshape(34)
        gp = pads[a * 34:(a + 1) * 34]
        for f in ("is_active", "cooldown", "cur_locked_car_id", "prev_locked_car_id"):
            np.testing.assert_array_equal(gp[f], rp[f], err_msg=f"arena {a} pads {f}")
    # a seed of -1 draws from the process's own engine: still a kickoff spot for every car
    b.reset_to_random_kickoff(0, -1)
    cars, _, _ = b.get_all_states()
    assert cars[0]["is_on_ground"] == 1 and cars[0]["pos"]["z"] == np.float32(17.0)
    b.close()


def test_ball_probably_going_in_matches_the_reference():
    import rocketsim_gb300 as rsg
    from rocketsim_gb300 import BALL_STATE_DTYPE, abi
    z = np.load(PATH)
    rsg.init_from_mem([mesh_bytes()])
    bs = z["going_balls"].copy().view(BALL_STATE_DTYPE).reshape(-1)
    n = len(bs)
    b = rsg.ArenaBatch(abi.GAMEMODE_SOCCAR, n, 1, 120.0)
    b.set_all_states(None, bs)
    for j, (mt, mg) in enumerate(z["pairs"]):
        going, team = b.is_ball_probably_going_in(float(mt), float(mg))
        np.testing.assert_array_equal(going.astype(np.int32), z["going"][j], err_msg=f"pair {j}")
        np.testing.assert_array_equal(team, z["team"][j], err_msg=f"pair {j}")
    b.close()
    void = rsg.ArenaBatch(abi.GAMEMODE_THE_VOID, 2, 1, 120.0)
    with pytest.raises(Exception):
        void.is_ball_probably_going_in()
    void.close()
