"""Ball prediction (rsg_ball_pred_*, the batched BallPredTracker) against the reference's own tracker
(tests/golden/ball_pred.npz, written by tests/golden/make_ballpred_golden.py).

* the same sequence of updates (creation, UpdatePredManual with the reference's ball states and
  tick gaps, one ForceUpdateAllPred) keeps, shifts and re-predicts exactly the entries the
  reference does (the tick count since the last state set of every predData entry, and
  lastUpdateTickCount, are equal), and the predicted states agree within the bounds below;
* UpdatePredFromArena through a batch gives bit for bit what the manual updates give;
* GetBallStateForTime picks the reference's entries; masks and argument checks.

Bounds: a predicted state i ticks ahead comes from i ticks of the ball-only arena tick from the
same start state; the reference normalises with SSE's reciprocal square root estimate, so the two
drift apart by float round-off per tick.  Over the 120 predicted ticks the bound is 0.05 uu,
0.1 uu/s and 5e-3 rad/s, plus 1e-5 relative (RocketSim's own BallState::Matches margins are 0.8
uu, 0.4 uu/s and 0.02 rad/s).
"""
from __future__ import annotations

import os

import numpy as np
import pytest

from scenarios import mesh_bytes

pytestmark = pytest.mark.gpu

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ball_pred.npz")
LIM = np.array([0.05] * 3 + [0.1] * 3 + [5e-3] * 3)


def vec9(rec: np.ndarray) -> np.ndarray:
    return np.stack([rec[f][c] for f in ("pos", "vel", "ang_vel") for c in "xyz"], axis=-1)


def balls(raw: np.ndarray):
    from rocketsim_gb300 import BALL_STATE_DTYPE
    return np.ascontiguousarray(raw).view(BALL_STATE_DTYPE).reshape(raw.shape[:-1])


def new_batch(z):
    import rocketsim_gb300 as rsg
    from rocketsim_gb300 import abi
    rsg.init_from_mem([mesh_bytes()])
    S = len(z["seeds"])
    b = rsg.ArenaBatch(abi.GAMEMODE_SOCCAR, S, 1, 120.0)
    _, bl, _ = b.get_all_states()
    bl[:] = balls(z["init_ball"])
    b.set_all_states(None, bl)
    return b


def check_update(tr, z, u, what):
    T = int(z["T"])
    got = tr.pred_all()
    assert got.shape == (len(z["seeds"]), T)
    np.testing.assert_array_equal(got["tick_count_since_update"], z["pred_ticks"][:, u], err_msg=f"{what}: kept entries")
    d = np.abs(vec9(got).astype(np.float64) - z["pred"][:, u])
    bad = d > LIM + 1e-5 * np.abs(z["pred"][:, u])
    assert not bad.any(), f"{what}: max diff {d.reshape(-1, 9).max(axis=0)}"
    for a in range(len(z["seeds"])):
        assert tr.last_update_tick(a) == z["last_update"][a, u], (what, a)
    return got


def k_of(z, u):
    """Ticks since the last update as UpdatePredFromArena computes them."""
    return (z["tick_count"][:, u] - z["last_update"][:, u - 1]).astype(np.int32)


def test_manual_updates_follow_the_reference():
    import rocketsim_gb300 as rsg
    z = np.load(PATH)
    b = new_batch(z)
    tr = rsg.BallPredTracker(b, int(z["T"]))
    check_update(tr, z, 0, "creation")
    for u in range(1, z["cur"].shape[1]):
        cur = balls(z["cur"][:, u])
        if u == int(z["force_at"]):
            tr.force_update_all(cur)
        else:
            tr.update_manual(cur, k_of(z, u))
        check_update(tr, z, u, f"update {u}")
        assert not tr.device_flags().any()
    tr.close()
    b.close()


def test_updates_from_a_batch_equal_manual_updates():
    import rocketsim_gb300 as rsg
    z = np.load(PATH)
    b, src = new_batch(z), new_batch(z)
    T = int(z["T"])
    manual, from_batch = rsg.BallPredTracker(b, T), rsg.BallPredTracker(src, T)
    S = len(z["seeds"])
    for u in range(1, z["cur"].shape[1]):
        # the batch keeps Bullet units: the manual tracker gets the states as the batch reports them
        _, bl, _ = src.get_all_states()
        bl[:] = balls(z["cur"][:, u])
        src.set_all_states(None, bl)
        for a in range(S):
            src.set_tick_count(a, int(z["tick_count"][a, u]))
        _, cur, _ = src.get_all_states()
        if u == int(z["force_at"]):
            manual.force_update_all(cur)
            from_batch.force_update_all(cur)
        else:
            manual.update_manual(cur, k_of(z, u))
            from_batch.update_from_batch(src)
        assert manual.pred_all().tobytes() == from_batch.pred_all().tobytes(), u
        assert [manual.last_update_tick(a) for a in range(S)] == [from_batch.last_update_tick(a) for a in range(S)]
    # GetBallStateForTime: the entry the reference picks
    for a in range(S):
        data = vec9(balls(np.stack([np.frombuffer(bytes(x), np.uint8) for x in manual.pred_data(a)])))
        ref_data = z["pred"][a, -1]
        for x, want in zip(z["times"], z["at_time"][a]):
            idx = int(np.flatnonzero((ref_data == want).all(axis=1))[0])
            got = vec9(balls(np.frombuffer(bytes(manual.get_ball_state_for_time(a, float(x))), np.uint8)[None]))[0]
            assert np.array_equal(got, data[idx]), (a, x, idx)
    manual.close()
    from_batch.close()
    b.close()
    src.close()


def test_mask_and_argument_checks():
    import rocketsim_gb300 as rsg
    from rocketsim_gb300 import abi
    z = np.load(PATH)
    b = new_batch(z)
    T = int(z["T"])
    tr = rsg.BallPredTracker(b, T)
    before = tr.pred_all()
    S = len(z["seeds"])
    mask = np.zeros(S, np.uint8)
    mask[1] = 1
    cur = balls(z["cur"][:, 10])
    tr.force_update_all(cur, mask=mask)
    after = tr.pred_all()
    for a in range(S):
        if a == 1:
            assert after[a, 0].tobytes() == cur[a].tobytes() and after[a].tobytes() != before[a].tobytes()
        else:
            assert after[a].tobytes() == before[a].tobytes()
    assert tr.num_pred_ticks == T and b.lib.rsg_ball_pred_num_pred_ticks(tr.h) == T
    other = rsg.ArenaBatch(abi.GAMEMODE_SOCCAR, S + 1, 1, 120.0)
    with pytest.raises(Exception):
        tr.update_from_batch(other)
    assert b.lib.rsg_ball_pred_create(b.h, 0) is None
    assert b.lib.rsg_ball_pred_get_pred(tr.h, S, None) == abi.ERR_ARG
    with pytest.raises(Exception):
        tr.pred_data(S)
    one = rsg.BallPredTracker(b, 1)  # predData of one entry: the state given, nothing simulated
    one.update_manual(cur, np.full(S, 3, np.int32))
    assert one.pred_all()[:, 0].tobytes() == cur.tobytes()
    one.close()
    other.close()
    tr.close()
    b.close()
