"""Writes tests/golden/ball_pred.npz from the reference RocketSim's BallPredTracker.

For each scenario (four cars driving about a moving ball, as the rollout fixtures make them) the
reference arena gets a BallPredTracker of 120 ticks at tick 0 (its constructor predicts from the
arena's ball), then plays the scenario's controls in chunks of 1 to 8 ticks.  After each chunk the
tracker is updated from the arena (UpdatePredFromArena: kept and extended when the ball matches its
prediction, predicted again when a car touched it), once a ForceUpdateAllPred replaces that; the
ball state it was given, the ticks since the last update, lastUpdateTickCount and the whole
predData (position, velocity, angular velocity, and the tick count since the last state set, which
shows which entries were kept) are recorded.  GetBallStateForTime is sampled at the end.

Run from the repository root with the reference library built (make -C oracle ref).
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from scenarios import _controls_struct, make_scenario, setup_cpu  # noqa: E402

OUT = os.path.join(HERE, "ball_pred.npz")
SEEDS = (610, 611, 612, 613)
T = 120
CHUNKS = (1, 1, 2, 3, 1, 5, 8, 1, 1, 4, 2, 6, 1, 3, 7, 1, 2, 8, 1, 1)
FORCE_AT = 9  # this update is a ForceUpdateAllPred instead
TIMES = (-1.0, 0.0, 0.004, 0.0084, 0.5, 0.99, 0.9999, 1.0, 7.0)


def vec9(s) -> list[float]:
    return [s.pos.x, s.pos.y, s.pos.z, s.vel.x, s.vel.y, s.vel.z, s.ang_vel.x, s.ang_vel.y, s.ang_vel.z]


def main():
    from oracle.pyoracle import build_ref, CarControls as OCtl
    build_ref()
    S, U = len(SEEDS), len(CHUNKS) + 1
    init_ball = np.zeros((S, 80), np.uint8)
    cur = np.zeros((S, U, 80), np.uint8)         # BallState given to the update (raw rsg_ball_state)
    ticks = np.zeros((S, U), np.int32)            # ticks since the last update (0 for the constructor)
    tick_count = np.zeros((S, U), np.int64)       # the arena's tick count at the update
    last_update = np.zeros((S, U), np.int32)      # lastUpdateTickCount after it
    pred = np.zeros((S, U, T, 9), np.float32)
    pred_ticks = np.zeros((S, U, T), np.uint64)   # tickCountSinceUpdate of each predData entry
    at_time = np.zeros((S, len(TIMES), 9), np.float32)
    scs = [make_scenario(s, ticks=sum(CHUNKS) + 1) for s in SEEDS]
    for si, sc in enumerate(scs):
        a, ids = setup_cpu("ref", sc)
        init_ball[si] = np.frombuffer(bytes(a.get_ball()), np.uint8)
        tr = a.ball_pred_tracker(T)

        def record(u, k):
            b = a.get_ball()
            cur[si, u] = np.frombuffer(bytes(b), np.uint8)
            ticks[si, u] = k
            tick_count[si, u] = a.get_tick()
            last_update[si, u] = tr.last_update_tick()
            d = tr.pred_data()
            assert len(d) == T
            pred[si, u] = [vec9(x) for x in d]
            pred_ticks[si, u] = [x.tick_count_since_update for x in d]
            return b
        record(0, 0)
        t = 0
        for u, k in enumerate(CHUNKS, start=1):
            for _ in range(k):
                for i, cid in enumerate(ids):
                    a.set_controls(cid, OCtl.from_buffer_copy(bytes(_controls_struct(sc.controls[t, i]))))
                a.step(1)
                t += 1
            if u == FORCE_AT:
                tr.force_update_all(a.get_ball())
            else:
                tr.update_from_arena(a)
            record(u, k)
        at_time[si] = [vec9(tr.state_for_time(x)) for x in TIMES]
        full = [int(pred_ticks[si, u, 1] == 1) for u in range(U)]
        print(f"seed {sc.seed}: updates predicted again {full}")
        tr.close()
        a.close()
    np.savez_compressed(OUT, seeds=np.array(SEEDS), chunks=np.array(CHUNKS), force_at=FORCE_AT, T=T,
                        times=np.array(TIMES, np.float32), init_ball=init_ball, cur=cur, ticks=ticks,
                        tick_count=tick_count, last_update=last_update, pred=pred, pred_ticks=pred_ticks,
                        at_time=at_time)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
