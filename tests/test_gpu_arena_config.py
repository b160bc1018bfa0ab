"""The CUDA tick in arenas created with a non-default ArenaConfig (24 custom boost pads, ball
rotation integrated) against the reference's own rollouts in such arenas
(tests/golden/arena_config_rollouts.npz, written by tests/golden/make_arena_config_golden.py).

Continuous state within golden_data.TOL after 1 and 8 ticks, the ball's rotation included;
discrete state (flags, timers, boost) and the 24 pads' state identical over 120 ticks.
"""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

from golden_data import TOL, Golden, check_continuous
from scenarios import discrete_car, discrete_pads, gpu_controls, gpu_snapshot, setup_gpu

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
from make_arena_config_golden import config, custom_pads  # noqa: E402

pytestmark = pytest.mark.gpu

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "arena_config_rollouts.npz")


def rot(ball):
    r = ball["rot_mat"][0]
    return np.array([[r[k][c] for c in ("x", "y", "z")] for k in ("forward", "right", "up")], np.float64)


def test_gpu_matches_reference_with_custom_pads_and_ball_rotation():
    import ctypes as C
    from rocketsim_gb300 import abi
    g = Golden(np.load(PATH))
    scs = g.scenarios
    batch, _ = setup_gpu(scs, config=config())
    assert batch.num_pads == 24
    pos, big = abi.Vec3(), C.c_int()
    for i, (x, y, z, b) in enumerate(custom_pads()):
        assert batch.lib.rsg_get_pad_config(batch.h, i, C.byref(pos), C.byref(big)) == abi.OK
        assert (pos.x, pos.y, pos.z, bool(big.value)) == (np.float32(x), np.float32(y), np.float32(z), b)
    snaps = []
    for t in range(120):
        batch.set_controls_all(gpu_controls(scs, t, batch.max_cars))
        batch.step(1)
        snaps.append(gpu_snapshot(batch, scs))
    picked = 0
    for si in range(g.S):
        for t in (1, 8):
            cars, ball, _ = snaps[t - 1][si]
            check_continuous(cars, ball, g.cars_at(si, t), g.ball_at(si, t), t, f"arena-config scenario {si}")
            assert np.abs(rot(ball) - rot(g.ball_at(si, t))).max() <= TOL[t]["rot"] * 10, (si, t)
        for t in range(120):
            cars, ball, pads = snaps[t][si]
            np.testing.assert_array_equal(discrete_car(cars).astype(np.float32), g.disc_cars(si)[t],
                                          err_msg=f"arena-config scenario {si} tick {t + 1}: car discrete state")
            np.testing.assert_array_equal(discrete_pads(pads).astype(np.float32), g.disc_pads(si)[t],
                                          err_msg=f"arena-config scenario {si} tick {t + 1}: pads")
        picked += int((g.disc_pads(si)[:, :, 0] == 0).any(axis=0).sum())
    assert picked >= 10  # custom pads, big and small, were picked up
    batch.close()


def test_arena_config_checks():
    import rocketsim_gb300 as rsg
    from rocketsim_gb300 import abi
    from scenarios import mesh_bytes
    rsg.init_from_mem([mesh_bytes()])
    c = rsg.arena_config(custom_boost_pads=[(0.0, 0.0, 70.0, False)] * 35)  # more than the 34 slots
    with pytest.raises(abi.RSGError):
        rsg.ArenaBatch(abi.GAMEMODE_SOCCAR, 1, 4, 120.0, c)
    c = rsg.arena_config()
    c.max_aabb_len = 500.0  # another broadphase cell size
    with pytest.raises(abi.RSGError):
        rsg.ArenaBatch(abi.GAMEMODE_SOCCAR, 1, 4, 120.0, c)
    b = rsg.ArenaBatch(abi.GAMEMODE_SOCCAR, 2, 4, 120.0, rsg.arena_config(custom_boost_pads=[]))
    assert b.num_pads == 0
    cars, balls, pads = b.get_all_states()
    assert pads.size == 0
    b.step(2)
    b.close()
