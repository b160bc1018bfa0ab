"""The CUDA tick under a non-default MutatorConfig against the reference's own rollouts under the same
mutators (tests/golden/mutator_rollouts.npz, written by tests/golden/make_mutator_golden.py), and the
argument checks of rsg_set_mutator_config.

Continuous state within golden_data.TOL after 1 and 8 ticks; discrete state (flags, timers, boost,
demolitions, pads) identical over all 120 ticks, the four car-car scenarios included: there the
bumping car drives on into the demolished car's box and climbs onto it, and its wheel rays against
that box follow the reference's subsimplex convex cast.  The demolitions happen at ticks 11-19.
"""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

from golden_data import Golden, check_continuous
from scenarios import discrete_car, discrete_pads, gpu_controls, gpu_snapshot, setup_gpu

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
from make_mutator_golden import mutators  # noqa: E402

pytestmark = pytest.mark.gpu

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "mutator_rollouts.npz")


def test_gpu_matches_reference_under_mutators():
    g = Golden(np.load(PATH))
    scs = g.scenarios
    batch, _ = setup_gpu(scs, mutators=mutators())
    snaps = []
    for t in range(120):
        batch.set_controls_all(gpu_controls(scs, t, batch.max_cars))
        batch.step(1)
        snaps.append(gpu_snapshot(batch, scs))
    demos = 0
    for si in range(g.S):
        for t in (1, 8):
            cars, ball, _ = snaps[t - 1][si]
            check_continuous(cars, ball, g.cars_at(si, t), g.ball_at(si, t), t, f"mutator scenario {si}")
        for t in range(120):
            cars, ball, pads = snaps[t][si]
            np.testing.assert_array_equal(discrete_car(cars).astype(np.float32), g.disc_cars(si)[t],
                                          err_msg=f"mutator scenario {si} tick {t + 1}: car discrete state")
            np.testing.assert_array_equal(discrete_pads(pads).astype(np.float32), g.disc_pads(si)[t],
                                          err_msg=f"mutator scenario {si} tick {t + 1}: pads")
        demos += int(snaps[44][si][0]["is_demoed"].sum())
    assert demos >= 4  # demolition on contact (teammates included) happened
    batch.close()


def test_mutator_config_round_trip_and_errors():
    import rocketsim_gb300 as rsg
    from rocketsim_gb300 import abi
    rsg.init_from_mem([__import__("scenarios").mesh_bytes()])
    b = rsg.ArenaBatch(abi.GAMEMODE_SOCCAR, 3, 4, 120.0)
    m = mutators()
    b.set_mutator_config(m)
    got = b.get_mutator_config()
    assert bytes(got) == bytes(m)
    # the ball was re-made at rest at (0, 0, radius), as Ball::_BulletSetup places it
    s = b.get_ball_state(2)
    assert (s.pos.x, s.pos.y, s.pos.z) == (0.0, 0.0, 100.0) and s.vel.z == 0.0
    # cars added now respawn with the mutator's boost
    cid = b.add_car(0, abi.TEAM_BLUE, abi.CAR_OCTANE, 0)
    assert b.get_car_state(0, cid).boost == pytest.approx(60.0)
    # the ball cannot change while cars exist; car mass and an oversize ball are refused
    m2 = mutators()
    m2.ball_radius = 95.0
    with pytest.raises(abi.RSGError):
        b.set_mutator_config(m2)
    m3 = mutators()
    m3.car_mass = 200.0
    with pytest.raises(abi.RSGError):
        b.set_mutator_config(m3)
    b.close()
    b = rsg.ArenaBatch(abi.GAMEMODE_SOCCAR, 1, 4, 120.0)
    m4 = mutators()
    m4.ball_radius = 120.0
    with pytest.raises(abi.RSGError):
        b.set_mutator_config(m4)
    b.close()
