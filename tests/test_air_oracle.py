"""The FP64 air-tick restatement (oracle/air_fp64.py) pinned to the reference (CPU only)."""
from __future__ import annotations

import os

import numpy as np
import pytest

from air_cases import (DT, OCTANE_HITBOX, TOL, gradient_case, load_golden, max_errors, state_vectors,
                       to_reference_layout, within)
from oracle import air_fp64 as F


def test_fp64_rollout_matches_reference_golden():
    cars, balls, controls, traj = load_golden()
    s0 = state_vectors(cars, balls).astype(np.float64)
    iinv = F.car_inv_inertia(OCTANE_HITBOX)
    _, tr = F.rollout(s0, controls.astype(np.float64), iinv, DT, trajectory=True)
    got = to_reference_layout(tr)
    for t in (1, 8, 60):
        errs = max_errors(got[t - 1], traj[t - 1])
        assert within(errs, TOL[t]), (t, errs)
    # every tick, not just the three checkpoints: nothing touched anything
    errs = max_errors(got, traj)
    assert within(errs, TOL[60]), errs


def test_golden_holds_both_boost_inputs_and_the_clamps():
    cars, balls, controls, traj = load_golden()
    assert set(np.unique(controls[..., 3])) == {0.0, 1.0}
    speeds = np.linalg.norm(traj[..., 3:6], axis=-1)
    spins = np.linalg.norm(traj[..., 6:9], axis=-1)
    assert speeds.max() >= 2299.0  # the car speed clamp is active in some rollouts
    assert spins.max() >= 5.49     # and so is the angular speed clamp


def test_loss_gradient_matches_finite_differences():
    s, u, target = gradient_case(3, 4, 2)
    fin = F.rollout(s.astype(np.float64), u.astype(np.float64), F.car_inv_inertia(OCTANE_HITBOX), DT)
    g = F.aim_loss_grad(fin, target)
    h = 1e-6
    for j in range(24):
        a, b = fin.copy(), fin.copy()
        a[:, j] += h
        b[:, j] -= h
        fd = (F.aim_loss(a, target) - F.aim_loss(b, target)) / (2 * h)
        np.testing.assert_allclose(g[:, j], fd, rtol=1e-6, atol=1e-8)


def test_finite_differences_are_step_stable():
    """The central differences used as the gradient reference agree between steps 1e-4 and 1e-5."""
    s, u, target = gradient_case(5, 3, 12)
    iinv = F.car_inv_inertia(OCTANE_HITBOX)
    loss = lambda fin: F.aim_loss(fin, target)  # noqa: E731
    which = [(t, c) for t in (0, 5, 11) for c in range(4)]
    g4 = F.fd_grad(s.astype(np.float64), u.astype(np.float64), iinv, DT, loss, h=1e-4, which=which)
    g5 = F.fd_grad(s.astype(np.float64), u.astype(np.float64), iinv, DT, loss, h=1e-5, which=which)
    sel = ~np.isnan(g4)
    np.testing.assert_allclose(g4[sel], g5[sel], rtol=1e-6, atol=1e-9)


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                                    "oracle", "_ref", "librsref.so")),
                    reason="reference library not built here")
def test_golden_reproduces_from_the_reference():
    """Re-runs two golden instances through the reference library: bit-identical."""
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    from make_air_golden import kinematics
    from oracle.pyoracle import SimArena, BallState as OBallState, CarControls as OCtl, CarState as OCarState
    from scenarios import mesh_bytes
    from rocketsim_gb300 import abi
    cars, balls, controls, traj = load_golden()
    SimArena("ref", mesh_bytes()).close()
    for i in (0, 7):
        a = SimArena("ref", None, game_mode=abi.GAMEMODE_THE_VOID)
        cid = a.add_car(0, abi.CAR_OCTANE)
        a.set_car(cid, OCarState.from_buffer_copy(bytes(cars[i])))
        a.set_ball(OBallState.from_buffer_copy(bytes(balls[i])))
        for t in range(controls.shape[0]):
            c = OCtl()
            c.pitch, c.yaw, c.roll = (float(x) for x in controls[t, i, :3])
            c.boost = int(controls[t, i, 3])
            a.set_controls(cid, c)
            a.step(1)
            assert np.array_equal(kinematics(a.get_car(cid), a.get_ball()), traj[t, i]), (i, t)
        a.close()
