"""The FP64 ground-driving restatement (oracle/ground_fp64.py) pinned to the reference (CPU only)."""
from __future__ import annotations

import numpy as np

from ground_cases import DT, TOL, gradient_case, load_golden, max_errors, state_vectors, within
from oracle import ground_fp64 as G


def test_fp64_rollout_matches_reference_golden():
    cars, balls, veh, controls, traj, vehicle = load_golden()
    s0 = state_vectors(cars, balls, veh).astype(np.float64)
    flags = np.zeros(len(cars), np.int64)
    _, tr = G.rollout(s0, controls.astype(np.float64), G.car_geometry(), DT, trajectory=True, flags=flags)
    assert not flags.any()
    for t in (1, 30, 120):
        errs = max_errors(tr[t - 1], traj[t - 1], vehicle[t - 1])
        assert within(errs, TOL[t]), (t, errs)
    errs = max_errors(tr, traj, vehicle)  # every tick
    assert within(errs, TOL[120]), errs


def test_golden_covers_the_driving_modes():
    cars, balls, veh, controls, traj, vehicle = load_golden()
    thr, boost = controls[..., 0], controls[..., 2]
    assert set(np.unique(boost)) == {0.0, 1.0}
    assert (thr == 0).any() and (thr < 0).any() and (thr == 1).all(axis=0).any()
    engine, brake = vehicle[..., 1], vehicle[..., 2]
    assert (engine > 0).any() and (engine < 0).any()        # forward and reverse drive
    assert ((engine == 0) & (brake > 0)).any()              # coasting / braking roll impulses
    speeds = np.linalg.norm(traj[..., 3:6], axis=-1)
    assert speeds.max() > 2000.0                             # boosting up to near top speed
    steer = vehicle[..., 0]
    assert np.abs(steer).max() > 0.3
    assert (vehicle[..., 11:15] > 0).any()                   # push-back of compressed wheels


def test_wheel_off_the_floor_sets_the_flag():
    cars, balls, veh, controls, _, _ = load_golden()
    s0 = state_vectors(cars[:2], balls[:2], veh[:2]).astype(np.float64)
    s0[1, 2] += 300 * 0.02  # 300 uu up in the air
    flags = np.zeros(2, np.int64)
    G.rollout(s0, controls[:3, :2].astype(np.float64), G.car_geometry(), DT, flags=flags)
    assert flags[0] == 0 and flags[1] & 1


def test_finite_differences_are_consistent():
    """The FP64 central differences that check the adjoint are converged: steps 1e-4 and 5e-5
    agree to 1e-6 of the gradient's scale on a 30-tick case."""
    s, u, txy, tdir = gradient_case(5, 4, 30)
    lf = lambda f: G.drive_loss(f, txy, tdir)  # noqa: E731
    which = [(0, 0), (0, 1), (0, 2), (15, 1), (29, 2)]
    geo = G.car_geometry()
    a = G.fd_grad(s.astype(np.float64), u.astype(np.float64), geo, DT, lf, h=1e-4, which=which)
    b = G.fd_grad(s.astype(np.float64), u.astype(np.float64), geo, DT, lf, h=5e-5, which=which)
    sel = ~np.isnan(a)
    scale = np.abs(a[sel]).max()
    assert scale > 0
    assert np.abs(a[sel] - b[sel]).max() <= 1e-6 * scale


def test_loss_gradient_matches_finite_differences():
    s, u, txy, tdir = gradient_case(6, 3, 4)
    geo = G.car_geometry()
    fin = G.rollout(s.astype(np.float64), u.astype(np.float64), geo, DT)
    g = G.drive_loss_grad(fin, txy, tdir)
    eps = 1e-6
    for j in (0, 1, 9, 12):
        f = fin.copy()
        f[:, j] += eps
        fd = (G.drive_loss(f, txy, tdir) - G.drive_loss(fin, txy, tdir)) / eps
        np.testing.assert_allclose(g[:, j], fd, rtol=1e-4, atol=1e-5)
