"""Ground-driving rollouts and their adjoint on the GPU, through the C ABI (rsg_ground_forward /
rsg_ground_backward) and the torch.autograd harness over it.

* forward: against the reference's own drives on the soccar floor (tests/golden/ground_rollouts.npz),
  every tick of 120, including the vehicle state (steer angle, engine, brake, friction factors,
  push-backs);
* gradients: against FP64 central finite differences (step 1e-4) of the FP64 restatement
  (oracle/ground_fp64.py), relative error <= 1e-3 per instance, for the controls over 120 ticks and
  for the initial state; checkpoint spacings give identical gradients;
* the model-exit flags and the argument checks of the entry points.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from ground_cases import DT, STATE, TOL, gradient_case, load_golden, max_errors, state_vectors, within
from oracle import ground_fp64 as G

pytestmark = pytest.mark.gpu

REL_ERR = 1e-3


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def rollout_gpu(torch, s0: np.ndarray, u: np.ndarray, ckpt_every: int = 16, grad: bool = False):
    from rocketsim_gb300 import adjoint
    s = torch.from_numpy(np.ascontiguousarray(s0, np.float32)).cuda().requires_grad_(grad)
    c = torch.from_numpy(np.ascontiguousarray(u, np.float32)).cuda().requires_grad_(grad)
    fin, flags = adjoint.ground_rollout(s, c, ckpt_every=ckpt_every, return_flags=True)
    return s, c, fin, flags


def test_ground_forward_matches_reference_golden(torch_cuda):
    """Every tick of the 24 reference drives: the states at each tick's start come back as
    checkpoints with ckpt_every = 1."""
    import rocketsim_gb300 as rsg
    from rocketsim_gb300 import abi
    torch = torch_cuda
    lib = abi.load(build_if_missing=False)
    cfg = rsg.car_config(abi.CAR_OCTANE)
    cars, balls, veh, controls, traj, vehicle = load_golden()
    n, T = len(cars), controls.shape[0]
    ds = torch.from_numpy(state_vectors(cars, balls, veh)).cuda()
    du = torch.from_numpy(np.ascontiguousarray(controls, np.float32)).cuda()
    fin = torch.empty_like(ds)
    ck = torch.empty((T, n, STATE), device="cuda")
    flags = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    P = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    assert lib.rsg_ground_forward(C.byref(cfg), 120.0, n, T, P(ds), P(du), P(fin), P(ck), 1, P(flags), None) == abi.OK
    torch.cuda.synchronize()
    assert int(flags.abs().max()) == 0
    states = torch.cat([ck[1:], fin[None]]).cpu().numpy()  # state after tick t at [t - 1]
    assert np.array_equal(ck[0].cpu().numpy(), ds.cpu().numpy())
    for t in (1, 30, 120):
        errs = max_errors(states[t - 1], traj[t - 1], vehicle[t - 1])
        assert within(errs, TOL[t]), (t, errs)
    errs = max_errors(states, traj, vehicle)
    assert within(errs, TOL[120]), errs


def _fd_check(torch, seed, n, ticks, ckpt_every, fd_ticks):
    from rocketsim_gb300 import adjoint
    s, u, txy, tdir = gradient_case(seed, n, ticks)
    sg, ug, fin, flags = rollout_gpu(torch, s, u, ckpt_every=ckpt_every, grad=True)
    assert int(flags.abs().max()) == 0
    t_xy = torch.from_numpy(txy.astype(np.float32)).cuda()
    t_dir = torch.from_numpy(tdir.astype(np.float32)).cuda()
    adjoint.drive_loss(fin, t_xy, t_dir).sum().backward()
    g = ug.grad.cpu().numpy().astype(np.float64)
    gs = sg.grad.cpu().numpy().astype(np.float64)
    geo = G.car_geometry()
    loss = lambda f: G.drive_loss(f, txy, tdir)  # noqa: E731
    which = [(t, c) for t in fd_ticks for c in range(3)]
    gfd = G.fd_grad(s.astype(np.float64), u.astype(np.float64), geo, DT, loss, h=1e-4, which=which)
    a = np.stack([g[t, :, c] for t, c in which], axis=1)
    b = np.stack([gfd[t, :, c] for t, c in which], axis=1)
    rel = np.linalg.norm(a - b, axis=1) / np.linalg.norm(b, axis=1)
    assert rel.max() <= REL_ERR, rel
    assert np.all(g[..., 3] == 0)
    return s, u, txy, tdir, g, gs, geo, loss


def test_ground_control_gradient_matches_fp64_fd(torch_cuda):
    """120 ticks, 8 cars; the finite differences cover all three controls at 12 ticks spread over
    the rollout (the first, the last and ones between)."""
    _fd_check(torch_cuda, 21, 8, 120, 16, [0, 1, 2, 10, 30, 50, 70, 90, 100, 110, 118, 119])


def test_ground_gradient_does_not_depend_on_checkpoints(torch_cuda):
    """The tape kernel recomputes each segment from its checkpoint with the forward's own
    arithmetic, so every checkpoint spacing gives the same gradient bit for bit."""
    from rocketsim_gb300 import adjoint
    torch = torch_cuda
    s, u, txy, tdir = gradient_case(22, 16, 100)
    t_xy = torch.from_numpy(txy.astype(np.float32)).cuda()
    t_dir = torch.from_numpy(tdir.astype(np.float32)).cuda()
    ref = None
    for ck in (1, 7, 16, 100, 250):
        sg, ug, fin, _ = rollout_gpu(torch, s, u, ckpt_every=ck, grad=True)
        adjoint.drive_loss(fin, t_xy, t_dir).sum().backward()
        got = (fin.detach().cpu().numpy(), ug.grad.cpu().numpy(), sg.grad.cpu().numpy())
        if ref is None:
            ref = got
        for a, b in zip(ref, got):
            assert np.array_equal(a, b), ck


def test_ground_state_gradient_matches_fp64_fd(torch_cuda):
    s, u, txy, tdir, g, gs, geo, loss = _fd_check(torch_cuda, 23, 6, 40, 16, [0, 20, 39])
    h = 1e-5
    s64, u64 = s.astype(np.float64), u.astype(np.float64)
    fd = np.zeros_like(s64)
    for j in range(STATE):
        a, b = s64.copy(), s64.copy()
        a[:, j] += h
        b[:, j] -= h
        fd[:, j] = (loss(G.rollout(a, u64, geo, DT)) - loss(G.rollout(b, u64, geo, DT))) / (2 * h)
    rel = np.linalg.norm(gs - fd, axis=1) / np.linalg.norm(fd, axis=1)
    assert rel.max() <= REL_ERR, rel


def test_ground_flags_and_c_abi_errors(torch_cuda):
    """Ticks outside the model set the flags; the entry points called through ctypes directly, as a
    C caller would, agree with the autograd harness bit for bit; argument errors return RSG_ERR_ARG."""
    import rocketsim_gb300 as rsg
    from rocketsim_gb300 import abi, adjoint
    torch = torch_cuda
    lib = abi.load(build_if_missing=False)
    cfg = rsg.car_config(abi.CAR_OCTANE)
    s, u, _, _ = gradient_case(24, 5, 9)
    s[4, 2] += 300 * 0.02  # 300 uu up in the air: the rays miss the floor
    ds = torch.from_numpy(s).cuda()
    du = torch.from_numpy(u).cuda()
    fin = torch.empty_like(ds)
    ck = torch.empty((3, 5, STATE), device="cuda")
    flags = torch.empty((5,), dtype=torch.int32, device="cuda")
    P = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    assert lib.rsg_ground_forward(C.byref(cfg), 120.0, 5, 9, P(ds), P(du), P(fin), P(ck), 4, P(flags), None) == abi.OK
    gfin = torch.ones_like(ds)
    gu = torch.empty_like(du)
    nb = C.c_size_t()
    assert lib.rsg_ground_backward_workspace_size(5, 9, C.byref(nb)) == abi.OK
    assert nb.value == 180 * 5 * 9
    work = torch.empty(nb.value, dtype=torch.uint8, device="cuda")
    assert lib.rsg_ground_backward(C.byref(cfg), 120.0, 5, 9, P(du), P(ck), 4, P(gfin), P(gu), None, P(work),
                                   nb.value, None) == abi.OK
    torch.cuda.synchronize()
    assert flags.cpu().tolist()[:4] == [0, 0, 0, 0] and flags.cpu().tolist()[4] & 1
    du2 = du.clone().requires_grad_(True)
    ref = adjoint.ground_rollout(ds, du2, cfg, ckpt_every=4)
    assert torch.equal(ref, fin)
    ref.backward(gfin)
    assert torch.equal(du2.grad, gu)
    # the FP64 restatement flags the same instance
    f64 = np.zeros(5, np.int64)
    G.rollout(s.astype(np.float64), u.astype(np.float64), G.car_geometry(), DT, flags=f64)
    assert f64.tolist() == flags.cpu().tolist()
    # argument errors come back as RSG_ERR_ARG, nothing is launched
    assert lib.rsg_ground_forward(C.byref(cfg), 120.0, 5, 9, P(ds), P(du), P(fin), P(ck), 0, None, None) == abi.ERR_ARG
    assert lib.rsg_ground_forward(C.byref(cfg), 120.0, -1, 9, P(ds), P(du), P(fin), None, 4, None, None) == abi.ERR_ARG
    assert lib.rsg_ground_forward(C.byref(cfg), 0.0, 5, 9, P(ds), P(du), P(fin), None, 4, None, None) == abi.ERR_ARG
    assert lib.rsg_ground_backward(C.byref(cfg), 120.0, 5, 9, P(du), None, 4, P(gfin), P(gu), None, P(work),
                                   nb.value, None) == abi.ERR_ARG
    assert lib.rsg_ground_backward(C.byref(cfg), 120.0, 5, 9, P(du), P(ck), 4, P(gfin), P(gu), None, P(work),
                                   nb.value - 1, None) == abi.ERR_ARG
    with pytest.raises(ValueError):
        adjoint.ground_rollout(torch.from_numpy(s), torch.from_numpy(u))
    with pytest.raises(ValueError):
        adjoint.ground_rollout(ds, du, ckpt_every=0)
