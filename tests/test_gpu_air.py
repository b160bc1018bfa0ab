"""Air rollouts and their adjoint on the GPU, through the C ABI (rsg_air_forward / rsg_air_backward)
and the torch.autograd harness over it.

* forward: against the reference's own rollouts in THE_VOID (tests/golden/air_rollouts.npz) and
  against the full arena tick (rsg_step) on the same airborne cars;
* gradients: against FP64 central finite differences (step 1e-4) of the FP64 restatement
  (oracle/air_fp64.py), relative error <= 1e-3 per instance over all 60 x 4 control entries, for
  several checkpoint spacings, and for the initial state;
* cost: one backward costs at most 3 forward rollouts.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from air_cases import (DT, OCTANE_HITBOX, TOL, gradient_case, load_golden, max_errors, state_vectors,
                       to_reference_layout, within)
from oracle import air_fp64 as F

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
    return s, c, adjoint.air_rollout(s, c, ckpt_every=ckpt_every)


def test_air_forward_matches_reference_golden(torch_cuda):
    torch = torch_cuda
    cars, balls, controls, traj = load_golden()
    s0 = state_vectors(cars, balls)
    for t in (1, 8, 60):
        _, _, fin = rollout_gpu(torch, s0, controls[:t])
        errs = max_errors(to_reference_layout(fin.cpu().numpy()), traj[t - 1])
        assert within(errs, TOL[t]), (t, errs)


def test_air_forward_matches_arena_tick(torch_cuda):
    """The same airborne cars stepped by rsg_step in THE_VOID: the contact-free rollout is the
    arena tick for boost inputs of 0 or 1 held over the rollout."""
    import rocketsim_gb300 as rsg
    from rocketsim_gb300 import abi, adjoint
    torch = torch_cuda
    cars, balls, controls, traj = load_golden()
    n = len(cars)
    b = rsg.ArenaBatch(abi.GAMEMODE_THE_VOID, n, 1)
    ids = []
    for i in range(n):
        cid = b.add_car(i, 0, abi.CAR_OCTANE, 0)
        b.set_car_state(i, cid, cars[i])
        b.set_ball_state(i, balls[i])
        ids.append(cid)
    s0 = state_vectors(cars, balls)
    done = 0
    for t in (1, 8, 60):
        for k in range(done, t):
            ctl = np.zeros(n, rsg.CONTROLS_DTYPE)
            ctl["pitch"], ctl["yaw"], ctl["roll"] = controls[k, :, 0], controls[k, :, 1], controls[k, :, 2]
            ctl["boost"] = controls[k, :, 3].astype(np.uint8)
            b.set_controls_all(ctl)
            b.step(1)
        done = t
        _, _, fin = rollout_gpu(torch, s0, controls[:t])
        fin = fin.cpu().numpy()
        for i in range(n):
            g = b.get_car_state(i, ids[i])
            a = adjoint.car_state_from_vector(fin[i])
            for f in ("pos", "vel", "ang_vel"):
                ga, aa = getattr(g, f), getattr(a, f)
                d = max(abs(ga.x - aa.x), abs(ga.y - aa.y), abs(ga.z - aa.z))
                scale = max(1.0, abs(ga.x), abs(ga.y), abs(ga.z))
                assert d <= 1e-6 * scale * t, (t, i, f, d)
    b.close()


def _fd_check(torch, seed, n, ticks, ckpt_every, fast=False):
    from rocketsim_gb300 import adjoint
    s, u, target = gradient_case(seed, n, ticks, fast=fast)
    sg, ug, fin = rollout_gpu(torch, s, u, ckpt_every=ckpt_every, grad=True)
    tgt = torch.from_numpy(target.astype(np.float32)).cuda()
    adjoint.aim_loss(fin, tgt).sum().backward()
    g = ug.grad.cpu().numpy().astype(np.float64)
    gs = sg.grad.cpu().numpy().astype(np.float64)
    iinv = F.car_inv_inertia(OCTANE_HITBOX)
    loss = lambda f: F.aim_loss(f, target)  # noqa: E731
    gfd = F.fd_grad(s.astype(np.float64), u.astype(np.float64), iinv, DT, loss, h=1e-4)
    num = np.linalg.norm((g - gfd).transpose(1, 0, 2).reshape(n, -1), axis=1)
    den = np.linalg.norm(gfd.transpose(1, 0, 2).reshape(n, -1), axis=1)
    rel = num / den
    assert rel.max() <= REL_ERR, rel
    return s, u, target, gs, iinv, loss


@pytest.mark.parametrize("ckpt_every", [1, 7, 16, 60, 100])
def test_air_control_gradient_matches_fp64_fd(torch_cuda, ckpt_every):
    _fd_check(torch_cuda, 11, 12, 60, ckpt_every)


def test_air_control_gradient_at_the_speed_clamps(torch_cuda):
    _fd_check(torch_cuda, 12, 12, 60, 16, fast=True)


def test_air_state_gradient_matches_fp64_fd(torch_cuda):
    s, u, target, gs, iinv, loss = _fd_check(torch_cuda, 13, 8, 60, 16)
    h = 1e-4
    s64, u64 = s.astype(np.float64), u.astype(np.float64)
    fd = np.zeros_like(s64)
    for j in range(24):
        a, b = s64.copy(), s64.copy()
        a[:, j] += h
        b[:, j] -= h
        fd[:, j] = (loss(F.rollout(a, u64, iinv, DT)) - loss(F.rollout(b, u64, iinv, DT))) / (2 * h)
    rel = np.linalg.norm(gs - fd, axis=1) / np.linalg.norm(fd, axis=1)
    assert rel.max() <= REL_ERR, rel


def test_air_c_abi_direct_and_errors(torch_cuda):
    """The entry points called through ctypes directly, as a C caller would, and their argument checks."""
    import rocketsim_gb300 as rsg
    from rocketsim_gb300 import abi, adjoint
    torch = torch_cuda
    lib = abi.load(build_if_missing=False)
    cfg = rsg.car_config(abi.CAR_OCTANE)
    s, u, _ = gradient_case(17, 5, 9)
    ds = torch.from_numpy(s).cuda()
    du = torch.from_numpy(u).cuda()
    fin = torch.empty_like(ds)
    ck = torch.empty((3, 5, 24), device="cuda")
    P = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    assert lib.rsg_air_forward(C.byref(cfg), 120.0, 5, 9, P(ds), P(du), P(fin), P(ck), 4, None) == abi.OK
    gfin = torch.ones_like(ds)
    gu = torch.empty_like(du)
    nb = C.c_size_t()
    assert lib.rsg_air_backward_workspace_size(5, 9, C.byref(nb)) == abi.OK
    assert nb.value == 152 * 5 * 9
    work = torch.empty(nb.value, dtype=torch.uint8, device="cuda")
    assert lib.rsg_air_backward(C.byref(cfg), 120.0, 5, 9, P(du), P(ck), 4, P(gfin), P(gu), None, P(work), nb.value,
                                None) == abi.OK
    torch.cuda.synchronize()
    du2 = du.clone().requires_grad_(True)
    ref = adjoint.air_rollout(ds, du2, cfg, ckpt_every=4)
    assert torch.equal(ref, fin)
    ref.backward(gfin)
    assert torch.equal(du2.grad, gu)
    # argument errors come back as RSG_ERR_ARG, nothing is launched
    assert lib.rsg_air_forward(C.byref(cfg), 120.0, 5, 9, P(ds), P(du), P(fin), P(ck), 0, None) == abi.ERR_ARG
    assert lib.rsg_air_forward(C.byref(cfg), 120.0, -1, 9, P(ds), P(du), P(fin), None, 4, None) == abi.ERR_ARG
    assert lib.rsg_air_forward(C.byref(cfg), 0.0, 5, 9, P(ds), P(du), P(fin), None, 4, None) == abi.ERR_ARG
    assert lib.rsg_air_backward(C.byref(cfg), 120.0, 5, 9, P(du), None, 4, P(gfin), P(gu), None, P(work), nb.value,
                                None) == abi.ERR_ARG
    assert lib.rsg_air_backward(C.byref(cfg), 120.0, 5, 9, P(du), P(ck), 4, P(gfin), P(gu), None, P(work),
                                nb.value - 1, None) == abi.ERR_ARG
    with pytest.raises(ValueError):
        adjoint.air_rollout(torch.from_numpy(s), torch.from_numpy(u))
    with pytest.raises(ValueError):
        adjoint.air_rollout(ds, du, ckpt_every=0)


def test_air_backward_costs_at_most_three_forwards(torch_cuda):
    from rocketsim_gb300 import adjoint
    torch = torch_cuda
    n, ticks = 1 << 16, 60
    rng = np.random.default_rng(3)
    s = np.zeros((n, 24), np.float32)
    s[:, 9:18] = np.eye(3, dtype=np.float32).reshape(9)
    s[:, 3:6] = rng.normal(size=(n, 3)) * 10
    ds = torch.from_numpy(s).cuda()
    du = (torch.rand((ticks, n, 4), device="cuda") * 2 - 1).clamp(-1, 1)
    du[..., 3] = du[..., 3].abs()
    du.requires_grad_(True)
    gfin = torch.randn((n, 24), device="cuda")

    def fwd():
        return adjoint.air_rollout(ds, du, ckpt_every=16)

    for _ in range(3):
        fwd().backward(gfin)
    e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    tf, tb = [], []
    for _ in range(5):
        e[0].record()
        out = fwd()
        e[1].record()
        out.backward(gfin)
        e[2].record()
        torch.cuda.synchronize()
        tf.append(e[0].elapsed_time(e[1]))
        tb.append(e[1].elapsed_time(e[2]))
    ratio = float(np.median(tb) / np.median(tf))
    assert ratio <= 3.0, (np.median(tf), np.median(tb), ratio)
