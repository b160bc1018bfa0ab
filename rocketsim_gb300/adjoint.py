"""Differentiable rollouts: torch.autograd over rsg_air_* (contact-free air phase) and
rsg_ground_* (driving on the floor).

A rollout advances, per instance, one airborne car and the ball through `ticks` arena ticks
under pitch/yaw/roll/boost controls, with nothing to touch (the air path of Arena::Step,
src/Sim/Arena/Arena.cpp:689-756, for a car with no wheel, body or world contact).  The boost
input is relaxed from {0, 1} to [0, 1] so that it has a gradient; for inputs of exactly 0 or 1
the forward is the arena tick.  The backward runs the hand-written adjoint kernel: the forward
stores the state every `ckpt_every` ticks; the backward recomputes all segments from their
checkpoints at once into a tape (152 bytes per instance and tick, from torch's allocator) and
sweeps it in reverse.

State vector, 24 floats per instance in Bullet units (1 BT = 50 uu): car position, velocity,
angular velocity, basis rows (row r = (forward[r], right[r], up[r])), ball position, ball
velocity.  ``state_vector`` / ``car_state_from_vector`` convert from and to RocketSim's states.

Example::

    from rocketsim_gb300 import adjoint
    s0 = adjoint.state_vector(car_states, ball_states).cuda()        # [n, 24]
    u = torch.zeros(60, n, 4, device="cuda", requires_grad=True)     # pitch, yaw, roll, boost
    final = adjoint.air_rollout(s0, u)
    adjoint.aim_loss(final, target_basis).sum().backward()           # u.grad: [60, n, 4]

Ground rollouts work the same way on a 39-float state (``ground_state_vector``: the kinematics,
the vehicle state of btVehicleRL's wheels, the ball) with throttle, steer and boost controls
(``ground_rollout``, ``drive_loss``); the boost input is relaxed the same way and its full
throttle becomes throttle + boost * (1 - throttle).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import abi
from .abi import BallState, CarConfig, CarState, check

STATE = 24
GROUND_STATE = 39
UU_TO_BT = np.float32(1.0 / 50.0)  # RLConst::UU_TO_BT, a float
BT_TO_UU = np.float32(50.0)


def _ptr(t: torch.Tensor | None):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _check_tensor(t: torch.Tensor, name: str, shape: tuple) -> None:
    if not t.is_cuda:
        raise ValueError(f"{name} must be a CUDA tensor (the rollout has no CPU path)")
    if t.dtype != torch.float32:
        raise TypeError(f"{name} must be float32, got {t.dtype}")
    if tuple(t.shape) != shape:
        raise ValueError(f"{name} must have shape {shape}, got {tuple(t.shape)}")


class AirRollout(torch.autograd.Function):
    """final_state = rollout(state0, controls); differentiable in both."""

    @staticmethod
    def forward(ctx, state0: torch.Tensor, controls: torch.Tensor, car: CarConfig, tick_rate: float,
                ckpt_every: int):
        lib = abi.load(build_if_missing=False)
        n = state0.shape[0]
        ticks = controls.shape[0]
        state0 = state0.contiguous()
        controls = controls.contiguous()
        _check_tensor(state0, "state0", (n, STATE))
        _check_tensor(controls, "controls", (ticks, n, 4))
        if state0.device != controls.device:
            raise ValueError("state0 and controls must be on the same device")
        if ckpt_every < 1:
            raise ValueError("ckpt_every must be >= 1")
        final = torch.empty_like(state0)
        need_grad = ctx.needs_input_grad[0] or ctx.needs_input_grad[1]
        ckpt = None
        if need_grad:
            nseg = (ticks + ckpt_every - 1) // ckpt_every
            ckpt = torch.empty((max(nseg, 1), n, STATE), device=state0.device, dtype=torch.float32)
        with torch.cuda.device(state0.device):
            check(lib.rsg_air_forward(C.byref(car), float(tick_rate), n, ticks, _ptr(state0), _ptr(controls),
                                      _ptr(final), _ptr(ckpt), ckpt_every, _stream()), "rsg_air_forward")
        if need_grad:
            ctx.save_for_backward(controls, ckpt)
        ctx.car = car
        ctx.tick_rate = float(tick_rate)
        ctx.ckpt_every = ckpt_every
        ctx.n = n
        return final

    @staticmethod
    @torch.autograd.function.once_differentiable
    def backward(ctx, grad_final: torch.Tensor):
        lib = abi.load(build_if_missing=False)
        controls, ckpt = ctx.saved_tensors
        ticks, n = controls.shape[0], ctx.n
        grad_final = grad_final.contiguous().to(torch.float32)
        grad_controls = torch.empty_like(controls)
        grad_state0 = torch.empty_like(grad_final) if ctx.needs_input_grad[0] else None
        nbytes = C.c_size_t()
        check(lib.rsg_air_backward_workspace_size(n, ticks, C.byref(nbytes)), "rsg_air_backward_workspace_size")
        work = torch.empty(max(nbytes.value, 1), dtype=torch.uint8, device=controls.device)
        with torch.cuda.device(controls.device):
            check(lib.rsg_air_backward(C.byref(ctx.car), ctx.tick_rate, n, ticks, _ptr(controls), _ptr(ckpt),
                                       ctx.ckpt_every, _ptr(grad_final), _ptr(grad_controls), _ptr(grad_state0),
                                       _ptr(work), nbytes.value, _stream()), "rsg_air_backward")
        return grad_state0, (grad_controls if ctx.needs_input_grad[1] else None), None, None, None


def air_rollout(state0: torch.Tensor, controls: torch.Tensor, car: CarConfig | int = abi.CAR_OCTANE,
                tick_rate: float = 120.0, ckpt_every: int = 16) -> torch.Tensor:
    """Final state [n, 24] after controls.shape[0] ticks from state0 [n, 24]; controls [ticks, n, 4]."""
    if not isinstance(car, CarConfig):
        from .arena import car_config
        car = car_config(car)
    return AirRollout.apply(state0, controls, car, tick_rate, ckpt_every)


class GroundRollout(torch.autograd.Function):
    """(final_state, flags) = ground rollout(state0, controls); final_state is differentiable in
    both inputs, flags ([n] int32, the ticks that left the ground model) is not."""

    @staticmethod
    def forward(ctx, state0: torch.Tensor, controls: torch.Tensor, car: CarConfig, tick_rate: float,
                ckpt_every: int):
        lib = abi.load(build_if_missing=False)
        n = state0.shape[0]
        ticks = controls.shape[0]
        state0 = state0.contiguous()
        controls = controls.contiguous()
        _check_tensor(state0, "state0", (n, GROUND_STATE))
        _check_tensor(controls, "controls", (ticks, n, 4))
        if state0.device != controls.device:
            raise ValueError("state0 and controls must be on the same device")
        if ckpt_every < 1:
            raise ValueError("ckpt_every must be >= 1")
        final = torch.empty_like(state0)
        flags = torch.empty((n,), dtype=torch.int32, device=state0.device)
        need_grad = ctx.needs_input_grad[0] or ctx.needs_input_grad[1]
        ckpt = None
        if need_grad:
            nseg = (ticks + ckpt_every - 1) // ckpt_every
            ckpt = torch.empty((max(nseg, 1), n, GROUND_STATE), device=state0.device, dtype=torch.float32)
        with torch.cuda.device(state0.device):
            check(lib.rsg_ground_forward(C.byref(car), float(tick_rate), n, ticks, _ptr(state0), _ptr(controls),
                                         _ptr(final), _ptr(ckpt), ckpt_every, _ptr(flags), _stream()),
                  "rsg_ground_forward")
        if need_grad:
            ctx.save_for_backward(controls, ckpt)
        ctx.car = car
        ctx.tick_rate = float(tick_rate)
        ctx.ckpt_every = ckpt_every
        ctx.n = n
        ctx.mark_non_differentiable(flags)
        return final, flags

    @staticmethod
    @torch.autograd.function.once_differentiable
    def backward(ctx, grad_final: torch.Tensor, grad_flags):
        lib = abi.load(build_if_missing=False)
        controls, ckpt = ctx.saved_tensors
        ticks, n = controls.shape[0], ctx.n
        grad_final = grad_final.contiguous().to(torch.float32)
        grad_controls = torch.empty_like(controls)
        grad_state0 = torch.empty_like(grad_final) if ctx.needs_input_grad[0] else None
        nbytes = C.c_size_t()
        check(lib.rsg_ground_backward_workspace_size(n, ticks, C.byref(nbytes)), "rsg_ground_backward_workspace_size")
        work = torch.empty(max(nbytes.value, 1), dtype=torch.uint8, device=controls.device)
        with torch.cuda.device(controls.device):
            check(lib.rsg_ground_backward(C.byref(ctx.car), ctx.tick_rate, n, ticks, _ptr(controls), _ptr(ckpt),
                                          ctx.ckpt_every, _ptr(grad_final), _ptr(grad_controls), _ptr(grad_state0),
                                          _ptr(work), nbytes.value, _stream()), "rsg_ground_backward")
        return grad_state0, (grad_controls if ctx.needs_input_grad[1] else None), None, None, None


def ground_rollout(state0: torch.Tensor, controls: torch.Tensor, car: CarConfig | int = abi.CAR_OCTANE,
                   tick_rate: float = 120.0, ckpt_every: int = 16, return_flags: bool = False):
    """Final state [n, 39] after controls.shape[0] ticks of driving on the floor from state0
    [n, 39]; controls [ticks, n, 4] = throttle, steer, boost, unused.  With `return_flags` also
    the [n] int32 flags: bit 0 where a wheel's ray missed the floor, bit 1 where the car tilted
    past the suspension's contact limit (ticks outside the model)."""
    if not isinstance(car, CarConfig):
        from .arena import car_config
        car = car_config(car)
    final, flags = GroundRollout.apply(state0, controls, car, tick_rate, ckpt_every)
    return (final, flags) if return_flags else final


def drive_loss(final: torch.Tensor, target_xy: torch.Tensor, target_dir: torch.Tensor) -> torch.Tensor:
    """Per-instance loss of a ground rollout: squared distance of the final car position to
    `target_xy` ([n, 2]) plus that of its forward axis to the unit vector `target_dir` ([n, 3])."""
    d = final[:, 0:2] - target_xy
    f = final[:, 9:18].reshape(-1, 3, 3)[:, :, 0] - target_dir
    return (d * d).sum(dim=1) + (f * f).sum(dim=1)


def aim_loss(final: torch.Tensor, target_basis: torch.Tensor, dist_scale: float = 1e-2) -> torch.Tensor:
    """Per-instance loss: squared Frobenius distance of the final basis to `target_basis`
    ([n, 3, 3]) plus dist_scale * |car position + forward - ball position|^2."""
    B = final[:, 9:18].reshape(-1, 3, 3)
    orient = ((B - target_basis) ** 2).sum(dim=(1, 2))
    d = final[:, 0:3] + B[:, :, 0] - final[:, 18:21]
    return orient + dist_scale * (d * d).sum(dim=1)


# front centre of the Octane hitbox in car space, Bullet units (hitbox offset plus half length
# along forward, offset along up; src/Sim/Car/CarConfig/CarConfig.cpp:20-27)
OCTANE_NOSE = (float(np.float32((13.8757 + 120.507 / 2) / 50.0)), 0.0, float(np.float32(20.755 / 50.0)))


def contact_loss(final: torch.Tensor, target_point: torch.Tensor, target_vel: torch.Tensor,
                 vel_scale: float = 1e-2, nose=OCTANE_NOSE) -> torch.Tensor:
    """Per-instance loss of a ground rollout at the end of the horizon: squared distance of the
    car's nose (`nose`, car space) to `target_point` ([n, 3]) plus vel_scale times the squared
    distance of its velocity to `target_vel` ([n, 3])."""
    B = final[:, 9:18].reshape(-1, 3, 3)
    d = final[:, 0:3] + B @ torch.tensor(nose, dtype=final.dtype, device=final.device) - target_point
    e = final[:, 3:6] - target_vel
    return (d * d).sum(dim=1) + vel_scale * (e * e).sum(dim=1)


# ---------------------------------------------------------------- state conversion
def state_vector(cars, balls) -> torch.Tensor:
    """[n, 24] float32 CPU tensor from sequences of CarState and BallState (uu units), converted
    as Car::SetState / Ball::SetState do (float multiply by UU_TO_BT, src/Sim/Car/Car.cpp:20-36)."""
    f32 = np.float32
    rows = np.zeros((len(cars), STATE), np.float32)
    for i, (c, b) in enumerate(zip(cars, balls)):
        rm = c.rot_mat
        rows[i, 0:3] = np.array([c.pos.x, c.pos.y, c.pos.z], f32) * UU_TO_BT
        rows[i, 3:6] = np.array([c.vel.x, c.vel.y, c.vel.z], f32) * UU_TO_BT
        rows[i, 6:9] = [c.ang_vel.x, c.ang_vel.y, c.ang_vel.z]
        rows[i, 9:18] = [rm.forward.x, rm.right.x, rm.up.x, rm.forward.y, rm.right.y, rm.up.y,
                         rm.forward.z, rm.right.z, rm.up.z]
        rows[i, 18:21] = np.array([b.pos.x, b.pos.y, b.pos.z], f32) * UU_TO_BT
        rows[i, 21:24] = np.array([b.vel.x, b.vel.y, b.vel.z], f32) * UU_TO_BT
    return torch.from_numpy(rows)


def ground_state_vector(cars, balls, vehicle=None) -> torch.Tensor:
    """[n, 39] float32 CPU tensor for ground rollouts: the kinematics of `state_vector`, then the
    vehicle state the next tick starts from (front steer angle, engine force, brake, lateral
    friction factor per wheel, longitudinal friction factor per wheel, extra push-back per wheel:
    15 floats per car, the btWheelInfoRL fields of src/Sim/btVehicleRL/btVehicleRL.h:9-27), then
    the ball.  Without `vehicle` ([n, 15]) the vehicle state is that of a car that has not run a
    tick yet: all zero."""
    kin = state_vector(cars, balls).numpy()
    out = np.zeros((kin.shape[0], GROUND_STATE), np.float32)
    out[:, 0:18] = kin[:, 0:18]
    if vehicle is not None:
        out[:, 18:33] = np.asarray(vehicle, np.float32).reshape(-1, 15)
    out[:, 33:39] = kin[:, 18:24]
    return torch.from_numpy(out)


def car_state_from_vector(v, template: CarState | None = None) -> CarState:
    """CarState (uu units) with the kinematic fields of one 24-float state vector, converted as
    Car::GetState does (float multiply by BT_TO_UU, src/Sim/Car/Car.cpp:10-18)."""
    v = np.asarray(v, np.float32)
    s = CarState.from_buffer_copy(bytes(template)) if template is not None else CarState()
    s.pos.x, s.pos.y, s.pos.z = (float(x) for x in v[0:3] * BT_TO_UU)
    s.vel.x, s.vel.y, s.vel.z = (float(x) for x in v[3:6] * BT_TO_UU)
    s.ang_vel.x, s.ang_vel.y, s.ang_vel.z = (float(x) for x in v[6:9])
    B = [float(x) for x in v[9:18]]
    s.rot_mat.forward.x, s.rot_mat.forward.y, s.rot_mat.forward.z = B[0], B[3], B[6]
    s.rot_mat.right.x, s.rot_mat.right.y, s.rot_mat.right.z = B[1], B[4], B[7]
    s.rot_mat.up.x, s.rot_mat.up.y, s.rot_mat.up.z = B[2], B[5], B[8]
    return s


def ball_state_from_vector(v, template: BallState | None = None) -> BallState:
    """BallState (uu units) with the position and velocity of one 24-float state vector."""
    v = np.asarray(v, np.float32)
    s = BallState.from_buffer_copy(bytes(template)) if template is not None else BallState()
    s.pos.x, s.pos.y, s.pos.z = (float(x) for x in v[18:21] * BT_TO_UU)
    s.vel.x, s.vel.y, s.vel.z = (float(x) for x in v[21:24] * BT_TO_UU)
    return s
