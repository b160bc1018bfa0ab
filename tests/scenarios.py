"""Seeded scenario generator and runners shared by the parity tests.

A scenario is one arena: cars with a config preset and team, their starting
CarState, the ball's starting BallState, the per-car update order and a
control sequence (the input process of the 2v2 workload: analog inputs
uniform in [-1, 1], jump/boost/handbrake Bernoulli(0.3), each car re-drawing
after a hold of 2..60 ticks).  Runners play a scenario on a CPU checker
(oracle.pyoracle.SimArena: the reference build or the restatement) or on the
GPU through the C ABI (rocketsim_gb300.ArenaBatch, many scenarios at once).
"""
from __future__ import annotations

import ctypes as C
import math
import os
import sys
from dataclasses import dataclass, field

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

from rocketsim_gb300 import abi  # noqa: E402
from rocketsim_gb300.arena_mesh import arena_cmf  # noqa: E402

MESH_SEED = 0
_CMF = None


def mesh_bytes() -> bytes:
    global _CMF
    if _CMF is None:
        _CMF = arena_cmf(MESH_SEED)
    return _CMF


def rot_cols(q) -> np.ndarray:
    """Rotation matrix (columns forward/right/up) of a unit quaternion (w, x, y, z)."""
    w, x, y, z = q
    return np.array([
        [1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
        [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
        [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)],
    ], dtype=np.float64)


def set_rot(rm, M):
    M = M.astype(np.float32)
    rm.forward = abi.Vec3(*map(float, M[:, 0]))
    rm.right = abi.Vec3(*map(float, M[:, 1]))
    rm.up = abi.Vec3(*map(float, M[:, 2]))


@dataclass
class Scenario:
    seed: int
    presets: list[int]
    teams: list[int]
    cars: list[abi.CarState]
    ball: abi.BallState
    order: list[int]                      # update order as indices into the car list
    controls: np.ndarray                  # [T, ncars] CONTROLS dtype
    pads: list[abi.PadState] = field(default_factory=list)


CONTROLS_DTYPE = np.dtype(abi.CarControls)


def control_sequence(rng: np.random.Generator, ticks: int, ncars: int) -> np.ndarray:
    out = np.zeros((ticks, ncars), CONTROLS_DTYPE)
    for c in range(ncars):
        t = 0
        while t < ticks:
            hold = int(rng.integers(2, 61))
            a = rng.uniform(-1, 1, 5).astype(np.float32)
            b = (rng.random(3) < 0.3).astype(np.uint8)
            sl = slice(t, min(ticks, t + hold))
            for k, name in enumerate(("throttle", "steer", "pitch", "yaw", "roll")):
                out[name][sl, c] = a[k]
            for k, name in enumerate(("jump", "boost", "handbrake")):
                out[name][sl, c] = b[k]
            t += hold
    return out


def make_scenario(seed: int, ncars: int = 4, ticks: int = 120, presets: list[int] | None = None,
                  air_frac: float = 0.3, max_car_speed: float = 2300.0, max_ball_speed: float = 3000.0,
                  random_order: bool = True) -> Scenario:
    rng = np.random.default_rng(seed)
    presets = list(presets) if presets is not None else [0] * ncars
    teams = [i % 2 for i in range(ncars)]
    cars = []
    for i in range(ncars):
        s = abi.CarState()
        s.ball_hit_info.tick_count_when_hit = (1 << 64) - 1
        s.ball_hit_info.tick_count_when_extra_impulse_applied = (1 << 64) - 1
        x, y = rng.uniform(-3500, 3500), rng.uniform(-4500, 4500)
        if rng.random() < air_frac:
            q = rng.normal(size=4)
            q /= np.linalg.norm(q)
            M = rot_cols(q)
            d = rng.normal(size=3)
            d /= np.linalg.norm(d)
            v = d * rng.uniform(0, max_car_speed)
            s.pos = abi.Vec3(x, y, rng.uniform(300, 1500))
            s.vel = abi.Vec3(*map(float, v))
            s.ang_vel = abi.Vec3(*map(float, rng.uniform(-3, 3, 3)))
            s.is_on_ground = 0
            s.has_jumped = int(rng.random() < 0.5)
        else:
            yaw = rng.uniform(0, 2 * math.pi)
            M = rot_cols((math.cos(yaw / 2), 0.0, 0.0, math.sin(yaw / 2)))
            sp = rng.uniform(0, 1400)
            s.pos = abi.Vec3(x, y, 17.0)
            s.vel = abi.Vec3(float(M[0, 0] * sp), float(M[1, 0] * sp), 0.0)
            s.is_on_ground = 1
        set_rot(s.rot_mat, M)
        s.boost = float(rng.uniform(0, 100))
        cars.append(s)
    b = abi.BallState()
    b.pos = abi.Vec3(rng.uniform(-3000, 3000), rng.uniform(-4000, 4000), rng.uniform(93.15, 1500))
    set_rot(b.rot_mat, np.eye(3))
    d = rng.normal(size=3)
    d /= np.linalg.norm(d)
    b.vel = abi.Vec3(*map(float, d * rng.uniform(0, max_ball_speed)))
    b.ang_vel = abi.Vec3(*map(float, rng.uniform(-2, 2, 3)))
    order = list(rng.permutation(ncars)) if random_order else list(range(ncars))
    ctl = control_sequence(rng, ticks, ncars)
    return Scenario(seed, presets, teams, cars, b, [int(o) for o in order], ctl)


def make_carcar_scenario(seed: int, ticks: int = 120) -> Scenario:
    """Two cars on the ground driving into each other at 800..2300 uu/s (full throttle and
    boost), so that bumps and demolitions happen within the first 30 ticks."""
    rng = np.random.default_rng(seed)
    sc = make_scenario(seed, ncars=2, ticks=ticks, air_frac=0.0, random_order=False)
    x0, y0 = rng.uniform(-2000, 2000), rng.uniform(-2000, 2000)
    ang = rng.uniform(0, 2 * math.pi)
    for i, s in enumerate(sc.cars):
        yaw = ang + (math.pi if i else 0) + rng.uniform(-0.6, 0.6)
        off = (-1 if i == 0 else 1) * 260
        M = rot_cols((math.cos(yaw / 2), 0, 0, math.sin(yaw / 2)))
        set_rot(s.rot_mat, M)
        sp = rng.uniform(800, 2300)
        s.pos = abi.Vec3(x0 + off * math.cos(ang), y0 + off * math.sin(ang), 17.0)
        s.vel = abi.Vec3(float(M[0, 0] * sp), float(M[1, 0] * sp), 0.0)
        s.is_supersonic = int(sp > 2200)
    sc.controls["throttle"] = 1.0
    sc.controls["boost"] = 1
    sc.controls["jump"] = 0
    return sc


def _controls_struct(row) -> abi.CarControls:
    c = abi.CarControls()
    c.throttle, c.steer, c.pitch, c.yaw, c.roll = (float(row[k]) for k in ("throttle", "steer", "pitch", "yaw", "roll"))
    c.jump, c.boost, c.handbrake = (int(row[k]) for k in ("jump", "boost", "handbrake"))
    return c


# ---------------------------------------------------------------- CPU checkers
def setup_cpu(kind: str, sc: Scenario, mutators=None, config=None, game_mode: int = 0):
    """Builds the scenario on a SimArena of `kind` ('ref', 'oracle', 'oracle_sse'); `mutators` (an
    abi.MutatorConfig) is set before the cars are added and `config` (an abi.ArenaConfig) passed
    to Arena::Create, both for the reference only."""
    from oracle.pyoracle import SimArena, CarState as OCarState, BallState as OBallState, CarControls as OCtl
    a = SimArena(kind, mesh_bytes(), game_mode=game_mode, config=config)
    if mutators is not None:
        a.set_mutator_config(mutators)
    ids = [a.add_car(t, p) for t, p in zip(sc.teams, sc.presets)]
    for cid, s in zip(ids, sc.cars):
        a.set_car(cid, OCarState.from_buffer_copy(bytes(s)))
    a.set_ball(OBallState.from_buffer_copy(bytes(sc.ball)))
    order = [ids[i] for i in sc.order]
    if kind == "ref":
        # the reference iterates its cars in hash-set order; the scenario follows it
        ref_order = a.car_order()
        sc.order = [ids.index(i) for i in ref_order]
    else:
        a.set_car_order(order)
    return a, ids


def run_cpu(kind: str, sc: Scenario, ticks: int, record=None, mutators=None, config=None):
    """Steps a fresh checker arena through `ticks` ticks of the scenario.

    `record(t, arena, ids)` is called after each tick."""
    from oracle.pyoracle import CarControls as OCtl
    a, ids = setup_cpu(kind, sc, mutators, config)
    for t in range(ticks):
        for i, cid in enumerate(ids):
            a.set_controls(cid, OCtl.from_buffer_copy(bytes(_controls_struct(sc.controls[t, i]))))
        a.step(1)
        if record:
            record(t, a, ids)
    return a, ids


def cpu_snapshot(a, ids):
    cars = np.frombuffer(b"".join(bytes(a.get_car(c)) for c in ids), np.dtype(abi.CarState)).copy()
    ball = np.frombuffer(bytes(a.get_ball()), np.dtype(abi.BallState)).copy()
    pads = np.frombuffer(b"".join(bytes(a.get_pad(i)) for i in range(a.num_pads())), np.dtype(abi.PadState)).copy()
    return cars, ball, pads


# ---------------------------------------------------------------- GPU
def setup_gpu(scs: list[Scenario], max_cars: int | None = None, mutators=None, config=None,
              game_mode: int = abi.GAMEMODE_SOCCAR):
    """One ArenaBatch holding one arena per scenario (`mutators` set before the cars are added,
    `config` an abi.ArenaConfig for the batch)."""
    import rocketsim_gb300 as rsg
    rsg.init_from_mem([mesh_bytes()])
    mc = max_cars or max(len(s.cars) for s in scs)
    batch = rsg.ArenaBatch(game_mode, len(scs), mc, 120.0, config)
    if mutators is not None:
        batch.set_mutator_config(mutators)
    all_ids = []
    for ai, sc in enumerate(scs):
        ids = [batch.add_car(ai, t, p, 0) for t, p in zip(sc.teams, sc.presets)]
        for cid, s in zip(ids, sc.cars):
            batch.set_car_state(ai, cid, s)
        batch.set_ball_state(ai, sc.ball)
        batch.set_car_update_order(ai, [ids[i] for i in sc.order])
        all_ids.append(ids)
    return batch, all_ids


def gpu_controls(scs: list[Scenario], t: int, mc: int) -> np.ndarray:
    out = np.zeros(len(scs) * mc, CONTROLS_DTYPE)
    for ai, sc in enumerate(scs):
        n = sc.controls.shape[1]
        out[ai * mc:ai * mc + n] = sc.controls[t]
    return out


def gpu_snapshot(batch, scs: list[Scenario]):
    cars, balls, pads = batch.get_all_states()
    mc = batch.max_cars
    out = []
    for ai, sc in enumerate(scs):
        n = len(sc.cars)
        out.append((cars[ai * mc:ai * mc + n].copy(), balls[ai:ai + 1].copy(),
                    pads[ai * batch.num_pads:(ai + 1) * batch.num_pads].copy()))
    return out


# ---------------------------------------------------------------- comparison
CONT_FIELDS = ("pos", "vel", "ang_vel")


def car_vec(cars: np.ndarray) -> np.ndarray:
    """[n, 9+9] float64: pos, vel, ang_vel, rot_mat."""
    parts = []
    for f in CONT_FIELDS:
        parts += [cars[f]["x"], cars[f]["y"], cars[f]["z"]]
    for col in ("forward", "right", "up"):
        parts += [cars["rot_mat"][col]["x"], cars["rot_mat"][col]["y"], cars["rot_mat"][col]["z"]]
    return np.stack(parts, axis=-1).astype(np.float64)


def ball_vec(ball: np.ndarray) -> np.ndarray:
    parts = []
    for f in CONT_FIELDS:
        parts += [ball[f]["x"], ball[f]["y"], ball[f]["z"]]
    return np.stack(parts, axis=-1).astype(np.float64)


CAR_DISCRETE = ("is_on_ground", "has_jumped", "has_double_jumped", "has_flipped", "is_flipping", "is_jumping",
                "is_boosting", "is_supersonic", "is_auto_flipping", "is_demoed", "world_contact_has_contact",
                "car_contact_other_car_id")
CAR_TIMERS = ("jump_time", "flip_time", "air_time", "air_time_since_jump", "boost", "time_since_boosted",
              "boosting_time", "supersonic_time", "handbrake_val", "auto_flip_timer", "demo_respawn_timer",
              "car_contact_cooldown_timer")


def discrete_car(cars: np.ndarray) -> np.ndarray:
    cols = [cars[k].astype(np.float64) for k in CAR_DISCRETE]
    cols += [cars["wheels_with_contact"][:, w].astype(np.float64) for w in range(4)]
    cols += [cars[k].astype(np.float64) for k in CAR_TIMERS]
    return np.stack(cols, axis=-1)


def discrete_pads(pads: np.ndarray) -> np.ndarray:
    return np.stack([pads["is_active"].astype(np.float64), pads["cooldown"].astype(np.float64),
                     pads["prev_locked_car_id"].astype(np.float64)], axis=-1)


HIT_COUNTERS = ("is_valid", "tick_count_when_hit", "tick_count_when_extra_impulse_applied")


def discrete_hit(cars: np.ndarray) -> np.ndarray:
    """[n, 4] uint64: ballHitInfo.isValid, tickCountWhenHit, tickCountWhenExtraImpulseApplied and
    CarState::tickCountSinceUpdate (BallHitInfo.h:9-26, Car.h:17-120), compared bit for bit."""
    hi = cars["ball_hit_info"]
    cols = [hi[k].astype(np.uint64) for k in HIT_COUNTERS]
    cols.append(cars["tick_count_since_update"].astype(np.uint64))
    return np.stack(cols, axis=-1)


def hit_vec(cars: np.ndarray) -> np.ndarray:
    """[n, 9] float64: ballHitInfo.relativePosOnBall, ballPos and extraHitVel (uu, uu/s)."""
    hi = cars["ball_hit_info"]
    parts = []
    for f in ("relative_pos_on_ball", "ball_pos", "extra_hit_vel"):
        parts += [hi[f]["x"], hi[f]["y"], hi[f]["z"]]
    return np.stack(parts, axis=-1).astype(np.float64)
