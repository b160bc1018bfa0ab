"""ctypes glue for the two CPU checkers (test infrastructure only).

``RefArena`` drives the reference RocketSim built from its own sources
(oracle/_ref/librsref.so, only present where the reference tree exists);
``OracleArena`` drives the CPU restatement (oracle/_build/liboracle.so).  Both
expose the same small surface so tests can run one scenario through either.
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF_SO = os.path.join(HERE, "_ref", "librsref.so")
ORACLE_SO = os.path.join(HERE, "_build", "liboracle.so")


class Vec3(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float)]


class RotMat(C.Structure):
    _fields_ = [("forward", Vec3), ("right", Vec3), ("up", Vec3)]


class CarControls(C.Structure):
    _fields_ = [("throttle", C.c_float), ("steer", C.c_float), ("pitch", C.c_float), ("yaw", C.c_float),
                ("roll", C.c_float), ("jump", C.c_uint8), ("boost", C.c_uint8), ("handbrake", C.c_uint8),
                ("_pad0", C.c_uint8)]


class BallHitInfo(C.Structure):
    _fields_ = [("is_valid", C.c_uint8), ("_pad0", C.c_uint8 * 3), ("relative_pos_on_ball", Vec3),
                ("ball_pos", Vec3), ("extra_hit_vel", Vec3), ("tick_count_when_hit", C.c_uint64),
                ("tick_count_when_extra_impulse_applied", C.c_uint64)]


class CarState(C.Structure):
    _fields_ = [
        ("pos", Vec3), ("rot_mat", RotMat), ("vel", Vec3), ("ang_vel", Vec3),
        ("tick_count_since_update", C.c_uint64),
        ("is_on_ground", C.c_uint8), ("wheels_with_contact", C.c_uint8 * 4), ("has_jumped", C.c_uint8),
        ("has_double_jumped", C.c_uint8), ("has_flipped", C.c_uint8),
        ("flip_rel_torque", Vec3), ("jump_time", C.c_float), ("flip_time", C.c_float),
        ("is_flipping", C.c_uint8), ("is_jumping", C.c_uint8), ("_pad0", C.c_uint8 * 2),
        ("air_time", C.c_float), ("air_time_since_jump", C.c_float), ("boost", C.c_float),
        ("time_since_boosted", C.c_float), ("is_boosting", C.c_uint8), ("_pad1", C.c_uint8 * 3),
        ("boosting_time", C.c_float), ("is_supersonic", C.c_uint8), ("_pad2", C.c_uint8 * 3),
        ("supersonic_time", C.c_float), ("handbrake_val", C.c_float), ("is_auto_flipping", C.c_uint8),
        ("_pad3", C.c_uint8 * 3), ("auto_flip_timer", C.c_float), ("auto_flip_torque_scale", C.c_float),
        ("world_contact_has_contact", C.c_uint8), ("_pad4", C.c_uint8 * 3), ("world_contact_normal", Vec3),
        ("car_contact_other_car_id", C.c_uint32), ("car_contact_cooldown_timer", C.c_float),
        ("is_demoed", C.c_uint8), ("_pad5", C.c_uint8 * 3), ("demo_respawn_timer", C.c_float),
        ("ball_hit_info", BallHitInfo), ("last_controls", CarControls),
    ]


class BallState(C.Structure):
    _fields_ = [("pos", Vec3), ("rot_mat", RotMat), ("vel", Vec3), ("ang_vel", Vec3),
                ("tick_count_since_update", C.c_uint64)]


class PadState(C.Structure):
    _fields_ = [("is_active", C.c_uint8), ("_pad0", C.c_uint8 * 3), ("cooldown", C.c_float),
                ("cur_locked_car_id", C.c_uint32), ("prev_locked_car_id", C.c_uint32)]


class WheelPairConfig(C.Structure):
    _fields_ = [("wheel_radius", C.c_float), ("suspension_rest_length", C.c_float),
                ("connection_point_offset", Vec3)]


class CarConfig(C.Structure):
    _fields_ = [("hitbox_size", Vec3), ("hitbox_pos_offset", Vec3), ("front_wheels", WheelPairConfig),
                ("back_wheels", WheelPairConfig), ("three_wheels", C.c_uint8), ("_pad0", C.c_uint8 * 3),
                ("dodge_deadzone", C.c_float)]


assert C.sizeof(CarState) == 272, C.sizeof(CarState)
assert C.sizeof(BallState) == 80
assert C.sizeof(PadState) == 16
assert C.sizeof(CarControls) == 24


def build_oracle() -> str:
    """Compile the CPU restatement (fast; safe to call repeatedly)."""
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)
    return ORACLE_SO


def reference_dir() -> str:
    """The reference source tree: $RSG_REFERENCE_DIR, else a checkout named `reference` beside the repository."""
    return os.environ.get("RSG_REFERENCE_DIR", os.path.abspath(os.path.join(HERE, os.pardir, os.pardir, "reference")))


def build_ref() -> str | None:
    """Compile the reference from its sources when they are present here."""
    ref = reference_dir()
    if not os.path.isdir(os.path.join(ref, "src")):
        return REF_SO if os.path.exists(REF_SO) else None
    subprocess.run(["make", "-s", "-C", HERE, f"-j{os.cpu_count() or 4}", "ref", f"REF={ref}"], check=True)
    return REF_SO


def _setup(lib, prefix: str):
    p = prefix
    lib[p + "init"].argtypes = [C.c_char_p, C.c_uint64]
    lib[p + "arena_create"].restype = C.c_void_p
    lib[p + "arena_create"].argtypes = [C.c_int, C.c_float]
    lib[p + "arena_destroy"].argtypes = [C.c_void_p]
    lib[p + "preset"].argtypes = [C.c_int, C.POINTER(CarConfig)]
    lib[p + "add_car"].restype = C.c_uint32
    lib[p + "add_car"].argtypes = [C.c_void_p, C.c_int, C.c_int]
    lib[p + "car_order"].argtypes = [C.c_void_p, C.POINTER(C.c_uint32), C.c_uint32]
    lib[p + "set_controls"].argtypes = [C.c_void_p, C.c_uint32, C.POINTER(CarControls)]
    lib[p + "get_car"].argtypes = [C.c_void_p, C.c_uint32, C.POINTER(CarState)]
    lib[p + "set_car"].argtypes = [C.c_void_p, C.c_uint32, C.POINTER(CarState)]
    lib[p + "get_ball"].argtypes = [C.c_void_p, C.POINTER(BallState)]
    lib[p + "set_ball"].argtypes = [C.c_void_p, C.POINTER(BallState)]
    lib[p + "num_pads"].argtypes = [C.c_void_p]
    lib[p + "get_pad"].argtypes = [C.c_void_p, C.c_int, C.POINTER(PadState)]
    lib[p + "set_pad"].argtypes = [C.c_void_p, C.c_int, C.POINTER(PadState)]
    lib[p + "pad_config"].argtypes = [C.c_void_p, C.c_int, C.POINTER(Vec3), C.POINTER(C.c_int)]
    lib[p + "get_tick"].restype = C.c_uint64
    lib[p + "get_tick"].argtypes = [C.c_void_p]
    lib[p + "set_tick"].argtypes = [C.c_void_p, C.c_uint64]
    lib[p + "step"].argtypes = [C.c_void_p, C.c_int]
    lib[p + "run"].argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int]
    lib[p + "is_scored"].argtypes = [C.c_void_p]
    lib[p + "pop_events"].argtypes = [C.c_void_p, C.POINTER(C.c_uint64), C.c_int]
    lib[p + "get_wheel_internals"].argtypes = [C.c_void_p, C.c_uint32, C.POINTER(C.c_float)]
    lib[p + "wheel_debug"].argtypes = [C.c_void_p, C.c_uint32, C.POINTER(C.c_float)]
    if p == "rsora_":
        lib[p + "set_car_order"].argtypes = [C.c_void_p, C.POINTER(C.c_uint32), C.c_uint32]
        lib[p + "get_counters"].argtypes = [C.c_void_p, C.POINTER(C.c_uint64), C.c_int]


class _Lib:
    def __init__(self, path: str, prefix: str):
        self.dll = C.CDLL(path)
        self.prefix = prefix
        self._fns = {}
        _setup(self, prefix)

    def __getitem__(self, name):
        if name not in self._fns:
            self._fns[name] = getattr(self.dll, name)
        return self._fns[name]


_LIBS: dict[str, _Lib] = {}
_INIT: dict[str, bytes] = {}


def load(kind: str) -> _Lib:
    if kind not in _LIBS:
        if kind == "ref":
            path = build_ref()
            if path is None or not os.path.exists(path):
                raise FileNotFoundError("reference library not available")
            _LIBS[kind] = _Lib(path, "rsref_")
        elif kind == "oracle_sse":
            subprocess.run(["make", "-s", "-C", HERE, "oracle-sse"], check=True)
            _LIBS[kind] = _Lib(os.path.join(HERE, "_build", "liboracle_sse.so"), "rsora_")
        else:
            _LIBS[kind] = _Lib(build_oracle(), "rsora_")
    return _LIBS[kind]


class SimArena:
    """One arena of the reference (kind='ref') or of the restatement (kind='oracle')."""

    def __init__(self, kind: str, cmf: bytes | None, game_mode: int = 0, tick_rate: float = 120.0,
                 config=None):
        self.kind = kind
        self.lib = load(kind)
        p = self.lib.prefix
        self.p = p
        if game_mode != 5:
            if cmf is None:
                raise ValueError("mesh required")
            prev = _INIT.get(kind)
            if prev is None:
                rc = self.lib[p + "init"](cmf, len(cmf))
                if rc != 0:
                    raise RuntimeError("init failed")
                _INIT[kind] = cmf
            elif prev != cmf:
                raise RuntimeError("a different mesh was already loaded in this process")
        if config is None:
            self.h = self.lib[p + "arena_create"](game_mode, tick_rate)
        else:  # an rsg_arena_config mirror (reference library only)
            fn = self.lib[p + "arena_create_ex"]
            fn.restype = C.c_void_p
            fn.argtypes = [C.c_int, C.c_float, C.c_void_p]
            self.h = fn(game_mode, tick_rate, C.addressof(config))
        if not self.h:
            raise RuntimeError("arena_create failed")

    def close(self):
        if self.h:
            self.lib[self.p + "arena_destroy"](self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_car(self, team: int, preset: int = 0) -> int:
        return int(self.lib[self.p + "add_car"](self.h, team, preset))

    def car_order(self) -> list[int]:
        buf = (C.c_uint32 * 16)()
        n = self.lib[self.p + "car_order"](self.h, buf, 16)
        return list(buf[:n])

    def set_controls(self, car_id: int, c: CarControls):
        assert self.lib[self.p + "set_controls"](self.h, car_id, C.byref(c)) == 0

    def get_car(self, car_id: int) -> CarState:
        s = CarState()
        assert self.lib[self.p + "get_car"](self.h, car_id, C.byref(s)) == 0
        return s

    def set_car(self, car_id: int, s: CarState):
        assert self.lib[self.p + "set_car"](self.h, car_id, C.byref(s)) == 0

    def get_ball(self) -> BallState:
        s = BallState()
        self.lib[self.p + "get_ball"](self.h, C.byref(s))
        return s

    def set_ball(self, s: BallState):
        self.lib[self.p + "set_ball"](self.h, C.byref(s))

    def reset_to_random_kickoff(self, seed: int) -> None:
        """Arena::ResetToRandomKickoff (reference library only)."""
        fn = self.lib[self.p + "reset_to_random_kickoff"]
        fn.argtypes = [C.c_void_p, C.c_int]
        fn(self.h, seed)

    def is_ball_probably_going_in(self, max_time: float, extra_margin: float) -> tuple[bool, int]:
        """Arena::IsBallProbablyGoingIn (reference library only): (going in, goal team or -1)."""
        fn = self.lib[self.p + "is_ball_probably_going_in"]
        fn.argtypes = [C.c_void_p, C.c_float, C.c_float, C.POINTER(C.c_int)]
        t = C.c_int()
        r = fn(self.h, max_time, extra_margin, C.byref(t))
        return bool(r), t.value

    def ball_pred_tracker(self, num_pred_ticks: int) -> "RefBallPredTracker":
        """BallPredTracker(arena, numPredTicks) (reference library only)."""
        return RefBallPredTracker(self, num_pred_ticks)

    def num_pads(self) -> int:
        return int(self.lib[self.p + "num_pads"](self.h))

    def get_pad(self, i: int) -> PadState:
        s = PadState()
        assert self.lib[self.p + "get_pad"](self.h, i, C.byref(s)) == 0
        return s

    def set_pad(self, i: int, s: PadState):
        assert self.lib[self.p + "set_pad"](self.h, i, C.byref(s)) == 0

    def get_tick(self) -> int:
        return int(self.lib[self.p + "get_tick"](self.h))

    def set_tick(self, t: int):
        self.lib[self.p + "set_tick"](self.h, t)

    def step(self, ticks: int = 1):
        assert self.lib[self.p + "step"](self.h, ticks) == 0

    def run(self, controls_ptr: int, ncars: int, ticks: int):
        """Steps `ticks` ticks with controls [ticks][ncars] (AddCar order) from native memory."""
        assert self.lib[self.p + "run"](self.h, controls_ptr, ncars, ticks) == 0

    def is_scored(self) -> bool:
        return bool(self.lib[self.p + "is_scored"](self.h))

    def pop_events(self) -> list[tuple[int, int, int, int, int]]:
        buf = (C.c_uint64 * (5 * 256))()
        n = self.lib[self.p + "pop_events"](self.h, buf, 256)
        return [tuple(int(x) for x in buf[i * 5:(i + 1) * 5]) for i in range(n)]

    def set_car_order(self, ids: list[int]):
        arr = (C.c_uint32 * len(ids))(*ids)
        assert self.lib[self.p + "set_car_order"](self.h, arr, len(ids)) == 0

    def counters(self) -> list[int]:
        buf = (C.c_uint64 * 16)()
        n = self.lib[self.p + "get_counters"](self.h, buf, 16)
        return list(buf[:n])

    def wheel_debug(self, car_id: int):
        buf = (C.c_float * 64)()
        self.lib[self.p + "wheel_debug"](self.h, car_id, buf)
        return [list(buf[i * 16:(i + 1) * 16]) for i in range(4)]

    def ball_heatseeker(self) -> tuple[float, float, float]:
        """BallState::hsInfo (yTargetDir, curTargetSpeed, timeSinceHit); reference library only."""
        fn = self.lib[self.p + "get_ball_hs"]
        fn.argtypes = [C.c_void_p, C.POINTER(C.c_float)]
        out = (C.c_float * 3)()
        assert fn(self.h, out) == 0
        return tuple(float(x) for x in out)

    def set_ball_heatseeker(self, hs) -> None:
        """Ball::SetState with the ball's state and the given hsInfo; reference library only."""
        fn = self.lib[self.p + "set_ball_hs"]
        fn.argtypes = [C.c_void_p, C.POINTER(C.c_float)]
        assert fn(self.h, (C.c_float * 3)(*hs)) == 0

    def serialize(self) -> bytes:
        """Arena::Serialize (reference library only)."""
        fn = self.lib[self.p + "serialize"]
        fn.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, C.POINTER(C.c_uint64)]
        n = C.c_uint64()
        fn(self.h, None, 0, C.byref(n))
        buf = (C.c_uint8 * n.value)()
        fn(self.h, buf, n.value, C.byref(n))
        return bytes(buf)

    @classmethod
    def deserialize_new(cls, data: bytes) -> "SimArena":
        """Arena::DeserializeNew (reference library only)."""
        self = cls.__new__(cls)
        self.kind, self.lib = "ref", load("ref")
        self.p = self.lib.prefix
        fn = self.lib[self.p + "deserialize_new"]
        fn.restype = C.c_void_p
        fn.argtypes = [C.c_void_p, C.c_uint64]
        buf = (C.c_uint8 * len(data)).from_buffer_copy(data)
        self.h = fn(buf, len(data))
        if not self.h:
            raise RuntimeError("DeserializeNew failed")
        return self

    def clone(self) -> "SimArena":
        """Arena::Clone (reference library only)."""
        other = type(self).__new__(type(self))
        other.kind, other.lib, other.p = self.kind, self.lib, self.p
        fn = self.lib[self.p + "clone"]
        fn.restype = C.c_void_p
        fn.argtypes = [C.c_void_p]
        other.h = fn(self.h)
        return other

    def set_mutator_config(self, config) -> None:
        """Arena::SetMutatorConfig from an rsg_mutator_config mirror (reference library only)."""
        fn = self.lib[self.p + "set_mutator_config"]
        fn.argtypes = [C.c_void_p, C.c_void_p]
        buf = C.create_string_buffer(bytes(config), len(bytes(config)))
        assert fn(self.h, buf) == 0

    def vehicle_state(self, car_id: int) -> list[float]:
        """Front steer angle, engine force, brake, lateral (4), longitudinal (4) friction
        factors and extra push-back (4) of a car (reference library only)."""
        buf = (C.c_float * 15)()
        fn = self.lib[self.p + "get_vehicle_state"]
        fn.argtypes = [C.c_void_p, C.c_uint32, C.POINTER(C.c_float)]
        assert fn(self.h, car_id, buf) == 0
        return list(buf)

    def wheel_internals(self, car_id: int) -> list[float]:
        buf = (C.c_float * 8)()
        self.lib[self.p + "get_wheel_internals"](self.h, car_id, buf)
        return list(buf)


def preset(kind: str, idx: int) -> CarConfig:
    lib = load(kind)
    c = CarConfig()
    assert lib[lib.prefix + "preset"](idx, C.byref(c)) == 0
    return c


class RefBallPredTracker:
    """The reference's BallPredTracker (src/Sim/BallPredTracker/BallPredTracker.cpp) over a SimArena."""

    def __init__(self, arena: SimArena, num_pred_ticks: int):
        self.lib, self.p, self.T = arena.lib, arena.p, num_pred_ticks
        fn = self.lib[self.p + "ballpred_create"]
        fn.restype, fn.argtypes = C.c_void_p, [C.c_void_p, C.c_uint32]
        self.h = fn(arena.h, num_pred_ticks)
        for name, args in (("ballpred_destroy", [C.c_void_p]), ("ballpred_update_from_arena", [C.c_void_p, C.c_void_p]),
                           ("ballpred_update_manual", [C.c_void_p, C.c_void_p, C.c_int]),
                           ("ballpred_force_update_all", [C.c_void_p, C.c_void_p]),
                           ("ballpred_get", [C.c_void_p, C.c_void_p, C.c_int]),
                           ("ballpred_state_for_time", [C.c_void_p, C.c_float, C.c_void_p]),
                           ("ballpred_last_update_tick", [C.c_void_p])):
            self.lib[self.p + name].argtypes = args

    def update_from_arena(self, arena: SimArena) -> None:
        self.lib[self.p + "ballpred_update_from_arena"](self.h, arena.h)

    def update_manual(self, state: BallState, ticks: int) -> None:
        self.lib[self.p + "ballpred_update_manual"](self.h, C.byref(state), ticks)

    def force_update_all(self, state: BallState) -> None:
        self.lib[self.p + "ballpred_force_update_all"](self.h, C.byref(state))

    def pred_data(self) -> list:
        buf = (BallState * self.T)()
        n = self.lib[self.p + "ballpred_get"](self.h, buf, self.T)
        return [buf[i] for i in range(n)]

    def state_for_time(self, t: float) -> BallState:
        s = BallState()
        self.lib[self.p + "ballpred_state_for_time"](self.h, t, C.byref(s))
        return s

    def last_update_tick(self) -> int:
        return int(self.lib[self.p + "ballpred_last_update_tick"](self.h))

    def close(self) -> None:
        if self.h:
            self.lib[self.p + "ballpred_destroy"](self.h)
            self.h = None
