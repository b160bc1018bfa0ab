"""Host API over the C ABI, mirroring RocketSim's Arena / Car / Ball classes.

``ArenaBatch`` is the batched form (many independent arenas stepped together
on the GPU); ``Arena`` is a one-arena view with the reference's method names
(src/Sim/Arena/Arena.h:60-140, src/Sim/Car/Car.h:140-160,
src/Sim/Ball/Ball.h:60-75) so code written against RocketSim reads the same.
"""
from __future__ import annotations

import ctypes as C
from typing import Callable, Iterable

import numpy as np

from . import abi
from .abi import (BallState, CarConfig, CarControls, CarState, PadState, Vec3, check)

_MESH_LOADED: dict[int, bytes] = {}


def init_from_mem(meshes: Iterable[bytes], game_mode: int = abi.GAMEMODE_SOCCAR) -> None:
    """RocketSim::InitFromMem (src/RocketSim.cpp:92-185) for one game mode."""
    lib = abi.load()
    blobs = [bytes(m) for m in meshes]
    n = len(blobs)
    bufs = [(C.c_uint8 * len(b)).from_buffer_copy(b) for b in blobs]
    ptrs = (C.POINTER(C.c_uint8) * n)(*[C.cast(b, C.POINTER(C.c_uint8)) for b in bufs])
    sizes = (C.c_uint64 * n)(*[len(b) for b in blobs])
    check(lib.rsg_init_from_mem(game_mode, ptrs, sizes, n), "rsg_init_from_mem")
    _MESH_LOADED[game_mode] = blobs[0] if blobs else b""


def init(path: str, game_mode: int = abi.GAMEMODE_SOCCAR) -> None:
    """RocketSim::Init(path) (src/RocketSim.cpp:53-90): loads every .cmf file of a folder."""
    import os
    files = sorted(f for f in os.listdir(path) if f.endswith(".cmf"))
    blobs = []
    for f in files:
        with open(os.path.join(path, f), "rb") as fh:
            blobs.append(fh.read())
    init_from_mem(blobs, game_mode)


def arena_config(custom_boost_pads=None, no_ball_rot: bool = True) -> "abi.ArenaConfig":
    """ArenaConfig with its defaults; `custom_boost_pads` (a list of (x, y, z, is_big), uu) switches
    to custom pads.  The returned struct keeps the pad array alive."""
    c = abi.ArenaConfig()
    check(abi.load().rsg_get_default_arena_config(C.byref(c)), "rsg_get_default_arena_config")
    c.no_ball_rot = 1 if no_ball_rot else 0
    if custom_boost_pads is not None:
        arr = (abi.BoostPadConfig * max(len(custom_boost_pads), 1))()
        for i, (x, y, z, big) in enumerate(custom_boost_pads):
            arr[i].pos = abi.Vec3(float(x), float(y), float(z))
            arr[i].is_big = 1 if big else 0
        c.use_custom_boost_pads = 1
        c.num_custom_boost_pads = len(custom_boost_pads)
        c.custom_boost_pads = C.cast(arr, C.POINTER(abi.BoostPadConfig))
        c._pads_keepalive = arr
    return c


def default_mutator_config(game_mode: int = abi.GAMEMODE_SOCCAR) -> "abi.MutatorConfig":
    """MutatorConfig(GameMode): the game mode's default mutators."""
    m = abi.MutatorConfig()
    check(abi.load().rsg_get_default_mutator_config(game_mode, C.byref(m)), "rsg_get_default_mutator_config")
    return m


def car_config(preset: int = abi.CAR_OCTANE) -> CarConfig:
    c = CarConfig()
    check(abi.load().rsg_get_car_config_preset(preset, C.byref(c)), "rsg_get_car_config_preset")
    return c


CAR_STATE_DTYPE = np.dtype(CarState)
BALL_STATE_DTYPE = np.dtype(BallState)
PAD_STATE_DTYPE = np.dtype(PadState)
CONTROLS_DTYPE = np.dtype(CarControls)


class ArenaBatch:
    """``n_arenas`` independent arenas of one game mode on the current CUDA device."""

    def __init__(self, game_mode: int = abi.GAMEMODE_SOCCAR, n_arenas: int = 1, max_cars: int = 4,
                 tick_rate: float = 120.0, config: "abi.ArenaConfig | None" = None):
        self.lib = abi.load()
        if config is None:
            h = self.lib.rsg_batch_create(game_mode, n_arenas, max_cars, tick_rate)
        else:
            h = self.lib.rsg_batch_create_ex(game_mode, n_arenas, max_cars, tick_rate, C.byref(config))
        if not h:
            raise abi.RSGError(abi.ERR_STATE, "rsg_batch_create")
        self.h = C.c_void_p(h)
        n = C.c_uint32()
        check(self.lib.rsg_batch_num_pads(self.h, C.byref(n)), "rsg_batch_num_pads")
        self.num_pads = n.value
        self.game_mode = game_mode
        self.n_arenas = n_arenas
        self.max_cars = max_cars
        self.tick_rate = tick_rate
        self._cbs = {}

    # ---- lifecycle
    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.rsg_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---- cars
    def add_car(self, arena: int, team: int, config: CarConfig | int = abi.CAR_OCTANE, respawn_index: int = -1) -> int:
        cfg = car_config(config) if isinstance(config, int) else config
        out = C.c_uint32()
        check(self.lib.rsg_add_car(self.h, arena, team, C.byref(cfg), respawn_index, C.byref(out)), "rsg_add_car")
        return int(out.value)

    def remove_car(self, arena: int, car_id: int) -> None:
        check(self.lib.rsg_remove_car(self.h, arena, car_id), "rsg_remove_car")

    def get_cars(self, arena: int) -> list[int]:
        buf = (C.c_uint32 * abi.MAX_CARS_PER_ARENA)()
        n = C.c_uint32()
        check(self.lib.rsg_get_car_ids(self.h, arena, buf, abi.MAX_CARS_PER_ARENA, C.byref(n)), "rsg_get_car_ids")
        return list(buf[:n.value])

    def set_car_update_order(self, arena: int, ids: list[int]) -> None:
        arr = (C.c_uint32 * len(ids))(*ids)
        check(self.lib.rsg_set_car_update_order(self.h, arena, arr, len(ids)), "rsg_set_car_update_order")

    def set_controls(self, arena: int, car_id: int, controls: CarControls) -> None:
        check(self.lib.rsg_set_car_controls(self.h, arena, car_id, C.byref(controls)), "rsg_set_car_controls")

    def set_controls_all(self, controls: np.ndarray) -> None:
        """controls: array of CONTROLS_DTYPE with n_arenas * max_cars entries ([arena][slot])."""
        arr = np.ascontiguousarray(controls, dtype=CONTROLS_DTYPE)
        check(self.lib.rsg_set_controls_all(self.h, arr.ctypes.data, arr.size), "rsg_set_controls_all")

    def get_car_state(self, arena: int, car_id: int) -> CarState:
        s = CarState()
        check(self.lib.rsg_get_car_state(self.h, arena, car_id, C.byref(s)), "rsg_get_car_state")
        return s

    def set_car_state(self, arena: int, car_id: int, state: CarState) -> None:
        check(self.lib.rsg_set_car_state(self.h, arena, car_id, C.byref(state)), "rsg_set_car_state")

    def demolish(self, arena: int, car_id: int, respawn_delay: float = 3.0) -> None:
        check(self.lib.rsg_demolish_car(self.h, arena, car_id, respawn_delay), "rsg_demolish_car")

    # ---- ball, pads, arena
    # ---- kickoffs and goal prediction
    def reset_to_random_kickoff(self, arena: int, seed: int = -1) -> None:
        """Arena::ResetToRandomKickoff(seed)."""
        check(self.lib.rsg_reset_to_random_kickoff(self.h, arena, seed), "rsg_reset_to_random_kickoff")

    def reset_to_random_kickoff_many(self, arenas, seeds=None) -> None:
        """ResetToRandomKickoff of arenas[k] with seeds[k] (None: -1 for all) in one transfer."""
        ar = np.ascontiguousarray(arenas, np.uint32)
        sd = None if seeds is None else np.ascontiguousarray(seeds, np.int32)
        check(self.lib.rsg_reset_to_random_kickoff_many(
            self.h, ar.ctypes.data_as(C.POINTER(C.c_uint32)),
            None if sd is None else sd.ctypes.data_as(C.POINTER(C.c_int32)), len(ar)), "rsg_reset_to_random_kickoff_many")

    def is_ball_probably_going_in(self, max_time: float = 2.0, extra_margin: float = 0.0):
        """Arena::IsBallProbablyGoingIn of every arena: (going_in [n_arenas] bool, goal team [n_arenas], -1 if none)."""
        out = np.zeros(self.n_arenas, np.int32)
        team = np.zeros(self.n_arenas, np.int32)
        check(self.lib.rsg_is_ball_probably_going_in(self.h, max_time, extra_margin,
                                                     out.ctypes.data_as(C.POINTER(C.c_int32)),
                                                     team.ctypes.data_as(C.POINTER(C.c_int32))),
              "rsg_is_ball_probably_going_in")
        return out.astype(bool), team

    # ---- serialisation (Arena::Serialize / DeserializeNew / Clone, RocketSim's byte format)
    def serialize(self, arena: int) -> bytes:
        n = C.c_uint64()
        check(self.lib.rsg_serialize_arena(self.h, arena, None, 0, C.byref(n)), "rsg_serialize_arena")
        buf = (C.c_uint8 * n.value)()
        check(self.lib.rsg_serialize_arena(self.h, arena, buf, n.value, C.byref(n)), "rsg_serialize_arena")
        return bytes(buf)

    def deserialize(self, arena: int, data: bytes) -> None:
        buf = (C.c_uint8 * len(data)).from_buffer_copy(data)
        check(self.lib.rsg_deserialize_arena(self.h, arena, buf, len(data)), "rsg_deserialize_arena")

    def clone_arena_from(self, arena: int, src: "ArenaBatch", src_arena: int) -> None:
        check(self.lib.rsg_clone_arena(self.h, arena, src.h, src_arena), "rsg_clone_arena")

    # ---- mutators (Arena::SetMutatorConfig / GetMutatorConfig, for every arena of the batch)
    def get_mutator_config(self) -> "abi.MutatorConfig":
        m = abi.MutatorConfig()
        check(self.lib.rsg_get_mutator_config(self.h, C.byref(m)), "rsg_get_mutator_config")
        return m

    def set_mutator_config(self, config: "abi.MutatorConfig") -> None:
        check(self.lib.rsg_set_mutator_config(self.h, C.byref(config)), "rsg_set_mutator_config")

    def get_ball_state(self, arena: int) -> BallState:
        s = BallState()
        check(self.lib.rsg_get_ball_state(self.h, arena, C.byref(s)), "rsg_get_ball_state")
        return s

    def set_ball_state(self, arena: int, state: BallState) -> None:
        check(self.lib.rsg_set_ball_state(self.h, arena, C.byref(state)), "rsg_set_ball_state")

    def get_ball_heatseeker(self, arena: int) -> "abi.HeatseekerInfo":
        """BallState::hsInfo: (y_target_dir, cur_target_speed, time_since_hit)."""
        s = abi.HeatseekerInfo()
        check(self.lib.rsg_get_ball_heatseeker(self.h, arena, C.byref(s)), "rsg_get_ball_heatseeker")
        return s

    def set_ball_heatseeker(self, arena: int, info: "abi.HeatseekerInfo") -> None:
        check(self.lib.rsg_set_ball_heatseeker(self.h, arena, C.byref(info)), "rsg_set_ball_heatseeker")

    def get_pad_state(self, arena: int, pad: int) -> PadState:
        s = PadState()
        check(self.lib.rsg_get_pad_state(self.h, arena, pad, C.byref(s)), "rsg_get_pad_state")
        return s

    def set_pad_state(self, arena: int, pad: int, state: PadState) -> None:
        check(self.lib.rsg_set_pad_state(self.h, arena, pad, C.byref(state)), "rsg_set_pad_state")

    def get_pad_config(self, pad: int) -> tuple[tuple[float, float, float], bool]:
        v = Vec3()
        big = C.c_int()
        check(self.lib.rsg_get_pad_config(self.h, pad, C.byref(v), C.byref(big)), "rsg_get_pad_config")
        return (v.x, v.y, v.z), bool(big.value)

    def get_tick_count(self, arena: int) -> int:
        t = C.c_uint64()
        check(self.lib.rsg_get_tick_count(self.h, arena, C.byref(t)), "rsg_get_tick_count")
        return int(t.value)

    def set_tick_count(self, arena: int, tick: int) -> None:
        check(self.lib.rsg_set_tick_count(self.h, arena, tick), "rsg_set_tick_count")

    def is_ball_scored(self, arena: int) -> bool:
        out = C.c_int()
        check(self.lib.rsg_is_ball_scored(self.h, arena, C.byref(out)), "rsg_is_ball_scored")
        return bool(out.value)

    # ---- bulk state
    def get_all_states(self, cars: np.ndarray | None = None, balls: np.ndarray | None = None,
                       pads: np.ndarray | None = None):
        A, M = self.n_arenas, self.max_cars
        cars = np.zeros(A * M, CAR_STATE_DTYPE) if cars is None else cars
        balls = np.zeros(A, BALL_STATE_DTYPE) if balls is None else balls
        has_pads = self.game_mode != abi.GAMEMODE_THE_VOID
        if pads is None and has_pads:
            pads = np.zeros(A * self.num_pads, PAD_STATE_DTYPE)
        check(self.lib.rsg_get_all_states(self.h, cars.ctypes.data, balls.ctypes.data,
                                          pads.ctypes.data if pads is not None else None), "rsg_get_all_states")
        return cars, balls, pads

    def set_all_states(self, cars: np.ndarray | None, balls: np.ndarray | None, pads: np.ndarray | None = None):
        check(self.lib.rsg_set_all_states(self.h, cars.ctypes.data if cars is not None else None,
                                          balls.ctypes.data if balls is not None else None,
                                          pads.ctypes.data if pads is not None else None), "rsg_set_all_states")

    def device_flags(self) -> np.ndarray:
        out = np.zeros(self.n_arenas, np.uint32)
        check(self.lib.rsg_get_device_flags(self.h, out.ctypes.data_as(C.POINTER(C.c_uint32))), "rsg_get_device_flags")
        return out

    # ---- stepping
    def tick_shape(self) -> tuple[int, int, int, int, int, int]:
        """Launch shape of the tick kernel (arenas per block, threads per car, header cache, leaf grid,
        collision barriers, persistent launch)."""
        out = (C.c_int32 * 6)()
        check(self.lib.rsg_get_tick_shape(self.h, out), "rsg_get_tick_shape")
        return tuple(int(x) for x in out)

    def tuning_log(self) -> str:
        buf = C.create_string_buffer(65536)
        check(self.lib.rsg_get_tuning_log(self.h, buf, 65536), "rsg_get_tuning_log")
        return buf.value.decode()

    def step(self, ticks: int = 1) -> None:
        check(self.lib.rsg_step(self.h, ticks), "rsg_step")

    def step_controls(self, controls: np.ndarray, ticks: int) -> None:
        """Steps `ticks` ticks with host controls for every tick ([ticks][arena][slot] CONTROLS_DTYPE)."""
        if controls.dtype != CONTROLS_DTYPE or controls.size != ticks * self.n_arenas * self.max_cars:
            raise ValueError("controls must be ticks * n_arenas * max_cars CONTROLS_DTYPE entries")
        c = np.ascontiguousarray(controls)
        check(self.lib.rsg_step_controls(self.h, c.ctypes.data, ticks), "rsg_step_controls")

    def step_async(self, d_controls_ptr: int | None, ticks: int) -> None:
        check(self.lib.rsg_step_async(self.h, d_controls_ptr, ticks), "rsg_step_async")

    def sync(self) -> None:
        check(self.lib.rsg_sync(self.h), "rsg_sync")

    def stream(self) -> int:
        return int(self.lib.rsg_batch_stream(self.h) or 0)

    # ---- callbacks (Arena::SetGoalScoreCallback / SetCarBumpCallback, Arena.h:98-108)
    def set_goal_score_callback(self, fn: Callable[[int, int], None] | None) -> None:
        cb = abi.GOAL_FN(lambda b, arena, team, u: fn(arena, team)) if fn else abi.GOAL_FN()
        self._cbs["goal"] = cb
        check(self.lib.rsg_set_goal_callback(self.h, cb, None), "rsg_set_goal_callback")

    def set_car_bump_callback(self, fn: Callable[[int, int, int, bool], None] | None) -> None:
        cb = abi.BUMP_FN(lambda b, arena, x, y, demo, u: fn(arena, x, y, bool(demo))) if fn else abi.BUMP_FN()
        self._cbs["bump"] = cb
        check(self.lib.rsg_set_bump_callback(self.h, cb, None), "rsg_set_bump_callback")

    def set_ball_hit_callback(self, fn: Callable[[int, int, int], None] | None) -> None:
        cb = abi.BALL_HIT_FN(lambda b, arena, car, tick, u: fn(arena, car, tick)) if fn else abi.BALL_HIT_FN()
        self._cbs["hit"] = cb
        check(self.lib.rsg_set_ball_hit_callback(self.h, cb, None), "rsg_set_ball_hit_callback")


class BallPredTracker:
    """BallPredTracker (src/Sim/BallPredTracker/BallPredTracker.h:7-35) for every arena of a batch:
    each arena gets a ball-only shadow arena and `num_pred_ticks` predicted ball states on the device.
    Creation predicts from the batch's balls, as the reference's constructor does."""

    def __init__(self, batch: ArenaBatch, num_pred_ticks: int):
        self.lib, self.n_arenas, self.num_pred_ticks = batch.lib, batch.n_arenas, num_pred_ticks
        self.h = self.lib.rsg_ball_pred_create(batch.h, num_pred_ticks)
        if not self.h:
            raise RuntimeError(abi.last_error())

    @staticmethod
    def _mask(mask):
        if mask is None:
            return None
        m = np.ascontiguousarray(mask, np.uint8)
        return m, m.ctypes.data_as(C.c_void_p)

    def update_from_batch(self, batch: ArenaBatch, mask=None) -> None:
        """UpdatePredFromArena for every arena (mask[a] != 0)."""
        m = self._mask(mask)
        check(self.lib.rsg_ball_pred_update_from_batch(self.h, batch.h, m and m[1]), "rsg_ball_pred_update_from_batch")

    def update_manual(self, states, ticks_since_last_update, mask=None) -> None:
        """UpdatePredManual for every arena: `states` n_arenas BallStates (a ctypes array or numpy
        records of the same layout), `ticks_since_last_update` n_arenas ints."""
        st = _ball_array(states, self.n_arenas)
        k = np.ascontiguousarray(ticks_since_last_update, np.int32)
        assert k.shape == (self.n_arenas,)
        m = self._mask(mask)
        check(self.lib.rsg_ball_pred_update_manual(self.h, st, k.ctypes.data_as(C.POINTER(C.c_int32)), m and m[1]),
              "rsg_ball_pred_update_manual")

    def force_update_all(self, states, mask=None) -> None:
        st = _ball_array(states, self.n_arenas)
        m = self._mask(mask)
        check(self.lib.rsg_ball_pred_force_update_all(self.h, st, m and m[1]), "rsg_ball_pred_force_update_all")

    def pred_data(self, arena: int) -> list[BallState]:
        out = (BallState * self.num_pred_ticks)()
        check(self.lib.rsg_ball_pred_get_pred(self.h, arena, out), "rsg_ball_pred_get_pred")
        return list(out)

    def pred_all(self) -> np.ndarray:
        """predData of every arena as [n_arenas, num_pred_ticks] BallState records."""
        out = np.zeros((self.n_arenas, self.num_pred_ticks), BALL_STATE_DTYPE)
        check(self.lib.rsg_ball_pred_get_all(self.h, out.ctypes.data_as(C.POINTER(BallState))), "rsg_ball_pred_get_all")
        return out

    def get_ball_state_for_time(self, arena: int, pred_time: float) -> BallState:
        s = BallState()
        check(self.lib.rsg_ball_pred_get_state_for_time(self.h, arena, pred_time, C.byref(s)),
              "rsg_ball_pred_get_state_for_time")
        return s

    def last_update_tick(self, arena: int) -> int:
        v = C.c_int32()
        check(self.lib.rsg_ball_pred_get_last_update_tick(self.h, arena, C.byref(v)), "rsg_ball_pred_get_last_update_tick")
        return v.value

    def device_flags(self) -> np.ndarray:
        out = np.zeros(self.n_arenas, np.uint32)
        check(self.lib.rsg_ball_pred_device_flags(self.h, out.ctypes.data_as(C.POINTER(C.c_uint32))),
              "rsg_ball_pred_device_flags")
        return out

    def close(self) -> None:
        if self.h:
            self.lib.rsg_ball_pred_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GameEventTracker:
    """GameEventTracker (src/Sim/GameEventTracker/GameEventTracker.h) for every arena of a batch:
    update() returns each arena's event of this update as records (kind, car_id, other_car_id)."""

    def __init__(self, batch: ArenaBatch, config: "abi.GameEventTrackerConfig | None" = None):
        self.lib, self.n_arenas = batch.lib, batch.n_arenas
        self.h = self.lib.rsg_game_event_tracker_create(batch.h, C.byref(config) if config is not None else None)
        if not self.h:
            raise RuntimeError(abi.last_error())

    @staticmethod
    def default_config() -> "abi.GameEventTrackerConfig":
        c = abi.GameEventTrackerConfig()
        check(abi.load().rsg_get_default_game_event_tracker_config(C.byref(c)), "rsg_get_default_game_event_tracker_config")
        return c

    def update(self, batch: ArenaBatch) -> np.ndarray:
        out = np.zeros(self.n_arenas, np.dtype(abi.GameEvent))
        check(self.lib.rsg_game_event_tracker_update(self.h, batch.h, out.ctypes.data_as(C.POINTER(abi.GameEvent))),
              "rsg_game_event_tracker_update")
        return out

    def reset_persistent_info(self, arena: int = -1) -> None:
        check(self.lib.rsg_game_event_tracker_reset_persistent_info(self.h, arena),
              "rsg_game_event_tracker_reset_persistent_info")

    def close(self) -> None:
        if self.h:
            self.lib.rsg_game_event_tracker_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _ball_array(states, n: int):
    if isinstance(states, np.ndarray):
        assert states.nbytes == n * C.sizeof(BallState)
        return np.ascontiguousarray(states).ctypes.data_as(C.POINTER(BallState))
    arr = (BallState * n)(*states)
    return arr


class Car:
    """Car handle of a one-arena view (src/Sim/Car/Car.h:140-160)."""

    def __init__(self, arena: "Arena", car_id: int, team: int, config: CarConfig):
        self._arena, self.id, self.team, self.config = arena, car_id, team, config
        self._controls = CarControls()

    @property
    def controls(self) -> CarControls:
        return self._controls

    @controls.setter
    def controls(self, c: CarControls) -> None:
        self._controls = c
        self._arena.batch.set_controls(0, self.id, c)

    def get_state(self) -> CarState:
        return self._arena.batch.get_car_state(0, self.id)

    def set_state(self, s: CarState) -> None:
        self._arena.batch.set_car_state(0, self.id, s)

    def demolish(self, respawn_delay: float = 3.0) -> None:
        self._arena.batch.demolish(0, self.id, respawn_delay)


class Ball:
    def __init__(self, arena: "Arena"):
        self._arena = arena

    def get_state(self) -> BallState:
        return self._arena.batch.get_ball_state(0)

    def set_state(self, s: BallState) -> None:
        self._arena.batch.set_ball_state(0, s)


class Arena:
    """One arena with RocketSim's method names (Arena::Create, AddCar, Step, ...)."""

    def __init__(self, game_mode: int = abi.GAMEMODE_SOCCAR, tick_rate: float = 120.0, max_cars: int = 8,
                 config: "abi.ArenaConfig | None" = None):
        self.batch = ArenaBatch(game_mode, 1, max_cars, tick_rate, config)
        self.game_mode = game_mode
        self.tick_time = 1.0 / tick_rate
        self.ball = Ball(self)
        self._cars: dict[int, Car] = {}

    @classmethod
    def create(cls, game_mode: int = abi.GAMEMODE_SOCCAR, tick_rate: float = 120.0,
               config: "abi.ArenaConfig | None" = None) -> "Arena":
        return cls(game_mode, tick_rate, config=config)

    def add_car(self, team: int, config: CarConfig | int = abi.CAR_OCTANE, respawn_index: int = -1) -> Car:
        cfg = car_config(config) if isinstance(config, int) else config
        cid = self.batch.add_car(0, team, cfg, respawn_index)
        car = Car(self, cid, team, cfg)
        self._cars[cid] = car
        return car

    def remove_car(self, car: Car | int) -> bool:
        cid = car.id if isinstance(car, Car) else car
        if cid not in self._cars:
            return False
        self.batch.remove_car(0, cid)
        del self._cars[cid]
        return True

    def get_car(self, car_id: int) -> Car | None:
        return self._cars.get(car_id)

    def get_cars(self) -> list[Car]:
        return [self._cars[i] for i in self.batch.get_cars(0)]

    @property
    def tick_count(self) -> int:
        return self.batch.get_tick_count(0)

    def step(self, ticks: int = 1) -> None:
        self.batch.step(ticks)

    def is_ball_scored(self) -> bool:
        return self.batch.is_ball_scored(0)

    def get_mutator_config(self) -> "abi.MutatorConfig":
        return self.batch.get_mutator_config()

    def set_mutator_config(self, config: "abi.MutatorConfig") -> None:
        self.batch.set_mutator_config(config)

    def set_goal_score_callback(self, fn) -> None:
        self.batch.set_goal_score_callback((lambda a, team: fn(self, team)) if fn else None)

    def set_car_bump_callback(self, fn) -> None:
        self.batch.set_car_bump_callback(
            (lambda a, x, y, demo: fn(self, self._cars.get(x), self._cars.get(y), demo)) if fn else None)

    def close(self) -> None:
        self.batch.close()
