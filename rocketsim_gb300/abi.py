"""ctypes mirror of include/rocketsim_gb300.h.

The structs restate the header's POD layouts field for field (sizes are
asserted); ``load()`` opens the in-tree CUDA library and declares every entry
point.  There is no fallback: if the library is missing or cannot be loaded
the import of the host API fails with the reason.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

OK = 0
ERR_ARG, ERR_STATE, ERR_CUDA, ERR_MESH, ERR_DEVICE = -1, -2, -3, -4, -5
GAMEMODE_SOCCAR, GAMEMODE_HEATSEEKER, GAMEMODE_THE_VOID = 0, 2, 5
TEAM_BLUE, TEAM_ORANGE = 0, 1
CAR_OCTANE, CAR_DOMINUS, CAR_PLANK, CAR_BREAKOUT, CAR_HYBRID, CAR_MERC = range(6)
MAX_CARS_PER_ARENA = 8
NUM_BOOST_PADS = 34
EVENT_GOAL, EVENT_BUMP, EVENT_BALL_HIT = 1, 2, 3
FLAG_WARN_EPA_SKIPPED = 1 << 8
FLAG_WARN_CARCAR_SKIPPED = 1 << 9


class Vec3(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float)]

    def __iter__(self):
        return iter((self.x, self.y, self.z))


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


class HeatseekerInfo(C.Structure):
    _fields_ = [("y_target_dir", C.c_float), ("cur_target_speed", C.c_float), ("time_since_hit", C.c_float)]


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


class MutatorConfig(C.Structure):
    _fields_ = [("gravity", Vec3)] + [(n, C.c_float) for n in (
        "car_mass", "car_world_friction", "car_world_restitution", "ball_mass", "ball_max_speed", "ball_drag",
        "ball_world_friction", "ball_world_restitution", "jump_accel", "jump_immediate_force", "boost_accel_ground",
        "boost_accel_air", "boost_used_per_second", "respawn_delay", "bump_cooldown_time", "boost_pad_cooldown_big",
        "boost_pad_cooldown_small", "car_spawn_boost_amount", "ball_hit_extra_force_scale", "bump_force_scale",
        "ball_radius")] + [
        ("unlimited_flips", C.c_uint8), ("unlimited_double_jumps", C.c_uint8), ("recharge_boost_enabled", C.c_uint8),
        ("_pad0", C.c_uint8), ("recharge_boost_per_second", C.c_float), ("recharge_boost_delay", C.c_float),
        ("demo_mode", C.c_uint8), ("enable_team_demos", C.c_uint8), ("_pad1", C.c_uint8 * 2),
        ("goal_base_threshold_y", C.c_float)]


DEMO_NORMAL, DEMO_ON_CONTACT, DEMO_DISABLED = 0, 1, 2


class BoostPadConfig(C.Structure):
    _fields_ = [("pos", Vec3), ("is_big", C.c_uint8), ("_pad0", C.c_uint8 * 3)]


class ArenaConfig(C.Structure):
    _fields_ = [("mem_weight_mode", C.c_uint8), ("no_ball_rot", C.c_uint8), ("use_custom_broadphase", C.c_uint8),
                ("use_custom_boost_pads", C.c_uint8), ("min_pos", Vec3), ("max_pos", Vec3),
                ("max_aabb_len", C.c_float), ("max_objects", C.c_int32), ("num_custom_boost_pads", C.c_uint32),
                ("custom_boost_pads", C.POINTER(BoostPadConfig))]

assert C.sizeof(MutatorConfig) == 116
assert C.sizeof(CarState) == 272
assert C.sizeof(BallState) == 80
assert C.sizeof(PadState) == 16
assert C.sizeof(CarControls) == 24
assert C.sizeof(CarConfig) == 72

GOAL_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_uint32, C.c_int, C.c_void_p)
BUMP_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_int, C.c_void_p)
BALL_HIT_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint64, C.c_void_p)

P = C.POINTER
class GameEventTrackerConfig(C.Structure):
    """rsg_game_event_tracker_config (GameEventTrackerConfig, GameEventTracker.h:10-40)."""
    _fields_ = [("shot_min_speed", C.c_float), ("shot_touch_min_delay", C.c_float),
                ("pred_score_extra_margin", C.c_float), ("shot_event_cooldown", C.c_float),
                ("shot_min_score_time", C.c_float), ("goal_max_touch_time", C.c_float),
                ("pass_max_touch_time", C.c_float), ("auto_state_set_detection", C.c_uint8), ("_pad0", C.c_uint8 * 3)]


class GameEvent(C.Structure):
    _fields_ = [("kind", C.c_int32), ("car_id", C.c_uint32), ("other_car_id", C.c_uint32)]


GAME_EVENT_NONE, GAME_EVENT_SHOT, GAME_EVENT_GOAL, GAME_EVENT_SAVE = 0, 1, 2, 3

u32, u64, i32, f32, vp = C.c_uint32, C.c_uint64, C.c_int, C.c_float, C.c_void_p

# name -> (restype, argtypes), in the order of include/rocketsim_gb300.h
PROTOTYPES = {
    "rsg_init_from_mem": (i32, [i32, P(P(C.c_uint8)), P(u64), i32]),
    "rsg_get_last_error": (i32, [C.c_char_p, u64]),
    "rsg_get_car_config_preset": (i32, [i32, P(CarConfig)]),
    "rsg_batch_create": (vp, [i32, u32, u32, f32]),
    "rsg_batch_destroy": (None, [vp]),
    "rsg_batch_num_arenas": (i32, [vp, P(u32)]),
    "rsg_add_car": (i32, [vp, u32, i32, P(CarConfig), i32, P(u32)]),
    "rsg_remove_car": (i32, [vp, u32, u32]),
    "rsg_get_car_ids": (i32, [vp, u32, P(u32), u32, P(u32)]),
    "rsg_set_car_update_order": (i32, [vp, u32, P(u32), u32]),
    "rsg_set_car_controls": (i32, [vp, u32, u32, P(CarControls)]),
    "rsg_set_controls_all": (i32, [vp, vp, u64]),
    "rsg_get_car_state": (i32, [vp, u32, u32, P(CarState)]),
    "rsg_set_car_state": (i32, [vp, u32, u32, P(CarState)]),
    "rsg_demolish_car": (i32, [vp, u32, u32, f32]),
    "rsg_get_ball_state": (i32, [vp, u32, P(BallState)]),
    "rsg_set_ball_state": (i32, [vp, u32, P(BallState)]),
    "rsg_get_ball_heatseeker": (i32, [vp, u32, P(HeatseekerInfo)]),
    "rsg_set_ball_heatseeker": (i32, [vp, u32, P(HeatseekerInfo)]),
    "rsg_get_pad_state": (i32, [vp, u32, u32, P(PadState)]),
    "rsg_set_pad_state": (i32, [vp, u32, u32, P(PadState)]),
    "rsg_get_pad_config": (i32, [vp, u32, P(Vec3), P(i32)]),
    "rsg_get_tick_count": (i32, [vp, u32, P(u64)]),
    "rsg_set_tick_count": (i32, [vp, u32, u64]),
    "rsg_is_ball_scored": (i32, [vp, u32, P(i32)]),
    "rsg_get_all_states": (i32, [vp, vp, vp, vp]),
    "rsg_set_all_states": (i32, [vp, vp, vp, vp]),
    "rsg_step": (i32, [vp, i32]),
    "rsg_step_controls": (i32, [vp, vp, i32]),
    "rsg_step_async": (i32, [vp, vp, i32]),
    "rsg_sync": (i32, [vp]),
    "rsg_batch_stream": (vp, [vp]),
    "rsg_set_goal_callback": (i32, [vp, GOAL_FN, vp]),
    "rsg_set_bump_callback": (i32, [vp, BUMP_FN, vp]),
    "rsg_set_ball_hit_callback": (i32, [vp, BALL_HIT_FN, vp]),
    "rsg_get_device_flags": (i32, [vp, P(u32)]),
    "rsg_get_tick_shape": (i32, [vp, P(C.c_int32)]),
    "rsg_get_tuning_log": (i32, [vp, C.c_char_p, C.c_uint64]),
    "rsg_air_forward": (i32, [P(CarConfig), f32, i32, i32, vp, vp, vp, vp, i32, vp]),
    "rsg_air_backward_workspace_size": (i32, [i32, i32, P(C.c_size_t)]),
    "rsg_air_backward": (i32, [P(CarConfig), f32, i32, i32, vp, vp, i32, vp, vp, vp, vp, C.c_size_t, vp]),
    "rsg_air_backward_noalloc": (i32, [P(CarConfig), f32, i32, i32, vp, vp, i32, vp, vp, vp, vp]),
    "rsg_batch_create_ex": (vp, [i32, u32, u32, f32, P(ArenaConfig)]),
    "rsg_get_default_arena_config": (i32, [P(ArenaConfig)]),
    "rsg_batch_num_pads": (i32, [vp, P(u32)]),
    "rsg_get_default_mutator_config": (i32, [i32, P(MutatorConfig)]),
    "rsg_serialize_arena": (i32, [vp, u32, vp, C.c_uint64, P(C.c_uint64)]),
    "rsg_deserialize_arena": (i32, [vp, u32, vp, C.c_uint64]),
    "rsg_clone_arena": (i32, [vp, u32, vp, u32]),
    "rsg_reset_to_random_kickoff": (i32, [vp, u32, C.c_int32]),
    "rsg_reset_to_random_kickoff_many": (i32, [vp, P(u32), P(C.c_int32), u32]),
    "rsg_is_ball_probably_going_in": (i32, [vp, f32, f32, P(i32), P(i32)]),
    "rsg_get_default_game_event_tracker_config": (i32, [P(GameEventTrackerConfig)]),
    "rsg_game_event_tracker_create": (vp, [vp, P(GameEventTrackerConfig)]),
    "rsg_game_event_tracker_destroy": (None, [vp]),
    "rsg_game_event_tracker_update": (i32, [vp, vp, P(GameEvent)]),
    "rsg_game_event_tracker_reset_persistent_info": (i32, [vp, C.c_int32]),
    "rsg_ball_pred_create": (vp, [vp, u32]),
    "rsg_ball_pred_destroy": (None, [vp]),
    "rsg_ball_pred_update_from_batch": (i32, [vp, vp, vp]),
    "rsg_ball_pred_update_manual": (i32, [vp, P(BallState), P(C.c_int32), vp]),
    "rsg_ball_pred_force_update_all": (i32, [vp, P(BallState), vp]),
    "rsg_ball_pred_num_pred_ticks": (u32, [vp]),
    "rsg_ball_pred_get_pred": (i32, [vp, u32, P(BallState)]),
    "rsg_ball_pred_get_all": (i32, [vp, P(BallState)]),
    "rsg_ball_pred_get_state_for_time": (i32, [vp, u32, f32, P(BallState)]),
    "rsg_ball_pred_get_last_update_tick": (i32, [vp, u32, P(C.c_int32)]),
    "rsg_ball_pred_device_buffers": (i32, [vp, P(vp), P(vp)]),
    "rsg_ball_pred_device_flags": (i32, [vp, P(u32)]),
    "rsg_set_mutator_config": (i32, [vp, P(MutatorConfig)]),
    "rsg_get_mutator_config": (i32, [vp, P(MutatorConfig)]),
    "rsg_ground_forward": (i32, [P(CarConfig), f32, i32, i32, vp, vp, vp, vp, i32, vp, vp]),
    "rsg_ground_backward_workspace_size": (i32, [i32, i32, P(C.c_size_t)]),
    "rsg_ground_backward": (i32, [P(CarConfig), f32, i32, i32, vp, vp, i32, vp, vp, vp, vp, C.c_size_t, vp]),
}

_LIB = None


def library_path() -> str:
    return _build.LIB_PATH


def load(build_if_missing: bool = True) -> C.CDLL:
    """Open the CUDA library (building it first when it is missing)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise ImportError(f"rocketsim_gb300 CUDA library not built: {path}")
        path = _build.build()
    lib = C.CDLL(path)
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def last_error() -> str:
    buf = C.create_string_buffer(512)
    load().rsg_get_last_error(buf, 512)
    return buf.value.decode(errors="replace")


class RSGError(RuntimeError):
    def __init__(self, code: int, what: str):
        super().__init__(f"{what} failed ({code}): {last_error()}")
        self.code = code


def check(rc: int, what: str) -> None:
    if rc != OK:
        raise RSGError(rc, what)
