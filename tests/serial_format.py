"""A reader of RocketSim's serialized arena (Arena::Serialize, src/Sim/Arena/Arena.cpp:546-574;
DataStreamOut): test infrastructure that turns the bytes into nested dicts so that the reference's
output and rsg_serialize_arena's can be compared field by field.

Layout: little-endian raw fields; every WriteMultiple group starts with its field count (uint32);
Vec = 4 floats (the fourth unused), RotMat = 3 Vec, bool and enums = 1 byte, CarControls = its
24-byte struct (5 floats, 3 bools, 1 padding byte).
"""
from __future__ import annotations

import struct


class Reader:
    def __init__(self, data: bytes):
        self.d, self.pos = data, 0

    def take(self, fmt: str):
        v = struct.unpack_from("<" + fmt, self.d, self.pos)
        self.pos += struct.calcsize("<" + fmt)
        return v if len(v) > 1 else v[0]

    def group(self, n: int):
        g = self.take("I")
        assert g == n, f"group of {g} fields where {n} were expected at byte {self.pos - 4}"

    def vec(self):
        x, y, z, _ = self.take("4f")
        return (x, y, z)

    def rot(self):
        return (self.vec(), self.vec(), self.vec())


CAR_FIELDS = ("pos", "rot_mat", "vel", "ang_vel", "is_on_ground", "has_jumped", "has_double_jumped", "has_flipped",
              "flip_rel_torque", "jump_time", "is_flipping", "flip_time", "is_jumping", "air_time_since_jump",
              "boost", "is_boosting", "boosting_time", "time_since_boosted", "supersonic_time", "handbrake_val",
              "is_auto_flipping", "auto_flip_timer", "auto_flip_torque_scale", "is_demoed", "demo_respawn_timer",
              "last_controls", "world_contact_has_contact", "world_contact_normal", "car_contact_other_car_id",
              "car_contact_cooldown_timer")
CAR_KINDS = "VRVVBBBBVfBfBfffBffffBffBfCBVIf"


def parse_arena(data: bytes) -> dict:
    r = Reader(data)
    out = {}
    r.group(4)
    out["game_mode"], out["tick_time"], out["tick_count"], out["last_car_id"] = r.take("BfQI")
    r.group(5)
    out["min_pos"], out["max_pos"] = r.vec(), r.vec()
    out["max_aabb_len"], out["no_ball_rot"], out["use_custom_broadphase"] = r.take("fBB")
    out["use_custom_boost_pads"] = r.take("B")
    pads_cfg = []
    if out["use_custom_boost_pads"]:
        for _ in range(r.take("I")):
            r.group(2)
            pads_cfg.append((r.vec(), r.take("B")))
    out["custom_boost_pads"] = pads_cfg
    cars = []
    out["cars_count_at"] = r.pos
    for _ in range(r.take("I")):
        start = r.pos
        c = {"team": r.take("B"), "id": r.take("I")}
        r.group(8)
        c["controls"] = r.take("5f3B")
        r.group(9)
        c["config"] = (r.take("f"), r.vec(), r.vec(), r.vec(), r.take("2f"), r.vec(), r.take("2f"))
        valid = r.take("B")
        c["ball_hit_info"] = None
        if valid:
            r.group(5)
            c["ball_hit_info"] = (r.vec(), r.vec(), r.vec(), r.take("QQ"))
        r.group(30)
        st = {}
        for name, kind in zip(CAR_FIELDS, CAR_KINDS):
            if kind == "V":
                st[name] = r.vec()
            elif kind == "R":
                st[name] = r.rot()
            elif kind == "B":
                st[name] = r.take("B")
            elif kind == "f":
                st[name] = r.take("f")
            elif kind == "I":
                st[name] = r.take("I")
            else:  # CarControls struct: 5 floats, 3 bools, a padding byte
                v = r.take("5f4B")
                st[name] = v[:8]
        c["state"] = st
        c["span"] = (start, r.pos)
        cars.append(c)
    out["cars"] = cars
    pads = []
    if out["game_mode"] != 5 and pos_left(r) > 0:
        peek = struct.unpack_from("<I", r.d, r.pos)[0]
        if peek != 12:  # a pad count (the ball's group has 12 fields; arenas hold 34 pads or custom ones)
            for _ in range(r.take("I")):
                r.group(3)
                pads.append(r.take("BfI"))
    out["pads"] = pads
    r.group(12)
    out["ball"] = {"pos": r.vec(), "rot_mat": r.rot(), "vel": r.vec(), "ang_vel": r.vec(),
                   "rest": r.take("3fi2fBQ")}
    assert r.take("H") == 30
    r.group(30)
    mut = [r.vec()] + list(r.take("21f")) + list(r.take("3B")) + list(r.take("2f")) + list(r.take("2B")) + \
        [r.take("f")]
    out["mutators"] = mut
    assert r.pos == len(data), (r.pos, len(data))
    return out


def pos_left(r: Reader) -> int:
    return len(r.d) - r.pos


def reorder_cars_ascending(data: bytes) -> bytes:
    """The same serialized arena with its cars by ascending id (RocketSim's DeserializeNew keeps every
    car only then: it gives each car read the next id before forcing the written one)."""
    d = parse_arena(data)
    if not d["cars"]:
        return data
    cars = sorted(d["cars"], key=lambda c: c["id"])
    first, last = d["cars"][0]["span"][0], d["cars"][-1]["span"][1]
    body = b"".join(data[c["span"][0]:c["span"][1]] for c in cars)
    return data[:first] + body + data[last:]
