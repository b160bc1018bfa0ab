"""Writes tests/golden/game_events.npz: the events of the reference RocketSim's GameEventTracker
(default config) along the scripts of tests/game_event_cases.py, one row (kind, car id, other car id)
per Update, plus the ball state at each Update.

Run from the repository root with the reference library built (make -C oracle ref).
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from game_event_cases import SCRIPTS, TEAMS  # noqa: E402
from scenarios import mesh_bytes  # noqa: E402

OUT = os.path.join(HERE, "game_events.npz")
DEFAULT_CFG = (1750.0, 0.3, 0.0, 1.0, 2.0, 4.0, 2.0)


def run_ref(auto, script):
    from oracle.pyoracle import SimArena, BallState as OBall
    a = SimArena("ref", mesh_bytes())
    lib, p = a.lib, a.p
    ids = [a.add_car(t, 0) for t in TEAMS]
    assert ids == [1, 2, 3, 4]
    lib[p + "gevt_create"].restype = C.c_void_p
    lib[p + "gevt_create"].argtypes = [C.POINTER(C.c_float), C.c_int]
    for n in ("gevt_update", "gevt_reset", "gevt_destroy"):
        lib[p + n].argtypes = [C.c_void_p] * (2 if n == "gevt_update" else 1) + ([C.POINTER(C.c_int)] if n == "gevt_update" else [])
    t = lib[p + "gevt_create"]((C.c_float * 7)(*DEFAULT_CFG), 1 if auto else 0)
    events, balls = [], []
    for op in script:
        if op[0] == "ball":
            s = OBall()
            s.pos.x, s.pos.y, s.pos.z = op[1]
            s.vel.x, s.vel.y, s.vel.z = op[2]
            s.rot_mat.forward.x = s.rot_mat.right.y = s.rot_mat.up.z = 1
            a.set_ball(s)
        elif op[0] == "hit":
            c = a.get_car(op[1])
            c.ball_hit_info.is_valid = 1
            c.ball_hit_info.tick_count_when_hit = a.get_tick() - op[2]
            a.set_car(op[1], c)
        elif op[0] == "car":
            c = a.get_car(op[1])
            c.pos.x, c.pos.y, c.pos.z = op[2]
            c.vel.x = c.vel.y = c.vel.z = c.ang_vel.x = c.ang_vel.y = c.ang_vel.z = 0.0
            c.rot_mat.forward.x, c.rot_mat.forward.y, c.rot_mat.forward.z = 0.0, 1.0, 0.0
            c.rot_mat.right.x, c.rot_mat.right.y, c.rot_mat.right.z = -1.0, 0.0, 0.0
            c.rot_mat.up.x, c.rot_mat.up.y, c.rot_mat.up.z = 0.0, 0.0, 1.0
            c.is_on_ground = 1
            a.set_car(op[1], c)
        elif op[0] == "step":
            a.step(op[1])
        elif op[0] == "update":
            e = (C.c_int * 3)()
            lib[p + "gevt_update"](t, a.h, e)
            events.append(list(e))
            b = a.get_ball()
            balls.append([b.pos.x, b.pos.y, b.pos.z, b.vel.x, b.vel.y, b.vel.z])
        elif op[0] == "reset":
            lib[p + "gevt_reset"](t)
    lib[p + "gevt_destroy"](t)
    a.close()
    return np.array(events, np.int32), np.array(balls, np.float32)


def main():
    from oracle.pyoracle import build_ref
    build_ref()
    out = {}
    for name, (auto, script) in SCRIPTS.items():
        ev, balls = run_ref(auto, script)
        out[f"{name}_events"], out[f"{name}_balls"] = ev, balls
        print(name, [tuple(e) for e in ev if e[0]])
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
