"""Writes tests/golden/arena_config_rollouts.npz from the reference RocketSim: seeded scenarios played
in arenas created with a non-default ArenaConfig.

Run here, where the reference sources exist: ``python tests/golden/make_arena_config_golden.py``.
The arenas use 24 custom boost pads (ArenaConfig::useCustomBoostPads: checked against every car
without BoostPadGrid, Arena.cpp:724-728), 18 of them where the scenarios' grounded cars start (6
big), and integrate the ball's rotation (noBallRot = false).  The file has the layout of
ref_rollouts.npz (make_golden.py) with 24 pads per arena.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, HERE)

from make_golden import record  # noqa: E402
from scenarios import make_carcar_scenario, make_scenario  # noqa: E402

OUT = os.path.join(HERE, "arena_config_rollouts.npz")


def custom_pads():
    """(x, y, z, is_big) in uu: at the start positions of the scenarios' cars that begin near the
    floor (so that they drive over them), the first 6 big, then a seeded scatter to 24 pads."""
    pads = []
    for sc in scenario_list():
        for c in sc.cars:
            if c.pos.z < 60 and len(pads) < 18:
                pads.append((round(float(c.pos.x), 1), round(float(c.pos.y), 1), 73.0 if len(pads) < 6 else 70.0,
                             len(pads) < 6))
    rng = np.random.default_rng(77)
    while len(pads) < 24:
        pads.append((float(rng.uniform(-3000, 3000)), float(rng.uniform(-4000, 4000)), 70.0, False))
    return pads


def config():
    import rocketsim_gb300 as rsg
    return rsg.arena_config(custom_boost_pads=custom_pads(), no_ball_rot=False)


def scenario_list():
    out = [make_scenario(seed) for seed in (300, 301, 302, 303, 304, 305)]
    out.append(make_scenario(306, ncars=6, presets=[0, 1, 2, 3, 4, 5]))
    out.append(make_scenario(307, ncars=4, presets=[3, 4, 5, 0], air_frac=0.0))
    out += [make_carcar_scenario(s) for s in (0, 6)]
    return out


def main():
    np.savez_compressed(OUT, **record(scenario_list(), None, epa=False, config=config()))
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
