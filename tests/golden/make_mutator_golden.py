"""Writes tests/golden/mutator_rollouts.npz from the reference RocketSim: seeded scenarios played
under a non-default MutatorConfig.

Run here, where the reference sources exist: ``python tests/golden/make_mutator_golden.py``.
The mutators (MUTATORS below) are set with Arena::SetMutatorConfig before the cars are added and
touch every field the tick reads: tilted gravity, car-world friction and restitution, a heavier,
larger, draggier and slower ball with other world friction and restitution, jump forces, boost
forces and use, pad cooldowns, ball-hit and bump force scales, unlimited flips and double jumps,
boost recharge, demolition on any bumper contact including teammates, a nearer goal line.  The
respawn delay stays above the 1 s the rollouts cover: RocketSim respawns a demolished car at a
randomly chosen spawn point.  The file has the layout of ref_rollouts.npz (make_golden.py).
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
from rocketsim_gb300 import abi  # noqa: E402

OUT = os.path.join(HERE, "mutator_rollouts.npz")


def mutators() -> abi.MutatorConfig:
    """The non-default mutator set of the fixture (uu units, like MutatorConfig)."""
    m = abi.MutatorConfig()
    m.gravity = abi.Vec3(30.0, -20.0, -900.0)
    m.car_mass = 180.0
    m.car_world_friction, m.car_world_restitution = 0.4, 0.2
    m.ball_mass, m.ball_radius, m.ball_max_speed, m.ball_drag = 45.0, 100.0, 5000.0, 0.05
    m.ball_world_friction, m.ball_world_restitution = 0.45, 0.5
    m.jump_accel, m.jump_immediate_force = 1600.0, 320.0
    m.boost_accel_ground, m.boost_accel_air, m.boost_used_per_second = 1100.0, 1150.0, 45.0
    m.respawn_delay, m.bump_cooldown_time = 1.5, 0.3
    m.boost_pad_cooldown_big, m.boost_pad_cooldown_small = 6.0, 3.0
    m.car_spawn_boost_amount = 60.0
    m.ball_hit_extra_force_scale, m.bump_force_scale = 1.4, 1.3
    m.unlimited_flips, m.unlimited_double_jumps = 1, 1
    m.recharge_boost_enabled, m.recharge_boost_per_second, m.recharge_boost_delay = 1, 12.0, 0.3
    m.demo_mode, m.enable_team_demos = abi.DEMO_ON_CONTACT, 1
    m.goal_base_threshold_y = 5000.0
    return m


def scenario_list():
    out = [make_scenario(seed) for seed in (200, 201, 202, 203, 204, 205)]
    out.append(make_scenario(206, ncars=6, presets=[0, 1, 2, 3, 4, 5]))
    out.append(make_scenario(207, ncars=4, air_frac=1.0))
    out += [make_carcar_scenario(s) for s in (0, 2, 6, 8)]
    return out


def main():
    np.savez_compressed(OUT, **record(scenario_list(), mutators(), epa=False))
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
