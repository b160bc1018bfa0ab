"""MutatorConfig defaults through the C ABI (CPU only: no batch is created)."""
from __future__ import annotations

import ctypes as C
import os

import pytest

from rocketsim_gb300 import abi

REF_SO = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "_ref", "librsref.so")


def fields(m):
    out = {}
    for name, _ in abi.MutatorConfig._fields_:
        if name.startswith("_"):
            continue
        v = getattr(m, name)
        out[name] = (v.x, v.y, v.z) if name == "gravity" else v
    return out


def test_default_mutators_are_the_game_constants():
    import rocketsim_gb300 as rsg
    m = fields(rsg.default_mutator_config(abi.GAMEMODE_SOCCAR))
    assert m["gravity"] == (0.0, 0.0, -650.0)
    assert m["car_mass"] == 180.0 and m["ball_mass"] == 30.0
    assert abs(m["ball_radius"] - 91.25) < 1e-6 and m["ball_max_speed"] == 6000.0
    assert abs(m["boost_used_per_second"] - 100 / 3) < 1e-5 and m["car_spawn_boost_amount"] == pytest.approx(100 / 3)
    assert m["boost_pad_cooldown_big"] == 10.0 and m["boost_pad_cooldown_small"] == 4.0
    assert m["demo_mode"] == abi.DEMO_NORMAL and not m["unlimited_flips"] and not m["recharge_boost_enabled"]
    assert fields(rsg.default_mutator_config(abi.GAMEMODE_THE_VOID)) == m
    lib = abi.load()
    bad = abi.MutatorConfig()
    assert lib.rsg_get_default_mutator_config(3, C.byref(bad)) == abi.ERR_ARG  # a mode the batch does not run


@pytest.mark.skipif(not os.path.exists(REF_SO), reason="the reference library is built only where its sources are")
def test_default_mutators_match_the_reference():
    import rocketsim_gb300 as rsg
    ref = C.CDLL(REF_SO)
    m = abi.MutatorConfig()
    for mode in (abi.GAMEMODE_SOCCAR, abi.GAMEMODE_HEATSEEKER):
        assert ref.rsref_default_mutator_config(mode, C.byref(m)) == 0
        assert fields(m) == fields(rsg.default_mutator_config(mode)), mode
