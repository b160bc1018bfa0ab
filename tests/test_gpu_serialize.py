"""Arena serialisation through the C ABI (rsg_serialize_arena / rsg_deserialize_arena /
rsg_clone_arena) against the reference's own serialized arenas (tests/golden/serial_arenas.npz,
written by tests/golden/make_serial_golden.py).

* the reference's bytes load into a batch arena with the states the reference reported, the boost
  excepted: DeserializeNew gives every car the game mode's spawn boost, and so does this code;
* play resumes from them: 8 ticks in the reference's car order match the reference's own 8 ticks
  (continuous state within golden_data.TOL[8], discrete state every tick);
* the bytes this code writes carry, field for field, what the reference wrote (states within float
  round-off of the uu / Bullet-unit conversion), and read back to the same arena;
* a cloned arena holds its source's states bit for bit and plays on like the reference's Arena::Clone.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

from golden_data import check_continuous
from scenarios import discrete_car, discrete_pads, mesh_bytes
from serial_format import parse_arena

pytestmark = pytest.mark.gpu

SPAWN_BOOST = np.float32(100 / 3)
PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "serial_arenas.npz")


def blobs(z):
    return [z["blob"][z["offsets"][i]:z["offsets"][i + 1]].tobytes() for i in range(len(z["offsets"]) - 1)]


def new_batch(n):
    import rocketsim_gb300 as rsg
    from rocketsim_gb300 import abi
    rsg.init_from_mem([mesh_bytes()])
    return rsg.ArenaBatch(abi.GAMEMODE_SOCCAR, n, 6, 120.0)


def close(a, b, tol):
    return np.max(np.abs(np.asarray(a, np.float64) - np.asarray(b, np.float64))) <= tol


def test_reference_bytes_load_and_resume():
    z = np.load(PATH)
    bl = blobs(z)
    b = new_batch(len(bl))
    for i, blob in enumerate(bl):
        b.deserialize(i, blob)
    for i in range(len(bl)):
        n = int(z["ncars"][i])
        assert sorted(b.get_cars(i)) == list(range(1, n + 1))
        for cid in range(1, n + 1):
            s, r = b.get_car_state(i, cid), z["cars_t0"][i][cid - 1]
            assert close((s.pos.x, s.pos.y, s.pos.z), tuple(r["pos"][k] for k in "xyz"), 1e-3)
            assert close((s.vel.x, s.vel.y, s.vel.z), tuple(r["vel"][k] for k in "xyz"), 1e-3)
            assert s.boost == SPAWN_BOOST and s.is_on_ground == r["is_on_ground"]
        assert b.get_tick_count(i) == 30
        b.set_car_update_order(i, [int(x) for x in z["order_ids"][i][:n]])
    mc = b.max_cars
    for t in range(8):
        ctl = np.zeros(len(bl) * mc, z["controls"].dtype)
        for i in range(len(bl)):
            n = int(z["ncars"][i])
            ctl[i * mc:i * mc + n] = z["controls"][i, t, :n]
        b.set_controls_all(ctl)
        b.step(1)
        cars, balls, pads = b.get_all_states()
        for i in range(len(bl)):
            n = int(z["ncars"][i])
            np.testing.assert_array_equal(discrete_car(cars[i * mc:i * mc + n]).astype(np.float32), z["disc"][i, t, :n],
                                          err_msg=f"arena {i} tick {31 + t}")
    cars, balls, pads = b.get_all_states()
    for i in range(len(bl)):
        n = int(z["ncars"][i])
        check_continuous(cars[i * mc:i * mc + n], balls[i:i + 1], z["cars_end"][i][:n], z["ball_end"][i:i + 1], 8,
                         f"resumed arena {i}")
        np.testing.assert_array_equal(discrete_pads(pads[i * 34:(i + 1) * 34]), discrete_pads(z["pads_end"][i]))
    b.close()


def test_written_bytes_carry_the_reference_fields():
    z = np.load(PATH)
    bl = blobs(z)
    b = new_batch(len(bl))
    for i, blob in enumerate(bl):
        b.deserialize(i, blob)
        ref, mine = parse_arena(blob), parse_arena(b.serialize(i))
        for k in ("game_mode", "tick_time", "tick_count", "last_car_id", "min_pos", "max_pos", "max_aabb_len",
                  "no_ball_rot", "use_custom_broadphase", "use_custom_boost_pads", "pads", "mutators"):
            assert mine[k] == ref[k], (i, k)
        assert [c["id"] for c in mine["cars"]] == sorted(c["id"] for c in ref["cars"])  # ascending ids
        by_id = {c["id"]: c for c in ref["cars"]}
        for c in mine["cars"]:
            r = by_id[c["id"]]
            assert c["team"] == r["team"] and c["controls"] == r["controls"] and c["config"] == r["config"]
            for f, v in c["state"].items():
                if f == "boost":
                    assert v == SPAWN_BOOST, (i, c["id"])
                elif f in ("pos", "vel", "world_contact_normal"):
                    assert close(v, r["state"][f], 1e-3), (i, c["id"], f)
                elif f in ("rot_mat", "ang_vel", "flip_rel_torque"):
                    assert close(v, r["state"][f], 1e-6), (i, c["id"], f)
                else:
                    assert v == r["state"][f], (i, c["id"], f)
        assert close(mine["ball"]["pos"], ref["ball"]["pos"], 1e-3) and close(mine["ball"]["vel"], ref["ball"]["vel"], 1e-3)
        # what this code writes, it reads back to the same arena
        b2 = new_batch(1)
        b2.deserialize(0, b.serialize(i))
        assert b2.serialize(0) == b.serialize(i)
        b2.close()
    b.close()


def test_clone_continues_like_the_reference_clone():
    """Arena::Clone of the reference's arena at tick 30 (its car states whole, the boost included) played
    8 ticks in the clone's car order: the batch's clone of an arena set to the same states plays them
    the same way; at the clone the two arenas hold the same states, controls, pads and tick count."""
    from rocketsim_gb300 import abi
    z = np.load(PATH)
    bl = blobs(z)
    S = len(bl)
    b = new_batch(2 * S)
    for i, blob in enumerate(bl):
        b.deserialize(i, blob)
        for cid in range(1, int(z["ncars"][i]) + 1):
            b.set_car_state(i, cid, abi.CarState.from_buffer_copy(z["cars_t0"][i][cid - 1].tobytes()))
    for i in range(S):
        b.clone_arena_from(S + i, b, i)
    mc = b.max_cars
    cars, balls, pads = b.get_all_states()
    cars["tick_count_since_update"] = 0  # Car::SetState and Ball::SetState zero it in the clone
    balls["tick_count_since_update"] = 0
    assert cars[:S * mc].tobytes() == cars[S * mc:].tobytes()
    assert balls[:S].tobytes() == balls[S:].tobytes() and pads[:S * 34].tobytes() == pads[S * 34:].tobytes()
    for i in range(S):
        n = int(z["ncars"][i])
        assert b.get_tick_count(S + i) == 30 and b.serialize(S + i) == b.serialize(i)
        b.set_car_update_order(S + i, [int(x) for x in z["clone_order"][i][:n]])
    for t in range(8):
        ctl = np.zeros(2 * S * mc, z["controls"].dtype)
        for i in range(S):
            n = int(z["ncars"][i])
            ctl[(S + i) * mc:(S + i) * mc + n] = z["controls"][i, t, :n]
        b.set_controls_all(ctl)
        b.step(1)
    cars, balls, pads = b.get_all_states()
    for i in range(S):
        n, a = int(z["ncars"][i]), S + i
        check_continuous(cars[a * mc:a * mc + n], balls[a:a + 1], z["clone_cars_end"][i][:n],
                         z["clone_ball_end"][i:i + 1], 8, f"cloned arena {i}")
        np.testing.assert_array_equal(discrete_car(cars[a * mc:a * mc + n]), discrete_car(z["clone_cars_end"][i][:n]))
        np.testing.assert_array_equal(discrete_pads(pads[a * 34:(a + 1) * 34]), discrete_pads(z["clone_pads_end"][i]))
    b.close()
