"""CUDA tick through the C ABI against the reference's golden rollouts and the
CPU restatement.

Continuous state (positions, velocities, angular velocities, rotation) is
compared after 1 and 8 ticks within golden_data.TOL; discrete state (flags,
jump/flip/air/boost/supersonic timers, boost amounts, pad activity and
cooldowns, demo timers) must be identical over 120-tick rollouts.
"""
import ctypes as C

import numpy as np
import pytest

from golden_data import TOL, check_continuous
from scenarios import (CONTROLS_DTYPE, cpu_snapshot, discrete_car, discrete_hit, discrete_pads, gpu_controls,
                       gpu_snapshot, make_scenario, mesh_bytes, run_cpu, setup_gpu)

pytestmark = pytest.mark.gpu


def play_gpu(scs, ticks, every_tick=True):
    batch, ids = setup_gpu(scs)
    snaps = []
    for t in range(ticks):
        batch.set_controls_all(gpu_controls(scs, t, batch.max_cars))
        batch.step(1)
        if every_tick or t in (0, 7, ticks - 1):
            snaps.append(gpu_snapshot(batch, scs))
        else:
            snaps.append(None)
    return batch, snaps


def test_gpu_matches_reference_golden(golden):
    """Continuous state after 1 and 8 ticks; discrete car state, ball-hit counters,
    tickCountSinceUpdate and pads after every tick; the goal and bump callbacks against the
    reference's events (tick, kind, car ids / team, demo flag) in order."""
    scs = golden.scenarios
    batch, ids = setup_gpu(scs)
    pos = [{cid: i for i, cid in enumerate(row)} for row in ids]
    events = [[] for _ in scs]
    cur = {"t": 0}
    batch.set_goal_score_callback(lambda a, team: events[a].append((cur["t"], 1, team, 0, 0)))
    batch.set_car_bump_callback(
        lambda a, x, y, demo: events[a].append((cur["t"], 2, pos[a][x] + 1, pos[a][y] + 1, int(demo))))
    snaps = []
    for t in range(120):
        cur["t"] = t
        batch.set_controls_all(gpu_controls(scs, t, batch.max_cars))
        batch.step(1)
        snaps.append(gpu_snapshot(batch, scs))
    z = golden.z
    for si in range(golden.S):
        n = golden.ncars(si)
        for t in (1, 8):
            cars, ball, _ = snaps[t - 1][si]
            check_continuous(cars, ball, golden.cars_at(si, t), golden.ball_at(si, t), t, f"golden scenario {si}")
        for t in range(120):
            cars, ball, pads = snaps[t][si]
            np.testing.assert_array_equal(discrete_car(cars).astype(np.float32), golden.disc_cars(si)[t],
                                          err_msg=f"golden scenario {si} tick {t + 1}: car discrete state")
            np.testing.assert_array_equal(discrete_hit(cars), z["disc_hit"][si, t, :n],
                                          err_msg=f"golden scenario {si} tick {t + 1}: ball-hit counters")
            np.testing.assert_array_equal(discrete_pads(pads).astype(np.float32), golden.disc_pads(si)[t],
                                          err_msg=f"golden scenario {si} tick {t + 1}: pads")
        ref = [(e[1], e[0], e[2], e[3], e[4]) for e in golden.events(si)]
        assert events[si] == ref, f"golden scenario {si}: events {events[si]} != reference {ref}"
    batch.close()


def test_gpu_follows_restatement_through_epa(golden):
    """The golden scenarios where the reference runs Bullet's GJK-EPA: the GPU tick (EPA in a pooled
    work slot) against the portable restatement over all 120 ticks, continuous state within the
    8-tick tolerance at the EPA tick and 8 ticks after it, discrete state equal every tick, and no
    arena flagged for a skipped EPA."""
    epa_scenarios = [si for si in range(golden.S) if golden.epa_tick(si) >= 0]
    assert epa_scenarios
    scs = [golden.scenarios[si] for si in epa_scenarios]
    batch, snaps = play_gpu(scs, 120)
    flags = batch.device_flags()
    assert not (int(np.bitwise_or.reduce(flags)) & 0x100), flags
    for k, si in enumerate(epa_scenarios):
        ref = []
        a, _ = run_cpu("oracle", scs[k], 120, lambda t, a, ids: ref.append(cpu_snapshot(a, ids)))
        a.close()
        e = golden.epa_tick(si)
        for t in (e + 1, min(e + 8, 120)):
            cars, ball, _ = snaps[t - 1][k]
            check_continuous(cars, ball, ref[t - 1][0], ref[t - 1][1], 8, f"epa scenario {si} tick {t}")
        for t in range(120):
            np.testing.assert_array_equal(discrete_car(snaps[t][k][0]), discrete_car(ref[t][0]),
                                          err_msg=f"epa scenario {si} tick {t + 1}")
    batch.close()


def random_scenarios(n, base_seed=1000):
    rng = np.random.default_rng(base_seed)
    out = []
    for k in range(n):
        nc = int(rng.choice([2, 4, 6]))
        presets = [int(p) for p in rng.integers(0, 6, nc)]
        out.append(make_scenario(base_seed + k, ncars=nc, presets=presets, air_frac=float(rng.uniform(0, 0.6)),
                                 max_ball_speed=6000.0))
    return out


def test_gpu_matches_restatement_random():
    scs = random_scenarios(40)
    batch, snaps = play_gpu(scs, 120)
    for si, sc in enumerate(scs):
        ref = []

        def rec(t, a, ids):
            ref.append(cpu_snapshot(a, ids))
        a, _ = run_cpu("oracle", sc, 120, rec)
        a.close()
        for t in (1, 8):
            cars, ball, _ = snaps[t - 1][si]
            check_continuous(cars, ball, ref[t - 1][0], ref[t - 1][1], t, f"random scenario {si}")
        for t in range(120):
            np.testing.assert_array_equal(discrete_car(snaps[t][si][0]), discrete_car(ref[t][0]),
                                          err_msg=f"random scenario {si} tick {t + 1}")
            np.testing.assert_array_equal(discrete_pads(snaps[t][si][2]), discrete_pads(ref[t][2]),
                                          err_msg=f"random scenario {si} tick {t + 1}: pads")
    batch.close()


@pytest.fixture(scope="module")
def full_size_runs():
    """4096 arenas holding 8 scenarios 512 times each, stepped 8 ticks with one block per group of 6
    arenas and with a persistent launch (683 groups, more than the blocks resident at once, so its
    blocks take further groups from the counter)."""
    import os
    base = random_scenarios(8, base_seed=2000)
    scs = [base[k % 8] for k in range(4096)]
    out = {}
    old = os.environ.get("RSG_TICK_SHAPE")
    try:
        for persistent in (0, 1):
            os.environ["RSG_TICK_SHAPE"] = f"6,4,-1,1,1,{persistent}"
            batch, ids = setup_gpu(scs, max_cars=6)
            assert batch.tick_shape()[5] == persistent
            for t in range(8):
                batch.set_controls_all(gpu_controls(scs, t, batch.max_cars))
                batch.step(1)
            out[persistent] = (batch.get_all_states(), batch.max_cars)
            batch.close()
    finally:
        if old is None:
            os.environ.pop("RSG_TICK_SHAPE", None)
        else:
            os.environ["RSG_TICK_SHAPE"] = old
    return base, out


@pytest.mark.parametrize("persistent", [0, 1])
def test_full_size_batch_is_deterministic_and_independent(full_size_runs, persistent):
    """Every copy of a scenario ends bit-identical after 8 ticks, all states stay finite, and the
    persistent launch gives the same bytes as one block per group."""
    base, out = full_size_runs
    (cars, balls, pads), mc = out[persistent]
    for k in range(8):
        n = len(base[k].cars)
        rows = [cars[a * mc:a * mc + n].tobytes() for a in range(k, 4096, 8)]
        assert len(set(rows)) == 1, f"scenario {k}: copies differ"
        brows = [balls[a].tobytes() for a in range(k, 4096, 8)]
        assert len(set(brows)) == 1
    for f in ("pos", "vel", "ang_vel"):
        for c in "xyz":
            assert np.isfinite(cars[f][c]).all() and np.isfinite(balls[f][c]).all()
    (c0, b0, p0), _ = out[0]
    assert cars.tobytes() == c0.tobytes() and balls.tobytes() == b0.tobytes() and pads.tobytes() == p0.tobytes()


def test_batch_wider_than_the_scratch_runs_persistent(monkeypatch):
    """8192 arenas in blocks of 16 need more warp slots than the tick scratch holds (two per warp an
    SM holds), so even a launch shape without the persistent launch runs as one: the same bytes as the
    persistent shape, and no arena flagged as not stepped."""
    base = random_scenarios(8, base_seed=2100)
    scs = [base[k % 8] for k in range(8192)]
    out = []
    for persistent in (0, 1):
        monkeypatch.setenv("RSG_TICK_SHAPE", f"16,4,-1,1,1,{persistent}")
        batch, _ = setup_gpu(scs)
        for t in range(8):
            batch.set_controls_all(gpu_controls(scs, t, batch.max_cars))
            batch.step(1)
        assert not (batch.device_flags() & 0xff).any()
        out.append(tuple(x.tobytes() for x in batch.get_all_states()))
        batch.close()
    assert out[0] == out[1]


def test_state_round_trip_and_ids():
    """Get after Set returns what the reference returns: the state converted to Bullet
    units and back (pos * (1/50) * 50 is not the identity in float), other fields as set."""
    from oracle.pyoracle import CarState as OCarState, BallState as OBallState
    sc = make_scenario(7)
    batch, ids = setup_gpu([sc])
    assert batch.get_cars(0) == [ids[0][i] for i in sc.order]
    a, oids = run_cpu("oracle", sc, 0)
    for cid, ocid, s in zip(ids[0], oids, sc.cars):
        g, r = batch.get_car_state(0, cid), a.get_car(ocid)
        assert bytes(g) == bytes(r), f"car {cid}"
    assert bytes(batch.get_ball_state(0)) == bytes(a.get_ball())
    a.close()
    batch.close()


def test_async_device_controls_match_host_controls():
    """Per-tick controls three ways give the same bytes: set before each one-tick step (the reference's
    pattern), as a device array for an asynchronous step, and as a host array for rsg_step_controls."""
    import torch
    scs = random_scenarios(6, base_seed=3000)
    b1, _ = setup_gpu(scs)
    for t in range(8):
        b1.set_controls_all(gpu_controls(scs, t, b1.max_cars))
        b1.step(1)
    s1 = b1.get_all_states()
    b2, _ = setup_gpu(scs)
    seq = np.concatenate([gpu_controls(scs, t, b2.max_cars) for t in range(8)])
    dev = torch.from_numpy(seq.view(np.uint8).copy()).cuda()
    torch.cuda.synchronize()
    b2.step_async(dev.data_ptr(), 8)
    b2.sync()
    s2 = b2.get_all_states()
    assert s1[0].tobytes() == s2[0].tobytes() and s1[1].tobytes() == s2[1].tobytes()
    # host controls for every tick in one synchronous call (rsg_step_controls), with the goal and
    # bump callbacks registered so that the ticks run in event-draining chunks
    b3, _ = setup_gpu(scs)
    b3.set_goal_score_callback(lambda arena, team: None)
    b3.set_car_bump_callback(lambda arena, a, b, demo: None)
    b3.step_controls(seq, 8)
    s3 = b3.get_all_states()
    assert all(x.tobytes() == y.tobytes() for x, y in zip(s1, s3))
    b1.close()
    b2.close()
    b3.close()


def _device_controls_run(scs, ticks, first_launch):
    """Steps `scs` with device-resident per-tick controls: one launch of `first_launch` ticks, then
    one-tick launches; returns the bytes of every state."""
    import torch
    b, _ = setup_gpu(scs)
    mc = b.max_cars
    n = len(scs) * mc * CONTROLS_DTYPE.itemsize
    seq = np.concatenate([gpu_controls(scs, t, mc) for t in range(ticks)])
    dev = torch.from_numpy(seq.view(np.uint8).copy()).cuda()
    torch.cuda.synchronize()
    b.step_async(dev.data_ptr(), first_launch)
    b.sync()
    for t in range(first_launch, ticks):
        b.step_async(dev[t * n:].data_ptr(), 1)
        b.sync()
    out = b"".join(x.tobytes() for x in b.get_all_states())
    b.close()
    return out


def test_device_controls_are_deterministic():
    """Device-resident controls are applied by the block's threads to every arena of the block, after
    every warp has loaded its arena: the same batch gives the same bytes on every run (40 arenas in
    three blocks, an 8-tick launch then one-tick launches), and a batch stepped while another batch
    exists gives the same bytes as alone."""
    scs = random_scenarios(40, base_seed=2000)
    runs = {_device_controls_run(scs, 24, 8) for _ in range(3)}
    assert len(runs) == 1
    small = random_scenarios(6, base_seed=3001)
    alone = _device_controls_run(small, 8, 8)
    other, _ = setup_gpu(random_scenarios(6, base_seed=3000))
    try:
        assert _device_controls_run(small, 8, 8) == alone
    finally:
        other.close()


def test_goal_event_matches_restatement():
    from rocketsim_gb300 import abi
    sc = make_scenario(11, ncars=2, air_frac=0.0)
    sc.ball.pos = abi.Vec3(0.0, 4700.0, 200.0)
    sc.ball.vel = abi.Vec3(0.0, 3000.0, 0.0)
    batch, ids = setup_gpu([sc])
    goals = []
    batch.set_goal_score_callback(lambda arena, team: goals.append((arena, team, batch.get_tick_count(arena))))
    for t in range(60):
        batch.set_controls_all(gpu_controls([sc], t, batch.max_cars))
        batch.step(1)
    a, _ = run_cpu("oracle", sc, 60)
    ev = [e for e in a.pop_events() if e[0] == 1]
    a.close()
    assert goals, "no goal event on the GPU"
    assert [(0, int(e[2])) for e in ev] == [(g[0], g[1]) for g in goals]
    batch.close()


def test_errors_are_reported():
    import rocketsim_gb300 as rsg
    from rocketsim_gb300 import abi
    rsg.init_from_mem([mesh_bytes()])
    b = rsg.ArenaBatch(abi.GAMEMODE_SOCCAR, 2, 2)
    with pytest.raises(abi.RSGError) as e:
        b.add_car(5, 0)
    assert e.value.code == abi.ERR_ARG
    b.add_car(0, 0)
    b.add_car(0, 1)
    with pytest.raises(abi.RSGError) as e:
        b.add_car(0, 0)
    assert e.value.code == abi.ERR_STATE
    with pytest.raises(abi.RSGError):
        b.set_car_update_order(0, [1, 1])
    with pytest.raises(abi.RSGError):
        b.get_car_state(1, 1)
    b.close()
    with pytest.raises(abi.RSGError):
        rsg.ArenaBatch(abi.GAMEMODE_SOCCAR, 1, 2, tick_rate=200.0)


def test_remove_car_keeps_the_others():
    sc = make_scenario(21, ncars=4)
    batch, ids = setup_gpu([sc])
    keep = [c for c in ids[0] if c != ids[0][1]]
    before = {c: bytes(batch.get_car_state(0, c)) for c in keep}
    batch.remove_car(0, ids[0][1])
    assert sorted(batch.get_cars(0)) == sorted(keep)
    for c in keep:
        assert bytes(batch.get_car_state(0, c)) == before[c]
    batch.step(4)
    batch.close()


def test_the_void_free_flight_matches_restatement():
    import rocketsim_gb300 as rsg
    from oracle.pyoracle import SimArena, CarState as OCarState
    from rocketsim_gb300 import abi
    sc = make_scenario(31, ncars=2, air_frac=1.0)
    b = rsg.ArenaBatch(abi.GAMEMODE_THE_VOID, 1, 2)
    ids = [b.add_car(0, t, 0, 0) for t in sc.teams]
    o = SimArena("oracle", None, game_mode=5)
    oids = [o.add_car(t, 0) for t in sc.teams]
    for cid, ocid, s in zip(ids, oids, sc.cars):
        b.set_car_state(0, cid, s)
        o.set_car(ocid, OCarState.from_buffer_copy(bytes(s)))
    o.set_car_order(oids)
    b.step(8)
    o.step(8)
    for cid, ocid in zip(ids, oids):
        g, r = b.get_car_state(0, cid), o.get_car(ocid)
        d = max(abs(getattr(g.pos, c) - getattr(r.pos, c)) for c in "xyz")
        assert d <= TOL[8]["pos"], d
    b.close()
    o.close()


def test_launch_shapes_give_identical_results(golden, monkeypatch):
    """Every launch shape the tuner may choose (arenas per block, threads per car, BVH headers in shared
    memory or not, leaf grid or BVH walk, block-wide barriers in the collision work or not, a persistent
    launch or not: at this size a persistent launch has a block per group), with the
    arenas re-placed in blocks by cost after every launch, steps the golden scenarios (each three times
    in the batch) to bit-identical states."""
    scs = golden.scenarios * 3
    results = []
    for shape in ("8,4,-1,1", "4,1,0,1", "6,2,1,0", "7,4,1,1,1", "5,1,0,0,1", "8,2,1,1,1", "8,4,0,1,1,1", "5,2,1,0,0,1",
                  "16,4,0,1,1,0", "12,1,1,1,0,1"):
        monkeypatch.setenv("RSG_TICK_SHAPE", shape)
        batch, _ = setup_gpu(scs)
        want, got = [int(x) for x in shape.split(",")], batch.tick_shape()
        assert got[1] == want[1] and 1 <= got[0] <= want[0]  # arenas per block as shared memory allows
        for t in range(24):
            batch.set_controls_all(gpu_controls(scs, t, batch.max_cars))
            batch.step(1)
        cars, balls, pads = batch.get_all_states()
        results.append((cars.tobytes(), balls.tobytes(), pads.tobytes()))
        batch.close()
    assert all(r == results[0] for r in results[1:])


def test_tuner_reports_its_trials():
    """The first launch of a batch runs the shape tuner from one saved state: the log lists the
    trials, the chosen shape is one of them, and the batch's results equal a fixed-shape batch's."""
    import os
    scs = random_scenarios(16, base_seed=4000)
    assert "RSG_TICK_SHAPE" not in os.environ
    b1, _ = setup_gpu(scs)
    for t in range(16):
        b1.set_controls_all(gpu_controls(scs, t, b1.max_cars))
        b1.step(1)
    log = b1.tuning_log()
    assert log.startswith("chose ") and "ms/tick" in log, log
    s1 = b1.get_all_states()
    b1.close()
    os.environ["RSG_TICK_SHAPE"] = "8,4,-1,1"
    try:
        b2, _ = setup_gpu(scs)
        for t in range(16):
            b2.set_controls_all(gpu_controls(scs, t, b2.max_cars))
            b2.step(1)
        s2 = b2.get_all_states()
        b2.close()
    finally:
        del os.environ["RSG_TICK_SHAPE"]
    assert s1[0].tobytes() == s2[0].tobytes() and s1[1].tobytes() == s2[1].tobytes()
