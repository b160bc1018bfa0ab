"""Writes tests/golden/serial_arenas.npz from the reference RocketSim: serialized arenas and how the
reference continues from them.

Run here, where the reference sources exist: ``python tests/golden/make_serial_golden.py``.
For each scenario the reference plays 30 ticks, writes Arena::Serialize's bytes and records the
car / ball / pad states.  The bytes are stored with their cars by ascending id (the reference's
DeserializeNew loses cars otherwise: it gives each car read the next id before forcing the written
one, Arena.cpp:590-606); an arena made from them by DeserializeNew then plays 8 more ticks of the
scenario's controls, and its car update order and its states after them (continuous and discrete)
are recorded: what resuming from the bytes gives in the reference (the vehicle state CarState does
not hold, such as the wheels' friction factors, starts afresh there too).  Arena::Clone of the
arena at tick 30 plays the same 8 ticks; its car update order and end states are recorded too.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from scenarios import (CONTROLS_DTYPE, _controls_struct, cpu_snapshot, discrete_car, discrete_pads,  # noqa: E402
                       make_carcar_scenario, make_scenario, setup_cpu)
from rocketsim_gb300 import abi  # noqa: E402
from serial_format import reorder_cars_ascending  # noqa: E402

OUT = os.path.join(HERE, "serial_arenas.npz")
T0, T1 = 30, 8


def scenario_list():
    return [make_scenario(400), make_scenario(401, ncars=6, presets=[0, 1, 2, 3, 4, 5]),
            make_scenario(402, ncars=2, presets=[1, 2]), make_carcar_scenario(3)]


def main():
    from oracle.pyoracle import SimArena, build_ref, CarControls as OCtl
    if build_ref() is None:
        raise SystemExit("reference sources not found")
    scs = scenario_list()
    S, MC = len(scs), max(len(s.cars) for s in scs)
    car_dt, ball_dt, pad_dt = np.dtype(abi.CarState), np.dtype(abi.BallState), np.dtype(abi.PadState)
    blobs, order_ids = [], np.zeros((S, MC), np.uint32)
    controls = np.zeros((S, T1, MC), CONTROLS_DTYPE)
    cars_t0 = np.zeros((S, MC), car_dt)
    ball_t0 = np.zeros(S, ball_dt)
    pads_t0 = np.zeros((S, 34), pad_dt)
    cars_end = np.zeros((S, MC), car_dt)
    ball_end = np.zeros(S, ball_dt)
    pads_end = np.zeros((S, 34), pad_dt)
    clone_order = np.zeros((S, MC), np.uint32)
    clone_cars_end = np.zeros((S, MC), car_dt)
    clone_ball_end = np.zeros(S, ball_dt)
    clone_pads_end = np.zeros((S, 34), pad_dt)
    disc = np.zeros((S, T1, MC, 28), np.float32)
    ncars = np.array([len(s.cars) for s in scs], np.int32)
    for si, sc in enumerate(scs):
        a, ids = setup_cpu("ref", sc)
        n = len(ids)

        def play(a, t):
            for i, cid in enumerate(ids):
                a.set_controls(cid, OCtl.from_buffer_copy(bytes(_controls_struct(sc.controls[t, i]))))
            a.step(1)
        for t in range(T0):
            play(a, t)
        blob = reorder_cars_ascending(a.serialize())
        blobs.append(np.frombuffer(blob, np.uint8))
        cars, ball, pads = cpu_snapshot(a, ids)
        cars_t0[si, :n] = cars
        ball_t0[si] = ball[0]
        pads_t0[si] = pads
        c = a.clone()
        a.close()
        clone_order[si, :n] = c.car_order()
        for t in range(T0, T0 + T1):
            play(c, t)
        cars, ball, pads = cpu_snapshot(c, ids)
        clone_cars_end[si, :n], clone_ball_end[si], clone_pads_end[si] = cars, ball[0], pads
        c.close()
        a = SimArena.deserialize_new(blob)
        assert sorted(a.car_order()) == ids
        order_ids[si, :n] = a.car_order()
        for t in range(T0, T0 + T1):
            controls[si, t - T0, :n] = sc.controls[t]
            play(a, t)
            cars, ball, pads = cpu_snapshot(a, ids)
            disc[si, t - T0, :n] = discrete_car(cars)
        cars_end[si, :n] = cars
        ball_end[si] = ball[0]
        pads_end[si] = pads
        a.close()
    offs = np.cumsum([0] + [len(b) for b in blobs]).astype(np.int64)
    np.savez_compressed(OUT, blob=np.concatenate(blobs), offsets=offs, ncars=ncars, order_ids=order_ids,
                        controls=controls, cars_t0=cars_t0, ball_t0=ball_t0, pads_t0=pads_t0, cars_end=cars_end, ball_end=ball_end, pads_end=pads_end, disc=disc,
                        clone_order=clone_order, clone_cars_end=clone_cars_end, clone_ball_end=clone_ball_end,
                        clone_pads_end=clone_pads_end,
                        ids=np.array([[i + 1 for i in range(MC)] for _ in scs], np.uint32))
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
