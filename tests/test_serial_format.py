"""The serialized arenas of the reference (tests/golden/serial_arenas.npz) read by the format reader
the GPU tests use (CPU only)."""
from __future__ import annotations

import os

import numpy as np

from serial_format import parse_arena

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "serial_arenas.npz")


def test_reference_bytes_parse_completely():
    z = np.load(PATH)
    for i in range(len(z["offsets"]) - 1):
        d = parse_arena(z["blob"][z["offsets"][i]:z["offsets"][i + 1]].tobytes())
        n = int(z["ncars"][i])
        assert len(d["cars"]) == n and sorted(c["id"] for c in d["cars"]) == list(range(1, n + 1))
        assert d["tick_count"] == 30 and len(d["pads"]) == 34 and d["game_mode"] == 0
        assert abs(d["tick_time"] - 1 / 120) < 1e-9 and d["mutators"][0] == (0.0, 0.0, -650.0)
        for c in d["cars"]:  # the states the reference wrote are the ones its GetState reported
            ref = z["cars_t0"][i][c["id"] - 1]
            assert c["state"]["pos"] == (ref["pos"]["x"], ref["pos"]["y"], ref["pos"]["z"])
            assert c["state"]["boost"] == ref["boost"] and c["state"]["is_on_ground"] == ref["is_on_ground"]
        b = z["ball_t0"][i]
        assert d["ball"]["vel"] == (b["vel"]["x"], b["vel"]["y"], b["vel"]["z"])
