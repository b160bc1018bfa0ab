"""The serialized arenas of the reference (tests/golden/serial_arenas.npz) read by the format reader
the GPU tests use (CPU only)."""
from __future__ import annotations

import os

import numpy as np

from serial_format import parse_arena, reorder_cars_ascending

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


def test_car_reordering_keeps_every_field():
    """The fixture's blobs hold their cars by ascending id; reordering them again is the identity, and
    reordering a blob with its cars reversed gives the same bytes back."""
    z = np.load(PATH)
    for i in range(len(z["offsets"]) - 1):
        blob = z["blob"][z["offsets"][i]:z["offsets"][i + 1]].tobytes()
        d = parse_arena(blob)
        assert [c["id"] for c in d["cars"]] == sorted(c["id"] for c in d["cars"])
        assert reorder_cars_ascending(blob) == blob
        first, last = d["cars"][0]["span"][0], d["cars"][-1]["span"][1]
        rev = blob[:first] + b"".join(blob[c["span"][0]:c["span"][1]] for c in reversed(d["cars"])) + blob[last:]
        assert reorder_cars_ascending(rev) == blob
