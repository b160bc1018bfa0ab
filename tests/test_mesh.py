"""The procedural arena mesh and its .cmf encoding."""
import struct

import numpy as np

from rocketsim_gb300.arena_mesh import arena_cmf, build_arena_mesh, parse_cmf


def test_cmf_round_trip_and_size():
    data = arena_cmf(0)
    nt, nv = struct.unpack_from("<ii", data, 0)
    assert len(data) == 8 + nt * 12 + nv * 12
    verts, tris = parse_cmf(data)
    assert tris.shape == (nt, 3) and verts.shape == (nv, 3)
    assert 15000 <= nt <= 30000, nt
    assert tris.min() >= 0 and tris.max() < nv


def test_mesh_is_seeded():
    assert arena_cmf(0) == arena_cmf(0)
    assert arena_cmf(0) != arena_cmf(1)


def test_mesh_extent():
    verts, tris = parse_cmf(arena_cmf(0))
    uu = verts * 50.0  # .cmf vertices are in Bullet units
    assert uu[:, 2].min() >= -1e-3
    assert abs(uu[:, 0].max() - 4096) < 5 and abs(uu[:, 2].max() - 2044) < 5
