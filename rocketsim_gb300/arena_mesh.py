"""Seeded procedural soccar arena written in RocketSim's ``.cmf`` mesh format.

The real Rocket League collision meshes are dumped from the game and are not
redistributable, so this module builds a stand-in hull with the same overall
shape:

* flat floor 8192 x 10240 uu (x in [-4096, 4096], y in [-5120, 5120]);
* side walls at x = +-4096, back walls at y = +-5120 and a ceiling at z = 2044;
* quarter-pipe fillets of radius 256 uu between floor and walls and between
  walls and ceiling, spherical fillets in the eight corners and cylindrical
  fillets on the four vertical edges;
* two goal openings 1786 uu wide and 642 uu high in the back walls, each with a
  goal box 840 uu deep behind it.

The seed only chooses the diagonal of every quad, so all seeds describe the same
surface with a different triangulation (about 20k triangles).

``.cmf`` layout (src/CollisionMeshFile/CollisionMeshFile.cpp:18-35): little
endian ``int32 numTris, int32 numVerts``, then ``numTris x 3 int32`` vertex
indices, then ``numVerts x 3 float32`` positions.  Positions are in Bullet units
(uu / 50) because the reference feeds them to Bullet unscaled
(CollisionMeshFile.cpp:63-73).
"""
from __future__ import annotations

import math
import struct

import numpy as np

UU_PER_BT = 50.0

EXT_X = 4096.0
EXT_Y = 5120.0
CEIL_Z = 2044.0
FILLET_R = 256.0
GOAL_HALF_W = 893.0
GOAL_H = 642.0
GOAL_DEPTH = 840.0
GRID = 256.0
SEGS = 16  # angular segments of every quarter-circle fillet


class _MeshBuilder:
    def __init__(self, seed: int):
        self.rng = np.random.default_rng(seed)
        self.verts: list[tuple[float, float, float]] = []
        self.index: dict[tuple[float, float, float], int] = {}
        self.tris: list[tuple[int, int, int]] = []

    def vid(self, p) -> int:
        key = (round(float(p[0]), 4), round(float(p[1]), 4), round(float(p[2]), 4))
        i = self.index.get(key)
        if i is None:
            i = len(self.verts)
            self.index[key] = i
            self.verts.append(key)
        return i

    def tri(self, a, b, c, inward) -> None:
        a, b, c = (np.asarray(v, dtype=np.float64) for v in (a, b, c))
        n = np.cross(b - a, c - a)
        area2 = float(np.dot(n, n))
        if area2 < 1e-6:
            return  # degenerate (fillet pole)
        centroid = (a + b + c) / 3.0
        if float(np.dot(n, inward(centroid))) < 0.0:
            b, c = c, b
        self.tris.append((self.vid(a), self.vid(b), self.vid(c)))

    def quad(self, p0, p1, p2, p3, inward) -> None:
        if self.rng.integers(0, 2) == 0:
            self.tri(p0, p1, p2, inward)
            self.tri(p0, p2, p3, inward)
        else:
            self.tri(p0, p1, p3, inward)
            self.tri(p1, p2, p3, inward)

    def surface(self, us, vs, f, inward) -> None:
        pts = [[np.asarray(f(u, v), dtype=np.float64) for v in vs] for u in us]
        for i in range(len(us) - 1):
            for j in range(len(vs) - 1):
                self.quad(pts[i][j], pts[i + 1][j], pts[i + 1][j + 1], pts[i][j + 1], inward)


def _breaks(lo: float, hi: float, step: float, extra=()) -> list[float]:
    vals = set()
    x = lo
    while x < hi - 1e-6:
        vals.add(round(x, 6))
        x += step
    vals.add(round(hi, 6))
    for e in extra:
        if lo < e < hi:
            vals.add(round(e, 6))
    return sorted(vals)


def build_arena_mesh(seed: int = 0) -> tuple[np.ndarray, np.ndarray]:
    """Return (vertices float32 [V,3] in uu, triangles int32 [T,3])."""
    m = _MeshBuilder(seed)
    r = FILLET_R
    ix, iy = EXT_X - r, EXT_Y - r  # fillet axis offsets
    lo_z, hi_z = r, CEIL_Z - r
    angs = [0.5 * math.pi * k / SEGS for k in range(SEGS + 1)]
    xs = _breaks(-ix, ix, GRID, extra=(-GOAL_HALF_W, GOAL_HALF_W))
    ys = _breaks(-iy, iy, GRID)
    up = lambda p: np.array([0.0, 0.0, 1.0])
    down = lambda p: np.array([0.0, 0.0, -1.0])

    # floor and ceiling
    m.surface(xs, ys, lambda x, y: (x, y, 0.0), up)
    m.surface(xs, ys, lambda x, y: (x, y, CEIL_Z), down)

    # goal-mouth floor strips between the fillet line and the goal line
    mouth_xs = [x for x in xs if -GOAL_HALF_W <= x <= GOAL_HALF_W]
    for s in (-1.0, 1.0):
        m.surface(mouth_xs, [s * iy, s * EXT_Y], lambda x, y: (x, y, 0.0), up)

    def toward_axis(center_fn):
        return lambda p: center_fn(p) - p

    # floor / ceiling fillets along the side walls (axis parallel to y)
    for sx in (-1.0, 1.0):
        for lower in (True, False):
            cz = lo_z if lower else hi_z
            def fx(a, y, sx=sx, cz=cz, lower=lower):
                return (sx * (ix + r * math.sin(a)), y, cz - r * math.cos(a) if lower else cz + r * math.cos(a))
            m.surface(angs, ys, fx, toward_axis(lambda p, sx=sx, cz=cz: np.array([sx * ix, p[1], cz])))

    # floor / ceiling fillets along the back walls (axis parallel to x); the
    # floor fillet is interrupted by the goal opening
    for sy in (-1.0, 1.0):
        for lower in (True, False):
            cz = lo_z if lower else hi_z
            segs = ([x for x in xs if x <= -GOAL_HALF_W], [x for x in xs if x >= GOAL_HALF_W]) if lower else (xs,)
            for seg in segs:
                def fy(a, x, sy=sy, cz=cz, lower=lower):
                    return (x, sy * (iy + r * math.sin(a)), cz - r * math.cos(a) if lower else cz + r * math.cos(a))
                m.surface(angs, seg, fy, toward_axis(lambda p, sy=sy, cz=cz: np.array([p[0], sy * iy, cz])))

    # spherical corner fillets (floor and ceiling) and vertical corner fillets
    for sx in (-1.0, 1.0):
        for sy in (-1.0, 1.0):
            for lower in (True, False):
                cz = lo_z if lower else hi_z
                c = np.array([sx * ix, sy * iy, cz])
                def fs(a, b, sx=sx, sy=sy, cz=cz, lower=lower):
                    zz = -r * math.cos(b) if lower else r * math.cos(b)
                    return (sx * (ix + r * math.cos(a) * math.sin(b)), sy * (iy + r * math.sin(a) * math.sin(b)), cz + zz)
                m.surface(angs, angs, fs, lambda p, c=c: c - p)
            zs = _breaks(lo_z, hi_z, GRID)
            def fv(a, z, sx=sx, sy=sy):
                return (sx * (ix + r * math.cos(a)), sy * (iy + r * math.sin(a)), z)
            m.surface(angs, zs, fv, lambda p, sx=sx, sy=sy: np.array([sx * ix, sy * iy, p[2]]) - p)

    # side walls
    zs = _breaks(lo_z, hi_z, GRID)
    for sx in (-1.0, 1.0):
        m.surface(ys, zs, lambda y, z, sx=sx: (sx * EXT_X, y, z), lambda p, sx=sx: np.array([-sx, 0.0, 0.0]))

    # back walls with the goal opening cut out
    zb = _breaks(lo_z, hi_z, GRID, extra=(GOAL_H,))
    for sy in (-1.0, 1.0):
        inward = lambda p, sy=sy: np.array([0.0, -sy, 0.0])
        for i in range(len(xs) - 1):
            for j in range(len(zb) - 1):
                x0, x1, z0, z1 = xs[i], xs[i + 1], zb[j], zb[j + 1]
                if x0 >= -GOAL_HALF_W and x1 <= GOAL_HALF_W and z1 <= GOAL_H:
                    continue
                y = sy * EXT_Y
                m.quad((x0, y, z0), (x1, y, z0), (x1, y, z1), (x0, y, z1), inward)
        # goal box behind the opening
        y0, y1 = sy * EXT_Y, sy * (EXT_Y + GOAL_DEPTH)
        gy = _breaks(min(y0, y1), max(y0, y1), GRID)
        gz = _breaks(0.0, GOAL_H, GRID)
        m.surface(mouth_xs, gy, lambda x, y: (x, y, 0.0), up)
        m.surface(mouth_xs, gy, lambda x, y: (x, y, GOAL_H), down)
        for sx in (-1.0, 1.0):
            m.surface(gy, gz, lambda y, z, sx=sx: (sx * GOAL_HALF_W, y, z), lambda p, sx=sx: np.array([-sx, 0.0, 0.0]))
        m.surface(mouth_xs, gz, lambda x, z, y1=y1: (x, y1, z), lambda p, sy=sy: np.array([0.0, -sy, 0.0]))

    verts = np.asarray(m.verts, dtype=np.float32)
    tris = np.asarray(m.tris, dtype=np.int32)
    return verts, tris


def to_cmf_bytes(verts_uu: np.ndarray, tris: np.ndarray) -> bytes:
    """Serialise to the ``.cmf`` byte layout with positions in Bullet units."""
    v_bt = (np.asarray(verts_uu, dtype=np.float64) / UU_PER_BT).astype("<f4")
    t = np.asarray(tris, dtype="<i4")
    return struct.pack("<ii", int(t.shape[0]), int(v_bt.shape[0])) + t.tobytes() + v_bt.tobytes()


def arena_cmf(seed: int = 0) -> bytes:
    v, t = build_arena_mesh(seed)
    return to_cmf_bytes(v, t)


def parse_cmf(data: bytes) -> tuple[np.ndarray, np.ndarray]:
    """Inverse of :func:`to_cmf_bytes`; returns (vertices in BT units, tris)."""
    nt, nv = struct.unpack_from("<ii", data, 0)
    off = 8
    tris = np.frombuffer(data, dtype="<i4", count=nt * 3, offset=off).reshape(nt, 3)
    off += nt * 12
    verts = np.frombuffer(data, dtype="<f4", count=nv * 3, offset=off).reshape(nv, 3)
    return verts, tris
