"""Plane walls of the reference (type PlaneWall, Prtcl_Geometry.f90:17-37).

plane_wall() computes the derived fields exactly as G_add_PlaneWall does
(Prtcl_Geometry.f90:222-236) and packs one wall into the sdem_set_walls layout
(25 doubles + 4 ints).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List, Sequence

import numpy as np

W_SIZE = 25
WF_SIZE = 4


def _cross(u, v):
    return (u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2], u[0] * v[1] - u[1] * v[0])


def _dot(a, b):
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]


@dataclass
class WallSet:
    walls: List[np.ndarray] = field(default_factory=list)   # each (25,)
    flags: List[np.ndarray] = field(default_factory=list)   # each (4,) int32

    def add(self, p1, p2, p3, p4, wall_type: int = 1, both: bool = False, infinite: bool = True,
            vel=(0.0, 0.0, 0.0), base_wall_id: int = 10000000) -> None:
        """G_add_PlaneWall; the program wall id is Base_wall_id + running count
        (Prtcl_Geometry.f90:242-243)."""
        w, f = plane_wall(p1, p2, p3, p4, wall_id=base_wall_id + len(self.walls) + 1, wall_type=wall_type,
                          both=both, infinite=infinite, vel=vel)
        self.walls.append(w)
        self.flags.append(f)

    @property
    def n(self) -> int:
        return len(self.walls)

    def arrays(self):
        if not self.walls:
            return np.zeros(0), np.zeros(0, dtype=np.int32)
        return np.concatenate(self.walls), np.concatenate(self.flags).astype(np.int32)


def plane_wall(p1, p2, p3, p4, wall_id: int, wall_type: int = 1, both: bool = False, infinite: bool = True,
               vel=(0.0, 0.0, 0.0)):
    p1, p2, p3, p4 = (tuple(float(c) for c in p) for p in (p1, p2, p3, p4))
    a = (p2[0] - p1[0], p2[1] - p1[1], p2[2] - p1[2])
    b = (p3[0] - p1[0], p3[1] - p1[1], p3[2] - p1[2])
    ln = _cross(a, b)
    nrm = math.sqrt(ln[0] * ln[0] + ln[1] * ln[1] + ln[2] * ln[2])
    n = (ln[0] / nrm, ln[1] / nrm, ln[2] / nrm)
    d = -(_dot(n, p1))
    mn = tuple(min(p4[k], min(p3[k], min(p2[k], p1[k]))) for k in range(3))
    mx = tuple(max(p4[k], max(p3[k], max(p2[k], p1[k]))) for k in range(3))
    if abs(_dot(n, p4) + d) >= 0.00001:
        raise ValueError("Cannot create a plane wall: the four points are not coplanar")
    w = np.array([*p1, *p2, *p3, *p4, *n, d, *[float(v) for v in vel], *mn, *mx], dtype=np.float64)
    f = np.array([int(both), int(infinite), int(wall_id), int(wall_type)], dtype=np.int32)
    return w, f


def box_walls(dmin: Sequence[float], dmax: Sequence[float], infinite: bool = True, top: bool = False,
              wall_type: int = 1, base_wall_id: int = 10000000, skip_axes: Sequence[int] = ()) -> WallSet:
    """Floor (y = min) and four side walls (x and z), normals pointing into the
    box, as &GeometryMakingParam planes.  top=True adds a lid.  Faces normal to
    an axis in skip_axes (a periodic direction) are left out."""
    x0, y0, z0 = dmin
    x1, y1, z1 = dmax
    ws = WallSet()
    kw = dict(wall_type=wall_type, infinite=infinite, base_wall_id=base_wall_id)
    faces = [
        (1, ((x0, y0, z0), (x0, y0, z1), (x1, y0, z1), (x1, y0, z0))),   # floor: normal +y
        (0, ((x0, y0, z0), (x0, y1, z0), (x0, y1, z1), (x0, y0, z1))),   # x = x0, normal +x
        (0, ((x1, y0, z0), (x1, y0, z1), (x1, y1, z1), (x1, y1, z0))),   # x = x1, normal -x
        (2, ((x0, y0, z0), (x1, y0, z0), (x1, y1, z0), (x0, y1, z0))),   # z = z0, normal +z
        (2, ((x0, y0, z1), (x0, y1, z1), (x1, y1, z1), (x1, y0, z1))),   # z = z1, normal -z
    ]
    if top:
        faces.append((1, ((x0, y1, z0), (x1, y1, z0), (x1, y1, z1), (x0, y1, z1))))
    for axis, pts in faces:
        if axis not in skip_axes:
            ws.add(*pts, **kw)
    return ws
