"""Triangle meshes of magnet shapes in lattice coordinates.

The reference voxelises binary STL files (src/mesh.rs:175-343).  Its two
shipped magnets (stl/disk-magnet.stl, stl/ring-magnet.stl) do not have the
proportions of the benchmark magnets, so these helpers tessellate a closed
cylinder (disk magnet) or annulus (ring magnet) directly; the triangles go
through the same voxeliser as an imported STL.
"""
from __future__ import annotations

import numpy as np


def _axis_frame(axis: int):
    e = np.eye(3, dtype=np.float64)
    a = e[axis]
    u = e[(axis + 1) % 3]
    v = e[(axis + 2) % 3]
    return a, u, v


def annulus(center, r_out: float, r_in: float, thickness: float, axis: int = 2, segments: int = 128):
    """Closed annulus (r_in > 0) or cylinder (r_in == 0): returns p0, p1, p2 as float32 [ntri][3]."""
    c = np.asarray(center, np.float64)
    a, u, v = _axis_frame(axis)
    ang = np.linspace(0.0, 2.0 * np.pi, segments, endpoint=False)
    ang1 = np.roll(ang, -1)
    h0, h1 = -0.5 * thickness, 0.5 * thickness

    def ring(r, th, h):
        return c + r * np.cos(th)[:, None] * u + r * np.sin(th)[:, None] * v + h * a

    tris = []
    # outer wall
    o00, o01, o10, o11 = ring(r_out, ang, h0), ring(r_out, ang1, h0), ring(r_out, ang, h1), ring(r_out, ang1, h1)
    tris += [(o00, o01, o11), (o00, o11, o10)]
    if r_in > 0.0:
        i00, i01, i10, i11 = ring(r_in, ang, h0), ring(r_in, ang1, h0), ring(r_in, ang, h1), ring(r_in, ang1, h1)
        tris += [(i00, i11, i01), (i00, i10, i11)]
        # caps between the circles
        tris += [(o10, o11, i11), (o10, i11, i10)]  # top
        tris += [(o00, i01, o01), (o00, i00, i01)]  # bottom
    else:
        ctop = np.repeat((c + h1 * a)[None], segments, 0)
        cbot = np.repeat((c + h0 * a)[None], segments, 0)
        tris += [(ctop, o10, o11), (cbot, o01, o00)]
    p0 = np.concatenate([t[0] for t in tris]).astype(np.float32)
    p1 = np.concatenate([t[1] for t in tris]).astype(np.float32)
    p2 = np.concatenate([t[2] for t in tris]).astype(np.float32)
    return p0, p1, p2


def cylinder(center, radius: float, thickness: float, axis: int = 2, segments: int = 128):
    """Closed cylinder (a disk magnet)."""
    return annulus(center, radius, 0.0, thickness, axis, segments)
