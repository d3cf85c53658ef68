"""Synthetic benchmark inputs and magnet meshes."""
import numpy as np

import oracle as O
from ionsolver_gb300 import workloads as W
from tests import _util as U


def test_mhd_inputs_are_seeded_and_shaped():
    a = W.mhd_box(n=32)
    b = W.mhd_box(n=32)
    for k in a["fields"]:
        assert np.array_equal(a["fields"][k], b["fields"][k])
    q = a["fields"]["q"]
    assert q.dtype == np.float32 and q.size == 32 ** 3 and np.abs(q).max() <= 1e-3
    u = a["fields"]["u"]
    assert abs(float(u.std()) - 1e-3) < 5e-5
    f = a["fields"]["flags"].reshape(32, 32, 32)
    assert f[0].all() and f[:, :, -1].all() and not f[1:-1, 1:-1, 1:-1].any()


def test_cylinder_mesh_is_closed():
    p0, p1, p2 = W.cylinder((0, 0, 0), 5.0, 2.0, segments=32)
    edges = {}
    for tri in zip(map(tuple, p0), map(tuple, p1), map(tuple, p2)):
        for a, b in ((0, 1), (1, 2), (2, 0)):
            key = tuple(sorted((tri[a], tri[b])))
            edges[key] = edges.get(key, 0) + 1
    assert set(edges.values()) == {2}


def test_voxelised_disk_volume():
    r, t = 8.0, 6.0
    case = W.mhd_box(n=32, depth=2, magnet_r=r, magnet_t=t)
    o = U.setup_oracle(case, "f32", 2)
    n_mag = int((o.field("flags") == 0x11).sum())
    assert abs(n_mag - np.pi * r * r * t) / (np.pi * r * r * t) < 0.1
