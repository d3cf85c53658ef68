"""File formats through the C ABI, against the CPU restatements of
oracle/ion_files.py:

* ``.ion`` (ion_lbm_save / ion_lbm_load): the writer's bytes equal, byte for
  byte, file::encode restated from src/file.rs:191-306 and FILE_LAYOUT.txt;
  a reference-layout MHD file without the N_C / N_M sections (what the
  reference's writer produces, file.rs:276-303) and one with them
  (FILE_LAYOUT.txt:42-57) load with every field and config value intact.
* STL import (ion_lbm_import_mesh / ion_lbm_import_mesh_reposition) of the
  reference's own fixtures (tests/golden/disk-magnet.stl, ring-magnet.stl)
  with non-zero rotations: triangles and bounds bit for bit against
  Mesh::read_stl_raw restated (src/mesh.rs:51-66, 94-109, 175-253); the
  voxelised flags and static field bit for bit against the oracle
  voxelising the restated triangles.
"""
from pathlib import Path

import numpy as np
import pytest

import ionsolver_gb300 as I
from ionsolver_gb300 import workloads as W
from oracle import ion_files as F
from tests import _util as U

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"


def _cfg_dict(lbm):
    c = lbm.config
    u = c.units
    return dict(velocity_set=int(c.velocity_set), relaxation_time=int(c.relaxation_time),
                float_type=int(c.float_type), units=dict(m=u.m, kg=u.kg, s=u.s, a=u.a), n_x=c.n_x, n_y=c.n_y,
                n_z=c.n_z, d_x=c.d_x, d_y=c.d_y, d_z=c.d_z, nu=c.nu, f_x=c.f_x, f_y=c.f_y, f_z=c.f_z,
                ext_equilibrium_boundaries=c.ext_equilibrium_boudaries, ext_volume_force=c.ext_volume_force,
                ext_force_field=c.ext_force_field, ext_magneto_hydro=c.ext_magneto_hydro,
                mhd_lod_depth=c.mhd_lod_depth)


@pytest.mark.parametrize("kind", ["plain_fp16s_trt", "mhd_plasma", "boundaries_force"])
def test_save_bytes_equal_the_reference_encoder(kind, tmp_path):
    if kind == "plain_fp16s_trt":
        case = W.taylor_green(shape=(24, 20, 16), amplitude=0.05, float_type=0, relaxation_time=1)
        case["fields"]["flags"] = W.shell_flags(24, 20, 16)
    elif kind == "mhd_plasma":
        case = W.mhd_plasma(n=16, depth=2, magnet_r=4.0, magnet_t=3.0, float_type=1)
    else:
        case = W.taylor_green(shape=(16, 12, 8), amplitude=0.03)
        case["config"].update(ext_equilibrium_boundaries=1, ext_volume_force=1, f_x=1e-6, f_y=-2e-6, f_z=3e-7)
    g = U.run_gpu(case, 3)
    p = tmp_path / "a.ion"
    g.write_file(p)
    mhd = bool(case["config"].get("ext_magneto_hydro"))
    ref = F.encode_ion(_cfg_dict(g), g.read("flags"), g.read("rho"), g.read("u"), g.read("q") if mhd else None)
    got = p.read_bytes()
    assert len(got) == 16 + 62 + g.n * (21 if mhd else 17) == len(ref)
    assert got == ref


@pytest.mark.parametrize("sections", [False, True], ids=["reference-writer", "with-NC-NM"])
def test_load_reference_layout_mhd(sections, tmp_path):
    rng = np.random.default_rng(21)
    nx, ny, nz = 16, 12, 8
    n = nx * ny * nz
    cfg = dict(velocity_set=2, relaxation_time=1, float_type=2, units=dict(m=0.5, kg=2.0, s=0.25, a=1e-3),
               n_x=nx, n_y=ny, n_z=nz, nu=0.05, f_x=1e-5, f_y=0.0, f_z=-2e-5, ext_volume_force=1,
               ext_magneto_hydro=1, ext_equilibrium_boundaries=1, mhd_lod_depth=2)
    flags = rng.choice(np.array([0, 1, 2, 0x11], np.uint8), n)
    rho = (1 + rng.normal(0, 1e-2, n)).astype(np.float32)
    u = rng.normal(0, 1e-2, 3 * n).astype(np.float32)
    q = rng.uniform(-1e-3, 1e-3, n).astype(np.float32)
    blob = F.encode_ion(cfg, flags, rho, u, q, sections=sections, charges=[(5, 1e-9), (77, -2e-9)],
                        magnets=[(100, (0.0, 0.0, 3e5))])
    p = tmp_path / "ref.ion"
    p.write_bytes(blob)
    g = I.Lbm.read_file(p)
    c = g.config
    assert (c.velocity_set, c.relaxation_time, c.float_type, c.n_x, c.n_y, c.n_z) == (2, 1, 2, nx, ny, nz)
    assert (c.units.m, c.units.kg, c.units.s, c.units.a) == (0.5, 2.0, 0.25, np.float32(1e-3))
    assert (c.nu, c.f_x, c.f_z) == (np.float32(0.05), np.float32(1e-5), np.float32(-2e-5))
    assert c.ext_magneto_hydro and c.ext_volume_force and c.ext_equilibrium_boudaries and not c.ext_force_field
    assert c.mhd_lod_depth == 2
    for name, ref in (("flags", flags), ("rho", rho), ("u", u), ("q", q)):
        assert U.bit_diff(g.read(name), ref) == 0, name
    # and the library writes the same bytes back (without the sections, as the reference's writer)
    out = tmp_path / "back.ion"
    g.write_file(out)
    assert out.read_bytes() == F.encode_ion(cfg, flags, rho, u, q)


STL_CASES = [
    ("disk-magnet.stl", "reposition", (40.0, 36.0, 30.0, 30.0, 45.0, 60.0, 40.0)),
    ("ring-magnet.stl", "reposition", (32.0, 32.0, 32.0, 90.0, 0.0, 17.5, 0.0)),  # size 0: fit the box
    ("disk-magnet.stl", "scale", (1.0, 30.0, 28.0, 33.0, -20.0, 10.0, 75.0)),     # SI scale, origin, rotation
]


@pytest.mark.parametrize("name,how,args", STL_CASES, ids=["disk-repos", "ring-fit", "disk-scale"])
def test_stl_import_and_voxelise(name, how, args):
    path = GOLDEN / name
    n = 64
    case = W.mhd_box(n=n, depth=2, magnet=False)
    # cells of 2.5 mm: the fixtures (0.1 m across, 0.01 m thick, centred on the origin) span 40 x 4 cells
    case["config"]["units"] = dict(m=2.5e-3, kg=1.0, s=1.0, a=1e-6, k=1.0, prop=0)
    g = U.setup_gpu(case)
    if how == "reposition":
        cx, cy, cz, rx, ry, rz, size = args
        idx = g.import_mesh_reposition(str(path), cx, cy, cz, rx, ry, rz, size)
        ref = F.import_mesh_reposition(path, (n, n, n), cx, cy, cz, rx, ry, rz, size)
    else:
        scale, ox, oy, oz, rx, ry, rz = args  # scale in SI: the fixtures are in metres
        idx = g.import_mesh(str(path), scale, ox, oy, oz, rx, ry, rz)
        ref = F.import_mesh(path, case["config"]["units"]["m"], scale, ox, oy, oz, rx, ry, rz)
    p0, p1, p2 = g.mesh_triangles(idx)
    for got, want in zip((p0, p1, p2), ref[:3]):
        assert U.bit_diff(got, want) == 0
    b = g.mesh_bounds(idx)
    assert U.bit_diff(np.asarray(b["p_min"], np.float32), ref[3]) == 0
    assert U.bit_diff(np.asarray(b["p_max"], np.float32), ref[4]) == 0
    assert U.bit_diff(np.asarray(b["center"], np.float32), ref[5]) == 0
    assert (ref[4] - ref[3]).max() > 8  # the mesh covers many cells
    # voxelise as a magnet, then the static field, against the oracle on the restated triangles
    g.voxelise_mesh(idx, I.ModelType.Magnet((0.0, 2e4, 1e4)))
    g.precompute_B()
    o = U.setup_oracle(case, canonical_nan=True)
    o.voxelise(ref[0], ref[1], ref[2], "magnet", (0.0, 2e4, 1e4))
    o.precompute_b()
    assert U.compare_bitwise(g, o, ["flags", "b_stat", "b_dyn"]) == {"flags": 0, "b_stat": 0, "b_dyn": 0}
    assert (g.read("flags") == 0x11).sum() > 50
