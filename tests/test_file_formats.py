"""CPU checks of the file-format restatements the GPU file tests compare
against (oracle/ion_files.py): the .ion byte layout of FILE_LAYOUT.txt (a
16-byte header, a 62-byte config block, 17 N bytes of cell data, 4 N more
with MHD, then the optional N_C / N_M sections) and the STL reader on the
reference's fixtures (84 + 50 T bytes; an identity rotation leaves the
vertices as stored, scaled and shifted)."""
import struct
from pathlib import Path

import numpy as np

from oracle import ion_files as F

GOLDEN = Path(__file__).resolve().parent / "golden"


def _cfg(mhd):
    return dict(velocity_set=2, relaxation_time=0, float_type=1, units=dict(m=1.0, kg=2.0, s=3.0, a=4.0),
                n_x=4, n_y=3, n_z=2, nu=0.1, f_x=1.0, f_y=2.0, f_z=3.0, ext_volume_force=1,
                ext_magneto_hydro=mhd, mhd_lod_depth=1)


def test_ion_layout():
    n = 24
    z = np.zeros(n, np.float32)
    plain = F.encode_ion(_cfg(0), np.zeros(n, np.uint8), z, np.zeros(3 * n, np.float32))
    mhd = F.encode_ion(_cfg(1), np.zeros(n, np.uint8), z, np.zeros(3 * n, np.float32), z)
    assert plain[:16] == b"IonSolver setup\n"
    assert len(plain) == 16 + 62 + 17 * n and len(mhd) == 16 + 62 + 21 * n
    # config block: enums, units, sizes, fixed-domain byte, domains, nu, force, extensions, LOD depth
    assert plain[16:19] == bytes([2, 0, 1])
    assert struct.unpack_from("<4f", plain, 19) == (1.0, 2.0, 3.0, 4.0)
    assert struct.unpack_from("<3I", plain, 35) == (4, 3, 2) and plain[47] == 0
    assert struct.unpack_from("<3I", plain, 48) == (1, 1, 1)
    assert plain[76:78] == bytes([0b0010, 1]) and mhd[76] == 0b1010
    sec = F.encode_ion(_cfg(1), np.zeros(n, np.uint8), z, np.zeros(3 * n, np.float32), z, sections=True,
                       charges=[(3, 1.5)], magnets=[(7, (1.0, 2.0, 3.0))])
    assert len(sec) == len(mhd) + 4 + 12 + 4 + 20
    assert struct.unpack_from("<IQf", sec, len(mhd)) == (1, 3, 1.5)


def test_stl_reader_identity_and_fit():
    path = GOLDEN / "disk-magnet.stl"
    data = path.read_bytes()
    nt = struct.unpack_from("<I", data, 80)[0]
    assert len(data) == 84 + 50 * nt
    raw = np.frombuffer(data, np.dtype([("n", "<f4", 3), ("v", "<f4", (3, 3)), ("a", "<u2")]), nt, 84)["v"]
    p0, p1, p2, pmin, pmax, c = F.read_stl_raw(path, False, (1, 1, 1), (0, 0, 0), F.rotation_deg(0, 0, 0), -1.0)
    assert np.array_equal(p0, raw[:, 0]) and np.array_equal(p2, raw[:, 2])
    # reposition + fit into a 64^3 box: centred on the given centre, longest side 64 * (the smallest ratio)
    p0, p1, p2, pmin, pmax, c = F.read_stl_raw(path, True, (64, 64, 64), (32, 32, 32), F.rotation_deg(0, 0, 0), 0.0)
    assert np.allclose(0.5 * (pmin + pmax), 32.0, atol=1e-4)
    assert np.isclose((pmax - pmin).max(), 64.0, rtol=1e-6)
    # a 90-degree turn about x swaps the thin axis (y) into z
    p0, p1, p2, pmin, pmax, c = F.read_stl_raw(path, True, (64, 64, 64), (0, 0, 0), F.rotation_deg(90, 0, 0), 40.0)
    ext = pmax - pmin
    assert ext[2] < 5 and ext[1] > 39
