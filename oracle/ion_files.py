"""CPU restatements of IonSolver's file formats -- TEST INFRASTRUCTURE, not
product code.  Only tests use this module, as the checker of the library's
``.ion`` writer/reader and STL import.

* ``encode_ion``: ``file::encode`` (IonSolver src/file.rs:191-306) in the byte
  layout of FILE_LAYOUT.txt:1-59: the 16-byte header, the 62-byte config
  block, then flags, densities, velocities and (MHD) charges, little endian.
  The reference's writer emits no fixed-charge / magnet sections (its code
  for them is commented out, file.rs:276-303); ``sections=True`` appends the
  N_C / N_M sections as FILE_LAYOUT.txt:42-57 describes them, with the
  given records, for reader tests.
* ``read_stl_raw``: ``Mesh::read_stl_raw`` (src/mesh.rs:175-220) with the
  rotation matrix of ``construct_rotation_matrix`` / ``rotm_around_v``
  (src/mesh.rs:51-66), the matrix products of src/mesh.rs:393-429 and
  ``update_bounds`` (src/mesh.rs:94-109), in float32 operation for
  operation.  sin and cos of the angle come from the C library's sinf/cosf,
  the functions Rust's f32::sin/cos and the library's C++ call.
* ``import_mesh`` / ``import_mesh_reposition``: src/mesh.rs:233-253.
"""
from __future__ import annotations

import ctypes as C
import ctypes.util
import struct

import numpy as np

f32 = np.float32

_libm = C.CDLL(ctypes.util.find_library("m") or "libm.so.6")
_libm.sinf.restype = C.c_float
_libm.sinf.argtypes = [C.c_float]
_libm.cosf.restype = C.c_float
_libm.cosf.argtypes = [C.c_float]

PI_F = f32(3.14159265358979323846)  # std::f32::consts::PI


# ---------------------------------------------------------------------------
# .ion
# ---------------------------------------------------------------------------
def encode_ion(cfg: dict, flags: np.ndarray, rho: np.ndarray, u: np.ndarray, q: np.ndarray | None = None,
               sections: bool = False, charges=(), magnets=()) -> bytes:
    """file::encode (src/file.rs:191-306).  cfg holds the LbmConfig fields
    (velocity_set, relaxation_time, float_type as the enums' u8 values, units
    m/kg/s/a, n_x.., d_x.., nu, f_x.., the ext_* switches, mhd_lod_depth)."""
    u_ = cfg["units"]
    b = bytearray(b"IonSolver setup\n")                                 # pushname (file.rs:346-350)
    b += bytes([cfg["velocity_set"], cfg["relaxation_time"], cfg["float_type"]])  # enums as u8 (195-197)
    b += struct.pack("<4f", u_["m"], u_["kg"], u_["s"], u_["a"])          # units (198-201)
    b += struct.pack("<3I", cfg["n_x"], cfg["n_y"], cfg["n_z"])           # sizes (202-204)
    b += b"\x00"                                                         # fixed domains (205)
    b += struct.pack("<3I", cfg.get("d_x", 1), cfg.get("d_y", 1), cfg.get("d_z", 1))  # (206-208)
    b += struct.pack("<4f", cfg["nu"], cfg.get("f_x", 0.0), cfg.get("f_y", 0.0), cfg.get("f_z", 0.0))  # (209-212)
    ext = (int(bool(cfg.get("ext_equilibrium_boundaries"))) + (int(bool(cfg.get("ext_volume_force"))) << 1)
           + (int(bool(cfg.get("ext_force_field"))) << 2) + (int(bool(cfg.get("ext_magneto_hydro"))) << 3))
    b += bytes([ext, cfg.get("mhd_lod_depth", 4)])                       # (213-217)
    b += np.ascontiguousarray(flags, np.uint8).tobytes()                 # flags (228-235)
    b += np.ascontiguousarray(rho, "<f4").tobytes()                      # densities (237-248)
    b += np.ascontiguousarray(u, "<f4").tobytes()                        # velocities (250-261)
    if cfg.get("ext_magneto_hydro"):
        b += np.ascontiguousarray(q, "<f4").tobytes()                    # charges (263-274)
    if sections:  # FILE_LAYOUT.txt:42-57 (the reference's reader reads them, file.rs:154-182)
        b += struct.pack("<I", len(charges))
        for idx, qq in charges:
            b += struct.pack("<Qf", idx, qq)
        b += struct.pack("<I", len(magnets))
        for idx, m in magnets:
            b += struct.pack("<Q3f", idx, *m)
    return bytes(b)


# ---------------------------------------------------------------------------
# STL
# ---------------------------------------------------------------------------
def _rotm_around_v(v, r):
    """rotm_around_v (src/mesh.rs:57-66); matrix as dict of float32."""
    sr, cr = f32(_libm.sinf(float(r))), f32(_libm.cosf(float(r)))
    vx, vy, vz = (f32(a) for a in v)
    one = f32(1.0)
    return {
        "xx": vx * vx + (one - vx * vx) * cr, "xy": vx * vy * (one - cr) - vz * sr, "xz": vx * vz * (one - cr) + vy * sr,
        "yx": vx * vy * (one - cr) + vz * sr, "yy": vy * vy + (one - vy * vy) * cr, "yz": vy * vz * (one - cr) - vx * sr,
        "zx": vx * vz * (one - cr) - vy * sr, "zy": vy * vz * (one - cr) + vx * sr, "zz": vz * vz + (one - vz * vz) * cr,
    }


def _matmul(a, m):
    """F32_3_3 * F32_3_3 (src/mesh.rs:418-429)."""
    r = {}
    for i in "xyz":
        for j in "xyz":
            r[i + j] = a[i + "x"] * m["x" + j] + a[i + "y"] * m["y" + j] + a[i + "z"] * m["z" + j]
    return r


def rotation_deg(rx: float, ry: float, rz: float):
    """construct_rotation_matrix(rx*PI/180, ...) (src/mesh.rs:51-55, 236, 251)."""
    ang = [f32(a) * PI_F / f32(180.0) for a in (rx, ry, rz)]
    return _matmul(_matmul(_rotm_around_v((1, 0, 0), ang[0]), _rotm_around_v((0, 1, 0), ang[1])),
                   _rotm_around_v((0, 0, 1), ang[2]))


def _bounds(p0, p1, p2):
    """update_bounds (src/mesh.rs:94-109): min/max over triangles in order."""
    pmin, pmax = p0[0].copy(), p0[0].copy()
    lo = np.minimum(p2, np.minimum(p1, p0))
    hi = np.maximum(p2, np.maximum(p1, p0))
    pmin = np.minimum(pmin, lo.min(axis=0))
    pmax = np.maximum(pmax, hi.max(axis=0))
    return pmin.astype(f32), pmax.astype(f32)


def read_stl_raw(path, reposition: bool, box, center, rotation, size: float):
    """Mesh::read_stl_raw (src/mesh.rs:175-220).  Returns (p0, p1, p2, pmin,
    pmax, center) with p* of shape [ntri][3], float32."""
    data = open(path, "rb").read()
    nt = struct.unpack_from("<I", data, 80)[0]
    if not (nt > 0 and len(data) == 84 + 50 * nt):
        raise ValueError("corrupted or unsupported STL")
    rec = np.frombuffer(data, dtype=np.dtype([("n", "<f4", 3), ("v", "<f4", (3, 3)), ("a", "<u2")]), count=nt,
                        offset=84)
    v = rec["v"].astype(f32)  # [nt][vertex][xyz]
    R = rotation
    pts = []
    for k in range(3):  # rotation * F32_3 (src/mesh.rs:393-402)
        x, y, z = v[:, k, 0], v[:, k, 1], v[:, k, 2]
        pts.append(np.stack([R["xx"] * x + R["xy"] * y + R["xz"] * z, R["yx"] * x + R["yy"] * y + R["yz"] * z,
                             R["zx"] * x + R["zy"] * y + R["zz"] * z], axis=1).astype(f32))
    p0, p1, p2 = pts
    pmin, pmax = _bounds(p0, p1, p2)
    size = f32(size)
    if size == 0.0:  # get_scale_for_box_fit (src/mesh.rs:166-168)
        bx, by, bz = (f32(a) for a in box)
        scale = min(bx / (pmax[0] - pmin[0]), min(by / (pmax[1] - pmin[1]), bz / (pmax[2] - pmin[2])))
    elif size > 0.0:  # size / get_max_size (src/mesh.rs:161-163)
        scale = size / max(pmax[0] - pmin[0], max(pmax[1] - pmin[1], pmax[2] - pmin[2]))
    else:
        scale = -size
    scale = f32(scale)
    off = (f32(-0.5) * (pmin + pmax)).astype(f32) if reposition else np.zeros(3, f32)
    c = np.asarray(center, f32)
    p0, p1, p2 = ((c + scale * (off + p)).astype(f32) for p in (p0, p1, p2))
    pmin, pmax = _bounds(p0, p1, p2)
    return p0, p1, p2, pmin, pmax, c


def import_mesh(path, units_m: float, scale: float, ox, oy, oz, rx, ry, rz):
    """Lbm::import_mesh (src/mesh.rs:233-239): SI scale -> lattice units."""
    scale_lu = f32(scale) / f32(units_m)  # len_si_lu (src/lbm/units.rs:102-104)
    return read_stl_raw(path, False, (1.0, 1.0, 1.0), (ox, oy, oz), rotation_deg(rx, ry, rz), -abs(scale_lu))


def import_mesh_reposition(path, n_xyz, cx, cy, cz, rx, ry, rz, size):
    """Lbm::import_mesh_reposition (src/mesh.rs:248-253)."""
    return read_stl_raw(path, True, tuple(float(a) for a in n_xyz), (cx, cy, cz), rotation_deg(rx, ry, rz), size)
