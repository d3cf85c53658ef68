"""Small cases whose reference outputs are stored as golden fixtures.

Each builder returns (case, steps, action) with ``action`` one of "run"
(initialize + steps) or "setup" (voxelise + static fields only)."""
import numpy as np

from ionsolver_gb300 import workloads as W


def plain(ft, rt, vs=2, shape=(12, 10, 8)):
    case = W.taylor_green(shape=shape, amplitude=0.05, float_type=ft, relaxation_time=rt)
    case["config"]["velocity_set"] = vs
    if vs != 2:
        rng = np.random.default_rng(5)
        n = shape[0] * shape[1] * shape[2]
        uz = rng.normal(0, 0.02 if shape[2] > 1 else 0, n)
        case["fields"]["u"] = np.concatenate([rng.normal(0, 0.02, 2 * n), uz]).astype(np.float32)
    return case


def boundaries(rt):
    nx, ny, nz = 12, 10, 8
    n = nx * ny * nz
    rng = np.random.default_rng(7)
    case = W.taylor_green(shape=(nx, ny, nz), amplitude=0.03, relaxation_time=rt)
    flags = W.shell_flags(nx, ny, nz)
    flags.reshape(nz, ny, nx)[:, :, 0] = 0x02
    flags.reshape(nz, ny, nx)[3:5, 3:6, 4:7] = 0x01
    case["fields"].update(flags=flags, F=rng.normal(0, 1e-5, 3 * n).astype(np.float32),
                          rho=(1.0 + rng.normal(0, 1e-3, n)).astype(np.float32))
    case["config"].update(ext_equilibrium_boundaries=1, ext_volume_force=1, ext_force_field=1, f_x=1e-6, f_y=-2e-6,
                          f_z=5e-7)
    return case


def mhd(ft, n, depth):
    return W.mhd_box(n=n, float_type=ft, depth=depth, magnet_r=n / 4, magnet_t=n / 5)


def geometry():
    case = W.mhd_box(n=16, depth=2, magnet_r=5.0, magnet_t=4.0)
    ring = W.annulus((8.0, 8.0, 11.0), 6.0, 3.0, 2.5, axis=0)
    case["meshes"].append((ring[0], ring[1], ring[2], "charged", (3e-9, 0, 0)))
    return case


def plasma(ft, n, depth):
    """The finite-plasma start (electron background, plasma units)."""
    return W.mhd_plasma(n=n, float_type=ft, depth=depth, magnet_r=n / 4, magnet_t=n / 5)


def ecr(ft, rt):
    return W.ecr_box(n=16, float_type=ft, depth=2, relaxation_time=rt)


CASES = {
    "tgv_fp32_srt": (lambda: plain(2, 0), 20, "run"),
    "tgv_fp16s_trt": (lambda: plain(0, 1), 20, "run"),
    "tgv_fp16c_srt": (lambda: plain(1, 0), 20, "run"),
    "d3q15_fp32": (lambda: plain(2, 0, 1, (10, 8, 6)), 20, "run"),
    "d2q9_fp32": (lambda: plain(2, 0, 0, (20, 16, 1)), 20, "run"),
    "boundaries_trt": (lambda: boundaries(1), 20, "run"),
    "mhd16_fp32_d2": (lambda: mhd(2, 16, 2), 6, "run"),
    "mhd16_fp16s_d2": (lambda: mhd(0, 16, 2), 6, "run"),
    "mhd16_fp32_d4": (lambda: mhd(2, 16, 4), 4, "run"),
    "plasma16_fp32_d2": (lambda: plasma(2, 16, 2), 30, "run"),
    "plasma16_fp16c_d2": (lambda: plasma(1, 16, 2), 30, "run"),
    "geometry": (geometry, 0, "setup"),
    "ecr16_fp32_srt": (lambda: ecr(2, 0), 4, "run"),
    "ecr16_fp16s_trt": (lambda: ecr(0, 1), 3, "run"),
}
