"""Synthetic inputs of the benchmark configurations (all seeded, no dataset).

* ``taylor_green``: plain D3Q19 SRT, periodic box, Taylor-Green vortex
  (u0 = 0.05, rho = 1), tau = 0.6 (nu = 1/30).
* ``mhd_box``: D3Q19 fluid + D3Q7 charge lattice, one-cell solid shell,
  charge i.i.d. U[-1e-3, 1e-3] (PCG64 seed 1), velocity N(0, 1e-3^2) per
  component (seed 2), rho = 1, an axially magnetised disk magnet centred on
  the z = 1 face, Units{m=1, kg=1, s=1, a=1e-6}, LOD depth 4.

* ``mhd_plasma``: ``mhd_box`` with the finite-plasma start (a background
  electron density; units in which the electron response per step is small).

A case is a dict ``{"config": {...C field names...}, "fields": {...},
"meshes": [(p0, p1, p2, model, values)], "precompute_b": bool}`` (optionally
``"electron_background": rho_e0``) that
``apply_case`` writes into any object with ``write``/``add_mesh``/
``voxelise_mesh``/``precompute_B`` (the GPU ``Lbm``; tests adapt the CPU
oracle to the same calls).
"""
from __future__ import annotations

import numpy as np

from .lbm import taylor_green_fields
from .meshes import annulus, cylinder

NU_1_30 = float(np.float32(1.0) / np.float32(30.0))  # tau = 0.6
MAGNETIZATION_SI = 8.0e10  # A/m: gives max |B_stat| of a few 1e-2 lattice units with a = 1e-6

# The finite-plasma start.  The reference's electron gas starts at density 0
# (sim_kernels.cl:823) and its velocity j/rho_e turns 0/0 within a few steps;
# from then on every MHD field is NaN.  With a background electron density
# rho_e0 the state stays finite if the units keep the electron response per
# step small: electron acceleration per unit net charge KE/(2|KKGE|) ~ 3e-3,
# cyclotron rotation B/(2|KKGE|) ~ 1e-2 per step and plasma frequency
# sqrt(4 pi KE rho_e0/|KKGE|) ~ 0.03 per step.  Units: cells of 6.46 cm,
# steps of 1 ns, gas 1e-3 kg/m^3 (kg = 1e-3 m^3), current unit 1 A; every
# intermediate of the float32 unit conversion stays a normal float.
PLASMA_UNITS = dict(m=0.0646, kg=2.7e-7, s=1e-9, a=1.0, k=1.0, prop=0)
PLASMA_MAGNETIZATION_SI = 300.0  # A/m: max |B_stat| ~ 1e-2 |2 KKGE| in these units
PLASMA_RHO_E0 = 0.01             # background electron density (lattice charge units)


def taylor_green(n: int = 64, amplitude: float = 0.05, float_type: int = 2, relaxation_time: int = 0,
                 shape: tuple | None = None) -> dict:
    nx, ny, nz = shape or (n, n, n)
    ux, uy, uz, rho = taylor_green_fields(nx, ny, nz, 1, amplitude, reference_density=False)
    return {
        "config": dict(velocity_set=2, relaxation_time=relaxation_time, float_type=float_type, n_x=nx, n_y=ny,
                       n_z=nz, nu=NU_1_30, update_fields=1),
        "fields": {"u": np.concatenate([ux, uy, uz]), "rho": rho},
        "meshes": [],
        "precompute_b": False,
    }


def shell_flags(nx: int, ny: int, nz: int) -> np.ndarray:
    f = np.zeros((nz, ny, nx), np.uint8)
    f[0], f[-1] = 1, 1
    f[:, 0], f[:, -1] = 1, 1
    f[:, :, 0], f[:, :, -1] = 1, 1
    return f.reshape(-1)


def mhd_box(n: int = 128, float_type: int = 2, depth: int = 4, field_mode: int = 0, magnet_r: float = 16.0,
            magnet_t: float = 8.0, magnet: bool = True, shape: tuple | None = None, seed_q: int = 1,
            seed_u: int = 2, update_fields: int = 1, magnetization: float = MAGNETIZATION_SI,
            rings: bool = False) -> dict:
    nx, ny, nz = shape or (n, n, n)
    N = nx * ny * nz
    q = np.random.Generator(np.random.PCG64(seed_q)).uniform(-1e-3, 1e-3, N).astype(np.float32)
    u = np.random.Generator(np.random.PCG64(seed_u)).normal(0.0, 1e-3, 3 * N).astype(np.float32)
    meshes = []
    if magnet and not rings:
        p0, p1, p2 = cylinder((0.5 * nx, 0.5 * ny, 1.0 + 0.5 * magnet_t), magnet_r, magnet_t, axis=2)
        meshes.append((p0, p1, p2, "magnet", (0.0, 0.0, magnetization)))
    if rings:  # two coaxial ring magnets, R_out 48, R_in 32, t 12, 128 apart (scaled to the box)
        s = nx / 384.0
        for zc in (0.5 * nz - 64.0 * s, 0.5 * nz + 64.0 * s):
            p0, p1, p2 = annulus((0.5 * nx, 0.5 * ny, zc), 48.0 * s, 32.0 * s, 12.0 * s, axis=2)
            meshes.append((p0, p1, p2, "magnet", (0.0, 0.0, magnetization)))
    return {
        "config": dict(velocity_set=2, relaxation_time=0, float_type=float_type, n_x=nx, n_y=ny, n_z=nz,
                       nu=NU_1_30, ext_volume_force=1, ext_magneto_hydro=1, mhd_lod_depth=depth,
                       update_fields=update_fields, field_mode=field_mode,
                       units=dict(m=1.0, kg=1.0, s=1.0, a=1e-6, k=1.0, prop=0)),
        "fields": {"flags": shell_flags(nx, ny, nz), "q": q, "u": u, "rho": np.ones(N, np.float32)},
        "meshes": meshes,
        "precompute_b": bool(meshes),
    }


def to_plasma(case: dict, rho_e0: float = PLASMA_RHO_E0) -> dict:
    """A case of ``mhd_box`` switched to the finite-plasma start: PLASMA_UNITS,
    every magnet at PLASMA_MAGNETIZATION_SI (same direction), the electron gas
    starting at rho_e0.  Fields, geometry and seeds are unchanged."""
    case["config"]["units"] = dict(PLASMA_UNITS)
    meshes = []
    for p0, p1, p2, model, vals in case["meshes"]:
        if model == "magnet":
            m = np.asarray(vals, np.float64)
            vals = tuple(float(v) for v in m / np.linalg.norm(m) * PLASMA_MAGNETIZATION_SI)
        meshes.append((p0, p1, p2, model, vals))
    case["meshes"] = meshes
    case["electron_background"] = float(rho_e0)
    return case


def mhd_plasma(n: int = 128, float_type: int = 2, depth: int = 4, field_mode: int = 0, magnet_r: float | None = None,
               magnet_t: float | None = None, shape: tuple | None = None, update_fields: int = 1,
               rho_e0: float = PLASMA_RHO_E0, rings: bool = False) -> dict:
    """``mhd_box`` with the finite-plasma start: the same seeded charge and
    velocity fields, wall shell and disk magnet (radius n/8, thickness n/16
    unless given: 16 and 8 cells at 128^3; or the two rings), in PLASMA_UNITS
    with the magnets at PLASMA_MAGNETIZATION_SI and the electron gas starting
    at rho_e0."""
    nx = (shape or (n, n, n))[0]
    case = mhd_box(n=n, float_type=float_type, depth=depth, field_mode=field_mode,
                   magnet_r=magnet_r if magnet_r is not None else nx / 8.0,
                   magnet_t=magnet_t if magnet_t is not None else nx / 16.0, shape=shape,
                   update_fields=update_fields, rings=rings)
    return to_plasma(case, rho_e0)


def ecr_box(n: int = 32, float_type: int = 2, depth: int = 2, relaxation_time: int = 0, seed_t: int = 9) -> dict:
    """The SUBGRID_ECR extension on an MHD box: a disk magnet, two ChargedECR plates
    (+/- 1e-13 C per cell, 1/4 and 3/4 of the box in y) for the oscillating field
    E_var, an initial electron temperature around 1 (seed 9), 2.45 GHz."""
    case = mhd_box(n=n, float_type=float_type, depth=depth, magnet_r=n / 4, magnet_t=n / 8)
    case["config"].update(ext_subgrid_ecr=1, ecr_freq=2.45e9, relaxation_time=relaxation_time)
    N = n ** 3
    case["fields"]["et"] = (1.0 + np.random.Generator(np.random.PCG64(seed_t)).normal(0.0, 0.05, N)).astype(np.float32)
    plates = []
    for yc, q in ((0.25 * n, 1e-13), (0.75 * n, -1e-13)):
        p0, p1, p2 = cylinder((0.5 * n, yc, 0.5 * n), n / 5, 2.0, axis=1)
        case["meshes"].append((p0, p1, p2, "charged_ecr", (q, 0.0, 0.0)))
        plates.append((p0, p1, p2, "solid", (0.0, 0.0, 0.0)))
    case["precompute_e_ecr"] = True
    # after the precomputes the magnet and the plates become solid: the reference's ECR
    # divides by |B|, which is 0 inside them (static_b_from_mesh skips such cells)
    case["meshes_after"] = [case["meshes"][0][:3] + ("solid", (0.0, 0.0, 0.0))] + plates
    return case


def batch_domains(count: int = 96, float_type: int = 2, field_mode: int = 1, seed_sizes: int = 3,
                  seed_magnets: int = 4, plasma: bool = False) -> list[dict]:
    """Uneven MHD domains: cube edges uniform from {32,48,64,80,96} (PCG64
    seed 3); a disk magnet per domain with radius uniform in {4..12} cells,
    thickness r/2, at a random centre that keeps it inside the walls (seed 4);
    charge and velocity as in mhd_box with per-domain seeds 100+i / 200+i."""
    edges = np.random.Generator(np.random.PCG64(seed_sizes)).choice([32, 48, 64, 80, 96], size=count)
    rm = np.random.Generator(np.random.PCG64(seed_magnets))
    cases = []
    for i, n in enumerate(int(e) for e in edges):
        r = float(rm.integers(4, 13))
        t = max(2.0, r / 2.0)
        lo_xy, hi_xy = r + 2.0, n - r - 2.0
        lo_z, hi_z = t / 2 + 2.0, n - t / 2 - 2.0
        c = (float(rm.uniform(lo_xy, hi_xy)), float(rm.uniform(lo_xy, hi_xy)), float(rm.uniform(lo_z, hi_z)))
        case = mhd_box(n=n, float_type=float_type, field_mode=field_mode, magnet=False, seed_q=100 + i,
                       seed_u=200 + i)
        p0, p1, p2 = cylinder(c, r, t, axis=2)
        case["meshes"] = [(p0, p1, p2, "magnet", (0.0, 0.0, MAGNETIZATION_SI))]
        case["precompute_b"] = True
        cases.append(to_plasma(case) if plasma else case)
    return cases


MODEL_IDS = {"solid": 0, "magnet": 1, "charged": 2, "charged_ecr": 3}


def lbm_config(case: dict):
    """The case's config as an LbmConfig."""
    from .lbm import LbmConfig, Units
    c = dict(case["config"])
    units = c.pop("units", None)
    if "ext_equilibrium_boundaries" in c:
        c["ext_equilibrium_boudaries"] = c.pop("ext_equilibrium_boundaries")
    cfg = LbmConfig(**c)
    if units:
        cfg.units = Units(**units)
    return cfg


def apply_case(lbm, case: dict) -> None:
    """Writes the case's fields and magnets into a GPU Lbm (order: fields, voxelise, precompute_B)."""
    from .lbm import ModelType
    for name, arr in case["fields"].items():
        lbm.write(name, arr)
    if case.get("electron_background"):
        lbm.set_electron_background(case["electron_background"])
    for p0, p1, p2, model, vals in case["meshes"]:
        idx = lbm.add_mesh(p0, p1, p2)
        lbm.voxelise_mesh(idx, ModelType(MODEL_IDS[model], tuple(vals)))
    if case["precompute_b"]:
        lbm.precompute_B()
    if case.get("precompute_e_ecr"):
        lbm.precompute_E_ECR()
    for p0, p1, p2, model, vals in case.get("meshes_after", []):
        idx = lbm.add_mesh(p0, p1, p2)
        lbm.voxelise_mesh(idx, ModelType(MODEL_IDS[model], tuple(vals)))
