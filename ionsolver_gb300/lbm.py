"""Python mirror of IonSolver's Rust API for the single-node timestep path.

Names follow the reference (``LbmConfig``, ``Lbm.initialize``, ``run``,
``do_time_step``, ``precompute_B``, ``import_mesh_reposition``,
``voxelise_mesh``, ``set_taylor_green``, file ``read``/``write``); every call
goes through the C ABI of include/ionsolver.h into libionsolver.so, which
owns the device memory and runs the sm_103a kernels.
"""
from __future__ import annotations

import ctypes as C
import enum
from dataclasses import dataclass, field
from typing import Sequence

import numpy as np

from . import _native as N


class VelocitySet(enum.IntEnum):  # src/lbm/types.rs:16-26
    D2Q9 = 0
    D3Q15 = 1
    D3Q19 = 2
    D3Q27 = 3


class RelaxationTime(enum.IntEnum):  # src/lbm/types.rs:55-61
    Srt = 0
    Trt = 1


class FloatType(enum.IntEnum):  # src/lbm/types.rs:75-83
    FP16S = 0
    FP16C = 1
    FP32 = 2


class FieldMode(enum.IntEnum):
    BITWISE = 0
    FAST = 1
    SURROGATE = 2


FIELDS = {"fi": 0, "rho": 1, "u": 2, "flags": 3, "F": 4, "e_stat": 5, "b_stat": 6, "e_dyn": 7, "b_dyn": 8,
          "fqi": 9, "ei": 10, "q": 11, "qu_lod": 12, "e_var": 13, "eti": 14, "et": 15}


@dataclass
class ModelType:
    """ModelType (src/mesh.rs:9-14): Solid, Magnet{magnetization}, Charged{charge}, ChargedECR{charge}."""
    kind: int
    values: tuple = (0.0, 0.0, 0.0)

    @staticmethod
    def Solid() -> "ModelType":
        return ModelType(0)

    @staticmethod
    def Magnet(magnetization: Sequence[float]) -> "ModelType":
        return ModelType(1, tuple(float(v) for v in magnetization))

    @staticmethod
    def Charged(charge: float) -> "ModelType":
        return ModelType(2, (float(charge), 0.0, 0.0))

    @staticmethod
    def ChargedECR(charge: float) -> "ModelType":
        return ModelType(3, (float(charge), 0.0, 0.0))


@dataclass
class Units:
    """Units (src/lbm/units.rs:14-197): lattice unit * factor = SI unit."""
    m: float = 1.0
    kg: float = 1.0
    s: float = 1.0
    a: float = 1.0
    k: float = 1.0
    prop: int = 0

    def _c(self) -> N.Units:
        return N.Units(self.m, self.kg, self.s, self.a, self.k, self.prop)

    def set(self, lbm_length, lbm_velocity, lbm_rho, lbm_charge, lbm_temp, si_length, si_velocity, si_rho,
            si_charge, si_temp) -> None:
        u = self._c()
        N.check(N.lib().ion_units_set(C.byref(u), lbm_length, lbm_velocity, lbm_rho, lbm_charge, lbm_temp, si_length,
                                      si_velocity, si_rho, si_charge, si_temp))
        self.m, self.kg, self.s, self.a, self.k = u.m, u.kg, u.s, u.a, u.k

    def _conv(self, what: int, v: float) -> float:
        out = C.c_float()
        N.check(N.lib().ion_units_si_to_lu(C.byref(self._c()), what, v, C.byref(out)))
        return out.value

    def nu_si_lu(self, nu: float) -> float:
        return self._conv(0, nu)

    def magnetization_si_lu(self, m: float) -> float:
        return self._conv(1, m)

    def charge_si_lu(self, q: float) -> float:
        return self._conv(2, q)

    def len_si_lu(self, length: float) -> float:
        return self._conv(3, length)


@dataclass
class LbmConfig:
    """LbmConfig (src/lbm/mod.rs:45-136) with LbmConfig::new() defaults.

    ``graphics_config`` is replaced by ``update_fields`` (its only effect on
    the timestep: UPDATE_FIELDS, src/lbm/domain.rs:856); ``field_mode`` is new.
    """
    velocity_set: int = VelocitySet.D2Q9
    relaxation_time: int = RelaxationTime.Srt
    float_type: int = FloatType.FP16S
    units: Units = field(default_factory=Units)
    n_x: int = 1
    n_y: int = 1
    n_z: int = 1
    d_x: int = 1
    d_y: int = 1
    d_z: int = 1
    nu: float = float(np.float32(1.0) / np.float32(6.0))
    f_x: float = 0.0
    f_y: float = 0.0
    f_z: float = 0.0
    ext_equilibrium_boudaries: bool = False
    ext_volume_force: bool = False
    ext_force_field: bool = False
    ext_magneto_hydro: bool = False
    ext_subgrid_ecr: bool = False
    mhd_lod_depth: int = 4
    ecr_freq: float = 0.0
    ecr_field_strength: float = 0.0
    update_fields: bool = True
    field_mode: int = FieldMode.BITWISE
    run_steps: int = 0

    def to_c(self) -> N.Config:
        c = N.Config()
        c.velocity_set, c.relaxation_time, c.float_type = int(self.velocity_set), int(self.relaxation_time), int(self.float_type)
        c.units = self.units._c()
        c.n_x, c.n_y, c.n_z, c.d_x, c.d_y, c.d_z = self.n_x, self.n_y, self.n_z, self.d_x, self.d_y, self.d_z
        c.nu, c.f_x, c.f_y, c.f_z = self.nu, self.f_x, self.f_y, self.f_z
        c.ext_equilibrium_boundaries = int(self.ext_equilibrium_boudaries)
        c.ext_volume_force = int(self.ext_volume_force)
        c.ext_force_field = int(self.ext_force_field)
        c.ext_magneto_hydro = int(self.ext_magneto_hydro)
        c.ext_subgrid_ecr = int(self.ext_subgrid_ecr)
        c.mhd_lod_depth = int(self.mhd_lod_depth)
        c.update_fields = int(self.update_fields)
        c.field_mode = int(self.field_mode)
        c.ecr_freq, c.ecr_field_strength, c.run_steps = self.ecr_freq, self.ecr_field_strength, int(self.run_steps)
        return c

    @staticmethod
    def from_c(c: N.Config) -> "LbmConfig":
        u = c.units
        return LbmConfig(c.velocity_set, c.relaxation_time, c.float_type, Units(u.m, u.kg, u.s, u.a, u.k, u.prop),
                         c.n_x, c.n_y, c.n_z, c.d_x, c.d_y, c.d_z, c.nu, c.f_x, c.f_y, c.f_z,
                         bool(c.ext_equilibrium_boundaries), bool(c.ext_volume_force), bool(c.ext_force_field),
                         bool(c.ext_magneto_hydro), bool(c.ext_subgrid_ecr), c.mhd_lod_depth, c.ecr_freq,
                         c.ecr_field_strength, bool(c.update_fields), c.field_mode, c.run_steps)

    def constants(self) -> dict:
        k = N.Constants()
        N.check(N.lib().ion_constants_from_config(C.byref(self.to_c()), C.byref(k)))
        return {name: getattr(k, name) for name, _ in N.Constants._fields_}


class Lbm:
    """Lbm (src/lbm/mod.rs:152-495) with its single LbmDomain on one GPU."""

    def __init__(self, config: LbmConfig | None = None, _handle: C.c_void_p | None = None):
        self._h = C.c_void_p()
        if _handle is not None:
            self._h = _handle
        else:
            N.check(N.lib().ion_lbm_create(C.byref(config.to_c()), C.byref(self._h)))
        c = N.Config()
        N.check(N.lib().ion_lbm_get_config(self._h, C.byref(c)))
        self.config = LbmConfig.from_c(c)

    # -- lifecycle ----------------------------------------------------------
    def close(self) -> None:
        if self._h:
            N.lib().ion_lbm_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    @property
    def n(self) -> int:
        return self.config.n_x * self.config.n_y * self.config.n_z

    # -- step loop ------------------------------------------------------------
    def initialize(self) -> None:
        N.check(N.lib().ion_lbm_initialize(self._h))

    def set_electron_background(self, rho_e0: float) -> None:
        """Finite-plasma start of the next initialize (no reference counterpart):
        electron gas at density rho_e0, charge lattice at Q + rho_e0."""
        N.check(N.lib().ion_lbm_set_electron_background(self._h, float(rho_e0)))

    def set_wait_limit(self, polls: int | None = None) -> None:
        """Polls before a device wait for staged data gives up (None: the default)."""
        N.check(N.lib().ion_lbm_set_wait_limit(self._h, N.ION_WAIT_LIMIT_DEFAULT if polls is None else int(polls)))

    def do_time_step(self) -> None:
        N.check(N.lib().ion_lbm_do_time_step(self._h))

    def run(self, steps: int) -> None:
        N.check(N.lib().ion_lbm_run(self._h, int(steps)))

    def get_time_step(self) -> int:
        t = C.c_uint64()
        N.check(N.lib().ion_lbm_get_time_step(self._h, C.byref(t)))
        return t.value

    def finish_queues(self, timeout_ms: int = -1) -> None:
        N.check(N.lib().ion_lbm_finish_queues(self._h, int(timeout_ms)))

    def update_fields(self) -> None:
        N.check(N.lib().ion_lbm_update_fields(self._h))

    # -- fields -----------------------------------------------------------------
    def field_info(self, name: str) -> tuple[int, int]:
        eb, cnt = C.c_size_t(), C.c_size_t()
        N.check(N.lib().ion_lbm_field_info(self._h, FIELDS[name], C.byref(eb), C.byref(cnt)))
        return eb.value, cnt.value

    def _dtype(self, name: str, eb: int):
        if name == "flags":
            return np.uint8
        return np.uint16 if eb == 2 else np.float32

    def read(self, name: str) -> np.ndarray:
        eb, cnt = self.field_info(name)
        out = np.empty(cnt, dtype=self._dtype(name, eb))
        if cnt:
            N.check(N.lib().ion_lbm_read_field(self._h, FIELDS[name], out.ctypes.data, out.nbytes))
        return out

    def write(self, name: str, values) -> None:
        eb, cnt = self.field_info(name)
        a = np.ascontiguousarray(np.asarray(values).reshape(-1), dtype=self._dtype(name, eb))
        if a.size > cnt:
            raise ValueError(f"{name}: {a.size} values for {cnt} elements")
        N.check(N.lib().ion_lbm_write_field(self._h, FIELDS[name], a.ctypes.data, a.nbytes))

    def device_ptr(self, name: str) -> tuple[int, int]:
        p, b = C.c_void_p(), C.c_size_t()
        N.check(N.lib().ion_lbm_field_device_ptr(self._h, FIELDS[name], C.byref(p), C.byref(b)))
        return p.value or 0, b.value

    # -- geometry ---------------------------------------------------------------
    def add_mesh(self, p0, p1, p2) -> int:
        a = [np.ascontiguousarray(np.asarray(p, np.float32).reshape(-1)) for p in (p0, p1, p2)]
        idx = C.c_uint32()
        N.check(N.lib().ion_lbm_add_mesh(self._h, a[0].ctypes.data, a[1].ctypes.data, a[2].ctypes.data,
                                         a[0].size // 3, C.byref(idx)))
        return idx.value

    def import_mesh(self, path: str, scale: float, ox, oy, oz, rx, ry, rz) -> int:
        idx = C.c_uint32()
        N.check(N.lib().ion_lbm_import_mesh(self._h, str(path).encode(), scale, ox, oy, oz, rx, ry, rz, C.byref(idx)))
        return idx.value

    def import_mesh_reposition(self, path: str, cx, cy, cz, rx, ry, rz, size) -> int:
        idx = C.c_uint32()
        N.check(N.lib().ion_lbm_import_mesh_reposition(self._h, str(path).encode(), cx, cy, cz, rx, ry, rz, size,
                                                       C.byref(idx)))
        return idx.value

    def mesh_translate(self, index: int, d: Sequence[float]) -> None:
        N.check(N.lib().ion_lbm_mesh_translate(self._h, index, float(d[0]), float(d[1]), float(d[2])))

    def mesh_triangles(self, index: int) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        """The mesh's vertex arrays p0, p1, p2, each [ntri][3] float32."""
        nt = C.c_uint32()
        N.check(N.lib().ion_lbm_mesh_triangles(self._h, index, None, None, None, 0, C.byref(nt)))
        p = [np.empty((nt.value, 3), np.float32) for _ in range(3)]
        N.check(N.lib().ion_lbm_mesh_triangles(self._h, index, p[0].ctypes.data, p[1].ctypes.data, p[2].ctypes.data,
                                               nt.value, C.byref(nt)))
        return p[0], p[1], p[2]

    def mesh_bounds(self, index: int) -> dict:
        out = (C.c_float * 9)()
        N.check(N.lib().ion_lbm_mesh_bounds(self._h, index, out))
        v = list(out)
        return {"p_min": v[0:3], "p_max": v[3:6], "center": v[6:9]}

    def voxelise_mesh(self, index: int, ctype: ModelType) -> None:
        v = tuple(ctype.values) + (0.0,) * (3 - len(ctype.values))
        N.check(N.lib().ion_lbm_voxelise_mesh(self._h, index, ctype.kind, v[0], v[1], v[2]))

    def precompute_B(self) -> None:
        N.check(N.lib().ion_lbm_precompute_b(self._h))

    def precompute_E(self) -> None:
        N.check(N.lib().ion_lbm_precompute_e(self._h))

    def precompute_E_ECR(self) -> None:
        """Lbm::precompute_E_ECR (src/lbm/mod.rs:319-331): the charges' field into E_var."""
        N.check(N.lib().ion_lbm_precompute_e_ecr(self._h))

    # -- diagnostics ---------------------------------------------------------------
    def mass_charge(self) -> tuple[float, float]:
        m, q = C.c_double(), C.c_double()
        N.check(N.lib().ion_lbm_mass_charge(self._h, C.byref(m), C.byref(q)))
        return m.value, q.value

    # -- setup helpers (src/setup.rs:458-598) ----------------------------------------
    def set_taylor_green(self, periodicity: int = 1, amplitude: float = 0.25, reference_density: bool = True) -> None:
        """Taylor-Green vortices (src/setup.rs:458-543), computed in float32.

        ``reference_density`` reproduces the reference's density expression
        (setup.rs:528-530, whose parentheses make it 2 - A^2 3/4 cos(..) + ...);
        pass False for a uniform density of 1."""
        ux, uy, uz, rho = taylor_green_fields(self.config.n_x, self.config.n_y, self.config.n_z, periodicity,
                                              amplitude, reference_density)
        self.write("u", np.concatenate([ux, uy, uz]))
        self.write("rho", rho)

    def setup_velocity_field(self, velocity: Sequence[float], density: float) -> None:
        """src/setup.rs:547-598"""
        n = self.n
        self.write("u", np.concatenate([np.full(n, velocity[i], np.float32) for i in range(3)]))
        self.write("rho", np.full(n, density, np.float32))

    # -- files (src/file.rs) ------------------------------------------------------------
    def write_file(self, path: str) -> None:
        N.check(N.lib().ion_lbm_save(self._h, str(path).encode()))

    @staticmethod
    def read_file(path: str, config: LbmConfig | None = None) -> "Lbm":
        c = (config or LbmConfig()).to_c()
        h = C.c_void_p()
        N.check(N.lib().ion_lbm_load(str(path).encode(), C.byref(c), C.byref(h)))
        return Lbm(_handle=h)

    def checkpoint(self, path: str) -> None:
        """Full state (the .ion image + every buffer the next step reads + the time step)."""
        N.check(N.lib().ion_lbm_checkpoint(self._h, str(path).encode()))

    @staticmethod
    def restore(path: str, config: LbmConfig | None = None) -> "Lbm":
        """A handle that continues a checkpoint bit for bit (no initialize() needed)."""
        c = (config or LbmConfig()).to_c()
        h = C.c_void_p()
        N.check(N.lib().ion_lbm_restore(str(path).encode(), C.byref(c), C.byref(h)))
        return Lbm(_handle=h)

    # -- learned far field ----------------------------------------------------------------
    def surrogate_train(self, samples: int = 2000, epochs: int = 20, batch: int = 8, lr: float = 1e-3,
                        seed: int = 5) -> float:
        err = C.c_float()
        N.check(N.lib().ion_lbm_surrogate_train(self._h, samples, epochs, batch, lr, seed, C.byref(err)))
        return err.value

    def surrogate_info(self) -> dict:
        r32, r16, n = C.c_float(), C.c_float(), C.c_uint32()
        loss = (C.c_float * 1024)()
        N.check(N.lib().ion_lbm_surrogate_info(self._h, C.byref(r32), C.byref(r16), loss, 1024, C.byref(n)))
        return {"rel_err_fp32": r32.value, "rel_err_bf16": r16.value, "loss": list(loss)[: n.value]}

    def surrogate_save(self, path: str) -> None:
        N.check(N.lib().ion_lbm_surrogate_save(self._h, str(path).encode()))

    def surrogate_load(self, path: str) -> None:
        N.check(N.lib().ion_lbm_surrogate_load(self._h, str(path).encode()))

    def surrogate_configure(self, tolerance: float = 1e-2, check_cells: int = 1024) -> None:
        N.check(N.lib().ion_lbm_surrogate_configure(self._h, tolerance, check_cells))

    def surrogate_stats(self) -> dict:
        c, f, nf, e, b = C.c_uint64(), C.c_uint64(), C.c_uint64(), C.c_float(), C.c_float()
        N.check(N.lib().ion_lbm_surrogate_stats(self._h, C.byref(c), C.byref(f), C.byref(nf), C.byref(e), C.byref(b)))
        return {"checks": c.value, "fallbacks": f.value, "nonfinite": nf.value, "err_e": e.value, "err_b": b.value}

    def surrogate_targets(self, x: np.ndarray) -> tuple[np.ndarray, float, float]:
        """Exact far-field targets of source snapshots x [S][4][V]; returns (t [S][168][V], yE, yB)."""
        x = np.ascontiguousarray(x, np.float32)
        S = x.shape[0]
        t = np.empty((S, self.SURROGATE_OUT, x.shape[-1]), np.float32)
        ye, yb = C.c_float(), C.c_float()
        N.check(N.lib().ion_lbm_surrogate_targets(self._h, x.ctypes.data, t.ctypes.data, S, C.byref(ye), C.byref(yb)))
        return t, ye.value, yb.value

    def surrogate_weights(self, values=None) -> np.ndarray:
        n = self._surrogate_count()
        out = np.empty(n, np.float32)
        src = None if values is None else np.ascontiguousarray(values, np.float32)
        N.check(N.lib().ion_lbm_surrogate_weights(self._h, out.ctypes.data, None if src is None else src.ctypes.data, n))
        return out

    SURROGATE_OUT = 168  # network output channels: 27 nodes x 6 components, padded to 168
    SURROGATE_NEAR_RADIUS = 1  # bins within this Chebyshev distance of a cell's bin are summed exactly

    def _surrogate_count(self) -> int:
        # layer table of the network (4->32, 8 x 32->32, 32->168; 3^3 kernels)
        return (4 * 32 + 8 * 32 * 32 + 32 * self.SURROGATE_OUT) * 27

    def surrogate_grad(self, x: np.ndarray, t: np.ndarray) -> tuple[float, np.ndarray]:
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        g = np.empty(self._surrogate_count(), np.float32)
        loss = C.c_float()
        N.check(N.lib().ion_lbm_surrogate_grad(self._h, x.ctypes.data, t.ctypes.data, x.shape[0], C.byref(loss),
                                               g.ctypes.data))
        return loss.value, g

    def surrogate_forward(self, x: np.ndarray, bf16: bool = False) -> np.ndarray:
        x = np.ascontiguousarray(x, np.float32).reshape(-1)
        V = x.size // 4
        y = np.empty(self.SURROGATE_OUT * V, np.float32)
        N.check(N.lib().ion_lbm_surrogate_forward(self._h, x.ctypes.data, y.ctypes.data, int(bf16)))
        return y

    def set_field_mode(self, mode: int) -> None:
        N.check(N.lib().ion_lbm_set_field_mode(self._h, int(mode)))
        self.config.field_mode = int(mode)

    # -- timing ---------------------------------------------------------------------------
    def record_event(self, slot: int) -> None:
        N.check(N.lib().ion_lbm_record_event(self._h, slot))

    def elapsed_ms(self, a: int, b: int) -> float:
        ms = C.c_float()
        N.check(N.lib().ion_lbm_event_elapsed(self._h, a, b, C.byref(ms)))
        return ms.value

    def set_kernel_timing(self, enable: bool) -> None:
        N.check(N.lib().ion_lbm_set_kernel_timing(self._h, int(enable)))

    def kernel_time(self, kernel: int) -> tuple[float, int]:
        ms, n = C.c_double(), C.c_uint64()
        N.check(N.lib().ion_lbm_kernel_time(self._h, kernel, C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def reset_kernel_time(self) -> None:
        N.check(N.lib().ion_lbm_reset_kernel_time(self._h))


def write_config(path: str, cfg: LbmConfig) -> None:
    """LbmConfig as JSON in the reference's serde layout (file::write_config, src/file.rs:324-334)."""
    N.check(N.lib().ion_config_write_json(str(path).encode(), C.byref(cfg.to_c())))


def read_config(path: str) -> LbmConfig:
    """LbmConfig from the reference's JSON (file::read_config, src/file.rs:310-322)."""
    c = N.Config()
    N.check(N.lib().ion_config_read_json(str(path).encode(), C.byref(c)))
    return LbmConfig.from_c(c)


class Batch:
    """Independent D3Q19 domains of uneven size advanced together, one
    persistent launch per timestep (ion_batch_* of include/ionsolver.h)."""

    def __init__(self, domains: Sequence[Lbm]):
        self.domains = list(domains)
        arr = (C.c_void_p * len(self.domains))(*[d.handle.value for d in self.domains])
        self._h = C.c_void_p()
        N.check(N.lib().ion_batch_create(arr, len(self.domains), C.byref(self._h)))

    def run(self, steps: int) -> None:
        N.check(N.lib().ion_batch_run(self._h, int(steps)))

    def set_wait_limits(self, barrier_polls: int | None = None, tile_polls: int | None = None) -> None:
        """Poll limits of the batch step's grid barriers and staged-tile waits (None: the defaults)."""
        N.check(N.lib().ion_batch_set_wait_limits(
            self._h, N.ION_BARRIER_LIMIT_DEFAULT if barrier_polls is None else int(barrier_polls),
            N.ION_WAIT_LIMIT_DEFAULT if tile_polls is None else int(tile_polls)))

    def finish(self, timeout_ms: int = -1) -> None:
        N.check(N.lib().ion_batch_finish(self._h, int(timeout_ms)))

    def tuning(self) -> list[tuple[int, int, float]]:
        out, i = [], 0
        while True:
            b, g, ms = C.c_uint32(), C.c_uint32(), C.c_float()
            if N.lib().ion_batch_tuning(self._h, i, C.byref(b), C.byref(g), C.byref(ms)) != 0:
                return out
            out.append((b.value, g.value, ms.value))
            i += 1

    def chosen(self) -> tuple[int, int]:
        b, g = C.c_uint32(), C.c_uint32()
        N.check(N.lib().ion_batch_tuning(self._h, 0xFFFFFFFF, C.byref(b), C.byref(g), None))
        return b.value, g.value

    def record_event(self, slot: int) -> None:
        N.check(N.lib().ion_batch_record_event(self._h, slot))

    def elapsed_ms(self, a: int, b: int) -> float:
        ms = C.c_float()
        N.check(N.lib().ion_batch_event_elapsed(self._h, a, b, C.byref(ms)))
        return ms.value

    def close(self) -> None:
        if self._h:
            N.lib().ion_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def taylor_green_fields(nx: int, ny: int, nz: int, periodicity: int = 1, amplitude: float = 0.25,
                        reference_density: bool = True):
    """Velocity (3 arrays) and density of src/setup.rs:458-543 in float32 (cell order n = x + (y + z ny) nx)."""
    f32 = np.float32
    A = f32(amplitude)
    a, b, c = f32(nx) / f32(periodicity), f32(ny) / f32(periodicity), f32(nz) / f32(periodicity)
    z, y, x = np.meshgrid(np.arange(nz, dtype=f32), np.arange(ny, dtype=f32), np.arange(nx, dtype=f32), indexing="ij")
    fx = x + f32(0.5) - f32(0.5) * f32(nx)
    fy = y + f32(0.5) - f32(0.5) * f32(ny)
    fz = z + f32(0.5) - f32(0.5) * f32(nz)
    tp = f32(2.0) * f32(np.pi)
    ux = A * np.cos(tp * fx / a) * np.sin(tp * fy / b) * np.sin(tp * fz / c)
    uy = -A * np.sin(tp * fx / a) * np.cos(tp * fy / b) * np.sin(tp * fz / c)
    uz = A * np.sin(tp * fx / a) * np.sin(tp * fy / b) * np.cos(tp * fz / c)
    if reference_density:
        fp = f32(4.0) * f32(np.pi)
        rho = f32(1.0) - (A * A) * f32(3.0) / f32(4.0) * np.cos(fp * fx / a) + np.cos(fp * fy / b)
    else:
        rho = np.ones_like(ux)
    return (ux.astype(f32).ravel(), uy.astype(f32).ravel(), uz.astype(f32).ravel(), rho.astype(f32).ravel())


def codec_roundtrip(float_type: int, values: np.ndarray, raw: np.ndarray):
    """Runs the device FP16S/FP16C codecs: (encode(values), decode(encode(values)), decode(raw))."""
    v = np.ascontiguousarray(values, np.float32)
    r = np.ascontiguousarray(raw, np.uint16)
    assert v.size == r.size
    enc = np.empty(v.size, np.uint16)
    dec = np.empty(v.size, np.float32)
    rdec = np.empty(v.size, np.float32)
    N.check(N.lib().ion_codec_roundtrip(int(float_type), v.ctypes.data, enc.ctypes.data, dec.ctypes.data,
                                        r.ctypes.data, rdec.ctypes.data, v.size))
    return enc, dec, rdec


def kernel_launch_count() -> int:
    return int(N.lib().ion_kernel_launch_count())
