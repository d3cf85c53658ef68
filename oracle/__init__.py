"""CPU oracles for IonSolver's timestep -- TEST INFRASTRUCTURE, not product code.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline /
reference arm use this package.  It offers three interchangeable back ends
behind one class, :class:`OracleLbm`:

* ``"f32"`` -- the C restatement (``oracle/ion_oracle.c``) in float, with the
  reference's FP16S/FP16C codecs: the bit-level parity target;
* ``"f64"`` -- the same restatement in double: the accuracy oracle;
* ``"ref"`` -- the reference's own kernel text (IonSolver
  ``src/kernels/sim_kernels.cl``) compiled as C++ (``oracle/build.py``), used
  to pin the restatement.  Available where the reference checkout (or its
  generated translation unit) is present.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from . import build as _build

# ---------------------------------------------------------------------------
# C structs of include/ionsolver.h, restated for ctypes
# ---------------------------------------------------------------------------


class IonUnits(C.Structure):
    _fields_ = [("m", C.c_float), ("kg", C.c_float), ("s", C.c_float), ("a", C.c_float), ("k", C.c_float),
                ("prop", C.c_int32)]


class IonConfig(C.Structure):
    _fields_ = [
        ("velocity_set", C.c_int32), ("relaxation_time", C.c_int32), ("float_type", C.c_int32),
        ("units", IonUnits),
        ("n_x", C.c_uint32), ("n_y", C.c_uint32), ("n_z", C.c_uint32),
        ("d_x", C.c_uint32), ("d_y", C.c_uint32), ("d_z", C.c_uint32),
        ("nu", C.c_float), ("f_x", C.c_float), ("f_y", C.c_float), ("f_z", C.c_float),
        ("ext_equilibrium_boundaries", C.c_uint8), ("ext_volume_force", C.c_uint8),
        ("ext_force_field", C.c_uint8), ("ext_magneto_hydro", C.c_uint8), ("ext_subgrid_ecr", C.c_uint8),
        ("mhd_lod_depth", C.c_uint8), ("update_fields", C.c_uint8), ("field_mode", C.c_uint8),
        ("ecr_freq", C.c_float), ("ecr_field_strength", C.c_float),
        ("run_steps", C.c_uint64),
    ]


class IonConstants(C.Structure):
    _fields_ = [(n, C.c_float) for n in ("w", "ke", "kmu", "kmu0", "kkge", "kimg", "kvev", "kme", "wq",
                                          "epsilon_0", "mu_0", "kkbme", "keabs")]


FIELDS = {"fi": 0, "rho": 1, "u": 2, "flags": 3, "F": 4, "e_stat": 5, "b_stat": 6, "e_dyn": 7, "b_dyn": 8,
          "fqi": 9, "ei": 10, "q": 11, "qu_lod": 12, "e_var": 13, "eti": 14, "et": 15}
MODEL = {"solid": 0, "magnet": 1, "charged": 2, "charged_ecr": 3}


def make_config(**kw) -> IonConfig:
    """LbmConfig::new() defaults (IonSolver src/lbm/mod.rs:105-135) with overrides."""
    c = IonConfig()
    c.velocity_set, c.relaxation_time, c.float_type = 0, 0, 0
    c.units = IonUnits(1.0, 1.0, 1.0, 1.0, 1.0, 0)
    c.n_x = c.n_y = c.n_z = 1
    c.d_x = c.d_y = c.d_z = 1
    c.nu = float(np.float32(1.0) / np.float32(6.0))
    c.mhd_lod_depth = 4
    c.update_fields = 1  # graphics_active defaults to true (graphics.rs:160) -> UPDATE_FIELDS
    for k, v in kw.items():
        if k == "units":
            if isinstance(v, dict):
                u = c.units
                for kk, vv in v.items():
                    setattr(u, kk, vv)
                c.units = u
            else:
                c.units = v
        else:
            setattr(c, k, v)
    return c


def config_dict(c: IonConfig) -> dict:
    return {name: getattr(c, name) for name, _ in IonConfig._fields_ if name != "units"}


# ---------------------------------------------------------------------------
# libraries
# ---------------------------------------------------------------------------
_LIBS: dict[str, C.CDLL] = {}


def _bind(lib: C.CDLL) -> C.CDLL:
    lib.orc_create.restype = C.c_void_p
    lib.orc_create.argtypes = [C.POINTER(IonConfig), C.POINTER(IonConstants)]
    lib.orc_destroy.argtypes = [C.c_void_p]
    lib.orc_field.restype = C.c_void_p
    lib.orc_field.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]
    for f in ("orc_initialize", "orc_do_time_step", "orc_update_fields", "orc_precompute_b", "orc_precompute_e",
              "orc_precompute_e_ecr"):
        getattr(lib, f).argtypes = [C.c_void_p]
    lib.orc_run.argtypes = [C.c_void_p, C.c_uint64]
    lib.orc_time_step.restype = C.c_uint64
    lib.orc_time_step.argtypes = [C.c_void_p]
    lib.orc_set_threads.argtypes = [C.c_int]
    if hasattr(lib, "orc_set_nan_model"):
        lib.orc_set_nan_model.argtypes = [C.c_int]
    if hasattr(lib, "orc_set_electron_background"):
        lib.orc_set_electron_background.argtypes = [C.c_void_p, C.c_float]
    fp = C.POINTER(C.c_float)
    lib.orc_voxelize.restype = C.c_int
    lib.orc_voxelize.argtypes = [C.c_void_p, fp, fp, fp, C.c_uint32, fp, fp, C.c_int, C.c_float, C.c_float,
                                 C.c_float]
    return lib


def oracle_lib(prec: str = "f32") -> C.CDLL:
    key = "orc_" + prec
    if key not in _LIBS:
        so = _build.build_oracle()[prec]
        lib = _bind(C.CDLL(str(so), mode=C.RTLD_LOCAL))
        if prec == "f32":
            lib.orc_constants.restype = C.c_int
            lib.orc_constants.argtypes = [C.POINTER(IonConfig), C.POINTER(IonConstants)]
            for n, rt, at in (("orc_fp16c_encode", C.c_uint16, C.c_float), ("orc_fp16s_encode", C.c_uint16, C.c_float),
                              ("orc_fp16c_decode", C.c_float, C.c_uint16), ("orc_fp16s_decode", C.c_float, C.c_uint16)):
                getattr(lib, n).restype = rt
                getattr(lib, n).argtypes = [at]
        _LIBS[key] = lib
    return _LIBS[key]


def reference_available() -> bool:
    try:
        return _build.reference_available()
    except Exception:
        return False


def ref_lib(cfg: IonConfig) -> C.CDLL | None:
    d = config_dict(cfg)
    key = "ref_" + _build.variant_key(d)
    if key not in _LIBS:
        so = _build.build_reference(d)
        if so is None:
            return None
        _LIBS[key] = _bind(C.CDLL(str(so), mode=C.RTLD_LOCAL))
    return _LIBS[key]


def constants(cfg: IonConfig) -> IonConstants:
    k = IonConstants()
    oracle_lib("f32").orc_constants(C.byref(cfg), C.byref(k))
    return k


# ---------------------------------------------------------------------------
# a simulation on the CPU
# ---------------------------------------------------------------------------
class OracleLbm:
    """One domain advanced by a CPU oracle; mirrors the product's Lbm class."""

    def __init__(self, cfg: IonConfig, kind: str = "f32", threads: int = 1, canonical_nan: bool = False):
        self.cfg = cfg
        self.kind = kind
        if kind == "ref":
            lib = ref_lib(cfg)
            if lib is None:
                raise RuntimeError("reference kernels unavailable (no IonSolver checkout and no generated copy)")
        else:
            lib = oracle_lib(kind)
        self.lib = lib
        self.threads = threads
        self.canonical_nan = canonical_nan
        k = constants(cfg)
        h = lib.orc_create(C.byref(cfg), C.byref(k))
        if not h:
            raise ValueError("oracle rejected the configuration")
        self.h = C.c_void_p(h)

    def close(self):
        if self.h:
            self.lib.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _threads(self):
        self.lib.orc_set_threads(int(self.threads))
        if hasattr(self.lib, "orc_set_nan_model"):
            self.lib.orc_set_nan_model(int(self.canonical_nan))

    @property
    def n(self) -> int:
        return int(self.cfg.n_x) * int(self.cfg.n_y) * int(self.cfg.n_z)

    def field(self, name: str) -> np.ndarray:
        """A writable numpy view of the oracle's array (no copy)."""
        eb, cnt = C.c_size_t(), C.c_size_t()
        p = self.lib.orc_field(self.h, FIELDS[name], C.byref(eb), C.byref(cnt))
        if not p:
            return np.zeros(0, np.float32)
        if name == "flags":
            dt = np.uint8
        elif eb.value == 2:
            dt = np.uint16
        elif eb.value == 8:
            dt = np.float64
        else:
            dt = np.float32
        buf = (C.c_char * (eb.value * cnt.value)).from_address(p)
        return np.frombuffer(buf, dtype=dt)

    def set_field(self, name: str, values) -> None:
        a = self.field(name)
        v = np.asarray(values).reshape(-1)
        a[: v.size] = v.astype(a.dtype)

    def set_electron_background(self, rho_e0: float) -> None:
        """The finite-plasma start of the next initialize (restatement only)."""
        self.lib.orc_set_electron_background(self.h, float(rho_e0))

    def initialize(self):
        self._threads()
        self.lib.orc_initialize(self.h)

    def do_time_step(self):
        self._threads()
        self.lib.orc_do_time_step(self.h)

    def run(self, steps: int):
        self._threads()
        self.lib.orc_run(self.h, int(steps))

    def update_fields(self):
        self._threads()
        self.lib.orc_update_fields(self.h)

    @property
    def time_step(self) -> int:
        return int(self.lib.orc_time_step(self.h))

    def voxelise(self, p0, p1, p2, model: str, v=(0.0, 0.0, 0.0)):
        p0 = np.ascontiguousarray(p0, np.float32).reshape(-1)
        p1 = np.ascontiguousarray(p1, np.float32).reshape(-1)
        p2 = np.ascontiguousarray(p2, np.float32).reshape(-1)
        pts = np.concatenate([p0.reshape(-1, 3), p1.reshape(-1, 3), p2.reshape(-1, 3)])
        pmin, pmax = mesh_bounds(p0, p1, p2)
        fp = C.POINTER(C.c_float)
        self._threads()
        r = self.lib.orc_voxelize(self.h, p0.ctypes.data_as(fp), p1.ctypes.data_as(fp), p2.ctypes.data_as(fp),
                                  p0.size // 3, pmin.ctypes.data_as(fp), pmax.ctypes.data_as(fp), MODEL[model],
                                  float(v[0]), float(v[1]), float(v[2]))
        del pts
        if r != 0:
            raise ValueError("voxelise failed")

    def precompute_b(self):
        self._threads()
        self.lib.orc_precompute_b(self.h)

    def precompute_e(self):
        self._threads()
        self.lib.orc_precompute_e(self.h)

    def precompute_e_ecr(self):
        self._threads()
        self.lib.orc_precompute_e_ecr(self.h)


def mesh_bounds(p0, p1, p2):
    """Mesh::update_bounds (IonSolver src/mesh.rs:94-109) in float32."""
    a = np.asarray(p0, np.float32).reshape(-1, 3)
    b = np.asarray(p1, np.float32).reshape(-1, 3)
    c = np.asarray(p2, np.float32).reshape(-1, 3)
    pmin = np.minimum(np.minimum(a, b), c).min(axis=0).astype(np.float32)
    pmax = np.maximum(np.maximum(a, b), c).max(axis=0).astype(np.float32)
    return np.ascontiguousarray(pmin), np.ascontiguousarray(pmax)


def cpu_count() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


__all__ = ["IonUnits", "IonConfig", "IonConstants", "make_config", "OracleLbm", "oracle_lib", "ref_lib",
           "reference_available", "constants", "mesh_bounds", "FIELDS", "MODEL", "cpu_count"]
_ = Path
