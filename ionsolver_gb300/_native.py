"""ctypes binding of include/ionsolver.h (libionsolver.so, built in-tree).

The library is the product: loading fails loudly when it is missing, and no
function here falls back to a CPU implementation.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_build" / "libionsolver.so"

ION_OK = 0
ION_E_TIMEOUT = -7
ION_WAIT_LIMIT_DEFAULT = 16777216      # include/ionsolver.h
ION_BARRIER_LIMIT_DEFAULT = 67108864
ERRORS = {-1: "ION_E_INVALID", -2: "ION_E_CONFIG", -3: "ION_E_CUDA", -4: "ION_E_NOMEM", -5: "ION_E_IO",
          -6: "ION_E_FORMAT", -7: "ION_E_TIMEOUT", -8: "ION_E_STATE"}


class IonError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"{ERRORS.get(code, code)}: {message}")
        self.code = code


class Units(C.Structure):
    """Units (IonSolver src/lbm/units.rs:14-27)."""
    _fields_ = [("m", C.c_float), ("kg", C.c_float), ("s", C.c_float), ("a", C.c_float), ("k", C.c_float),
                ("prop", C.c_int32)]


class Config(C.Structure):
    """ion_config, the C form of LbmConfig (IonSolver src/lbm/mod.rs:45-101)."""
    _fields_ = [
        ("velocity_set", C.c_int32), ("relaxation_time", C.c_int32), ("float_type", C.c_int32),
        ("units", Units),
        ("n_x", C.c_uint32), ("n_y", C.c_uint32), ("n_z", C.c_uint32),
        ("d_x", C.c_uint32), ("d_y", C.c_uint32), ("d_z", C.c_uint32),
        ("nu", C.c_float), ("f_x", C.c_float), ("f_y", C.c_float), ("f_z", C.c_float),
        ("ext_equilibrium_boundaries", C.c_uint8), ("ext_volume_force", C.c_uint8),
        ("ext_force_field", C.c_uint8), ("ext_magneto_hydro", C.c_uint8), ("ext_subgrid_ecr", C.c_uint8),
        ("mhd_lod_depth", C.c_uint8), ("update_fields", C.c_uint8), ("field_mode", C.c_uint8),
        ("ecr_freq", C.c_float), ("ecr_field_strength", C.c_float),
        ("run_steps", C.c_uint64),
    ]


class Constants(C.Structure):
    _fields_ = [(n, C.c_float) for n in ("w", "ke", "kmu", "kmu0", "kkge", "kimg", "kvev", "kme", "wq",
                                          "epsilon_0", "mu_0", "kkbme", "keabs")]


# exported symbols and their signatures (every declaration of include/ionsolver.h)
_P = C.c_void_p
_SIGS = {
    "ion_abi_version": (C.c_int, []),
    "ion_select_device": (C.c_int, [C.c_int]),
    "ion_probe_fp32_peak": (C.c_int, [C.POINTER(C.c_double)]),
    "ion_last_error": (C.c_char_p, []),
    "ion_kernel_launch_count": (C.c_uint64, []),
    "ion_config_default": (C.c_int, [C.POINTER(Config)]),
    "ion_units_default": (C.c_int, [C.POINTER(Units)]),
    "ion_units_set": (C.c_int, [C.POINTER(Units)] + [C.c_float] * 10),
    "ion_constants_from_config": (C.c_int, [C.POINTER(Config), C.POINTER(Constants)]),
    "ion_units_si_to_lu": (C.c_int, [C.POINTER(Units), C.c_int, C.c_float, C.POINTER(C.c_float)]),
    "ion_lbm_create": (C.c_int, [C.POINTER(Config), C.POINTER(_P)]),
    "ion_lbm_destroy": (C.c_int, [_P]),
    "ion_lbm_get_config": (C.c_int, [_P, C.POINTER(Config)]),
    "ion_lbm_initialize": (C.c_int, [_P]),
    "ion_lbm_set_electron_background": (C.c_int, [_P, C.c_float]),
    "ion_lbm_set_wait_limit": (C.c_int, [_P, C.c_uint32]),
    "ion_lbm_do_time_step": (C.c_int, [_P]),
    "ion_lbm_run": (C.c_int, [_P, C.c_uint64]),
    "ion_lbm_get_time_step": (C.c_int, [_P, C.POINTER(C.c_uint64)]),
    "ion_lbm_finish_queues": (C.c_int, [_P, C.c_int]),
    "ion_lbm_update_fields": (C.c_int, [_P]),
    "ion_lbm_field_info": (C.c_int, [_P, C.c_int, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]),
    "ion_lbm_write_field": (C.c_int, [_P, C.c_int, _P, C.c_size_t]),
    "ion_lbm_read_field": (C.c_int, [_P, C.c_int, _P, C.c_size_t]),
    "ion_lbm_field_device_ptr": (C.c_int, [_P, C.c_int, C.POINTER(_P), C.POINTER(C.c_size_t)]),
    "ion_lbm_stream": (C.c_int, [_P, C.POINTER(_P)]),
    "ion_lbm_add_mesh": (C.c_int, [_P, _P, _P, _P, C.c_uint32, C.POINTER(C.c_uint32)]),
    "ion_lbm_import_mesh": (C.c_int, [_P, C.c_char_p] + [C.c_float] * 7 + [C.POINTER(C.c_uint32)]),
    "ion_lbm_import_mesh_reposition": (C.c_int, [_P, C.c_char_p] + [C.c_float] * 7 + [C.POINTER(C.c_uint32)]),
    "ion_lbm_mesh_translate": (C.c_int, [_P, C.c_uint32, C.c_float, C.c_float, C.c_float]),
    "ion_lbm_mesh_bounds": (C.c_int, [_P, C.c_uint32, C.POINTER(C.c_float)]),
    "ion_lbm_mesh_triangles": (C.c_int, [_P, C.c_uint32, _P, _P, _P, C.c_uint32, C.POINTER(C.c_uint32)]),
    "ion_lbm_voxelise_mesh": (C.c_int, [_P, C.c_uint32, C.c_int, C.c_float, C.c_float, C.c_float]),
    "ion_lbm_precompute_b": (C.c_int, [_P]),
    "ion_lbm_precompute_e": (C.c_int, [_P]),
    "ion_lbm_precompute_e_ecr": (C.c_int, [_P]),
    "ion_lbm_mass_charge": (C.c_int, [_P, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "ion_lbm_save": (C.c_int, [_P, C.c_char_p]),
    "ion_lbm_load": (C.c_int, [C.c_char_p, C.POINTER(Config), C.POINTER(_P)]),
    "ion_lbm_record_event": (C.c_int, [_P, C.c_int]),
    "ion_lbm_event_elapsed": (C.c_int, [_P, C.c_int, C.c_int, C.POINTER(C.c_float)]),
    "ion_lbm_set_kernel_timing": (C.c_int, [_P, C.c_int]),
    "ion_lbm_kernel_time": (C.c_int, [_P, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_uint64)]),
    "ion_lbm_reset_kernel_time": (C.c_int, [_P]),
    "ion_check_shared_division": (C.c_int, [C.c_uint64, C.c_uint64, C.POINTER(C.c_uint64), C.POINTER(C.c_float)]),
    "ion_check_tcgen05_conv": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_uint64, C.POINTER(C.c_float)]),
    "ion_codec_roundtrip": (C.c_int, [C.c_int, _P, _P, _P, _P, _P, C.c_uint64]),
    "ion_ddf_sum_f64_noalloc": (C.c_int, [_P, C.c_int, C.c_uint64, _P, _P]),
    "ion_config_write_json": (C.c_int, [C.c_char_p, C.POINTER(Config)]),
    "ion_config_read_json": (C.c_int, [C.c_char_p, C.POINTER(Config)]),
    "ion_lbm_checkpoint": (C.c_int, [_P, C.c_char_p]),
    "ion_lbm_restore": (C.c_int, [C.c_char_p, C.POINTER(Config), C.POINTER(_P)]),
    "ion_lbm_surrogate_train": (C.c_int, [_P, C.c_uint32, C.c_uint32, C.c_uint32, C.c_float, C.c_uint64,
                                          C.POINTER(C.c_float)]),
    "ion_lbm_surrogate_info": (C.c_int, [_P, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float),
                                         C.c_uint32, C.POINTER(C.c_uint32)]),
    "ion_lbm_surrogate_save": (C.c_int, [_P, C.c_char_p]),
    "ion_lbm_surrogate_load": (C.c_int, [_P, C.c_char_p]),
    "ion_lbm_surrogate_configure": (C.c_int, [_P, C.c_float, C.c_uint32]),
    "ion_lbm_surrogate_stats": (C.c_int, [_P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.POINTER(C.c_uint64),
                                          C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "ion_lbm_surrogate_targets": (C.c_int, [_P, _P, _P, C.c_uint32, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "ion_lbm_surrogate_weights": (C.c_int, [_P, _P, _P, C.c_size_t]),
    "ion_lbm_surrogate_grad": (C.c_int, [_P, _P, _P, C.c_uint32, C.POINTER(C.c_float), _P]),
    "ion_lbm_surrogate_forward": (C.c_int, [_P, _P, _P, C.c_int]),
    "ion_lbm_set_field_mode": (C.c_int, [_P, C.c_int]),
    "ion_batch_create": (C.c_int, [C.POINTER(_P), C.c_uint32, C.POINTER(_P)]),
    "ion_batch_destroy": (C.c_int, [_P]),
    "ion_batch_run": (C.c_int, [_P, C.c_uint64]),
    "ion_batch_finish": (C.c_int, [_P, C.c_int]),
    "ion_batch_set_wait_limits": (C.c_int, [_P, C.c_uint32, C.c_uint32]),
    "ion_batch_tuning": (C.c_int, [_P, C.c_uint32, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                   C.POINTER(C.c_float)]),
    "ion_batch_record_event": (C.c_int, [_P, C.c_int]),
    "ion_batch_event_elapsed": (C.c_int, [_P, C.c_int, C.c_int, C.POINTER(C.c_float)]),
}

_lib: C.CDLL | None = None


def lib() -> C.CDLL:
    """Load libionsolver.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`"
                              " or `python ionsolver_gb300/build.py`")
        L = C.CDLL(str(LIB_PATH))
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(rc: int) -> None:
    if rc != ION_OK:
        raise IonError(rc, lib().ion_last_error().decode(errors="replace"))


def exported_symbols() -> list[str]:
    return list(_SIGS)
