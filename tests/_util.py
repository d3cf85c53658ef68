"""Shared helpers of the test-suite: run one synthetic case on the GPU and on
a CPU oracle, and compare the results."""
from __future__ import annotations

import numpy as np

import oracle as O
from ionsolver_gb300 import workloads as W

MODEL_NAMES = {v: k for k, v in W.MODEL_IDS.items()}


def oracle_config(case):
    return O.make_config(**case["config"])


def setup_oracle(case, kind="f32", threads=None, canonical_nan=False):
    o = O.OracleLbm(oracle_config(case), kind, threads or O.cpu_count(), canonical_nan)
    o._threads()
    for name, arr in case["fields"].items():
        o.set_field(name, arr)
    if case.get("electron_background") and kind != "ref":  # "ref": see initialize_oracle
        o.set_electron_background(case["electron_background"])
    for p0, p1, p2, model, vals in case["meshes"]:
        o.voxelise(p0, p1, p2, model, vals)
    if case["precompute_b"]:
        o.precompute_b()
    if case.get("precompute_e_ecr"):
        o.precompute_e_ecr()
    for p0, p1, p2, model, vals in case.get("meshes_after", []):
        o.voxelise(p0, p1, p2, model, vals)
    return o


def initialize_oracle(o, case):
    """initialize, plus the finite-plasma start where the case asks for it.  The
    reference's kernels have no such start (their electron gas starts at 0), so
    for them the electron and charge DDFs after initialize are taken from the
    restatement's initialize: the same calculate_f_eq / calculate_a_eq, at
    density rho_e0 and Q + rho_e0."""
    o.initialize()
    if case.get("electron_background") and o.kind == "ref":
        r = setup_oracle(case, "f32", o.threads, o.canonical_nan)
        r.initialize()
        for name in ("ei", "fqi"):
            o.set_field(name, r.field(name))
        r.close()


def run_oracle(case, steps, kind="f32", threads=None, canonical_nan=False):
    o = setup_oracle(case, kind, threads, canonical_nan)
    initialize_oracle(o, case)
    o.run(steps)
    return o


def setup_gpu(case):
    import ionsolver_gb300 as I
    lbm = I.Lbm(W.lbm_config(case))
    W.apply_case(lbm, case)
    return lbm


def run_gpu(case, steps, graph=True):
    lbm = setup_gpu(case)
    lbm.initialize()
    if graph:
        lbm.run(steps)
    else:
        for _ in range(steps):
            lbm.do_time_step()
    lbm.finish_queues(120000)
    return lbm


def field_names(case):
    names = ["fi", "rho", "u", "flags"]
    if case["config"].get("ext_magneto_hydro"):
        names += ["fqi", "ei", "q", "e_dyn", "b_dyn", "b_stat", "e_stat", "qu_lod"]
    if case["config"].get("ext_subgrid_ecr"):
        names += ["e_var", "eti", "et"]
    return names


def bit_diff(a: np.ndarray, b: np.ndarray) -> int:
    """Number of elements whose bit patterns differ."""
    assert a.dtype.itemsize == b.dtype.itemsize and a.size == b.size, (a.dtype, b.dtype, a.size, b.size)
    ia = a.view(np.uint8).reshape(a.size, a.dtype.itemsize)
    ib = b.view(np.uint8).reshape(b.size, b.dtype.itemsize)
    return int(np.any(ia != ib, axis=1).sum())


def _nan_mask(a: np.ndarray, float_type: int | None) -> np.ndarray:
    if a.dtype == np.float32 or a.dtype == np.float64:
        return np.isnan(a)
    if a.dtype == np.uint16 and float_type == 0:  # FP16S: IEEE half NaN
        return ((a & 0x7C00) == 0x7C00) & ((a & 0x03FF) != 0)
    return np.zeros(a.shape, bool)


def bit_diff_nan(a: np.ndarray, b: np.ndarray, float_type: int | None = None) -> int:
    """Elements whose bits differ, counting two NaNs as equal (IEEE leaves NaN
    payloads to the hardware: GPUs return one canonical NaN, CPUs propagate
    operand payloads)."""
    na, nb = _nan_mask(a, float_type), _nan_mask(b, float_type)
    both = na & nb
    ia = a.view(np.uint8).reshape(a.size, a.dtype.itemsize)
    ib = b.view(np.uint8).reshape(b.size, b.dtype.itemsize)
    return int((np.any(ia != ib, axis=1) & ~both).sum())


def compare_bitwise(gpu, orc, names):
    """Bit-level comparison of GPU and oracle fields (NaN equals NaN)."""
    ft = int(orc.cfg.float_type)
    out = {}
    for n in names:
        g = gpu.read(n)
        o = orc.field(n)
        if o.dtype != g.dtype:
            o = o.astype(g.dtype)
        out[n] = bit_diff_nan(g, o, ft if n in ("fi", "fqi", "ei", "eti") else None)
    return out


def rel_err(a, b):
    """max |a-b| / max |b| (normwise relative error)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    d = np.max(np.abs(a - b)) if a.size else 0.0
    s = np.max(np.abs(b)) if b.size else 0.0
    return float(d / s) if s > 0 else float(d)
