#!/usr/bin/env python3
"""Benchmark of the IonSolver MHD-LBM timestep on GB300 (one JSON line on rank 0).

Workloads (``--workload``; default ``mhd128``, the headline configuration):
  mhd128 / mhd256 : D3Q19 fluid + D3Q7 charge lattice + electron gas, FP32
      storage (``--float-type`` for FP16S/FP16C), tau 0.6, one-cell solid walls,
      charge U[-1e-3,1e-3] (seed 1), velocity N(0,1e-3^2) (seed 2), an axially
      magnetised disk magnet (r 16, t 8 at 128^3) on the z = 1 face, LOD depth
      4, the exact LOD E/B update every step.  ``--start plasma`` (default for
      every MHD workload): the finite-plasma start of workloads.mhd_plasma
      (electron gas at a background density in units where the state stays
      finite); ``--start reference``: the reference's start, whose electron
      gas is empty and turns every MHD field NaN within a few steps.
      The mhd128 line also carries a ``surrogate`` record: the rings384
      workload below (training, step-1 field error, timed learned-field steps,
      fallbacks) against the exact FP32 step of the same box.
  batch96 : 96 independent MHD domains, cube edges from {32,48,64,80,96}
      (seed 3), a disk magnet each (radius 4..12, seed 4), one persistent
      launch per step for all of them, autotuned launch shape, CUDA graph
      (batch16: 16 such domains, a case small enough for a full ncu capture).
  rings384 : 384^3, FP16S storage, two coaxial ring magnets (R_out 48, R_in 32,
      t 12, centres 128 apart, axis z; rings192 and rings288 the same at 1/2 and
      3/4 scale, for profiling), LOD depth 4, the learned far field
      (network trained before the timed region on 2000 exact snapshots, seed
      5) with the sampled exact check and device-decided exact fallback; the
      line also carries the exact FP32 step of the same box for comparison.
  tgv64/256/384 : plain D3Q19 SRT FP32, periodic Taylor-Green vortex (u0 0.05).
A step is one timestep of every cell (stream_collide, LOD bins, E/B update).
Metric: MLUPs/s = cells * steps / seconds / 1e6.

  value       : CUDA-event time of K steps on the library's stream, inputs
                resident in HBM.
  e2e         : the same job through the C ABI with host buffers: upload of
                the inputs from pinned memory, initialize, K steps (CUDA graph),
                download of the result fields, inside the timed region.
  roofline    : the dominant kernel -- the E/B update, FP32-bound -- against
                the measured FP32 FMA peak (ion_probe_fp32_peak); the plain
                workloads' dominant kernel is stream_collide against the
                measured HBM bandwidth (MEASURED_PEAKS.json).
  cpu_baseline: the reference's kernels compiled for the host (or the C
                restatement when the reference copy is absent), all host cores,
                a bounded sample of the same workload.

``--impl reference`` runs only that CPU implementation and prints its line.
Multi-GPU (torchrun): replicas only -- every rank advances its own copy of the
workload on its own GPU, no data exchange; value = ranks * cells * steps /
max-over-ranks time.
"""
from __future__ import annotations

import argparse
import datetime as _dt
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

FLOP_PER_INTERACTION = 34  # one source's E and B: 34 FLOP + 1 sqrt (sim_kernels.cl:950-954)
# kernel-time results of one ncu capture (dram__bytes_read.sum + dram__bytes_write.sum per launch);
# the summaries with the commands that produced them are in profiles/
# (rings384: the rings192 capture of k_sc_rows_ws scaled by the cell count, (384/192)^3; every
# stream is read and written once per cell, so the traffic is proportional to the cells)
NCU_TRAFFIC = {("tgv256", "k_sc_rows_ws"): 2.505911e9, ("mhd128", "k_sc_rows_ws"): 0.816344e9,
               ("mhd128", "k_update_e_b_fast"): 63.815e6, ("rings384", "k_sc_rows_ws"): 8 * 1.627825e9}


def stencil_kernel(cfg: dict) -> str:
    """The stream_collide kernel the library launches for a domain: the row-staged
    D3Q19 kernel when rows are whole 16-byte streams (and not SUBGRID_ECR)."""
    rows = cfg.get("velocity_set", 2) == 2 and not cfg.get("ext_subgrid_ecr") and cfg["n_x"] % 16 == 0
    if not rows:
        return "k_stream_collide"
    return "k_sc_rows_ws" if cfg["n_x"] <= 384 else "k_sc_rows"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=50)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--workload", default="mhd128",
                   choices=["mhd128", "mhd256", "mhd64", "batch96", "batch16", "rings384", "rings192", "rings192d3", "rings288", "tgv64",
                            "tgv256", "tgv384"])
    p.add_argument("--field-mode", default=None, choices=["bitwise", "fast", "surrogate"],
                   help="default: surrogate for rings384, fast otherwise")
    p.add_argument("--float-type", default=None, choices=["FP32", "FP16S", "FP16C"],
                   help="default: FP16S for rings384, FP32 otherwise")
    p.add_argument("--train-samples", type=int, default=2000, help="rings384: exact snapshots to train on")
    p.add_argument("--train-epochs", type=int, default=20)
    p.add_argument("--ref-seconds", type=float, default=20.0, help="CPU time budget of the reference/baseline sample")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--clocks-dir", default=None, help="keep the raw nvidia-smi samples as clocks_rank<i>.csv here")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--start", default="plasma", choices=["plasma", "reference"],
                   help="initial electron gas of the MHD workloads (see the module docstring)")
    p.add_argument("--update-fields", default=None, choices=["on", "off"],
                   help="rho/u written by every stream_collide (default: on for MHD, as the reference with its "
                        "graphics active; off for the plain TGV boxes)")
    p.add_argument("--no-surrogate-record", action="store_true",
                   help="mhd128: leave out the learned-far-field record (rings384)")
    p.add_argument("--surrogate-size", type=int, default=384, help="box edge of the mhd128 line's surrogate record")
    a = p.parse_args()
    rings = a.workload.startswith("rings")
    a.field_mode = a.field_mode or ("surrogate" if rings else "fast")
    a.float_type = a.float_type or ("FP16S" if rings else "FP32")
    if a.field_mode == "surrogate" and not rings:
        p.error("--field-mode surrogate needs --workload rings384 or rings192")
    return a


FT = {"FP16S": 0, "FP16C": 1, "FP32": 2}
FM = {"bitwise": 0, "fast": 1, "surrogate": 2}


def make_cases(a) -> list[dict]:
    cases = _make_cases(a)
    if getattr(a, "update_fields", None) is not None:
        for c in cases:
            c["config"]["update_fields"] = int(a.update_fields == "on")
    return cases


def _make_cases(a) -> list[dict]:
    from ionsolver_gb300 import workloads as W
    fm = FM[a.field_mode]
    ft = FT[a.float_type]
    w = a.workload
    plasma = a.start == "plasma"
    if w.startswith("batch"):  # batch16: 16 domains drawn as batch96's are (a profiling case)
        return W.batch_domains(int(w[5:]), float_type=ft, field_mode=fm, plasma=plasma)
    if w.startswith("rings"):  # rings192: the same box at half the size; rings192d3: LOD depth 3, i.e. the
        n, _, d = w[5:].partition("d")  # 24^3-cell bins of rings384 (profiling cases)
        case = W.mhd_box(n=int(n), float_type=ft, depth=int(d or 4), field_mode=fm, rings=True)
        return [W.to_plasma(case) if plasma else case]
    n = int(w[3:])
    if w.startswith("mhd"):
        case = W.mhd_box(n=n, float_type=ft, field_mode=fm, magnet_r=16.0 * n / 128, magnet_t=8.0 * n / 128)
        return [W.to_plasma(case) if plasma else case]
    case = W.taylor_green(n=n, amplitude=0.05, float_type=ft)
    case["config"]["update_fields"] = 0
    return [case]


def bytes_per_lup(cfg: dict) -> int:
    """Algorithmic DRAM bytes of one lattice update of stream_collide."""
    db = 4 if cfg.get("float_type", 2) == 2 else 2
    b = 2 * 19 * db + 1                      # DDFs loaded and stored once, flags
    if cfg.get("update_fields"):
        b += 16                              # rho, u written
    if cfg.get("ext_magneto_hydro"):
        b += 2 * (19 + 7) * db               # electron and charge DDFs
        b += 24 + 4                          # E, B read; Q written
        if cfg.get("mhd_lod_depth", 4) > 0:
            b += 12                          # velocity contribution to the LOD bins
    return b


def near_interactions(cfg: dict, flags: np.ndarray, rnear: int) -> int:
    """Source terms the learned-far-field path sums exactly per step: fluid
    cells x bins within Chebyshev distance rnear of their own bin (own bin
    and bins below the source range excluded)."""
    D = int(cfg["mhd_lod_depth"])
    nd = 1 << D
    n_own = 1 + sum(8 ** (i + 1) for i in range(D))
    first = n_own - nd ** 3
    nx, ny, nz = cfg["n_x"], cfg["n_y"], cfg["n_z"]
    fl = ((flags & 0x1F) != 0x01).reshape(nd, nz // nd, nd, ny // nd, nd, nx // nd)
    fluid_per_bin = fl.sum(axis=(1, 3, 5))  # [bz][by][bx]
    idx = np.arange(nd ** 3).reshape(nd, nd, nd)
    total = 0
    for bz in range(nd):
        for by in range(nd):
            for bx in range(nd):
                sl = idx[max(bz - rnear, 0):bz + rnear + 1, max(by - rnear, 0):by + rnear + 1,
                         max(bx - rnear, 0):bx + rnear + 1]
                own = bx + (by + bz * nd) * nd
                total += int(fluid_per_bin[bz, by, bx]) * int(((sl >= first) & (sl != own)).sum())
    return total


def field_interactions(cfg: dict, flags: np.ndarray) -> int:
    """Source terms the E/B update evaluates (fluid cells x LOD bins in range, own bin excluded)."""
    D = int(cfg["mhd_lod_depth"])
    nd = 1 << D
    n_own = 1 + sum(8 ** (i + 1) for i in range(D))
    first = n_own - nd ** 3
    nx, ny, nz = cfg["n_x"], cfg["n_y"], cfg["n_z"]
    fl = ((flags & 0x1F) != 0x01).reshape(nz, ny, nx)
    bz = (np.arange(nz) // (nz // nd))[:, None, None]
    by = (np.arange(ny) // (ny // nd))[None, :, None]
    bx = (np.arange(nx) // (nx // nd))[None, None, :]
    own = bx + (by + bz * nd) * nd
    fluid = int(fl.sum())
    return fluid * (nd ** 3 - first) - int((fl & (own >= first)).sum())


# ---------------------------------------------------------------------------
class Dist:
    """Rank bookkeeping; N > 1 runs independent replicas (gloo for barrier/max)."""

    def __init__(self):
        self.rank = int(os.environ.get("RANK", "0"))
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo", rank=self.rank, world_size=self.world)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x: float) -> float:
        if not self.pg:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


class Clocks:
    """nvidia-smi samples every 50 ms; the summary uses the samples taken inside the timed window."""
    QUERY = ("timestamp,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
    NAMES = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]

    def __init__(self, index: int, keep_dir: str | None = None):
        # the raw samples go to a temporary file unless --clocks-dir asks to keep them
        self.index = index
        self.proc = None
        self.keep = keep_dir is not None
        self.path = (Path(keep_dir) / f"clocks_rank{index}.csv" if self.keep else
                     Path(tempfile.gettempdir()) / f"ion_bench_clocks_{os.getpid()}_{index}.csv")
        self.t0 = self.t1 = None

    def start(self):
        try:
            self.path.parent.mkdir(parents=True, exist_ok=True)
            self.f = open(self.path, "w")
        except OSError:
            return
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "50"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
            time.sleep(0.5)
        except Exception:  # no nvidia-smi: no clock record
            self.proc = None
            self.f.close()
            if not self.keep:
                self.path.unlink(missing_ok=True)

    def mark(self, which: str):
        setattr(self, which, _dt.datetime.now())

    def stop(self) -> dict | None:
        if not self.proc:
            return None
        time.sleep(0.3)
        self.proc.terminate()
        try:
            self.proc.wait(5)
        except Exception:
            self.proc.kill()
        self.f.close()
        rows = []
        text = self.path.read_text()
        if not self.keep:
            self.path.unlink(missing_ok=True)
        for line in text.splitlines():
            p = [x.strip() for x in line.split(",")]
            if len(p) < 8:
                continue
            try:
                ts = _dt.datetime.strptime(p[0], "%Y/%m/%d %H:%M:%S.%f")
                rows.append((ts, float(p[1]), float(p[2]), p[3], p[4:8]))
            except ValueError:
                continue
        if not rows:
            return None
        inside = [r for r in rows if self.t0 and self.t1 and self.t0 <= r[0] <= self.t1]
        use = inside if inside else rows
        reasons = sorted({n for r in use for n, v in zip(self.NAMES, r[4]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(r[1] for r in use), "sm_max_mhz": max(r[2] for r in use),
                "reasons": reasons, "samples": len(use), "window": "timed region" if inside else "whole run"}


def cpu_sample_cases(a, cases: list[dict]) -> list[dict]:
    """The host-core sample of a workload.  rings384: the same two-ring box at
    96^3 -- at LOD depth 4 the reference's E/B update costs 4095 source terms
    per cell at any box size, so its MLUPs/s carry over; a 384^3 step would
    take minutes on the host cores."""
    if a.workload.startswith("rings"):
        from ionsolver_gb300 import workloads as W
        return [W.mhd_box(n=96, float_type=FT[a.float_type], depth=4, field_mode=0, rings=True)]
    return cases


# ---------------------------------------------------------------------------
def _oracle_for(case: dict, kind: str, cores: int, init: dict):
    """An initialized CPU oracle of the case ("ref": the reference's kernels,
    "f32": the restatement), with the case's start.  The reference's kernels
    have no finite-plasma start, so for them the electron and charge DDFs
    after initialize come from the restatement's initialize of the same
    fields (the reference's calculate_f_eq / calculate_a_eq at rho_e0 and
    Q + rho_e0)."""
    import oracle as O
    from tests import _util as U

    def make(k):
        o = O.OracleLbm(U.oracle_config(case), k, cores)
        for name, arr in case["fields"].items():
            o.set_field(name, arr)
        for name, arr in init.items():  # static fields (setup, untimed)
            o.set_field(name, arr)
        return o
    o = make(kind)
    rho_e0 = case.get("electron_background")
    if rho_e0 and kind != "ref":
        o.set_electron_background(rho_e0)
    o.initialize()
    if rho_e0 and kind == "ref":
        r = make("f32")
        r.set_electron_background(rho_e0)
        r.initialize()
        for name in ("ei", "fqi"):
            o.set_field(name, r.field(name))
        r.close()
    return o


def cpu_run(cases: list[dict], steps: int, budget_s: float, init_fields: list[dict] | None, warmup: int = 0):
    """Advances the cases on the host cores: `warmup` untimed steps of the
    first case, then timed steps until `steps` are done or the time budget is
    spent (a step that starts inside the budget is finished).

    Returns (MLUPs/s, sample description, kind, cores, timed steps, warm-up steps)."""
    import oracle as O
    cores = O.cpu_count()
    kind = "reference" if O.reference_available() else "port"
    done_cells, done_steps, t_total, used, warm = 0, 0, 0.0, 0, 0
    for i, case in enumerate(cases):
        init = (init_fields or [{}] * len(cases))[i] or {}
        try:
            o = _oracle_for(case, "ref" if kind == "reference" else "f32", cores, init)
        except Exception:
            kind = "port"
            o = _oracle_for(case, "f32", cores, init)
        if i == 0:
            for _ in range(warmup):
                o.do_time_step()
                warm += 1
        t0 = time.perf_counter()
        s = 0
        while done_steps + s < steps:
            o.do_time_step()
            s += 1
            if t_total + time.perf_counter() - t0 > budget_s:
                break
        t_total += time.perf_counter() - t0
        done_cells += o.n * s
        done_steps += s
        used += 1
        o.close()
        if t_total > budget_s or done_steps >= steps:
            break
    mlups = done_cells / t_total / 1e6
    if len(cases) == 1:
        c = cases[0]["config"]
        sample = (f"{done_steps} full timestep(s) of the {c['n_x']}x{c['n_y']}x{c['n_z']} case after initialize"
                  f"{' and ' + str(warm) + ' untimed warm-up step(s)' if warm else ''}, {t_total:.1f} s")
    else:
        sample = f"{done_steps} domain-step(s) over the first {used} of {len(cases)} domains, {t_total:.1f} s"
    return mlups, sample, kind, cores, done_steps, warm


# ---------------------------------------------------------------------------
def _restart(lbm, case):
    """The case's initial state again (initialize() reads rho, u, q and the LOD bins)."""
    for n in ("rho", "u", "q"):
        lbm.write(n, case["fields"][n])
    lbm.write("qu_lod", np.zeros(lbm.field_info("qu_lod")[1], np.float32))
    lbm.initialize()


def _dyn(lbm, n):
    """E_dyn and B_dyn, the fields the next step uses."""
    return lbm.read("e_dyn")[:3 * n].astype(np.float64), lbm.read("b_dyn")[:3 * n].astype(np.float64)


def _rel(x, ref):
    return float(np.max(np.abs(x - ref)) / max(np.max(np.abs(ref)), 1e-300))


def surrogate_setup(a, case: dict, lbm) -> dict:
    """Trains the learned far field (untimed setup) and measures its field
    error after the first step against the exact sum on the same state."""
    t0 = time.perf_counter()
    lbm.surrogate_train(samples=a.train_samples, epochs=a.train_epochs, batch=8, lr=2e-3, seed=5)
    train_s = time.perf_counter() - t0
    info = lbm.surrogate_info()
    n = case["config"]["n_x"] * case["config"]["n_y"] * case["config"]["n_z"]
    lbm.surrogate_configure(tolerance=1e30, check_cells=1024)
    _restart(lbm, case)
    lbm.do_time_step()
    e_s, b_s = _dyn(lbm, n)
    lbm.set_field_mode(1)
    _restart(lbm, case)
    lbm.do_time_step()
    e_x, b_x = _dyn(lbm, n)
    lbm.set_field_mode(2)
    lbm.surrogate_configure(tolerance=1e-2, check_cells=1024)  # the run's settings; restarts the statistics
    _restart(lbm, case)
    return {"train_s": train_s, "train_samples": a.train_samples, "train_epochs": a.train_epochs, "seed": 5,
            "rel_err_fp32_heldout": info["rel_err_fp32"], "rel_err_bf16_heldout": info["rel_err_bf16"],
            "field_rel_err_step1": {"e": _rel(e_s, e_x), "b": _rel(b_s, b_x),
                                    "against": "E_dyn, B_dyn of the exact FAST sum of the same state, "
                                               "max|diff|/max|exact| (B_dyn is B_stat to float precision)"},
            "loss_first_last": [info["loss"][0], info["loss"][-1]] if info["loss"] else None,
            "check": {"tolerance": 1e-2, "cells": 1024}}


def exact_fp32_step(case: dict, src) -> dict:
    """The exact FP32 step (FAST field mode) of the same box, CUDA-event timed."""
    import ionsolver_gb300 as I
    from ionsolver_gb300 import workloads as W
    cfg = dict(case["config"], float_type=2, field_mode=1)
    ex = I.Lbm(W.lbm_config(dict(case, config=cfg)))
    for n in ("flags", "b_stat"):
        ex.write(n, src.read(n))
    for n in ("rho", "u", "q"):
        ex.write(n, case["fields"][n])
    ex.initialize()
    ex.do_time_step()
    ex.finish_queues(600000)
    steps = 2
    ex.record_event(0)
    for _ in range(steps):
        ex.do_time_step()
    ex.record_event(1)
    ms = ex.elapsed_ms(0, 1)
    ex.finish_queues(600000)
    ex.close()
    n = cfg["n_x"] * cfg["n_y"] * cfg["n_z"]
    return {"exact_fp32_ms_per_step": ms / steps, "exact_fp32_mlups": n * steps / (ms * 1e-3) / 1e6,
            "exact_fp32_steps_timed": steps}


def surrogate_record(a) -> dict:
    """Configuration 4 inside the headline line: the two-ring box at
    --surrogate-size with FP16S storage and the learned far field.  Trains the
    network (untimed setup), measures the step-1 field error against the exact
    sum of the same state, times learned-field steps (CUDA events, graph
    replay) with the sampled check and fallback active, and times the exact
    FP32 step of the same box."""
    import ionsolver_gb300 as I
    from ionsolver_gb300 import workloads as W
    n = a.surrogate_size
    case = W.mhd_box(n=n, float_type=0, depth=4, field_mode=2, rings=True)
    if a.start == "plasma":
        case = W.to_plasma(case)
    lbm = I.Lbm(W.lbm_config(case))
    W.apply_case(lbm, case)
    lbm.initialize()
    rec = surrogate_setup(a, case, lbm)
    warm, steps = 3, 20
    for _ in range(warm):
        lbm.do_time_step()
    lbm.finish_queues(600000)
    lbm.record_event(0)
    lbm.run(steps)
    lbm.record_event(1)
    ms = lbm.elapsed_ms(0, 1)
    lbm.finish_queues(600000)
    st = lbm.surrogate_stats()
    cells = n ** 3
    rec.update(workload=f"rings{n}", float_type="FP16S", steps_timed=steps, warmup=warm,
               ms_per_step=ms / steps, mlups=cells * steps / (ms * 1e-3) / 1e6,
               checks_in_run=st["checks"], fallbacks_in_run=st["fallbacks"],
               nonfinite_checks_in_run=st["nonfinite"], last_check_err_e=st["err_e"], last_check_err_b=st["err_b"])
    u = lbm.read("u")
    rec["state_finite_after_run"] = bool(np.isfinite(u).all() and np.isfinite(lbm.read("e_dyn")).all())
    rec.update(exact_fp32_step(case, lbm))
    rec["speedup_vs_exact_fp32"] = rec["exact_fp32_ms_per_step"] / rec["ms_per_step"]
    rec["targets"] = {"speedup_vs_exact_fp32": ">= 2", "field_rel_err_step1": "<= 1e-2"}
    lbm.close()
    return rec


def main():
    a = parse()
    dist = Dist()
    cases = make_cases(a)
    cfg0 = cases[0]["config"]
    mhd = bool(cfg0.get("ext_magneto_hydro"))
    cells = sum(c["config"]["n_x"] * c["config"]["n_y"] * c["config"]["n_z"] for c in cases)
    bpl = bytes_per_lup(cfg0)
    workload_cfg = {"workload": a.workload, "cells": cells, "domains": len(cases),
                    "size": [cfg0["n_x"], cfg0["n_y"], cfg0["n_z"]] if len(cases) == 1 else "uneven",
                    "velocity_set": "D3Q19", "float_type": a.float_type, "relaxation": "SRT", "tau": 0.6,
                    "mhd": mhd, "lod_depth": cfg0.get("mhd_lod_depth") if mhd else None,
                    "field_mode": a.field_mode if mhd else None,
                    "update_fields": bool(cfg0.get("update_fields")),
                    "l2": "working set %.0f MB > L2 (126 MB): no flush needed" % (cells * bpl / 1e6),
                    "parallelism": f"replicas x{dist.world}"}
    if mhd:
        workload_cfg["start"] = ("finite plasma: electron gas at a background density, plasma units "
                                 "(workloads.mhd_plasma)" if a.start == "plasma" else
                                 "reference: electron gas empty, fields NaN within a few steps")
    metric = "D3Q19-MHD MLUPs/s" if mhd else "D3Q19 MLUPs/s"
    dtype = {"FP32": "f32", "FP16S": "f32 (FP16S storage)", "FP16C": "f32 (FP16C storage)"}[a.float_type]

    if a.impl == "reference":
        if dist.rank != 0:
            dist.close()
            return
        # all K steps when they fit the reference arm's budget (--ref-seconds, at least 240 s here), else as
        # many as fit; the line states the steps and warm-up steps actually run
        ccases = cpu_sample_cases(a, cases)
        mlups, sample, kind, cores, timed, warm = cpu_run(ccases, max(a.steps, 1), max(a.ref_seconds, 240.0), None,
                                                          warmup=min(a.warmup, 1))
        ccells = sum(c["config"]["n_x"] * c["config"]["n_y"] * c["config"]["n_z"] for c in ccases) / len(ccases)
        line = {"metric": metric, "value": mlups, "unit": "MLUPs/s", "n_gpus": a.gpus, "steps": timed,
                "steps_requested": a.steps, "warmup": warm, "warmup_requested": a.warmup,
                "ms_per_step": ccells / mlups / 1e3, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": dtype, "data": "synthetic", "config": workload_cfg,
                "impl": "reference",
                "cpu_baseline": {"value": mlups, "unit": "MLUPs/s", "cores": cores, "kind": kind, "sample": sample},
                "e2e": {"value": mlups, "unit": "MLUPs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        dist.close()
        return

    import ctypes as C
    import ionsolver_gb300 as I
    from ionsolver_gb300 import _native as NAT
    from ionsolver_gb300 import workloads as W
    NAT.check(NAT.lib().ion_select_device(dist.local))

    doms = []
    for case in cases:
        lbm = I.Lbm(W.lbm_config(case))
        W.apply_case(lbm, case)
        lbm.initialize()
        doms.append(lbm)
    batch = I.Batch(doms) if len(doms) > 1 else None
    sur = None
    if a.field_mode == "surrogate":
        sur = surrogate_setup(a, cases[0], doms[0])
    clocks = Clocks(dist.local, a.clocks_dir)
    clocks.start()

    # ---- warm-up, then K timed steps (device time, CUDA events) -----------------
    if batch is None:
        lbm = doms[0]
        lbm.set_kernel_timing(True)
        for _ in range(a.warmup):
            lbm.do_time_step()
        lbm.finish_queues(600000)
        lbm.reset_kernel_time()
    else:
        batch.run(max(a.warmup, 1) + 2 * 8)  # includes the autotuner's trial steps (2 per launch shape)
        batch.finish(600000)
    launches0 = I.kernel_launch_count()
    dist.barrier()
    clocks.mark("t0")
    if batch is None:
        lbm.record_event(0)
        for _ in range(a.steps):
            lbm.do_time_step()
        lbm.record_event(1)
        ms = lbm.elapsed_ms(0, 1)
        lbm.finish_queues(600000)
    else:
        batch.record_event(0)
        batch.run(a.steps)
        batch.record_event(1)
        ms = batch.elapsed_ms(0, 1)
        batch.finish(600000)
    clocks.mark("t1")
    launches = I.kernel_launch_count() - launches0
    dist.barrier()
    ms_max = dist.max(ms)
    value = cells * a.steps * dist.world / (ms_max * 1e-3) / 1e6

    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except Exception:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    hbm_src = "measured (MEASURED_PEAKS.json)" if "hbm_gbs" in peaks else "fallback"
    share, roof_stencil, roofline, extra = {}, None, None, {}
    if batch is None:
        sc_ms, sc_n = lbm.kernel_time(0)
        eb_ms, eb_n = lbm.kernel_time(1)
        bins_ms, _ = lbm.kernel_time(2)
        sc_avg = sc_ms / max(sc_n, 1)
        gbs = cells * bpl / (sc_avg * 1e-3) / 1e9
        sk = stencil_kernel(cases[0]["config"])
        tr = NCU_TRAFFIC.get((a.workload, sk))
        roof_stencil = {"bound": "hbm", "achieved": gbs, "peak": hbm_peak, "unit": "GB/s", "frac": gbs / hbm_peak,
                        "traffic": tr, "kernel": sk, "bytes_per_lup": bpl,
                        "bytes_per_launch": cells * bpl, "avg_launch_ms": sc_avg, "peak_source": hbm_src}
        share = {"stream_collide_ms": sc_ms}
        roofline = roof_stencil
        if mhd:
            share.update(update_e_b_ms=eb_ms, lod_bins_ms=bins_ms)
    tf = C.c_double()
    if mhd:
        NAT.check(NAT.lib().ion_probe_fp32_peak(C.byref(tf)))
    if sur is not None:
        inter = near_interactions(cfg0, doms[0].read("flags"), doms[0].SURROGATE_NEAR_RADIUS)
        avg = eb_ms / max(eb_n, 1)
        tflops = inter * FLOP_PER_INTERACTION / (avg * 1e-3) / 1e12
        roof_field = {"bound": "fp32", "achieved": tflops, "peak": tf.value, "unit": "TFLOP/s",
                      "frac": tflops / tf.value, "traffic": None,
                      "kernel": "learned far field phase (k_surrogate_cells near-bin sums + network + check)",
                      "flop_per_launch": inter * FLOP_PER_INTERACTION, "interactions_per_launch": inter,
                      "avg_launch_ms": avg, "peak_source": "measured FP32 FMA throughput (ion_probe_fp32_peak)",
                      "note": "FLOPs counted: the exact near-bin terms only (the network adds ~2 GFLOP on tensor cores)"}
        roofline = roof_field if eb_ms >= sc_ms else roof_stencil
        if roofline is roof_stencil:
            extra["roofline_field"] = roof_field
        st = doms[0].surrogate_stats()
        sur.update(checks_in_run=st["checks"], fallbacks_in_run=st["fallbacks"],
                   nonfinite_checks_in_run=st["nonfinite"])
    elif mhd:
        inter = sum(field_interactions(c["config"], d.read("flags")) for c, d in zip(cases, doms))
        if batch is None:
            avg = eb_ms / max(eb_n, 1)
            kname = "k_update_e_b_exact" if a.field_mode == "bitwise" else "k_update_e_b_fast"
        else:
            avg = ms / a.steps
            kname = (f"k_batch_stream{'_rows' if all(c['config']['n_x'] % 16 == 0 and c['config']['n_x'] <= 96 for c in cases) else ''}"
                     f" + k_batch_field<{a.field_mode}> (whole step; FLOPs of its E/B phase)")
        tflops = inter * FLOP_PER_INTERACTION / (avg * 1e-3) / 1e12
        roofline = {"bound": "fp32", "achieved": tflops, "peak": tf.value, "unit": "TFLOP/s",
                    "frac": tflops / tf.value, "traffic": NCU_TRAFFIC.get((a.workload, kname)), "kernel": kname,
                    "flop_per_launch": inter * FLOP_PER_INTERACTION, "interactions_per_launch": inter,
                    "avg_launch_ms": avg, "peak_source": "measured FP32 FMA throughput (ion_probe_fp32_peak)"}
    if batch is not None:
        extra["autotuner"] = {"chosen": batch.chosen(), "trials": batch.tuning()}
    if sur is not None:
        sur.update(exact_fp32_step(cases[0], doms[0]))
        sur["speedup_vs_exact_fp32"] = sur["exact_fp32_ms_per_step"] / (ms_max / a.steps)
        extra["surrogate"] = sur

    # ---- end to end through the C ABI with host buffers ----------------------------
    e2e = None
    if not a.no_e2e:
        try:
            import torch
            lib = NAT.lib()
            jobs, h2d, d2h = [], 0, 0
            for case, d in zip(cases, doms):
                d.set_kernel_timing(False)
                ins = dict(case["fields"])
                if mhd:
                    ins["b_stat"] = d.read("b_stat")
                    ins["flags"] = d.read("flags")
                pin_in = {}
                for k, v in ins.items():
                    t = torch.empty(v.size, dtype=torch.from_numpy(v[:1]).dtype, pin_memory=True)
                    t.numpy()[:] = v
                    pin_in[k] = t
                pin_out = {}
                for k in ["rho", "u"] + (["q", "e_dyn", "b_dyn"] if mhd else []):
                    pin_out[k] = torch.empty(d.field_info(k)[1], dtype=torch.float32, pin_memory=True)
                jobs.append((d, pin_in, pin_out))
                h2d += sum(t.numel() * t.element_size() for t in pin_in.values())
                d2h += sum(t.numel() * t.element_size() for t in pin_out.values())
            dist.barrier()
            for d in doms:
                d.finish_queues(600000)
            t0 = time.perf_counter()
            for d, pin_in, _ in jobs:
                for k, t in pin_in.items():
                    NAT.check(lib.ion_lbm_write_field(d.handle, I.FIELDS[k], t.data_ptr(), t.numel() * t.element_size()))
                NAT.check(lib.ion_lbm_initialize(d.handle))
            if batch is None:
                NAT.check(lib.ion_lbm_run(doms[0].handle, a.steps))
            else:
                batch.run(a.steps)
                batch.finish(600000)
            for d, _, pin_out in jobs:
                for k, t in pin_out.items():
                    NAT.check(lib.ion_lbm_read_field(d.handle, I.FIELDS[k], t.data_ptr(), t.numel() * t.element_size()))
            dt = dist.max(time.perf_counter() - t0)
            path = ("ion_lbm_write_field, ion_lbm_initialize, " +
                    ("ion_lbm_run(K)" if batch is None else "ion_batch_run(K)") + ", ion_lbm_read_field")
            e2e = {"value": cells * a.steps * dist.world / dt / 1e6, "unit": "MLUPs/s",
                   "h2d_bytes_per_step": h2d / a.steps, "d2h_bytes_per_step": d2h / a.steps, "path": path}
        except Exception as ex:  # reported as missing rather than faked
            e2e = {"value": None, "unit": "MLUPs/s", "error": str(ex)[:200]}
    clk = clocks.stop()
    if (a.workload == "mhd128" and not a.no_surrogate_record and dist.rank == 0 and batch is None
            and a.field_mode != "surrogate"):
        try:
            extra["surrogate"] = surrogate_record(a)
        except Exception as ex:  # reported as missing rather than faked
            extra["surrogate"] = {"error": str(ex)[:300]}

    cpu = None
    if dist.rank == 0 and not a.no_cpu_baseline:
        ccases = cpu_sample_cases(a, cases)
        if ccases is cases:
            init = [({"b_stat": d.read("b_stat"), "flags": d.read("flags")} if mhd else {}) for d in doms]
        else:  # static field of the sample box, computed on the GPU (setup, untimed)
            init = []
            for c in ccases:
                d = I.Lbm(W.lbm_config(c))
                W.apply_case(d, c)
                init.append({"b_stat": d.read("b_stat"), "flags": d.read("flags")})
                d.close()
        mlups, sample, kind, cores, _, _ = cpu_run(ccases, 10 ** 6, a.ref_seconds, init)
        cpu = {"value": mlups, "unit": "MLUPs/s", "cores": cores, "kind": kind, "sample": sample}

    if dist.rank == 0:
        line = {"metric": metric, "value": value, "unit": "MLUPs/s", "n_gpus": dist.world, "steps": a.steps,
                "warmup": a.warmup, "ms_per_step": ms_max / a.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": dtype, "data": "synthetic (seeded, no dataset)",
                "config": workload_cfg, "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
                "gpu_launches": launches, "clocks": clk}
        if roof_stencil is not None and roofline is not roof_stencil:
            line["roofline_stencil"] = roof_stencil
        if share:
            line["kernel_ms_in_timed_region"] = share
        line.update(extra)
        print(json.dumps(line), flush=True)
    if batch is not None:
        batch.close()
    for d in doms:
        d.close()
    dist.close()


if __name__ == "__main__":
    main()
