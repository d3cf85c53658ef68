#!/usr/bin/env python3
"""Benchmark of the IonSolver MHD-LBM timestep on GB300 (one JSON line on rank 0).

Workload (default ``mhd128``): 128^3 D3Q19 fluid + D3Q7 charge lattice,
FP32 storage, tau = 0.6, one-cell solid walls, charge U[-1e-3,1e-3] (seed 1),
velocity N(0,1e-3^2) (seed 2), an axially magnetised disk magnet (r 16,
t 8) on the z=1 face, exact LOD E/B update every step (LOD depth 4).  A
"step" is one timestep of the whole domain: stream_collide, LOD bin sums,
E/B update.  Metric: MLUPs/s = cells * steps / seconds / 1e6.

  value      : device time (CUDA events on the library's stream) of K steps
               with all inputs resident in HBM.
  e2e        : the same job through the C ABI with host buffers: upload of
               the inputs from pinned memory, initialize, K steps (CUDA
               graph), download of rho/u/Q/E/B, all inside the timed region.
  roofline   : the dominant kernel (the E/B update, FP32-bound) against the
               measured FP32 FMA peak; roofline_stencil: stream_collide
               against the measured HBM bandwidth (MEASURED_PEAKS.json).
  cpu_baseline: the reference's kernels compiled for the host (or the C
               restatement of them when the reference copy is absent), all
               host cores, on a bounded sample of the same workload.

``--impl reference`` runs only that CPU implementation and prints its line.
Multi-GPU (torchrun): replicas only -- every rank advances its own domain,
no data exchange; value = cells * steps * ranks / max-over-ranks time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

# Algorithmic bytes per lattice update (FP32 storage, D3Q19 + D3Q7 + electron gas):
#   fi 19 loads + 19 stores, ei 19+19, fqi 7+7 (4 B each) = 360; E,B dyn 24;
#   flags 1; Q 4; LOD velocity 12; rho,u 16 (update_fields)          -> 417
BYTES_PER_LUP_MHD_FP32 = 417
BYTES_PER_LUP_PLAIN_FP32 = 169  # 38 DDF accesses x 4 B + flags + rho,u
FLOP_PER_INTERACTION = 34       # E and B from one source: 34 FLOP + 1 sqrt


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--workload", default="mhd128", choices=["mhd128", "mhd256", "tgv64", "tgv256", "tgv384"])
    p.add_argument("--field-mode", default="fast", choices=["bitwise", "fast"])
    p.add_argument("--ref-seconds", type=float, default=20.0, help="CPU time budget of the reference/baseline sample")
    p.add_argument("--no-cpu-baseline", action="store_true")
    return p.parse_args()


def make_case(workload: str, field_mode: str):
    from ionsolver_gb300 import workloads as W
    fm = 0 if field_mode == "bitwise" else 1
    if workload.startswith("mhd"):
        n = int(workload[3:])
        case = W.mhd_box(n=n, field_mode=fm, magnet_r=16.0 * n / 128, magnet_t=8.0 * n / 128)
    else:
        n = int(workload[3:])
        case = W.taylor_green(n=n, amplitude=0.05)
        case["config"]["update_fields"] = 0
    return case


# ---------------------------------------------------------------------------
# distributed plumbing (replicas only)
# ---------------------------------------------------------------------------
class Dist:
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


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class Clocks:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = ROOT / "gpurun_out" / f"clocks_rank{index}.csv"

    def start(self):
        try:
            self.path.parent.mkdir(exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict | None:
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = max(smax, float(parts[2]))
            except ValueError:
                continue
            for name, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# CPU implementations (the reference's kernels on host cores, or the port)
# ---------------------------------------------------------------------------
def cpu_run(case, steps: int, budget_s: float, init_fields: dict | None):
    """Advances the case on the host cores; returns (MLUPs/s, sample text, kind, cores)."""
    import oracle as O
    from tests import _util as U
    cores = O.cpu_count()
    kind = "reference"
    try:
        if not O.reference_available():
            raise RuntimeError("no reference copy")
        o = O.OracleLbm(U.oracle_config(case), "ref", cores)
    except Exception:
        kind = "port"
        o = O.OracleLbm(U.oracle_config(case), "f32", cores)
    for name, arr in case["fields"].items():
        o.set_field(name, arr)
    for name, arr in (init_fields or {}).items():  # static field precomputed on the GPU (setup, untimed)
        o.set_field(name, arr)
    o.initialize()
    N = o.n
    done, t0 = 0, time.perf_counter()
    while done < steps:
        o.do_time_step()
        done += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    mlups = N * done / dt / 1e6
    sample = f"{done} full timestep(s) of the {case['config']['n_x']}^3 case after initialize, {dt:.1f} s wall"
    return mlups, sample, kind, cores


# ---------------------------------------------------------------------------
def main():
    a = parse()
    dist = Dist()
    case = make_case(a.workload, a.field_mode)
    c = case["config"]
    N = c["n_x"] * c["n_y"] * c["n_z"]
    mhd = bool(c.get("ext_magneto_hydro"))
    workload_cfg = {"workload": a.workload, "cells": N, "size": [c["n_x"], c["n_y"], c["n_z"]],
                    "velocity_set": "D3Q19", "float_type": "FP32", "relaxation": "SRT", "tau": 0.6,
                    "mhd": mhd, "lod_depth": c.get("mhd_lod_depth") if mhd else None,
                    "field_mode": a.field_mode if mhd else None,
                    "l2": "working set (%.0f MB) larger than L2 (126 MB)" % (
                        N * (BYTES_PER_LUP_MHD_FP32 if mhd else BYTES_PER_LUP_PLAIN_FP32) / 1e6),
                    "parallelism": f"replicas x{dist.world}"}
    metric = "D3Q19-MHD MLUPs/s" if mhd else "D3Q19 MLUPs/s"

    if a.impl == "reference":
        if dist.rank != 0:
            dist.close()
            return
        mlups, sample, kind, cores = cpu_run(case, max(a.steps, 1), a.ref_seconds, None)
        line = {"metric": metric, "value": mlups, "unit": "MLUPs/s", "n_gpus": a.gpus, "steps": a.steps,
                "warmup": a.warmup, "ms_per_step": N / mlups / 1e3, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": workload_cfg,
                "impl": "reference",
                "cpu_baseline": {"value": mlups, "unit": "MLUPs/s", "cores": cores, "kind": kind, "sample": sample},
                "e2e": {"value": mlups, "unit": "MLUPs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        dist.close()
        return

    import ionsolver_gb300 as I
    from ionsolver_gb300 import _native as NAT
    from ionsolver_gb300 import workloads as W
    NAT.check(NAT.lib().ion_select_device(dist.local))

    lbm = I.Lbm(W.lbm_config(case))
    W.apply_case(lbm, case)
    lbm.initialize()
    lbm.set_kernel_timing(True)
    for _ in range(a.warmup):
        lbm.do_time_step()
    lbm.finish_queues(600000)
    lbm.reset_kernel_time()

    clocks = Clocks(dist.local)
    launches0 = I.kernel_launch_count()
    dist.barrier()
    lbm.finish_queues(600000)
    clocks.start()
    lbm.record_event(0)
    for _ in range(a.steps):
        lbm.do_time_step()
    lbm.record_event(1)
    ms = lbm.elapsed_ms(0, 1)
    lbm.finish_queues(600000)
    clk = clocks.stop()
    launches = I.kernel_launch_count() - launches0
    dist.barrier()
    ms_max = dist.max(ms)
    value = N * a.steps * dist.world / (ms_max * 1e-3) / 1e6

    sc_ms, sc_n = lbm.kernel_time(0)
    eb_ms, eb_n = lbm.kernel_time(1)
    bins_ms, bins_n = lbm.kernel_time(2)
    flags = lbm.read("flags")
    fluid = int(((flags & 0x1F) != 0x01).sum())

    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except Exception:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    hbm_src = "measured" if "hbm_gbs" in peaks else "fallback"
    bpl = BYTES_PER_LUP_MHD_FP32 if mhd else BYTES_PER_LUP_PLAIN_FP32
    sc_avg = sc_ms / max(sc_n, 1)
    stencil_gbs = N * bpl / (sc_avg * 1e-3) / 1e9
    roof_stencil = {"bound": "hbm", "achieved": stencil_gbs, "peak": hbm_peak, "unit": "GB/s",
                    "frac": stencil_gbs / hbm_peak, "traffic": None, "kernel": "k_stream_collide",
                    "bytes_per_lup": bpl, "peak_source": hbm_src, "avg_launch_ms": sc_avg}
    roofline = roof_stencil
    if mhd:
        import ctypes as C
        tf = C.c_double()
        NAT.check(NAT.lib().ion_probe_fp32_peak(C.byref(tf)))
        # sources per fluid cell: the depth-4 bins [585, 4096) minus the cell's own bin when it is among them
        nd = 1 << c["mhd_lod_depth"]
        n_own = 1 + sum(8 ** (i + 1) for i in range(c["mhd_lod_depth"]))
        first = n_own - nd ** 3
        bs = c["n_x"] // nd
        z_first = first // (nd * nd)  # bins below `first` are whole z-layers plus part of one
        own_in = fluid - sum(1 for _ in range(0))  # refined below
        fl3 = ((flags & 0x1F) != 0x01).reshape(c["n_z"], c["n_y"], c["n_x"])
        zb = np.arange(c["n_z"]) // bs
        yb = np.arange(c["n_y"]) // bs
        xb = np.arange(c["n_x"]) // bs
        own = xb[None, None, :] + (yb[None, :, None] + zb[:, None, None] * nd) * nd
        own_in = int((fl3 & (own >= first)).sum())
        interactions = fluid * (nd ** 3 - first) - own_in
        eb_avg = eb_ms / max(eb_n, 1)
        tflops = interactions * FLOP_PER_INTERACTION / (eb_avg * 1e-3) / 1e12
        roofline = {"bound": "fp32", "achieved": tflops, "peak": tf.value, "unit": "TFLOP/s",
                    "frac": tflops / tf.value, "traffic": None, "kernel": "k_update_e_b<%s>" % a.field_mode,
                    "flop_per_launch": interactions * FLOP_PER_INTERACTION, "avg_launch_ms": eb_avg,
                    "peak_source": "measured FP32 FMA probe (ion_probe_fp32_peak)", "z_first_layer": z_first}
        share = {"update_e_b": eb_ms, "stream_collide": sc_ms, "lod_bins": bins_ms}
    else:
        share = {"stream_collide": sc_ms}

    # ---- end to end through the C ABI with host buffers -----------------------------
    lbm.set_kernel_timing(False)
    e2e = None
    try:
        import torch
        ins = {k: v for k, v in case["fields"].items()}
        if mhd:
            ins["b_stat"] = lbm.read("b_stat")
            ins["flags"] = flags
        pinned = {}
        for k, v in ins.items():
            t = torch.empty(v.size, dtype=torch.from_numpy(v[:1]).dtype, pin_memory=True)
            t.numpy()[:] = v
            pinned[k] = t
        outs = ["rho", "u"] + (["q", "e_dyn", "b_dyn"] if mhd else [])
        out_pinned = {}
        for k in outs:
            eb, cnt = lbm.field_info(k)
            out_pinned[k] = torch.empty(cnt, dtype=torch.uint8 if k == "flags" else torch.float32, pin_memory=True)
        lib = NAT.lib()
        h = lbm.handle
        e2e_lbm = lbm
        h2d = sum(t.numel() * t.element_size() for t in pinned.values())
        d2h = sum(t.numel() * t.element_size() for t in out_pinned.values())
        dist.barrier()
        e2e_lbm.finish_queues(600000)
        t0 = time.perf_counter()
        for k, t in pinned.items():
            NAT.check(lib.ion_lbm_write_field(h, I.FIELDS[k], t.data_ptr(), t.numel() * t.element_size()))
        NAT.check(lib.ion_lbm_initialize(h))
        NAT.check(lib.ion_lbm_run(h, a.steps))
        for k, t in out_pinned.items():
            NAT.check(lib.ion_lbm_read_field(h, I.FIELDS[k], t.data_ptr(), t.numel() * t.element_size()))
        dt = time.perf_counter() - t0
        dt = dist.max(dt)
        e2e = {"value": N * a.steps * dist.world / dt / 1e6, "unit": "MLUPs/s",
               "h2d_bytes_per_step": h2d / a.steps, "d2h_bytes_per_step": d2h / a.steps,
               "path": "ion_lbm_write_field x%d, ion_lbm_initialize, ion_lbm_run(%d), ion_lbm_read_field x%d"
                       % (len(pinned), a.steps, len(out_pinned))}
    except Exception as ex:  # e2e is reported as missing rather than faked
        e2e = {"value": None, "unit": "MLUPs/s", "error": str(ex)[:200]}

    cpu = None
    if dist.rank == 0 and not a.no_cpu_baseline:
        init = {"b_stat": lbm.read("b_stat"), "flags": flags} if mhd else None
        mlups, sample, kind, cores = cpu_run(case, 1000, a.ref_seconds, init)
        cpu = {"value": mlups, "unit": "MLUPs/s", "cores": cores, "kind": kind, "sample": sample}

    if dist.rank == 0:
        line = {"metric": metric, "value": value, "unit": "MLUPs/s", "n_gpus": dist.world, "steps": a.steps,
                "warmup": a.warmup, "ms_per_step": ms_max / a.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded, no dataset)",
                "config": workload_cfg, "roofline": roofline, "roofline_stencil": roof_stencil,
                "kernel_ms_in_timed_region": share, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches,
                "clocks": clk}
        print(json.dumps(line), flush=True)
    lbm.close()
    dist.close()


if __name__ == "__main__":
    main()
