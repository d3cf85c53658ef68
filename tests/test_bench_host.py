"""Host-side logic of bench.py: which stencil kernel a workload runs, the
algorithmic bytes per lattice update, workload-name parsing, and the source-term
counts the field rooflines divide by (checked against a direct count), and the
clock record of a line."""
import types

import numpy as np

import bench
from ionsolver_gb300 import workloads as W


def test_stencil_kernel_names():
    cfg = dict(velocity_set=2, n_x=128)
    assert bench.stencil_kernel(cfg) == "k_sc_rows_ws"
    assert bench.stencil_kernel(dict(cfg, n_x=384)) == "k_sc_rows_ws"
    assert bench.stencil_kernel(dict(cfg, n_x=400)) == "k_sc_rows"
    assert bench.stencil_kernel(dict(cfg, n_x=24)) == "k_stream_collide"
    assert bench.stencil_kernel(dict(cfg, ext_subgrid_ecr=1)) == "k_stream_collide"
    assert bench.stencil_kernel(dict(cfg, velocity_set=1)) == "k_stream_collide"


def test_bytes_per_lattice_update():
    assert bench.bytes_per_lup(dict(float_type=2)) == 153
    assert bench.bytes_per_lup(dict(float_type=2, update_fields=1)) == 169
    mhd = dict(float_type=2, update_fields=1, ext_magneto_hydro=1, mhd_lod_depth=4)
    assert bench.bytes_per_lup(mhd) == 417
    assert bench.bytes_per_lup(dict(mhd, float_type=0)) == 237


def test_workload_names(monkeypatch):
    seen = []
    monkeypatch.setattr(W, "mhd_box", lambda **kw: seen.append(kw) or {"config": {}})
    a = types.SimpleNamespace(field_mode="surrogate", float_type="FP16S", workload="rings192d3", start="reference")
    bench.make_cases(a)
    a.workload = "rings384"
    bench.make_cases(a)
    assert (seen[0]["n"], seen[0]["depth"], seen[0]["rings"]) == (192, 3, True)
    assert (seen[1]["n"], seen[1]["depth"]) == (384, 4)


def test_update_fields_option():
    """--update-fields on/off overrides the workloads' default (on for MHD, off for TGV)."""
    a = types.SimpleNamespace(field_mode="fast", float_type="FP32", workload="mhd64", start="plasma")
    assert bench.make_cases(a)[0]["config"]["update_fields"] == 1
    a.update_fields = "off"
    c = bench.make_cases(a)[0]["config"]
    assert c["update_fields"] == 0 and bench.bytes_per_lup(c) == bench.bytes_per_lup(dict(c, update_fields=1)) - 16
    a = types.SimpleNamespace(field_mode="fast", float_type="FP32", workload="tgv64", start="plasma", update_fields="on")
    assert bench.make_cases(a)[0]["config"]["update_fields"] == 1


def test_plasma_start_cases():
    """--start plasma: the same geometry and seeds, plasma units, the electron background."""
    a = types.SimpleNamespace(field_mode="fast", float_type="FP32", workload="mhd64", start="plasma")
    c = bench.make_cases(a)[0]
    r = bench.make_cases(types.SimpleNamespace(**dict(vars(a), start="reference")))[0]
    assert c["electron_background"] == W.PLASMA_RHO_E0 and "electron_background" not in r
    assert c["config"]["units"] == W.PLASMA_UNITS
    for k in ("q", "u", "flags"):
        assert np.array_equal(c["fields"][k], r["fields"][k])
    assert np.array_equal(c["meshes"][0][0], r["meshes"][0][0])
    assert c["meshes"][0][4] == (0.0, 0.0, W.PLASMA_MAGNETIZATION_SI)


def test_reference_arm_reports_the_steps_it_ran(monkeypatch):
    """A CPU sample that runs out of budget reports the steps it timed, not the steps asked for."""
    case = W.mhd_plasma(n=16, depth=2, magnet_r=4.0, magnet_t=3.0)
    mlups, sample, kind, cores, timed, warm = bench.cpu_run([case], 1000, 0.0, None, warmup=1)
    assert timed == 1 and warm == 1 and mlups > 0 and "1 full timestep" in sample
    mlups, sample, kind, cores, timed, warm = bench.cpu_run([case], 3, 1e9, None)
    assert timed == 3 and warm == 0


def _bins(cfg):
    D = int(cfg["mhd_lod_depth"])
    nd = 1 << D
    n_own = 1 + sum(8 ** (i + 1) for i in range(D))
    return nd, n_own - nd ** 3


def test_source_term_counts_against_a_direct_count():
    case = W.mhd_box(n=32, depth=2, magnet_r=5.0, magnet_t=3.0)
    cfg, flags = case["config"], case["fields"]["flags"].copy()
    flags.reshape(32, 32, 32)[10:14, 8:20, 3:9] = 0x01  # an extra solid block
    nd, first = _bins(cfg)
    bs = 32 // nd
    far = near = 0
    for n in np.flatnonzero((flags & 0x1F) != 0x01):
        x, y, z = n % 32, (n // 32) % 32, n // 1024
        own = x // bs + (y // bs + z // bs * nd) * nd
        for d in range(first, nd ** 3):
            if d == own:
                continue
            far += 1
            if max(abs(d % nd - x // bs), abs(d // nd % nd - y // bs), abs(d // (nd * nd) - z // bs)) <= 1:
                near += 1
    assert bench.field_interactions(cfg, flags) == far
    assert bench.near_interactions(cfg, flags, 1) == near


def _samples(rows):
    return "".join(f"2026/01/01 00:00:{s:06.3f}, {mhz}, 2070, 900.0, {hw}, Not Active, Not Active, {cap}\n"
                   for s, mhz, hw, cap in rows)


def test_clock_summary_inside_the_timed_window(tmp_path):
    """The clock record of a line: median SM clock and the throttle reasons seen in
    the samples between the two marks (all samples when none fall inside)."""
    import datetime as dt

    class Done:  # stands in for the nvidia-smi process
        def terminate(self): pass
        def wait(self, t): pass

    c = bench.Clocks(0, str(tmp_path))
    c.path.write_text(_samples([(1.0, 1200, "Active", "Not Active"), (2.0, 2070, "Not Active", "Active"),
                                (2.5, 2060, "Not Active", "Not Active"), (4.0, 900, "Active", "Not Active")]))
    c.proc, c.f = Done(), open(tmp_path / "unused", "w")
    c.t0, c.t1 = dt.datetime(2026, 1, 1, 0, 0, 1, 500000), dt.datetime(2026, 1, 1, 0, 0, 3)
    r = c.stop()
    assert (r["sm_mhz"], r["sm_max_mhz"], r["reasons"], r["samples"]) == (2065.0, 2070.0, ["sw_power_cap"], 2)
    assert c.path.exists()  # kept: --clocks-dir was given


def test_clock_samples_not_kept_by_default():
    """Without --clocks-dir the raw samples live in a temporary file that is removed,
    also when nvidia-smi cannot be started (no record at all, as on a host without GPU)."""
    c = bench.Clocks(0)
    c.start()
    if c.proc is None:
        assert c.stop() is None
    else:
        c.mark("t0"); c.mark("t1"); c.stop()
    assert not c.path.exists()
