"""The MHD step on a finite state, and the FAST field per cell.

The reference's electron gas starts at density 0 and its velocity j/rho_e
turns 0/0 within a few steps (sim_kernels.cl:230-232, 823), after which every
MHD field is NaN.  ``workloads.mhd_plasma`` starts the electron gas at a
background density instead (``ion_lbm_set_electron_background``, applied
identically by the oracle), in units where the state stays finite.  On it:

* BITWISE: 100 steps at 32^3, LOD depth 4, every field bit-identical to the
  oracle in FP32, FP16S and FP16C storage, and every float field finite;
* conservation: the GPU's FP64 reductions of mass and charge equal float64
  sums of the oracle's arrays; mass is conserved to 1e-8 relative; the total
  charge moves only by the reference's own float32 bias (below);
* FAST: E and B of ``k_update_e_b_fast`` against BITWISE on the same sources,
  per cell, at config 1's 128^3 state after one step (with and without the
  magnet, the latter for B's dynamic part) and on the finite 32^3 trajectory
  after 100 steps.
"""
import numpy as np
import pytest

import ionsolver_gb300 as I
import oracle as O
from ionsolver_gb300 import workloads as W
from tests import _util as U

pytestmark = pytest.mark.gpu

# Per-cell bound of the FAST field against BITWISE (the target: <= 1e-4 in FP32),
# vector norms per cell: |dF_cell| / max(|F_cell|, FLOOR * max_cells |F_cell|).  The
# floor keeps cells where the sum of thousands of +-q/r^2 terms nearly cancels from
# dividing by a residue.  F is E_dyn and B_dyn, the fields the next step uses; their
# dynamic parts KE e and KMU b are compared too, where a float can resolve them (with
# a magnet B_stat dwarfs KMU b by ~1e7 in these units, so B's dynamic part is checked
# on magnet-free boxes).
FAST_CELL_BOUND = 1e-4
FAST_FLOOR = 1e-2


def _decoded_sum(o, name, ft):
    a = o.field(name)
    if a.dtype == np.float32:
        return float(np.sum(a.astype(np.float64)))
    lib = O.oracle_lib("f32")
    dec = lib.orc_fp16s_decode if ft == 0 else lib.orc_fp16c_decode
    table = np.array([dec(i) for i in range(65536)], np.float64)
    return float(np.sum(table[a]))


def _finite_fields(g, case):
    bad = {}
    for n in U.field_names(case):
        a = g.read(n)
        if a.dtype == np.float32 and not np.isfinite(a).all():
            bad[n] = int((~np.isfinite(a)).sum())
    return bad


@pytest.mark.parametrize("ft", [2, 0, 1], ids=["FP32", "FP16S", "FP16C"])
def test_plasma_bitwise_100_steps_finite_and_conserved(ft):
    case = W.mhd_plasma(n=32, float_type=ft, depth=4, field_mode=0)
    names = U.field_names(case)
    n = 32 ** 3
    g = U.setup_gpu(case)
    g.initialize()
    o = U.setup_oracle(case, canonical_nan=True)
    U.initialize_oracle(o, case)
    m0, q0 = g.mass_charge()
    for _ in range(2):
        g.run(50)
        g.finish_queues(120000)
        o.run(50)
        diff = U.compare_bitwise(g, o, names)
        assert all(v == 0 for v in diff.values()), (g.get_time_step(), diff)
        assert _finite_fields(g, case) == {}, g.get_time_step()
        # the FP64 reductions against float64 sums of the oracle's arrays
        mass, charge = g.mass_charge()
        m_ref = _decoded_sum(o, "fi", ft) + n
        q_ref = (_decoded_sum(o, "fqi", ft) + n) - (_decoded_sum(o, "ei", ft) + n)
        assert abs(mass - m_ref) <= 1e-12 * m_ref
        assert abs(charge - q_ref) <= 1e-12 * (_decoded_sum(o, "fqi", ft) + n)
    assert g.get_time_step() == 100
    m1, q1 = g.mass_charge()
    assert abs(m1 - m0) <= 1e-8 * m0, (m0, m1)
    # Charge: the reference's own float32 arithmetic moves it.  Its charge collision
    # is fma(1 - DEF_WQ, q, DEF_WQ * qeq) and (1 - 0.4f) + 0.4f != 1 in float32, so each
    # step scales the shifted DDF sum (about -N at rho ~ 0.01) by 1 + O(3e-8); the
    # electron gas has the same bias through (1 - w) + w.  Measured over these 100
    # steps: 4.2e-3 (FP32), 2.47 (FP16S), 2.63 (FP16C; 16-bit storage rounds every
    # DDF of both lattices each step) against a total ion charge of ~326; the float64
    # oracle conserves both lattices to 1e-9 (tests/test_oracle_physics.py).
    ion_total = _decoded_sum(o, "fqi", ft) + n
    bound = 2e-5 if ft == 2 else 1.5e-2
    assert abs(q1 - q0) <= bound * ion_total, (q0, q1, ion_total)


def _vec(lbm, name, n, minus=None):
    v = lbm.read(name)[:3 * n].astype(np.float64)
    if minus is not None:
        v = v - lbm.read(minus).astype(np.float64)
    return v.reshape(3, n)


def _cell_error(a, b):
    """max over cells of |a - b| / max(|b|, FAST_FLOOR max|b|), and max|a - b| / max|b|."""
    nb = np.sqrt((b * b).sum(0))
    d = np.sqrt(((a - b) ** 2).sum(0))
    if nb.max() == 0:
        return float(d.max()), float(d.max())
    return float((d / np.maximum(nb, FAST_FLOOR * nb.max())).max()), float(d.max() / nb.max())


def _field_errors(fast, exact, n, dynamic_b):
    out = {"E_dyn": _cell_error(_vec(fast, "e_dyn", n), _vec(exact, "e_dyn", n)),
           "B_dyn": _cell_error(_vec(fast, "b_dyn", n), _vec(exact, "b_dyn", n)),
           "KE e": _cell_error(_vec(fast, "e_dyn", n, "e_stat"), _vec(exact, "e_dyn", n, "e_stat"))}
    if dynamic_b:
        out["KMU b"] = _cell_error(_vec(fast, "b_dyn", n, "b_stat"), _vec(exact, "b_dyn", n, "b_stat"))
    return out


@pytest.mark.parametrize("magnet", [True, False], ids=["disk-magnet", "no-magnet"])
def test_fast_field_per_cell_config1_128_step1(magnet):
    """Config 1's state (128^3, reference start, depth 4) after one step: two
    handles from the same inputs, one BITWISE and one FAST, so the sources of the
    field are identical and only the field arithmetic differs."""
    n = 128 ** 3
    res = [U.run_gpu(W.mhd_box(n=128, depth=4, field_mode=mode, magnet=magnet), 1) for mode in (0, 1)]
    for name in ("fi", "fqi", "ei", "q", "qu_lod"):  # identical sources
        assert U.bit_diff(res[0].read(name), res[1].read(name)) == 0, name
    err = _field_errors(res[1], res[0], n, dynamic_b=not magnet)
    print("FAST vs BITWISE per cell (max, normwise), 128^3 step 1:", err)
    for k, (cell, norm) in err.items():
        assert cell <= FAST_CELL_BOUND, (k, cell, norm)


def test_fast_field_per_cell_plasma32_step100(tmp_path):
    """The finite 32^3 trajectory: 99 BITWISE steps, then the 100th step from
    the same checkpoint once BITWISE and once FAST; per-cell error of the field."""
    case = W.mhd_plasma(n=32, depth=4, field_mode=0)
    n = 32 ** 3
    g = U.run_gpu(case, 99)
    p = tmp_path / "s99.ion"
    g.checkpoint(p)
    f = I.Lbm.restore(p)
    f.set_field_mode(1)
    g.do_time_step()
    f.do_time_step()
    g.finish_queues(60000)
    f.finish_queues(60000)
    for name in ("fi", "fqi", "ei", "q", "qu_lod"):  # identical sources
        assert U.bit_diff(g.read(name), f.read(name)) == 0, name
    err = _field_errors(f, g, n, dynamic_b=False)
    print("FAST vs BITWISE per cell (max, normwise), plasma 32^3 step 100:", err)
    for k, (cell, norm) in err.items():
        assert cell <= FAST_CELL_BOUND, (k, cell, norm)


def test_config0_tgv64_1000_steps_bitwise():
    """Config 0 in full: 64^3 periodic Taylor-Green, FP32 SRT, tau 0.6, 1000 steps."""
    case = W.taylor_green(n=64, amplitude=0.05)
    g = U.run_gpu(case, 1000)
    o = U.run_oracle(case, 1000, canonical_nan=True)
    assert U.compare_bitwise(g, o, ["fi", "rho", "u"]) == {"fi": 0, "rho": 0, "u": 0}


def test_config1_mhd128_bitwise_two_steps():
    """Config 1's size: 128^3 MHD, depth 4, disk magnet r 16 t 8, BITWISE field,
    two steps (before the reference start's NaN onset), every field bit-identical."""
    case = W.mhd_box(n=128, depth=4, field_mode=0)
    g = U.run_gpu(case, 2)
    o = U.run_oracle(case, 2, canonical_nan=True)
    names = U.field_names(case)
    diff = U.compare_bitwise(g, o, names)
    assert all(v == 0 for v in diff.values()), diff
    assert _finite_fields(g, case) == {}


def test_plasma128_bitwise_two_steps():
    """The finite-plasma start at config 1's size (128^3): two BITWISE steps
    bit-identical to the oracle."""
    case = W.mhd_plasma(n=128, depth=4, field_mode=0)
    g = U.run_gpu(case, 2)
    o = U.run_oracle(case, 2, canonical_nan=True)
    diff = U.compare_bitwise(g, o, U.field_names(case))
    assert all(v == 0 for v in diff.values()), diff
