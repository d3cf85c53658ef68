"""Storage precision against the float64 oracle (the accuracy half of the
FP16S/FP16C configuration): the GPU with FP32, FP16S and FP16C DDF storage
against the double-precision restatement of the same timestep on the same
seeded inputs.

Bars (max |diff| / max |fp64|): the Taylor-Green velocity after 200 steps
1e-5 (FP32), 2e-2 (FP16S, FP16C); the MHD box after two steps (the
reference's electron gas turns non-finite from the third): gas velocity
5e-5 (FP32), 2e-2 (FP16S, FP16C).  The charge Q and the E field are printed,
not bounded there: the reference starts the electron gas at density 0
(sim_kernels.cl:823-826), so its velocity j/rho_e divides by a rounding
residue and any difference in rounding -- FP32 against FP64 included --
changes Q = rho_q - rho_e at O(1).  On the finite-plasma start
(workloads.mhd_plasma) every field is bounded after 50 steps
(test_plasma_storage_accuracy_against_float64)."""
import numpy as np
import pytest

import oracle as O
from ionsolver_gb300 import workloads as W
from tests import _util as U

pytestmark = pytest.mark.gpu

BAR = {2: 1e-5, 0: 2e-2, 1: 2e-2}
NAME = {2: "FP32", 0: "FP16S", 1: "FP16C"}


def _f64(case):
    cfg = dict(case["config"], float_type=2)
    return O.OracleLbm(O.make_config(**cfg), "f64", O.cpu_count())


@pytest.mark.parametrize("ft", [2, 0, 1], ids=["FP32", "FP16S", "FP16C"])
def test_taylor_green_storage_accuracy(ft):
    case = W.taylor_green(n=64, amplitude=0.05, float_type=ft)
    g = U.run_gpu(case, 200)
    o = _f64(case)
    for name, arr in case["fields"].items():
        o.set_field(name, arr)
    o.initialize()
    o.run(200)
    eu = U.rel_err(g.read("u"), o.field("u"))
    er = U.rel_err(g.read("rho").astype(np.float64) - 1.0, o.field("rho") - 1.0)
    print(f"\naccuracy tgv64 200 steps {NAME[ft]}: u {eu:.3e} rho-1 {er:.3e}")
    assert eu < BAR[ft]
    assert er < 10 * BAR[ft]


@pytest.mark.parametrize("ft", [2, 0, 1], ids=["FP32", "FP16S", "FP16C"])
def test_mhd_storage_accuracy(ft):
    case = W.mhd_box(n=64, depth=4, magnet_r=8.0, magnet_t=4.0, float_type=ft, field_mode=0)
    g = U.setup_gpu(case)
    g.initialize()
    g.run(2)
    g.finish_queues(60000)
    o = _f64(case)
    for name, arr in case["fields"].items():
        o.set_field(name, arr)
    # geometry and static field from the GPU: the comparison is about the timestep
    o.set_field("flags", g.read("flags"))
    o.set_field("b_stat", g.read("b_stat"))
    o.initialize()
    o.run(2)
    out = {}
    n = 64 ** 3
    for name in ("u", "q", "e_dyn"):
        a = g.read(name)[: 3 * n if name != "q" else n].astype(np.float64)
        b = o.field(name)[: a.size]
        assert np.isfinite(a).all() and np.isfinite(b).all(), name
        if name == "e_dyn":
            a = a - g.read("e_stat").astype(np.float64)
            b = b - o.field("e_stat")[: a.size]
        out[name] = U.rel_err(a, b)
    print(f"\naccuracy mhd64 2 steps {NAME[ft]}: " + " ".join(f"{k} {v:.3e}" for k, v in out.items()))
    assert out["u"] < max(BAR[ft], 5e-5)


@pytest.fixture(scope="module")
def plasma64_f64():
    """The float64 oracle's run of the finite-plasma box (64^3, depth 4, 50 steps)."""
    case = W.mhd_plasma(n=64, depth=4, float_type=2, field_mode=0)
    o = U.setup_oracle(case, kind="f64")
    U.initialize_oracle(o, case)
    o.run(PLASMA_STEPS)
    return o


PLASMA_STEPS = 50
# max |diff| / max |fp64| after 50 steps of the finite-plasma box, about twice the
# measured values (GB300): FP32 rho-1 8.5e-4, u 2.4e-4, q 2.8e-2, E 1.2e-2, B 3.0e-6;
# FP16S 8.9e-4, 3.6e-4, 25, 19, 3.0e-6; FP16C 1.5e-3, 8.6e-4, 15, 18, 3.0e-6.
# The net charge q = rho_q - rho_e is the difference of two DDF-shifted lattice sums at
# rho ~ 0.01, and it decays to ~5e-5 by step 50: FP32 rounding of the two lattices is a
# few percent of it, and 16-bit storage (FP16S resolves ~3e-5 per DDF near -w_i) cannot
# resolve it at all, so with 16-bit storage q and the E field it drives are noise of
# the storage while the gas (rho, u) and B stay within the bars below.
PLASMA_BAR = {2: {"rho-1": 2e-3, "u": 5e-4, "q": 6e-2, "E": 3e-2, "B": 1e-5},
              0: {"rho-1": 2e-3, "u": 1e-3, "q": 50.0, "E": 40.0, "B": 1e-5},
              1: {"rho-1": 3e-3, "u": 2e-3, "q": 30.0, "E": 40.0, "B": 1e-5}}


@pytest.mark.parametrize("ft", [2, 0, 1], ids=["FP32", "FP16S", "FP16C"])
def test_plasma_storage_accuracy_against_float64(ft, plasma64_f64):
    """Configuration 2's accuracy half on a finite state: FP32, FP16S and FP16C
    storage against the float64 oracle, every compared field bounded."""
    o = plasma64_f64
    case = W.mhd_plasma(n=64, depth=4, float_type=ft, field_mode=0)
    g = U.run_gpu(case, PLASMA_STEPS)
    n = 64 ** 3
    got = {"rho-1": U.rel_err(g.read("rho").astype(np.float64) - 1.0, o.field("rho") - 1.0),
           "u": U.rel_err(g.read("u"), o.field("u")),
           "q": U.rel_err(g.read("q"), o.field("q")),
           "E": U.rel_err(g.read("e_dyn")[:3 * n], o.field("e_dyn")[:3 * n]),
           "B": U.rel_err(g.read("b_dyn"), o.field("b_dyn")[:3 * n])}
    print(f"\naccuracy plasma64 {PLASMA_STEPS} steps {NAME[ft]}: " + " ".join(f"{k} {v:.3e}" for k, v in got.items()))
    for k, v in got.items():
        assert v <= PLASMA_BAR[ft][k], (k, v)
