"""How much a field error moves the gas velocity (CPU, float64 oracle).

The learned far field is accepted while its sampled error stays within the check
tolerance (1% of the largest dynamic field, else the step falls back to the exact
sum). The velocity error of that step against the float64 oracle is then at most the
storage error (measured on the GPU against the same oracle: FP16S gas velocity 2.6e-4
after two MHD steps) plus what such a field error adds. This test bounds the second
part. It runs the two-ring box twice, the second time with its dynamic E and B
perturbed between the steps by 1% of their largest value (uniform noise). The gas feels
the field through the Lorentz force rho_q (E + u x B) and its Guo forcing
(sim_kernels.cl:660-662, 681-685, 716). The velocity moves by about 6e-8 of its largest
value per step, linearly in the perturbation.
"""
import numpy as np

import oracle as O
from ionsolver_gb300 import workloads as W
from tests import _util as U


def _run(case, n, eps, steps=2):
    o = U.setup_oracle(case, "f64", O.cpu_count())
    o.initialize()
    rng = np.random.default_rng(7)
    for s in range(steps):
        o.do_time_step()
        if eps and s + 1 < steps:
            for dyn, stat in (("e_dyn", "e_stat"), ("b_dyn", "b_stat")):
                d = o.field(dyn)[:3 * n]
                scale = np.max(np.abs(d - o.field(stat)[:3 * n]))
                d += eps * scale * rng.uniform(-1.0, 1.0, 3 * n)
    u = o.field("u")[:3 * n].copy()
    o.close()
    return u


def test_velocity_moves_little_under_a_one_percent_field_error():
    n = 64
    case = W.mhd_box(n=n, depth=4, float_type=2, field_mode=0, rings=True)
    cells = n ** 3
    u0 = _run(case, cells, 0.0)
    u1 = _run(case, cells, 1e-2)
    assert np.isfinite(u0).all() and np.isfinite(u1).all()
    rel = float(np.max(np.abs(u1 - u0)) / np.max(np.abs(u0)))
    print(f"\nvelocity change under a 1% field error, one step: {rel:.3e}")
    assert 0.0 < rel < 1e-5
