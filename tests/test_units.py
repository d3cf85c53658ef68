"""Kernel constants from Units (IonSolver src/lbm/units.rs:149-197,
src/lbm/domain.rs:808-848): the library, the oracle and an independent
numpy float32 restatement agree bit for bit."""
import numpy as np
import pytest

import oracle as O
import ionsolver_gb300 as I

f32 = np.float32
UNITS = [dict(m=1.0, kg=1.0, s=1.0, a=1.0, k=1.0, prop=0), dict(m=1.0, kg=1.0, s=1.0, a=1e-6, k=1.0, prop=0),
         dict(m=0.0078125, kg=1.8692e-6, s=7.8125e-4, a=1e-7, k=1.0, prop=5)]


def numpy_constants(u, nu):
    a, s, kg, m = f32(u["a"]), f32(u["s"]), f32(u["kg"]), f32(u["m"])
    pi = f32(np.pi)
    eps0 = f32(8.8541878128e-12) / ((a * a * ((s * s) * s * s)) / (kg * ((m * m) * m)))
    eps0 = f32(8.8541878128e-12) / ((f32(a * a) * f32(f32(f32(s * s) * s) * s)) / (kg * f32(f32(m * m) * m)))
    ke = f32(1.0) / (f32(f32(4.0) * pi) * eps0)
    mu0 = f32(1.256637062e-6) / (f32(kg * m) / f32(f32(a * a) * f32(s * s)))
    return {"w": f32(1.0) / (f32(f32(3.0) * f32(nu)) + f32(0.5)), "ke": ke, "mu_0": mu0,
            "kmu": mu0 / f32(f32(4.0) * pi), "kkge": f32(9.1093837139e-31 / -1.602176634e-19) / f32(kg / f32(a * s)),
            "wq": f32(0.4)}


@pytest.mark.parametrize("u", UNITS)
def test_constants_agree(u):
    nu = float(f32(1.0) / f32(30.0))
    cfg = I.LbmConfig(velocity_set=2, nu=nu, units=I.Units(**u))
    lib = cfg.constants()
    orc = O.constants(O.make_config(velocity_set=2, nu=nu, units=u))
    for k in lib:
        assert f32(lib[k]).view(np.uint32) == f32(getattr(orc, k)).view(np.uint32), k
    npc = numpy_constants(u, nu)
    for k, v in npc.items():
        assert f32(lib[k]).view(np.uint32) == f32(v).view(np.uint32), k


def test_units_set_and_conversions():
    un = I.Units()
    un.set(128.0, 1.0, 1.0, 1.0, 1.0, 0.1, 1.0, 1.2250, 0.0000000001, 1.0)
    m = f32(0.1) / f32(128.0)
    assert f32(un.m) == m
    assert f32(un.magnetization_si_lu(1000.0)) == f32(1000.0) / (f32(un.a) / f32(un.m))
    assert f32(un.len_si_lu(0.05)) == f32(0.05) / f32(un.m)
