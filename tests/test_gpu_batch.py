"""Batched uneven domains (one persistent launch per step) against the same
domains stepped one at a time: bit-identical (NaN equals NaN).  Batches whose rows
are all whole 16-byte streams of at most 96 cells run the row-staged stencil
(k_batch_stream_rows), others the tiles of cells with global loads (k_batch_stream);
both are covered."""
import numpy as np
import pytest

import ionsolver_gb300 as I
from ionsolver_gb300 import workloads as W
from tests import _util as U

pytestmark = pytest.mark.gpu


def _cases_mhd(ft, fm):
    out = []
    for i, (n, r) in enumerate(((16, 4.0), (24, 5.0), (32, 6.0), (20, 4.0))):
        c = W.mhd_box(n=n, float_type=ft, depth=2, magnet_r=r, magnet_t=r / 2, field_mode=fm, seed_q=10 + i,
                      seed_u=20 + i)
        out.append(c)
    return out


@pytest.mark.parametrize("ft,fm", [(2, 0), (2, 1), (0, 1), (1, 1)], ids=["FP32-bitwise", "FP32-fast", "FP16S-fast",
                                                                       "FP16C-fast"])
def test_batch_equals_individual_mhd(ft, fm):
    cases = _cases_mhd(ft, fm)
    steps = 26
    solo = [U.run_gpu(c, steps) for c in cases]
    doms = [U.setup_gpu(c) for c in cases]
    for d in doms:
        d.initialize()
    b = I.Batch(doms)
    b.run(steps)
    b.finish(120000)
    assert len(b.tuning()) >= 2  # the autotuner tried several launch shapes
    for c, d, s in zip(cases, doms, solo):
        assert d.get_time_step() == s.get_time_step() == steps
        for name in U.field_names(c):
            ft_ = c["config"]["float_type"] if name in ("fi", "fqi", "ei") else None
            assert U.bit_diff_nan(d.read(name), s.read(name), ft_) == 0, name
    b.close()


def _cases_rows(ft, fm):
    """Domains whose rows are whole 16-byte streams of at most 96 cells: the batch runs
    its row-staged stencil; one domain uses TRT."""
    out = []
    for i, (shape, r) in enumerate((((16, 16, 16), 4.0), ((32, 24, 16), 5.0), ((48, 16, 12), 4.0), ((96, 16, 8), 3.0))):
        c = W.mhd_plasma(shape=shape, float_type=ft, depth=2, magnet_r=r, magnet_t=r / 2, field_mode=fm)
        if i == 2:
            c["config"]["relaxation_time"] = 1
        out.append(c)
    return out


@pytest.mark.parametrize("ft,fm", [(2, 0), (2, 1), (0, 1), (1, 1)], ids=["FP32-bitwise", "FP32-fast", "FP16S-fast",
                                                                       "FP16C-fast"])
def test_batch_row_staged_equals_individual_mhd(ft, fm):
    cases = _cases_rows(ft, fm)
    steps = 26
    solo = [U.run_gpu(c, steps) for c in cases]
    doms = [U.setup_gpu(c) for c in cases]
    for d in doms:
        d.initialize()
    b = I.Batch(doms)
    b.run(steps)
    b.finish(120000)
    for c, d, s in zip(cases, doms, solo):
        assert d.get_time_step() == s.get_time_step() == steps
        for name in U.field_names(c):
            ft_ = c["config"]["float_type"] if name in ("fi", "fqi", "ei") else None
            assert U.bit_diff_nan(d.read(name), s.read(name), ft_) == 0, name
    b.close()


def test_batch_row_staged_equals_individual_plain():
    cases = [W.taylor_green(shape=s, amplitude=0.05, relaxation_time=rt)
             for s, rt in (((16, 16, 16), 0), ((32, 24, 16), 1), ((96, 8, 12), 0))]
    steps = 30
    solo = [U.run_gpu(c, steps) for c in cases]
    doms = [U.setup_gpu(c) for c in cases]
    b = I.Batch(doms)
    b.run(steps)
    b.finish(120000)
    for d, s in zip(doms, solo):
        for name in ("fi", "rho", "u"):
            assert U.bit_diff(d.read(name), s.read(name)) == 0, name


def test_batch_equals_individual_plain():
    cases = [W.taylor_green(shape=s, amplitude=0.05) for s in ((16, 16, 16), (32, 24, 16), (40, 8, 12))]
    steps = 30
    solo = [U.run_gpu(c, steps) for c in cases]
    doms = [U.setup_gpu(c) for c in cases]
    b = I.Batch(doms)  # initialises the domains
    b.run(steps)
    b.finish(120000)
    for d, s in zip(doms, solo):
        for name in ("fi", "rho", "u"):
            assert U.bit_diff(d.read(name), s.read(name)) == 0, name


def test_batch_rejects_mixed_domains():
    a = U.setup_gpu(W.mhd_box(n=16, depth=2, magnet_r=4.0, magnet_t=2.0))
    b = U.setup_gpu(W.mhd_box(n=16, depth=2, magnet_r=4.0, magnet_t=2.0, float_type=0))
    with pytest.raises(I.IonError) as e:
        I.Batch([a, b])
    assert e.value.code == -2
