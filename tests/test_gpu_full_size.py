"""The row-staged stencil at full size, against the global-load stencil.

The single-domain step runs the row-staged stream_collide (`k_sc_rows_ws`: rows staged
and written back through shared memory, a fixed row stride of 128, 256 or 384
elements).  The batched step runs the same per-cell code with loads and stores
straight from global memory (`k_batch_stream`).  Both are pinned to the oracle on
small boxes (test_gpu_parity.py, test_gpu_batch.py).  Here they meet at sizes the
oracle cannot step in a test: configuration 2's 256^3 finite-plasma MHD box in FP16S
and FP16C storage (rows of 256 cells), and a 384 x 96 x 96 box (rows of 384 cells, as
configuration 4's 384^3).  Each is stepped alone and as one domain of a two-domain
batch (with a small second domain); every field is bit-identical after 3 steps.
"""
import pytest

import ionsolver_gb300 as I
from ionsolver_gb300 import workloads as W
from tests import _util as U

pytestmark = pytest.mark.gpu

STEPS = 3


@pytest.mark.parametrize("ft,shape", [(0, (256, 256, 256)), (1, (256, 256, 256)), (0, (384, 96, 96)),
                                      (2, (384, 96, 96))],
                         ids=["FP16S-256c", "FP16C-256c", "FP16S-384x96x96", "FP32-384x96x96"])
def test_row_staged_equals_global_loads_at_full_size(ft, shape):
    case = W.mhd_plasma(shape=shape, float_type=ft, depth=4, field_mode=1, magnet_r=16.0, magnet_t=8.0)
    small = W.mhd_plasma(n=32, float_type=ft, depth=4, field_mode=1, magnet_r=6.0, magnet_t=4.0)
    solo = U.run_gpu(case, STEPS)
    doms = [U.setup_gpu(case), U.setup_gpu(small)]
    for d in doms:
        d.initialize()
    b = I.Batch(doms)
    b.run(STEPS)
    b.finish(600000)
    big = doms[0]
    assert big.get_time_step() == solo.get_time_step() == STEPS
    for name in U.field_names(case):
        ft_ = ft if name in ("fi", "fqi", "ei") else None
        assert U.bit_diff_nan(big.read(name), solo.read(name), ft_) == 0, name
    b.close()
