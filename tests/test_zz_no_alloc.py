"""ion_ddf_sum_f64_noalloc: the FP64 DDF sum for callers that cannot allocate
device memory (a host whose device memory is fully reserved by its own pool
allocator, or a stepping loop that must not take cudaFree's implicit
synchronisation).  Called through the C ABI on device buffers; checked against
ion_lbm_mass_charge, the entry point that runs the same sum with scratch
allocated by the handle, on two calls in a row."""
import ctypes as C

import numpy as np
import pytest

import ionsolver_gb300 as I
from ionsolver_gb300 import _native as N
from ionsolver_gb300 import workloads as W
from tests import _util as U

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _noalloc_sum(lbm, d_out) -> float:
    ptr, nbytes = lbm.device_ptr("fi")
    eb, count = lbm.field_info("fi")
    stream = C.c_void_p()
    N.check(N.lib().ion_lbm_stream(lbm.handle, C.byref(stream)))
    N.check(N.lib().ion_ddf_sum_f64_noalloc(C.c_void_p(ptr), int(lbm.config.float_type), count,
                                            C.c_void_p(d_out.data_ptr()), stream))
    lbm.finish_queues(60000)
    return float(d_out.item())


@pytest.mark.parametrize("ft", [2, 0, 1], ids=["FP32", "FP16S", "FP16C"])
def test_noalloc_sum_matches_mass_charge_on_two_calls(ft):
    case = W.taylor_green(shape=(48, 40, 32), amplitude=0.05, float_type=ft)
    case["fields"]["flags"] = W.shell_flags(48, 40, 32)
    lbm = U.setup_gpu(case)
    lbm.initialize()
    d_out = torch.zeros(1, dtype=torch.float64, device="cuda")
    n = lbm.n
    for steps in (10, 7):  # two calls in a row, on different states
        lbm.run(steps)
        lbm.finish_queues(60000)
        mass, _ = lbm.mass_charge()
        got = _noalloc_sum(lbm, d_out) + n
        assert abs(got - mass) <= 1e-12 * abs(mass), (got, mass)
    lbm.close()


def test_noalloc_rejects_oversized_and_null():
    lib = N.lib()
    d_out = torch.zeros(1, dtype=torch.float64, device="cuda")
    too_many = int(N_MAX) + 1
    rc = lib.ion_ddf_sum_f64_noalloc(C.c_void_p(d_out.data_ptr()), 2, too_many, C.c_void_p(d_out.data_ptr()), None)
    assert rc == -1 and b"ION_NOALLOC_MAX_VALUES" in lib.ion_last_error()
    assert lib.ion_ddf_sum_f64_noalloc(None, 2, 10, C.c_void_p(d_out.data_ptr()), None) == -1


N_MAX = 268435456
