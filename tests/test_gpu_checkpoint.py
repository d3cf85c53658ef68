"""Full checkpoint (ion_lbm_checkpoint / ion_lbm_restore): a restored handle
continues bit for bit -- every field after M further steps equals the
uninterrupted run's (NaN = NaN for the reference's electron gas) -- and the
file still reads as a plain .ion file (ion_lbm_load)."""
import numpy as np
import pytest

import ionsolver_gb300 as I
from ionsolver_gb300 import workloads as W
from tests import _util as U

pytestmark = pytest.mark.gpu


def _fields(lbm, case):
    return {n: lbm.read(n) for n in U.field_names(case)}


@pytest.mark.parametrize("kind", ["mhd", "tgv_fp16s_trt"])
def test_restore_continues_bit_for_bit(kind, tmp_path):
    if kind == "mhd":
        case = W.mhd_box(n=32, depth=2, magnet_r=6.0, magnet_t=4.0, field_mode=1)
        before, after = 3, 5
    else:
        case = W.taylor_green(shape=(32, 24, 16), amplitude=0.05, float_type=0, relaxation_time=1)
        before, after = 5, 7
    a = U.setup_gpu(case)
    a.initialize()
    a.run(before)
    p = tmp_path / "state.ion"
    a.checkpoint(p)
    a.run(after)
    a.finish_queues(60000)
    ref = _fields(a, case)
    b = I.Lbm.restore(p)
    assert b.get_time_step() == before
    b.run(after)
    b.finish_queues(60000)
    got = _fields(b, case)
    ft = case["config"]["float_type"]
    for n in ref:
        assert U.bit_diff_nan(got[n], ref[n], ft) == 0, n
    # the same file as a plain .ion file: flags, rho, u (and Q) at the checkpoint
    c = I.Lbm.read_file(p)
    assert np.array_equal(c.read("flags"), a.read("flags"))


def test_restore_rejects_plain_ion(tmp_path):
    case = W.taylor_green(shape=(16, 16, 8), amplitude=0.05, float_type=2)
    a = U.setup_gpu(case)
    a.initialize()
    p = tmp_path / "plain.ion"
    a.write_file(p)
    with pytest.raises(I.IonError, match="not a checkpoint"):
        I.Lbm.restore(p)
