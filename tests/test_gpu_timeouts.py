"""Bounded device waits run out on purpose, and the context stays usable.

The row-staged stream_collide, the E/B update and the batched step wait for
data they staged with bulk copies (and the batch for its grid barriers).  A
poll limit of 0 makes every such wait give up at once: the kernels record the
failure, let their copies in flight land, skip the rest of the launch and
return.  The host then sees ION_E_TIMEOUT from ion_lbm_finish_queues /
ion_batch_finish; with the default limits restored and the state initialized
again, the next run is bit-identical to an untouched handle's.  No wait is
unbounded and nothing faults."""
import pytest

import ionsolver_gb300 as I
from ionsolver_gb300 import _native as N
from ionsolver_gb300 import workloads as W
from tests import _util as U

pytestmark = pytest.mark.gpu


def _reset(lbm, case):
    for name in ("rho", "u", "q"):
        lbm.write(name, case["fields"][name])
    import numpy as np
    lbm.write("qu_lod", np.zeros(lbm.field_info("qu_lod")[1], np.float32))
    lbm.initialize()


@pytest.mark.parametrize("nx", [32, 272, 400], ids=["producer-warp-rows", "producer-warp-384-rows", "long-rows"])
def test_single_domain_wait_expires_and_recovers(nx):
    case = W.mhd_plasma(shape=(nx, 16, 16), depth=2, magnet_r=4.0, magnet_t=3.0, field_mode=1)
    g = U.setup_gpu(case)
    g.initialize()
    g.finish_queues(60000)
    g.set_wait_limit(0)
    g.do_time_step()
    with pytest.raises(N.IonError) as e:
        g.finish_queues(60000)
    assert e.value.code == N.ION_E_TIMEOUT
    g.set_wait_limit(None)
    _reset(g, case)
    g.run(6)
    g.finish_queues(60000)  # no error left over
    ref = U.run_gpu(case, 6)
    for name in U.field_names(case):
        assert U.bit_diff(g.read(name), ref.read(name)) == 0, name


def test_batch_barrier_and_tile_waits_expire_and_recover():
    cases = W.batch_domains(count=4, field_mode=1, plasma=True)
    doms = [U.setup_gpu(c) for c in cases]
    for d in doms:
        d.initialize()
    b = I.Batch(doms)
    b.run(2)
    b.finish(60000)
    b.set_wait_limits(0, 0)
    b.run(1)
    with pytest.raises(N.IonError) as e:
        b.finish(60000)
    assert e.value.code == N.ION_E_TIMEOUT
    b.set_wait_limits(None, None)
    for d, c in zip(doms, cases):
        _reset(d, c)
    t0 = doms[0].get_time_step()
    b.close()
    b = I.Batch(doms)
    b.run(4)
    b.finish(60000)
    for d, c in zip(doms, cases):
        ref = U.setup_gpu(c)
        ref.initialize()
        ref.run(4)
        ref.finish_queues(60000)
        assert d.get_time_step() == t0 + 4 and ref.get_time_step() == 4
        for name in ("fi", "ei", "fqi", "e_dyn", "q"):
            assert U.bit_diff(d.read(name), ref.read(name)) == 0, name
