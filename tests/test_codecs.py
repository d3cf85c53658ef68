"""FP16S / FP16C storage codecs of the oracle against the reference's own
functions (sim_kernels.cl:79-90; vload_half/vstore_half_rte of
domain.rs:773-776) and against numpy's IEEE half conversion."""
import numpy as np
import pytest

import oracle as O

RAW = np.arange(65536, dtype=np.uint16)


def _floats():
    rng = np.random.default_rng(0)
    special = np.array([0.0, -0.0, 1.0, -1.0, 1.9995, 2.0, 1e-8, 6.1e-5, 65504 / 32768, 65520 / 32768], np.float32)
    halfway = (np.arange(0, 65536, 37, dtype=np.uint32) << 13) + (1 << 12)  # exact ties of the FP16S grid
    return np.concatenate([special, rng.uniform(-2, 2, 60000).astype(np.float32),
                           rng.normal(0, 1e-3, 30000).astype(np.float32),
                           (halfway.view(np.float32) / np.float32(32768.0)).astype(np.float32),
                           np.ldexp(rng.uniform(-1, 1, 20000), rng.integers(-40, 2, 20000)).astype(np.float32)])


def test_fp16s_against_numpy_half():
    lib = O.oracle_lib("f32")
    vals = _floats()
    enc = np.array([lib.orc_fp16s_encode(float(v)) for v in vals], np.uint16)
    with np.errstate(over="ignore", invalid="ignore"):  # the special values: overflow to +-inf, NaN
        ref = (vals * np.float32(32768.0)).astype(np.float16).view(np.uint16)
        h = RAW.view(np.float16).astype(np.float32) * np.float32(3.0517578e-05)
    assert np.array_equal(enc, ref)
    dec = np.array([lib.orc_fp16s_decode(int(r)) for r in RAW], np.float32)
    fin = np.isfinite(h)
    assert np.array_equal(dec[fin].view(np.uint32), h[fin].view(np.uint32))


@pytest.mark.skipif(not O.reference_available(), reason="reference kernels unavailable")
@pytest.mark.parametrize("codec", ["fp16s", "fp16c"])
def test_codecs_against_reference_functions(codec):
    mine = O.oracle_lib("f32")
    ref = O.ref_lib(O.make_config(velocity_set=2, float_type=2))
    import ctypes as C
    for n, rt, at in ((f"orc_{codec}_encode", C.c_uint16, C.c_float), (f"orc_{codec}_decode", C.c_float, C.c_uint16)):
        getattr(ref, n).restype = rt
        getattr(ref, n).argtypes = [at]
    enc_m, enc_r = getattr(mine, f"orc_{codec}_encode"), getattr(ref, f"orc_{codec}_encode")
    dec_m, dec_r = getattr(mine, f"orc_{codec}_decode"), getattr(ref, f"orc_{codec}_decode")
    for v in _floats()[::3]:
        assert enc_m(float(v)) == enc_r(float(v)), v
    a = np.array([dec_m(int(r)) for r in RAW], np.float32)
    b = np.array([dec_r(int(r)) for r in RAW], np.float32)
    fin = np.isfinite(b)
    assert np.array_equal(a[fin].view(np.uint32), b[fin].view(np.uint32))


def test_fp16c_round_trip_properties():
    lib = O.oracle_lib("f32")
    # every normal FP16C pattern decodes and re-encodes to itself
    for r in range(0x0800, 0x8000, 7):
        v = lib.orc_fp16c_decode(r)
        assert lib.orc_fp16c_encode(v) == r
