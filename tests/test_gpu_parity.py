"""GPU kernels against the CPU oracle on the same seeded inputs.

Bar: bit-identical results (integer and floating point) for the timestep in
BITWISE field mode, the voxeliser and the static magnet field; the FAST
field mode within a stated relative error."""
import numpy as np
import pytest

import oracle as O
from ionsolver_gb300 import workloads as W
from tests import _util as U

pytestmark = pytest.mark.gpu


def orc_run(case, steps):
    """The oracle with the GPU's NaN model (see oracle.OracleLbm)."""
    return U.run_oracle(case, steps, canonical_nan=True)


@pytest.mark.parametrize("ft", [2, 0, 1], ids=["FP32", "FP16S", "FP16C"])
@pytest.mark.parametrize("rt", [0, 1], ids=["SRT", "TRT"])
def test_plain_taylor_green_bitwise(ft, rt):
    case = W.taylor_green(shape=(32, 24, 16), amplitude=0.05, float_type=ft, relaxation_time=rt)
    g = U.run_gpu(case, 100)
    o = orc_run(case, 100)
    assert U.compare_bitwise(g, o, ["fi", "rho", "u"]) == {"fi": 0, "rho": 0, "u": 0}


@pytest.mark.parametrize("vs,shape", [(1, (16, 12, 10)), (0, (40, 24, 1))], ids=["D3Q15", "D2Q9"])
def test_other_velocity_sets_bitwise(vs, shape):
    case = W.taylor_green(shape=shape, amplitude=0.05)
    case["config"]["velocity_set"] = vs
    if vs == 0:  # a 2-D shear field (the 3-D vortex has no in-plane flow at n_z = 1)
        n2 = shape[0] * shape[1]
        rng = np.random.default_rng(11)
        case["fields"]["u"] = np.concatenate([rng.normal(0, 0.02, 2 * n2), np.zeros(n2)]).astype(np.float32)
    g = U.run_gpu(case, 50)
    o = orc_run(case, 50)
    assert U.compare_bitwise(g, o, ["fi", "rho", "u"]) == {"fi": 0, "rho": 0, "u": 0}


@pytest.mark.parametrize("nx", [24, 32], ids=["global-loads", "row-staged"])
@pytest.mark.parametrize("rt", [0, 1], ids=["SRT", "TRT"])
def test_boundaries_and_forces_bitwise(rt, nx):
    """Solid cells, equilibrium (inflow/outflow) cells, volume force and force field
    (rows of 24 cells run the global-load stream_collide, rows of 32 the row-staged one)."""
    ny, nz = 20, 16
    N = nx * ny * nz
    rng = np.random.default_rng(7)
    case = W.taylor_green(shape=(nx, ny, nz), amplitude=0.03, relaxation_time=rt)
    flags = W.shell_flags(nx, ny, nz)
    flags.reshape(nz, ny, nx)[:, :, 0] = 0x02      # equilibrium inlet plane
    flags.reshape(nz, ny, nx)[4:8, 5:9, 6:10] = 0x01  # an obstacle
    case["fields"]["flags"] = flags
    case["fields"]["F"] = rng.normal(0, 1e-5, 3 * N).astype(np.float32)
    case["fields"]["rho"] = (1.0 + rng.normal(0, 1e-3, N)).astype(np.float32)
    case["config"].update(ext_equilibrium_boundaries=1, ext_volume_force=1, ext_force_field=1,
                          f_x=1e-6, f_y=-2e-6, f_z=5e-7)
    g = U.run_gpu(case, 60)
    o = orc_run(case, 60)
    assert U.compare_bitwise(g, o, ["fi", "rho", "u", "flags"]) == {"fi": 0, "rho": 0, "u": 0, "flags": 0}


@pytest.mark.parametrize("nx", [24, 32], ids=["global-loads", "row-staged"])
@pytest.mark.parametrize("ft", [2, 1], ids=["FP32", "FP16C"])
def test_mhd_boundaries_and_forces_bitwise(ft, nx):
    """MHD with equilibrium (inflow) cells, an obstacle and a force field on the
    finite-plasma start: the electron gas, the gas and the charge lattice at the
    equilibrium cells (sim_kernels.cl:651-655), 30 steps, every field bit-identical."""
    ny, nz = 20, 16
    N = nx * ny * nz
    rng = np.random.default_rng(27)
    case = W.mhd_plasma(shape=(nx, ny, nz), float_type=ft, depth=2, magnet_r=4.0, magnet_t=3.0, field_mode=0)
    flags = W.shell_flags(nx, ny, nz)
    flags.reshape(nz, ny, nx)[:, :, 0] = 0x02      # equilibrium inlet plane
    flags.reshape(nz, ny, nx)[8:11, 5:9, 14:18] = 0x01  # an obstacle
    case["fields"].update(flags=flags, F=rng.normal(0, 1e-5, 3 * N).astype(np.float32),
                          rho=(1.0 + rng.normal(0, 1e-3, N)).astype(np.float32))
    case["config"].update(ext_equilibrium_boundaries=1, ext_force_field=1, f_x=1e-6, f_y=-2e-6, f_z=5e-7)
    g = U.run_gpu(case, 30)
    o = orc_run(case, 30)
    diff = U.compare_bitwise(g, o, U.field_names(case))
    assert all(v == 0 for v in diff.values()), diff


@pytest.mark.parametrize("ft", [2, 0, 1], ids=["FP32", "FP16S", "FP16C"])
@pytest.mark.parametrize("n,depth,r,t", [(32, 4, 6.0, 4.0), (16, 2, 4.0, 3.0), (24, 3, 5.0, 4.0)],
                         ids=["32c-D4", "16c-D2", "24c-D3"])
def test_mhd_bitwise(ft, n, depth, r, t):
    case = W.mhd_box(n=n, float_type=ft, depth=depth, magnet_r=r, magnet_t=t, field_mode=0)
    g = U.run_gpu(case, 12)
    o = orc_run(case, 12)
    diff = U.compare_bitwise(g, o, U.field_names(case))
    assert all(v == 0 for v in diff.values()), diff


@pytest.mark.parametrize("nx", [24, 32], ids=["global-loads", "row-staged"])
def test_mhd_without_field_output_bitwise(nx):
    """update_fields off (rho and u are not written by stream_collide) with MHD on the
    finite-plasma start, LOD depth 1: every other field bit-identical after 20 steps."""
    case = W.mhd_plasma(shape=(nx, 16, 16), depth=1, magnet_r=4.0, magnet_t=3.0, field_mode=0, update_fields=0)
    g = U.run_gpu(case, 20)
    o = orc_run(case, 20)
    diff = U.compare_bitwise(g, o, U.field_names(case))
    assert all(v == 0 for v in diff.values()), diff


@pytest.mark.parametrize("ft", [2, 0, 1], ids=["FP32", "FP16S", "FP16C"])
def test_mhd_d3q15_bitwise(ft):
    """MHD on the D3Q15 velocity set (the global-load stream_collide), finite-plasma
    start, 20 steps, every field bit-identical."""
    case = W.mhd_plasma(shape=(16, 16, 16), float_type=ft, depth=2, magnet_r=4.0, magnet_t=3.0, field_mode=0)
    case["config"]["velocity_set"] = 1
    g = U.run_gpu(case, 20)
    o = orc_run(case, 20)
    diff = U.compare_bitwise(g, o, U.field_names(case))
    assert all(v == 0 for v in diff.values()), diff


@pytest.mark.parametrize("depth", [0, 1])
def test_mhd_shallow_lod_bitwise(depth):
    """LOD depth 0 (no bins: the field is the static one) and 1 (8 bins), finite-plasma
    start, the row-staged stencil: every field bit-identical to the oracle after 20 steps."""
    case = W.mhd_plasma(shape=(32, 16, 16), depth=depth, magnet_r=4.0, magnet_t=3.0, field_mode=0)
    g = U.run_gpu(case, 20)
    o = orc_run(case, 20)
    diff = U.compare_bitwise(g, o, U.field_names(case))
    assert all(v == 0 for v in diff.values()), diff


def test_mhd_fast_field_close():
    """FAST field mode: same sources and order, rsqrt/FMA arithmetic."""
    case = W.mhd_box(n=32, depth=4, magnet_r=6.0, magnet_t=4.0, field_mode=1)
    g = U.run_gpu(case, 1)
    ref_case = dict(case, config=dict(case["config"], field_mode=0))
    o = orc_run(ref_case, 1)
    # dynamic part of the field only: subtract the static field first
    for dyn, stat in (("e_dyn", "e_stat"), ("b_dyn", "b_stat")):
        N = 32 ** 3
        gd = g.read(dyn)[:3 * N].astype(np.float64) - g.read(stat).astype(np.float64)
        od = o.field(dyn)[:3 * N].astype(np.float64) - o.field(stat).astype(np.float64)
        assert U.rel_err(gd, od) < 1e-4, dyn


def test_voxelise_and_static_field_bitwise():
    case = W.mhd_box(n=32, depth=4, magnet_r=7.0, magnet_t=5.0)
    case["meshes"].append(tuple(list(W.annulus((16.0, 16.0, 22.0), 9.0, 5.0, 3.0, axis=0)) + ["solid", (0, 0, 0)]))
    g = U.setup_gpu(case)
    o = U.setup_oracle(case, canonical_nan=True)
    d = U.compare_bitwise(g, o, ["flags", "b_dyn", "b_stat", "e_dyn"])
    assert d == {"flags": 0, "b_dyn": 0, "b_stat": 0, "e_dyn": 0}
    flags = g.read("flags")
    assert (flags == 0x11).sum() > 100 and ((flags & 0x1F) == 0x01).sum() > 0


def test_static_e_bitwise():
    case = W.mhd_box(n=16, depth=2, magnet=False)
    p = W.cylinder((8.0, 8.0, 8.0), 3.0, 3.0, axis=1)
    case["meshes"] = [(p[0], p[1], p[2], "charged", (2e-9, 0, 0))]
    g = U.setup_gpu(case)
    g.precompute_E()
    o = U.setup_oracle(case, canonical_nan=True)
    o.precompute_e()
    assert U.compare_bitwise(g, o, ["flags", "e_stat", "b_dyn"]) == {"flags": 0, "e_stat": 0, "b_dyn": 0}


def test_update_fields_bitwise():
    case = W.taylor_green(shape=(16, 16, 16))
    case["config"]["update_fields"] = 0
    g = U.run_gpu(case, 7)
    o = orc_run(case, 7)
    g.update_fields()
    o.update_fields()
    assert U.compare_bitwise(g, o, ["rho", "u"]) == {"rho": 0, "u": 0}


def test_graph_run_equals_single_steps():
    case = W.mhd_box(n=16, depth=2, magnet_r=4.0, magnet_t=3.0)
    a = U.run_gpu(case, 37, graph=True)
    b = U.run_gpu(case, 37, graph=False)
    assert a.get_time_step() == b.get_time_step() == 37
    for name in U.field_names(case):
        assert U.bit_diff(a.read(name), b.read(name)) == 0, name


def test_mass_conservation_fp64():
    """Sum of all DDFs (FP64 reduction) over 300 steps of a walled TGV box."""
    case = W.taylor_green(shape=(64, 64, 64), amplitude=0.05)
    case["fields"]["flags"] = W.shell_flags(64, 64, 64)
    g = U.setup_gpu(case)
    g.initialize()
    m0, _ = g.mass_charge()
    g.run(300)
    m1, _ = g.mass_charge()
    assert abs(m1 - m0) / m0 < 1e-6, (m0, m1)


def test_mhd_strict_bitwise_before_nan_onset_and_charge_conservation():
    """Before the reference's electron gas produces its first NaN (step 3 of
    this case), every bit agrees and the gas charge sum is conserved."""
    case = W.mhd_box(n=32, depth=4, magnet_r=6.0, magnet_t=4.0, field_mode=0)
    g = U.setup_gpu(case)
    g.initialize()
    g.run(2)
    g.finish_queues(60000)
    o = orc_run(case, 2)
    for n in U.field_names(case):
        a, b = g.read(n), o.field(n)
        if a.dtype == np.float32:
            assert not np.isnan(a).any(), n
        assert U.bit_diff(a, b.astype(a.dtype)) == 0, n
    # the FP64 reductions agree with a float64 sum of the oracle's arrays
    mass, charge = g.mass_charge()
    n = 32 ** 3
    m_ref = float(np.sum(o.field("fi").astype(np.float64))) + n
    q_ref = (float(np.sum(o.field("fqi").astype(np.float64))) + n) - (float(np.sum(o.field("ei").astype(np.float64))) + n)
    assert abs(mass - m_ref) <= 1e-12 * m_ref
    assert abs(charge - q_ref) <= 1e-9


def test_codecs_exhaustive_against_oracle():
    import ionsolver_gb300 as I
    lib = O.oracle_lib("f32")
    rng = np.random.default_rng(3)
    # every float exponent from 2^-35 to 2^9 with the mantissas where the FP16C encoder's
    # rounding carries or its normal/subnormal/zero cases switch, both signs; +-0, +-inf
    # and NaNs (encoded as the canonical NaN, the oracle's GPU NaN model)
    mant = np.array([0, 1, 0x7FF, 0x800, 0x801, 0xFFF, 0x1000, 0x3FF800, 0x7FF7FF, 0x7FF800, 0x7FFFFF], np.uint32)
    exps = np.arange(92, 137, dtype=np.uint32)
    edge = ((exps[:, None] << 23) | mant[None, :]).ravel()
    special = np.array([0, 0x7F800000, 0x7FC00000, 0x7F800001, 0x7FFFFFFF], np.uint32)
    bits = np.concatenate([edge, edge | 0x80000000, special, special | 0x80000000])
    vals = np.concatenate([np.concatenate([rng.uniform(-2.0, 2.0, 40000), rng.normal(0, 1e-3, 20000),
                                           np.ldexp(rng.uniform(-1, 1, 5536), rng.integers(-30, 2, 5536))]
                                          ).astype(np.float32),
                           bits.view(np.float32)])  # the bit patterns as they are (no cast)
    raw = (np.arange(vals.size) % 65536).astype(np.uint16)  # every 16-bit pattern (and some twice)
    lib.orc_set_nan_model(1)
    try:
        for ft, enc_f, dec_f in ((0, lib.orc_fp16s_encode, lib.orc_fp16s_decode),
                                 (1, lib.orc_fp16c_encode, lib.orc_fp16c_decode)):
            enc, dec, rdec = I.codec_roundtrip(ft, vals, raw)
            e_ref = np.array([enc_f(float(v)) for v in vals], np.uint16)
            d_ref = np.array([dec_f(int(r)) for r in raw[:65536]], np.float32)
            rdec = rdec[:65536]
            # FP16S: IEEE half of 2^15 x (a NaN's payload is not part of the format)
            keep = ~np.isnan(vals) if ft == 0 else np.ones(len(vals), bool)
            assert np.array_equal(enc[keep], e_ref[keep])
            finite = np.isfinite(d_ref)
            assert np.array_equal(rdec[finite].view(np.uint32), d_ref[finite].view(np.uint32))
    finally:
        lib.orc_set_nan_model(0)


def test_shared_division_matches_ieee():
    """The BITWISE field divides by |R|^3 through one correctly rounded reciprocal
    and two FMA corrections (Markstein); bit for bit the IEEE quotient on 2^30
    pseudo-random operands in the field's ranges, two seeds."""
    import ctypes as C
    from ionsolver_gb300 import _native as N
    for seed in (1, 0x5eed):
        bad = C.c_uint64()
        first = (C.c_float * 2)()
        N.check(N.lib().ion_check_shared_division(1 << 30, seed, C.byref(bad), first))
        assert bad.value == 0, (bad.value, first[0], first[1])


@pytest.mark.parametrize("ft,rt", [(2, 0), (0, 1), (1, 0)], ids=["FP32-SRT", "FP16S-TRT", "FP16C-SRT"])
def test_subgrid_ecr_bitwise(ft, rt):
    """SUBGRID_ECR on the GPU against the oracle: every field bit-identical (NaN =
    NaN) after two and after four steps; with FP32 storage the first two steps
    stay finite (16-bit storage reaches the reference's electron-gas NaN sooner)."""
    case = W.ecr_box(n=16, float_type=ft, depth=2, relaxation_time=rt)
    names = U.field_names(case)
    g = U.setup_gpu(case)
    g.initialize()
    g.run(2)
    g.finish_queues(60000)
    o = orc_run(case, 2)
    if ft == 2:
        for n in names:
            a = g.read(n)
            assert a.dtype != np.float32 or not np.isnan(a).any(), n
    assert U.compare_bitwise(g, o, names) == {n: 0 for n in names}
    g.run(2)
    g.finish_queues(60000)
    o.run(2)
    assert U.compare_bitwise(g, o, names) == {n: 0 for n in names}


@pytest.mark.parametrize("nx", [272, 400])
@pytest.mark.parametrize("ft,rt", [(2, 0), (0, 0), (1, 1)], ids=["FP32-SRT", "FP16S-SRT", "FP16C-TRT"])
def test_long_rows_bitwise(ft, rt, nx):
    """Rows of 257-384 cells take the producer-warp form with the 384-cell row stride,
    longer rows the CTA-barrier form: elongated MHD boxes (nx x 16 x 16) bit-identical
    to the oracle after 2 steps."""
    case = W.mhd_box(shape=(nx, 16, 16), depth=2, magnet_r=5.0, magnet_t=3.0, float_type=ft)
    case["config"]["relaxation_time"] = rt
    g = U.run_gpu(case, 2)
    o = orc_run(case, 2)
    diff = U.compare_bitwise(g, o, U.field_names(case))
    assert all(v == 0 for v in diff.values()), diff


@pytest.mark.parametrize("nx", [288, 400])
@pytest.mark.parametrize("ft", [2, 0, 1], ids=["FP32", "FP16S", "FP16C"])
def test_long_rows_plain_trt_bitwise(ft, nx):
    """Both long-row forms without MHD: an nx x 8 x 8 Taylor-Green box, TRT, 20 steps."""
    case = W.taylor_green(shape=(nx, 8, 8), amplitude=0.05, float_type=ft, relaxation_time=1)
    g = U.run_gpu(case, 20)
    o = orc_run(case, 20)
    assert U.compare_bitwise(g, o, ["fi", "rho", "u"]) == {"fi": 0, "rho": 0, "u": 0}


@pytest.mark.parametrize("nx", [16, 144, 240, 368])
def test_row_strides_bitwise(nx):
    """Rows that fill the shared-memory row stride only partly (128-element stride: 16
    cells; 256: 144, 240; 384: 368): an MHD box in FP16C (the written-back rows, the
    shared two-pass code) and a plain FP16S TRT box, bit-identical to the oracle."""
    case = W.mhd_box(shape=(nx, 16, 8), depth=2, magnet_r=3.0, magnet_t=2.0, float_type=1)
    g = U.run_gpu(case, 2)
    o = orc_run(case, 2)
    diff = U.compare_bitwise(g, o, U.field_names(case))
    assert all(v == 0 for v in diff.values()), diff
    case = W.taylor_green(shape=(nx, 8, 4), amplitude=0.05, float_type=0, relaxation_time=1)
    g = U.run_gpu(case, 10)
    o = orc_run(case, 10)
    assert U.compare_bitwise(g, o, ["fi", "rho", "u"]) == {"fi": 0, "rho": 0, "u": 0}


@pytest.mark.parametrize("ft", [2, 0, 1], ids=["FP32", "FP16S", "FP16C"])
def test_mhd_trt_bitwise(ft):
    """MHD with TRT collision through the row-staged stream_collide (32^3, depth 4)."""
    case = W.mhd_box(n=32, float_type=ft, depth=4, magnet_r=6.0, magnet_t=4.0, field_mode=0)
    case["config"]["relaxation_time"] = 1
    g = U.run_gpu(case, 8)
    o = orc_run(case, 8)
    diff = U.compare_bitwise(g, o, U.field_names(case))
    assert all(v == 0 for v in diff.values()), diff
