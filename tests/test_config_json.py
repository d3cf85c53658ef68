"""LbmConfig as JSON in the reference's serde layout (file::read_config /
file::write_config, src/file.rs:310-334): field names and enum spellings of
LbmConfig (src/lbm/mod.rs:45-101), Units and GraphicsConfig; no device needed."""
import json

import pytest

import ionsolver_gb300 as I
from ionsolver_gb300 import _native as N

# a configuration file as the reference writes it (serde_json, compact): every
# LbmConfig field, the nested Units and GraphicsConfig::new()
REFERENCE_STYLE = (
    '{"velocity_set":"D3Q19","relaxation_time":"Trt","float_type":"FP16C",'
    '"units":{"m":0.5,"kg":2.0,"s":0.001,"a":1e-6,"k":1.0,"prop":"Xe"},'
    '"n_x":128,"n_y":96,"n_z":64,"d_x":1,"d_y":1,"d_z":1,"nu":0.033333335,"f_x":0.0,"f_y":1e-5,"f_z":0.0,'
    '"ext_equilibrium_boudaries":true,"ext_volume_force":true,"ext_force_field":false,"ext_magneto_hydro":true,'
    '"ext_subgrid_ecr":false,"mhd_lod_depth":3,"ecr_freq":0.0,"ecr_field_strength":0.0,'
    '"graphics_config":{"graphics_active":false,"background_color":0,"camera_width":1920,"camera_height":1080,'
    '"v_max":0.25,"q_min":0.0001,"f_max":0.002,"rho_delta":0.5,"streamline_every":4,"stream_line_lenght":128,'
    '"vec_vis_mode":"U","slice_mode":"Off","slice_x":0,"slice_y":0,"slice_z":0,"max_slice_x":0,"max_slice_y":0,'
    '"max_slice_z":0,"field_vis":"Vector","streamline_mode":false,"field_mode":false,"field_slice_mode":false,'
    '"q_mode":false,"q_field_mode":false,"flags_mode":false,"flags_surface_mode":false,"axes_mode":false,'
    '"ecrc_mode":false,"render_intervals":false,"keyframes":[]},"run_steps":5000}')


def test_read_reference_style(tmp_path):
    p = tmp_path / "cfg.json"
    p.write_text(REFERENCE_STYLE)
    c = I.read_config(p)
    assert (c.velocity_set, c.relaxation_time, c.float_type) == (2, 1, 1)
    assert (c.n_x, c.n_y, c.n_z, c.mhd_lod_depth, c.run_steps) == (128, 96, 64, 3, 5000)
    assert c.nu == pytest.approx(1 / 30, rel=1e-7) and c.f_y == pytest.approx(1e-5)
    assert c.ext_equilibrium_boudaries and c.ext_volume_force and c.ext_magneto_hydro and not c.ext_force_field
    assert not c.update_fields  # graphics_active false -> no UPDATE_FIELDS (domain.rs:856)
    u = c.units
    assert (u.m, u.kg, u.s, u.a, u.prop) == (0.5, 2.0, pytest.approx(0.001), pytest.approx(1e-6), 5)


def test_round_trip_and_layout(tmp_path):
    c = I.LbmConfig(velocity_set=1, relaxation_time=0, float_type=2, n_x=48, n_y=40, n_z=32, nu=0.1234567,
                    f_x=-2.5e-7, ext_volume_force=1, ext_force_field=1, update_fields=1, field_mode=1)
    p = tmp_path / "out.json"
    I.write_config(p, c)
    text = p.read_text()
    d = json.loads(text)  # valid JSON
    keys = list(d)
    assert keys[:4] == ["velocity_set", "relaxation_time", "float_type", "units"]
    assert "ext_equilibrium_boudaries" in d and d["graphics_config"]["graphics_active"] is True
    assert d["velocity_set"] == "D3Q15" and d["float_type"] == "FP32" and d["units"]["prop"] == "H"
    back = I.read_config(p)
    c = I.LbmConfig.from_c(c.to_c())  # the float32 values the library holds
    for f in ("velocity_set", "relaxation_time", "float_type", "n_x", "n_y", "n_z", "nu", "f_x", "f_y", "f_z",
              "ext_volume_force", "ext_force_field", "ext_magneto_hydro", "mhd_lod_depth", "update_fields",
              "field_mode", "run_steps"):
        assert getattr(back, f) == getattr(c, f), f  # floats are written in round-trip form


def test_errors(tmp_path):
    p = tmp_path / "bad.json"
    p.write_text('{"velocity_set":"D4Q99"}')
    with pytest.raises(N.IonError, match="Could not parse file"):
        I.read_config(p)
    p.write_text('{"velocity_set": ')
    with pytest.raises(N.IonError):
        I.read_config(p)
    with pytest.raises(N.IonError, match="Could not find file"):
        I.read_config(tmp_path / "missing.json")
