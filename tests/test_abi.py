"""The C ABI without a GPU: libionsolver.so loads, exports every function
include/ionsolver.h declares, and rejects bad configurations and files with
the documented status codes before touching the device."""
import ctypes as C
import os
import re
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

import ionsolver_gb300 as I
from ionsolver_gb300 import _native as N

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "ionsolver.h"


def declared_functions():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(ion_\w+)\s*\(", text, flags=re.M)))


def test_library_exports_every_declared_function():
    lib = C.CDLL(str(N.LIB_PATH))
    names = declared_functions()
    assert len(names) >= 40
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing
    assert set(names) == set(N.exported_symbols())


def test_abi_version_and_defaults():
    assert N.lib().ion_abi_version() == 2
    c = N.Config()
    N.check(N.lib().ion_config_default(C.byref(c)))
    # LbmConfig::new (src/lbm/mod.rs:105-135)
    assert (c.velocity_set, c.relaxation_time, c.float_type) == (0, 0, 0)
    assert (c.n_x, c.n_y, c.n_z, c.d_x, c.d_y, c.d_z) == (1, 1, 1, 1, 1, 1)
    assert np.float32(c.nu) == np.float32(1.0) / np.float32(6.0)
    assert c.mhd_lod_depth == 4 and c.update_fields == 1
    assert (c.units.m, c.units.kg, c.units.s, c.units.a, c.units.k) == (1, 1, 1, 1, 1)


@pytest.mark.parametrize("change,code", [
    (dict(d_x=2), -2), (dict(velocity_set=3), -2), (dict(velocity_set=0, n_z=4), -2),
    (dict(ext_magneto_hydro=1), -2), (dict(ext_magneto_hydro=1, ext_volume_force=1, n_x=20), -2),
    (dict(ext_subgrid_ecr=1), -2), (dict(n_x=0), -2), (dict(float_type=7), -2),
    (dict(ext_magneto_hydro=1, ext_volume_force=1, mhd_lod_depth=5), -2),
    (dict(n_x=2048, n_y=2048, n_z=1024), -2), (dict(n_x=65536, n_y=65536, n_z=1), -2),
    # products that wrap past 2^64 if formed before the check: 2^31 * 2^31 * 4 = 2^64 -> 0,
    # (2^32-1)^2 * 2^31 -> 2^31 modulo 2^64
    (dict(n_x=2 ** 31, n_y=2 ** 31, n_z=4), -2), (dict(n_x=2 ** 32 - 1, n_y=2 ** 32 - 1, n_z=2 ** 31), -2)])
def test_create_rejects_configs(change, code):
    c = I.LbmConfig(velocity_set=2, n_x=32, n_y=32, n_z=32, float_type=2)
    for k, v in change.items():
        setattr(c, k, v)
    h = C.c_void_p()
    rc = N.lib().ion_lbm_create(C.byref(c.to_c()), C.byref(h))
    assert rc == code and not h.value
    assert N.lib().ion_last_error()


def test_load_rejects_bad_files(tmp_path):
    c = I.LbmConfig().to_c()
    h = C.c_void_p()
    assert N.lib().ion_lbm_load(str(tmp_path / "missing.ion").encode(), C.byref(c), C.byref(h)) == -5
    bad = tmp_path / "bad.ion"
    bad.write_bytes(b"NotIonSolver....\x02\x00\x02")
    assert N.lib().ion_lbm_load(str(bad).encode(), C.byref(c), C.byref(h)) == -6
    hdr = b"IonSolver setup\n" + bytes([2, 0, 2]) + np.array([1, 1, 1, 1], np.float32).tobytes()
    hdr += np.array([4, 4, 4], np.uint32).tobytes() + b"\x00" + np.array([1, 1, 1], np.uint32).tobytes()
    hdr += np.array([0.1, 0, 0, 0], np.float32).tobytes() + b"\x00\x04"
    trunc = tmp_path / "trunc.ion"
    trunc.write_bytes(hdr + b"\x00" * 10)           # body of 64 cells is 1088 bytes
    assert N.lib().ion_lbm_load(str(trunc).encode(), C.byref(c), C.byref(h)) == -6
    extra = tmp_path / "extra.ion"
    extra.write_bytes(hdr + b"\x00" * (64 * 17 + 3))  # trailing bytes (file.rs:183-185)
    assert N.lib().ion_lbm_load(str(extra).encode(), C.byref(c), C.byref(h)) == -6
    assert not h.value


def test_null_arguments_are_errors():
    lib = N.lib()
    assert lib.ion_lbm_initialize(None) == -1
    assert lib.ion_lbm_run(None, 3) == -1
    assert lib.ion_config_default(None) == -1


def test_create_without_a_device_is_an_error_not_an_abort():
    """A valid configuration in a process that sees no CUDA device: ION_E_CUDA and a
    message (the reference exits the process instead, opencl.rs:11-13).  Runs in a
    child process with CUDA_VISIBLE_DEVICES empty, so it holds on a GPU host too."""
    code = (
        "import ctypes as C, sys\n"
        "sys.path.insert(0, %r)\n"
        "import ionsolver_gb300 as I\n"
        "from ionsolver_gb300 import _native as N\n"
        "c = I.LbmConfig(velocity_set=2, n_x=32, n_y=32, n_z=32, float_type=2)\n"
        "h = C.c_void_p()\n"
        "rc = N.lib().ion_lbm_create(C.byref(c.to_c()), C.byref(h))\n"
        "if h.value: N.lib().ion_lbm_destroy(h)\n"
        "print(rc, N.lib().ion_last_error().decode())\n" % str(ROOT))
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    rc, msg = r.stdout.strip().split(" ", 1)
    assert int(rc) == -3 and "CUDA" in msg
