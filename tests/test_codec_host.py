"""The FP16C codec of the device header (ion_device.cuh, fp16c_encode/fp16c_decode,
compiled here for the host) against the oracle's restatement of the reference's
float_to_half_custom / half_to_float_custom (sim_kernels.cl:79-90; the oracle is pinned
to the reference's own kernels by test_codecs.py): every one of the 2^32 float inputs of
the encoder (NaNs in the oracle's GPU model: every NaN encodes as the canonical NaN
would) and all 2^16 inputs of the decoder, bit for bit.  The device form differs only
in two primitives (PTX shr with its clamped shift, the device fmaf), and
test_gpu_parity.py::test_codecs_exhaustive_against_oracle runs it on the GPU."""
import os
import shutil
import subprocess
from pathlib import Path

import pytest

from oracle import build as OB

ROOT = Path(__file__).resolve().parent.parent

SRC = r"""
#include <cstdint>
#include <cstdio>
#include <cstring>
#include "ion_device.cuh"
extern "C" uint16_t orc_fp16c_encode(float);
extern "C" float orc_fp16c_decode(uint16_t);
extern "C" void orc_set_nan_model(int);
int main() {
    orc_set_nan_model(1);
    unsigned long long bad_enc = 0, bad_dec = 0;
#pragma omp parallel for reduction(+ : bad_enc) schedule(static)
    for (long long i = 0; i < (1ll << 32); i++) {
        const uint32_t u = (uint32_t)i;
        float f;
        memcpy(&f, &u, 4);
        if (ion::fp16c_encode(f) != orc_fp16c_encode(f)) bad_enc++;
    }
    for (uint32_t r = 0; r < 65536u; r++) {
        const float a = ion::fp16c_decode((uint16_t)r), b = orc_fp16c_decode((uint16_t)r);
        uint32_t ua, ub;
        memcpy(&ua, &a, 4);
        memcpy(&ub, &b, 4);
        if (ua != ub) bad_dec++;
    }
    printf("%llu %llu\n", bad_enc, bad_dec);
    return 0;
}
"""


def _nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and Path(c).exists():
            return c
    return None


def test_fp16c_codec_all_inputs(tmp_path):
    nvcc = _nvcc()
    if nvcc is None:
        pytest.skip("nvcc not found")
    so = Path(OB.build_oracle()["f32"])
    src = tmp_path / "codec_host.cu"
    src.write_text(SRC)
    exe = tmp_path / "codec_host"
    cmd = [nvcc, "-O2", "-std=c++17", "-Xcompiler", "-fopenmp,-ffp-contract=off", f"-I{ROOT / 'include'}",
           f"-I{ROOT / 'ionsolver_gb300' / 'csrc'}", str(src), "-o", str(exe), f"-L{so.parent}",
           f"-l:{so.name}", f"-Xlinker", f"-rpath={so.parent}", "-lgomp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    bad_enc, bad_dec = map(int, out.stdout.split())
    assert (bad_enc, bad_dec) == (0, 0)
