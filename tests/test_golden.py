"""The restated oracle reproduces the reference's golden outputs bit for bit
(tests/golden: inputs + SHA-256 of every output field, produced by the
reference's own kernels; see tests/golden/make_golden.py)."""
import json
from pathlib import Path

import numpy as np
import pytest

from tests.golden.cases import CASES
from tests.golden.make_golden import digest, outputs, run_case

HERE = Path(__file__).resolve().parent / "golden"
META = json.loads((HERE / "golden.json").read_text())
INPUTS = dict(np.load(HERE / "golden.npz"))


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_matches_reference_golden(name):
    case, o = run_case(name, "f32", INPUTS)
    got = {k: digest(v) for k, v in outputs(o, case).items()}
    assert got == META[name]["sha256"]


def test_fixture_inventory():
    assert set(META) == set(CASES)
    assert all(len(m["sha256"]) >= 3 for m in META.values())
