"""Regenerates tests/golden/golden.npz + golden.json from the reference's own
kernels (IonSolver src/kernels/sim_kernels.cl compiled as C++ by
oracle/build.py).  Run here, where the reference checkout is present:

    python tests/golden/make_golden.py

golden.npz holds every case's input arrays (so the inputs do not depend on
the platform's numpy); golden.json holds the SHA-256 of the raw bytes of
every output field and a few summary numbers.
"""
import hashlib
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

import oracle as O  # noqa: E402
from tests import _util as U  # noqa: E402
from tests.golden.cases import CASES  # noqa: E402


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).view(np.uint8).tobytes()).hexdigest()


def outputs(o, case):
    names = U.field_names(case)
    if case["config"].get("ext_force_field"):
        names = names + ["F"]
    return {n: o.field(n) for n in names}


def run_case(name, kind, inputs=None):
    build, steps, action = CASES[name]
    case = build()
    if inputs is not None:
        for k in list(case["fields"]):
            case["fields"][k] = inputs[f"{name}/{k}"]
    o = U.setup_oracle(case, kind, 1)
    if action == "setup":
        o.precompute_e()
    else:
        U.initialize_oracle(o, case)
        o.run(steps)
    return case, o


def main():
    if not O.reference_available():
        raise SystemExit("reference kernels unavailable")
    arrays, meta = {}, {}
    for name in CASES:
        case = CASES[name][0]()
        for k, v in case["fields"].items():
            arrays[f"{name}/{k}"] = v
        case, o = run_case(name, "ref", arrays)
        outs = outputs(o, case)
        meta[name] = {"steps": CASES[name][1], "action": CASES[name][2],
                      "sha256": {k: digest(v) for k, v in outs.items()},
                      "rho_sum": float(np.sum(outs["rho"].astype(np.float64))),
                      "source": "reference kernels (sim_kernels.cl) run in cell order on one thread"}
    np.savez_compressed(HERE / "golden.npz", **arrays)
    (HERE / "golden.json").write_text(json.dumps(meta, indent=1, sort_keys=True))
    print("wrote", len(meta), "cases")


if __name__ == "__main__":
    main()
