"""Build recipe for the oracles (test infrastructure, not product code).

Two CPU oracles are built here:

* ``oracle/_build/libionoracle_f32.so`` / ``_f64.so`` -- the C restatement of
  the reference algorithm (``oracle/ion_oracle.c``), compiled with the state
  and arithmetic type ``float`` (bit-level parity target) or ``double`` (the
  FP64 accuracy oracle).
* ``oracle/_ref/libionref_<variant>.so`` -- the reference's own kernel text
  (IonSolver ``src/kernels/sim_kernels.cl``) compiled as C++ through
  ``oracle/ref_shim/ion_ref_compat.hpp``.  As in the reference (one OpenCL
  program per domain, ``src/lbm/domain.rs:128-145``), every combination of
  compile-time switches is its own build; sizes and unit constants are
  runtime values here.

The kernel text is taken from the reference checkout (``ION_REFERENCE_ROOT``,
or ``--reference PATH`` when this file runs as a script) as
``src/opencl.rs:67-75`` does: everything after
the ``EndTempDefines%`` marker.  Two mechanical rewrites make it C++:
OpenCL vector literals ``(float3)(a,b,c)`` become constructor calls, and the
voxeliser's ``distances`` array gets one guard element in front (its
insertion sort reads ``distances[-1]``, ``sim_kernels.cl:1197``).  The
generated text goes to ``oracle/_ref/`` only (git-ignored).
"""
from __future__ import annotations

import hashlib
import os
import re
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parent
BUILD = HERE / "_build"
REF = HERE / "_ref"
SHIM = HERE / "ref_shim"
INCLUDE = REPO / "include"

CXX = os.environ.get("CXX", "g++")
CC = os.environ.get("CC", "gcc")
# No FMA contraction anywhere: a*b+c stays two roundings unless the source
# calls fma().  -fwrapv: the reference relies on wrapping integer shifts.
COMMON_FLAGS = ["-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fwrapv", "-fno-fast-math"]


def reference_root() -> Path | None:
    """The IonSolver checkout: ION_REFERENCE_ROOT, or ``--reference PATH`` on this
    script's command line (which sets it).  None when neither is given."""
    root = os.environ.get("ION_REFERENCE_ROOT")
    return Path(root) if root else None


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


# --------------------------------------------------------------------------
# restated C oracle
# --------------------------------------------------------------------------
def build_oracle(force: bool = False) -> dict[str, Path]:
    BUILD.mkdir(parents=True, exist_ok=True)
    src = HERE / "ion_oracle.c"
    out = {}
    for prec, real in (("f32", "float"), ("f64", "double")):
        so = BUILD / f"libionoracle_{prec}.so"
        if force or not so.exists() or so.stat().st_mtime < max(src.stat().st_mtime, (INCLUDE / "ionsolver.h").stat().st_mtime):
            _run([CC, "-std=c11", *COMMON_FLAGS, f"-DORC_REAL={real}", f"-DORC_PREC_{prec.upper()}",
                  f"-I{INCLUDE}", str(src), "-o", str(so), "-lm"])
        out[prec] = so
    return out


# --------------------------------------------------------------------------
# the reference's kernels
# --------------------------------------------------------------------------
BODY = REF / "sim_kernels_body.inc"


def generate_reference_body() -> bool:
    """Regenerate oracle/_ref/sim_kernels_body.inc from the reference checkout.

    Returns False when neither the checkout nor a previously generated body
    is available (the reference oracle is then unavailable)."""
    root = reference_root()
    cl = root / "src" / "kernels" / "sim_kernels.cl" if root else None
    if cl is None or not cl.exists():
        return BODY.exists()
    text = cl.read_text()
    parts = text.split("EndTempDefines%")
    if len(parts) != 2:
        raise RuntimeError("sim_kernels.cl: expected exactly one EndTempDefines% marker")
    body = parts[1]
    body = re.sub(r"\((float3|uint3|int3)\)\s*\(", r"\1(", body)
    old = "ushort distances[64];"
    if body.count(old) != 1:
        raise RuntimeError("sim_kernels.cl: voxelize_mesh distances array not found")
    body = body.replace(old, "ushort distances_pad_[65] = {0}; ushort* distances = distances_pad_ + 1;")
    REF.mkdir(parents=True, exist_ok=True)
    header = "// generated from IonSolver src/kernels/sim_kernels.cl by oracle/build.py -- do not edit\n"
    new = header + body
    if not BODY.exists() or BODY.read_text() != new:
        BODY.write_text(new)
    return True


_VS = {0: ("D2Q9", 2, 9, 3), 1: ("D3Q15", 3, 15, 5), 2: ("D3Q19", 3, 19, 5), 3: ("D3Q27", 3, 27, 9)}


def variant_key(cfg: dict) -> str:
    vs = int(cfg.get("velocity_set", 2))
    ft = int(cfg.get("float_type", 2))
    return (f"v{vs}f{ft}r{int(cfg.get('relaxation_time', 0))}e{int(bool(cfg.get('ext_equilibrium_boundaries')))}"
            f"vf{int(bool(cfg.get('ext_volume_force')))}ff{int(bool(cfg.get('ext_force_field')))}"
            f"m{int(bool(cfg.get('ext_magneto_hydro')))}d{int(cfg.get('mhd_lod_depth', 4))}"
            f"u{int(bool(cfg.get('update_fields')))}x{int(bool(cfg.get('ext_subgrid_ecr')))}")


def variant_header(cfg: dict) -> str:
    """The #define block of get_device_defines (src/lbm/domain.rs:736-858).

    Sizes and unit constants become runtime values of the host program; the
    switches the kernel text tests with #if/#ifdef stay preprocessor
    literals."""
    vs = int(cfg.get("velocity_set", 2))
    name, dims, q, transfers = _VS[vs]
    weights = {
        0: ["#define DEF_W0 (1.0f/2.25f)", "#define DEF_WS (1.0f/9.0f)", "#define DEF_WE (1.0f/36.0f)"],
        1: ["#define DEF_W0 (1.0f/4.5f)", "#define DEF_WS (1.0f/9.0f)", "#define DEF_WC (1.0f/72.0f)"],
        2: ["#define DEF_W0 (1.0f/3.0f)", "#define DEF_WS (1.0f/18.0f)", "#define DEF_WE (1.0f/36.0f)"],
        3: ["#define DEF_W0 (1.0f/3.0f)", "#define DEF_WS (1.0f/18.0f)", "#define DEF_WE (1.0f/36.0f)"],
    }[vs]
    ft = int(cfg.get("float_type", 2))
    if ft == 0:  # FP16S
        fdefs = ["#define fpxx half", "#define fpxx_copy ushort",
                 "#define load(p,o) vload_half(o,p)*3.0517578E-5f",
                 "#define store(p,o,x) vstore_half_rte((x)*32768.0f,o,p)"]
    elif ft == 1:  # FP16C
        fdefs = ["#define fpxx ushort", "#define fpxx_copy ushort",
                 "#define load(p,o) half_to_float_custom(p[o])",
                 "#define store(p,o,x) p[o]=float_to_half_custom(x)"]
    else:
        fdefs = ["#define fpxx float", "#define fpxx_copy float",
                 "#define load(p,o) p[o]", "#define store(p,o,x) p[o]=x"]
    lines = [
        "// generated by oracle/build.py (restates get_device_defines, src/lbm/domain.rs:736-858)",
        "#define DEF_NX ionref::g_nx", "#define DEF_NY ionref::g_ny", "#define DEF_NZ ionref::g_nz",
        "#define DEF_N ionref::g_n",
        "#define DEF_DX 1u", "#define DEF_DY 1u", "#define DEF_DZ 1u", "#define DEF_DI 0u",
        "#define DEF_OX ionref::g_ox", "#define DEF_OY ionref::g_oy", "#define DEF_OZ ionref::g_oz",
        "#define DEF_AX ionref::g_ax", "#define DEF_AY ionref::g_ay", "#define DEF_AZ ionref::g_az",
        "#define DEF_DOMAIN_OFFSET_X ionref::g_dox", "#define DEF_DOMAIN_OFFSET_Y ionref::g_doy",
        "#define DEF_DOMAIN_OFFSET_Z ionref::g_doz",
        f"#define {name}",
        f"#define DEF_VELOCITY_SET {q}u", f"#define DEF_DIMENSIONS {dims}u", f"#define DEF_TRANSFERS {transfers}u",
        "#define DEF_C 0.57735027f", "#define DEF_W ionref::g_w",
        *weights,
        "#define TRT" if int(cfg.get("relaxation_time", 0)) == 1 else "#define SRT",
        "#define TYPE_S  0x01", "#define TYPE_E  0x02", "#define TYPE_C  0x04", "#define TYPE_F  0x08",
        "#define TYPE_M  0x10", "#define TYPE_G  0x20", "#define TYPE_X  0x40", "#define TYPE_Y  0x80",
        "#define TYPE_MS 0x03", "#define TYPE_BO 0b00011111",
        *fdefs,
    ]
    if cfg.get("ext_equilibrium_boundaries"):
        lines.append("#define EQUILIBRIUM_BOUNDARIES")
    if cfg.get("ext_volume_force"):
        lines.append("#define VOLUME_FORCE")
    if cfg.get("ext_magneto_hydro"):
        d = int(cfg.get("mhd_lod_depth", 4))
        lines += ["#define MAGNETO_HYDRO", "#define DEF_KE ionref::g_ke", "#define DEF_KMU ionref::g_kmu",
                  "#define DEF_KMU0 ionref::g_kmu0", "#define DEF_KKGE ionref::g_kkge",
                  "#define DEF_KIMG ionref::g_kimg", "#define DEF_KVEV ionref::g_kvev",
                  "#define DEF_KME ionref::g_kme", f"#define DEF_LOD_DEPTH {d}u",
                  "#define DEF_NUM_LOD ionref::g_num_lod", "#define DEF_NUM_LOD_OWN ionref::g_num_lod_own",
                  "#define DEF_WQ ionref::g_wq"]
    if cfg.get("ext_subgrid_ecr") and cfg.get("ext_magneto_hydro"):
        lines += ["#define SUBGRID_ECR", "#define DEF_KKBME ionref::g_kkbme", "#define DEF_KEABS ionref::g_keabs"]
    if cfg.get("ext_force_field"):
        lines.append("#define FORCE_FIELD")
    if cfg.get("update_fields"):
        lines.append("#define UPDATE_FIELDS")
    return "\n".join(lines) + "\n"


def reference_available() -> bool:
    return generate_reference_body()


def build_reference(cfg: dict) -> Path | None:
    """Compile (once) the reference kernels for the switches in cfg."""
    if not generate_reference_body():
        return None
    key = variant_key(cfg)
    hdr = REF / f"variant_{key}.h"
    text = variant_header(cfg)
    if not hdr.exists() or hdr.read_text() != text:
        hdr.write_text(text)
    so = REF / f"libionref_{key}.so"
    deps = [BODY, hdr, SHIM / "ion_ref_host.cpp", SHIM / "ion_ref_compat.hpp", INCLUDE / "ionsolver.h"]
    if so.exists() and so.stat().st_mtime >= max(d.stat().st_mtime for d in deps):
        return so
    tmp = so.with_suffix(f".{os.getpid()}.tmp")
    _run([CXX, "-std=c++20", *COMMON_FLAGS, "-w", f"-I{REF}", f"-I{SHIM}", f"-I{INCLUDE}",
          f'-DION_REF_VARIANT="variant_{key}.h"', str(SHIM / "ion_ref_host.cpp"), "-o", str(tmp)])
    os.replace(tmp, so)
    return so


def main() -> int:
    if "--reference" in sys.argv:
        os.environ["ION_REFERENCE_ROOT"] = sys.argv[sys.argv.index("--reference") + 1]
    print(build_oracle(force="--force" in sys.argv))
    print("reference kernels available:", reference_available())
    return 0


if __name__ == "__main__":
    sys.exit(main())
