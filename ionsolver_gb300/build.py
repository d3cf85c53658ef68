"""Builds libionsolver.so (the sm_103a kernels and the C ABI) in-tree with nvcc.

Translation units are compiled in parallel and linked into
``ionsolver_gb300/_build/libionsolver.so``.  Arithmetic flags are part of the
contract with the reference: no FMA contraction (-fmad=false) except where
the code calls fmaf(), IEEE division and square root, no flush-to-zero; the
host side is compiled with -ffp-contract=off for the same reason.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
REPO = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
LIB = OUT / "libionsolver.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
              "-Xcompiler", "-fPIC,-ffp-contract=off", "-Xptxas", "-v", f"-I{REPO / 'include'}", f"-I{CSRC}"]
SOURCES = ["lbm_q19.cu", "lbm_q15.cu", "lbm_q9.cu", "field_kernels.cu", "setup_kernels.cu", "batch_kernels.cu",
           "noalloc.cu", "surrogate.cu", "config_json.cpp", "ion_api.cu"]
# (source, object name, extra flags): one translation unit compiled more than once
VARIANTS = [("lbm_q19_sc.cu", f"lbm_q19_sc_{ft.lower()}", [f"-DION_SC_FT=ION_{ft}"]) for ft in ("FP32", "FP16S", "FP16C")]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and Path(c).exists():
            return c
    raise RuntimeError("nvcc not found")


def _compile(src: Path, obj: Path, extra: list[str] | None = None) -> str:
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *(extra or []), "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")
    return r.stderr


def _stale(obj: Path, deps: list[Path]) -> bool:
    return not obj.exists() or obj.stat().st_mtime < max(d.stat().st_mtime for d in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    OUT.mkdir(parents=True, exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + [REPO / "include" / "ionsolver.h"]
    units = [(s, Path(s).stem, []) for s in SOURCES] + VARIANTS
    jobs = []
    for s, stem, extra in units:
        src = CSRC / s
        obj = OUT / (stem + ".o")
        if force or _stale(obj, [src, *headers]):
            jobs.append((src, obj, extra))
    if jobs:
        # the largest units first, so the longest compile starts at once
        jobs.sort(key=lambda j: 0 if j[0].name.startswith("lbm_q19") or j[0].name == "batch_kernels.cu" else 1)
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            logs = list(ex.map(lambda j: _compile(*j), jobs))
        (OUT / "ptxas.log").write_text("\n".join(logs))
        if verbose:
            print("\n".join(logs))
    objs = [OUT / (stem + ".o") for _, stem, _ in units]
    if force or jobs or not LIB.exists():
        tmp = LIB.with_suffix(f".{os.getpid()}.tmp")
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
