"""Build the engine library in-tree: lmweather_gb300/_lib/liblmw_gb300.so (sm_103a only).

Each translation unit compiles in parallel; the plane kernels use --fmad=false (bitwise parity with the
reference's unfused arithmetic) and every host file -ffp-contract=off (table construction and seeded
initialisers reproduce the reference's arithmetic exactly). Portable host flags only: the same recipe builds
on x86_64 and aarch64.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(HERE, "_lib", "obj")
LIB = os.path.join(OUT_DIR, "liblmw_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# (source, extra flags)
UNITS = [
    ("plane.cu", ["--fmad=false", "-Xcompiler=-ffp-contract=off"]),
    ("sphere.cu", []),
    ("ensemble.cu", []),
    ("capi.cu", []),
    ("tc_gemm.cu", []),
    ("surrogate.cu", []),
    ("sphere_tables.cpp", []),
    ("wx_capi.cpp", []),
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build lmweather_gb300")


def _deps() -> list[str]:
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    inc = os.path.join(ROOT, "include")
    files += [os.path.join(inc, f) for f in os.listdir(inc)]
    files.append(os.path.abspath(__file__))
    return files


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _compile(src: str, extra: list[str]) -> str:
    path = os.path.join(CSRC, src)
    obj = os.path.join(OBJ_DIR, src + ".o")
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-I" + CSRC,
              "-I" + os.path.join(ROOT, "include")]
    if src.endswith(".cu"):
        cmd = [nvcc(), *ARCH, "-lineinfo", "-Xptxas", "-v" if os.environ.get("LMW_PTXAS_V") else "-O3", *common, *extra,
               "-c", path, "-o", obj]
    else:
        cmd = [nvcc(), "-x", "c++", *common, *extra, "-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compiling {src} failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if os.environ.get("LMW_PTXAS_V") and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile every translation unit (in parallel) and link the shared library. Returns its path."""
    os.makedirs(OBJ_DIR, exist_ok=True)
    units = [(s, f) for s, f in UNITS if os.path.exists(os.path.join(CSRC, s))]
    deps = _deps()
    todo = [(s, f) for s, f in units if force or _stale(os.path.join(OBJ_DIR, s + ".o"), deps)]
    if todo:
        with ThreadPoolExecutor(max_workers=min(8, len(todo))) as ex:
            list(ex.map(lambda sf: _compile(*sf), todo))
    objs = [os.path.join(OBJ_DIR, s + ".o") for s, _ in units]
    if force or todo or _stale(LIB, objs):
        tmp = LIB + ".tmp"
        cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"linking failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
