"""Build libsunnygb300.so in-tree for sm_103a with nvcc (no cmake).

Each translation unit is compiled in parallel into ``_build/`` and linked with
cuFFT. The product is ``sunny.jl_gb300/libsunnygb300.so``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libsunnygb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# (source, object name, extra flags): the two largest units are built once per precision
SOURCES = [("sgb_api.cu", "sgb_api", []), ("sgb_dipole.cu", "sgb_dipole_f32", ["-DSGB_INST_PRECISION=32"]),
           ("sgb_dipole.cu", "sgb_dipole_f64", ["-DSGB_INST_PRECISION=64"]),
           ("sgb_sun.cu", "sgb_sun_f32", ["-DSGB_INST_PRECISION=32"]), ("sgb_sun.cu", "sgb_sun_f64", ["-DSGB_INST_PRECISION=64"]),
           ("sgb_corr.cu", "sgb_corr", []), ("sgb_tdft.cu", "sgb_tdft", []), ("sgb_batch.cu", "sgb_batch", []), ("sgb_batch_blk.cu", "sgb_batch_blk", []),
           ("sgb_static.cu", "sgb_static", []),
           ("sgb_adjoint.cu", "sgb_adjoint", []), ("sgb_mc.cu", "sgb_mc", []), ("sgb_opt.cu", "sgb_opt", []),
           ("sgb_ewald.cu", "sgb_ewald", [])]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libsunnygb300.so")


def _compile(entry, extra: list[str]) -> Path:
    src, name, flags = entry
    obj = BUILD / (name + ".o")
    deps = [CSRC / src] + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + [PKG.parent / "include" / "sunny_gb300.h"]
    if obj.exists() and all(obj.stat().st_mtime >= d.stat().st_mtime for d in deps if d.exists()):
        return obj
    cmd = [nvcc(), *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-c",
           str(CSRC / src), "-o", str(obj), *flags, *extra]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False, extra: list[str] | None = None) -> Path:
    BUILD.mkdir(exist_ok=True)
    extra = extra or []
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), SOURCES))
    if LIB.exists() and all(LIB.stat().st_mtime >= o.stat().st_mtime for o in objs):
        return LIB
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcufft", "-lcudart",
           "-Xlinker", "-rpath", "-Xlinker", "/usr/local/cuda/lib64"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(f"built {LIB}", file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
