"""Builds libns_gb300.so in-tree with nvcc for sm_103a.

The library is plain CUDA C++ behind the C ABI of include/ns_gb300.h (no
PyTorch types), so it is compiled with nvcc directly: one object per
translation unit, in parallel, then linked as a shared object next to this
file.  Rebuilds only when a source or header is newer than the library.

build(checked=True) makes the checked build instead, libns_gb300_checked.so
(-DNS_CHECKED): every kernel range-checks the tile, halo, segment and
work-list indices it derives and reports a failed check as NS_ERR_CHECK
(navierstokes_gb300/csrc/ns_check.cuh).  Setting NS_GB300_LIB to its path
makes the Python binding load it in place of the ordinary library.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIB = PKG / "libns_gb300.so"
LIB_CHECKED = PKG / "libns_gb300_checked.so"
DRIVER = PKG / "ns_euler"
BUILD_DIR = PKG / "_build"
BUILD_DIR_CHECKED = PKG / "_build_checked"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-fvisibility=hidden", "--expt-relaxed-constexpr"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libns_gb300.so")


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False, checked: bool = False) -> Path:
    srcs = sources()
    headers = (list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) +
               list((ROOT / "include").glob("*.h")))
    drv = [CSRC / "main" / "ns_euler.cpp"]
    lib = LIB_CHECKED if checked else LIB
    bdir = BUILD_DIR_CHECKED if checked else BUILD_DIR
    defs = ["-DNS_CHECKED"] if checked else []
    if not force and not _stale(lib, srcs + headers + [Path(__file__)]):
        if not checked and _stale(DRIVER, drv + [LIB]):
            _build_driver()
        return lib
    nvcc = _nvcc()
    bdir.mkdir(exist_ok=True)

    def compile_one(src: Path) -> Path:
        obj = bdir / (src.stem + ".o")
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, *defs, "-I", str(ROOT / "include"), "-c", str(src),
               "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 1))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = lib.with_suffix(".so.tmp")
    cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link of {lib.name} failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    if not checked:
        _build_driver()
    return lib


def _build_driver() -> None:
    """ns_euler, the euler.f90 program over the library (rpath $ORIGIN)."""
    src = CSRC / "main" / "ns_euler.cpp"
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        raise RuntimeError("a C++ compiler is required to build ns_euler")
    tmp = DRIVER.with_suffix(".tmp")
    cmd = [cxx, "-O2", "-std=c++17", "-I", str(ROOT / "include"), str(src), "-o", str(tmp),
           "-L", str(PKG), "-lns_gb300", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build of ns_euler failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, DRIVER)


if __name__ == "__main__":
    print(build(verbose=True, force=True))
