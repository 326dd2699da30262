"""Builds libfsk.so in-tree from csrc/*.cu for sm_103a (GB300).

Each translation unit is compiled by its own nvcc process (in parallel),
without relocatable device code except the units in RDC_UNITS (chosen by
measurement), then linked with ``nvcc -shared`` (with the device link step
for those units).  The CUDA runtime is linked statically so the
library does not depend on the exact libcudart the host process has loaded.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG_ROOT = Path(__file__).resolve().parent.parent          # flash-sd-kde_gb300/
CSRC = PKG_ROOT / "csrc"
INCLUDE = PKG_ROOT.parent / "include"
BUILD_DIR = PKG_ROOT / "_build"
LIB_PATH = Path(__file__).resolve().parent / "libfsk.so"
# The bounds-check build (-DFSK_BOUNDS_CHECK: the hot kernels check their
# global write indices and report FSK_ERR_DEVICE_BOUNDS instead of writing
# out of range) goes to its own library and object directory.
CHECKED_BUILD_DIR = PKG_ROOT / "_build_checked"
CHECKED_LIB_PATH = Path(__file__).resolve().parent / "libfsk_checked.so"
CHECKED_FLAGS = ["-DFSK_BOUNDS_CHECK"]

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
]


# Units compiled as relocatable device code (a device link step joins them):
# measured on the GB300, the tensor-core KDE kernel runs 1.7 % faster built
# this way (186.6 vs 189.8 ms at n = m = 2^20) and the score kernel 1.9 %
# slower (410.2 vs 402.6 ms); the other units do not care.  No unit
# references device symbols of another, so both modes link.
RDC_UNITS = {"fsk_tc_kde16"}


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found; the CUDA 13 toolkit is required to build libfsk.so")


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _stale(extra_flags: list[str], lib_path: Path = LIB_PATH, build_dir: Path = BUILD_DIR) -> bool:
    if not lib_path.exists():
        return True
    stamp = build_dir / "flags.txt"
    if not stamp.exists() or stamp.read_text() != " ".join(NVCC_FLAGS + extra_flags + sorted(RDC_UNITS)):
        return True
    lib_mtime = lib_path.stat().st_mtime
    deps = list(CSRC.glob("*")) + list(INCLUDE.glob("*.h"))
    return any(p.stat().st_mtime > lib_mtime for p in deps)


def build(force: bool = False, verbose: bool = False, extra_flags: list[str] | None = None,
          checked: bool = False) -> Path:
    """Compile every csrc/*.cu for sm_103a and link libfsk.so (checked=True:
    the bounds-check build, libfsk_checked.so); returns the library's path."""
    extra_flags = list(extra_flags or []) + (CHECKED_FLAGS if checked else [])
    lib_path = CHECKED_LIB_PATH if checked else LIB_PATH
    build_dir = CHECKED_BUILD_DIR if checked else BUILD_DIR
    if not force and not _stale(extra_flags, lib_path, build_dir):
        return lib_path
    nvcc = _nvcc()
    build_dir.mkdir(exist_ok=True)
    srcs = sources()

    def compile_one(src: Path) -> Path:
        obj = build_dir / (src.stem + ".o")
        rdc = ["-rdc=true"] if src.stem in RDC_UNITS else []
        cmd = [nvcc, *ARCH_FLAGS, *NVCC_FLAGS, *rdc, *extra_flags, f"-I{INCLUDE}", "-c", str(src), "-o", str(obj)]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src.name}:\n{res.stdout}\n{res.stderr}")
        if verbose and (res.stdout or res.stderr):
            sys.stderr.write(res.stdout + res.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = lib_path.with_suffix(".so.tmp")
    link_rdc = ["-rdc=true"] if any(o.stem in RDC_UNITS for o in objs) else []
    cmd = [nvcc, *ARCH_FLAGS, *link_rdc, "-shared", "-o", str(tmp), *map(str, objs)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, lib_path)
    (build_dir / "flags.txt").write_text(" ".join(NVCC_FLAGS + extra_flags + sorted(RDC_UNITS)))
    return lib_path


if __name__ == "__main__":
    v = "-v" in sys.argv
    extra = ["-Xptxas", "-v"] if "--ptxas-v" in sys.argv else []
    print(build(force=True, verbose=v or bool(extra), extra_flags=extra, checked="--checked" in sys.argv))
