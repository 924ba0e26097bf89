"""Build recipe for libgas_gb300.so (sm_103a), in-tree.

Every translation unit is compiled by nvcc for ``-gencode
arch=compute_103a,code=sm_103a`` (host code by the same nvcc/g++), in
parallel, into ``vertexapi2_gb300/_build/`` and linked into one shared
library exporting the C ABI declared in ``include/gas_gb300.h`` and
``include/gas_gb300_core.h``.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(BUILD, "libgas_gb300.so")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-fvisibility=hidden",
          "-I", INCLUDE, "-I", CSRC]


def sources() -> list[str]:
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


def headers() -> list[str]:
    return (glob.glob(os.path.join(INCLUDE, "**", "*.h"), recursive=True)
            + glob.glob(os.path.join(INCLUDE, "**", "*.cuh"), recursive=True)
            + glob.glob(os.path.join(CSRC, "*.h")))


_ZLIB = None


def zlib_available() -> bool:
    """Whether zlib's header and library are present (gzip graph files)."""
    global _ZLIB
    if _ZLIB is None:
        prog = "#include <zlib.h>\nint main() { return gzopen(0, 0) != 0; }\n"
        try:
            r = subprocess.run(["g++", "-x", "c++", "-", "-lz", "-o", os.devnull], input=prog,
                               capture_output=True, text=True, timeout=60)
            _ZLIB = r.returncode == 0
        except (OSError, subprocess.SubprocessError):
            _ZLIB = False
    return _ZLIB


def _compile(src: str, extra: list[str]) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    zl = ["-DGAS_HAVE_ZLIB"] if zlib_available() else []
    cmd = [NVCC] + ARCH + COMMON + zl + extra + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, extra: list[str] | None = None) -> str:
    extra = extra or []
    srcs = sources()
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(p) <= t for p in srcs + headers()):
            return LIB
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 1))) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), srcs))
    tmp = LIB + ".tmp"
    cmd = [NVCC] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"] + (["-lz"] if zlib_available() else [])
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="-f" in sys.argv))
