"""Build recipe for the oracle (test infrastructure only).

Two libraries, both outside the product:

* ``oracle/_build/libgas_oracle.so`` -- the C restatement of the
  reference's CPU engine (gas_oracle.c).  Built here and on any machine
  with gcc; it is the checker in tests/, smoke() and bench.py's CPU legs.
* ``oracle/_ref/libgas_ref.so`` -- the reference's own CPU engine
  (refgas.h, util.h, graphio.cpp) compiled in place from the reference
  tree by g++ with ref_harness.cpp.  Only built where that tree exists
  (see ``ref_dir``); it pins the restatement and produces the golden
  vectors under tests/golden/.

Run ``python oracle/build.py`` to build both (the second only when the
reference tree is present).
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_OUT_DIR = os.path.join(HERE, "_ref")
PORT_LIB = os.path.join(BUILD_DIR, "libgas_oracle.so")
REF_LIB = os.path.join(REF_OUT_DIR, "libgas_ref.so")


REPO = os.path.dirname(HERE)
# Where this recipe looks for the reference source tree, in order: the
# GAS_REF_DIR override, an installed copy under baseline/_ref, and the
# read-only checkout that the development container mounts.
REF_DIR_CANDIDATES = (os.path.join(REPO, "baseline", "_ref"), "/root/reference")


def ref_dir() -> str:
    if os.environ.get("GAS_REF_DIR"):
        return os.environ["GAS_REF_DIR"]
    for d in REF_DIR_CANDIDATES:
        if os.path.exists(os.path.join(d, "refgas.h")):
            return d
    return REF_DIR_CANDIDATES[0]


def _newer(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources if os.path.exists(s))


def build_port(force: bool = False) -> str:
    srcs = [os.path.join(HERE, f) for f in ("gas_oracle.c", "gas_oracle_gen.c", "gas_oracle.h",
                                            "gas_oracle_engine.inc")]
    if not force and _newer(PORT_LIB, srcs):
        return PORT_LIB
    os.makedirs(BUILD_DIR, exist_ok=True)
    # -ffp-contract=off: identical FP32 results on x86-64 and aarch64
    cmd = ["gcc", "-O2", "-std=c99", "-fPIC", "-shared", "-ffp-contract=off", "-pthread",
           "-o", PORT_LIB, srcs[0], srcs[1], "-lm"]
    subprocess.run(cmd, check=True)
    return PORT_LIB


def build_ref(force: bool = False) -> str | None:
    rd = ref_dir()
    needed = [os.path.join(rd, f) for f in ("refgas.h", "util.h", "graphio.cpp", "graphio.h")]
    if not all(os.path.exists(p) for p in needed):
        return None
    harness = os.path.join(HERE, "ref_harness.cpp")
    if not force and _newer(REF_LIB, needed + [harness, os.path.join(HERE, "gas_oracle.h")]):
        return REF_LIB
    os.makedirs(REF_OUT_DIR, exist_ok=True)
    # graphio.cpp unoptimised and without unreachable traps:
    # loadGraph_binaryCSR (graphio.cpp:274-362) has no return statement;
    # g++ 13 turns falling off its end into a crash (-O2: stack corruption;
    # -O0 by default: a trap instruction) whenever a .gr file is read.  This
    # way it returns an unused garbage value, as older compilers did.
    gio = os.path.join(REF_OUT_DIR, "graphio.o")
    subprocess.run(["g++", "-O0", "-fno-unreachable-traps", "-std=c++17", "-fPIC", "-w", "-I", rd, "-c",
                    os.path.join(rd, "graphio.cpp"), "-o", gio], check=True)
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-w",
           "-I", rd, "-I", HERE, "-o", REF_LIB, harness, gio, "-lz"]
    subprocess.run(cmd, check=True)
    return REF_LIB


if __name__ == "__main__":
    print(build_port(force="-f" in sys.argv))
    print(build_ref(force="-f" in sys.argv) or "reference tree absent: oracle/_ref not built")
