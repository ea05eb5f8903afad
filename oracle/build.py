"""Build the CPU oracle (test infrastructure) and, where the reference tree exists,
the reference's own CPU code under oracle/_ref/.

  oracle/build/liboracle.so   oracle.c + gold_port.cpp (gcc/g++, -ffp-contract=off)
  oracle/_ref/rng_driver      LinearScan/randomVectorGenerator.cpp + ref_drivers/rng_driver.cpp
  oracle/_ref/goldstandard    GoldStandard/goldstandard.cpp, unmodified

The reference sources are compiled where they lie (read-only); nothing of them is
copied into this repository.  Outputs of the reference build go to oracle/_ref only.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "build")
REF_OUT = os.path.join(HERE, "_ref")
REFERENCE = os.environ.get("LSHG_REFERENCE_TREE", "/root/reference")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def lib_path() -> str:
    return os.path.join(BUILD, "liboracle.so")


def build_oracle() -> str:
    os.makedirs(BUILD, exist_ok=True)
    c_obj = os.path.join(BUILD, "oracle.o")
    cpp_obj = os.path.join(BUILD, "gold_port.o")
    flags = ["-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math"]
    _run(["gcc", *flags, "-std=gnu11", "-pthread", "-c", os.path.join(HERE, "oracle.c"), "-o", c_obj])
    _run(["g++", *flags, "-std=c++17", "-pthread", "-c", os.path.join(HERE, "gold_port.cpp"), "-o", cpp_obj])
    out = lib_path()
    _run(["g++", "-shared", "-pthread", "-o", out + ".tmp", c_obj, cpp_obj, "-lm"])
    os.replace(out + ".tmp", out)
    return out


def reference_available() -> bool:
    return os.path.isdir(os.path.join(REFERENCE, "LinearScan"))


def build_reference() -> list[str]:
    """Compile the reference's CPU code (only where the reference tree is mounted)."""
    if not reference_available():
        return []
    os.makedirs(REF_OUT, exist_ok=True)
    ls = os.path.join(REFERENCE, "LinearScan")
    outs = []
    rng = os.path.join(REF_OUT, "rng_driver")
    _run(["g++", "-O2", "-std=c++11", "-o", rng, os.path.join(HERE, "ref_drivers", "rng_driver.cpp"),
          os.path.join(ls, "randomVectorGenerator.cpp")])
    outs.append(rng)
    gs = os.path.join(REF_OUT, "goldstandard")
    _run(["g++", "-O2", "-std=c++11", "-o", gs, os.path.join(REFERENCE, "GoldStandard", "goldstandard.cpp")])
    outs.append(gs)
    return outs


def build(with_reference: bool = True) -> str:
    out = build_oracle()
    if with_reference:
        build_reference()
    return out


if __name__ == "__main__":
    print(build())
    if reference_available():
        print("reference CPU code built into", REF_OUT)
    sys.exit(0)
