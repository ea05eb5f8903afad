"""Build liblshg.so (the engine's C-ABI shared library) in-tree for sm_103a.

Every translation unit under csrc/ is compiled by nvcc in parallel with one
-gencode (compute_103a -> sm_103a) and linked into lshongpu_gb300/lib/liblshg.so.
Objects are cached by source/flags hash so rebuilds only touch changed files.
"""
from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
OBJDIR = os.path.join(LIBDIR, "obj")
LIBNAME = "liblshg.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = [
    "-O3",
    "-std=c++17",
    "-lineinfo",
    "-Xcompiler",
    "-fPIC,-ffp-contract=off",
    "--expt-relaxed-constexpr",
    "-I" + os.path.join(ROOT, "include"),
    "-I" + CSRC,
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the lshg engine needs the CUDA 13 toolkit to build")


def sources() -> list[str]:
    return sorted(
        os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp"))
    )


def _headers_digest() -> str:
    h = hashlib.sha256()
    for d in (CSRC, os.path.join(ROOT, "include")):
        for f in sorted(os.listdir(d)):
            if f.endswith((".h", ".cuh")):
                with open(os.path.join(d, f), "rb") as fh:
                    h.update(f.encode() + fh.read())
    return h.hexdigest()


def _compile(src: str, hdr: str, verbose: bool) -> str:
    with open(src, "rb") as fh:
        digest = hashlib.sha256(fh.read() + hdr.encode() + " ".join(ARCH + COMMON).encode()).hexdigest()[:16]
    obj = os.path.join(OBJDIR, os.path.basename(src) + "." + digest + ".o")
    if os.path.exists(obj):
        return obj
    cmd = [nvcc(), *ARCH, *COMMON, "-c", src, "-o", obj + ".tmp"]
    if src.endswith(".cpp"):
        cmd[1:1] = ["-x", "cu"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")
    os.replace(obj + ".tmp", obj)
    return obj


def lib_path() -> str:
    return os.path.join(LIBDIR, LIBNAME)


def build(verbose: bool = False, jobs: int | None = None) -> str:
    os.makedirs(OBJDIR, exist_ok=True)
    hdr = _headers_digest()
    srcs = sources()
    jobs = jobs or min(len(srcs), max(2, os.cpu_count() or 2))
    with ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, hdr, verbose), srcs))
    out = lib_path()
    tmp = out + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-cudart", "shared"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, out)
    # knn-compatible command line, linked against the library (rpath $ORIGIN)
    cli_src = os.path.join(HERE, "cli", "lshg_knn.cpp")
    cli = os.path.join(LIBDIR, "lshg_knn")
    cmd = ["g++", "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"), "-o", cli + ".tmp", cli_src,
           "-L" + LIBDIR, "-llshg", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"CLI build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(cli + ".tmp", cli)
    # drop stale objects of earlier source versions
    keep = {os.path.basename(o) for o in objs}
    for f in os.listdir(OBJDIR):
        if f.endswith(".o") and f not in keep:
            os.remove(os.path.join(OBJDIR, f))
    return out


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
