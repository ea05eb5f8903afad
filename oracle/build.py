"""Build the CPU oracle (test infrastructure) and, where the reference tree exists,
the reference's own CPU code under oracle/_ref/.

  oracle/build/liboracle.so   oracle.c + gold_port.cpp (gcc/g++, -ffp-contract=off)
  oracle/_ref/rng_driver      LinearScan/randomVectorGenerator.cpp + ref_drivers/rng_driver.cpp
  oracle/_ref/goldstandard    GoldStandard/goldstandard.cpp, unmodified
  oracle/_ref/parse_driver    LinearScan/gloveparser.cu (host code, nvcc) + ref_drivers/parse_driver.cpp

The reference sources are compiled where they lie (read-only); nothing of them is
copied into this repository.  Outputs of the reference build go to oracle/_ref only.
"""
from __future__ import annotations

import os
import shutil
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
    # the text reader is host code in a .cu file that includes thrust: nvcc for it, g++
    # for the driver, nvcc to link
    nvcc = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    gp_obj = os.path.join(REF_OUT, "gloveparser.o")
    pd_obj = os.path.join(REF_OUT, "parse_driver.o")
    pd = os.path.join(REF_OUT, "parse_driver")
    _run([nvcc, "-O2", "-std=c++17", "-w", "-c", os.path.join(ls, "gloveparser.cu"), "-o", gp_obj])
    _run(["g++", "-O2", "-c", os.path.join(HERE, "ref_drivers", "parse_driver.cpp"), "-o", pd_obj])
    _run([nvcc, gp_obj, pd_obj, "-o", pd])
    outs.append(pd)
    return outs


# Reference kernels driven by oracle/ref_harness.cpp: (tag, translation unit, demangled signature)
REF_KERNELS = [
    ("knn", "memOptimizedLinearScan.cu", "knn(float*, float*, int, int, int, int, Point*, int)"),
    ("simhash_sketch", "simHash.cu", "simHash::sketch(float*, float*, int, int, int, unsigned int*)"),
    ("crosspoly", "kernel.cu", "void crosspoly::generateHashCrossPoly<float, unsigned short>(LaunchDTO<float>, "
                               "float*, unsigned short*, int, int, int*, float*, float*, int)"),
    ("wmh_byte", "kernel.cu", "void weightedMinHash::sketchDataOriginal<unsigned char, unsigned char>("
                              "LaunchDTO<unsigned char>, float*, int, int, int*, int*, int, int*, unsigned char*)"),
    ("wmh_onebit", "kernel.cu", "void weightedMinHash::sketchDataOneBit<unsigned int, unsigned int>("
                                "LaunchDTO<unsigned int>, float*, int, int, int, int*, int*, int, int*, bool*, "
                                "unsigned int*)"),
    ("jl_sketch", "kernel.cu", "void simHashJl::sketch<float>(LaunchDTO<float>, float*, float*, int, float*)"),
]


def build_reference_gpu() -> list[str]:
    """Compile the reference's GPU translation units, unmodified, to sm_103a cubins in
    oracle/_ref/ (device code only; nothing of the reference is copied), and record the
    mangled names of the kernels the harness drives (read from the symbol table of host
    objects compiled from the same sources)."""
    if not reference_available():
        return []
    os.makedirs(REF_OUT, exist_ok=True)
    if os.path.exists(os.path.join(REF_OUT, "ref_kernels.txt")) and not os.environ.get("LSHG_REBUILD_REF"):
        return [os.path.join(REF_OUT, f) for f in os.listdir(REF_OUT) if f.endswith(".cubin")]
    ls = os.path.join(REFERENCE, "LinearScan")
    nvcc = os.environ.get("NVCC", "nvcc")
    # template kernels keep external linkage so the harness can look them up by name
    flags = ["-std=c++17", "-O3", "-include", "cuda.h", "-I" + ls, "-w", "-static-global-template-stub=false"]
    outs = []
    names = {}
    for tu in sorted({k[1] for k in REF_KERNELS}):
        stem = os.path.splitext(tu)[0]
        cubin = os.path.join(REF_OUT, f"ref_{stem}.cubin")
        _run([nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", *flags, os.path.join(ls, tu), "-o", cubin])
        outs.append(cubin)
        obj = os.path.join(REF_OUT, f"host_{stem}.o")
        _run([nvcc, "-c", "-gencode", "arch=compute_103a,code=sm_103a", *flags, os.path.join(ls, tu), "-o", obj])
        syms = subprocess.run(["nm", "--defined-only", obj], capture_output=True, text=True, check=True).stdout
        mangled = [line.split()[-1] for line in syms.splitlines() if len(line.split()) >= 3]
        dem = subprocess.run(["c++filt"], input="\n".join(mangled), capture_output=True, text=True,
                             check=True).stdout.splitlines()
        for tag, unit, sig in REF_KERNELS:
            if unit != tu:
                continue
            for m, d in zip(mangled, dem):
                if d == sig:
                    names[tag] = (f"ref_{stem}.cubin", m)
        os.remove(obj)
    missing = [t for t, _, _ in REF_KERNELS if t not in names]
    if missing:
        raise RuntimeError("reference kernels not found in the symbol tables: " + ", ".join(missing))
    with open(os.path.join(REF_OUT, "ref_kernels.txt"), "w") as f:
        for tag, (cubin, m) in sorted(names.items()):
            f.write(f"{tag} {cubin} {m}\n")
    return outs


def harness_path() -> str:
    return os.path.join(BUILD, "libref_harness.so")


def build_harness() -> str:
    """The driver-API harness that runs the reference cubins (needs only the CUDA
    toolkit; the cubins come prebuilt from oracle/_ref)."""
    os.makedirs(BUILD, exist_ok=True)
    out = harness_path()
    nvcc = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    stubs = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "lib64", "stubs")
    _run([nvcc, "-O2", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", "-o", out + ".tmp",
          os.path.join(HERE, "ref_harness.cpp"), "-L" + stubs, "-lcuda"])
    os.replace(out + ".tmp", out)
    return out


def build(with_reference: bool = True) -> str:
    out = build_oracle()
    build_harness()
    if with_reference:
        build_reference()
        build_reference_gpu()
    return out


if __name__ == "__main__":
    print(build())
    if reference_available():
        print("reference CPU code built into", REF_OUT)
    sys.exit(0)
