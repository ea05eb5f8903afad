"""Shared test setup.

Markers: `gpu` = needs a CUDA device (run with -m gpu on a GB300); everything else runs
on CPU.  The engine library and the CPU oracle are built on first use.
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session")
def engine():
    import lshongpu_gb300 as L
    from lshongpu_gb300 import build

    if not os.path.exists(build.lib_path()):
        build.build()
    L.lib()
    return L


@pytest.fixture(scope="session")
def orc():
    import oracle

    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def golden():
    g = os.path.join(ROOT, "tests", "golden")
    return {
        "rng": dict(np.load(os.path.join(g, "rng_streams.npz"))),
        "gold": dict(np.load(os.path.join(g, "goldstandard.npz"))),
    }


@pytest.fixture(scope="session")
def uniforms():
    """cuRAND uniforms for seeds h*1234+92138 (createSeedArr, weightedMinHash.cuh:252-262),
    from an independent test-side program; returns get(H, T) -> float32 [H][T]."""
    src = os.path.join(ROOT, "tests", "golden", "curand_uniforms.cu")
    exe = os.path.join(tempfile.mkdtemp(), "curand_uniforms")
    subprocess.run(["nvcc", "-O2", "-gencode", "arch=compute_103a,code=sm_103a", "-o", exe, src], check=True)

    def get(H, T):
        out = subprocess.run([exe, str(H), str(T)], capture_output=True, check=True).stdout
        return np.frombuffer(out, np.float32).reshape(H, T)

    return get


def ids_equal_up_to_ties(ids_a, d_a, ids_b, d_b, tol):
    """Row-wise: the id sets agree except for entries whose distance lies within `tol`
    of that row's last (k-th) distance.  Returns the number of rows that violate it."""
    bad = 0
    for ia, da, ib, db in zip(ids_a, d_a, ids_b, d_b):
        sa, sb = set(ia.tolist()), set(ib.tolist())
        if sa == sb:
            continue
        kth = max(float(da[-1]), float(db[-1]))
        diff_a = [d for i, d in zip(ia, da) if i not in sb]
        diff_b = [d for i, d in zip(ib, db) if i not in sa]
        if all(abs(float(d) - kth) <= tol for d in diff_a + diff_b):
            continue
        bad += 1
    return bad
