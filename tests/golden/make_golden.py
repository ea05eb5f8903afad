"""Generate the golden fixtures in tests/golden/ from the reference's own CPU code.

Run in a container where the reference tree is mounted (it is compiled into
oracle/_ref/ by oracle/build.py; nothing of it is copied here):

    python tests/golden/make_golden.py

Outputs (small .npz files, committed):
  rng_streams.npz  generateRandomVectors N(0,1) and N(0,1/16), the +-1 diagonal
                   stream and the 255-entry bool bitmap, as the reference's
                   randomVectorGenerator.cpp / libstdc++ produce them
  goldstandard.npz a 512 x 64 clustered base, 8 queries, and the top-32 ids and
                   -cos distances written by GoldStandard/goldstandard.cpp
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import build as obuild  # noqa: E402
from lshongpu_gb300 import datasets  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref")


def rng(kind: int, count: int, extra: int | None = None, dtype=np.float32) -> np.ndarray:
    cmd = [os.path.join(REF, "rng_driver"), str(kind), str(count)] + ([str(extra)] if extra else [])
    out = subprocess.run(cmd, capture_output=True, check=True).stdout
    return np.frombuffer(out, dtype=dtype).copy()


def write_text(path: str, x: np.ndarray) -> None:
    with open(path, "w") as f:
        f.write(f"{x.shape[0]}\n{x.shape[1]}\n")
        for i, row in enumerate(x):
            f.write(f"{i} " + " ".join(f"{v:.9g}" for v in row) + " \n")


def parse_truth(path: str, nq: int, k: int):
    ids = np.empty((nq, k), np.int32)
    ds = np.empty((nq, k), np.float32)
    with open(path) as f:
        toks = f.read().split()
    assert int(toks[0]) == nq and int(toks[1]) == k
    p = 2
    for q in range(nq):
        assert toks[p].endswith(":")
        p += 1
        for j in range(k):
            ids[q, j] = int(toks[p])
            ds[q, j] = float(toks[p + 1])
            p += 2
    return ids, ds


def main() -> None:
    if not obuild.reference_available():
        raise SystemExit("reference tree not mounted: fixtures can only be regenerated where it is")
    obuild.build()
    np.savez_compressed(
        os.path.join(HERE, "rng_streams.npz"),
        normals=rng(0, 8192),
        jl16=rng(1, 2048, 16),
        plus_minus=rng(2, 3072, dtype=np.int32),
        bools=rng(3, 255, dtype=np.uint8),
    )
    x = datasets.clustered(512, 64, seed=11, count=16)
    q = datasets.clustered(8, 64, seed=12, count=16)
    with tempfile.TemporaryDirectory() as td:
        xf, qf, tf = (os.path.join(td, n) for n in ("data.txt", "queries.txt", "truth.txt"))
        write_text(xf, x)
        write_text(qf, q)
        subprocess.run([os.path.join(REF, "goldstandard"), "32", xf, qf, tf], capture_output=True, check=True)
        ids, ds = parse_truth(tf, q.shape[0], 32)
    np.savez_compressed(os.path.join(HERE, "goldstandard.npz"), data=x, queries=q, ids=ids, dists=ds)
    print("wrote", os.listdir(HERE))


if __name__ == "__main__":
    main()
