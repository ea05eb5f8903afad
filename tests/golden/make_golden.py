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
  text_reader.npz  text files in the reference's dataset format (writer output and
                   files that exercise the reader's rules) and the values that
                   LinearScan/gloveparser.cu's parseFile reads from them
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


def reader_cases() -> list[bytes]:
    """Dataset files for the text reader; each stores exactly n * d values, so that every
    entry the reference reader returns is set."""
    rng_ = np.random.default_rng(3)
    w = (rng_.standard_normal((6, 5)) * 40).astype(np.float32)
    writer = "6\n5\n" + "".join(f"{i} " + "".join(f"{v:.6f} " for v in row) + "\n" for i, row in enumerate(w))
    long_frac = "2\n2\n0 0.12345678901234567890123456789 -0.99999999999999999999 \n1 3.000000000000000000001 7.5 \n"
    return [
        writer.encode(),
        b"3\n4\n0 12.5 -3.25 0.125 1e3 \n1 1.2.3 3-4 +7 a9 \n2  0.1 0.000001 99.999999999999 \n",
        b"2\n2\n0 1.5 2.5 -9\n1 3.5 4.5 \n",                       # a dropped '-' field
        b"2\r\n2\r\n0 0.5 0.25 \r\n1 -0.75 1.0\r \r\n",              # CR line ends
        long_frac.encode(),
        b"2\n3\n 5.5 6.5 -0 \n\n-12.5 0.0625 .5 5. \n",                 # empty id, empty line
        b"1\n4\n0 2\xc3\xa95 -\x001.5 1,5 9.-9 ",                      # other bytes, no final newline
    ]


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
    texts, shapes, vals = [], [], []
    with tempfile.TemporaryDirectory() as td:
        for i, text in enumerate(reader_cases()):
            path = os.path.join(td, f"case{i}.txt")
            with open(path, "wb") as f:
                f.write(text)
            out = subprocess.run([os.path.join(REF, "parse_driver"), path], capture_output=True, check=True).stdout
            n, d = np.frombuffer(out[:8], np.int32)
            texts.append(np.frombuffer(text, np.uint8))
            shapes.append((n, d))
            vals.append(np.frombuffer(out[8:], np.float32))
    np.savez_compressed(os.path.join(HERE, "text_reader.npz"),
                        text=np.concatenate(texts), text_len=np.array([len(t) for t in texts], np.int64),
                        shape=np.array(shapes, np.int32), values=np.concatenate(vals))
    print("wrote", os.listdir(HERE))


if __name__ == "__main__":
    main()
