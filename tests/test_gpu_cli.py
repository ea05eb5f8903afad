"""End-to-end run of the knn-compatible command line (lshg_knn, the reference's 15
positional arguments) on reference-format text files, with GoldStandard-format truth."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from lshongpu_gb300 import build, datasets

pytestmark = pytest.mark.gpu


def test_cli_exact_scan_validates_and_writes_csv(engine, orc):
    x = datasets.clustered(2000, 48, 91, count=10)
    q = datasets.clustered(12, 48, 92, count=10)
    with tempfile.TemporaryDirectory() as td:
        dp, qp, tp, rp = (os.path.join(td, f) for f in ("d.txt", "q.txt", "t.txt", "r.csv"))
        engine.write_file(dp, x)
        engine.write_file(qp, q)
        xs, qs = engine.parse_file(dp), engine.parse_file(qp)  # what the program will read
        ids, ds = orc.exact_topk(xs, qs, 32, dist=1)
        truth = np.zeros(ids.shape, dtype=engine.POINT_DTYPE)
        truth["ID"], truth["distance"] = ids, ds
        engine.write_truth(tp, truth)
        exe = os.path.join(os.path.dirname(build.lib_path()), "lshg_knn")
        args = [exe, dp, qp, tp, "1", "1", "20", "2", "0", "1", "0", "0", "0", "0", "0", rp]
        out = subprocess.run(args, capture_output=True, text=True, check=True).stdout
        line = open(rp).read().strip().split(",")
    assert line[:8] == ["2", "0", "0", "32", "128", "0", "0", "0"]
    assert float(line[11]) == 1.0  # recall@20
    # printed results (writeResult format) equal the API's answer
    toks = out.split("Averge recall")[1].splitlines()
    api = engine.linear_scans(2, 32, 48, 12, 2000, xs, qs, 0, 1)
    first = toks.index("0:")
    got = [int(t.split()[0]) for t in toks[first + 1:first + 21]]
    assert got == api.ids[0, :20].tolist()
