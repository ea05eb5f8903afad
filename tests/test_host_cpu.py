"""CPU tests of the C ABI's host-side pieces: symbol table, k rounding, validation
(validation.cpp), top-k merging for shards, the reference text format
(gloveparser.cu / DataParsing writer), and the 2-rank sharded query over gloo."""
import os
import re
import socket
import tempfile

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_exports_every_declared_symbol(engine):
    hdr = open(os.path.join(ROOT, "include", "lshg.h")).read()
    declared = set(re.findall(r"\b(lshg_[a-z_0-9]+)\s*\(", hdr))
    lib = engine.lib()
    missing = [s for s in sorted(declared) if not hasattr(lib, s)]
    assert not missing
    assert declared <= set(engine.SYMBOLS)


def test_calculate_k_matches_reference(engine):
    # launchHelper.cuh:21-25: divisor = (k-1)/32; return divisor*32 + 32
    for k in [1, 10, 31, 32, 33, 64, 100, 1000, 1024]:
        assert engine.calculate_k(k) == ((k - 1) // 32) * 32 + 32


def test_version_and_options(engine):
    assert b"lshg" in engine.lib().lshg_version()
    o = engine.make_options()
    assert o.thread_queue_size == 128 and o.cp_rounds == 3 and o.cp_hashes == 1


def _validation_reference(truth, res, k, reportK):
    """validation.cpp:129-198 restated: recall by ID set, distance ratio over the result
    set (unique IDs, summed in ID order)."""
    rec_tot, rat_tot = np.float32(0), np.float32(0)
    for t, r in zip(truth, res):
        first = {}
        for p in r[:reportK]:
            first.setdefault(int(p["ID"]), np.float32(p["distance"]))
        found = sum(1 for p in t[:reportK] if int(p["ID"]) in first)
        tsum = np.float32(0)
        for p in t[:reportK]:
            tsum = np.float32(tsum + np.float32(p["distance"]))
        rsum = np.float32(0)
        for i in sorted(first):
            rsum = np.float32(rsum + first[i])
        rec_tot = np.float32(rec_tot + np.float32(np.float32(found) / np.float32(reportK)))
        rat_tot = np.float32(rat_tot + np.float32(rsum / tsum))
    n = np.float32(len(truth))
    return float(np.float32(rec_tot / n)), float(np.float32(rat_tot / n))


def test_validate_matches_restatement(engine):
    rng = np.random.default_rng(0)
    nq, k = 20, 64
    truth = np.zeros((nq, k), dtype=engine.POINT_DTYPE)
    res = np.zeros((nq, k), dtype=engine.POINT_DTYPE)
    for q in range(nq):
        truth["ID"][q] = rng.permutation(200)[:k]
        truth["distance"][q] = np.sort(rng.random(k)).astype(np.float32)
        ids = np.where(rng.random(k) < 0.7, truth["ID"][q], rng.integers(200, 400, k))
        ids[5] = ids[4]  # a duplicate ID counts once
        res["ID"][q] = ids
        res["distance"][q] = np.sort(rng.random(k) + 0.01).astype(np.float32)
    for reportK in (10, 32, 64):
        got = engine.validate(truth, res, reportK)
        want = _validation_reference(truth, res, k, reportK)
        assert got == pytest.approx(want, rel=0, abs=0)


def test_merge_topk(engine):
    rng = np.random.default_rng(1)
    shards, nq, kin, k = 3, 7, 16, 20
    lists = np.zeros((shards, nq, kin), dtype=engine.POINT_DTYPE)
    for s in range(shards):
        lists["ID"][s] = rng.integers(0, 60, (nq, kin)) + 1000 * s
        lists["distance"][s] = np.round(rng.random((nq, kin)), 2).astype(np.float32)
    lists["ID"][1, :, -1] = -1  # empty entries are ignored
    out = engine.merge_topk(lists, k)
    for q in range(nq):
        pool = {}
        for s in range(shards):
            for p in lists[s, q]:
                if p["ID"] >= 0:
                    key = (float(p["distance"]), int(p["ID"]))
                    pool.setdefault(int(p["ID"]), key)
                    pool[int(p["ID"])] = min(pool[int(p["ID"])], key)
        want = sorted(pool.values())[:k]
        got = [(float(p["distance"]), int(p["ID"])) for p in out[q] if p["ID"] >= 0]
        assert got == want


def test_text_format_roundtrip_and_quirks(engine):
    rng = np.random.default_rng(2)
    x = (rng.random((13, 7)) * 2 - 1).astype(np.float32)
    with tempfile.TemporaryDirectory() as td:
        p = os.path.join(td, "d.txt")
        engine.write_file(p, x)
        y = engine.parse_file(p)
        assert y.shape == x.shape
        assert np.allclose(x, y, atol=1.5e-6)
        # parseFile keeps only the last digit before the point and ignores exponents
        with open(p, "w") as f:
            f.write("2\n3\n0 12.5 -3.25 0.125 \n1 1e3 7 -0.5 \n")
        z = engine.parse_file(p)
        assert z[0].tolist() == [2.5, -3.25, 0.125]
        assert z[1, 1:].tolist() == [7.0, -0.5]


def test_text_reader_matches_reference_reader(engine, tmp_path):
    """The reader against the reference's parseFile (LinearScan/gloveparser.cu), run on
    the same files by tests/golden/make_golden.py: writer output, multi-digit integer
    parts, exponents, repeated points, inner '-', other bytes, double spaces, CR line
    ends, long fractions, an empty id, an empty line, a dropped '-' field carrying its
    sign to the next line, and a file without a final newline -- bit for bit."""
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "text_reader.npz"))
    toff = voff = 0
    for i, (ln, (n, d)) in enumerate(zip(z["text_len"], z["shape"])):
        p = tmp_path / f"case{i}.txt"
        p.write_bytes(z["text"][toff:toff + ln].tobytes())
        want = z["values"][voff:voff + n * d].reshape(n, d)
        toff += ln
        voff += n * d
        got = engine.parse_file(str(p))
        assert got.shape == (n, d)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), i


def _fnv1a64(data: bytes) -> bytes:
    h = 1469598103934665603
    for b in data:
        h = ((h ^ b) * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return h.to_bytes(8, "little")


def test_damaged_index_files_refused_before_device_work(engine, tmp_path):
    """lshg_index_load reads the whole file, compares its checksum and parses and checks
    every field before its first CUDA call: on this GPU-less host each damaged file is
    refused with LSHG_ERR_IO (a CUDA call would have failed with LSHG_ERR_CUDA first)."""
    magic = b"LSHGIDX4"
    body = magic + bytes(range(256)) * 4
    cases = {
        "missing": None,
        "truncated": magic[:5],
        "magic": b"NOTANIDX" + bytes(64) + _fnv1a64(b"NOTANIDX" + bytes(64)),
        "checksum": body + b"\0" * 8,
        # checksum right, contents not an index: the parser refuses it
        "contents": body + _fnv1a64(body),
        "zeros": magic + bytes(4096) + _fnv1a64(magic + bytes(4096)),
    }
    expect = {"missing": "cannot open", "truncated": "truncated", "magic": "not an lshg index",
              "checksum": "checksum mismatch", "contents": "corrupt index file", "zeros": "corrupt index file"}
    for name, data in cases.items():
        p = tmp_path / f"{name}.lshg"
        if data is not None:
            p.write_bytes(data)
        with pytest.raises(engine.LshgError) as e:
            engine.Index.load(str(p))
        assert e.value.status == 9, (name, str(e.value))  # LSHG_ERR_IO
        assert expect[name] in str(e.value), (name, str(e.value))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _shard_worker(rank, world, port, x, q, k, out_path):
    import torch.distributed as dist

    import oracle
    from lshongpu_gb300 import sharded

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    lo, hi = sharded.shard_bounds(len(x), world, rank)
    ids, ds = oracle.exact_topk(x[lo:hi], q, k, dist=1)  # stands in for the rank's GPU index
    from lshongpu_gb300.api import POINT_DTYPE

    local = np.zeros(ids.shape, dtype=POINT_DTYPE)
    local["ID"], local["distance"] = ids, ds
    merged = sharded.merge_across_ranks(local, lo, k)
    if rank == 0:
        np.save(out_path, merged)
    dist.barrier()
    dist.destroy_process_group()


def test_sharded_query_two_ranks_gloo(engine, orc):
    import torch.multiprocessing as mp

    from lshongpu_gb300 import datasets

    x = datasets.clustered(3001, 32, 5, count=10)
    q = datasets.clustered(9, 32, 6, count=10)
    k = 32
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "merged.npy")
        mp.start_processes(_shard_worker, args=(2, _free_port(), x, q, k, out), nprocs=2, join=True,
                           start_method="spawn")
        merged = np.load(out)
    ids, ds = orc.exact_topk(x, q, k, dist=1)
    assert np.array_equal(merged["ID"], ids)
    assert np.array_equal(merged["distance"], ds)


def test_truth_file_roundtrip(engine):
    rng = np.random.default_rng(4)
    t = np.zeros((5, 8), dtype=engine.POINT_DTYPE)
    t["ID"] = rng.integers(0, 1000, (5, 8))
    t["distance"] = -rng.random((5, 8)).astype(np.float32)
    with tempfile.TemporaryDirectory() as td:
        p = os.path.join(td, "truth.txt")
        engine.write_truth(p, t)
        r = engine.read_truth(p)
    assert np.array_equal(r, t)
