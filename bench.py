"""Benchmark: queries/sec at recall@32 >= 0.99 on 1.2M x 100 unit vectors.

Workload (one "step"): a batch of Q = 10,000 queries answered with k = 32 against a
resident index of N = 1,200,000 base points, d = 100 (clustered synthetic data: 1,000
Gaussian clusters, centres uniform on the sphere, sigma 0.05, L2-normalised; queries
from the same centres with the next seed).  The base (480 MB fp32, 300 MB bf16) is
larger than the 129 MB L2, so no flush is needed between steps.

  --path tc       tensor-core exact scan (BF16 tcgen05 GEMM + fused top-candidates +
                  FP32 re-rank)                       [default, the headline]
  --path exact    plain FP32 SIMT exact scan (the denominator of the speed-up)
  --path simhash  1024-bit SimHash + Hamming top-C + FP32 re-rank

`--config` selects one of the measurement configurations instead of the headline (each
prints its own line with its own metric; the headline is the default):

  1       exact angular k-NN, N = 100k, d = 100, Q = 1000, k = 32 (--path exact or tc)
  2       1024-bit SimHash, N = 1.2M, Q = 10k, C = 1024 candidates re-ranked (2-c128: C = 128)
  3       tensor-core exact scan, N = 1M, d = 128 (100 + 28 zero dims), Q = 16,384 (3-fp8:
          E4M3 tensor-core scores; --path tc8 runs E4M3 at any size)
  4a      cross-polytope LSH, L = 32 tables, K = 2 hashes a key, 3 rounds, N = 1M, d = 128
          padded, Q = 10k, exact angular distance on candidates (4a-k1: K = 1; 4a-l48: L = 48,
          the table count that reaches recall@32 >= 0.99)
  4b      weighted MinHash, 256 byte samples, N = 500k, d = 100 sparse Gamma(2,1) values
          (30% nonzero), Q = 10k, Jaccard sketch scan + generalized-Jaccard re-rank
          (4b-1bit: 256 one-bit samples)

`value` is whole-job queries/sec with queries and results resident in HBM; `e2e` is the
same metric through the C ABI with host (pinned) buffers, every batch's upload and
download inside the timed region, measured two ways -- lshg_index_query_async over two
streams (copies overlap the other stream's scan) and the one-batch-at-a-time
lshg_index_query -- and reported as the better of the two (`e2e.api` names it).  `--impl reference` times the reference's CPU brute force (a port of
GoldStandard/goldstandard.cpp -- the reference binary is x86-only here) on the host
cores over a bounded query sample.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "queries/sec at recall@32>=0.99 on 1.2Mx100 (TC+serving vs plain scan)"
N_BASE, DIM, N_QUERY, K = 1_200_000, 100, 10_000, 32
PAD_DIM = 0        # zero dimensions appended to every vector
DATA = "clustered"  # or "sparse" (weighted MinHash configuration)
CAND = 1024         # SimHash candidates re-ranked
CP_HASHES = 2       # cross-polytope hashes a key
CP_TABLES = 32      # LSH tables

# measurement configurations: path and shape overrides
CONFIGS = {
    "1": dict(path="exact", N_BASE=100_000, N_QUERY=1000),
    "2": dict(path="simhash", CAND=1024),
    "2-c128": dict(path="simhash", CAND=128),
    "3": dict(path="tc", N_BASE=1_000_000, N_QUERY=16_384, PAD_DIM=28),
    "3-fp8": dict(path="tc8", N_BASE=1_000_000, N_QUERY=16_384, PAD_DIM=28),
    "4a": dict(path="cplsh", N_BASE=1_000_000, PAD_DIM=28, CP_HASHES=2),
    "4a-k1": dict(path="cplsh", N_BASE=1_000_000, PAD_DIM=28, CP_HASHES=1),
    "4a-l48": dict(path="cplsh", N_BASE=1_000_000, PAD_DIM=28, CP_HASHES=2, CP_TABLES=48),
    "4b": dict(path="wmh", N_BASE=500_000, DATA="sparse"),
    "4b-1bit": dict(path="wmh1", N_BASE=500_000, DATA="sparse"),
    "4b-cws": dict(path="cws", N_BASE=500_000, DATA="sparse"),
}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return p["hbm_gbs"], p["bf16_tflops"], p.get("bf16_tflops_sustained", p["bf16_tflops"]), "measured"
    except Exception:
        return 6800.0, 1900.0, 1700.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = tempfile.mktemp(suffix=".csv")

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
            # the timed region starts once the sampler has written its first sample
            t0 = time.perf_counter()
            while os.path.getsize(self.path) == 0 and self.proc.poll() is None and time.perf_counter() - t0 < 3.0:
                time.sleep(0.01)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()
            self.f.close()

    def summary(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def make_data(seed_offset: int):
    from lshongpu_gb300 import datasets

    if DATA == "sparse":
        x = datasets.sparse_gamma(N_BASE, DIM, seed=100 + seed_offset)
        q = datasets.sparse_gamma(N_QUERY, DIM, seed=101 + seed_offset)
    else:
        x = datasets.clustered(N_BASE, DIM, seed=100 + seed_offset)
        q = datasets.clustered(N_QUERY, DIM, seed=101 + seed_offset)
    if PAD_DIM:
        x = np.ascontiguousarray(np.pad(x, ((0, 0), (0, PAD_DIM))))
        q = np.ascontiguousarray(np.pad(q, ((0, 0), (0, PAD_DIM))))
    return x, q


FP64_RECHECK = -1  # lshg_options.fp64_recheck of the benchmarked index
CWS_PLANES = 16    # bit planes of the benchmarked CWS index's codes (read from the index)


def build_index(L, x, path: str):
    if path == "tc":
        return L.Index(x, implementation=L.IMPL_TC, distanceFunc=1,
                       options=L.make_options(candidates=64, fp64_recheck=FP64_RECHECK))
    if path == "tc8":
        return L.Index(x, implementation=L.IMPL_TC_FP8, distanceFunc=1,
                       options=L.make_options(fp64_recheck=FP64_RECHECK))
    if path == "exact":
        return L.Index(x, implementation=2, distanceFunc=1)
    if path == "simhash":
        return L.Index(x, implementation=3, sketchDim=32, options=L.make_options(candidates=CAND))
    if path == "cplsh":
        return L.Index(x, implementation=2, distanceFunc=1, framework=1, keysImplementation=7,
                       bucketKeyBits=8 * CP_HASHES, tables=CP_TABLES, options=L.make_options(cp_hashes=CP_HASHES))
    if path == "wmh":
        return L.Index(x, implementation=4, distanceFunc=2, sketchDim=256)
    if path == "wmh1":
        return L.Index(x, implementation=5, distanceFunc=2, sketchDim=8)
    if path == "cws":
        return L.Index(x, implementation=L.IMPL_CWS, distanceFunc=2, sketchDim=256)
    raise SystemExit(f"unknown path {path}")


# FP32 SIMT peak (no measured figure exists for it): 152 SMs x 128 FMA/clk x 2 x 2.07 GHz
FP32_SIMT_NOMINAL_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12
# 32-bit population count: 16 a clock an SM (nominal), 152 SMs at 2.07 GHz, in G word/s
POPC_NOMINAL_GWORDS = 152 * 16 * 2.07e9 / 1e9
# integer ALU pipe (logic operations): 64 lanes a clock an SM, in G operations/s
ALU_NOMINAL_GOPS = 152 * 64 * 2.07e9 / 1e9


def algorithmic(path: str, prof: dict, nq: int, lsh_counts=None):
    """(kernel, bound, work per launch, unit) for the dominant kernel of the path.  FLOPs
    count the index dimension (100 at the headline: the kernel's own padding to 112/128 is
    not counted; 128 at configuration 3, whose vectors carry 28 zero dimensions); sketch
    scans count the sketch bytes streamed once per batch."""
    d = DIM
    if path == "tc":
        return "tc_filter", "tensor", 2.0 * nq * N_BASE * (d + PAD_DIM) / 1e12, "TFLOP/s"
    if path == "tc8":
        return "tc_filter", "tensor8", 2.0 * nq * N_BASE * (d + PAD_DIM) / 1e12, "TFLOP/s"
    if path == "exact":
        return "scan_float", "fp32", 2.0 * nq * N_BASE * (d + PAD_DIM) / 1e12, "TFLOP/s"
    # Hamming / one-bit Jaccard scans on the tensor cores: a +-1 E4M3 GEMM over the sketch
    # bits, 2 x Q x N x bits FLOP, against the dense FP8 rate (2 x the measured bf16 figure)
    if path in ("simhash", "wmh1") and "tc_hamming" in prof:
        bits = 1024 if path == "simhash" else 256
        return "tc_hamming", "tensor8", 2.0 * nq * N_BASE * bits / 1e12, "TFLOP/s"
    # byte samples through the bit-sliced threshold filter: every (query, point) pair
    # compares 8 bit-plane words a group of 32 samples, one three-input logic operation a
    # word on the integer ALU pipe; work = Q x N x 64 plane words (256 samples)
    if path == "wmh" and "scan_bytes_filter" in prof:
        return "scan_bytes_filter", "alu", nq * N_BASE * 64 / 1e9, "Gword/s"
    # CWS codes through the same filter: 8 planes a 32-sample group for dictionary ranks,
    # 16 for raw codes (64 or 128 plane words a pair at 256 samples)
    if path == "cws":
        return "scan_cws", "alu", nq * N_BASE * 8 * CWS_PLANES / 1e9, "Gword/s"
    # sketch scans on the popcount path are integer-bound at these batch sizes: work = sketch
    # words compared (one XOR + POPC each, zero-byte count for byte samples), Q x N x words
    if path == "simhash":
        return "scan_bits", "popc", nq * N_BASE * 32 / 1e9, "Gword/s"
    if path == "wmh":
        return "scan_bits", "popc", nq * N_BASE * 64 / 1e9, "Gword/s"
    if path == "wmh1":
        return "scan_bits", "popc", nq * N_BASE * 8 / 1e9, "Gword/s"
    # LSH gather: bytes the query kernel must move -- every bucket entry walked (4 B id),
    # every distinct candidate's row and norm, the queries and the results -- from the
    # kernel's own counters over the timed launches
    if lsh_counts is None:
        return "lsh_query", "gather", None, None
    entries, distinct = lsh_counts
    dims = d + PAD_DIM
    return ("lsh_query", "gather",
            (entries * 4 + distinct * (4 * dims + 4) + nq * (4 * dims + 8 * K)) / 1e9, "GB/s")


def dram_traffic(kernel: str, workload: str):
    """DRAM bytes (read + write) of one launch of `kernel` on `workload`, as an ncu capture
    of the same kernel and workload measured them (profiles/dram_traffic.json, which names
    the capture's command); None where no capture of that pair exists."""
    try:
        with open(os.path.join(ROOT, "profiles", "dram_traffic.json")) as f:
            rows = json.load(f)["captures"]
    except Exception:
        return None
    for r in rows:
        if r["kernel"] == kernel and r["workload"] == workload:
            return r["dram_bytes_per_launch"]
    return None


def serving_run(L, indexes: dict, rate_qps: float, seconds: float, truth=None, seed: int = 7,
                window_us: int = 200, streams: int = 3) -> dict:
    """Open-loop Poisson arrivals of requests (batch size log-uniform in [1, 4096], k from
    {10, 32, 100}, index drawn uniformly) against the continuous-batching server;
    latency = submit -> results on the host, as stamped by the library.  truth: (pool,
    {index: (ids of the FP64 top-100 of the first rows of the pool)}) -- served rows of
    those pool queries are scored for recall@k."""
    import threading

    rng = np.random.default_rng(seed)
    pool = truth[0] if truth else make_pool()
    srv = L.Server(max_batch=4096, streams=streams, use_graphs=True, batch_window_us=window_us)
    for i, ix in indexes.items():
        srv.add_index(i, ix)
    ids = list(indexes)
    # untimed warm-up: record every (index, k, power-of-two batch class) graph once
    for which in ids:
        for k in (10, 32, 100):
            size = 1
            while size <= 4096:
                srv.wait(srv.submit(which, pool[:size], k))
                size *= 2
    st0 = srv.stats()
    mean_size = (4096 - 1) / np.log(4096.0)
    req_rate = rate_qps / mean_size
    nreq = max(1, int(req_rate * seconds))
    gaps = rng.exponential(1.0 / req_rate, size=nreq)
    sizes = np.exp(rng.uniform(0, np.log(4096), size=nreq)).astype(int)
    ks = rng.choice([10, 32, 100], size=nreq)
    which_i = rng.integers(0, len(ids), size=nreq)
    offs = [int(rng.integers(0, 4096 - int(sz) + 1)) for sz in sizes]
    tickets, lat = [], []
    hits = {}  # index -> [matched, total]
    done = threading.Event()
    tlim = truth[1] if truth else {}

    def waiter():
        i = 0
        while not (done.is_set() and i >= len(tickets)):
            if i < len(tickets):
                tk, which, off, sz, k = tickets[i]
                out, l = srv.wait(tk)
                lat.append(l / 1e3)
                tid = tlim.get(which)
                if tid is not None and off < len(tid):
                    rows = range(off, min(off + sz, len(tid)))
                    h = hits.setdefault(which, [0, 0])
                    for r in rows:
                        h[0] += len(set(out["ID"][r - off].tolist()) & set(tid[r][:k].tolist()))
                        h[1] += k
                i += 1
            else:
                time.sleep(0.0002)

    th = threading.Thread(target=waiter)
    th.start()
    t0 = time.perf_counter()
    nxt = t0
    submitted = 0
    for j in range(nreq):
        nxt += gaps[j]
        while time.perf_counter() < nxt:
            pass
        which, sz, k, off = ids[int(which_i[j])], int(sizes[j]), int(ks[j]), offs[j]
        try:
            tickets.append((srv.submit(which, pool[off:off + sz], k), which, off, sz, k))
            submitted += sz
        except L.LshgError:
            pass  # refused by admission: counted in stats
    done.set()
    th.join()
    wall = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    lat_a = np.array(lat)
    res = {"offered_qps": rate_qps, "achieved_qps": submitted / wall, "requests": len(tickets),
           "p50_ms": float(np.percentile(lat_a, 50)), "p99_ms": float(np.percentile(lat_a, 99)),
           "p999_ms": float(np.percentile(lat_a, 99.9)), "launches": st["launches"] - st0["launches"],
           "graph_replays": st["graph_replays"] - st0["graph_replays"], "rejected": st["rejected"] - st0["rejected"],
           "batch_window_us": window_us, "slots": streams}
    res["launches_per_request"] = res["launches"] / max(1, res["requests"])
    if hits:
        res["recall_at_k"] = {str(w): h[0] / h[1] for w, h in hits.items() if h[1]}
        res["recall_rows"] = {str(w): h[1] for w, h in hits.items()}
    return res


def make_pool():
    from lshongpu_gb300 import datasets

    return datasets.clustered(4096, DIM, seed=9001)


def fp64_distances(x, q, ids, dist_fn):
    """Double-precision distance of every (query, returned id): angular 1 - cos, or
    generalized Jaccard 1 - sum(min)/sum(max) on the shifted, normalised rows."""
    if dist_fn == 2:
        xs = x.astype(np.float64)
        qs = q.astype(np.float64)
        sh = np.abs(np.minimum(0, np.floor(np.minimum(xs.min(axis=0), qs.min(axis=0)))))
        xs, qs = xs + sh, qs + sh
        xs /= np.linalg.norm(xs, axis=1, keepdims=True)
        qs /= np.linalg.norm(qs, axis=1, keepdims=True)
        rows = xs[ids]
        return 1.0 - np.minimum(rows, qs[:, None, :]).sum(-1) / np.maximum(rows, qs[:, None, :]).sum(-1)
    qq = q.astype(np.float64)
    rows = x[ids].astype(np.float64)
    dot = np.einsum("qd,qkd->qk", qq, rows)
    return 1.0 - dot / (np.linalg.norm(qq, axis=1)[:, None] * np.linalg.norm(rows, axis=2))


def workload_text(args) -> str:
    d = f"{DIM}" if not PAD_DIM else f"{DIM + PAD_DIM} ({DIM} + {PAD_DIM} zero dims)"
    data = ("sparse Gamma(2,1) values, 30% nonzero" if DATA == "sparse"
            else "clustered unit vectors (1000 clusters, sigma 0.05)")
    what = {"tc": "tensor-core exact scan", "tc8": "tensor-core exact scan, E4M3 (FP8) scores",
            "exact": "FP32 SIMT exact scan",
            "simhash": f"1024-bit SimHash, {CAND} candidates re-ranked",
            "cplsh": f"cross-polytope LSH, L={CP_TABLES}, K={CP_HASHES}, 3 rounds, exact angular on candidates",
            "wmh": "weighted MinHash, 256 byte samples, Jaccard scan + generalized-Jaccard re-rank",
            "wmh1": "weighted MinHash, 256 one-bit samples, Jaccard scan + generalized-Jaccard re-rank",
            "cws": "consistent weighted sampling, 256 (index, int32) samples, exact match counts + "
                   "generalized-Jaccard re-rank"}[args.path]
    cfg = f"configuration {args.config}: " if args.config else ""
    return f"{cfg}{what}: N={N_BASE}, d={d}, Q={N_QUERY}, k={K}, {data}"


def run_reference_arm(args, world, rank):
    import oracle

    if rank != 0:
        return
    if args.steps is None:
        args.steps = 5
    x, q = make_data(0)
    threads = os.cpu_count() or 1
    sample = max(threads, min(N_QUERY, 2 * threads))
    qs = q[:sample]
    for _ in range(max(0, min(args.warmup, 1))):
        oracle.goldstandard(x, qs[:threads], K, threads)
    times = []
    for _ in range(args.steps):
        _, _, t = oracle.goldstandard(x, qs, K, threads)
        times.append(t)
    per_q = sum(times) / (args.steps * sample)
    qps = 1.0 / per_q
    line = {
        "impl": "reference", "metric": METRIC, "value": qps, "unit": "queries/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": per_q * N_QUERY * 1e3,
        "ms_per_step_kind": f"extrapolated: the measured time of a {sample}-query sample scaled to the {N_QUERY}-query "
                            f"batch",
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"exact angular k-NN, N={N_BASE}, d={DIM}, Q={N_QUERY} (timed on a {sample}-query "
                               f"sample per step), k={K}", "global_batch": N_QUERY, "l2": "inputs larger than L2"},
        "cpu_baseline": {"value": qps, "unit": "queries/s", "cores": threads, "kind": "port",
                         "sample": f"{sample} queries x {N_BASE} points per step, {args.steps} steps",
                         "note": "port of GoldStandard/goldstandard.cpp computeGoldStandard (same arithmetic: float "
                                 "magnitudes, double-accumulated dot, full sort), run on all host threads without the "
                                 "reference's per-point struct copies: faster than the single-threaded reference"},
        "e2e": {"value": qps, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default: about one second of timed work, at least 5; the reference arm: 5)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--path", default=None, choices=["tc", "tc8", "exact", "simhash", "cplsh", "wmh", "wmh1", "cws"])
    ap.add_argument("--config", default=None, choices=sorted(CONFIGS), help="measurement configuration")
    ap.add_argument("--no-extras", action="store_true", help="skip recall / baselines / serving extras")
    ap.add_argument("--n", type=int, default=None, help="base size (profiling cases only)")
    ap.add_argument("--nq", type=int, default=None, help="queries per step (profiling cases only)")
    ap.add_argument("--tables", type=int, default=None, help="LSH tables (cross-polytope configurations)")
    ap.add_argument("--fp64-recheck", type=int, default=-1, choices=[-1, 0, 1],
                    help="lshg_options.fp64_recheck of the index (-1: the library default)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.config:
        over = dict(CONFIGS[args.config])
        path = over.pop("path")
        args.path = args.path or path
        globals().update(over)
        globals()["METRIC"] = f"queries/sec, configuration {args.config}"
    # explicit sizes (small profiling cases) take precedence over a configuration's
    if args.n is not None:
        globals()["N_BASE"] = args.n
    if args.nq is not None:
        globals()["N_QUERY"] = args.nq
    if args.tables is not None:
        globals()["CP_TABLES"] = args.tables
    globals()["FP64_RECHECK"] = args.fp64_recheck
    args.path = args.path or "tc"

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        run_reference_arm(args, world, rank)
        return

    import torch

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    import lshongpu_gb300 as L

    x, q = make_data(rank)
    tb = time.perf_counter()
    idx = build_index(L, x, args.path)
    global CWS_PLANES
    if args.path == "cws":  # bit planes the CWS scan compares (8: dictionary ranks, 16: raw codes)
        CWS_PLANES = int(np.frombuffer(idx.export(L.EXPORT_CWS_CODES), np.int32)[4]) or 16
    build_s = time.perf_counter() - tb  # host wall time of the index build (synchronous)
    dev = torch.device("cuda", local)
    qd = torch.from_numpy(q).to(dev)
    out = torch.empty((N_QUERY, K, 2), dtype=torch.int32, device=dev)
    stream = torch.cuda.Stream(device=dev)
    sh = stream.cuda_stream

    # batches are enqueued back to back on one stream (lshg_index_query_async); the timed
    # region ends with lshg_index_sync, which also reports any device-side error
    def step():
        idx.query_device_async(qd.data_ptr(), N_QUERY, K, out.data_ptr(), stream=sh)

    tw = time.perf_counter()
    for _ in range(args.warmup):
        step()
    idx.sync(sh)
    torch.cuda.synchronize()
    if args.steps is None:
        # about one second of timed work, so that the clock sampler (an nvidia-smi sample
        # every 200 ms) sees the timed region several times; rank 0's count for every rank
        per_step = (time.perf_counter() - tw) / args.warmup
        k = torch.tensor([min(2000, max(5, math.ceil(1.0 / max(per_step, 1e-6))))], device=dev)
        if dist:
            dist.broadcast(k, 0)
        args.steps = int(k.item())

    def barrier():
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    counts0 = idx.query_counters()
    launches0 = L.launch_count()
    L.profile_enable(True)
    L.profile_report()
    with ClockSampler(local) as clk:
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        idx.sync(sh)
        barrier()
    L.profile_enable(False)
    launches = L.launch_count() - launches0
    prof = L.profile_report()
    counts1 = idx.query_counters()  # the timed launches only (the e2e loop below queries too)
    ms = e0.elapsed_time(e1)
    if dist:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    ms_step = ms / args.steps
    value = world * N_QUERY / (ms_step / 1e3)

    # e2e through the C ABI with pinned host buffers: every step uploads its query batch
    # and downloads its results.  Pipelined: lshg_index_query_async on host buffers,
    # alternating two streams so one batch's copies overlap the previous batch's scan;
    # the host wall clock spans the first enqueue to the last stream's completion.
    qh = torch.from_numpy(q).pin_memory()
    ohs = [torch.empty((N_QUERY, K, 2), dtype=torch.int32).pin_memory() for _ in range(2)]
    streams = [stream, torch.cuda.Stream(device=dev)]
    lib = L.lib()

    def e2e_step(i):
        st = streams[i & 1]
        idx.query_host_async(qh.data_ptr(), N_QUERY, K, ohs[i & 1].data_ptr(), stream=st.cuda_stream)

    def e2e_wait():
        for st in streams:
            idx.sync(st.cuda_stream)

    for i in range(max(3, args.warmup)):
        e2e_step(i)
    e2e_wait()
    barrier()
    t0 = time.perf_counter()
    for i in range(args.steps):
        e2e_step(i)
    e2e_wait()
    barrier()
    e2e_ms = (time.perf_counter() - t0) * 1e3 / args.steps
    pipelined_value = world * N_QUERY / (e2e_ms / 1e3)
    # the same with the reference-shaped blocking call (one batch at a time)
    for _ in range(2):
        L.api.check(lib.lshg_index_query(idx.handle, qh.data_ptr(), N_QUERY, K, ohs[0].data_ptr(), 0, sh))
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        L.api.check(lib.lshg_index_query(idx.handle, qh.data_ptr(), N_QUERY, K, ohs[0].data_ptr(), 0, sh))
    barrier()
    blocking_value = world * N_QUERY / ((time.perf_counter() - t0) / args.steps)
    # reported: the better of the two ways a caller can drive the ABI (two concurrent LSH
    # batches contend for L2 -- their dedupe bitmaps -- and lose to one at a time)
    e2e_value = max(pipelined_value, blocking_value)
    e2e_api = ("lshg_index_query_async, host buffers, 2 streams" if pipelined_value >= blocking_value
               else "lshg_index_query, host buffers, one batch at a time")

    hbm, bf16, bf16s, peak_kind = peaks()
    lsh_counts = None
    if args.path == "cplsh":
        lsh_counts = tuple((b - a) / args.steps for a, b in zip(counts0, counts1))
    kname, bound, work, unit = algorithmic(args.path, prof, N_QUERY, lsh_counts)
    cnt, kms = prof.get(kname, (0, 0.0))
    achieved = (work / (kms / cnt / 1e3)) if (cnt and work) else None
    if bound in ("hbm", "gather"):
        peak = hbm
    elif bound == "fp32":
        peak, peak_kind = FP32_SIMT_NOMINAL_TFLOPS, "nominal (152 SMs x 128 FMA/clk x 2 x 2.07 GHz)"
    elif bound == "tensor":
        peak = bf16
    elif bound == "tensor8":  # no measured FP8 figure: the dense FP8 rate is twice BF16's
        peak, peak_kind = 2 * bf16, "2 x measured bf16 (dense FP8 rate = 2 x BF16)"
    elif bound == "popc":
        peak, peak_kind = POPC_NOMINAL_GWORDS, "nominal (152 SMs x 16 popc/clk x 2.07 GHz)"
    elif bound == "alu":
        peak, peak_kind = ALU_NOMINAL_GOPS, "nominal (152 SMs x 64 integer ALU lanes/clk x 2.07 GHz)"
    else:
        peak = None
    traffic = dram_traffic(kname, workload_text(args))
    roofline = {"bound": bound, "kernel": kname, "achieved": achieved, "peak": peak, "unit": unit,
                "frac": (achieved / peak) if (achieved and peak) else None, "peak_source": peak_kind,
                "traffic": traffic, "traffic_unit": "bytes per launch" if traffic else None, "kernel_ms_per_launch": (kms / cnt) if cnt else None,
                "kernel_share": (kms / sum(v[1] for v in prof.values())) if prof else None}
    if lsh_counts:
        roofline["lsh_entries_per_query"] = lsh_counts[0] / N_QUERY
        roofline["lsh_distinct_per_query"] = lsh_counts[1] / N_QUERY
    if bound == "popc" and cnt:
        # the memory side of a sketch scan: every CTA streams the whole base's sketches for
        # its block of queries (16 a block for C <= 128, 4 up to 1024, 2 beyond), bytes
        # actually moved to the SMs (mostly from L2) over the kernel time; the integer
        # roofline above is the one that bounds these batch sizes
        cand = {"simhash": CAND}.get(args.path, 4096)
        qb = 16 if cand <= 128 else (4 if cand <= 1024 else 2)
        row = {"simhash": 128, "wmh": 256, "wmh1": 32}[args.path]
        streamed = -(-N_QUERY // qb) * N_BASE * row
        gbs = streamed / (kms / cnt / 1e3) / 1e9
        roofline["secondary"] = {"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s", "frac": gbs / hbm,
                                 "work": f"{streamed / 1e9:.1f} GB of sketches streamed a batch "
                                         f"({-(-N_QUERY // qb)} query blocks x {N_BASE} x {row} B)"}

    extras = {}
    if rank == 0 and not args.no_extras:
        import oracle

        threads = os.cpu_count() or 1
        got = out.cpu().numpy()
        res = got[:, :, 0]
        headline = args.config is None and args.path == "tc"
        dist_fn = 2 if DATA == "sparse" else 1
        if DATA == "sparse":  # generalized-Jaccard truth (single-threaded oracle: small sample)
            nchk = 50
            tids, tds = oracle.exact_topk(x, q[:nchk], K, dist=2)
        else:
            nchk = 200
            tids, tds = oracle.fp64_topk(x, q[:nchk], K, threads=threads)
        rec = np.mean([len(set(res[i].tolist()) & set(tids[i].tolist())) / K for i in range(nchk)])
        extras["recall_at_32"] = float(rec)
        extras["recall_queries"] = nchk
        # distance error of the returned points against their FP64 distances, and the
        # reference's distance ratio (validation.cpp:160-198: sum of returned distances over
        # sum of the truth's, averaged over queries)
        rid = res[:nchk]
        rd32 = got[:nchk, :, 1].view(np.float32).astype(np.float64)
        ok = rid >= 0
        d64 = fp64_distances(x, q[:nchk], np.where(ok, rid, 0), dist_fn)
        extras["max_dist_err_vs_fp64"] = float(np.max(np.abs(rd32 - d64)[ok])) if ok.any() else None
        truth = np.zeros((nchk, K), dtype=L.POINT_DTYPE)
        truth["ID"], truth["distance"] = tids, np.asarray(tds, np.float64).astype(np.float32)
        _, ratio = L.validate(truth, np.ascontiguousarray(got[:nchk]).view(L.POINT_DTYPE).reshape(nchk, K), K)
        extras["distance_ratio"] = float(ratio)
        extras["truth"] = "FP64 oracle" if DATA != "sparse" else "FP32 generalized-Jaccard oracle"
        # CPU baseline: GoldStandard port, bounded sample, all host threads
        if DATA != "sparse":
            sample = 2 * threads
            _, _, tcpu = oracle.goldstandard(x, q[:sample], K, threads)
            cpu_qps = sample / tcpu
            extras["cpu_baseline"] = {"value": cpu_qps, "unit": "queries/s", "cores": threads, "kind": "port",
                                      "sample": f"{sample} queries x {N_BASE} points (GoldStandard port)"}
        # denominator of the headline ratio: the engine's own tuned FP32 SIMT exact scan
        # (implementation 2) on the same GPU, same base, 1024 of the same queries
        if args.path == "tc":
            simt = L.Index(x, implementation=2, distanceFunc=1)
            nsub = min(1024, N_QUERY)
            qs_dev = qd[:nsub].contiguous()
            outs = torch.empty((nsub, K, 2), dtype=torch.int32, device=dev)
            for _ in range(2):
                simt.query_device(qs_dev.data_ptr(), nsub, K, outs.data_ptr(), stream=sh)
            torch.cuda.synchronize()
            g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            g0.record(stream)
            simt.query_device(qs_dev.data_ptr(), nsub, K, outs.data_ptr(), stream=sh)
            g1.record(stream)
            torch.cuda.synchronize()
            simt_qps = nsub / (g0.elapsed_time(g1) / 1e3)
            extras["denominators"] = {
                "engine_simt_exact": {"value": simt_qps, "unit": "queries/s",
                                      "sample": f"{nsub} queries x {N_BASE} points, FP32 SIMT exact scan"},
                "ratio_value_over_simt": value / simt_qps}
            del simt
        # serving: the same resident base behind the continuous-batching loop, offered up
        # to and past the batch capacity, then mixed with a 1024-bit SimHash index and a
        # cross-polytope LSH index (L=32, K=2) of it; served rows of the first 256 pool
        # queries are scored against the FP64 oracle's top-k
        if headline:
            pool = make_pool()
            t64, _ = oracle.fp64_topk(x, pool[:256], 100, threads=threads)
            serve_ix = {0: idx,
                        1: L.Index(x, implementation=3, sketchDim=32, options=L.make_options(candidates=1024)),
                        2: L.Index(x, implementation=2, distanceFunc=1, framework=1, keysImplementation=7,
                                   bucketKeyBits=16, tables=32, options=L.make_options(cp_hashes=2))}
            extras["serving"] = [serving_run(L, {0: idx}, rate, 2.0, truth=(pool, {0: t64}))
                                 for rate in (500_000, 2_000_000, 4_000_000)]
            extras["serving_mixed"] = serving_run(L, serve_ix, 300_000, 3.0, truth=(pool, {0: t64, 1: t64, 2: t64}))
            best = max(extras["serving"], key=lambda r: r["achieved_qps"] if r["p99_ms"] < 50 else 0)
            extras["latency_ms"] = {k: best[k] for k in ("p50_ms", "p99_ms", "p999_ms")}
            extras["latency_ms"]["at_offered_qps"] = best["offered_qps"]

    line = {
        "metric": METRIC, "value": value, "unit": "queries/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": ({"tc": "bf16", "tc8": "e4m3", "wmh": "u8", "cws": "int32 pairs (u16 codes)"}.get(args.path)
              or ("e4m3 (+-1 sketch bits)" if "tc_hamming" in prof else None)
              or {"simhash": "u32", "wmh1": "u32"}.get(args.path, "f32")),
        "data": "synthetic",
        "config": {"workload": workload_text(args), "global_batch": N_QUERY * world,
                   "path": args.path, "parallelism": f"replicas{world}", "l2": "inputs larger than L2 (no flush)",
                   "fp64_recheck": FP64_RECHECK},
        "roofline": roofline,
        "e2e": {"value": e2e_value, "unit": "queries/s", "h2d_bytes_per_step": N_QUERY * (DIM + PAD_DIM) * 4,
                "d2h_bytes_per_step": N_QUERY * K * 8, "api": e2e_api,
                "pipelined_value": pipelined_value, "blocking_value": blocking_value},
        "gpu_launches": launches,
        "index_build_s": build_s,
        "clocks": clk.summary(),
        "kernels": {k: {"launches": v[0], "ms": v[1]} for k, v in prof.items()},
    }
    line.update(extras)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
