"""Pin the oracle and the engine's host code to the reference's own outputs.

Golden vectors were produced by the reference's CPU code compiled from its sources
(randomVectorGenerator.cpp, GoldStandard/goldstandard.cpp) -- see tests/golden/make_golden.py.
"""
import numpy as np

from conftest import ids_equal_up_to_ties


def test_oracle_rng_matches_reference(orc, golden):
    r = golden["rng"]
    assert np.array_equal(orc.random_normals(len(r["normals"])), r["normals"])
    assert np.array_equal(orc.random_normals(len(r["jl16"]), 1.0 / 16), r["jl16"])
    assert np.array_equal(orc.random_plus_minus(len(r["plus_minus"])), r["plus_minus"])
    assert np.array_equal(orc.random_bools(len(r["bools"])), r["bools"])


def test_engine_host_rng_matches_reference(engine, golden):
    r = golden["rng"]
    assert np.array_equal(engine.random_normals(len(r["normals"])), r["normals"])
    assert np.array_equal(engine.random_normals(len(r["jl16"]), 1.0 / 16), r["jl16"])
    assert np.array_equal(engine.random_plus_minus(len(r["plus_minus"])), r["plus_minus"])
    assert np.array_equal(engine.random_bools(len(r["bools"])), r["bools"])


def test_rng_prefix_property(engine):
    # lshFramework.cuh:24-27: the sketch planes come from a fresh default engine, so
    # their prefix equals the key planes
    a = engine.random_normals(1000)
    b = engine.random_normals(3000)
    assert np.array_equal(a, b[:1000])


def test_goldstandard_port_matches_reference(orc, golden):
    g = golden["gold"]
    ids, ds, _ = orc.goldstandard(g["data"], g["queries"], 32, threads=2)
    # the reference prints distances with 6 significant digits
    assert np.allclose(ds, g["dists"], rtol=2e-6, atol=2e-6)
    assert ids_equal_up_to_ties(ids, ds, g["ids"], g["dists"], 1e-6) == 0


def test_exact_oracle_agrees_with_goldstandard(orc, golden):
    g = golden["gold"]
    ids, ds = orc.exact_topk(g["data"], g["queries"], 32, dist=1)
    # 1 - cos (engine) vs -cos (GoldStandard): same order up to rounding ties
    assert ids_equal_up_to_ties(ids, ds, g["ids"], g["dists"] + 1.0, 2e-6) == 0
    assert np.allclose(ds, g["dists"] + 1.0, atol=2e-6)


def test_fp64_oracle_agrees_with_goldstandard(orc, golden):
    g = golden["gold"]
    ids, ds = orc.fp64_topk(g["data"], g["queries"], 32)
    assert ids_equal_up_to_ties(ids, ds, g["ids"], g["dists"] + 1.0, 2e-6) == 0
