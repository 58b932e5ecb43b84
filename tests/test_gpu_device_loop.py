"""GPU tests of the device proof loop (sid_prove_opts.device_loop_blocks): the whole proof -- root partition,
static recursion with hull join, final generation, dynamic re-split -- in one persistent kernel. Counts,
escalations and critical boxes must be those of the host-driven loop (and so the reference's published counts),
in both precision forms and on grids from one block to the device's limit."""
import json
import os

import numpy as np
import pytest

import kat_expect
import sid_gb300 as sid

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PUBLISHED = json.load(open(os.path.join(REPO, "tests", "golden", "published_counts.json")))
ALL_BLOCKS = 1 << 20          # clamped to the device's limit for the kernel


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)


@pytest.mark.parametrize("blocks", [1, 16, ALL_BLOCKS])
@pytest.mark.parametrize("precision", [sid.PRECISION_PLAIN, sid.PRECISION_FP32])
@pytest.mark.parametrize("name", ["top_packing_1", "top_packing_2", "five_subcontainer", "six_subcontainer",
                                  "seven_subcontainer", "one_subcontainer", "three_subcontainer"])
def test_device_loop_counts_equal_the_host_loop(engine, name, precision, blocks):
    lid = engine.register(sid.lemma_ir(name))
    d = engine.prove(lid, precision=precision, device_loop=blocks)
    h = engine.prove(lid, precision=precision)
    assert [d["cuboids"], d["leaves"]] == PUBLISHED[name] and d["criticals"] == 0
    assert d["escalated"] == h["escalated"]
    assert d["complete"]


@pytest.mark.parametrize("precision", [sid.PRECISION_PLAIN, sid.PRECISION_FP32])
@pytest.mark.parametrize("name,gens", [("expected_critical_f64", 2), ("expected_critical_f32", 2), ("pos_neg1_sat", 7),
                                       ("run_prover_sat_f32", 11), ("expected_critical2_f64", 1)])
def test_device_loop_criticals_equal_the_host_loop(engine, name, gens, precision):
    ir = sid.lemma_ir(name)
    n = sid.ir_nargs(ir)
    lid = engine.register(ir)
    d = engine.prove(lid, generations=gens, nargs=n, fetch=True, precision=precision, device_loop=64)
    h = engine.prove(lid, generations=gens, nargs=n, fetch=True, precision=precision)
    for k in ("cuboids", "leaves", "criticals", "escalated"):
        assert d[k] == h[k], k
    assert d["criticals"] > 0
    assert np.array_equal(bits(kat_expect.sort_boxes(d["boxes"])), bits(kat_expect.sort_boxes(h["boxes"])))


def test_device_loop_shards_sum_to_the_whole_proof(engine):
    lid = engine.register(sid.lemma_ir("one_subcontainer"))
    parts = [engine.prove(lid, part=(i, 3), device_loop=ALL_BLOCKS) for i in range(3)]
    hosts = [engine.prove(lid, part=(i, 3)) for i in range(3)]
    assert [(p["cuboids"], p["leaves"]) for p in parts] == [(p["cuboids"], p["leaves"]) for p in hosts]
    assert [sum(p["cuboids"] for p in parts), sum(p["leaves"] for p in parts)] == PUBLISHED["one_subcontainer"]


def test_device_loop_falls_back_where_the_host_loop_is_needed(engine):
    """Re-iteration needs the host between passes: the option is ignored and the counts are the host loop's."""
    ir = sid.lemma_ir("expected_critical_f64")
    lid = engine.register(ir)
    d = engine.prove(lid, generations=2, max_iterations=4, device_loop=8)
    assert (d["cuboids"], d["leaves"], d["criticals"], d["repeated"]) == (1248, 1024, 128, 168)
