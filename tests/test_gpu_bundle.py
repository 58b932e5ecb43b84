"""GPU tests of bundled proofs (sid_prove_bundle): several lemmas proved together by one persistent kernel whose
grid drains the step lists of all of them at once. Each lemma's counts, escalations and critical boxes must be
exactly those of the lemma proved alone (and so the reference's published counts), whatever the grid size and
the order in which the caller lists the lemmas."""
import json
import os

import numpy as np
import pytest

import kat_expect
import sid_gb300 as sid

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PUBLISHED = json.load(open(os.path.join(REPO, "tests", "golden", "published_counts.json")))
BATCHED = ["four_subcontainer", "five_subcontainer", "six_subcontainer", "seven_subcontainer"]


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)


@pytest.mark.parametrize("precision", [sid.PRECISION_PLAIN, sid.PRECISION_FP32])
def test_bundle_counts_equal_each_proof_alone(engine, precision):
    ids = [engine.register(sid.lemma_ir(n)) for n in BATCHED]
    got = engine.prove_bundle(ids, precision=precision)
    for name, lid, g in zip(BATCHED, ids, got):
        alone = engine.prove(lid, precision=precision)
        assert [g["cuboids"], g["leaves"]] == PUBLISHED[name], name
        assert g["criticals"] == 0 and g["complete"]
        assert g["escalated"] == alone["escalated"], name
        if precision == sid.PRECISION_PLAIN:
            assert g["escalated"] == 0


@pytest.mark.parametrize("blocks", [1, 7, 152, 0])
def test_bundle_counts_do_not_depend_on_the_grid_or_the_order(engine, blocks):
    ids = [engine.register(sid.lemma_ir(n)) for n in BATCHED]
    order = [3, 1, 0, 2]
    got = engine.prove_bundle([ids[k] for k in order], precision=sid.PRECISION_FP32, blocks=blocks)
    for k, g in zip(order, got):
        assert [g["cuboids"], g["leaves"]] == PUBLISHED[BATCHED[k]], BATCHED[k]


@pytest.mark.parametrize("precision", [sid.PRECISION_PLAIN, sid.PRECISION_FP32])
@pytest.mark.parametrize("gens", [1, 2, 3])
def test_bundle_criticals_equal_each_proof_alone_and_the_oracle(engine, oracle, precision, gens):
    """The reference's expected_criticals systems (double forms), bundled: exact critical boxes."""
    names = ["expected_critical_f64", "expected_critical2_f64"]
    irs = [sid.lemma_ir(n) for n in names]
    nargs = [sid.ir_nargs(ir) for ir in irs]
    ids = [engine.register(ir) for ir in irs]
    got = engine.prove_bundle(ids, generations=gens, precision=precision, nargs=nargs, fetch=True, blocks=64)
    for name, ir, lid, n, g in zip(names, irs, ids, nargs, got):
        alone = engine.prove(lid, generations=gens, nargs=n, fetch=True, precision=precision)
        want = oracle.prove(ir, generations=gens, max_criticals=1 << 20, fp32_first=precision == sid.PRECISION_FP32)
        for k in ("cuboids", "leaves", "criticals", "escalated"):
            assert g[k] == alone[k], (name, k)
        for k in ("cuboids", "leaves", "criticals"):
            assert g[k] == want[k], (name, k)
        assert g["criticals"] > 0
        if g["criticals"] > g["stored"]:
            continue          # beyond the store's capacity, which criticals are kept depends on the order
        assert np.array_equal(bits(kat_expect.sort_boxes(g["boxes"])), bits(kat_expect.sort_boxes(alone["boxes"])))
        assert np.array_equal(bits(kat_expect.sort_boxes(g["boxes"])), bits(kat_expect.sort_boxes(want["boxes"])))


def test_bundle_rejects_what_it_cannot_prove(engine):
    four = engine.register(sid.lemma_ir("four_subcontainer"))
    five = engine.register(sid.lemma_ir("five_subcontainer"))
    one = engine.register(sid.lemma_ir("one_subcontainer"))
    f32 = engine.register(sid.lemma_ir("expected_critical_f32"))
    with pytest.raises(sid.SidError) as e:
        engine.prove_bundle([four, five])                 # no bundle was generated for this pair
    assert e.value.status == -3
    with pytest.raises(sid.SidError) as e:
        engine.prove_bundle([one, four, five, f32])       # a float lemma
    assert e.value.status == -6
    with pytest.raises(sid.SidError) as e:
        engine.prove_bundle([four, four])
    assert e.value.status == -1
    with pytest.raises(sid.SidError) as e:
        engine.prove_bundle([])
    assert e.value.status == -1
    # the engine proves correctly afterwards
    ids = [engine.register(sid.lemma_ir(n)) for n in BATCHED]
    got = engine.prove_bundle(ids, precision=sid.PRECISION_FP32)
    assert [[g["cuboids"], g["leaves"]] for g in got] == [PUBLISHED[n] for n in BATCHED]
