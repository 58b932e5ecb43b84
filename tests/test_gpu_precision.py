"""GPU tests of the precision form (SID_PRECISION_FP32_ESCALATE): every child cuboid is first tested in FP32
with outward rounding (by default on its unpropagated float box, optionally after a float propagation); only
children FP32 cannot refute are evaluated in FP64, whose results are used.

The oracle restates the same form on the CPU (ProveOptions::fp32_first), so counts, the number of escalated
children and the critical boxes must agree exactly. Every lemma must still be proved (no critical cuboid
in the final generation), and the cuboid counts are compared with the reference's published counts: the
form may differ from them only where FP32 refutes a child that FP64 would not.
"""
import json
import os

import numpy as np
import pytest

import kat_expect
import sid_gb300 as sid

pytestmark = pytest.mark.gpu

PRECISION_FP32 = 1
REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PUBLISHED = json.load(open(os.path.join(REPO, "tests", "golden", "published_counts.json")))
ORACLE_FAST = ["top_packing_1", "top_packing_2", "one_subcontainer", "two_subcontainer", "three_subcontainer",
               "five_subcontainer", "six_subcontainer", "seven_subcontainer"]


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)


@pytest.mark.parametrize("name", ORACLE_FAST)
def test_precision_form_matches_oracle(engine, oracle, name):
    ir = sid.lemma_ir(name)
    lid = engine.register(ir)
    g = engine.prove(lid, precision=PRECISION_FP32)
    o = oracle.prove(ir, fp32_first=True)
    assert (g["cuboids"], g["leaves"], g["criticals"]) == (o["cuboids"], o["leaves"], o["criticals"])
    assert g["escalated"] == o["escalated"]
    assert g["escalated"] < g["cuboids"]


@pytest.mark.parametrize("name", ORACLE_FAST)
def test_split_invariant_float_pass_matches_oracle(engine, oracle, name):
    """Float pass without propagation on every level (k_prelude_f32 + k_filter_hoisted where the level has a
    split-invariant form): counts and escalations equal the oracle's form without float propagation, and
    the counts are the published ones."""
    ir = sid.lemma_ir(name)
    lid = engine.register(ir)
    g = engine.prove(lid, precision=PRECISION_FP32, fp32_noprop_mask=0xFFFFFFFF)
    o = oracle.prove(ir, fp32_first=True, fp32_noprop_mask=0xFFFFFFFF)
    for k in ("cuboids", "leaves", "criticals", "escalated"):
        assert g[k] == o[k], k
    assert [g["cuboids"], g["leaves"]] == PUBLISHED[name]


@pytest.mark.parametrize("name,gens", [("pos_neg1_sat", 7), ("run_prover_sat_f64", 11), ("pos_neg2_sat", 4)])
def test_split_invariant_float_pass_criticals_match_oracle(engine, oracle, name, gens):
    ir = sid.lemma_ir(name)
    n = sid.ir_nargs(ir)
    lid = engine.register(ir)
    g = engine.prove(lid, generations=gens, nargs=n, fetch=True, precision=PRECISION_FP32, fp32_noprop_mask=0xFFFFFFFF)
    o = oracle.prove(ir, generations=gens, max_criticals=1 << 20, fp32_first=True, fp32_noprop_mask=0xFFFFFFFF)
    for k in ("cuboids", "leaves", "criticals", "escalated"):
        assert g[k] == o[k], k
    assert np.array_equal(bits(kat_expect.sort_boxes(g["boxes"])), bits(kat_expect.sort_boxes(o["boxes"])))


def test_split_invariant_float_pass_acos_lemma(engine):
    """The lemmas with acos keep their published counts with the split-invariant float pass."""
    for name in ("more_subcontainers_2", "more_subcontainers_1"):
        lid = engine.register(sid.lemma_ir(name))
        r = engine.prove(lid, precision=PRECISION_FP32, fp32_noprop_mask=0xFFFFFFFF)
        assert [r["cuboids"], r["leaves"]] == PUBLISHED[name] and r["criticals"] == 0


@pytest.mark.parametrize("name", ["one_subcontainer", "three_subcontainer", "five_subcontainer", "seven_subcontainer"])
def test_propagating_float_pass_matches_oracle(engine, oracle, name):
    """The float pass that propagates in float first on every level (fp32_noprop_mask 0): counts and escalations
    equal the oracle's same form, and the counts are the published ones."""
    ir = sid.lemma_ir(name)
    lid = engine.register(ir)
    g = engine.prove(lid, precision=PRECISION_FP32, fp32_noprop_mask=0)
    o = oracle.prove(ir, fp32_first=True, fp32_noprop_mask=0)
    for k in ("cuboids", "leaves", "criticals", "escalated"):
        assert g[k] == o[k], k
    assert [g["cuboids"], g["leaves"]] == PUBLISHED[name]


def test_precision_form_acos_lemma_matches_oracle(engine, oracle):
    """The float pass bounds acos with acos_bound_f32 (sound, not correctly rounded); the oracle restates it, so
    the escalations of a lemma that uses acos (123 M cuboids; about a minute in the oracle) agree exactly."""
    ir = sid.lemma_ir("more_subcontainers_2")
    lid = engine.register(ir)
    g = engine.prove(lid, precision=PRECISION_FP32)
    o = oracle.prove(ir, fp32_first=True)
    for k in ("cuboids", "leaves", "criticals", "escalated"):
        assert g[k] == o[k], k
    assert [g["cuboids"], g["leaves"]] == PUBLISHED["more_subcontainers_2"]


@pytest.mark.parametrize("name", sid.lemma_names())
def test_precision_form_proves_every_lemma(engine, name):
    lid = engine.register(sid.lemma_ir(name))
    r = engine.prove(lid, precision=PRECISION_FP32)
    assert r["criticals"] == 0
    cuboids, leaves = PUBLISHED[name]
    # the default float pass tests unpropagated boxes, so a float refutation is a double one: the counts are
    # the published ones by construction
    assert (r["cuboids"], r["leaves"]) == (cuboids, leaves)


@pytest.mark.parametrize("name,gens", [("pos_neg1_sat", 7), ("run_prover_sat_f64", 11), ("pos_neg2_sat", 4)])
def test_precision_form_criticals_match_oracle(engine, oracle, name, gens):
    ir = sid.lemma_ir(name)
    n = sid.ir_nargs(ir)
    lid = engine.register(ir)
    g = engine.prove(lid, generations=gens, nargs=n, fetch=True, precision=PRECISION_FP32)
    o = oracle.prove(ir, generations=gens, max_criticals=1 << 20, fp32_first=True)
    for k in ("cuboids", "leaves", "criticals", "escalated"):
        assert g[k] == o[k], k
    assert g["criticals"] > 0
    assert np.array_equal(bits(kat_expect.sort_boxes(g["boxes"])), bits(kat_expect.sort_boxes(o["boxes"])))


def test_precision_form_expected_criticals2_boxes_are_double_results(engine):
    """Survivors are evaluated in double, so the critical boxes of the known-answer test are the exact ones."""
    ir = sid.lemma_ir("expected_critical2_f64")
    lid = engine.register(ir)
    r = engine.prove(lid, generations=2, nargs=4, fetch=True, precision=PRECISION_FP32)
    assert {k: r[k] for k in kat_expect.EC2_COUNTS[2]} == kat_expect.EC2_COUNTS[2]
    assert np.array_equal(bits(kat_expect.sort_boxes(r["boxes"])), bits(kat_expect.expected_critical2_gen2_boxes()))


def test_precision_form_on_float_lemma_is_plain(engine):
    ir = sid.lemma_ir("expected_critical_f32")
    lid = engine.register(ir)
    a = engine.prove(lid, generations=2, nargs=2)
    b = engine.prove(lid, generations=2, nargs=2, precision=PRECISION_FP32)
    assert (a["cuboids"], a["leaves"], a["criticals"]) == (b["cuboids"], b["leaves"], b["criticals"])
    assert b["escalated"] == 0


def test_unknown_precision_mode_is_rejected(engine):
    lid = engine.register(sid.lemma_ir("top_packing_1"))
    with pytest.raises(sid.SidError) as e:
        engine.prove(lid, precision=7)
    assert e.value.status == -1
