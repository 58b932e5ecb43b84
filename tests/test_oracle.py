"""CPU tests of the oracle against the reference's golden numbers (published counts, known-answer tests)."""
import json
import os
import sys

import numpy as np
import pytest

import kat_expect
import sid_gb300 as sid

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PUBLISHED = json.load(open(os.path.join(REPO, "tests", "golden", "published_counts.json")))

# lemmas the oracle proves in seconds here; the four-subcontainer lemma takes ~20 s on 8 threads
FAST = ["top_packing_1", "top_packing_2", "one_subcontainer", "two_subcontainer", "three_subcontainer",
        "five_subcontainer", "six_subcontainer", "seven_subcontainer"]


@pytest.mark.parametrize("name", FAST)
def test_oracle_matches_published_counts(oracle, name):
    r = oracle.prove(sid.lemma_ir(name))
    assert [r["cuboids"], r["leaves"]] == PUBLISHED[name]
    assert r["criticals"] == 0 and r["repeated"] == 0


def test_oracle_four_subcontainer_published_counts(oracle):
    """The Four Subcontainer Lemma (37.2 M cuboids, ~20 s on 8 threads) against its published counts."""
    r = oracle.prove(sid.lemma_ir("four_subcontainer"))
    assert [r["cuboids"], r["leaves"]] == PUBLISHED["four_subcontainer"]
    assert r["criticals"] == 0


@pytest.mark.parametrize("variant", ["f64", "f32"])
def test_oracle_expected_criticals(oracle, variant):
    r = oracle.prove(sid.lemma_ir("expected_critical_" + variant), generations=2, max_criticals=1000)
    assert {k: r[k] for k in kat_expect.EC_COUNTS} == kat_expect.EC_COUNTS
    got = kat_expect.sort_boxes(r["boxes"])
    want = kat_expect.sort_boxes(kat_expect.expected_critical_boxes())
    assert np.array_equal(got, want)


@pytest.mark.parametrize("gen", [0, 1, 2])
@pytest.mark.parametrize("variant", ["f64", "f32"])
def test_oracle_expected_criticals2(oracle, gen, variant):
    r = oracle.prove(sid.lemma_ir("expected_critical2_" + variant), generations=gen,
                     max_criticals=300000 if gen == 2 else 0)
    assert {k: r[k] for k in kat_expect.EC2_COUNTS[gen]} == kat_expect.EC2_COUNTS[gen]
    if gen == 2:
        got = kat_expect.sort_boxes(r["boxes"])
        assert np.array_equal(got, kat_expect.expected_critical2_gen2_boxes())


@pytest.mark.parametrize("name,gens,proves", [("pos_neg1_unsat", 7, True), ("pos_neg1_sat", 7, False),
                                              ("run_prover_unsat_f64", 11, True), ("run_prover_sat_f64", 11, False),
                                              ("run_prover_unsat_f32", 11, True), ("run_prover_sat_f32", 11, False)])
def test_oracle_verdicts(oracle, name, gens, proves):
    r = oracle.prove(sid.lemma_ir(name), generations=gens)
    assert (r["criticals"] == 0) == proves
    assert r["cuboids"] > r["leaves"] > 0


def test_oracle_root_box_inside_ct_bounds(oracle):
    ir = sid.lemma_ir("one_subcontainer")
    box = oracle.root_box(ir, 3)
    assert box[0, 0] == 0.295 or abs(box[0, 0] - 0.295) < 1e-15
    assert np.all(box[:, 0] <= box[:, 1])


@pytest.mark.parametrize("name", ["one_subcontainer", "two_subcontainer", "five_subcontainer", "seven_subcontainer"])
def test_oracle_precision_form_without_float_propagation_keeps_published_counts(oracle, name):
    """With the float pass testing rows on the unpropagated child box (every level, the default), a float
    refutation implies the double one, so counts are the published ones; escalations grow against the form
    that propagates in float first (fewer float refutations)."""
    ir = sid.lemma_ir(name)
    a = oracle.prove(ir, fp32_first=True, fp32_noprop_mask=0)
    b = oracle.prove(ir, fp32_first=True)
    assert [b["cuboids"], b["leaves"]] == PUBLISHED[name] and b["criticals"] == 0
    assert b["escalated"] >= a["escalated"]


@pytest.mark.parametrize("name", [n for n in sid.lemma_names() if "numtype f64" in sid.lemma_ir(n)])
def test_oracle_batch_float_rows_first_is_exact(oracle, name):
    """Testing the constraints in float on the propagated box rounded outward first (the device's batch order)
    changes no verdict and no box: a float refutation is a double refutation."""
    ir = sid.lemma_ir(name)
    n = sid.ir_nargs(ir)
    lo, hi = sid.synthetic_batch(oracle.root_box(ir, n), 1 << 14, seed=0x5EED0009)
    a = oracle.eval_batch(ir, lo, hi)
    b = oracle.eval_batch(ir, lo, hi, float_rows_first=True)
    assert np.array_equal(a[2], b[2])
    assert np.array_equal(a[0].view(np.uint64), b[0].view(np.uint64))
    assert np.array_equal(a[1].view(np.uint64), b[1].view(np.uint64))
    assert len(np.unique(a[2])) >= 2


@pytest.mark.parametrize("name,parts", [("one_subcontainer", 3), ("three_subcontainer", 2), ("top_packing_2", 5)])
def test_oracle_shards_sum_to_the_whole_proof(oracle, name, parts):
    """Sharding the root partition's first split: the parts' counts add up to the published counts."""
    ir = sid.lemma_ir(name)
    res = [oracle.prove(ir, part=(i, parts)) for i in range(parts)]
    assert [sum(r["cuboids"] for r in res), sum(r["leaves"] for r in res)] == PUBLISHED[name]
    assert all(r["cuboids"] > 0 for r in res)


def test_oracle_row_order_is_the_code_generators(oracle):
    """The oracle's copy of the engine's constraint order (used to count the engine's operations) equals the
    order the code generator emits, for every row of every lemma and known-answer system."""
    import tempfile
    sys.path.insert(0, os.path.join(REPO, "squares-in-disk_gb300", "csrc"))
    import codegen
    names = [(n, sid.lemma_ir(n)) for n in sid.lemma_names()]
    names += [(f[:-6], open(os.path.join(sid.KAT_DIR, f)).read()) for f in sorted(os.listdir(sid.KAT_DIR))
              if f.endswith(".sidir")]
    for name, ir in names:
        with tempfile.NamedTemporaryFile("w", suffix=".sidir", delete=False) as f:
            f.write(ir)
        try:
            L = codegen.Lemma(f.name)
        finally:
            os.unlink(f.name)
        for r in range(L.nargs):
            assert oracle.device_row_order(ir, r) == codegen.row_order(L, r), (name, r)
