"""GPU parity tests: the engine (through the C ABI) against the CPU oracle and the reference's golden numbers.

Integer results (cuboid / leaf / critical counts) must be identical; interval endpoints (root boxes,
propagated boxes, critical boxes) must be bit-identical doubles.
"""
import json
import os

import numpy as np
import pytest

import kat_expect
import sid_gb300 as sid

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PUBLISHED = json.load(open(os.path.join(REPO, "tests", "golden", "published_counts.json")))


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)


def built_lemmas():
    return sid.lemma_names()


@pytest.mark.parametrize("name", built_lemmas())
def test_root_box_bit_exact(engine, oracle, name):
    ir = sid.lemma_ir(name)
    n = sid.ir_nargs(ir)
    lid = engine.register(ir)
    assert np.array_equal(bits(engine.root_box(lid, n)), bits(oracle.root_box(ir, n)))


@pytest.mark.parametrize("name", built_lemmas())
def test_full_proof_counts_match_published(engine, name):
    ir = sid.lemma_ir(name)
    lid = engine.register(ir)
    r = engine.prove(lid)
    assert [r["cuboids"], r["leaves"]] == PUBLISHED[name]
    assert r["criticals"] == 0


@pytest.mark.parametrize("name", built_lemmas())
def test_eval_batch_bit_exact(engine, oracle, name):
    ir = sid.lemma_ir(name)
    n = sid.ir_nargs(ir)
    lid = engine.register(ir)
    root = engine.root_box(lid, n)
    lo, hi = sid.synthetic_batch(root, 1 << 15, seed=0x5EED0001)
    glo, ghi, gv = engine.eval_batch(lid, lo, hi)
    olo, ohi, ov = oracle.eval_batch(ir, lo, hi)
    assert np.array_equal(gv, ov)
    assert np.array_equal(bits(glo), bits(olo))
    assert np.array_equal(bits(ghi), bits(ohi))
    assert len(np.unique(gv)) >= 2, "batch should exercise more than one verdict"


@pytest.mark.parametrize("n", [(2 << 20) + 777, (4 << 20) + 4321])
def test_host_batch_pipeline_equals_device_batch(engine, n):
    """sid_eval_batch moves host buffers in chunks (uniform below 4 Mi cuboids, with short first and last chunks
    above); every output must equal the device-resident single-call evaluation bit for bit."""
    torch = pytest.importorskip("torch")
    ir = sid.lemma_ir("one_subcontainer")
    lid = engine.register(ir)
    lo, hi = sid.synthetic_batch(engine.root_box(lid, sid.ir_nargs(ir)), n, seed=0x5EED0005)
    hlo, hhi, hv = engine.eval_batch(lid, lo, hi)
    d_lo, d_hi = torch.from_numpy(lo).cuda(), torch.from_numpy(hi).cuda()
    o_lo, o_hi = torch.empty_like(d_lo), torch.empty_like(d_hi)
    o_v = torch.empty(n, dtype=torch.int8, device="cuda")
    engine.eval_batch_device(lid, d_lo.data_ptr(), d_hi.data_ptr(), n, o_lo.data_ptr(), o_hi.data_ptr(), o_v.data_ptr())
    torch.cuda.synchronize()
    assert np.array_equal(hv, o_v.cpu().numpy())
    assert np.array_equal(bits(hlo), bits(o_lo.cpu().numpy()))
    assert np.array_equal(bits(hhi), bits(o_hi.cpu().numpy()))


@pytest.mark.parametrize("name", ["one_subcontainer", "seven_subcontainer", "more_subcontainers_2", "top_packing_1"])
def test_batch_order_modes_give_identical_results(engine, name):
    """Ordered, unordered and adaptive batch evaluation give the same verdicts and boxes bit for bit; after a
    synchronous call the sampled share of cuboids that needed the double constraints is available."""
    ir = sid.lemma_ir(name)
    lid = engine.register(ir)
    lo, hi = sid.synthetic_batch(engine.root_box(lid, sid.ir_nargs(ir)), 1 << 16, seed=0x5EED0007)
    outs = []
    for mode in (sid.BATCH_ORDER_ON, sid.BATCH_ORDER_OFF, sid.BATCH_ORDER_AUTO):
        engine.batch_order(lid, mode)
        outs.append(engine.eval_batch(lid, lo, hi))
    for o in outs[1:]:
        assert np.array_equal(o[2], outs[0][2])
        assert np.array_equal(bits(o[0]), bits(outs[0][0])) and np.array_equal(bits(o[1]), bits(outs[0][1]))
    share = engine.batch_order(lid)
    assert 0.0 <= share <= 1.0
    if name == "one_subcontainer":
        assert share < 0.05      # the float test decides nearly every cuboid of this batch
    with pytest.raises(sid.SidError):
        engine.batch_order(lid, 7)


@pytest.mark.parametrize("variant", ["f64", "f32"])
def test_expected_criticals_kat(engine, variant):
    ir = sid.lemma_ir("expected_critical_" + variant)
    lid = engine.register(ir)
    r = engine.prove(lid, generations=2, nargs=2, fetch=True)
    assert {k: r[k] for k in kat_expect.EC_COUNTS} == kat_expect.EC_COUNTS
    got = kat_expect.sort_boxes(r["boxes"])
    want = kat_expect.sort_boxes(kat_expect.expected_critical_boxes())
    assert np.array_equal(bits(got), bits(want))


@pytest.mark.parametrize("gen", [0, 1, 2])
@pytest.mark.parametrize("variant", ["f64", "f32"])
def test_expected_criticals2_kat(engine, gen, variant):
    ir = sid.lemma_ir("expected_critical2_" + variant)
    lid = engine.register(ir)
    r = engine.prove(lid, generations=gen, nargs=4, fetch=(gen == 2))
    assert {k: r[k] for k in kat_expect.EC2_COUNTS[gen]} == kat_expect.EC2_COUNTS[gen]
    if gen == 2:
        assert np.array_equal(bits(kat_expect.sort_boxes(r["boxes"])),
                              bits(kat_expect.expected_critical2_gen2_boxes()))


@pytest.mark.parametrize("name,gens", [("pos_neg1_unsat", 7), ("pos_neg1_sat", 7), ("run_prover_unsat_f64", 11),
                                       ("run_prover_sat_f64", 11), ("run_prover_unsat_f32", 11),
                                       ("run_prover_sat_f32", 11), ("pos_neg2_unsat", 4), ("pos_neg2_sat", 4)])
def test_kat_systems_match_oracle(engine, oracle, name, gens):
    ir = sid.lemma_ir(name)
    n = sid.ir_nargs(ir)
    lid = engine.register(ir)
    g = engine.prove(lid, generations=gens, nargs=n, fetch=True, max_criticals=1 << 20)
    o = oracle.prove(ir, generations=gens, max_criticals=1 << 20)
    for k in ("cuboids", "leaves", "criticals"):
        assert g[k] == o[k], k
    if g["criticals"]:
        assert np.array_equal(bits(kat_expect.sort_boxes(g["boxes"])), bits(kat_expect.sort_boxes(o["boxes"])))


def test_small_batches_and_chunking_give_same_counts(engine):
    """Batch size and level-list chunking must not change the counts (they are order independent)."""
    ir = sid.lemma_ir("two_subcontainer")
    lid = engine.register(ir)
    a = engine.prove(lid)
    b = engine.prove(lid, batch=37)
    assert (a["cuboids"], a["leaves"]) == (b["cuboids"], b["leaves"])


def test_unknown_lemma_is_rejected(engine):
    ir = sid.lemma_ir("one_subcontainer").replace("split 1 0 256 0", "split 1 0 255 0")
    with pytest.raises(sid.SidError) as e:
        engine.register(ir)
    assert e.value.status == -3
