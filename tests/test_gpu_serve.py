"""GPU tests of the served form (sid_server_*): a request loop with continuous batching.

* Whole-lemma requests reproduce the published counts (plain form) and sid_prove's counts (precision form).
* Each request's result is the same alone and in a mix: seeded synthetic sub-box requests over several lemmas
  are run one at a time, then all submitted at once (so their elements share steps and lanes run
  concurrently); counts are integers and must be identical, critical boxes bit-identical as sets.
* A memory budget smaller than any request admits requests one at a time without changing results.
* The known-answer test with 262,144 critical boxes comes back exactly through a request.
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
WAIT_MS = 300000


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)


def _register(engine, name):
    ir = sid.lemma_ir(name)
    return engine.register(ir), sid.ir_nargs(ir)


def _mix(engine, seed):
    """Seeded synthetic requests: (lemma id, nargs, boxes)."""
    rng = np.random.default_rng(seed)
    out = []
    for name, k in [("one_subcontainer", 1), ("two_subcontainer", 8), ("five_subcontainer", 64),
                    ("more_subcontainers_2", 8), ("top_packing_2", 16), ("one_subcontainer", 64),
                    ("three_subcontainer", 4), ("six_subcontainer", 1), ("more_subcontainers_1", 2),
                    ("top_packing_1", 1), ("seven_subcontainer", 32), ("four_subcontainer", 8),
                    ("pos_neg1_sat", 4), ("run_prover_sat_f64", 16), ("pos_neg1_sat", None)]:
        lid, nargs = _register(engine, name)
        # k None: the whole lemma (root partition); this satisfiable system always leaves criticals
        boxes = None if k is None else sid.synthetic_request(engine.root_box(lid, nargs), rng, k=k)
        out.append((lid, nargs, boxes))
    return out


def _result(srv, rid, nargs):
    st = srv.wait(rid, WAIT_MS)
    assert st["state"] == sid.REQ_DONE
    boxes = srv.criticals(rid, nargs, st["stored"]) if st["stored"] else np.zeros((0, nargs, 2))
    srv.release(rid)
    return st, kat_expect.sort_boxes(boxes) if len(boxes) else boxes


def test_whole_lemma_requests_match_published_counts(engine):
    names = ["top_packing_1", "top_packing_2", "one_subcontainer", "two_subcontainer", "three_subcontainer",
             "five_subcontainer", "six_subcontainer", "seven_subcontainer", "four_subcontainer",
             "more_subcontainers_2"]
    with sid.Server(engine, precision=sid.PRECISION_PLAIN) as srv:
        ids = {name: srv.submit(_register(engine, name)[0]) for name in names}
        for name, rid in ids.items():
            st = srv.wait(rid, WAIT_MS)
            assert [st["cuboids"], st["leaves"]] == PUBLISHED[name], name
            assert st["proved"] and st["criticals"] == 0
            assert st["seconds_to_verdict"] >= st["seconds_queued"] >= 0


def test_whole_lemma_requests_match_sid_prove_in_precision_form(engine):
    names = ["two_subcontainer", "five_subcontainer", "more_subcontainers_1"]
    with sid.Server(engine, precision=sid.PRECISION_FP32) as srv:
        ids = {name: srv.submit(_register(engine, name)[0]) for name in names}
        for name, rid in ids.items():
            st = srv.wait(rid, WAIT_MS)
            p = engine.prove(_register(engine, name)[0], precision=sid.PRECISION_FP32)
            assert (st["cuboids"], st["leaves"], st["escalated"]) == (p["cuboids"], p["leaves"], p["escalated"])


@pytest.mark.parametrize("precision", [sid.PRECISION_PLAIN, sid.PRECISION_FP32])
def test_results_are_the_same_alone_and_in_the_mix(engine, precision):
    reqs = _mix(engine, seed=0xC0FFEE + precision)
    with sid.Server(engine, precision=precision, generations=3, max_criticals=1 << 16) as srv:
        alone = [_result(srv, srv.submit(lid, boxes), nargs) for lid, nargs, boxes in reqs]
        ids = [srv.submit(lid, boxes) for lid, nargs, boxes in reqs]
        mixed = [_result(srv, rid, nargs) for rid, (lid, nargs, boxes) in zip(ids, reqs)]
    for (a, ca), (m, cm) in zip(alone, mixed):
        for k in ("cuboids", "leaves", "criticals", "escalated", "stored", "proved"):
            assert a[k] == m[k], k
        assert np.array_equal(bits(ca), bits(cm))
    assert any(a["criticals"] > 0 for a, _ in alone), "the mix should exercise unproved requests"
    assert any(a["proved"] for a, _ in alone)


def test_tiny_memory_budget_admits_one_request_at_a_time(engine):
    reqs = _mix(engine, seed=7)[:6]
    with sid.Server(engine, generations=3) as srv:
        base = [_result(srv, srv.submit(lid, boxes), nargs)[0] for lid, nargs, boxes in reqs]
    with sid.Server(engine, generations=3, memory_budget=1) as srv:
        ids = [srv.submit(lid, boxes) for lid, nargs, boxes in reqs]
        tight = [_result(srv, rid, nargs)[0] for rid, (lid, nargs, boxes) in zip(ids, reqs)]
    for a, b in zip(base, tight):
        assert (a["cuboids"], a["leaves"], a["criticals"]) == (b["cuboids"], b["leaves"], b["criticals"])
    # one at a time: every later request waited for admission
    assert all(t["seconds_queued"] > 0 for t in tight[1:])


def test_known_answer_criticals_through_a_request(engine):
    lid, nargs = _register(engine, "expected_critical2_f64")
    with sid.Server(engine, precision=sid.PRECISION_PLAIN, generations=2, max_criticals=300000) as srv:
        rid = srv.submit(lid)
        st, boxes = _result(srv, rid, nargs)
    assert {k: st[k] for k in kat_expect.EC2_COUNTS[2]} == kat_expect.EC2_COUNTS[2]
    assert np.array_equal(bits(boxes), bits(kat_expect.expected_critical2_gen2_boxes()))


def test_submit_rejects_bad_requests(engine):
    lid, nargs = _register(engine, "one_subcontainer")
    with sid.Server(engine) as srv:
        bad = np.array([[[0.5, 0.4]] * nargs])
        with pytest.raises(sid.SidError) as e:
            srv.submit(lid, bad)
        assert e.value.status == -1
        with pytest.raises(sid.SidError):
            srv.submit(12345)
        with pytest.raises(sid.SidError):
            srv.poll(987654321)
