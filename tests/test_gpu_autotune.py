"""GPU tests of the precision form's per-level float-pass mask and of the autotuner (sid_lemma_autotune).

The mask only decides which levels run the float pass before double; counts must stay the published ones,
and with the same mask the oracle's precision form must give the same counts and escalations. The autotuner
keeps only configurations that reproduce its baseline proof's counts and stores the fastest with the lemma
(used by SID_PRECISION_FP32_TUNED proofs).
"""
import json
import os

import pytest

import sid_gb300 as sid

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PUBLISHED = json.load(open(os.path.join(REPO, "tests", "golden", "published_counts.json")))


@pytest.mark.parametrize("name,mask", [("three_subcontainer", 0b01111), ("three_subcontainer", 0b10111),
                                       ("two_subcontainer", 0b0101), ("one_subcontainer", 0b110),
                                       ("seven_subcontainer", 0b011110111)])
def test_partial_float_pass_masks_match_oracle(engine, oracle, name, mask):
    ir = sid.lemma_ir(name)
    lid = engine.register(ir)
    g = engine.prove(lid, precision=sid.PRECISION_FP32, fp32_level_mask=mask)
    o = oracle.prove(ir, fp32_first=True, fp32_level_mask=mask)
    assert (g["cuboids"], g["leaves"], g["criticals"], g["escalated"]) == \
        (o["cuboids"], o["leaves"], o["criticals"], o["escalated"])
    assert [g["cuboids"], g["leaves"]] == PUBLISHED[name]


@pytest.mark.parametrize("name", ["two_subcontainer", "four_subcontainer", "more_subcontainers_2"])
def test_autotune_keeps_published_counts(engine, name):
    lid = engine.register(sid.lemma_ir(name))
    t = engine.autotune(lid, max_seconds=3.0)
    assert t["candidates"] >= 1
    assert t["seconds"] <= t["default_seconds"]
    assert all(e == -1.0 or 0.0 <= e <= 1.0 for e in t["level_escalation"])
    assert t["level_escalation"][-1] < 0.05          # the innermost static level is where float pays off
    r = engine.prove(lid, precision=sid.PRECISION_TUNED)
    assert [r["cuboids"], r["leaves"]] == PUBLISHED[name] and r["criticals"] == 0


def test_tuned_configuration_is_used_by_a_server(engine):
    lid = engine.register(sid.lemma_ir("more_subcontainers_2"))
    t = engine.autotune(lid, max_seconds=3.0)
    direct = engine.prove(lid, precision=sid.PRECISION_TUNED)
    with sid.Server(engine, precision=sid.PRECISION_TUNED) as srv:
        st = srv.wait(srv.submit(lid), 300000)
    assert (st["cuboids"], st["leaves"], st["escalated"]) == (direct["cuboids"], direct["leaves"], direct["escalated"])
    assert t["fp32_level_mask"] != 0


@pytest.mark.parametrize("name", ["top_packing_1", "top_packing_2", "six_subcontainer"])
def test_autotune_tries_the_device_loop_on_short_proofs(engine, name):
    """Proofs under 5 ms also time the device proof loop; whichever form wins, a tuned proof keeps the published
    counts, and a tuned served request (host-driven lanes) gives the same counts and escalations."""
    lid = engine.register(sid.lemma_ir(name))
    t = engine.autotune(lid, max_seconds=3.0)
    assert t["default_seconds"] < 0.005 and t["candidates"] >= 4
    assert t["loop_blocks"] in (0, 38, 152, 608)
    r = engine.prove(lid, precision=sid.PRECISION_TUNED)
    assert [r["cuboids"], r["leaves"]] == PUBLISHED[name] and r["criticals"] == 0
    with sid.Server(engine, precision=sid.PRECISION_TUNED) as srv:
        st = srv.wait(srv.submit(lid), 120000)
    assert (st["cuboids"], st["leaves"], st["escalated"]) == (r["cuboids"], r["leaves"], r["escalated"])
