"""GPU tests of checkpoint/resume (sid_prove with checkpoint_path / stop_after_steps, sid_prove_resume).

A proof stopped after a few steps writes its frontier queue, counters and stored criticals; resuming from the
file must end with exactly the counts (and critical boxes) of the uninterrupted proof, also when the resumed
proof is interrupted and resumed again, and in the precision form.
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


@pytest.mark.parametrize("name,precision", [("more_subcontainers_2", sid.PRECISION_PLAIN),
                                            ("more_subcontainers_2", sid.PRECISION_FP32),
                                            ("two_subcontainer", sid.PRECISION_PLAIN)])
def test_stop_and_resume_gives_the_uninterrupted_counts(engine, tmp_path, name, precision):
    lid = engine.register(sid.lemma_ir(name))
    batch = 32
    full = engine.prove(lid, precision=precision, batch=batch)
    assert [full["cuboids"], full["leaves"]] == PUBLISHED[name]
    assert full["complete"] and full["steps"] >= 6
    a, b = full["steps"] // 3, full["steps"] // 3
    ck = str(tmp_path / "proof.ckpt")
    part = engine.prove(lid, precision=precision, batch=batch, checkpoint=ck, stop_after=a)
    assert not part["complete"] and part["steps"] == a and os.path.exists(ck)
    assert part["cuboids"] < full["cuboids"]
    again = engine.prove(lid, precision=precision, batch=batch, checkpoint=ck, stop_after=b, resume_from=ck)
    assert not again["complete"] and again["steps"] == a + b
    done = engine.prove(lid, precision=precision, batch=batch, resume_from=ck)
    assert done["complete"] and done["steps"] == full["steps"]
    for k in ("cuboids", "leaves", "criticals", "escalated"):
        assert done[k] == full[k], k


def test_resume_keeps_the_critical_boxes(engine, tmp_path):
    ir = sid.lemma_ir("expected_critical2_f64")
    lid = engine.register(ir)
    ck = str(tmp_path / "kat.ckpt")
    part = engine.prove(lid, generations=2, nargs=4, batch=4, checkpoint=ck, stop_after=2)
    assert not part["complete"]
    done = engine.prove(lid, generations=2, nargs=4, batch=4, resume_from=ck, fetch=True)
    assert {k: done[k] for k in kat_expect.EC2_COUNTS[2]} == kat_expect.EC2_COUNTS[2]
    got = kat_expect.sort_boxes(done["boxes"])
    assert np.array_equal(got.view(np.uint64), kat_expect.expected_critical2_gen2_boxes().view(np.uint64))


def test_resume_rejects_a_checkpoint_of_another_lemma(engine, tmp_path):
    a = engine.register(sid.lemma_ir("two_subcontainer"))
    b = engine.register(sid.lemma_ir("three_subcontainer"))
    ck = str(tmp_path / "a.ckpt")
    engine.prove(a, batch=32, checkpoint=ck, stop_after=1)
    with pytest.raises(sid.SidError) as e:
        engine.prove(b, resume_from=ck)
    assert e.value.status == -1 and "another lemma" in str(e.value)
