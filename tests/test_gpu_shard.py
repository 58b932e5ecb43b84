"""GPU tests of sharded proofs (sid_prove_opts part_index/part_count): each part proves the children i of the
root partition's first split with i % parts == index. On one GPU the parts run one after the other; their
counts must add up to the published counts, each part must equal the oracle's same part, and the parts'
critical boxes together must be the whole proof's."""
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


@pytest.mark.parametrize("precision", [sid.PRECISION_PLAIN, sid.PRECISION_FP32])
@pytest.mark.parametrize("name,parts", [("one_subcontainer", 3), ("three_subcontainer", 2), ("five_subcontainer", 4),
                                        ("top_packing_2", 5)])
def test_parts_sum_to_the_published_counts_and_match_the_oracle(engine, oracle, name, parts, precision):
    ir = sid.lemma_ir(name)
    lid = engine.register(ir)
    res = [engine.prove(lid, precision=precision, part=(i, parts)) for i in range(parts)]
    assert [sum(r["cuboids"] for r in res), sum(r["leaves"] for r in res)] == PUBLISHED[name]
    assert all(r["criticals"] == 0 for r in res)
    o = oracle.prove(ir, fp32_first=precision != sid.PRECISION_PLAIN, part=(1, parts))
    keys = ("cuboids", "leaves", "criticals") + (("escalated",) if precision != sid.PRECISION_PLAIN else ())
    for k in keys:
        assert res[1][k] == o[k], k


def test_parts_criticals_together_are_the_whole_proofs(engine):
    ir = sid.lemma_ir("pos_neg1_sat")
    n = sid.ir_nargs(ir)
    lid = engine.register(ir)
    whole = engine.prove(lid, generations=7, nargs=n, fetch=True)
    parts = [engine.prove(lid, generations=7, nargs=n, fetch=True, part=(i, 2)) for i in range(2)]
    assert sum(p["criticals"] for p in parts) == whole["criticals"] > 0
    got = np.concatenate([p["boxes"] for p in parts if p["criticals"]])
    assert np.array_equal(bits(kat_expect.sort_boxes(got)), bits(kat_expect.sort_boxes(whole["boxes"])))


def test_part_index_outside_part_count_is_rejected(engine):
    lid = engine.register(sid.lemma_ir("top_packing_1"))
    with pytest.raises(sid.SidError):
        engine.prove(lid, part=(3, 3))


@pytest.mark.parametrize("precision", [sid.PRECISION_PLAIN, sid.PRECISION_FP32])
@pytest.mark.parametrize("name,parts,index", [("four_subcontainer", 16, 5), ("more_subcontainers_2", 64, 17),
                                              ("more_subcontainers_1", 128, 37)])
def test_large_lemma_part_matches_the_oracle(engine, oracle, name, parts, index, precision):
    """The three lemmas whose whole proofs the CPU oracle does not run in the test suite (37 M to 1.06 G cuboids):
    one part of the root partition proved by the engine and by the oracle gives the same counts (and escalations in
    the precision form), so these lemmas are pinned to the oracle directly, not only to the published totals."""
    ir = sid.lemma_ir(name)
    lid = engine.register(ir)
    g = engine.prove(lid, precision=precision, part=(index, parts))
    o = oracle.prove(ir, fp32_first=precision != sid.PRECISION_PLAIN, part=(index, parts))
    assert g["cuboids"] > 0
    keys = ("cuboids", "leaves", "criticals") + (("escalated",) if precision != sid.PRECISION_PLAIN else ())
    for k in keys:
        assert g[k] == o[k], k
