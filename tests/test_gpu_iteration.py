"""GPU tests of node re-iteration (ProverSettings::max_iterations_per_node > 1).

The reference's CPU prover core runs the static splits of a queue element again on the hull of its surviving
leaves while fewer than max_iterations_per_node passes ran and the hull is still large against the element
(iteration_single_dimension_criterion 0.66, iteration_volume_criterion 0.25), counting each repeat as one
cuboid and one repeated node (ivarp/include/ivarp/cpu_prover/cpu_prover_core.hpp:113-177). Its default for
an unset setting is 4 passes (cpu_prover_core.hpp:79-92), which is what ivarp::run_prover uses when a lemma
program leaves the setting alone. The reference's own tests set 1 or 0, so no published number pins this
path; the CPU oracle restates it from the reference's source, and the engine must match the oracle's counts
(cuboids, leaves, criticals, repeated nodes) and critical boxes exactly.
"""
import numpy as np
import pytest

import kat_expect
import sid_gb300 as sid

pytestmark = pytest.mark.gpu

KATS = [("expected_critical_f64", 2), ("expected_critical_f32", 2), ("expected_critical2_f64", 2),
        ("expected_critical2_f32", 1), ("pos_neg1_sat", 7), ("pos_neg1_unsat", 7), ("run_prover_sat_f64", 11),
        ("run_prover_unsat_f32", 11), ("pos_neg2_sat", 4), ("pos_neg2_unsat", 4)]


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)


@pytest.mark.parametrize("iterations", [2, 4])
@pytest.mark.parametrize("name,gens", KATS)
def test_reiteration_matches_oracle_on_kat_systems(engine, oracle, name, gens, iterations):
    ir = sid.lemma_ir(name)
    n = sid.ir_nargs(ir)
    lid = engine.register(ir)
    g = engine.prove(lid, generations=gens, nargs=n, fetch=True, max_criticals=1 << 20, max_iterations=iterations)
    o = oracle.prove(ir, generations=gens, max_criticals=1 << 20, max_iterations=iterations)
    for k in ("cuboids", "leaves", "criticals", "repeated"):
        assert g[k] == o[k], (k, g[k], o[k])
    if g["criticals"]:
        assert np.array_equal(bits(kat_expect.sort_boxes(g["boxes"])), bits(kat_expect.sort_boxes(o["boxes"])))


def test_reiteration_repeats_nodes_on_a_kat_system(engine):
    """The default of 4 passes re-iterates many nodes of the expected_criticals system (168 of them); one pass
    gives the reference test's published counts."""
    ir = sid.lemma_ir("expected_critical_f64")
    lid = engine.register(ir)
    r4 = engine.prove(lid, generations=2, max_iterations=4)
    r1 = engine.prove(lid, generations=2, max_iterations=1)
    assert (r4["cuboids"], r4["leaves"], r4["criticals"], r4["repeated"]) == (1248, 1024, 128, 168)
    assert {k: r1[k] for k in kat_expect.EC_COUNTS} == kat_expect.EC_COUNTS and r1["repeated"] == 0


@pytest.mark.parametrize("precision", [sid.PRECISION_PLAIN, sid.PRECISION_FP32])
@pytest.mark.parametrize("name", ["top_packing_1", "top_packing_2", "five_subcontainer", "seven_subcontainer",
                                  "one_subcontainer"])
def test_reiteration_matches_oracle_on_lemmas(engine, oracle, name, precision):
    """Lemmas at the reference's default of 4 passes: Top Packing 2 (no static split: every element is its own
    hull) repeats 15 nodes; the others repeat none, and their counts stay the published ones."""
    ir = sid.lemma_ir(name)
    lid = engine.register(ir)
    g = engine.prove(lid, max_iterations=4, precision=precision)
    o = oracle.prove(ir, max_iterations=4)
    for k in ("cuboids", "leaves", "criticals", "repeated"):
        assert g[k] == o[k], (k, g[k], o[k])


def test_reiteration_in_the_served_form(engine, oracle):
    ir = sid.lemma_ir("pos_neg1_unsat")
    lid = engine.register(ir)
    o = oracle.prove(ir, generations=8, max_iterations=3)
    with sid.Server(engine, precision=sid.PRECISION_PLAIN, max_iterations=3) as srv:
        st = srv.wait(srv.submit(lid), 120000)
    assert st["state"] == sid.REQ_DONE
    assert (st["cuboids"], st["leaves"], st["criticals"], st["repeated"]) == \
        (o["cuboids"], o["leaves"], o["criticals"], o["repeated"])
    assert st["repeated"] > 0
