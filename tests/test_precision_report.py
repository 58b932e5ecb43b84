"""CPU test of the precision form's soundness against the 256-bit judge (tests/mp_judge.py), on a few hundred
seeded leaves per lemma: float intervals enclose double intervals, double intervals enclose the 256-bit ones,
and no comparison verdict of float or double contradicts the judge. tests/precision_report.py produces the
full per-lemma width report with the same code."""
import pytest

import precision_report

pytest.importorskip("mpmath")

LEMMAS = ["top_packing_2", "one_subcontainer", "three_subcontainer", "five_subcontainer", "more_subcontainers_2"]


@pytest.mark.parametrize("name", LEMMAS)
def test_float_and_double_are_sound_against_the_256_bit_judge(oracle, name):
    r = precision_report.lemma_report(name, leaves=400, judge_leaves=100, jobs=1)
    assert r["enclosure_violations"] == 0
    assert r["contradicted_verdicts"] == 0
    assert r["width_ratio_f32_over_f64"]["values"] > 0
    # outward float evaluation is never narrower than double; double is within rounding of 256 bits
    assert r["width_ratio_f32_over_f64"]["mean"] >= 1.0
    assert 1.0 <= r["width_ratio_f64_over_mp256"]["mean"] < 1.001
