"""CPU test of the lemma description (sid_gb300.describe_ir, the counterpart of the reference's
print_prover_input): every argument, runtime bound and constraint row of each compiled lemma is listed."""
import pytest

import sid_gb300 as sid


@pytest.mark.parametrize("name", sid.lemma_names())
def test_description_lists_arguments_bounds_and_constraints(name):
    ir = sid.lemma_ir(name)
    lines = ir.splitlines()
    nargs = sid.ir_nargs(ir)
    nbounds = sum(1 for l in lines if l.startswith("bound "))
    nrow_constraints = sum(int(l.split()[2]) for l in lines if l.startswith("row "))
    text = sid.describe_ir(ir, root=[[0.0, 1.0]] * nargs)
    head, rest = text.split("[Bounds]\n")
    bounds, cons = rest.split("[Constraints]\n")
    assert head.startswith("[Arguments]\n") and head.count("compile time bounds") == nargs
    assert head.count("initial range") == nargs
    assert len(bounds.splitlines()) == nbounds
    assert sum(1 for l in cons.splitlines() if l.startswith("        ")) == nrow_constraints
    if "acos" in ir:
        assert "acos(" in cons
