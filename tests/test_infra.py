"""CPU tests of the host-side pieces: C ABI exports, IR tooling, front-end arithmetic, lemma export."""
import os
import re
import subprocess
import sys
from fractions import Fraction

import numpy as np
import pytest

import sid_gb300 as sid

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(REPO, "include", "sid.h")).read()
    return sorted(set(re.findall(r"\b(sid_[a-z_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(engine_lib):
    names = declared_symbols()
    assert set(names) == set(sid.EXPORTED)
    for n in names:
        assert hasattr(engine_lib, n), n


def test_engine_fails_loudly_without_gpu(engine_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(sid.SidError):
        sid.Engine(0)


def test_codegen_runs_on_all_ir(tmp_path):
    irs = [os.path.join(sid.LEMMA_DIR, f) for f in os.listdir(sid.LEMMA_DIR) if f.endswith(".sidir")]
    irs += [os.path.join(sid.KAT_DIR, f) for f in os.listdir(sid.KAT_DIR) if f.endswith(".sidir")]
    subprocess.run([sys.executable, os.path.join(sid.PKG, "csrc", "codegen.py"), "--out", str(tmp_path), *irs],
                   check=True, stdout=subprocess.DEVNULL)
    assert (tmp_path / "registry.cu").exists()


def test_codegen_writes_bundles(tmp_path):
    """Bundles (bundles.txt beside the IRs): one kernel unit per bundle that calls each lemma's separately compiled
    proof-loop parts, one part unit per bundled lemma, the bundle in the registry; float lemmas and unknown names
    are rejected."""
    irs = [os.path.join(sid.LEMMA_DIR, f) for f in os.listdir(sid.LEMMA_DIR) if f.endswith(".sidir")]
    irs += [os.path.join(sid.KAT_DIR, f) for f in os.listdir(sid.KAT_DIR) if f.endswith(".sidir")]
    bundles = [os.path.join(sid.LEMMA_DIR, "bundles.txt"), os.path.join(sid.KAT_DIR, "bundles.txt")]
    cmd = [sys.executable, os.path.join(sid.PKG, "csrc", "codegen.py"), "--out", str(tmp_path)]
    subprocess.run(cmd + [x for b in bundles for x in ("--bundles", b)] + irs, check=True, stdout=subprocess.DEVNULL)
    unit = (tmp_path / "bundle_subcontainers_4to7.cu").read_text()
    assert "launch_proof_loop_bundle<lemma_four_subcontainer::M, lemma_five_subcontainer::M, " \
           "lemma_six_subcontainer::M, lemma_seven_subcontainer::M>" in unit
    for n in ("four_subcontainer", "five_subcontainer", "six_subcontainer", "seven_subcontainer",
              "expected_critical_f64", "expected_critical2_f64"):
        part = (tmp_path / ("bpart_lemma_%s.cu" % n)).read_text()
        assert "#define SID_LEMMA_DEFS_ONLY" in part and "loop_elements" in part
    reg = (tmp_path / "registry.cu").read_text()
    assert "&bundle_subcontainers_4to7," in reg and "kNumBundles = 2;" in reg
    # the lemma unit included by a part keeps its host launch table out of the part
    lemma = (tmp_path / "lemma_four_subcontainer.cu").read_text()
    assert lemma.count("#ifndef SID_LEMMA_DEFS_ONLY") == 2
    bad = tmp_path / "bad.txt"
    for line in ("f32: expected_critical_f32", "ghost: no_such_lemma", "too_many: a b c d e"):
        bad.write_text(line + "\n")
        r = subprocess.run(cmd + ["--bundles", str(bad)] + irs, capture_output=True, text=True)
        assert r.returncode != 0, line


def test_slow_bounds_are_the_costly_bound_functions():
    """The batch kernel defers cuboids whose propagation reaches a slow bound. One Subcontainer's slow bounds
    are 7 and 10 (a square root, and two square roots with a division); a bound that only copies a
    variable's or a constant's range is never slow."""
    sys.path.insert(0, os.path.join(sid.PKG, "csrc"))
    import codegen
    L = codegen.Lemma(os.path.join(sid.LEMMA_DIR, "one_subcontainer.sidir"))
    slow = [k for k, b in enumerate(L.bounds) if codegen.slow_bound(L, b[2])]
    assert slow == [7, 10]
    for name in sid.lemma_names():
        L = codegen.Lemma(os.path.join(sid.LEMMA_DIR, name + ".sidir"))
        for tgt, d, fn, defined in L.bounds:
            if L.nodes[fn].op in ("arg", "const"):
                assert not codegen.slow_bound(L, fn), (name, fn)


def test_fingerprints_match_cpp_and_python():
    sys.path.insert(0, os.path.join(sid.PKG, "csrc"))
    import codegen
    ir = sid.lemma_ir("one_subcontainer")
    renamed = re.sub(r"^name .*$", "name other", ir, count=1, flags=re.M)
    assert codegen.fingerprint(ir) == codegen.fingerprint(renamed)
    assert codegen.fingerprint(ir) != codegen.fingerprint(ir.replace("split 1 0 256 0", "split 1 0 255 0"))


def test_lemma_ir_matches_unchanged_reference_sources():
    """The committed IR is what the reference's unchanged src/*.cpp produce with this front end."""
    sys.path.insert(0, os.path.join(sid.PKG, "lemmas"))
    import export_lemmas
    ref = export_lemmas.reference_dir()
    if not os.path.isdir(os.path.join(ref, "src")):
        pytest.skip("reference sources not present (set SID_REFERENCE_DIR)")
    r = subprocess.run([sys.executable, os.path.join(sid.PKG, "lemmas", "export_lemmas.py"), "--check",
                        "--reference", ref], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


def test_kat_ir_is_reproducible(tmp_path):
    before = {f: open(os.path.join(sid.KAT_DIR, f)).read() for f in os.listdir(sid.KAT_DIR)}
    subprocess.run([sys.executable, os.path.join(REPO, "tests", "golden", "make_kat_ir.py")], check=True,
                   stdout=subprocess.DEVNULL)
    after = {f: open(os.path.join(sid.KAT_DIR, f)).read() for f in os.listdir(sid.KAT_DIR)}
    assert before == after


def _parse_consts(ir):
    return [l.split() for l in ir.splitlines() if l.startswith("const ")]


def test_folded_constants_are_tight_outward_roundings():
    """Folded irrational constants (e.g. sqrt(1.6), 2/sqrt(5)) are the two doubles around the exact value,
    checked with 256-bit mpmath."""
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.prec = 256
    ir = sid.lemma_ir("one_subcontainer")
    targets = {"sqrt(1.6)": mpmath.sqrt(mpmath.mpf(16) / 10), "2/sqrt(5)": 2 / mpmath.sqrt(5),
               "1/sqrt(2)": 1 / mpmath.sqrt(2)}
    consts = [(float.fromhex(c[2]), float.fromhex(c[3])) for c in _parse_consts(ir)]
    for name, v in targets.items():
        hits = [(lo, hi) for lo, hi in consts if lo <= v <= hi and lo != hi]
        assert hits, name
        lo, hi = hits[0]
        assert np.nextafter(lo, np.inf) == hi, name


def test_decimal_literal_constants_are_exact_or_adjacent():
    ir = sid.lemma_ir("one_subcontainer")
    for c in _parse_consts(ir):
        lo, hi = float.fromhex(c[2]), float.fromhex(c[3])
        assert lo == hi or np.nextafter(lo, np.inf) == hi
        flo, fhi = float.fromhex(c[4]), float.fromhex(c[5])
        assert flo <= lo and hi <= fhi
