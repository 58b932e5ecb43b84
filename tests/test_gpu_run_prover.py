"""The reference's C++ entry point, ivarp::run_prover, proving on the GPU.

tests/run_prover_gpu.cpp is compiled against include/ivarp (the front end the unchanged lemma sources compile
against) and linked with libsid.so; it proves the known-answer systems through run_prover with the settings
of the reference's tests (ivarp/test/expected_criticals.cpp, expected_criticals2.cpp,
positive_and_negative_proof1.cpp, positive_and_negative_proof2.cpp, run_prover.cpp). Checked here:
  * the verdict run_prover returns (true iff no critical cuboid remains, proof_driver.hpp:488);
  * the ProofInformation it fills (the reference tests' exact counts where they state them, else the CPU
    oracle's counts, including repeated nodes when the settings are left at their defaults);
  * the boxes handed to on_critical (bit-exact against the reference tests' closed forms or the oracle);
  * the progress observer: observe_progress between steps, observe_done once, observe_error never;
  * the ProgressPrinter line format, and an engine error surfacing as ivarp::EngineError.
"""
import os
import re
import subprocess

import numpy as np
import pytest

import kat_expect
import sid_gb300 as sid

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)


@pytest.fixture(scope="module")
def runs(engine_lib, tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("run_prover") / "run_prover_gpu")
    libdir = os.path.dirname(sid.LIB_PATH)
    subprocess.run(["g++", "-std=c++17", "-O1", "-I" + os.path.join(REPO, "include"), "-I" + os.path.join(REPO, "tests"),
                    os.path.join(REPO, "tests", "run_prover_gpu.cpp"), "-L" + libdir, "-lsid", "-Wl,-rpath," + libdir,
                    "-lpthread", "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=900)
    assert out.returncode == 0, out.stdout[-2000:] + out.stderr[-2000:]
    runs, boxes, extra = [], {}, {}
    for line in out.stdout.splitlines():
        t = line.split()
        if t[0] == "run":
            r = dict(name=t[1], generations=int(t[2]), iterations=int(t[3]), result=bool(int(t[4])),
                     cuboids=int(t[5]), leaves=int(t[6]), criticals=int(t[7]), repeated=int(t[8]), calls=int(t[9]),
                     progress=int(t[10]), done=int(t[11]), errors=int(t[12]), boxes=[])
            runs.append(r)
        elif t[0] == "box":
            runs[-1]["boxes"].append([float.fromhex(x) for x in t[2:]])
        else:
            extra[t[0]] = line[len(t[0]) + 1:]
    for r in runs:
        if r["boxes"]:
            r["boxes"] = np.array(r["boxes"]).reshape(len(r["boxes"]), -1, 2)
    return runs, extra


def find(runs, name, generations, iterations):
    return next(r for r in runs[0] if (r["name"], r["generations"], r["iterations"]) == (name, generations, iterations))


def test_every_run_reports_to_the_observer_and_the_handler(runs):
    assert len(runs[0]) == 15
    for r in runs[0]:
        assert r["done"] == 1 and r["errors"] == 0, r["name"]
        assert r["calls"] == r["criticals"], r["name"]          # on_critical once per critical cuboid
        assert r["result"] == (r["criticals"] == 0), r["name"]
    assert find(runs, "pos_neg2_sat", 16, 0)["progress"] > 0


@pytest.mark.parametrize("name", ["expected_critical_f64", "expected_critical_f32"])
def test_expected_criticals(runs, name):
    """expected_criticals.cpp:72-94: run_prover returns false with the exact counts and critical boxes."""
    r = find(runs, name, 2, 1)
    assert not r["result"] and r["repeated"] == 0
    assert {k: r[k] for k in kat_expect.EC_COUNTS} == kat_expect.EC_COUNTS
    want = kat_expect.sort_boxes(kat_expect.expected_critical_boxes())
    assert np.array_equal(bits(kat_expect.sort_boxes(r["boxes"])), bits(want))


@pytest.mark.parametrize("gen", [0, 1, 2])
def test_expected_criticals2(runs, oracle, gen):
    """expected_criticals2.cpp:150-226: the counts of 0, 1 and 2 generations (max_iterations_per_node 0)."""
    r = find(runs, "expected_critical2_f64", gen, 0)
    assert not r["result"]
    assert {k: r[k] for k in kat_expect.EC2_COUNTS[gen]} == kat_expect.EC2_COUNTS[gen]
    if gen == 0:
        o = oracle.prove(sid.lemma_ir("expected_critical2_f64"), generations=0, max_iterations=0, max_criticals=1 << 12)
        assert np.array_equal(bits(kat_expect.sort_boxes(r["boxes"])), bits(kat_expect.sort_boxes(o["boxes"])))
    f = find(runs, "expected_critical2_f32", 2, 0)
    assert {k: f[k] for k in kat_expect.EC2_COUNTS[2]} == kat_expect.EC2_COUNTS[2]


def test_default_settings_reiterate_nodes(runs, oracle):
    """Settings left unset: run_prover uses the reference's default of 4 passes per node (cpu_prover_core.hpp:79-92)."""
    r = find(runs, "expected_critical_f64", 2, -1)
    o = oracle.prove(sid.lemma_ir("expected_critical_f64"), generations=2, max_iterations=4, max_criticals=1 << 12)
    assert (r["cuboids"], r["leaves"], r["criticals"], r["repeated"]) == \
        (o["cuboids"], o["leaves"], o["criticals"], o["repeated"]) == (1248, 1024, 128, 168)
    assert np.array_equal(bits(kat_expect.sort_boxes(r["boxes"])), bits(kat_expect.sort_boxes(o["boxes"])))


@pytest.mark.parametrize("name,gens,iters,proved", [
    ("pos_neg1_sat", 7, 1, False), ("pos_neg1_unsat", 7, 1, True),
    ("pos_neg2_sat", 16, 0, False), ("pos_neg2_unsat", 16, 0, True),
    ("run_prover_sat_f64", 11, 1, False), ("run_prover_unsat_f64", 11, 1, True),
    ("run_prover_sat_f32", 11, 1, False), ("run_prover_unsat_f32", 11, 1, True)])
def test_verdicts_and_counts(runs, oracle, name, gens, iters, proved):
    """positive_and_negative_proof1.cpp:79,106, positive_and_negative_proof2.cpp:41,64, run_prover.cpp:65,88: the
    verdicts; counts and critical boxes equal the oracle's."""
    r = find(runs, name, gens, iters)
    assert r["result"] == proved
    ir = sid.lemma_ir(name)
    o = oracle.prove(ir, generations=gens, max_iterations=max(iters, 1), max_criticals=1 << 20)
    for k in ("cuboids", "leaves", "criticals", "repeated"):
        assert r[k] == o[k], k
    if len(r["boxes"]):
        assert np.array_equal(bits(kat_expect.sort_boxes(r["boxes"])), bits(kat_expect.sort_boxes(o["boxes"])))
    if name.startswith("run_prover_sat"):   # run_prover.cpp:66-70
        assert r["cuboids"] > 64 * 32 and r["leaves"] > r["cuboids"] // 2 and r["leaves"] > r["criticals"]


def test_progress_printer_line(runs):
    line = runs[1]["printer"]
    assert re.fullmatch(r"Queue size: \d+, cuboids: \d+\(\d+\), x: \[[^\]]+\], y: \[[^\]]+\]", line), line


def test_engine_error_surfaces_as_exception(runs):
    status, msg = runs[1]["error"].split(" ", 1)
    assert int(status) == -3 and "sid_lemma_register" in msg and "no GPU kernels" in msg
