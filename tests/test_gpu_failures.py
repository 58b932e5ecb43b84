"""Error paths of the C ABI, exercised by host-side injection (no fault is ever caused on the GPU).

sid_debug_inject_failure makes the n-th following device allocation or kernel launch fail on the host, as if
CUDA had returned cudaErrorMemoryAllocation or cudaErrorLaunchFailure, without allocating or launching
anything. Each failure must reach the caller as its status (SID_ERR_NOMEM, SID_ERR_CUDA; a served request as
SID_REQ_FAILED), and the engine and the server must keep proving correctly afterwards. The reference rethrows
a worker's error on the caller's thread (prover/proof_driver.hpp:99-118) and turns CUDA failures into
CUDAError (with_cuda/ivarp_cuda/error.hpp:37-59); here they are status codes across the ABI.
"""
import json
import os

import numpy as np
import pytest

import sid_gb300 as sid

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PUBLISHED = json.load(open(os.path.join(REPO, "tests", "golden", "published_counts.json")))
NOMEM, CUDA = -4, -2


@pytest.fixture(autouse=True)
def disarm():
    yield
    sid.inject_failure(sid.INJECT_ALLOC, 0)
    sid.inject_failure(sid.INJECT_LAUNCH, 0)


def counts(r):
    return [r["cuboids"], r["leaves"]]


@pytest.mark.parametrize("precision", [sid.PRECISION_PLAIN, sid.PRECISION_FP32])
@pytest.mark.parametrize("kind,status", [(sid.INJECT_ALLOC, NOMEM), (sid.INJECT_LAUNCH, CUDA)])
def test_prove_reports_injected_failures_and_recovers(engine, kind, status, precision):
    lid = engine.register(sid.lemma_ir("six_subcontainer"))
    failed = 0
    for countdown in (1, 2, 3, 5, 8, 13, 40):
        sid.inject_failure(kind, countdown)
        try:
            r = engine.prove(lid, precision=precision)
            assert counts(r) == PUBLISHED["six_subcontainer"]     # fewer failure points than the countdown
        except sid.SidError as e:
            failed += 1
            assert e.status == status, str(e)
            assert "injected" in str(e) or "memory" in str(e).lower()
        sid.inject_failure(kind, 0)
        r = engine.prove(lid, precision=precision)
        assert counts(r) == PUBLISHED["six_subcontainer"] and r["criticals"] == 0
    assert failed >= 3


def test_register_survives_an_allocation_failure(engine_lib):
    eng = sid.Engine(0)
    try:
        sid.inject_failure(sid.INJECT_ALLOC, 1)
        with pytest.raises(sid.SidError) as e:
            eng.register(sid.lemma_ir("top_packing_2"))
        assert e.value.status == NOMEM
        lid = eng.register(sid.lemma_ir("top_packing_2"))
        assert counts(eng.prove(lid)) == PUBLISHED["top_packing_2"]
    finally:
        eng.close()


def test_eval_batch_reports_a_launch_failure_and_recovers(engine, oracle):
    ir = sid.lemma_ir("one_subcontainer")
    lid = engine.register(ir)
    lo, hi = sid.synthetic_batch(engine.root_box(lid, 3), 1 << 14, seed=5)
    sid.inject_failure(sid.INJECT_LAUNCH, 1)
    with pytest.raises(sid.SidError) as e:
        engine.eval_batch(lid, lo, hi)
    assert e.value.status == CUDA
    glo, ghi, gv = engine.eval_batch(lid, lo, hi)
    olo, ohi, ov = oracle.eval_batch(ir, lo, hi)
    assert np.array_equal(gv, ov)
    assert np.array_equal(glo.view(np.uint64), olo.view(np.uint64))
    assert np.array_equal(ghi.view(np.uint64), ohi.view(np.uint64))


@pytest.mark.parametrize("kind", [sid.INJECT_ALLOC, sid.INJECT_LAUNCH])
def test_server_fails_the_request_and_keeps_serving(engine, kind):
    lids = {n: engine.register(sid.lemma_ir(n)) for n in ("five_subcontainer", "seven_subcontainer")}
    with sid.Server(engine) as srv:
        warm = srv.submit(lids["five_subcontainer"])             # the lane exists before the injection
        assert srv.wait(warm, 120000)["state"] == sid.REQ_DONE
        srv.release(warm)
        sid.inject_failure(kind, 2)
        bad = srv.submit(lids["five_subcontainer"])
        with pytest.raises(sid.SidError) as e:
            srv.wait(bad, 120000)
        assert e.value.status == (NOMEM if kind == sid.INJECT_ALLOC else CUDA), str(e.value)
        with pytest.raises(sid.SidError):
            srv.poll(bad)
        sid.inject_failure(kind, 0)
        with pytest.raises(sid.SidError):
            srv.criticals(bad, 7, 16)                            # a failed request has no results
        srv.release(bad)
        good = [srv.submit(lids[n]) for n in ("five_subcontainer", "seven_subcontainer", "five_subcontainer")]
        res = [srv.wait(rid, 120000) for rid in good]
        for rid, n, st in zip(good, ("five_subcontainer", "seven_subcontainer", "five_subcontainer"), res):
            assert st["state"] == sid.REQ_DONE and st["proved"], st
            assert counts(st) == PUBLISHED[n]
            srv.release(rid)


def test_server_survives_a_failed_lane_setup(engine):
    """The first request of a lemma creates its lane; if that fails, the waiting requests fail, and the next
    request creates the lane again."""
    lid = engine.register(sid.lemma_ir("seven_subcontainer"))
    with sid.Server(engine) as srv:
        sid.inject_failure(sid.INJECT_ALLOC, 1)
        with pytest.raises(sid.SidError) as e:
            srv.wait(srv.submit(lid), 120000)
        assert e.value.status == NOMEM
        sid.inject_failure(sid.INJECT_ALLOC, 0)
        st = srv.wait(srv.submit(lid), 120000)
        assert st["state"] == sid.REQ_DONE and counts(st) == PUBLISHED["seven_subcontainer"]


def test_budget_below_one_request_still_serves_one_at_a_time(engine):
    """A memory budget smaller than any request's frontier: requests are admitted one at a time (never none),
    and every result is the whole lemma's."""
    lid = engine.register(sid.lemma_ir("six_subcontainer"))
    with sid.Server(engine, memory_budget=1) as srv:
        ids = [srv.submit(lid) for _ in range(3)]
        res = [srv.wait(rid, 120000) for rid in ids]
    for st in res:
        assert st["state"] == sid.REQ_DONE and counts(st) == PUBLISHED["six_subcontainer"]


BATCHED = ["four_subcontainer", "five_subcontainer", "six_subcontainer", "seven_subcontainer"]


@pytest.mark.parametrize("kind,status", [(sid.INJECT_ALLOC, NOMEM), (sid.INJECT_LAUNCH, CUDA)])
def test_device_loop_and_bundle_report_injected_failures_and_recover(engine, kind, status):
    """A failure while a one-kernel proof or a bundle is set up or launched reaches the caller as its status; the
    cached lanes then prove correctly again, in the loop and in the bundle."""
    ids = [engine.register(sid.lemma_ir(n)) for n in BATCHED]
    six = ids[2]
    failed = 0
    for countdown in (1, 2, 3, 5, 8, 13):
        sid.inject_failure(kind, countdown)
        try:
            got = engine.prove_bundle(ids, precision=sid.PRECISION_FP32, blocks=152)
            assert [counts(g) for g in got] == [PUBLISHED[n] for n in BATCHED]
        except sid.SidError as e:
            failed += 1
            assert e.status == status, str(e)
        sid.inject_failure(kind, 0)
        sid.inject_failure(kind, countdown)
        try:
            assert counts(engine.prove(six, precision=sid.PRECISION_FP32, device_loop=152)) == PUBLISHED[BATCHED[2]]
        except sid.SidError as e:
            failed += 1
            assert e.status == status, str(e)
        sid.inject_failure(kind, 0)
    assert failed > 0
    got = engine.prove_bundle(ids, precision=sid.PRECISION_FP32)
    assert [counts(g) for g in got] == [PUBLISHED[n] for n in BATCHED]
    assert counts(engine.prove(six, precision=sid.PRECISION_FP32, device_loop=152)) == PUBLISHED[BATCHED[2]]
