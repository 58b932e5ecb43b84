"""GPU test of progress reporting (sid_prove_opts.progress; the reference's progress observer,
default_progress_observer.hpp:30-35, fed by ivarp::run_prover's ProgressPrinter): called between steps with
the queue size, growing counts and one queued element inside the root box."""
import numpy as np
import pytest

import sid_gb300 as sid

pytestmark = pytest.mark.gpu


def test_progress_callback_reports_growing_counts_and_a_queued_box(engine):
    ir = sid.lemma_ir("more_subcontainers_1")
    n = sid.ir_nargs(ir)
    lid = engine.register(ir)
    root = np.asarray(engine.root_box(lid, n)).reshape(n, 2)
    seen = []
    r = engine.prove(lid, precision=sid.PRECISION_FP32, nargs=n, progress=seen.append, progress_first_ms=0,
                     progress_every_ms=0)
    assert r["criticals"] == 0 and len(seen) >= 2
    cub = [s["cuboids"] for s in seen]
    assert cub == sorted(cub) and 0 < cub[-1] <= r["cuboids"]
    assert all(s["leaves"] <= s["cuboids"] for s in seen)
    heads = [s["queue_head"] for s in seen if s["queue_size"] > 0]
    assert heads and all(h is not None for h in heads)
    for h in heads:
        assert np.all(h[:, 0] <= h[:, 1])
        assert np.all(root[:, 0] <= h[:, 0]) and np.all(h[:, 1] <= root[:, 1])


def test_no_progress_before_the_first_delay(engine):
    lid = engine.register(sid.lemma_ir("top_packing_1"))
    seen = []
    engine.prove(lid, nargs=1, progress=seen.append, progress_first_ms=60000, progress_every_ms=1)
    assert seen == []
