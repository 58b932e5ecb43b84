"""CPU tests of the request-scheduling planner of the served form (squares-in-disk_gb300/csrc/serve_plan.hpp):
admission under a device-memory budget, the fair-share filling of a lane step from many requests, and
frontier-queue sizing. The same header is compiled into the engine; here it is built for the host with
tests/serve_plan_check.cpp."""
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "squares-in-disk_gb300", "csrc")


@pytest.fixture(scope="module")
def plan(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("plan") / "serve_plan_check")
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-I", CSRC, os.path.join(HERE, "serve_plan_check.cpp"),
                    "-o", exe], check=True)

    def run(lines):
        out = subprocess.run([exe], input="\n".join(lines) + "\n", capture_output=True, text=True, check=True)
        return out.stdout.splitlines()
    return run


def _takes(s):
    return [tuple(int(x) for x in t.split()) for t in s.split(";")] if s else []


def test_admission(plan):
    out = plan(["admit 0 100 0 10 40 40 40",      # budget fits two
                "admit 0 100 0 10 500 1",         # oversized first request, nothing running: admitted alone
                "admit 0 100 1 10 500",           # oversized while another runs: waits
                "admit 0 100 0 1 10 10",          # one free slot
                "admit 90 100 2 10 20",           # no room
                "admit 0 100 0 10"])              # nothing pending
    assert [int(x) for x in out] == [2, 1, 0, 1, 0, 0]


def test_fill_step_examples(plan):
    out = plan(["fill 100 0 1000", "fill 100 3 10 5 1000", "fill 100 1 0 2 30 4 30 6 30", "fill 90 1 50 2 50 3 50",
                "fill 10 1 0 2 0", "fill 0 1 5"])
    assert _takes(out[0]) == [(0, 900, 100, 0)]
    assert _takes(out[1]) == [(3, 0, 10, 0), (5, 910, 90, 10)]         # the small request gets all it has
    assert _takes(out[2]) == [(2, 0, 30, 0), (4, 0, 30, 30), (6, 0, 30, 60)]
    assert _takes(out[3]) == [(1, 20, 30, 0), (2, 20, 30, 30), (3, 20, 30, 60)]
    assert _takes(out[4]) == [] and _takes(out[5]) == []


def test_fill_step_properties(plan):
    rng = np.random.default_rng(5)
    cases = []
    for _ in range(300):
        k = int(rng.integers(1, 12))
        q = [int(x) for x in rng.choice([0, 1, 3, 50, 1000, 70000], size=k)]
        cap = int(rng.choice([1, 7, 100, 65536]))
        cases.append((cap, q))
    out = plan(["fill %d %s" % (cap, " ".join("%d %d" % (i, x) for i, x in enumerate(q))) for cap, q in cases])
    for (cap, q), line in zip(cases, out):
        takes = _takes(line)
        counts = {s: c for s, b, c, d in takes}
        assert sum(counts.values()) == min(cap, sum(q))                   # fills the step when work exists
        dst = 0
        for s, b, c, d in takes:
            assert d == dst and c > 0 and b + c == q[s]                   # contiguous, from the queue top
            dst += c
        with_work = [i for i, x in enumerate(q) if x > 0]
        if with_work:
            fair = cap // len(with_work)
            for i in with_work:                                           # everyone gets its fair share
                assert counts.get(i, 0) >= min(q[i], fair)


def test_queue_sizing(plan):
    out = plan(["need 100 40 64", "need 5 5 1", "grow 100 90", "grow 100 150", "grow 100 500", "bytes 5 1000 10"])
    assert [int(x) for x in out] == [60 + 40 * 64, 5, 100, 200, 500, 1000 * 81 + 10 * 80]
