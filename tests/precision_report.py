#!/usr/bin/env python3
"""Width and soundness report of the precision form (test infrastructure).

For each lemma, on N seeded sampled leaves (synthetic boxes inside the lemma's root box, as in bench.py),
every expression the constraints compare at run time is evaluated
  * in float with outward rounding (the precision form's first pass),
  * in double with outward rounding (the plain form),
  * at 256 bits (tests/mp_judge.py, the "MPFR judge") on the first M of those leaves.
The float and double intervals come from the GPU engine's endpoint dump (sid_eval_operands_device,
--source device) or from the CPU oracle's evaluators (--source oracle); the GPU tests require the two to be
equal bit for bit on these leaves.
Reported per lemma: the mean and maximum interval-width ratio float/double and float/256-bit and
double/256-bit (over expression values with positive finite widths), the number of enclosure violations
(256-bit not inside double, or double not inside float; must be 0) and of contradicted verdicts (a
comparison float or double calls definitely true where the judge calls it definitely false, or the
reverse; must be 0).

    python tests/precision_report.py [--source oracle|device] [--leaves 100000] [--judge 10000] [--jobs 8]
                                     [--out FILE.json]
"""
import argparse
import json
import math
import multiprocessing
import os
import sys
from concurrent.futures import ProcessPoolExecutor

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.join(REPO, "squares-in-disk_gb300", "python"))

SEED = 0x9E3779B9


def _judge_chunk(args):
    ir, lo, hi, ids = args
    import mp_judge
    j = mp_judge.Judge(ir)
    out = []
    for i in range(lo.shape[1]):
        r = j.eval_box(lo[:, i], hi[:, i], ids)
        out.append([r[nid][:3] for nid in ids])
    return out


def lemma_report(name, leaves, judge_leaves, jobs=1, engine=None):
    """engine: a sid_gb300.Engine whose endpoint dump supplies the float and double intervals (else the oracle)."""
    import mp_judge
    import oracle_py
    import sid_gb300 as sid
    ir = sid.lemma_ir(name)
    nargs = sid.ir_nargs(ir)
    root = oracle_py.root_box(ir, nargs)
    lo, hi = sid.synthetic_batch(root, leaves, seed=SEED)
    ops = oracle_py.operand_nodes(ir)
    judge = mp_judge.Judge(ir)
    trivial = {nid for nid in ops if judge.nodes[nid].op in ("arg", "const")}
    # the comparisons (pairs of operand positions) and the unique non-trivial operand expressions
    comps = [(ops[k], ops[k + 1]) for k in range(0, len(ops), 2)]
    cmp_nodes = [n for n in judge.L.nodes if n.op in ("lt", "le", "gt", "ge", "eq", "ne") and n.lb != n.ub]
    uniq = sorted({nid for nid in ops} - trivial)
    pos = {nid: ops.index(nid) for nid in uniq}
    if engine is not None:
        lid = engine.register(ir)
        f32, u32 = engine.eval_operands(lid, lo, hi, True)
        f64, u64 = engine.eval_operands(lid, lo, hi, False)
    else:
        f32, u32 = oracle_py.eval_operands(ir, lo, hi, True)
        f64, u64 = oracle_py.eval_operands(ir, lo, hi, False)

    def widths(a):
        return a[..., 1] - a[..., 0]

    cols = [pos[nid] for nid in uniq]
    w32, w64 = widths(f32[:, cols]), widths(f64[:, cols])
    ok = (u32[:, cols] == 0) & (u64[:, cols] == 0) & np.isfinite(w32) & np.isfinite(w64) & (w64 > 0)
    r3264 = (w32 / np.where(ok, w64, 1.0))[ok]
    enc_64_in_32 = int(np.sum(ok & ((f32[:, cols, 0] > f64[:, cols, 0]) | (f32[:, cols, 1] < f64[:, cols, 1]))))

    # the judge on the first judge_leaves leaves
    m = min(judge_leaves, leaves)
    chunks = max(1, jobs * 4)
    bounds = np.linspace(0, m, chunks + 1).astype(int)
    tasks = [(ir, lo[:, a:b], hi[:, a:b], uniq) for a, b in zip(bounds[:-1], bounds[1:]) if b > a]
    if jobs > 1:
        # spawned workers: a process forked after CUDA was initialised must not run
        with ProcessPoolExecutor(max_workers=jobs, mp_context=multiprocessing.get_context("spawn")) as ex:
            parts = list(ex.map(_judge_chunk, tasks))
    else:
        parts = [_judge_chunk(t) for t in tasks]
    mp = [row for part in parts for row in part]
    mlo = np.array([[v[0] for v in row] for row in mp]) if mp else np.zeros((0, len(uniq)))
    mhi = np.array([[v[1] for v in row] for row in mp]) if mp else np.zeros((0, len(uniq)))
    mu = np.array([[v[2] for v in row] for row in mp], dtype=bool) if mp else np.zeros((0, len(uniq)), bool)
    wmp = mhi - mlo
    okm = ok[:m] & ~mu & np.isfinite(wmp) & (wmp > 0)
    r32mp = (w32[:m] / np.where(okm, wmp, 1.0))[okm]
    r64mp = (w64[:m] / np.where(okm, wmp, 1.0))[okm]
    enc_mp_in_64 = int(np.sum(okm & ((f64[:m, cols, 0] > mlo) | (f64[:m, cols, 1] < mhi))))

    # verdicts of the comparisons: float/double against the judge (definitely true vs definitely false)
    contradictions = 0
    col_of = {nid: k for k, nid in enumerate(uniq)}
    for cn in cmp_nodes:
        a, b = cn.ch
        for i in range(m):
            def iv(arr_lo, arr_hi, nid, src):
                if nid in col_of:
                    return (arr_lo[i, col_of[nid]], arr_hi[i, col_of[nid]])
                k = ops.index(nid) if nid in ops else None
                return (src[i, k, 0], src[i, k, 1]) if k is not None else None
            ja, jb = iv(mlo, mhi, a, f64), iv(mlo, mhi, b, f64)
            if ja is None or jb is None:
                continue
            jd, jp = mp_judge.compare(cn.op, ja, jb)
            for src, und in ((f32, u32), (f64, u64)):
                ka, kb = ops.index(a), ops.index(b)
                if und[i, ka] or und[i, kb]:
                    continue
                d, p = mp_judge.compare(cn.op, tuple(src[i, ka]), tuple(src[i, kb]))
                if (d and not jp) or (not p and jd):
                    contradictions += 1

    def stats(r):
        return {"mean": float(np.mean(r)) if len(r) else None, "max": float(np.max(r)) if len(r) else None,
                "values": int(len(r))}

    return {"lemma": name, "endpoints": "device" if engine is not None else "oracle", "leaves": leaves,
            "judged_leaves": m, "expressions": len(uniq),
            "comparisons": len(cmp_nodes),
            "width_ratio_f32_over_f64": stats(r3264), "width_ratio_f32_over_mp256": stats(r32mp),
            "width_ratio_f64_over_mp256": stats(r64mp),
            "enclosure_violations": enc_64_in_32 + enc_mp_in_64, "contradicted_verdicts": contradictions}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--leaves", type=int, default=100000)
    ap.add_argument("--judge", type=int, default=10000)
    ap.add_argument("--jobs", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--lemmas", nargs="*")
    ap.add_argument("--out")
    ap.add_argument("--source", choices=["oracle", "device"], default="oracle",
                    help="float and double endpoints from the CPU oracle or from the GPU engine's dump")
    args = ap.parse_args()
    import oracle_py
    import sid_gb300 as sid
    oracle_py.build()
    engine = sid.Engine(0) if args.source == "device" else None
    names = args.lemmas or sid.lemma_names()
    rows = []
    for name in names:
        r = lemma_report(name, args.leaves, args.judge, args.jobs, engine=engine)
        rows.append(r)
        print(json.dumps(r), flush=True)
    if args.out:
        with open(args.out, "w") as f:
            json.dump({"seed": SEED, "endpoints": args.source, "rows": rows}, f, indent=1)
    if engine is not None:
        engine.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
