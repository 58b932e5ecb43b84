#!/usr/bin/env python3
"""Write tests/golden/ops_per_cuboid.json: IEEE directed-rounding operations (additions/subtractions,
multiplications, divisions, square roots, arc cosines) per cuboid, counted by the op-counting build of the
CPU oracle (oracle/_build/liboracle_ops.so, -DSIDO_COUNT_OPS):
  * "batch": leaf evaluation (propagation after a change of the last variable, all constraints) of a
    seeded sample of bench.py's synthetic batch, per lemma, in the device's order (each row's constraints
    cheapest first, as the code generator emits them): double operations with
    the constraints tested in float first and in double only where float does not refute them ("batch_f32":
    the float operations of that order; "batch_plain": double operations of the all-double order);
  * "proof": whole plain proofs of the lemmas the oracle proves in seconds, per cuboid considered.
bench.py turns the One Subcontainer batch figure into an FP64 operation rate for its roofline line.

  python tests/golden/make_ops_table.py
"""
import ctypes
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.join(REPO, "squares-in-disk_gb300", "python"))

SAMPLE = 1 << 16
SEED = 0x5EED0001          # bench.py's batch seed
KINDS = ["add_sub", "mul", "div", "sqrt", "acos"]
PROOF_LEMMAS = ["top_packing_1", "top_packing_2", "one_subcontainer", "two_subcontainer", "three_subcontainer",
                "five_subcontainer", "six_subcontainer", "seven_subcontainer"]


def main():
    import oracle_py
    import sid_gb300 as sid
    oracle_py.build()
    L = ctypes.CDLL(os.path.join(REPO, "oracle", "_build", "liboracle_ops.so"))
    L.sido_set_device_row_order(1)       # count the engine's operations: its constraint order within each row
    counts = (ctypes.c_ulonglong * 10)()

    def take(which="f64"):
        if L.sido_count_ops(counts) != 0:
            raise RuntimeError("op counting failed")
        c = [int(x) for x in counts]
        return c[:5] if which == "f64" else c[5:]

    take()
    out = {"sample": SAMPLE, "seed": SEED, "kinds": KINDS, "batch": {}, "batch_f32": {}, "batch_plain": {},
           "proof": {}}
    for name in sid.lemma_names():
        ir = sid.lemma_ir(name)
        nargs = sid.ir_nargs(ir)
        if sid.ir_uses(ir, "acos") is None:
            continue
        root = oracle_py.root_box(ir, nargs)
        lo, hi = sid.synthetic_batch(root, SAMPLE, seed=SEED)
        lo = np.ascontiguousarray(lo)
        hi = np.ascontiguousarray(hi)
        olo, ohi = np.empty_like(lo), np.empty_like(hi)
        vd = np.empty(SAMPLE, dtype=np.int8)
        for float_first, key in ((0, "batch_plain"), (1, "batch")):
            rc = L.sido_eval_batch(ir.encode(), ctypes.c_void_p(lo.ctypes.data), ctypes.c_void_p(hi.ctypes.data),
                                   ctypes.c_ulonglong(SAMPLE), ctypes.c_void_p(olo.ctypes.data),
                                   ctypes.c_void_p(ohi.ctypes.data), ctypes.c_void_p(vd.ctypes.data), ctypes.c_int(8),
                                   ctypes.c_int(float_first))
            if rc != 0:
                raise RuntimeError("batch evaluation failed for " + name)
            c = [int(x) for x in counts] if L.sido_count_ops(counts) == 0 else None
            if c is None:
                raise RuntimeError("op counting failed")
            out[key][name] = dict(zip(KINDS, [x / SAMPLE for x in c[:5]]), total=sum(c[:5]) / SAMPLE)
            if float_first:
                out["batch_f32"][name] = dict(zip(KINDS, [x / SAMPLE for x in c[5:]]), total=sum(c[5:]) / SAMPLE)
    for name in PROOF_LEMMAS:
        r = oracle_py.prove(sid.lemma_ir(name))   # the normal library: warm-up only
        take()
        L.sido_prove.argtypes = None
        cnt = (ctypes.c_ulonglong * 6)()
        secs = ctypes.c_double()
        rc = L.sido_prove(sid.lemma_ir(name).encode(), ctypes.c_uint(8), ctypes.c_int(1), ctypes.c_float(0.25),
                          ctypes.c_float(0.66), ctypes.c_int(8), ctypes.c_int(0), ctypes.c_uint(0xFFFFFFFF),
                          ctypes.c_uint(0), ctypes.c_uint(0), ctypes.c_uint(0), cnt,
                          ctypes.byref(secs), None, ctypes.c_ulonglong(0), None)
        if rc != 0:
            raise RuntimeError("proof failed for " + name)
        c = take()
        assert cnt[0] == r["cuboids"]
        out["proof"][name] = dict(zip(KINDS, [x / cnt[0] for x in c]), total=sum(c) / cnt[0], cuboids=int(cnt[0]))
    path = os.path.join(HERE, "ops_per_cuboid.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print(path)


if __name__ == "__main__":
    main()
