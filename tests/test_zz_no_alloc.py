"""GPU test of the allocation-free entry point sid_leaf_hull_noalloc.

Callers that may not allocate device memory (fixed-budget serving loops, host applications that own
all GPU memory through their own pool) use sid_leaf_hull_noalloc: it evaluates the innermost static
level of the prover core over caller-provided parent cuboids and joins the surviving pieces into one
hull per parent, with its working memory in a fixed array inside the library.

Its results are checked against the existing entry point sid_eval_batch: every parent is split on the
host into its pieces (the parents' last variable has a dyadic range, so the split is exact and equals
the device's rounded-down split), the pieces are evaluated with sid_eval_batch, and the hull of the
surviving pieces is formed on the host with the reference's join rule (minimum of lower bounds, maximum
of upper bounds, the first of equal zero endpoints kept). Bit-exact agreement is required, on two calls
in a row with different lemmas and sizes (the shared working array must be cleared between calls).

This file is collected last so that a run stopping at the first failure has already run every other test.
"""
import numpy as np
import pytest
import torch

import sid_gb300 as sid

pytestmark = pytest.mark.gpu

MAX_CUBOID_VARIABLES = 262136


def _split_spec(ir):
    """(argument, subdivisions) of the lemma's last static split."""
    last = None
    for line in ir.splitlines():
        if line.startswith("split "):
            _, arg, initial, sub, dyn = line.split()
            if dyn == "0":
                last = (int(arg), int(sub))
    return last


def _parents(root, n, rng, last, nsub):
    """Parent cuboids inside the root box; the last split variable's range is a multiple of 2^-20 wide
    enough to be split exactly into nsub pieces."""
    nargs = root.shape[0]
    lo = np.empty((nargs, n))
    hi = np.empty((nargs, n))
    q = 2.0 ** -20
    for v in range(nargs):
        a, b = float(root[v, 0]), float(root[v, 1])
        if v == last:
            m = rng.integers(1, 17, n)
            k0 = int(np.ceil(a / q))
            k1 = int(np.floor(b / q)) - 16 * nsub
            k = rng.integers(k0, max(k0 + 1, k1), n)
            lo[v] = k * q
            hi[v] = lo[v] + m * nsub * q
        else:
            width = rng.uniform(0.0, 1.0, n) ** 3 * (b - a)
            start = rng.uniform(a, b, n)
            lo[v] = start
            hi[v] = np.minimum(start + width, b)
    return lo, hi


def _pieces(lo, hi, last, nsub):
    """Children of every parent on its last split variable, parent-major (exact for dyadic ranges)."""
    nargs, n = lo.shape
    clo = np.repeat(lo, nsub, axis=1)
    chi = np.repeat(hi, nsub, axis=1)
    c = np.tile(np.arange(nsub, dtype=np.float64), n)
    w = np.repeat((hi[last] - lo[last]) / nsub, nsub)
    base = np.repeat(lo[last], nsub)
    clo[last] = base + c * w
    chi[last] = np.where(c + 1 < nsub, base + (c + 1) * w, np.repeat(hi[last], nsub))
    return clo, chi


def _host_hulls(out_lo, out_hi, verdict, n, nsub):
    """Join the surviving pieces of each parent: min of lower bounds, max of upper bounds; for a zero
    endpoint the sign of the first piece (in split order) attaining it."""
    nargs = out_lo.shape[0]
    alive = (verdict == 0).reshape(n, nsub)
    lo = out_lo.reshape(nargs, n, nsub)
    hi = out_hi.reshape(nargs, n, nsub)
    hull_lo = np.where(alive[None], lo, np.inf).min(axis=2)
    hull_hi = np.where(alive[None], hi, -np.inf).max(axis=2)
    for arr, hull in ((lo, hull_lo), (hi, hull_hi)):
        zero = alive[None] & (arr == 0.0)
        first = zero.argmax(axis=2)
        sign = np.take_along_axis(np.signbit(arr), first[..., None], axis=2)[..., 0]
        z = hull == 0.0
        hull[z] = np.where(sign[z], -0.0, 0.0)
    return hull_lo, hull_hi, alive.any(axis=1)


def _run_noalloc(engine, lid, lo, hi):
    nargs, n = lo.shape
    boxes = torch.from_numpy(np.stack([lo, hi], axis=-1).copy()).cuda()           # (nargs, n, 2)
    hulls = torch.full((nargs, n, 2), float("nan"), dtype=torch.float64, device="cuda")
    nonempty = torch.full((n,), 7, dtype=torch.uint8, device="cuda")
    leaves = torch.zeros(1, dtype=torch.int64, device="cuda")
    stream = torch.cuda.current_stream()
    engine.leaf_hull_noalloc(lid, boxes.data_ptr(), n, hulls.data_ptr(), nonempty.data_ptr(), leaves.data_ptr(),
                             stream.cuda_stream)
    torch.cuda.synchronize()
    return hulls.cpu().numpy(), nonempty.cpu().numpy().astype(bool), int(leaves.item())


def _check_lemma(engine, name, n, seed):
    ir = sid.lemma_ir(name)
    nargs = sid.ir_nargs(ir)
    last, nsub = _split_spec(ir)
    lid = engine.register(ir)
    root = engine.root_box(lid, nargs)
    lo, hi = _parents(root, n, np.random.default_rng(seed), last, nsub)
    clo, chi = _pieces(lo, hi, last, nsub)
    out_lo, out_hi, verdict = engine.eval_batch(lid, clo, chi)          # existing entry point
    want_lo, want_hi, want_nonempty = _host_hulls(out_lo, out_hi, verdict, n, nsub)
    hulls, nonempty, leaves = _run_noalloc(engine, lid, lo, hi)
    assert leaves == n * nsub
    assert np.array_equal(nonempty, want_nonempty)
    got_lo = hulls[:, :, 0][:, nonempty]
    got_hi = hulls[:, :, 1][:, nonempty]
    assert np.array_equal(got_lo.view(np.uint64), want_lo[:, nonempty].view(np.uint64))
    assert np.array_equal(got_hi.view(np.uint64), want_hi[:, nonempty].view(np.uint64))
    return int(nonempty.sum())


def test_leaf_hull_noalloc_matches_eval_batch_two_calls(engine):
    # first call: every piece survives (w+x+y+z >= 0 with an integer constant stays undecided)
    kept1 = _check_lemma(engine, "expected_critical2_f64", 3000, seed=11)
    # second call in a row, different lemma and size: pieces are pruned by propagation and constraints
    kept2 = _check_lemma(engine, "pos_neg1_sat", 5000, seed=12)
    assert kept1 == 3000
    assert 0 < kept2 < 5000


def test_leaf_hull_noalloc_rejects_oversized_calls(engine):
    ir = sid.lemma_ir("pos_neg1_sat")
    lid = engine.register(ir)
    nargs = sid.ir_nargs(ir)
    n = MAX_CUBOID_VARIABLES // nargs + 1
    small = torch.zeros(16, dtype=torch.float64, device="cuda")
    flags = torch.zeros(16, dtype=torch.uint8, device="cuda")
    with pytest.raises(sid.SidError) as e:
        engine.leaf_hull_noalloc(lid, small.data_ptr(), n, small.data_ptr(), flags.data_ptr(), 0)
    assert e.value.status == -7
    assert "allocation-free limit" in str(e.value)


def test_leaf_hull_noalloc_empty_call_and_float_lemmas(engine):
    """An empty call writes 0 leaves; float lemmas are rejected (as sid_eval_batch rejects them)."""
    lid = engine.register(sid.lemma_ir("pos_neg1_sat"))
    leaves = torch.full((1,), 12345, dtype=torch.int64, device="cuda")
    engine.leaf_hull_noalloc(lid, 0, 0, 0, 0, leaves.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert int(leaves.item()) == 0
    flid = engine.register(sid.lemma_ir("expected_critical2_f32"))
    small = torch.zeros(16, dtype=torch.float64, device="cuda")
    flags = torch.zeros(16, dtype=torch.uint8, device="cuda")
    with pytest.raises(sid.SidError) as e:
        engine.leaf_hull_noalloc(flid, small.data_ptr(), 1, small.data_ptr(), flags.data_ptr(), 0)
    assert e.value.status == -6
