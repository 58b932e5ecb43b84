"""GPU parity of the criteria's interval endpoints and of the all-double batch kernel.

The constraints of a lemma compare pairs of expressions (F_OC against 0 for the One Subcontainer Lemma, the
side constraints against variables and constants, ...). sid_eval_operands_device dumps every compared
expression's interval on each box: in double (the plain form, the reference's IDouble evaluation) and in float
on the box rounded outward (the precision form's first pass). Both must equal the CPU oracle's evaluation bit
for bit, on the propagated boxes the batch kernel produced (the values the constraints saw), for every lemma,
and on the full 2^24-cuboid One Subcontainer batch of the benchmark. sid_eval_batch_plain_device (the
reference's order, all in double) must give the float-first kernel's outputs bit for bit.

NaN endpoints (e.g. inf - inf) compare equal whatever their payload; everything else compares by bits.
"""
import numpy as np
import pytest

import sid_gb300 as sid

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

SEED = 0x5EED0001
WIDTH_REPORT_SEED = 0x9E3779B9     # tests/precision_report.py's leaves


def same_bits(a, b):
    a = np.array(a, dtype=np.float64, copy=True)
    b = np.array(b, dtype=np.float64, copy=True)
    if a.shape != b.shape:
        return False
    na, nb = np.isnan(a), np.isnan(b)
    if not np.array_equal(na, nb):
        return False
    a[na] = 0.0
    b[nb] = 0.0
    return np.array_equal(a.view(np.uint64), b.view(np.uint64))


def device_batch(engine, lid, lo, hi, plain=False):
    """Propagated boxes and verdicts of one device call (float-first kernel, or the all-double one)."""
    n = lo.shape[1]
    d_lo, d_hi = torch.from_numpy(lo).cuda(), torch.from_numpy(hi).cuda()
    o_lo, o_hi = torch.empty_like(d_lo), torch.empty_like(d_hi)
    o_v = torch.empty(n, dtype=torch.int8, device="cuda")
    fn = engine.eval_batch_plain_device if plain else engine.eval_batch_device
    fn(lid, d_lo.data_ptr(), d_hi.data_ptr(), n, o_lo.data_ptr(), o_hi.data_ptr(), o_v.data_ptr(),
       torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return o_lo.cpu().numpy(), o_hi.cpu().numpy(), o_v.cpu().numpy()


def check_operands(engine, oracle, ir, lid, lo, hi):
    """Device endpoints (double and float) of every compared expression against the oracle's, bit for bit."""
    k = engine.operand_count(lid)
    assert k == len(oracle.operand_nodes(ir))
    for use_float in (False, True):
        g, gu = engine.eval_operands(lid, lo, hi, use_float)
        o, ou = oracle.eval_operands(ir, lo, hi, use_float)
        assert np.array_equal(gu, ou), "undefined flags (float=%s)" % use_float
        assert same_bits(g, o), "endpoints (float=%s)" % use_float
    return k


@pytest.mark.parametrize("name", sid.lemma_names())
def test_criterion_endpoints_bit_exact_on_propagated_boxes(engine, oracle, name):
    ir = sid.lemma_ir(name)
    n = sid.ir_nargs(ir)
    lid = engine.register(ir)
    lo, hi = sid.synthetic_batch(engine.root_box(lid, n), 1 << 15, seed=SEED)
    plo, phi, v = device_batch(engine, lid, lo, hi)
    keep = v != 1                      # boxes that propagation did not empty
    assert keep.sum() > 0
    k = check_operands(engine, oracle, ir, lid, np.ascontiguousarray(plo[:, keep]), np.ascontiguousarray(phi[:, keep]))
    assert k >= 2


@pytest.mark.parametrize("name", sid.lemma_names())
def test_plain_batch_kernel_equals_float_first_kernel_and_oracle(engine, oracle, name):
    ir = sid.lemma_ir(name)
    n = sid.ir_nargs(ir)
    lid = engine.register(ir)
    lo, hi = sid.synthetic_batch(engine.root_box(lid, n), 1 << 15, seed=SEED + 1)
    a = device_batch(engine, lid, lo, hi)
    b = device_batch(engine, lid, lo, hi, plain=True)
    o = oracle.eval_batch(ir, lo, hi)
    for x in (a, b):
        assert np.array_equal(x[2], o[2])
        assert same_bits(x[0], o[0]) and same_bits(x[1], o[1])


@pytest.mark.parametrize("name", ["one_subcontainer", "more_subcontainers_2", "top_packing_2"])
def test_endpoints_on_width_report_leaves(engine, oracle, name):
    """The width and soundness report (tests/precision_report.py) evaluates the compared expressions on its
    seeded raw leaves with the oracle; on those leaves the device's float and double endpoints are the
    oracle's bit for bit, so the report's widths are the device's."""
    ir = sid.lemma_ir(name)
    n = sid.ir_nargs(ir)
    lid = engine.register(ir)
    lo, hi = sid.synthetic_batch(oracle.root_box(ir, n), 100000, seed=WIDTH_REPORT_SEED)
    check_operands(engine, oracle, ir, lid, lo, hi)


def test_bench_batch_2e24_bit_exact(engine, oracle):
    """The benchmark's whole 2^24-cuboid One Subcontainer batch (seed 0x5EED0001): propagated boxes and verdicts
    of both kernels, and the double and float endpoints of every compared expression on the propagated boxes,
    equal the oracle's (compared in chunks of 2^22 cuboids)."""
    ir = sid.lemma_ir("one_subcontainer")
    n = sid.ir_nargs(ir)
    lid = engine.register(ir)
    lo, hi = sid.synthetic_batch(engine.root_box(lid, n), 1 << 24, seed=SEED)
    glo, ghi, gv = device_batch(engine, lid, lo, hi)
    plo, phi, pv = device_batch(engine, lid, lo, hi, plain=True)
    assert np.array_equal(gv, pv) and same_bits(glo, plo) and same_bits(ghi, phi)
    chunk = 1 << 22
    verdicts = np.zeros(3, dtype=np.int64)
    for c0 in range(0, 1 << 24, chunk):
        s = slice(c0, c0 + chunk)
        olo, ohi, ov = oracle.eval_batch(ir, lo[:, s], hi[:, s])
        assert np.array_equal(gv[s], ov)
        assert same_bits(glo[:, s], olo) and same_bits(ghi[:, s], ohi)
        verdicts += np.bincount(ov, minlength=3)[:3]
        keep = ov != 1
        check_operands(engine, oracle, ir, lid, np.ascontiguousarray(glo[:, s][:, keep]),
                       np.ascontiguousarray(ghi[:, s][:, keep]))
    assert verdicts.min() > 0, verdicts


@pytest.mark.parametrize("name", ["top_packing_2", "one_subcontainer", "two_subcontainer", "four_subcontainer"])
def test_large_ragged_batch_equals_the_all_double_kernel(engine, name):
    """A ragged batch just above 2^22 cuboids (a partial last block, deferred cuboids from many blocks) gives the
    all-double kernel's boxes and verdicts bit for bit, for lemmas of 2 to 4 variables."""
    ir = sid.lemma_ir(name)
    n = sid.ir_nargs(ir)
    lid = engine.register(ir)
    lo, hi = sid.synthetic_batch(engine.root_box(lid, n), (1 << 22) + 12345, seed=SEED + 7)
    glo, ghi, gv = device_batch(engine, lid, lo, hi)
    plo, phi, pv = device_batch(engine, lid, lo, hi, plain=True)
    assert np.array_equal(gv, pv) and same_bits(glo, plo) and same_bits(ghi, phi)
    assert len(np.unique(gv)) >= 2           # the batch exercises more than one verdict
