"""CPU ORACLE -- test infrastructure only: ctypes binding of oracle/_build/liboracle.so.

Used by tests/ and by the CPU-baseline leg of bench.py; never by the product.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE, "-j4"], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        _lib = ctypes.CDLL(LIB)
        _lib.sido_prove.restype = ctypes.c_int
        _lib.sido_prove.argtypes = [ctypes.c_char_p, ctypes.c_uint, ctypes.c_int, ctypes.c_float, ctypes.c_float,
                                    ctypes.c_int, ctypes.c_int, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint,
                                    ctypes.c_uint, ctypes.POINTER(ctypes.c_ulonglong),
                                    ctypes.POINTER(ctypes.c_double),
                                    ctypes.c_void_p, ctypes.c_ulonglong, ctypes.POINTER(ctypes.c_ulonglong)]
        _lib.sido_root_box.restype = ctypes.c_int
        _lib.sido_root_box.argtypes = [ctypes.c_char_p, ctypes.c_void_p]
        _lib.sido_eval_batch.restype = ctypes.c_int
        _lib.sido_eval_batch.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_ulonglong,
                                         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        _lib.sido_last_error.restype = ctypes.c_char_p
        _lib.sido_acos_rounded.argtypes = [ctypes.c_void_p, ctypes.c_ulonglong, ctypes.c_int, ctypes.c_void_p]
        _lib.sido_acos_rounded_f32.argtypes = [ctypes.c_void_p, ctypes.c_ulonglong, ctypes.c_int, ctypes.c_void_p]
        _lib.sido_acos_bound_f32.argtypes = [ctypes.c_void_p, ctypes.c_ulonglong, ctypes.c_int, ctypes.c_void_p]
        _lib.sido_operand_nodes.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int]
        _lib.sido_eval_operands.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_ulonglong,
                                            ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        _lib.sido_acos_rounded_f32.argtypes = [ctypes.c_void_p, ctypes.c_ulonglong, ctypes.c_int, ctypes.c_void_p]
    return _lib


def _err():
    return lib().sido_last_error().decode()


def prove(ir_text, generations=8, max_iterations=1, threads=0, max_criticals=0, nargs=None, fp32_first=False,
          fp32_level_mask=0xFFFFFFFF, fp32_noprop_mask=0xFFFFFFFF, part=None):
    """Run the oracle proof; returns dict(cuboids, leaves, criticals, repeated, fp32_refuted, escalated, seconds,
    boxes). fp32_first selects the precision form (float first, double for what float cannot refute);
    fp32_noprop_mask its levels whose float pass skips bound propagation; part = (index, count) proves one
    shard of the root partition's first split."""
    L = lib()
    counts = (ctypes.c_ulonglong * 6)()
    secs = ctypes.c_double()
    n_pairs = ctypes.c_ulonglong(0)
    buf = None
    if max_criticals:
        if nargs is None:
            nargs = int([l for l in ir_text.splitlines() if l.startswith("nargs ")][0].split()[1])
        buf = np.zeros(max_criticals * 2 * nargs, dtype=np.float64)
    rc = L.sido_prove(ir_text.encode(), generations, max_iterations, 0.25, 0.66, threads, 1 if fp32_first else 0,
                      fp32_level_mask, fp32_noprop_mask, part[0] if part else 0, part[1] if part else 0, counts,
                      ctypes.byref(secs),
                      buf.ctypes.data if buf is not None else None, max_criticals, ctypes.byref(n_pairs))
    if rc != 0:
        raise RuntimeError("oracle: " + _err())
    out = dict(cuboids=counts[0], leaves=counts[1], criticals=counts[2], repeated=counts[3], fp32_refuted=counts[4],
               escalated=counts[5], seconds=secs.value)
    if buf is not None:
        out["boxes"] = buf[: n_pairs.value * 2].reshape(-1, nargs, 2)
    return out


def root_box(ir_text, nargs):
    out = np.zeros(2 * nargs, dtype=np.float64)
    if lib().sido_root_box(ir_text.encode(), out.ctypes.data) != 0:
        raise RuntimeError("oracle: " + _err())
    return out.reshape(nargs, 2)


def eval_batch(ir_text, lo, hi, threads=0, float_rows_first=False):
    """lo, hi: float64 arrays of shape (nargs, n). Returns (out_lo, out_hi, verdict). float_rows_first: the
    device's order (constraints in float first, in double where float does not refute); same results."""
    lo = np.ascontiguousarray(lo, dtype=np.float64)
    hi = np.ascontiguousarray(hi, dtype=np.float64)
    n = lo.shape[1]
    out_lo = np.empty_like(lo)
    out_hi = np.empty_like(hi)
    verdict = np.empty(n, dtype=np.int8)
    rc = lib().sido_eval_batch(ir_text.encode(), lo.ctypes.data, hi.ctypes.data, n, out_lo.ctypes.data,
                               out_hi.ctypes.data, verdict.ctypes.data, threads, 1 if float_rows_first else 0)
    if rc != 0:
        raise RuntimeError("oracle: " + _err())
    return out_lo, out_hi, verdict


def acos_rounded(x, up, dtype=np.float64):
    """acos of every element of x rounded down (up=False) or up (up=True) to dtype (float64 or float32)."""
    x = np.ascontiguousarray(x, dtype=dtype)
    out = np.empty_like(x)
    fn = lib().sido_acos_rounded if dtype == np.float64 else lib().sido_acos_rounded_f32
    if fn(x.ctypes.data, x.size, 1 if up else 0, out.ctypes.data) != 0:
        raise RuntimeError(_err())
    return out


def acos_bound_f32(x, up):
    """The precision form's float arc cosine bound (lower for up=False, upper for up=True) of every element."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    out = np.empty_like(x)
    if lib().sido_acos_bound_f32(x.ctypes.data, x.size, 1 if up else 0, out.ctypes.data) != 0:
        raise RuntimeError(_err())
    return out


def device_row_order(ir_text, row):
    """Constraint ids of a row in the engine's evaluation order (cheapest not yet evaluated constraint first)."""
    L = lib()
    L.sido_device_row_order.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int]
    out = np.zeros(1024, dtype=np.int32)
    k = L.sido_device_row_order(ir_text.encode(), row, out.ctypes.data, len(out))
    if k < 0:
        raise RuntimeError(_err())
    return [int(x) for x in out[:k]]


def operand_nodes(ir_text):
    """Node ids of the expressions the constraints compare at run time (left, right per comparison)."""
    ids = np.zeros(4096, dtype=np.int32)
    k = lib().sido_operand_nodes(ir_text.encode(), ids.ctypes.data, len(ids))
    if k < 0:
        raise RuntimeError(_err())
    return [int(x) for x in ids[:k]]


def eval_operands(ir_text, lo, hi, use_float, threads=0):
    """Intervals of those expressions on raw boxes (SoA lo/hi, shape (nargs, n)), in float or double:
    returns (lohi array (n, k, 2), undefined flags (n, k))."""
    lo = np.ascontiguousarray(lo, dtype=np.float64)
    hi = np.ascontiguousarray(hi, dtype=np.float64)
    n = lo.shape[1]
    k = len(operand_nodes(ir_text))
    out = np.empty((n, k, 2), dtype=np.float64)
    und = np.empty((n, k), dtype=np.int8)
    if lib().sido_eval_operands(ir_text.encode(), lo.ctypes.data, hi.ctypes.data, n, 1 if use_float else 0,
                                out.ctypes.data, und.ctypes.data, threads) != 0:
        raise RuntimeError(_err())
    return out, und
