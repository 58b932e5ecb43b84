"""A 256-bit interval evaluation of lemma IR expressions (test infrastructure): the "MPFR judge" of the precision
form. Every operation rounds its lower endpoint down and its upper endpoint up at 256 bits (mpmath's libmp
primitives with floor/ceiling rounding; the arc cosine is computed with 32 guard bits and widened by 2^-256),
so the result encloses the exact range of the expression over the box. It follows the lemma IR's generic
meaning, not the reference's case analysis: products and quotients take the extreme endpoint products,
quotients by intervals containing zero and square roots of negative ranges are marked unbounded, and
if_then_else joins both branches unless its condition is decided. Constants are the IR's double enclosures.

    judge = Judge(ir_text)
    values = judge.eval_box(lo_row, hi_row)   # {node id: (lo, hi, unbounded)} for the operand nodes
"""
import os
import sys

from mpmath import libmp

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "squares-in-disk_gb300", "csrc"))
import codegen  # noqa: E402  (the IR parser of the code generator)

PREC = 256
F, C = libmp.round_floor, libmp.round_ceiling
INF, NINF, ZERO, ONE = libmp.finf, libmp.fninf, libmp.fzero, libmp.fone


def _f(x):
    return libmp.from_float(float(x))


def _lt(a, b):
    return libmp.mpf_lt(a, b)


def _min(a, b):
    return a if libmp.mpf_cmp(a, b) <= 0 else b


def _max(a, b):
    return a if libmp.mpf_cmp(a, b) >= 0 else b


def _finite(x):
    return x not in (INF, NINF) and x != libmp.fnan


class Judge:
    def __init__(self, ir_text):
        import tempfile
        with tempfile.NamedTemporaryFile("w", suffix=".sidir", delete=False) as f:
            f.write(ir_text)
            path = f.name
        try:
            self.L = codegen.Lemma(path)
        finally:
            os.unlink(path)
        self.nodes = {n.id: n for n in self.L.nodes}
        self.consts = [(_f(float.fromhex(c[0])), _f(float.fromhex(c[1]))) for c in self.L.consts]

    # --- interval operations: values are (lo, hi, unbounded) with mpf endpoints
    @staticmethod
    def _mul(a, b):
        if not all(_finite(x) for x in (a[0], a[1], b[0], b[1])):
            return (NINF, INF, True)
        ps_lo = [libmp.mpf_mul(x, y, PREC, F) for x in a[:2] for y in b[:2]]
        ps_hi = [libmp.mpf_mul(x, y, PREC, C) for x in a[:2] for y in b[:2]]
        lo, hi = ps_lo[0], ps_hi[0]
        for p in ps_lo[1:]:
            lo = _min(lo, p)
        for p in ps_hi[1:]:
            hi = _max(hi, p)
        return (lo, hi, a[2] or b[2])

    @staticmethod
    def _div(a, b):
        if not (_lt(ZERO, b[0]) or _lt(b[1], ZERO)):
            return (NINF, INF, True)
        if not all(_finite(x) for x in (a[0], a[1], b[0], b[1])):
            return (NINF, INF, True)
        qs_lo = [libmp.mpf_div(x, y, PREC, F) for x in a[:2] for y in b[:2]]
        qs_hi = [libmp.mpf_div(x, y, PREC, C) for x in a[:2] for y in b[:2]]
        lo, hi = qs_lo[0], qs_hi[0]
        for q in qs_lo[1:]:
            lo = _min(lo, q)
        for q in qs_hi[1:]:
            hi = _max(hi, q)
        return (lo, hi, a[2] or b[2])

    @staticmethod
    def _pow(a, p):
        if p == 0:
            return (ONE, ONE, a[2])
        if not (_finite(a[0]) and _finite(a[1])):
            return (NINF, INF, True)
        lo, hi = a[0], a[1]
        if p % 2 == 1:
            return (libmp.mpf_pow_int(lo, p, PREC, F), libmp.mpf_pow_int(hi, p, PREC, C), a[2])
        if not _lt(lo, ZERO):
            return (libmp.mpf_pow_int(lo, p, PREC, F), libmp.mpf_pow_int(hi, p, PREC, C), a[2])
        if not _lt(ZERO, hi):
            return (libmp.mpf_pow_int(hi, p, PREC, F), libmp.mpf_pow_int(lo, p, PREC, C), a[2])
        m = _max(libmp.mpf_neg(lo), hi)
        return (ZERO, libmp.mpf_pow_int(m, p, PREC, C), a[2])

    @staticmethod
    def _acos_dir(x, up):
        v = libmp.mpf_acos(x, PREC + 32, libmp.round_nearest)
        m = libmp.from_man_exp(1, -PREC)
        return libmp.mpf_add(v, m, PREC, C) if up else libmp.mpf_sub(v, m, PREC, F)

    def _pred(self, nid, cache):
        n = self.nodes[nid]
        if n.lb == n.ub:
            return (n.lb != 0, n.ub != 0)
        op = n.op
        if op in ("lt", "le", "gt", "ge", "eq", "ne"):
            a, b = self._val(n.ch[0], cache), self._val(n.ch[1], cache)
            return compare(op, a, b)
        if op in ("orseq", "or"):
            vals = [self._pred(c, cache) for c in n.ch]
            return (any(v[0] for v in vals), any(v[1] for v in vals))
        if op in ("andseq", "and"):
            vals = [self._pred(c, cache) for c in n.ch]
            return (all(v[0] for v in vals), all(v[1] for v in vals))
        if op == "not":
            v = self._pred(n.ch[0], cache)
            return (not v[1], not v[0])
        if op == "bconst":
            return (n.aux != 0, n.aux != 0)
        raise ValueError(op)

    def _val(self, nid, cache):
        if nid in cache:
            return cache[nid]
        n = self.nodes[nid]
        op = n.op
        ch = [self._val(c, cache) for c in n.ch] if op not in ("ite",) else None
        if op == "arg":
            r = cache[("arg", n.aux)]
        elif op == "const":
            lo, hi = self.consts[n.aux]
            r = (lo, hi, False)
        elif op == "neg":
            r = (libmp.mpf_neg(ch[0][1]), libmp.mpf_neg(ch[0][0]), ch[0][2])
        elif op == "add":
            r = (libmp.mpf_add(ch[0][0], ch[1][0], PREC, F), libmp.mpf_add(ch[0][1], ch[1][1], PREC, C),
                 ch[0][2] or ch[1][2])
        elif op == "sub":
            r = (libmp.mpf_sub(ch[0][0], ch[1][1], PREC, F), libmp.mpf_sub(ch[0][1], ch[1][0], PREC, C),
                 ch[0][2] or ch[1][2])
        elif op == "mul":
            r = self._mul(ch[0], ch[1])
        elif op == "div":
            r = self._div(ch[0], ch[1])
        elif op == "sqrt":
            lo, hi, u = ch[0]
            if _lt(hi, ZERO) or not _finite(hi):
                r = (NINF, INF, True)
            else:
                if _lt(lo, ZERO):
                    lo, u = ZERO, True
                r = (libmp.mpf_sqrt(lo, PREC, F), libmp.mpf_sqrt(hi, PREC, C), u)
        elif op == "pow":
            r = self._pow(ch[0], n.aux)
        elif op == "acos":
            lo, hi, u = ch[0]
            if _lt(hi, libmp.mpf_neg(ONE)) or _lt(ONE, lo) or not (_finite(lo) and _finite(hi)):
                r = (NINF, INF, True)
            else:
                if _lt(lo, libmp.mpf_neg(ONE)):
                    lo, u = libmp.mpf_neg(ONE), True
                if _lt(ONE, hi):
                    hi, u = ONE, True
                r = (self._acos_dir(hi, False), self._acos_dir(lo, True), u)
        elif op in ("min", "max"):
            acc = ch[-1]
            for a in reversed(ch[:-1]):
                if op == "min":
                    acc = (_min(a[0], acc[0]), _min(a[1], acc[1]), a[2] or acc[2])
                else:
                    acc = (_max(a[0], acc[0]), _max(a[1], acc[1]), a[2] or acc[2])
            r = acc
        elif op == "ite":
            c = self._pred(n.ch[0], cache)
            if c[0]:
                r = self._val(n.ch[1], cache)
            elif not c[1]:
                r = self._val(n.ch[2], cache)
            else:
                t, e = self._val(n.ch[1], cache), self._val(n.ch[2], cache)
                r = (_min(t[0], e[0]), _max(t[1], e[1]), t[2] or e[2])
        else:
            raise ValueError("judge: unsupported operation %s" % op)
        cache[nid] = r
        return r

    def eval_box(self, lo_row, hi_row, node_ids):
        """Intervals of the given nodes on the box (lo_row[v], hi_row[v]) as (lo, hi, unbounded) floats
        rounded outward from the 256-bit endpoints (lo down, hi up to the next double)."""
        cache = {("arg", v): (_f(lo_row[v]), _f(hi_row[v]), False) for v in range(self.L.nargs)}
        out = {}
        for nid in node_ids:
            lo, hi, u = self._val(nid, cache)
            out[nid] = (libmp.to_float(lo, rnd=F), libmp.to_float(hi, rnd=C), u, lo, hi)
        return out


def compare(op, a, b):
    """(definitely, possibly) of a op b for intervals a, b with comparable endpoints (mpf or float)."""
    def lt(x, y):
        return libmp.mpf_lt(x, y) if isinstance(x, tuple) else x < y
    def less(p, q):
        return (lt(p[1], q[0]), lt(p[0], q[1]))
    if op == "lt":
        return less(a, b)
    if op == "gt":
        return less(b, a)
    if op == "le":
        d, p = less(b, a)
        return (not p, not d)
    if op == "ge":
        d, p = less(a, b)
        return (not p, not d)
    ov = not lt(a[1], b[0]) and not lt(b[1], a[0])
    eq = (a[0] == a[1] and b[0] == b[1] and a[0] == b[0], ov)
    return eq if op == "eq" else (not eq[1], not eq[0])
