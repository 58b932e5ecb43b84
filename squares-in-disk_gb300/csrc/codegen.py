#!/usr/bin/env python3
"""Generate CUDA device code for compiled lemmas.

For every lemma IR file (written by the front end, include/ivarp/sid_fe/compile.hpp) this emits one
.cu translation unit with a lemma type `L` providing, for the frontier kernels of engine.cuh:

  * apply_bound<T>(k, box): evaluate bound function k on the box and apply it to its target
    variable (straight-line interval code, common subexpressions shared, if_then_else branches
    evaluated only when needed, like the reference's if_then_else evaluation);
  * rows_status<T>(r0, r1, box): 0 if a constraint of rows [r0, r1) cannot hold, 2 if all hold
    definitely, else 1; rows_ok<T> is status != 0 (stops at the first
    violated constraint, like CPUProverCore::p_cuboid_violates_constraint_row);
  * the update lists as 64-bit masks, the targets and the compile-time variable bounds;
  * for double lemmas, per level that tests rows, the split-invariant form of the precision form's float
    pass (H<level>): prelude() evaluates once per parent every row subexpression that does not depend on
    the level's split variable and stores the ones the other subexpressions consume; child() evaluates
    the rest per child from those values.

Interval operations whose case analysis depends on compile-time bounds get those decisions as
template arguments (see interval.cuh). The code is generic in the number type T so the same lemma
can run in double (the reference's IDouble) and float.

  python codegen.py --out DIR lemma1.sidir lemma2.sidir ...
"""
import argparse
import os
import re
import sys

FXMAX = 9223372036854775807
FXMIN = -FXMAX
FX_ONE = 1000000

OPS = ["arg", "const", "bconst", "neg", "add", "sub", "mul", "div", "sqrt", "pow", "acos", "asin", "min",
       "max", "ite", "lt", "le", "gt", "ge", "eq", "ne", "orseq", "andseq", "or", "and", "not"]
PRED_OPS = {"bconst", "lt", "le", "gt", "ge", "eq", "ne", "orseq", "andseq", "or", "and", "not"}


class Node:
    __slots__ = ("id", "op", "lb", "ub", "aux", "ch")

    def __init__(self, nid, op, lb, ub, aux, ch):
        self.id, self.op, self.lb, self.ub, self.aux, self.ch = nid, op, lb, ub, aux, ch


class Lemma:
    def __init__(self, path):
        self.path = path
        self.slug = os.path.splitext(os.path.basename(path))[0]
        self.consts, self.nodes, self.bounds, self.constraints = [], [], [], []
        self.upd = {}
        self.rows = {}
        self.ct = {}
        self.splits = []
        text = open(path).read()
        self.text = text
        for line in text.splitlines():
            t = line.split()
            if not t:
                continue
            kw = t[0]
            if kw == "numtype":
                self.numtype = t[1]
            elif kw == "nargs":
                self.nargs = int(t[1])
            elif kw == "arg":
                self.ct[int(t[1])] = (int(t[3]), int(t[4]))
            elif kw == "split":
                self.splits.append(tuple(int(x) for x in t[1:]))
            elif kw == "const":
                self.consts.append((t[2], t[3], t[4], t[5], int(t[6])))
            elif kw == "node":
                nc = int(t[6])
                self.nodes.append(Node(int(t[1]), t[2], int(t[3]), int(t[4]), int(t[5]), [int(x) for x in t[7:7 + nc]]))
            elif kw == "bound":
                self.bounds.append((int(t[2]), {"leq": 1, "geq": 2, "both": 3}[t[3]], int(t[4]), int(t[5])))
            elif kw == "update":
                self.upd[(int(t[1]), t[2])] = [int(x) for x in t[4:]]
            elif kw == "constraint":
                self.constraints.append(int(t[2]))
            elif kw == "row":
                self.rows[int(t[1])] = [int(x) for x in t[3:]]
        self.fingerprint = fingerprint(text)
        if len(self.bounds) > 64:
            raise ValueError("%s: more than 64 bounds are not supported" % path)

    def uses(self, op):
        return any(n.op == op for n in self.nodes)


BUNDLE_MAX = 4   # lemmas per bundle (kBundleMax of proof_loop.cuh)


def fingerprint(text):
    """FNV-1a over the IR lines except the name line (same as lemma_ir.hpp)."""
    h = 1469598103934665603
    for line in text.split("\n")[:-1] if text.endswith("\n") else text.split("\n"):
        if line.startswith("name "):
            continue
        for c in line.encode():
            h ^= c
            h = (h * 1099511628211) & 0xFFFFFFFFFFFFFFFF
        h ^= 10
        h = (h * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return h


CMP_OPS = {"lt", "le", "gt", "ge", "eq", "ne"}


def cheap_constraint(L, nid):
    """A constraint that only compares variables and constants (no arithmetic), or a constant one."""
    n = L.nodes[nid]
    if n.lb == n.ub:
        return True
    return n.op in CMP_OPS and all(L.nodes[c].op in ("arg", "const") for c in n.ch)


SLOW_OPS = {"sqrt", "div", "acos"}


def slow_bound(L, fn):
    """A bound function with a square root, a division or an arc cosine, or with 4 or more operations: the
    batch kernel defers the cuboids whose propagation reaches one (they are evaluated afterwards on full
    warps), so that the few lanes needing it do not hold up their warps."""
    seen, ops = set(), []

    def walk(nid):
        if nid in seen:
            return
        seen.add(nid)
        n = L.nodes[nid]
        if n.op not in ("arg", "const", "bconst"):
            ops.append(n.op)
        for c in n.ch:
            walk(c)

    walk(fn)
    return any(o in SLOW_OPS for o in ops) or len(ops) >= 4


def comparison_operands(L):
    """The expressions compared by the constraints' comparison nodes that are not decided at compile time, in
    the oracle's order (oracle/oracle.cpp, comparison_operands): constraints in table order, each predicate tree
    in pre-order, (left, right) per comparison, every comparison node once."""
    out, seen = [], set()
    for root in L.constraints:
        stack = [root]
        while stack:
            nid = stack.pop()
            if nid in seen:
                continue
            seen.add(nid)
            n = L.nodes[nid]
            if n.lb == n.ub:
                continue
            if n.op in CMP_OPS:
                out += [n.ch[0], n.ch[1]]
            elif n.op in ("orseq", "andseq", "or", "and", "not"):
                stack.extend(reversed(n.ch))
    return out


# weights of the operations in the evaluation order below (directed-rounding square roots and quotients take
# several instructions; arc cosines many)
OP_WEIGHT = {"sqrt": 12, "div": 12, "acos": 40, "mul": 2, "pow": 3}


def op_weight(n):
    return 0 if n.op in ("arg", "const", "bconst") else OP_WEIGHT.get(n.op, 1)


def row_order(L, r):
    """The constraints of row r in evaluation order: repeatedly the one whose not yet evaluated nodes weigh least
    (ties: table order). A row holds iff all its constraints hold, so the order changes no verdict; testing cheap
    constraints first lets the first refuted one stop the row early at lower cost."""
    cons = list(L.rows.get(r, []))
    nodes = {}
    for ci in cons:
        acc, stack = set(), [L.constraints[ci]]
        while stack:
            nid = stack.pop()
            if nid not in acc:
                acc.add(nid)
                stack.extend(L.nodes[nid].ch)
        nodes[ci] = acc
    done, order = set(), []
    while cons:
        ci = min(cons, key=lambda c: (sum(op_weight(L.nodes[x]) for x in nodes[c] - done), cons.index(c)))
        order.append(ci)
        cons.remove(ci)
        done |= nodes[ci]
    return order


def tri_nn(n):
    return 1 if n.lb >= 0 else (0 if n.ub <= 0 else -1)


def tri_np(n):
    return 1 if n.ub <= 0 else (0 if n.lb >= 0 else -1)


def tri_pos(n):
    return 1 if n.lb > 0 else (0 if n.ub <= 0 else -1)


def tri_neg(n):
    return 1 if n.ub < 0 else (0 if n.lb >= 0 else -1)


def finite(n):
    return n.lb > FXMIN and n.ub < FXMAX


def float_literal(hexstr):
    # "%a" output of a float value printed as double; append the f suffix after an exponent
    return hexstr + "f" if "p" in hexstr else hexstr + ".0f"


class Emitter:
    def __init__(self, lemma):
        self.L = lemma
        self.lines = []
        self.counter = 0
        self.indent = 1

    def fresh(self, prefix):
        self.counter += 1
        return "%s%d" % (prefix, self.counter)

    def emit(self, s):
        self.lines.append("    " * self.indent + s)

    def expr(self, nid, scope):
        if nid in scope:
            return scope[nid]
        n = self.L.nodes[nid]
        op = n.op
        if op in PRED_OPS:
            raise ValueError("predicate node %d used as expression" % nid)
        if op == "arg":
            name = "box[%d]" % n.aux
            scope[nid] = name
            return name
        name = self.fresh("v")
        if op == "const":
            dlo, dhi, flo, fhi, und = self.L.consts[n.aux]
            self.emit("const Iv<T> %s = cst<T>(%s, %s, %s, %s, %s);" % (
                name, dlo, dhi, float_literal(flo), float_literal(fhi), "true" if und else "false"))
        elif op == "ite":
            c = self.pred(n.ch[0], scope)
            t_name, e_name = self.fresh("t"), self.fresh("e")
            self.emit("Iv<T> %s{T(0), T(0), false}, %s{T(0), T(0), false};" % (t_name, e_name))
            self.emit("if(%s.ub) {" % c)
            self.indent += 1
            inner = dict(scope)
            self.emit("%s = %s;" % (t_name, self.expr(n.ch[1], inner)))
            self.indent -= 1
            self.emit("}")
            self.emit("if(!%s.lb) {" % c)
            self.indent += 1
            inner = dict(scope)
            self.emit("%s = %s;" % (e_name, self.expr(n.ch[2], inner)))
            self.indent -= 1
            self.emit("}")
            self.emit("const Iv<T> %s = %s.lb ? %s : (!%s.ub ? %s : iv_join(%s, %s));" % (
                name, c, t_name, c, e_name, t_name, e_name))
        else:
            ch = [self.expr(c, scope) for c in n.ch]
            cn = [self.L.nodes[c] for c in n.ch]
            if op == "neg":
                rhs = "iv_neg(%s)" % ch[0]
            elif op == "add":
                rhs = "iv_add(%s, %s)" % (ch[0], ch[1])
            elif op == "sub":
                rhs = "iv_sub(%s, %s)" % (ch[0], ch[1])
            elif op == "mul":
                rhs = "iv_mul<T, %d, %d, %d, %d, %s>(%s, %s)" % (
                    tri_nn(cn[0]), tri_np(cn[0]), tri_nn(cn[1]), tri_np(cn[1]),
                    "true" if finite(cn[0]) and finite(cn[1]) else "false", ch[0], ch[1])
            elif op == "div":
                rhs = "iv_div<T, %d, %d, %d, %d, %s>(%s, %s)" % (
                    tri_nn(cn[0]), tri_np(cn[0]), tri_pos(cn[1]), tri_neg(cn[1]),
                    "true" if finite(cn[0]) and finite(cn[1]) else "false", ch[0], ch[1])
            elif op == "sqrt":
                rhs = "iv_sqrt<T, %d>(%s)" % (tri_nn(cn[0]), ch[0])
            elif op == "pow":
                rhs = "iv_pow<T, %du>(%s)" % (n.aux, ch[0])
            elif op in ("min", "max"):
                acc = ch[-1]
                for x in reversed(ch[:-1]):
                    acc = "iv_%s(%s, %s)" % (op, x, acc)
                rhs = acc
            elif op == "acos":
                rhs = "%s<T, %s, %s>(%s)" % ("iv_acos" if self.L.numtype == "f32" else "iv_acos_f64",
                                             "true" if cn[0].lb < -FX_ONE else "false",
                                                  "true" if cn[0].ub > FX_ONE else "false", ch[0])
            else:
                raise ValueError("unsupported expression operation %s" % op)
            self.emit("const Iv<T> %s = %s;" % (name, rhs))
        scope[nid] = name
        return name

    def pred(self, nid, scope):
        if nid in scope:
            return scope[nid]
        n = self.L.nodes[nid]
        op = n.op
        if op not in PRED_OPS:
            raise ValueError("expression node %d used as predicate" % nid)
        name = self.fresh("p")
        if n.lb == n.ub:
            v = "true" if n.lb else "false"
            self.emit("const IB %s{%s, %s};" % (name, v, v))
        elif op in ("lt", "le", "gt", "ge", "eq", "ne"):
            a = self.expr(n.ch[0], scope)
            b = self.expr(n.ch[1], scope)
            self.emit("const IB %s = iv_%s(%s, %s);" % (name, op, a, b))
        elif op in ("orseq", "andseq"):
            is_or = op == "orseq"
            self.emit("IB %s{%s, %s};" % (name, "false" if is_or else "true", "false" if is_or else "true"))
            opened = 0
            for i, c in enumerate(n.ch):
                sub = scope if i == 0 else dict(scope)
                if i > 0:
                    self.emit("if(%s%s) {" % ("!" if is_or else "", name + (".lb" if is_or else ".ub")))
                    self.indent += 1
                    opened += 1
                x = self.pred(c, sub)
                if is_or:
                    self.emit("%s.lb = %s.lb || %s.lb; %s.ub = %s.ub || %s.ub;" % (name, name, x, name, name, x))
                else:
                    self.emit("%s.lb = %s.lb && %s.lb; %s.ub = %s.ub && %s.ub;" % (name, name, x, name, name, x))
            for _ in range(opened):
                self.indent -= 1
                self.emit("}")
            if is_or:
                self.emit("if(%s.lb) %s.ub = true;" % (name, name))
            else:
                self.emit("if(!%s.ub) %s.lb = false;" % (name, name))
        elif op in ("or", "and"):
            xs = [self.pred(c, scope) for c in n.ch]
            j = " || " if op == "or" else " && "
            self.emit("const IB %s{%s, %s};" % (name, j.join(x + ".lb" for x in xs), j.join(x + ".ub" for x in xs)))
        elif op == "not":
            x = self.pred(n.ch[0], scope)
            self.emit("const IB %s = ib_not(%s);" % (name, x))
        elif op == "bconst":
            self.emit("const IB %s{%s, %s};" % (name, "true" if n.lb else "false", "true" if n.ub else "false"))
        else:
            raise ValueError("unsupported predicate operation %s" % op)
        scope[nid] = name
        return name


def levels_with_rows(L):
    """(level id, split variable, r0, r1) of the levels that test constraint rows [r0, r1): the last dynamic
    level tests the last row, static level j the rows from its variable up to the next static variable.
    Level ids: dynamic levels 0..D-1, then static levels D + j."""
    dyn = [s for s in L.splits if s[3]]
    stat = [s for s in L.splits if not s[3]]
    out = []
    if dyn:
        out.append((len(dyn) - 1, dyn[-1][0], L.nargs - 1, L.nargs))
    for j, sp in enumerate(stat):
        r1 = stat[j + 1][0] if j + 1 < len(stat) else L.nargs
        if r1 > sp[0]:
            out.append((len(dyn) + j, sp[0], sp[0], r1))
    return out


HOIST_BITS = 63   # flag bits per parent (bit 63 marks a parent whose split-invariant constraints already fail)


def hoist_plan(L, var, r0, r1):
    """Split the rows [r0, r1) for a split of `var`: constraints independent of var (tested once per parent),
    constraints that depend on it (tested per child), and the frontier: nodes independent of var that
    var-dependent nodes consume (stored per parent). None if the frontier's flags do not fit the flag word."""
    memo = {}

    def deps(nid):
        if nid not in memo:
            n = L.nodes[nid]
            d = {n.aux} if n.op == "arg" else set()
            for c in n.ch:
                d |= deps(c)
            memo[nid] = frozenset(d)
        return memo[nid]

    top = [L.constraints[ci] for r in range(r0, r1) for ci in row_order(L, r)]
    if not top:
        return None
    inv_top = [p for p in top if var not in deps(p)]
    dep_top = [p for p in top if var in deps(p)]
    frontier, seen, fset = [], set(), set()

    def walk(x):
        if x in seen:
            return
        seen.add(x)
        for c in L.nodes[x].ch:
            cn = L.nodes[c]
            if var in deps(c):
                walk(c)
            elif cn.op in ("arg", "const", "bconst") or (cn.op in PRED_OPS and cn.lb == cn.ub):
                continue
            elif c not in fset:
                fset.add(c)
                frontier.append(c)

    for p in dep_top:
        walk(p)
    bits = sum(2 if L.nodes[f].op in PRED_OPS else 1 for f in frontier)
    if bits > HOIST_BITS:
        return None
    return inv_top, dep_top, frontier


def emit_hoisted(L, level, var, plan, w):
    """H<level>: prelude (once per parent: split-invariant constraints, stored frontier values and flags) and
    child (per child: the constraints that depend on the split variable)."""
    inv_top, dep_top, frontier = plan
    slots, bit = {}, 0
    nval = 0
    for f in frontier:
        if L.nodes[f].op in PRED_OPS:
            slots[f] = ("p", bit)
            bit += 2
        else:
            slots[f] = ("v", nval, bit)
            nval += 1
            bit += 1
    w("template<> struct H<%d> {" % level)
    w("    static constexpr int VAR = %d;" % var)
    w("    static constexpr int NVAL = %d;" % nval)
    w("    __device__ static bool prelude(const Iv<float>* box, float2* hv, std::uint64_t stride, std::uint64_t j,")
    w("                                   std::uint64_t& bits) {")
    w("        using T = float;")
    w("        std::uint64_t b = 0;")
    e = Emitter(L)
    e.indent = 2
    scope = {}
    for p in inv_top:
        x = e.pred(p, scope)
        e.emit("if(!%s.ub) return false;" % x)
    for f in frontier:
        sl = slots[f]
        if sl[0] == "p":
            x = e.pred(f, scope)
            e.emit("if(%s.lb) b |= 0x%xull;" % (x, 1 << sl[1]))
            e.emit("if(%s.ub) b |= 0x%xull;" % (x, 1 << (sl[1] + 1)))
        else:
            x = e.expr(f, scope)
            e.emit("hv[%d * stride + j] = make_float2(%s.lo, %s.hi);" % (sl[1], x, x))
            e.emit("if(%s.und) b |= 0x%xull;" % (x, 1 << sl[2]))
    w("\n".join(e.lines))
    w("        (void)box; (void)hv; (void)stride; (void)j;")
    w("        bits = b;")
    w("        return true;")
    w("    }")
    w("    __device__ static bool child(const Iv<float>* box, const float2* hv, std::uint64_t stride, std::uint64_t j,")
    w("                                 std::uint64_t bits) {")
    w("        using T = float;")
    e = Emitter(L)
    e.indent = 2
    scope = {}
    for f in frontier:
        sl = slots[f]
        if sl[0] == "p":
            name = "q%d" % f
            e.emit("const IB %s{(bits & 0x%xull) != 0, (bits & 0x%xull) != 0};" % (name, 1 << sl[1], 1 << (sl[1] + 1)))
        else:
            name = "h%d" % f
            e.emit("const float2 %s_ = hv[%d * stride + j];" % (name, sl[1]))
            e.emit("const Iv<T> %s{%s_.x, %s_.y, (bits & 0x%xull) != 0};" % (name, name, name, 1 << sl[2]))
        scope[f] = name
    for p in dep_top:
        x = e.pred(p, scope)
        e.emit("if(!%s.ub) return false;" % x)
    w("\n".join(e.lines))
    w("        (void)box; (void)hv; (void)stride; (void)j; (void)bits;")
    w("        return true;")
    w("    }")
    w("};")
    w("")
    return nval


def mask(ids):
    m = 0
    for i in ids:
        m |= 1 << i
    return m


def generate(lemma):
    L = lemma
    T_plain = "float" if L.numtype == "f32" else "double"
    ns = "lemma_" + re.sub(r"[^A-Za-z0-9_]", "_", L.slug)
    out = []
    w = out.append
    w("// Generated by csrc/codegen.py from lemmas/%s -- do not edit." % os.path.basename(L.path))
    w('#include "engine.cuh"')
    w('#include "proof_loop.cuh"')
    w('#include "acos.cuh"')
    w("")
    w("namespace sid {")
    w("namespace %s {" % ns)
    w("")
    w("struct L {")
    w("    static constexpr int NARGS = %d;" % L.nargs)
    w("    static constexpr int NBOUNDS = %d;" % len(L.bounds))
    w("    static constexpr std::uint64_t SLOW_BOUNDS = 0x%xull;   // bounds the batch kernel defers" %
      mask(k for k, b in enumerate(L.bounds) if slow_bound(L, b[2])))
    for kind in ("lb", "ub", "both"):
        w("    __device__ __forceinline__ static std::uint64_t upd_%s(int a) {" % kind)
        w("        switch(a) {")
        for a in range(L.nargs):
            m = mask(L.upd.get((a, kind), []))
            if m:
                w("            case %d: return 0x%xull;" % (a, m))
        w("            default: return 0ull;")
        w("        }")
        w("    }")
    w("    __device__ __forceinline__ static int target(int k) {")
    w("        switch(k) {")
    for k, b in enumerate(L.bounds):
        w("            case %d: return %d;" % (k, b[0]))
    w("            default: return 0;")
    w("        }")
    w("    }")
    for which, idx in (("lb", 0), ("ub", 1)):
        w("    __device__ __forceinline__ static long long ct_%s(int v) {" % which)
        w("        switch(v) {")
        for a in range(L.nargs):
            w("            case %d: return %dll;" % (a, L.ct[a][idx]))
        w("            default: return 0ll;")
        w("        }")
        w("    }")
    w("    template<class T> __device__ static int apply_bound(int k, Iv<T>* box);")
    w("    template<int K, class T> __device__ static int apply_bound_c(Iv<T>* box);   // bound K, K known at compile time")
    w("    // the bounds a change of the last variable queues first (upd_both of the last variable)")
    w("    static constexpr std::uint64_t SEED_LAST = 0x%xull;" % mask(L.upd.get((L.nargs - 1, "both"), [])))
    w("    template<class T, bool ALL> __device__ static int rows_eval(int r0, int r1, const Iv<T>* box);")
    w("    template<class T> __device__ static int rows_status(int r0, int r1, const Iv<T>* box) {")
    w("        return rows_eval<T, true>(r0, r1, box);")
    w("    }")
    w("    template<class T> __device__ static bool rows_ok(int r0, int r1, const Iv<T>* box) {")
    w("        return rows_eval<T, false>(r0, r1, box) != 0;")
    w("    }")
    for r in range(L.nargs):
        w("    template<class T, bool ALL> __device__ static int row_%d(const Iv<T>* box);" % r)
    rest_rows = sum(1 << r for r in range(L.nargs) if any(not cheap_constraint(L, L.constraints[ci])
                                                          for ci in L.rows.get(r, [])))
    w("    // rows_ok split in two: comparisons of variables and constants, and the constraints that compute")
    w("    static constexpr std::uint64_t REST_ROWS = 0x%xull;   // rows with constraints that compute" % rest_rows)
    w("    __device__ __forceinline__ static bool has_rest(int r0, int r1) {")
    w("        return ((REST_ROWS >> r0) & ((1ull << (r1 - r0)) - 1)) != 0;")
    w("    }")
    w("    template<class T> __device__ static bool rows_cheap(int r0, int r1, const Iv<T>* box);")
    w("    template<int R, class T> __device__ static bool row_cheap_c(const Iv<T>* box);   // rowc_R, R known at compile time")
    w("    template<class T> __device__ static bool rows_rest(int r0, int r1, const Iv<T>* box);")
    for r in range(L.nargs):
        w("    template<class T> __device__ static bool rowc_%d(const Iv<T>* box);" % r)
        w("    template<class T> __device__ static bool rowx_%d(const Iv<T>* box);" % r)
    operands = comparison_operands(L)
    w("    // the expressions the constraints compare (left, right per comparison), for endpoint dumps")
    w("    static constexpr int NOPERANDS = %d;" % len(operands))
    w("    template<class T> __device__ static void operands(const Iv<T>* box, double2* out, std::int8_t* und,")
    w("                                                      std::uint64_t stride, std::uint64_t i);")
    w("};")
    w("")
    # bound functions: one per bound, dispatched at run time (apply_bound) or at compile time (apply_bound_c)
    for k, (tgt, d, fn, defined) in enumerate(L.bounds):
        e = Emitter(L)
        e.indent = 1
        v = e.expr(fn, {})
        w("template<class T> __device__ __forceinline__ int bound_%d(Iv<T>* box) {" % k)
        out.extend(e.lines)
        w("    return apply_to<%d, %s>(box[%d], %s);" % (d, "true" if defined else "false", tgt, v))
        w("}")
    w("template<class T> __device__ int L::apply_bound(int k, Iv<T>* box) {")
    w("    switch(k) {")
    for k in range(len(L.bounds)):
        w("    case %d: return bound_%d<T>(box);" % (k, k))
    w("    default: return B_NONE;")
    w("    }")
    w("}")
    w("template<int K, class T> __device__ __forceinline__ int L::apply_bound_c(Iv<T>* box) {")
    for k in range(len(L.bounds)):
        w("    %sif constexpr(K == %d) return bound_%d<T>(box);" % ("" if k == 0 else "else ", k, k))
    w("    %sreturn B_NONE;" % ("else " if L.bounds else ""))
    w("}")
    w("")
    for r in range(L.nargs):
        w("template<class T, bool ALL> __device__ int L::row_%d(const Iv<T>* box) {" % r)
        w("    bool all = true;")
        e = Emitter(L)
        scope = {}
        for ci in row_order(L, r):
            p = e.pred(L.constraints[ci], scope)
            e.emit("if(!%s.ub) return 0;" % p)
            e.emit("if constexpr(ALL) all = all && %s.lb;" % p)
        out.extend(e.lines)
        w("    (void)all;")
        w("    return (ALL && all) ? 2 : 1;")
        w("}")
        w("")
    for r in range(L.nargs):
        for cheap, fname in ((True, "rowc"), (False, "rowx")):
            w("template<class T> __device__ bool L::%s_%d(const Iv<T>* box) {" % (fname, r))
            e = Emitter(L)
            scope = {}
            for ci in row_order(L, r):
                if cheap_constraint(L, L.constraints[ci]) == cheap:
                    p = e.pred(L.constraints[ci], scope)
                    e.emit("if(!%s.ub) return false;" % p)
            out.extend(e.lines)
            w("    return true;")
            w("}")
            w("")
    for fname, part in (("rows_cheap", "rowc"), ("rows_rest", "rowx")):
        w("template<class T> __device__ bool L::%s(int r0, int r1, const Iv<T>* box) {" % fname)
        w("    for(int r = r0; r < r1; ++r) {")
        w("        bool ok = true;")
        w("        switch(r) {")
        for r in range(L.nargs):
            w("            case %d: ok = %s_%d<T>(box); break;" % (r, part, r))
        w("            default: break;")
        w("        }")
        w("        if(!ok) return false;")
        w("    }")
        w("    return true;")
        w("}")
        w("")
    w("template<int R, class T> __device__ __forceinline__ bool L::row_cheap_c(const Iv<T>* box) {")
    for r in range(L.nargs):
        w("    %sif constexpr(R == %d) return rowc_%d<T>(box);" % ("" if r == 0 else "else ", r, r))
    w("    else return true;")
    w("}")
    w("")
    w("template<class T, bool ALL> __device__ int L::rows_eval(int r0, int r1, const Iv<T>* box) {")
    w("    int status = 2;")
    w("    for(int r = r0; r < r1; ++r) {")
    w("        int st = 2;")
    w("        switch(r) {")
    for r in range(L.nargs):
        w("            case %d: st = row_%d<T, ALL>(box); break;" % (r, r))
    w("            default: break;")
    w("        }")
    w("        if(st == 0) return 0;")
    w("        if(st == 1) status = 1;")
    w("    }")
    w("    return status;")
    w("}")
    w("")
    w("template<class T> __device__ void L::operands(const Iv<T>* box, double2* out, std::int8_t* und,")
    w("                                              std::uint64_t stride, std::uint64_t i) {")
    e = Emitter(L)
    scope = {}
    for j, nid in enumerate(operands):
        x = e.expr(nid, scope)
        e.emit("out[%d * stride + i] = make_double2(double(%s.lo), double(%s.hi));" % (j, x, x))
        e.emit("und[%d * stride + i] = %s.und ? 1 : 0;" % (j, x))
    out.extend(e.lines)
    w("    (void)box; (void)out; (void)und; (void)stride; (void)i;")
    w("}")
    w("")
    hoisted = []
    if L.numtype != "f32":
        w("template<int LV> struct H;")
        w("")
        for level, var, r0, r1 in levels_with_rows(L):
            plan = hoist_plan(L, var, r0, r1)
            if plan is not None:
                hoisted.append((level, emit_hoisted(L, level, var, plan, w)))
        w("#ifndef SID_LEMMA_DEFS_ONLY   // host launchers and launch table (a bundle part includes only the definitions)")
        w("static int hoist_values(int lv) {")
        w("    switch(lv) {")
        for level, nval in hoisted:
            w("        case %d: return %d;" % (level, nval))
        w("        default: return -1;")
        w("    }")
        w("}")
        w("static cudaError_t prelude_f32(int lv, const LevelArgs& a, std::uint64_t n_items, float2* hv, std::uint64_t* hb,")
        w("                               cudaStream_t s) {")
        w("    switch(lv) {")
        for level, _ in hoisted:
            w("        case %d: return launch_prelude_f32<L, H<%d>>(a, n_items, hv, hb, s);" % (level, level))
        w("        default: return cudaErrorInvalidValue;")
        w("    }")
        w("}")
        w("static cudaError_t filter_hoisted(int lv, const LevelArgs& a, cudaStream_t s) {")
        w("    switch(lv) {")
        for level, _ in hoisted:
            w("        case %d: return launch_filter_hoisted<L, H<%d>>(a, s);" % (level, level))
        w("        default: return cudaErrorInvalidValue;")
        w("    }")
        w("}")
        w("")
    if L.numtype == "f32":
        w("#ifndef SID_LEMMA_DEFS_ONLY   // host launchers and launch table (a bundle part includes only the definitions)")
    w("static cudaError_t level(int mode, const LevelArgs& a, cudaStream_t s) { return launch_level<L, %s>(mode, a, s); }" % T_plain)
    w("static cudaError_t root_box(double2* o, cudaStream_t s) { return launch_root_box<L, %s>(o, s); }" % T_plain)
    w("static cudaError_t eval_batch(const BatchArgs& a, cudaStream_t s) { return launch_eval_batch<L, %s>(a, s); }" % T_plain)
    w("static cudaError_t eval_batch_plain(const BatchArgs& a, cudaStream_t s) {")
    w("    return launch_eval_batch_plain<L, %s>(a, s);" % T_plain)
    w("}")
    w("static cudaError_t proof_loop(const LoopArgs& a, unsigned blocks, cudaStream_t s) {")
    w("    return launch_proof_loop<L, %s>(a, blocks, s);" % T_plain)
    w("}")
    w("static int proof_loop_occupancy() { return sid::proof_loop_occupancy<L, %s>(); }" % T_plain)
    w("static cudaError_t eval_operands(int use_float, const double* lo, const double* hi, std::uint64_t n,")
    w("                                 std::uint64_t stride, double2* o, std::int8_t* u, cudaStream_t s) {")
    w("    return launch_eval_operands<L, %s>(use_float, lo, hi, n, stride, o, u, s);" % T_plain)
    w("}")
    if L.numtype != "f32":
        w("static cudaError_t filter_f32(const LevelArgs& a, cudaStream_t s) { return launch_filter_f32<L>(a, s); }")
        w("static cudaError_t level_esc(int mode, const LevelArgs& a, unsigned blocks, cudaStream_t s) {")
        w("    return launch_level_esc<L>(mode, a, blocks, s);")
        w("}")
    w("#endif")
    w("")
    w("} // namespace %s" % ns)
    w("")
    w("#ifndef SID_LEMMA_DEFS_ONLY")
    w("extern const LemmaKernels kernels_%s;" % ns)
    prec = ("nullptr, nullptr, nullptr, nullptr, nullptr" if L.numtype == "f32" else
            "&{0}::filter_f32, &{0}::level_esc, &{0}::hoist_values, &{0}::prelude_f32, &{0}::filter_hoisted".format(ns))
    w("const LemmaKernels kernels_%s = {\"%s\", 0x%016xull, %d, %d, %s, &%s::level, &%s::root_box, &%s::eval_batch, %s," % (
        ns, L.slug, L.fingerprint, L.nargs, len(L.bounds), "true" if L.numtype == "f32" else "false", ns, ns, ns, prec))
    w("    &%s::eval_batch_plain, %d, &%s::eval_operands, &%s::proof_loop, &%s::proof_loop_occupancy};" % (
        ns, len(operands), ns, ns, ns))
    w("#endif")
    w("")
    w("} // namespace sid")
    return ns, "\n".join(out) + "\n"


def read_bundles(path):
    """Bundle specifications of a bundles file: one `name: lemma lemma ...` per line (# comments)."""
    out = []
    for line in open(path):
        line = line.split("#", 1)[0].strip()
        if not line:
            continue
        name, _, rest = line.partition(":")
        slugs = rest.split()
        if not re.fullmatch(r"[A-Za-z0-9_]+", name.strip()) or not 1 <= len(slugs) <= BUNDLE_MAX:
            raise ValueError("%s: bad bundle line %r" % (path, line))
        out.append((name.strip(), slugs))
    return out


def generate_bundle_part(lemma):
    """The proof-loop parts of one lemma that bundle kernels call, in a unit of their own built with separate
    compilation: the lemma unit's definitions (without its host launchers and launch table) and two exported
    device functions, its root partition and its element processing."""
    ns = "lemma_" + re.sub(r"[^A-Za-z0-9_]", "_", lemma.slug)
    return "\n".join([
        "// Generated by csrc/codegen.py -- do not edit.",
        "// The proof-loop parts of %s that bundle kernels call (separate compilation)." % lemma.slug,
        "#define SID_LEMMA_DEFS_ONLY",
        '#include "%s.cu"' % ns,
        "",
        "namespace sid {",
        "namespace %s {" % ns,
        "__device__ bool loop_root(const LoopArgs& la, unsigned& gen) { return grid_root_partition<L, double>(la, gen); }",
        "__device__ void loop_elements(const LoopArgs& la, std::uint64_t e0, std::uint64_t k) {",
        "    block_elements<L, double>(la, e0, k);",
        "}",
        "} // namespace %s" % ns,
        "} // namespace sid", ""])


def generate_bundle(name, lemmas):
    """A translation unit holding one persistent kernel over the listed lemmas (proof_loop.cuh's bundle loop),
    instantiated with the lemmas in list order. Each lemma's root partition and element processing are the
    loop_root/loop_elements functions of its bundle part (generate_bundle_part), linked by the device-link step,
    so this unit compiles in seconds."""
    for L in lemmas:
        if L.numtype == "f32":
            raise ValueError("bundle %s: %s is a float lemma; bundles hold double lemmas" % (name, L.slug))
    nss = ["lemma_" + re.sub(r"[^A-Za-z0-9_]", "_", L.slug) for L in lemmas]
    types = ", ".join("%s::M" % ns for ns in nss)
    out = ["// Generated by csrc/codegen.py -- do not edit.",
           "// Bundle %s: %s proved together by one persistent kernel." % (name, ", ".join(L.slug for L in lemmas)),
           '#include "engine.cuh"', '#include "proof_loop.cuh"', "", "namespace sid {"]
    for ns in nss:
        out += ["namespace %s {" % ns,
                "__device__ bool loop_root(const LoopArgs& la, unsigned& gen);",
                "__device__ void loop_elements(const LoopArgs& la, std::uint64_t e0, std::uint64_t k);",
                "struct M {",
                "    __device__ static bool root(const LoopArgs& la, unsigned& gen) { return loop_root(la, gen); }",
                "    __device__ static void elements(const LoopArgs& la, std::uint64_t e0, std::uint64_t k) {",
                "        loop_elements(la, e0, k);",
                "    }",
                "};",
                "} // namespace %s" % ns]
    out += ["static cudaError_t bundle_launch_%s(const BundleArgs& b, unsigned blocks, cudaStream_t s) {" % name,
            "    return launch_proof_loop_bundle<%s>(b, blocks, s);" % types,
            "}",
            "static int bundle_occupancy_%s() { return proof_loop_bundle_occupancy<%s>(); }" % (name, types),
            "extern const BundleKernels bundle_%s;" % name,
            "const BundleKernels bundle_%s = {\"%s\", %d, {%s}, &bundle_launch_%s, &bundle_occupancy_%s};" % (
                name, name, len(lemmas), ", ".join("0x%016xull" % L.fingerprint for L in lemmas), name, name),
            "} // namespace sid"]
    return "\n".join(out) + "\n"


def write_if_changed(dest, code):
    old = open(dest).read() if os.path.exists(dest) else None
    if old != code:
        with open(dest, "w") as f:
            f.write(code)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    ap.add_argument("--bundles", action="append", default=[], help="bundles file (name: lemma lemma ...)")
    ap.add_argument("irs", nargs="+")
    args = ap.parse_args()
    os.makedirs(args.out, exist_ok=True)
    names = []
    by_slug = {}
    for p in args.irs:
        lemma = Lemma(p)
        ns, code = generate(lemma)
        write_if_changed(os.path.join(args.out, ns + ".cu"), code)
        names.append(ns)
        by_slug[lemma.slug] = lemma
    bundles = []
    for bf in args.bundles:
        for name, slugs in read_bundles(bf):
            missing = [x for x in slugs if x not in by_slug]
            if missing:
                raise ValueError("bundle %s names lemmas without IR: %s" % (name, ", ".join(missing)))
            write_if_changed(os.path.join(args.out, "bundle_%s.cu" % name),
                             generate_bundle(name, [by_slug[x] for x in slugs]))
            for x in slugs:
                ns = "lemma_" + re.sub(r"[^A-Za-z0-9_]", "_", x)
                write_if_changed(os.path.join(args.out, "bpart_%s.cu" % ns), generate_bundle_part(by_slug[x]))
            bundles.append(name)
    reg = ["// Generated by csrc/codegen.py -- do not edit.", '#include "engine.cuh"', '#include "proof_loop.cuh"', "",
           "namespace sid {"]
    for ns in names:
        reg.append("extern const LemmaKernels kernels_%s;" % ns)
    reg.append("extern const LemmaKernels* const kAllLemmas[] = {")
    for ns in names:
        reg.append("    &kernels_%s," % ns)
    reg.append("};")
    reg.append("extern const int kNumLemmas = %d;" % len(names))
    for b in bundles:
        reg.append("extern const BundleKernels bundle_%s;" % b)
    reg.append("extern const BundleKernels* const kAllBundles[] = {")
    for b in bundles:
        reg.append("    &bundle_%s," % b)
    if not bundles:
        reg.append("    nullptr,")
    reg.append("};")
    reg.append("extern const int kNumBundles = %d;" % len(bundles))
    reg.append("} // namespace sid")
    write_if_changed(os.path.join(args.out, "registry.cu"), "\n".join(reg) + "\n")
    for ns in names:
        print(os.path.join(args.out, ns + ".cu"))
    for b in bundles:
        print(os.path.join(args.out, "bundle_%s.cu" % b))
    return 0


if __name__ == "__main__":
    sys.exit(main())
