// Constraint compiler: turns a constraint system into the lemma IR.
//
// This restates, as ordinary run-time code over the expression tree, what
// ivarp does with template metaprogramming when a prover input is created
// (ivarp/include/ivarp/prover_input/make_prover_input_impl.hpp:61-83):
//  1. constant subexpressions are folded to outward-rounded constants
//     (cuda_transformer.hpp:73-76, constant_folding/fold_constants.hpp);
//  2. 5*nargs iterations of bound-and-simplify with fixed-point bounds,
//     each followed by tightening the argument bounds from the constraints that
//     have an argument on one side (refactor_constraints_impl.hpp:31-63,
//     refactor_constraint_system.hpp:63-150, compile_time_bound.hpp:140-170);
//  3. a final bound-and-simplify pass that drops constraints known to hold
//     (filter_constraints.hpp:35-61), after which the runtime bound table
//     (runtime_bound_table.hpp:132-210) and the per-argument constraint rows
//     (runtime_constraint_table.hpp:31-115) are built;
//  4. the update lists used by bound propagation, from the bound-dependency
//     analysis (bound_dependency_analysis/*.hpp, runtime_bound_table.hpp:54-123).
// The result is serialised as a line-based text IR (see write_ir) that both the
// GPU engine and the CPU oracle consume.
#pragma once

#include <algorithm>
#include <cctype>
#include <cstdio>
#include <map>
#include <sstream>
#include <string>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "expr.hpp"
#include "types.hpp"

namespace ivarp {
namespace sid_fe {

using Bounds = std::pair<i64, i64>;

struct Dir { enum : int { NONE = 0, LEQ = 1, GEQ = 2, BOTH = 3 }; };

// ------------------------------------------------------------------------------------------------
// Fixed-point evaluation of bounds (EvalBounds of each operation tag).
// ------------------------------------------------------------------------------------------------
inline Bounds eval_expr_bounds(const Node& n, const std::vector<Bounds>& c) {
    using namespace fxp;
    switch(n.op) {
        case Op::Neg: return {-c[0].second, -c[0].first};
        case Op::Add: return {add_rd(c[0].first, c[1].first), add_ru(c[0].second, c[1].second)};
        case Op::Sub: return {add_rd(c[0].first, -c[1].second), add_ru(c[0].second, -c[1].first)};
        case Op::Mul: return {iv_mul_lb(c[0].first, c[0].second, c[1].first, c[1].second),
                              iv_mul_ub(c[0].first, c[0].second, c[1].first, c[1].second)};
        case Op::Div: return {iv_div_lb(c[0].first, c[0].second, c[1].first, c[1].second),
                              iv_div_ub(c[0].first, c[0].second, c[1].first, c[1].second)};
        case Op::Sqrt:
            if(c[0].first < 0) return {min_bound, max_bound};
            return {sqrt_rd(c[0].first), sqrt_ru(c[0].second)};
        case Op::Pow: return {pow_lb(c[0].first, c[0].second, n.power), pow_ub(c[0].first, c[0].second, n.power)};
        case Op::Min: {
            i64 l = c[0].first, u = c[0].second;
            for(std::size_t i = 1; i < c.size(); ++i) { l = std::min(l, c[i].first); u = std::min(u, c[i].second); }
            return {l, u};
        }
        case Op::Max: {
            i64 l = c[0].first, u = c[0].second;
            for(std::size_t i = 1; i < c.size(); ++i) { l = std::max(l, c[i].first); u = std::max(u, c[i].second); }
            return {l, u};
        }
        case Op::Acos: case Op::Asin: return {min_bound, max_bound};
        default: throw std::logic_error("eval_expr_bounds: not an arithmetic operation");
    }
}

/// Predicate bounds are (definitely, possibly), encoded as 0/1.
inline Bounds eval_pred_bounds(const Node& n, const std::vector<Bounds>& c) {
    using fxp::Order;
    auto rel = [&](Op op) -> Bounds {
        Order o = fxp::iv_order(c[0].first, c[0].second, c[1].first, c[1].second);
        bool lb = false, ub = true;
        switch(op) {
            case Op::Le: lb = (o == Order::LE || o == Order::LT || o == Order::EQ);
                         ub = (o == Order::UNKNOWN || o == Order::LE || o == Order::GE || o == Order::LT || o == Order::EQ); break;
            case Op::Lt: lb = (o == Order::LT); ub = (o == Order::UNKNOWN || o == Order::LE || o == Order::LT); break;
            case Op::Ge: lb = (o == Order::GE || o == Order::GT || o == Order::EQ);
                         ub = (o == Order::UNKNOWN || o == Order::GE || o == Order::LE || o == Order::GT || o == Order::EQ); break;
            case Op::Gt: lb = (o == Order::GT); ub = (o == Order::UNKNOWN || o == Order::GE || o == Order::GT); break;
            case Op::Eq: lb = (o == Order::EQ); ub = (o != Order::GT && o != Order::LT); break;
            case Op::Ne: lb = (o == Order::GT || o == Order::LT); ub = (o != Order::EQ); break;
            default: break;
        }
        return {lb ? 1 : 0, ub ? 1 : 0};
    };
    switch(n.op) {
        case Op::Lt: case Op::Le: case Op::Gt: case Op::Ge: case Op::Eq: case Op::Ne: return rel(n.op);
        case Op::OrSeq: case Op::Or: {
            bool l = false, u = false;
            for(const auto& b : c) { l = l || b.first; u = u || b.second; }
            return {l, u};
        }
        case Op::AndSeq: case Op::And: {
            bool l = true, u = true;
            for(const auto& b : c) { l = l && b.first; u = u && b.second; }
            return {l, u};
        }
        case Op::Not: return {c[0].second ? 0 : 1, c[0].first ? 0 : 1};
        default: throw std::logic_error("eval_pred_bounds: not a predicate operation");
    }
}

/// Compile-time bounds of a tree given argument bounds (the reference's CompileTimeBounds): nodes that
/// already carry bounds use them; everything else is evaluated from the children.
inline Bounds ct_bounds(const NP& n, const std::vector<Bounds>& vb) {
    if(n->bounded) {
        if(is_pred_op(n->op)) return {n->blb, n->bub};
        return {n->lb, n->ub};
    }
    switch(n->op) {
        case Op::Arg:
            if(n->arg >= int(vb.size())) throw std::invalid_argument("bound expression uses a later variable");
            return vb[std::size_t(n->arg)];
        case Op::Const: return {n->cst->lb, n->cst->ub};
        case Op::BoolConst: return {n->blb, n->bub};
        case Op::Ite: {
            Bounds c = ct_bounds(n->ch[0], vb), t = ct_bounds(n->ch[1], vb), e = ct_bounds(n->ch[2], vb);
            Bounds b3 = c.first ? t : e;
            Bounds b2 = !c.second ? e : t;
            return {std::min(b2.first, b3.first), std::max(b2.second, b3.second)};
        }
        default: break;
    }
    std::vector<Bounds> cb;
    for(const auto& c : n->ch) cb.push_back(ct_bounds(c, vb));
    if(is_pred_op(n->op)) return eval_pred_bounds(*n, cb);
    return eval_expr_bounds(*n, cb);
}

// ------------------------------------------------------------------------------------------------
// Constant folding on exact rationals (IRational evaluation with 256-bit square roots).
// ------------------------------------------------------------------------------------------------
struct RatBool { bool lb, ub; };

inline RatInterval rat_eval(const NP& n);

inline RatBool rat_pred(const NP& n) {
    switch(n->op) {
        case Op::BoolConst: return {n->blb, n->bub};
        case Op::Lt: case Op::Le: case Op::Gt: case Op::Ge: {
            RatInterval a = rat_eval(n->ch[0]), b = rat_eval(n->ch[1]);
            auto less = [](const RatInterval& x, const RatInterval& y) -> RatBool {
                if(x.undefined || y.undefined) return {false, true};
                return {x.hi < y.lo, x.lo < y.hi};
            };
            RatBool r;
            if(n->op == Op::Lt) r = less(a, b);
            else if(n->op == Op::Gt) r = less(b, a);
            else if(n->op == Op::Le) { RatBool t = less(b, a); r = {!t.ub, !t.lb}; }
            else { RatBool t = less(a, b); r = {!t.ub, !t.lb}; }
            return r;
        }
        case Op::Not: { RatBool c = rat_pred(n->ch[0]); return {!c.ub, !c.lb}; }
        case Op::OrSeq: case Op::Or: {
            RatBool r{false, false};
            for(const auto& c : n->ch) { RatBool v = rat_pred(c); r.lb |= v.lb; r.ub |= v.ub; }
            return r;
        }
        case Op::AndSeq: case Op::And: {
            RatBool r{true, true};
            for(const auto& c : n->ch) { RatBool v = rat_pred(c); r.lb &= v.lb; r.ub &= v.ub; }
            return r;
        }
        default: throw std::invalid_argument("unsupported operation in constant predicate");
    }
}

inline Rat rat_ipow(const Rat& r, unsigned p) {
    Rat x = r, y = (p % 2) ? r : Rat(1);
    for(p /= 2; p > 0; p /= 2) { x = x * x; if(p % 2) y = y * x; }
    return y;
}

inline RatInterval rat_eval(const NP& n) {
    constexpr std::size_t prec = 256;
    switch(n->op) {
        case Op::Const: return n->cst->exact;
        case Op::Neg: { auto a = rat_eval(n->ch[0]); return {-a.hi, -a.lo, a.undefined}; }
        case Op::Add: { auto a = rat_eval(n->ch[0]), b = rat_eval(n->ch[1]); return {a.lo + b.lo, a.hi + b.hi, a.undefined || b.undefined}; }
        case Op::Sub: { auto a = rat_eval(n->ch[0]), b = rat_eval(n->ch[1]); return {a.lo - b.hi, a.hi - b.lo, a.undefined || b.undefined}; }
        case Op::Mul: {
            auto a = rat_eval(n->ch[0]), b = rat_eval(n->ch[1]);
            Rat p[4] = {a.lo * b.lo, a.lo * b.hi, a.hi * b.lo, a.hi * b.hi};
            Rat lo = p[0], hi = p[0];
            for(auto& v : p) { if(v < lo) lo = v; if(hi < v) hi = v; }
            return {lo, hi, a.undefined || b.undefined};
        }
        case Op::Div: {
            auto a = rat_eval(n->ch[0]), b = rat_eval(n->ch[1]);
            if(!(Rat(0) < b.lo) && !(b.hi < Rat(0))) throw std::invalid_argument("constant division by an interval containing zero");
            Rat p[4] = {a.lo / b.lo, a.lo / b.hi, a.hi / b.lo, a.hi / b.hi};
            Rat lo = p[0], hi = p[0];
            for(auto& v : p) { if(v < lo) lo = v; if(hi < v) hi = v; }
            return {lo, hi, a.undefined || b.undefined};
        }
        case Op::Sqrt: {
            auto a = rat_eval(n->ch[0]);
            RatInterval r{Rat(0), Rat(0), a.undefined};
            if(a.lo.is_negative()) {
                if(a.hi.is_negative()) throw std::invalid_argument("sqrt of a negative constant");
                r.undefined = true;
            } else {
                r.lo = a.lo.sqrt_prec(prec, true);
            }
            r.hi = a.hi.sqrt_prec(prec, false);
            return r;
        }
        case Op::Pow: {
            auto a = rat_eval(n->ch[0]);
            unsigned p = n->power;
            if(p % 2 == 1) return {rat_ipow(a.lo, p), rat_ipow(a.hi, p), a.undefined};
            if(a.hi.is_negative()) return {rat_ipow(-a.hi, p), rat_ipow(-a.lo, p), a.undefined};
            if(a.lo.is_negative()) {
                Rat m = -a.lo;
                if(m < a.hi) m = a.hi;
                return {p == 0 ? Rat(1) : Rat(0), rat_ipow(m, p), a.undefined};
            }
            return {rat_ipow(a.lo, p), rat_ipow(a.hi, p), a.undefined};
        }
        case Op::Min: case Op::Max: {
            RatInterval r = rat_eval(n->ch[0]);
            for(std::size_t i = 1; i < n->ch.size(); ++i) {
                RatInterval b = rat_eval(n->ch[i]);
                if(n->op == Op::Min) { if(b.lo < r.lo) r.lo = b.lo; if(b.hi < r.hi) r.hi = b.hi; }
                else { if(r.lo < b.lo) r.lo = b.lo; if(r.hi < b.hi) r.hi = b.hi; }
                r.undefined = r.undefined || b.undefined;
            }
            return r;
        }
        case Op::Ite: {
            RatBool c = rat_pred(n->ch[0]);
            if(c.lb) return rat_eval(n->ch[1]);
            if(!c.ub) return rat_eval(n->ch[2]);
            RatInterval t = rat_eval(n->ch[1]), e = rat_eval(n->ch[2]);
            if(e.lo < t.lo) t.lo = e.lo;
            if(t.hi < e.hi) t.hi = e.hi;
            t.undefined = t.undefined || e.undefined;
            return t;
        }
        default: throw std::invalid_argument(std::string("unsupported operation in constant expression: ") + op_name(n->op));
    }
}

/// Fold every argument-free subtree that is not already a constant into a single constant leaf whose
/// compile-time bounds are computed from the subtree and whose value is the exact (or 256-bit) result.
inline NP fold_constants(const NP& n, std::unordered_map<const Node*, NP>& memo) {
    auto it = memo.find(n.get());
    if(it != memo.end()) return it->second;
    NP r;
    if(n->op == Op::Const || n->op == Op::BoolConst) {
        r = n;
    } else if(num_args(n) == 0) {
        Bounds b = ct_bounds(n, {});
        if(is_pred_op(n->op)) {
            RatBool v = rat_pred(n);
            auto c = std::make_shared<Node>();
            c->op = Op::BoolConst;
            c->blb = v.lb;
            c->bub = v.ub;
            // bounds differ from the value only in degenerate cases; the reference keeps both
            c->bounded = true;
            if(b.first != (v.lb ? 1 : 0) || b.second != (v.ub ? 1 : 0)) {
                throw std::invalid_argument("folded constant predicate with bounds differing from its value");
            }
            r = c;
        } else {
            auto ci = std::make_shared<ConstInfo>();
            ci->exact = rat_eval(n);
            ci->lb = b.first;
            ci->ub = b.second;
            ci->round_outward();
            r = make_const(ci);
        }
    } else {
        auto c = std::make_shared<Node>(*n);
        for(auto& ch : c->ch) ch = fold_constants(ch, memo);
        r = c;
    }
    memo.emplace(n.get(), r);
    return r;
}

// ------------------------------------------------------------------------------------------------
// Bound-and-simplify.
// ------------------------------------------------------------------------------------------------
class BoundAndSimplify {
public:
    explicit BoundAndSimplify(const std::vector<Bounds>& vb) : vb(vb) {}

    NP apply(const NP& n) {
        auto it = memo.find(n.get());
        if(it != memo.end()) return it->second;
        NP r;
        if(n->op == Op::Const || n->op == Op::BoolConst) {
            r = n;
        } else if(n->wrapped) {
            NP cr = inner(n);
            if(!is_pred_op(n->op)) {
                if(cr->op == Op::Const || !cr->wrapped) {
                    throw std::invalid_argument("simplification replaced a bounded expression by a constant (not supported)");
                }
                auto w = std::make_shared<Node>(*cr);
                w->lb = std::max(cr->lb, n->lb);
                w->ub = std::min(cr->ub, n->ub);
                r = w;
            } else {
                if(cr->op == Op::BoolConst) {
                    throw std::invalid_argument("simplification of a bounded predicate produced a constant");
                }
                bool nl = cr->blb || n->blb, nu = cr->bub && n->bub;
                if(nl && nu) r = make_bool_const(true, true);
                else if(!nl && !nu) r = make_bool_const(false, false);
                else if(!nl && nu) {
                    auto w = std::make_shared<Node>(*cr);
                    w->blb = false;
                    w->bub = true;
                    r = w;
                } else {
                    throw std::logic_error("inconsistent predicate bounds");
                }
            }
        } else {
            r = inner(n);
        }
        memo.emplace(n.get(), r);
        return r;
    }

private:
    static NP wrap(const Node& proto, std::vector<NP> ch, i64 lb, i64 ub) {
        auto w = std::make_shared<Node>(proto);
        w->ch = std::move(ch);
        w->bounded = true;
        w->wrapped = true;
        w->lb = lb;
        w->ub = ub;
        return w;
    }

    static NP wrap_pred(const Node& proto, std::vector<NP> ch, bool lb, bool ub) {
        auto w = std::make_shared<Node>(proto);
        w->ch = std::move(ch);
        w->bounded = true;
        w->wrapped = true;
        w->blb = lb;
        w->bub = ub;
        return w;
    }

    /// Simplify the node itself (ignoring any wrapper it may carry).
    NP inner(const NP& n) {
        if(n->op == Op::Arg) {
            const Bounds& b = vb.at(std::size_t(n->arg));
            return wrap(*n, {}, b.first, b.second);
        }
        std::vector<NP> ch;
        for(const auto& c : n->ch) ch.push_back(apply(c));
        if(n->op == Op::Ite) {
            const NP& c = ch[0];
            if(c->blb && c->bub) return ch[1];
            if(!c->blb && !c->bub) return ch[2];
            return wrap(*n, ch, std::min(ch[1]->lb, ch[2]->lb), std::max(ch[1]->ub, ch[2]->ub));
        }
        std::vector<Bounds> cb;
        for(const auto& c : ch) cb.push_back(is_pred_op(c->op) ? Bounds{c->blb, c->bub} : Bounds{c->lb, c->ub});
        if(is_pred_op(n->op)) {
            Bounds pb = eval_pred_bounds(*n, cb);
            return wrap_pred(*n, std::move(ch), pb.first != 0, pb.second != 0);
        }
        Bounds eb = eval_expr_bounds(*n, cb);
        return wrap(*n, std::move(ch), eb.first, eb.second);
    }

    const std::vector<Bounds>& vb;
    std::unordered_map<const Node*, NP> memo;
};

inline const Node* strip(const NP& n) { return n.get(); }

inline bool is_arg_side(int target, const NP& side, bool* negated) {
    if(side->op == Op::Arg) { *negated = false; return side->arg == target; }
    if(side->op == Op::Neg && side->ch[0]->op == Op::Arg) { *negated = true; return side->ch[0]->arg == target; }
    return false;
}

inline int swap_sides(int dir) { return dir == Dir::LEQ ? Dir::GEQ : dir == Dir::GEQ ? Dir::LEQ : dir; }

inline int lhs_direction(Op op) {
    switch(op) {
        case Op::Le: case Op::Lt: return Dir::LEQ;
        case Op::Ge: case Op::Gt: return Dir::GEQ;
        case Op::Eq: return Dir::BOTH;
        default: return Dir::NONE;
    }
}

struct BoundFn {
    int target;
    int dir;
    NP fn;
};

/// Rewrite a relational constraint with the target argument alone on one side into a bound on that
/// argument (the relational-operator and negation rewriters, rewriters/relational_ops.hpp:64-129,
/// rewriters/negation.hpp:36-101).
inline bool rewrite_to_bound(int target, const NP& constraint, BoundFn* out) {
    const Node* c = strip(constraint);
    bool negate_result = false;
    if(c->op == Op::Not) {
        if(!depends_on(constraint, target)) return false;
        c = c->ch[0].get();
        negate_result = true;
    }
    int d0 = lhs_direction(c->op);
    if(d0 == Dir::NONE) return false;
    bool n1 = false, n2 = false;
    bool a1 = is_arg_side(target, c->ch[0], &n1);
    bool a2 = is_arg_side(target, c->ch[1], &n2);
    if(a1 == a2) return false;
    bool negated = a1 ? n1 : n2;
    if(negated) {
        throw std::invalid_argument("constraints with a negated variable alone on one side are not supported");
    }
    int dir = a1 ? d0 : swap_sides(d0);
    if(negate_result) {
        if(dir == Dir::BOTH) return false;
        dir = swap_sides(dir);
    }
    *out = BoundFn{target, dir, a1 ? c->ch[1] : c->ch[0]};
    return true;
}

struct Deps { bool ll = false, lu = false, ul = false, uu = false; bool any() const { return ll || lu || ul || uu; } };

/// Which bound of the expression depends on which bound of argument `a`
/// (bound_dependency_analysis/cbd_*.hpp).
inline Deps bound_deps(const NP& n, int a, std::map<const Node*, Deps>& memo) {
    auto it = memo.find(n.get());
    if(it != memo.end()) return it->second;
    Deps r;
    auto uses_lb = [](int b) { return b == 1 || b == 3; };
    auto uses_ub = [](int b) { return b == 2 || b == 3; };
    auto dep_lb = [&](int used, const Deps& d) { return (uses_lb(used) && d.ll) || (uses_ub(used) && d.ul); };
    auto dep_ub = [&](int used, const Deps& d) { return (uses_lb(used) && d.lu) || (uses_ub(used) && d.uu); };
    const int LB = 1, UB = 2, BOTH = 3;
    switch(n->op) {
        case Op::Arg: if(n->arg == a) { r.ll = true; r.uu = true; } break;
        case Op::Const: case Op::BoolConst: break;
        case Op::Neg: { Deps c = bound_deps(n->ch[0], a, memo); r = {c.ul, c.uu, c.ll, c.lu}; break; }
        case Op::Add: {
            Deps c1 = bound_deps(n->ch[0], a, memo), c2 = bound_deps(n->ch[1], a, memo);
            r = {c1.ll || c2.ll, c1.lu || c2.lu, c1.ul || c2.ul, c1.uu || c2.uu};
            break;
        }
        case Op::Sub: {
            Deps c1 = bound_deps(n->ch[0], a, memo), c2 = bound_deps(n->ch[1], a, memo);
            r = {c1.ll || c2.ul, c1.lu || c2.uu, c1.ul || c2.ll, c1.uu || c2.lu};
            break;
        }
        case Op::Mul: case Op::Div: {
            const NP& x = n->ch[0];
            const NP& y = n->ch[1];
            Deps c1 = bound_deps(x, a, memo), c2 = bound_deps(y, a, memo);
            int s1 = x->lb >= 0 ? 1 : (x->ub <= 0 ? -1 : 0);
            int lb1, ub1, lb2, ub2;
            if(n->op == Op::Mul) {
                int s2 = y->lb >= 0 ? 1 : (y->ub <= 0 ? -1 : 0);
                lb1 = s2 == 1 ? LB : s2 == -1 ? UB : s1 == 1 ? UB : s1 == -1 ? LB : BOTH;
                ub1 = s2 == 1 ? UB : s2 == -1 ? LB : s1 == 1 ? UB : s1 == -1 ? LB : BOTH;
                lb2 = s1 == 1 ? LB : s1 == -1 ? UB : s2 == 1 ? UB : s2 == -1 ? LB : BOTH;
                ub2 = s1 == 1 ? UB : s1 == -1 ? LB : s2 == 1 ? UB : s2 == -1 ? LB : BOTH;
            } else {
                int s2 = y->lb > 0 ? 1 : (y->ub < 0 ? -1 : 0);
                lb1 = s2 == 1 ? LB : s2 == -1 ? UB : BOTH;
                ub1 = s2 == 1 ? UB : s2 == -1 ? LB : BOTH;
                lb2 = s2 == 0 ? BOTH : s1 == 1 ? UB : s1 == -1 ? LB : s2 == 1 ? LB : UB;
                ub2 = s2 == 0 ? BOTH : s1 == 1 ? LB : s1 == -1 ? UB : s2 == 1 ? LB : UB;
            }
            r.ll = dep_lb(lb1, c1) || dep_lb(lb2, c2);
            r.lu = dep_ub(lb1, c1) || dep_ub(lb2, c2);
            r.ul = dep_lb(ub1, c1) || dep_lb(ub2, c2);
            r.uu = dep_ub(ub1, c1) || dep_ub(ub2, c2);
            break;
        }
        default: {
            bool any = false;
            for(const auto& c : n->ch) any = any || bound_deps(c, a, memo).any();
            if(any) r = {true, true, true, true};
            break;
        }
    }
    memo.emplace(n.get(), r);
    return r;
}

struct SplitSpec {
    int arg;
    std::uint32_t initial;
    std::uint32_t subdivisions;
    bool dynamic;
};

/// The compiled form of a constraint system plus split configuration.
struct CompiledLemma {
    std::string name;
    std::string number_type;        // "f64" or "f32"
    int nargs = 0;
    std::vector<std::string> arg_names;
    std::vector<Bounds> ct_bounds;
    std::vector<SplitSpec> splits;
    std::vector<BoundFn> bounds;    // runtime bound table (target-major, constraint order)
    std::vector<NP> constraints;    // filtered constraints
    std::vector<std::vector<int>> rows;
    std::vector<std::vector<int>> upd_lb, upd_ub, upd_both;
};

struct VarDesc {
    int arg;
    std::string name;
    NP lb, ub;
    bool is_value = false;   ///< a value description: one constraint arg == lb (== ub)
};

/// Run the refactoring on folded constraints. `vars` are in the order they were given.
inline CompiledLemma compile_system(const std::vector<VarDesc>& vars, const std::vector<NP>& user_constraints,
                                    const std::vector<std::uint64_t>& split_cfg, const std::string& number_type)
{
    CompiledLemma L;
    L.number_type = number_type;
    L.nargs = int(vars.size());
    const int n = L.nargs;
    L.arg_names.assign(std::size_t(n), std::string());

    // per-argument descriptions in argument order
    std::vector<const VarDesc*> by_arg(std::size_t(n), nullptr);
    for(const auto& v : vars) {
        if(v.arg < 0 || v.arg >= n || by_arg[std::size_t(v.arg)]) {
            throw std::invalid_argument("there must be exactly one description for each argument index");
        }
        by_arg[std::size_t(v.arg)] = &v;
        L.arg_names[std::size_t(v.arg)] = v.name;
    }

    // initial compile-time bounds (extract_ct_bounds.hpp)
    std::vector<Bounds> vb;
    for(int i = 0; i < n; ++i) {
        const VarDesc* d = by_arg[std::size_t(i)];
        Bounds lbb = ct_bounds(d->lb, vb);
        Bounds ubb = ct_bounds(d->ub, vb);
        if(lbb.first > ubb.second) throw std::invalid_argument("empty initial variable bounds");
        vb.push_back({lbb.first, ubb.second});
    }

    // constraints: variable bounds first (in description order), then the user's
    std::vector<NP> cons;
    for(const auto& v : vars) {
        if(v.is_value) {
            cons.push_back(make_node(Op::Eq, {make_arg(v.arg), v.lb}));
        } else {
            cons.push_back(make_node(Op::Ge, {make_arg(v.arg), v.lb}));
            cons.push_back(make_node(Op::Le, {make_arg(v.arg), v.ub}));
        }
    }
    cons.insert(cons.end(), user_constraints.begin(), user_constraints.end());

    // constant folding
    {
        std::unordered_map<const Node*, NP> memo;
        for(auto& c : cons) c = fold_constants(c, memo);
    }

    auto make_table = [&](const std::vector<NP>& cs) {
        std::vector<std::vector<BoundFn>> table(static_cast<std::size_t>(n));
        for(int t = 0; t < n; ++t) {
            for(const auto& c : cs) {
                BoundFn b;
                if(rewrite_to_bound(t, c, &b)) table[std::size_t(t)].push_back(b);
            }
        }
        return table;
    };

    const int iterations = 5 * n;
    for(int it = 0; it < iterations; ++it) {
        BoundAndSimplify bs(vb);
        for(auto& c : cons) c = bs.apply(c);
        auto table = make_table(cons);
        std::vector<Bounds> nvb = vb;
        for(int t = 0; t < n; ++t) {
            Bounds b = vb[std::size_t(t)];
            for(const auto& bf : table[std::size_t(t)]) {
                if(bf.dir & Dir::GEQ) b.first = std::max(b.first, bf.fn->lb);
                if(bf.dir & Dir::LEQ) b.second = std::min(b.second, bf.fn->ub);
            }
            if(b.first > b.second) throw std::invalid_argument("empty bounds at compile time (proof trivially done?)");
            nvb[std::size_t(t)] = b;
        }
        vb = nvb;
    }
    {
        BoundAndSimplify bs(vb);
        for(auto& c : cons) c = bs.apply(c);
        std::vector<NP> kept;
        for(const auto& c : cons) {
            if(!c->blb) kept.push_back(c);
        }
        cons = kept;
    }
    L.ct_bounds = vb;
    L.constraints = cons;

    auto table = make_table(cons);
    for(int t = 0; t < n; ++t) {
        for(const auto& b : table[std::size_t(t)]) {
            if(!b.fn->bounded) throw std::logic_error("unbounded bound function");
            L.bounds.push_back(b);
        }
    }

    // constraint rows
    L.rows.assign(std::size_t(n), {});
    for(std::size_t ci = 0; ci < cons.size(); ++ci) {
        bool rewritten = false;
        for(int t = 0; t < n && !rewritten; ++t) {
            BoundFn b;
            rewritten = rewrite_to_bound(t, cons[ci], &b);
        }
        int na = num_args(cons[ci]);
        for(int r = 0; r < n - 1; ++r) {
            if(!rewritten && na == r + 1) L.rows[std::size_t(r)].push_back(int(ci));
        }
        L.rows[std::size_t(n - 1)].push_back(int(ci));
    }

    // update lists (NeedsUpdate)
    L.upd_lb.assign(std::size_t(n), {});
    L.upd_ub.assign(std::size_t(n), {});
    L.upd_both.assign(std::size_t(n), {});
    for(int a = 0; a < n; ++a) {
        std::map<const Node*, Deps> memo;
        for(std::size_t bi = 0; bi < L.bounds.size(); ++bi) {
            const BoundFn& b = L.bounds[bi];
            Deps d = bound_deps(b.fn, a, memo);
            bool need_lb = (b.dir & Dir::GEQ) != 0;
            bool need_ub = (b.dir & Dir::LEQ) != 0;
            bool on_lb = (need_lb && d.ll) || (need_ub && d.ul);
            bool on_ub = (need_lb && d.lu) || (need_ub && d.uu);
            if(on_lb) L.upd_lb[std::size_t(a)].push_back(int(bi));
            if(on_ub) L.upd_ub[std::size_t(a)].push_back(int(bi));
            if(on_lb || on_ub) L.upd_both[std::size_t(a)].push_back(int(bi));
        }
    }

    // split configuration (process_var_splitting.hpp:94-139)
    if(split_cfg.size() != std::size_t(n)) throw std::invalid_argument("wrong number of elements in variable splitting");
    bool seen_static = false;
    for(int i = 0; i < n; ++i) {
        std::uint64_t s = split_cfg[std::size_t(i)];
        bool dyn = (s >> 32) != 0;
        if(i == 0 && !dyn) { s = dynamic_subdivision(std::uint32_t(s), 4); dyn = true; }
        if(dyn && seen_static) throw std::invalid_argument("dynamically split variables must be a consecutive prefix");
        if(!dyn) seen_static = true;
        L.splits.push_back(SplitSpec{i, std::uint32_t(s >> 32), std::uint32_t(s & 0xffffffffu), dyn});
    }
    return L;
}

// ------------------------------------------------------------------------------------------------
// IR serialisation.
// ------------------------------------------------------------------------------------------------
inline std::string hexd(double v) {
    char buf[64];
    std::snprintf(buf, sizeof(buf), "%a", v);
    return buf;
}

inline std::string escape_token(const std::string& s) {
    std::string r;
    for(unsigned char c : s) {
        if(std::isalnum(c) || c == '_' || c == '-' || c == '.' || c == ',' || c == '{' || c == '}' || c == '>' ||
           c == '<' || c == '=' || c == '(' || c == ')') {
            r += char(c);
        } else {
            char buf[8];
            std::snprintf(buf, sizeof(buf), "%%%02X", unsigned(c));
            r += buf;
        }
    }
    return r.empty() ? std::string("%") : r;
}

class IrWriter {
public:
    std::string write(const CompiledLemma& L) {
        std::ostringstream body;
        for(const auto& b : L.bounds) intern(b.fn);
        for(const auto& c : L.constraints) intern(c);
        std::ostringstream o;
        o << "sidir 1\n";
        o << "name " << escape_token(L.name) << "\n";
        o << "numtype " << L.number_type << "\n";
        o << "nargs " << L.nargs << "\n";
        for(int i = 0; i < L.nargs; ++i) {
            o << "arg " << i << " " << escape_token(L.arg_names[std::size_t(i)]) << " "
              << L.ct_bounds[std::size_t(i)].first << " " << L.ct_bounds[std::size_t(i)].second << "\n";
        }
        for(const auto& s : L.splits) {
            o << "split " << s.arg << " " << s.initial << " " << s.subdivisions << " " << (s.dynamic ? 1 : 0) << "\n";
        }
        for(std::size_t i = 0; i < consts.size(); ++i) {
            const ConstInfo& c = *consts[i];
            o << "const " << i << " " << hexd(c.dlo) << " " << hexd(c.dhi) << " " << hexd(double(c.flo)) << " "
              << hexd(double(c.fhi)) << " " << (c.exact.undefined ? 1 : 0) << "\n";
        }
        o << lines.str();
        for(std::size_t i = 0; i < L.bounds.size(); ++i) {
            const auto& b = L.bounds[i];
            bool defined = fxp::is_lb(b.fn->lb) || fxp::is_ub(b.fn->ub);
            o << "bound " << i << " " << b.target << " " << (b.dir == Dir::LEQ ? "leq" : b.dir == Dir::GEQ ? "geq" : "both")
              << " " << ids.at(b.fn.get()) << " " << (defined ? 1 : 0) << "\n";
        }
        auto list = [&](const char* kind, int a, const std::vector<int>& v) {
            o << "update " << a << " " << kind << " " << v.size();
            for(int x : v) o << " " << x;
            o << "\n";
        };
        for(int a = 0; a < L.nargs; ++a) {
            list("lb", a, L.upd_lb[std::size_t(a)]);
            list("ub", a, L.upd_ub[std::size_t(a)]);
            list("both", a, L.upd_both[std::size_t(a)]);
        }
        for(std::size_t i = 0; i < L.constraints.size(); ++i) {
            o << "constraint " << i << " " << ids.at(L.constraints[i].get()) << "\n";
        }
        for(int r = 0; r < L.nargs; ++r) {
            o << "row " << r << " " << L.rows[std::size_t(r)].size();
            for(int c : L.rows[std::size_t(r)]) o << " " << c;
            o << "\n";
        }
        o << "end\n";
        return o.str();
    }

private:
    int const_id(const std::shared_ptr<const ConstInfo>& c) {
        auto key = std::make_tuple(hexd(c->dlo), hexd(c->dhi), hexd(double(c->flo)), hexd(double(c->fhi)), c->exact.undefined);
        auto it = const_ids.find(key);
        if(it != const_ids.end()) return it->second;
        int id = int(consts.size());
        consts.push_back(c);
        const_ids.emplace(key, id);
        return id;
    }

    /// Hash-cons nodes structurally (op, parameters, children, bounds) and emit them in topological order.
    int intern(const NP& n) {
        auto it = ids.find(n.get());
        if(it != ids.end()) return it->second;
        std::vector<int> cids;
        for(const auto& c : n->ch) cids.push_back(intern(c));
        bool pred = is_pred_op(n->op);
        long long aux = 0;
        if(n->op == Op::Arg) aux = n->arg;
        else if(n->op == Op::Const) aux = const_id(n->cst);
        else if(n->op == Op::Pow) aux = n->power;
        long long lb = pred ? (n->blb ? 1 : 0) : n->lb;
        long long ub = pred ? (n->bub ? 1 : 0) : n->ub;
        std::ostringstream key;
        key << op_name(n->op) << " " << lb << " " << ub << " " << aux << " " << cids.size();
        for(int c : cids) key << " " << c;
        std::string k = key.str();
        auto sit = structural.find(k);
        int id;
        if(sit != structural.end()) {
            id = sit->second;
        } else {
            id = next_id++;
            structural.emplace(k, id);
            lines << "node " << id << " " << k << "\n";
        }
        ids.emplace(n.get(), id);
        return id;
    }

    std::unordered_map<const Node*, int> ids;
    std::unordered_map<std::string, int> structural;
    std::map<std::tuple<std::string, std::string, std::string, std::string, bool>, int> const_ids;
    std::vector<std::shared_ptr<const ConstInfo>> consts;
    std::ostringstream lines;
    int next_id = 0;
};

inline std::string to_ir(const CompiledLemma& L) {
    IrWriter w;
    return w.write(L);
}

} // namespace sid_fe
} // namespace ivarp
