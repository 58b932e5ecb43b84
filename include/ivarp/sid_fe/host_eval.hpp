// Interval evaluation of a front-end expression on one box, on the host: the values that the critical
// printer shows next to each critical cuboid (the reference's CriticalPrinter evaluates its
// printable_expression()s with array_evaluate on IDouble, critical_printer.hpp:53-57). Critical cuboids
// are few and only printed, so this is a straightforward recursive evaluator, not part of the proof path.
//
// Arithmetic follows the reference's CPU convention: the FPU rounds downward inside the evaluation and
// upper endpoints use the "opposite" form -((-a) op b), so every endpoint is rounded outward
// (ivarp/src/init_rounding.cpp, number/float_interval_addsub.hpp). Products and quotients choose their
// endpoint products from the operands' run-time signs; quotients by intervals containing zero, square
// roots of negative ranges and arc cosines outside [-1, 1] are marked possibly undefined. Constants are
// folded by the constraint compiler (exact rationals or 256-bit values) and rounded outward to double;
// the arc cosine is the correctly rounded one of the device code.
#pragma once

#include <cfenv>
#include <cmath>
#include <limits>
#include <memory>
#include <unordered_map>

#include "compile.hpp"
#include "types.hpp"
#include "../../../squares-in-disk_gb300/csrc/acos.cuh"

namespace ivarp {
namespace sid_fe {

/// Result of a predicate on intervals: definitely true / possibly true.
struct HostBool {
    bool d, p;
    HostBool(bool definitely, bool possibly) : d(definitely), p(possibly) {}
    bool definitely() const { return d; }
    bool possibly() const { return p; }
};

class HostEvaluator {
public:
    /// Evaluate `e` on the box (one interval per argument). The expression is constant-folded once.
    explicit HostEvaluator(const NP& e) {
        std::unordered_map<const Node*, NP> memo;
        root = fold_constants(e, memo);
    }

    IDouble operator()(const IDouble* box) const {
        const int saved = std::fegetround();
        std::fesetround(FE_DOWNWARD);
        std::unordered_map<const Node*, IDouble> cache;
        IDouble r = eval(root.get(), box, cache);
        std::fesetround(saved);
        return r;
    }

private:
    using Iv = IDouble;
    static constexpr double kInf = std::numeric_limits<double>::infinity();

    // round-down mode is active: a op b rounds down, -((-a) op b) rounds up
    static double up_add(double a, double b) { return -((-a) - b); }
    static double up_sub(double a, double b) { return -((-a) + b); }
    static double up_mul(double a, double b) { return -((-a) * b); }
    static double up_div(double a, double b) { return -((-a) / b); }
    static double up_sqrt(double x) {
        const double r = std::sqrt(x);
        return r * r < x ? std::nextafter(r, kInf) : r;   // r*r < x (rounded down) only if r is too small
    }
    static double nan0(double v) { return v != v ? 0.0 : v; }   // 0 * inf in a product endpoint counts as 0

    static Iv mul(const Iv& a, const Iv& b) {
        const double p[4] = {a.lb() * b.lb(), a.lb() * b.ub(), a.ub() * b.lb(), a.ub() * b.ub()};
        const double q[4] = {up_mul(a.lb(), b.lb()), up_mul(a.lb(), b.ub()), up_mul(a.ub(), b.lb()), up_mul(a.ub(), b.ub())};
        double lo = nan0(p[0]), hi = nan0(q[0]);
        for(int k = 1; k < 4; ++k) {
            lo = std::fmin(lo, nan0(p[k]));
            hi = std::fmax(hi, nan0(q[k]));
        }
        return Iv(lo, hi, a.possibly_undefined() || b.possibly_undefined());
    }

    static Iv div(const Iv& a, const Iv& b) {
        const bool und = a.possibly_undefined() || b.possibly_undefined();
        if(!(b.lb() > 0.0 || b.ub() < 0.0)) return Iv(-kInf, kInf, true);
        const double p[4] = {a.lb() / b.lb(), a.lb() / b.ub(), a.ub() / b.lb(), a.ub() / b.ub()};
        const double q[4] = {up_div(a.lb(), b.lb()), up_div(a.lb(), b.ub()), up_div(a.ub(), b.lb()), up_div(a.ub(), b.ub())};
        double lo = nan0(p[0]), hi = nan0(q[0]);
        for(int k = 1; k < 4; ++k) {
            lo = std::fmin(lo, nan0(p[k]));
            hi = std::fmax(hi, nan0(q[k]));
        }
        return Iv(lo, hi, und);
    }

    static Iv power(const Iv& x, unsigned p) {
        if(p == 0) return Iv(1.0, 1.0, x.possibly_undefined());
        Iv r = x;
        Iv acc(1.0, 1.0, x.possibly_undefined());
        for(unsigned k = p; k > 0; k >>= 1) {   // square-and-multiply on intervals
            if(k & 1u) acc = mul(acc, r);
            if(k > 1) r = mul(r, r);
        }
        if(p % 2 == 0) {                         // even powers are non-negative and monotone in |x|
            const double m = std::fmax(std::fabs(x.lb()), std::fabs(x.ub()));
            double lo = 0.0, hi = m;
            for(unsigned k = 1; k < p; ++k) hi = up_mul(hi, m);
            if(x.lb() > 0.0 || x.ub() < 0.0) {
                const double s = std::fmin(std::fabs(x.lb()), std::fabs(x.ub()));
                lo = s;
                for(unsigned k = 1; k < p; ++k) lo = lo * s;
            }
            return Iv(std::fmax(lo, acc.lb()), std::fmin(hi, acc.ub()), x.possibly_undefined());
        }
        return acc;
    }

    static HostBool less(const Iv& a, const Iv& b) {
        const bool und = a.possibly_undefined() || b.possibly_undefined();
        return HostBool(!und && a.ub() < b.lb(), und || a.lb() < b.ub());
    }

    HostBool pred(const Node* n, const IDouble* box, std::unordered_map<const Node*, Iv>& cache) const {
        switch(n->op) {
            case Op::BoolConst: return HostBool(n->blb, n->bub);
            case Op::Lt: return less(eval(n->ch[0].get(), box, cache), eval(n->ch[1].get(), box, cache));
            case Op::Gt: return less(eval(n->ch[1].get(), box, cache), eval(n->ch[0].get(), box, cache));
            case Op::Le: {
                HostBool v = less(eval(n->ch[1].get(), box, cache), eval(n->ch[0].get(), box, cache));
                return HostBool(!v.possibly(), !v.definitely());
            }
            case Op::Ge: {
                HostBool v = less(eval(n->ch[0].get(), box, cache), eval(n->ch[1].get(), box, cache));
                return HostBool(!v.possibly(), !v.definitely());
            }
            case Op::Eq: case Op::Ne: {
                const Iv a = eval(n->ch[0].get(), box, cache), b = eval(n->ch[1].get(), box, cache);
                const bool und = a.possibly_undefined() || b.possibly_undefined();
                const bool overlap = !(a.ub() < b.lb()) && !(b.ub() < a.lb());
                HostBool eq(!und && a.lb() == a.ub() && b.lb() == b.ub() && a.lb() == b.lb(), und || overlap);
                return n->op == Op::Eq ? eq : HostBool(!eq.possibly(), !eq.definitely());
            }
            case Op::Not: {
                HostBool v = pred(n->ch[0].get(), box, cache);
                return HostBool(!v.possibly(), !v.definitely());
            }
            case Op::Or: case Op::OrSeq: {
                bool d = false, p = false;
                for(const auto& c : n->ch) {
                    HostBool v = pred(c.get(), box, cache);
                    d = d || v.definitely();
                    p = p || v.possibly();
                }
                return HostBool(d, p);
            }
            case Op::And: case Op::AndSeq: {
                bool d = true, p = true;
                for(const auto& c : n->ch) {
                    HostBool v = pred(c.get(), box, cache);
                    d = d && v.definitely();
                    p = p && v.possibly();
                }
                return HostBool(d, p);
            }
            default: return HostBool(false, true);
        }
    }

    Iv eval(const Node* n, const IDouble* box, std::unordered_map<const Node*, Iv>& cache) const {
        auto it = cache.find(n);
        if(it != cache.end()) return it->second;
        auto C = [&](std::size_t k) { return eval(n->ch[k].get(), box, cache); };
        Iv r(0.0, 0.0, false);
        switch(n->op) {
            case Op::Arg: r = box[n->arg]; break;
            case Op::Const: r = Iv(n->cst->dlo, n->cst->dhi, n->cst->exact.undefined); break;
            case Op::Neg: { Iv a = C(0); r = Iv(-a.ub(), -a.lb(), a.possibly_undefined()); break; }
            case Op::Add: { Iv a = C(0), b = C(1); r = Iv(a.lb() + b.lb(), up_add(a.ub(), b.ub()), a.possibly_undefined() || b.possibly_undefined()); break; }
            case Op::Sub: { Iv a = C(0), b = C(1); r = Iv(a.lb() - b.ub(), up_sub(a.ub(), b.lb()), a.possibly_undefined() || b.possibly_undefined()); break; }
            case Op::Mul: r = mul(C(0), C(1)); break;
            case Op::Div: r = div(C(0), C(1)); break;
            case Op::Sqrt: {
                Iv a = C(0);
                if(a.ub() < 0.0) { r = Iv(-kInf, kInf, true); break; }
                const bool und = a.possibly_undefined() || a.lb() < 0.0;
                r = Iv(std::sqrt(std::fmax(a.lb(), 0.0)), up_sqrt(a.ub()), und);
                break;
            }
            case Op::Pow: r = power(C(0), n->power); break;
            case Op::Acos: case Op::Asin: {
                Iv a = C(0);
                if(a.ub() < -1.0 || a.lb() > 1.0) { r = Iv(-kInf, kInf, true); break; }
                const bool und = a.possibly_undefined() || a.lb() < -1.0 || a.ub() > 1.0;
                const double lo = std::fmax(a.lb(), -1.0), hi = std::fmin(a.ub(), 1.0);
                if(n->op == Op::Acos) {
                    r = Iv(::sid::acos_cr::acos_rd(hi), ::sid::acos_cr::acos_ru(lo), und);
                } else {   // asin(x) = pi/2 - acos(x)
                    const Iv ph(1.5707963267948966, 1.5707963267948968, false);
                    r = Iv(ph.lb() - ::sid::acos_cr::acos_ru(lo), up_sub(ph.ub(), ::sid::acos_cr::acos_rd(hi)), und);
                }
                break;
            }
            case Op::Min: case Op::Max: {
                Iv acc = C(n->ch.size() - 1);
                for(std::size_t k = n->ch.size() - 1; k-- > 0;) {
                    Iv a = C(k);
                    const bool und = a.possibly_undefined() || acc.possibly_undefined();
                    acc = n->op == Op::Min ? Iv(std::fmin(a.lb(), acc.lb()), std::fmin(a.ub(), acc.ub()), und)
                                           : Iv(std::fmax(a.lb(), acc.lb()), std::fmax(a.ub(), acc.ub()), und);
                }
                r = acc;
                break;
            }
            case Op::Ite: {
                HostBool c = pred(n->ch[0].get(), box, cache);
                if(c.definitely()) r = C(1);
                else if(!c.possibly()) r = C(2);
                else {
                    Iv a = C(1), b = C(2);
                    r = Iv(std::fmin(a.lb(), b.lb()), std::fmax(a.ub(), b.ub()),
                           a.possibly_undefined() || b.possibly_undefined());
                }
                break;
            }
            default: r = Iv(-kInf, kInf, true); break;   // predicates are not printable values
        }
        cache.emplace(n, r);
        return r;
    }

    NP root;
};

} // namespace sid_fe
} // namespace ivarp
