// Expression and predicate front end.
//
// The lemma sources build their criteria with ivarp's expression API: argument
// placeholders x0..x9, the literal suffixes _Z / _X, arithmetic and relational
// operators, sqrt/square/fixed_pow/minimum/maximum/acos/if_then_else,
// symbolic calls such as T(-T_inv(s1) + h1), and the junctors || && | & !.
// The reference implements these as expression templates
// (ivarp/include/ivarp/math_fn/*.hpp); here they build a runtime tree with the
// same shape, which the constraint compiler (compile.hpp) later lowers to the
// lemma IR consumed by the GPU engine.
//
// Shape-affecting rules kept from the reference:
//  * literal arithmetic (e.g. 1_Z/3_Z, 2_Z*0.645_X) is evaluated immediately on
//    exact rationals with fixed-point bounds (number/bounded_rational.hpp:43-92);
//  * unary minus of a unary minus cancels (math_fn/unary_ops.hpp:55-77);
//  * chains of || (and &&, |, &) are flattened into one n-ary node
//    (math_fn/math_pred/n_ary_ops.hpp:133-224);
//  * a symbolic call is plain substitution of the arguments
//    (math_fn/symbolic_call.hpp:35-61).
#pragma once

#include <cstdint>
#include <climits>
#include <limits>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <unordered_map>
#include <utility>
#include <vector>

#include "bignum.hpp"
#include "fixed_point.hpp"

namespace ivarp {
namespace sid_fe {

enum class Op : std::uint8_t {
    Arg, Const, BoolConst,
    Neg, Add, Sub, Mul, Div, Sqrt, Pow, Acos, Asin, Min, Max, Ite,
    Lt, Le, Gt, Ge, Eq, Ne, OrSeq, AndSeq, Or, And, Not
};

inline bool is_pred_op(Op o) noexcept {
    switch(o) {
        case Op::BoolConst: case Op::Lt: case Op::Le: case Op::Gt: case Op::Ge: case Op::Eq: case Op::Ne:
        case Op::OrSeq: case Op::AndSeq: case Op::Or: case Op::And: case Op::Not:
            return true;
        default:
            return false;
    }
}

inline const char* op_name(Op o) noexcept {
    switch(o) {
        case Op::Arg: return "arg"; case Op::Const: return "const"; case Op::BoolConst: return "bconst";
        case Op::Neg: return "neg"; case Op::Add: return "add"; case Op::Sub: return "sub";
        case Op::Mul: return "mul"; case Op::Div: return "div"; case Op::Sqrt: return "sqrt";
        case Op::Pow: return "pow"; case Op::Acos: return "acos"; case Op::Asin: return "asin";
        case Op::Min: return "min"; case Op::Max: return "max"; case Op::Ite: return "ite";
        case Op::Lt: return "lt"; case Op::Le: return "le"; case Op::Gt: return "gt"; case Op::Ge: return "ge";
        case Op::Eq: return "eq"; case Op::Ne: return "ne"; case Op::OrSeq: return "orseq";
        case Op::AndSeq: return "andseq"; case Op::Or: return "or"; case Op::And: return "and";
        case Op::Not: return "not";
    }
    return "?";
}

using fxp::i64;

/// A constant leaf: its exact value (a rational interval; a point for literals), its fixed-point
/// compile-time bounds, and the outward roundings used at run time.
struct ConstInfo {
    RatInterval exact;
    i64 lb = fxp::min_bound, ub = fxp::max_bound;
    double dlo = 0, dhi = 0;
    float flo = 0, fhi = 0;

    void round_outward() {
        dlo = exact.lo.to_double_rd();
        dhi = exact.hi.to_double_ru();
        flo = exact.lo.to_float_rd();
        fhi = exact.hi.to_float_ru();
    }
};

struct Node;
using NP = std::shared_ptr<const Node>;

/// One node of an expression/predicate tree. Nodes produced by the constraint compiler additionally carry
/// compile-time bounds (`bounded`), and `wrapped` marks nodes that already went through one
/// bound-and-simplify pass (the reference's BoundedMathExpr / BoundedPredicate wrappers).
struct Node {
    Op op = Op::Const;
    std::vector<NP> ch;
    int arg = -1;
    unsigned power = 0;
    std::shared_ptr<const ConstInfo> cst;
    bool blb = false, bub = true;      // BoolConst value / predicate bounds
    bool bounded = false, wrapped = false;
    i64 lb = fxp::min_bound, ub = fxp::max_bound;   // expression bounds (fixed point)
};

inline NP make_node(Op op, std::vector<NP> ch) {
    auto n = std::make_shared<Node>();
    n->op = op;
    n->ch = std::move(ch);
    return n;
}

inline NP make_arg(int k) {
    auto n = std::make_shared<Node>();
    n->op = Op::Arg;
    n->arg = k;
    return n;
}

inline NP make_const(std::shared_ptr<const ConstInfo> c) {
    auto n = std::make_shared<Node>();
    n->op = Op::Const;
    n->cst = std::move(c);
    n->lb = n->cst->lb;
    n->ub = n->cst->ub;
    n->bounded = true;
    return n;
}

inline NP make_bool_const(bool lb, bool ub) {
    auto n = std::make_shared<Node>();
    n->op = Op::BoolConst;
    n->blb = lb;
    n->bub = ub;
    n->bounded = true;
    return n;
}

/// Number of arguments used (largest argument index + 1).
inline int num_args(const NP& n) {
    if(n->op == Op::Arg) return n->arg + 1;
    int m = 0;
    for(const auto& c : n->ch) m = std::max(m, num_args(c));
    return m;
}

inline bool depends_on(const NP& n, int k) {
    if(n->op == Op::Arg) return n->arg == k;
    for(const auto& c : n->ch) if(depends_on(c, k)) return true;
    return false;
}

/// Replace argument k by args[k] everywhere (the reference's symbolic call).
inline NP substitute(const NP& n, const std::vector<NP>& args, std::unordered_map<const Node*, NP>& memo) {
    auto it = memo.find(n.get());
    if(it != memo.end()) return it->second;
    NP r;
    if(n->op == Op::Arg) {
        r = args.at(std::size_t(n->arg));
    } else if(n->ch.empty()) {
        r = n;
    } else {
        auto c = std::make_shared<Node>(*n);
        for(auto& ch : c->ch) ch = substitute(ch, args, memo);
        r = c;
    }
    memo.emplace(n.get(), r);
    return r;
}

} // namespace sid_fe

class MathExpr;
class MathPred;

/// A rational literal with fixed-point bounds (the reference's BoundedRational); produced by the
/// _Z and _X suffixes. Arithmetic between such numbers stays exact.
struct BoundedQ {
    sid_fe::Rat value;
    sid_fe::i64 lb, ub;
    bool defined = true;
};

inline BoundedQ operator-(const BoundedQ& q) { return {-q.value, -q.ub, -q.lb, q.defined}; }
inline BoundedQ operator+(const BoundedQ& a, const BoundedQ& b) {
    using namespace sid_fe::fxp;
    return {a.value + b.value, add_rd(a.lb, b.lb), add_ru(a.ub, b.ub), a.defined && b.defined};
}
inline BoundedQ operator-(const BoundedQ& a, const BoundedQ& b) {
    using namespace sid_fe::fxp;
    return {a.value - b.value, add_rd(a.lb, -b.ub), add_ru(a.ub, -b.lb), a.defined && b.defined};
}
inline BoundedQ operator*(const BoundedQ& a, const BoundedQ& b) {
    using namespace sid_fe::fxp;
    return {a.value * b.value, iv_mul_lb(a.lb, a.ub, b.lb, b.ub), iv_mul_ub(a.lb, a.ub, b.lb, b.ub),
            a.defined && b.defined};
}
inline BoundedQ operator/(const BoundedQ& a, const BoundedQ& b) {
    using namespace sid_fe::fxp;
    return {a.value / b.value, iv_div_lb(a.lb, a.ub, b.lb, b.ub), iv_div_ub(a.lb, a.ub, b.lb, b.ub),
            a.defined && b.defined};
}

namespace sid_fe {

inline std::shared_ptr<ConstInfo> point_const(const Rat& v, i64 lb, i64 ub) {
    auto c = std::make_shared<ConstInfo>();
    c->exact.lo = v;
    c->exact.hi = v;
    c->lb = lb;
    c->ub = ub;
    c->round_outward();
    return c;
}

inline NP const_from(const BoundedQ& q) {
    return make_const(point_const(q.value, q.defined ? q.lb : fxp::min_bound, q.defined ? q.ub : fxp::max_bound));
}

/// Integer constants get the fixed-point range of their C++ type as bounds, not their value
/// (the reference's BoundsFromIntType, number/fixed_point_bounds.hpp:443-466).
template<typename I> inline NP const_from_int(I v) {
    using L = std::numeric_limits<I>;
    i64 lb, ub;
    if(std::is_signed<I>::value) {
        intmax_t mn = intmax_t(L::min()), mx = intmax_t(L::max());
        lb = (-fxp::fp_maxint <= mn) ? fxp::int_to_fp(i64(mn)) : fxp::min_bound;
        ub = (mx <= fxp::fp_maxint) ? fxp::int_to_fp(i64(mx)) : fxp::max_bound;
    } else {
        uintmax_t mx = uintmax_t(L::max());
        lb = 0;
        ub = (mx <= uintmax_t(fxp::fp_maxint)) ? fxp::int_to_fp(i64(mx)) : fxp::max_bound;
    }
    return make_const(point_const(Rat(std::int64_t(v)), lb, ub));
}

/// Floating-point constants are unbounded at compile time.
inline NP const_from_double(double v) {
    return make_const(point_const(Rat::from_double(v), fxp::min_bound, fxp::max_bound));
}

template<typename T> struct IsNumberOperand :
    std::integral_constant<bool, std::is_arithmetic<std::decay_t<T>>::value &&
                                 !std::is_same<std::decay_t<T>, bool>::value> {};

} // namespace sid_fe

/// Handle to a (symbolic) real-valued expression.
class MathExpr {
public:
    MathExpr() = default;
    explicit MathExpr(sid_fe::NP n) : node(std::move(n)) {}

    const sid_fe::NP& get() const noexcept { return node; }

    /// Symbolic call: substitute the given expressions for x0, x1, ...
    template<typename... A> MathExpr operator()(const A&... a) const;

private:
    sid_fe::NP node;
};

/// Handle to a (symbolic) predicate.
class MathPred {
public:
    MathPred() = default;
    explicit MathPred(sid_fe::NP n) : node(std::move(n)) {}
    const sid_fe::NP& get() const noexcept { return node; }
    template<typename... A> MathPred operator()(const A&... a) const;

private:
    sid_fe::NP node;
};

namespace sid_fe {
template<typename T> struct IsExprLike : std::integral_constant<bool,
    std::is_same<std::decay_t<T>, MathExpr>::value || std::is_same<std::decay_t<T>, BoundedQ>::value ||
    IsNumberOperand<T>::value> {};
template<typename T> struct IsExpr : std::is_same<std::decay_t<T>, MathExpr> {};
template<typename T> struct IsPredLike : std::integral_constant<bool,
    std::is_same<std::decay_t<T>, MathPred>::value || std::is_same<std::decay_t<T>, bool>::value> {};

inline NP to_node(const MathExpr& e) { return e.get(); }
inline NP to_node(const BoundedQ& q) { return const_from(q); }
template<typename T, std::enable_if_t<std::is_integral<T>::value && !std::is_same<T,bool>::value, int> = 0>
inline NP to_node(T v) { return const_from_int(v); }
template<typename T, std::enable_if_t<std::is_floating_point<T>::value, int> = 0>
inline NP to_node(T v) { return const_from_double(double(v)); }

inline NP to_pred_node(const MathPred& p) { return p.get(); }
inline NP to_pred_node(bool b) { return make_bool_const(b, b); }

inline MathExpr unary(Op op, const MathExpr& a) { return MathExpr(make_node(op, {a.get()})); }
template<typename A, typename B> inline MathExpr binary(Op op, const A& a, const B& b) {
    return MathExpr(make_node(op, {to_node(a), to_node(b)}));
}
template<typename A, typename B> inline MathPred relation(Op op, const A& a, const B& b) {
    return MathPred(make_node(op, {to_node(a), to_node(b)}));
}

/// Build an n-ary junctor, merging operands that already are the same junctor.
inline MathPred junctor(Op op, const NP& a, const NP& b) {
    std::vector<NP> ch;
    if(a->op == op) ch.insert(ch.end(), a->ch.begin(), a->ch.end()); else ch.push_back(a);
    if(b->op == op) ch.insert(ch.end(), b->ch.begin(), b->ch.end()); else ch.push_back(b);
    return MathPred(make_node(op, std::move(ch)));
}

template<typename... A> inline std::vector<NP> call_args(const A&... a) { return {to_node(a)...}; }
} // namespace sid_fe

template<typename... A> MathExpr MathExpr::operator()(const A&... a) const {
    std::vector<sid_fe::NP> args = sid_fe::call_args(a...);
    if(int(args.size()) != sid_fe::num_args(node)) {
        throw std::invalid_argument("symbolic call with wrong number of arguments");
    }
    std::unordered_map<const sid_fe::Node*, sid_fe::NP> memo;
    return MathExpr(sid_fe::substitute(node, args, memo));
}

template<typename... A> MathPred MathPred::operator()(const A&... a) const {
    std::vector<sid_fe::NP> args = sid_fe::call_args(a...);
    if(int(args.size()) != sid_fe::num_args(node)) {
        throw std::invalid_argument("symbolic call with wrong number of arguments");
    }
    std::unordered_map<const sid_fe::Node*, sid_fe::NP> memo;
    return MathPred(sid_fe::substitute(node, args, memo));
}

// ---- arithmetic operators ----
#define SID_FE_BINOP(sym, OPC)                                                                           \
    template<typename A, typename B,                                                                     \
             std::enable_if_t<sid_fe::IsExprLike<A>::value && sid_fe::IsExprLike<B>::value &&            \
                              (sid_fe::IsExpr<A>::value || sid_fe::IsExpr<B>::value), int> = 0>          \
    inline MathExpr operator sym(const A& a, const B& b) { return sid_fe::binary(sid_fe::Op::OPC, a, b); }
SID_FE_BINOP(+, Add)
SID_FE_BINOP(-, Sub)
SID_FE_BINOP(*, Mul)
SID_FE_BINOP(/, Div)
#undef SID_FE_BINOP

inline MathExpr operator-(const MathExpr& a) {
    if(a.get()->op == sid_fe::Op::Neg) return MathExpr(a.get()->ch[0]);
    return sid_fe::unary(sid_fe::Op::Neg, a);
}

// ---- relational operators (between expressions, or an expression and a number) ----
#define SID_FE_RELOP(sym, OPC)                                                                           \
    template<typename A, typename B,                                                                     \
             std::enable_if_t<sid_fe::IsExprLike<A>::value && sid_fe::IsExprLike<B>::value &&            \
                              (sid_fe::IsExpr<A>::value || sid_fe::IsExpr<B>::value), int> = 0>          \
    inline MathPred operator sym(const A& a, const B& b) { return sid_fe::relation(sid_fe::Op::OPC, a, b); }
SID_FE_RELOP(<, Lt)
SID_FE_RELOP(<=, Le)
SID_FE_RELOP(>, Gt)
SID_FE_RELOP(>=, Ge)
SID_FE_RELOP(==, Eq)
SID_FE_RELOP(!=, Ne)
#undef SID_FE_RELOP

// ---- logical junctors ----
#define SID_FE_JUNCTOR(sym, OPC)                                                                         \
    template<typename A, typename B,                                                                     \
             std::enable_if_t<sid_fe::IsPredLike<A>::value && sid_fe::IsPredLike<B>::value &&            \
                              (std::is_same<std::decay_t<A>, MathPred>::value ||                         \
                               std::is_same<std::decay_t<B>, MathPred>::value), int> = 0>                \
    inline MathPred operator sym(const A& a, const B& b) {                                              \
        return sid_fe::junctor(sid_fe::Op::OPC, sid_fe::to_pred_node(a), sid_fe::to_pred_node(b));       \
    }
SID_FE_JUNCTOR(||, OrSeq)
SID_FE_JUNCTOR(&&, AndSeq)
SID_FE_JUNCTOR(|, Or)
SID_FE_JUNCTOR(&, And)
#undef SID_FE_JUNCTOR

inline MathPred operator!(const MathPred& p) { return MathPred(sid_fe::make_node(sid_fe::Op::Not, {p.get()})); }

// ---- functions ----
inline MathExpr ensure_expr(const MathExpr& e) { return e; }
inline MathExpr ensure_expr(const BoundedQ& q) { return MathExpr(sid_fe::const_from(q)); }
template<typename T, std::enable_if_t<sid_fe::IsNumberOperand<T>::value, int> = 0>
inline MathExpr ensure_expr(T v) { return MathExpr(sid_fe::to_node(v)); }

inline MathExpr sqrt(const MathExpr& a) { return sid_fe::unary(sid_fe::Op::Sqrt, a); }
inline MathExpr acos(const MathExpr& a) { return sid_fe::unary(sid_fe::Op::Acos, a); }
inline MathExpr asin(const MathExpr& a) { return sid_fe::unary(sid_fe::Op::Asin, a); }

template<unsigned P> inline MathExpr fixed_pow(const MathExpr& a) {
    auto n = std::make_shared<sid_fe::Node>();
    n->op = sid_fe::Op::Pow;
    n->power = P;
    n->ch = {a.get()};
    return MathExpr(n);
}
inline MathExpr square(const MathExpr& a) { return fixed_pow<2>(a); }
// literals (2_Z, 0.5_X) are expressions too
inline MathExpr sqrt(const BoundedQ& a) { return sqrt(ensure_expr(a)); }
inline MathExpr acos(const BoundedQ& a) { return acos(ensure_expr(a)); }
inline MathExpr asin(const BoundedQ& a) { return asin(ensure_expr(a)); }
inline MathExpr square(const BoundedQ& a) { return square(ensure_expr(a)); }
template<unsigned P> inline MathExpr fixed_pow(const BoundedQ& a) { return fixed_pow<P>(ensure_expr(a)); }

template<typename A1, typename... As,
         std::enable_if_t<sid_fe::IsExprLike<A1>::value, int> = 0>
inline MathExpr maximum(const A1& a1, const As&... as) {
    return MathExpr(sid_fe::make_node(sid_fe::Op::Max, {sid_fe::to_node(a1), sid_fe::to_node(as)...}));
}
template<typename A1, typename... As,
         std::enable_if_t<sid_fe::IsExprLike<A1>::value, int> = 0>
inline MathExpr minimum(const A1& a1, const As&... as) {
    return MathExpr(sid_fe::make_node(sid_fe::Op::Min, {sid_fe::to_node(a1), sid_fe::to_node(as)...}));
}

template<typename P, typename T, typename E,
         std::enable_if_t<sid_fe::IsPredLike<P>::value && sid_fe::IsExprLike<T>::value &&
                          sid_fe::IsExprLike<E>::value, int> = 0>
inline MathExpr if_then_else(const P& p, const T& t, const E& e) {
    return MathExpr(sid_fe::make_node(sid_fe::Op::Ite,
                                      {sid_fe::to_pred_node(p), sid_fe::to_node(t), sid_fe::to_node(e)}));
}

// ---- argument placeholders ----
namespace args {
    static const MathExpr x0{sid_fe::make_arg(0)};
    static const MathExpr x1{sid_fe::make_arg(1)};
    static const MathExpr x2{sid_fe::make_arg(2)};
    static const MathExpr x3{sid_fe::make_arg(3)};
    static const MathExpr x4{sid_fe::make_arg(4)};
    static const MathExpr x5{sid_fe::make_arg(5)};
    static const MathExpr x6{sid_fe::make_arg(6)};
    static const MathExpr x7{sid_fe::make_arg(7)};
    static const MathExpr x8{sid_fe::make_arg(8)};
    static const MathExpr x9{sid_fe::make_arg(9)};
}

// ---- literals ----
namespace sid_fe {
/// Integer literal: exact value, point fixed-point bounds (number/int_literal.hpp semantics).
inline BoundedQ int_literal(const std::string& digits) {
    std::string d = digits;
    std::size_t i = 0;
    while(i + 1 < d.size() && d[i] == '0') ++i;
    d = d.substr(i);
    bool fits = d.size() < 19 || (d.size() == 19 && d[0] < '9');
    Rat v = Rat::from_decimal(d);
    if(!fits) return {v, fxp::max_bound, fxp::max_bound, true};
    i64 iv = 0;
    for(char c : d) iv = iv * 10 + (c - '0');
    i64 fp = fxp::int_to_fp(iv);
    return {v, fp, fp, true};
}

/// Decimal literal: the fixed-point bounds keep six fractional digits, rounding the upper bound up if
/// more non-zero digits follow (number/decimal_literal.hpp:51-100).
inline BoundedQ decimal_literal(const std::string& text) {
    std::size_t dot = text.find('.');
    std::string before = dot == std::string::npos ? text : text.substr(0, dot);
    std::string after = dot == std::string::npos ? std::string() : text.substr(dot + 1);
    i64 iv = 0;
    for(char c : before) iv = iv * 10 + (c - '0');
    i64 ifp = fxp::int_to_fp(iv);
    i64 flb = 0, fub = 0, mult = fxp::denom / 10;
    bool tail_nonzero = false;
    for(char c : after) {
        if(mult > 0) { flb += mult * (c - '0'); mult /= 10; }
        else if(c != '0') tail_nonzero = true;
    }
    fub = flb + (tail_nonzero ? 1 : 0);
    std::string all = before.empty() ? "0" : before;
    Rat v = Rat::from_decimal(all + (after.empty() ? std::string() : "." + after));
    return {v, fxp::uadd(std::uint64_t(ifp), std::uint64_t(flb)), fxp::uadd(std::uint64_t(ifp), std::uint64_t(fub)), true};
}
} // namespace sid_fe

template<char... C> inline BoundedQ operator""_Z() {
    const char s[] = {C..., '\0'};
    return sid_fe::int_literal(s);
}

template<char... C> inline BoundedQ operator""_X() {
    const char s[] = {C..., '\0'};
    return sid_fe::decimal_literal(s);
}

} // namespace ivarp
