// CPU ORACLE -- test infrastructure only (see oracle.hpp for what it restates).
// Build: oracle/Makefile (-frounding-math -ffp-contract=off, no -ffast-math).
#include "oracle.hpp"

#include "../squares-in-disk_gb300/csrc/lemma_ir.hpp"
#include "acos_cr.hpp"

#include <algorithm>
#include <atomic>
#include <cfenv>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <limits>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <thread>
#include <type_traits>

namespace sido {
namespace {

using sid::LemmaIR;
using sid::NodeOp;

constexpr std::int64_t FXMAX = sid::kFxpMax;
constexpr std::int64_t FXMIN = sid::kFxpMin;
constexpr std::int64_t FX_ONE = 1000000;

/// Sets the round-down mode for the lifetime of the object (the reference sets it globally at load
/// time, ivarp/src/init_rounding.cpp:57) and checks that the compiler kept the directed operations.
struct RoundDownScope {
    int old;
    RoundDownScope() : old(std::fegetround()) {
        std::fesetround(FE_DOWNWARD);
        volatile double a = 1.1, b = 10.1;
        double dn = a * b;
        double up = -((-a) * b);
        if(!(dn < up)) throw std::runtime_error("oracle: directed rounding is not effective");
    }
    ~RoundDownScope() { std::fesetround(old); }
};

// Operation counting (the op-counting build, -DSIDO_COUNT_OPS, used to measure IEEE directed-rounding
// operations per cuboid): additions/subtractions, multiplications, divisions, square roots, arc cosines.
#ifdef SIDO_COUNT_OPS
std::atomic<unsigned long long> g_ops[10];   // per kind, double then float
#define SIDO_COUNT(k) (g_ops[(k) + (sizeof(T) == sizeof(float) ? 5 : 0)].fetch_add(1, std::memory_order_relaxed))
#else
#define SIDO_COUNT(k) ((void)0)
#endif

// Directed basic operations; the ambient mode is round-down, upper bounds use the sign trick.
template<class T> inline T add_rd(T a, T b) { SIDO_COUNT(0); return a + b; }
template<class T> inline T add_ru(T a, T b) { SIDO_COUNT(0); return -((-a) - b); }
template<class T> inline T sub_rd(T a, T b) { SIDO_COUNT(0); return a - b; }
template<class T> inline T sub_ru(T a, T b) { SIDO_COUNT(0); return -(b - a); }
template<class T> inline T mul_rd(T a, T b) { SIDO_COUNT(1); return a * b; }
template<class T> inline T mul_ru(T a, T b) { SIDO_COUNT(1); return -((-a) * b); }
template<class T> inline T div_rd(T a, T b) { SIDO_COUNT(2); return a / b; }
template<class T> inline T div_ru(T a, T b) { SIDO_COUNT(2); return -((-a) / b); }
template<class T> inline T sqrt_rd(T x) { SIDO_COUNT(3); return std::sqrt(x); }
template<class T> __attribute__((noinline)) T sqrt_ru(T x) {
    SIDO_COUNT(3);
    std::fesetround(FE_UPWARD);
    volatile T vx = x;
    T r = std::sqrt(vx);
    volatile T vr = r;
    std::fesetround(FE_DOWNWARD);
    return vr;
}

template<class T> struct Iv { T lo, hi; bool und; };
struct IB { bool lb, ub; };

inline bool isfin(std::int64_t l, std::int64_t u) { return l > FXMIN && u < FXMAX; }

template<class T> inline T nan0(T v, bool finite) { return (!finite && v != v) ? T(0) : v; }
template<class T> inline T inf() { return std::numeric_limits<T>::infinity(); }
template<class T> inline int sgn(T v) { return (v > 0) - (v < 0); }

template<class T> struct Evaluator {
    const LemmaIR& L;
    std::vector<Iv<T>> val;
    std::vector<IB> pval;
    std::vector<std::uint32_t> stamp;
    std::uint32_t epoch = 1;
    const Iv<T>* box = nullptr;

    // the precision form's float pass of a lemma in double bounds acos with acos_bound_f32 instead of the
    // correctly rounded float arc cosine
    const bool fast_acos;

    explicit Evaluator(const LemmaIR& l) : L(l), val(l.nodes.size()), pval(l.nodes.size()), stamp(l.nodes.size(), 0),
        fast_acos(std::is_same<T, float>::value && l.numtype != "f32") {}

    void begin(const Iv<T>* b) {
        box = b;
        if(++epoch == 0) { std::fill(stamp.begin(), stamp.end(), 0u); epoch = 1; }
    }

    Iv<T> cval(int id) const {
        const auto& c = L.consts[std::size_t(id)];
        if(sizeof(T) == sizeof(double)) return {T(c.dlo), T(c.dhi), c.undefined};
        return {T(c.flo), T(c.fhi), c.undefined};
    }

    // ia_do_mul: lower = rd(l1*l2), upper = ru(u1*u2), NaN -> 0 unless bounded finitely
    static void do_mul(T l1, T l2, T u1, T u2, bool finite, T& lo, T& hi) {
        lo = nan0(mul_rd(l1, l2), finite);
        hi = nan0(mul_ru(u1, u2), finite);
    }

    static Iv<T> mul(const Iv<T>& a, const Iv<T>& b, std::int64_t al, std::int64_t au, std::int64_t bl,
                     std::int64_t bu) {
        const bool finite = isfin(al, au) && isfin(bl, bu);
        auto nonneg = [](std::int64_t l, std::int64_t u, T x) { return l >= 0 ? true : (u <= 0 ? false : x >= 0); };
        auto nonpos = [](std::int64_t l, std::int64_t u, T x) { return u <= 0 ? true : (l >= 0 ? false : x <= 0); };
        T lo, hi;
        if(nonneg(al, au, a.lo)) {
            if(nonneg(bl, bu, b.lo)) do_mul(a.lo, b.lo, a.hi, b.hi, finite, lo, hi);
            else if(nonpos(bl, bu, b.hi)) do_mul(a.hi, b.lo, a.lo, b.hi, finite, lo, hi);
            else do_mul(a.hi, b.lo, a.hi, b.hi, finite, lo, hi);
        } else if(nonpos(al, au, a.hi)) {
            if(nonneg(bl, bu, b.lo)) do_mul(a.lo, b.hi, a.hi, b.lo, finite, lo, hi);
            else if(nonpos(bl, bu, b.hi)) do_mul(a.hi, b.hi, a.lo, b.lo, finite, lo, hi);
            else do_mul(a.lo, b.hi, a.lo, b.lo, finite, lo, hi);
        } else if(nonneg(bl, bu, b.lo)) {
            do_mul(a.lo, b.hi, a.hi, b.hi, finite, lo, hi);
        } else if(nonpos(bl, bu, b.hi)) {
            do_mul(a.hi, b.lo, a.lo, b.lo, finite, lo, hi);
        } else {
            T l1, h1, l2, h2;
            do_mul(a.lo, b.hi, a.lo, b.lo, finite, l1, h1);
            do_mul(b.lo, a.hi, a.hi, b.hi, finite, l2, h2);
            lo = (l2 <= l1) ? l2 : l1;
            hi = (h1 <= h2) ? h2 : h1;
        }
        return {lo, hi, a.und || b.und};
    }

    static void divide_by_zero(Iv<T>& num, const Iv<T>& den, int snl, int snu, int sds) {
        num.und = true;
        if(sds == 0 || snu - snl == 2) { num.lo = -inf<T>(); num.hi = inf<T>(); return; }
        if(sds > 0) {
            if(snl >= 0) { num.lo = div_rd(num.lo, den.hi); num.hi = inf<T>(); }
            else { num.hi = div_ru(num.hi, den.hi); num.lo = -inf<T>(); }
        } else {
            if(snl >= 0) { num.hi = div_ru(num.lo, den.lo); num.lo = -inf<T>(); }
            else { num.lo = div_rd(num.hi, den.lo); num.hi = inf<T>(); }
        }
    }

    struct WI { T v; int inf_sign; };
    static T div_lb_inf(const WI& n, const WI& d) {
        if(!n.inf_sign && !d.inf_sign) return div_rd(n.v, d.v);
        if(d.inf_sign != 0) return T(0);
        return -inf<T>();
    }
    static T div_ub_inf(const WI& n, const WI& d) {
        if(!n.inf_sign && !d.inf_sign) return div_ru(n.v, d.v);
        if(d.inf_sign != 0) return T(0);
        return inf<T>();
    }

    static Iv<T> div(Iv<T> num, const Iv<T>& den, std::int64_t nl, std::int64_t nu, std::int64_t dl, std::int64_t du) {
        bool ct_finite = isfin(nl, nu) && isfin(dl, du);
        bool rt_finite = std::isfinite(num.lo) && std::isfinite(num.hi) && std::isfinite(den.lo) && std::isfinite(den.hi);
        num.und = num.und || den.und;
        if(ct_finite || rt_finite) {
            auto nonneg = [&](T x) { return nl >= 0 ? true : (nu <= 0 ? false : x >= 0); };
            auto nonpos = [&](T x) { return nu <= 0 ? true : (nl >= 0 ? false : x <= 0); };
            bool positive = dl > 0 ? true : (du <= 0 ? false : den.lo > 0);
            bool negative = false;
            if(!positive) negative = du < 0 ? true : (dl >= 0 ? false : den.hi < 0);
            if(positive) {
                if(nonneg(num.lo)) { T l = div_rd(num.lo, den.hi), h = div_ru(num.hi, den.lo); num.lo = l; num.hi = h; }
                else if(nonpos(num.hi)) { T l = div_rd(num.lo, den.lo), h = div_ru(num.hi, den.hi); num.lo = l; num.hi = h; }
                else { T l = div_rd(num.lo, den.lo), h = div_ru(num.hi, den.lo); num.lo = l; num.hi = h; }
            } else if(negative) {
                if(nonneg(num.lo)) { T l = div_rd(num.hi, den.hi), h = div_ru(num.lo, den.lo); num.lo = l; num.hi = h; }
                else if(nonpos(num.hi)) { T l = div_rd(num.hi, den.lo), h = div_ru(num.lo, den.hi); num.lo = l; num.hi = h; }
                else { T l = div_rd(num.hi, den.hi), h = div_ru(num.lo, den.hi); num.lo = l; num.hi = h; }
            } else {
                divide_by_zero(num, den, sgn(num.lo), sgn(num.hi), sgn(den.lo) + sgn(den.hi));
            }
            return num;
        }
        int snl = sgn(num.lo), snu = sgn(num.hi), sdl = sgn(den.lo), sdu = sgn(den.hi);
        WI n_lb{num.lo, std::isfinite(num.lo) ? 0 : -1}, n_ub{num.hi, std::isfinite(num.hi) ? 0 : 1};
        WI d_lb{den.lo, std::isfinite(den.lo) ? 0 : -1}, d_ub{den.hi, std::isfinite(den.hi) ? 0 : 1};
        auto set = [&](const WI& a, const WI& b, const WI& c, const WI& d) {
            T l = div_lb_inf(a, b), h = div_ub_inf(c, d);
            num.lo = l; num.hi = h;
        };
        if(sdl > 0) {
            if(snl >= 0) set(n_lb, d_ub, n_ub, d_lb);
            else if(snu <= 0) set(n_lb, d_lb, n_ub, d_ub);
            else set(n_lb, d_lb, n_ub, d_lb);
        } else if(sdu < 0) {
            if(snl >= 0) set(n_ub, d_ub, n_lb, d_lb);
            else if(snu <= 0) set(n_ub, d_lb, n_lb, d_ub);
            else set(n_ub, d_ub, n_lb, d_ub);
        } else {
            divide_by_zero(num, den, snl, snu, sdl + sdu);
        }
        return num;
    }

    /// Integer power P >= 3 as computed by the reference's CPU path (two lanes in round-down mode with sign
    /// bookkeeping; fixed_pow.hpp:93-126).
    static Iv<T> pow_lanes(T lb, T ub, bool und, unsigned p, bool even) {
        T u = -ub;
        bool nl = std::signbit(lb), nu = std::signbit(u);
        T xl = lb, xu = u;
        T nxl = nl ? -xl : xl, nxu = nu ? -xu : xu;
        T yl = even ? T(1) : lb, yu = even ? T(-1) : u;
        for(p /= 2; p > 0; p /= 2) {
            xl = xl * nxl; xu = xu * nxu;
            SIDO_COUNT(1);
            SIDO_COUNT(1);
            nxl = nl ? -xl : xl; nxu = nu ? -xu : xu;
            if(p % 2) { yl = yl * nxl; yu = yu * nxu; SIDO_COUNT(1); SIDO_COUNT(1); }
        }
        return {yl, -yu, und};
    }

    static Iv<T> power(const Iv<T>& x, unsigned p) {
        if(p == 0) return {T(1), T(1), x.und};
        if(p == 1) return x;
        if(p == 2) {
            Iv<T> r = mul(x, x, FXMIN, FXMAX, FXMIN, FXMAX);
            if(r.lo < 0) r.lo = 0;
            return r;
        }
        if(p % 2) return pow_lanes(x.lo, x.hi, x.und, p, false);
        if(x.hi < 0) return pow_lanes(-x.hi, -x.lo, x.und, p, true);
        if(x.lo < 0) {
            T a = std::fabs(x.lo), b = std::fabs(x.hi);
            T m = a < b ? b : a;
            return pow_lanes(T(0), m, x.und, p, true);
        }
        return pow_lanes(x.lo, x.hi, x.und, p, true);
    }

    Iv<T> eval(int id) {
        if(stamp[std::size_t(id)] == epoch) return val[std::size_t(id)];
        const auto& n = L.nodes[std::size_t(id)];
        Iv<T> r;
        auto C = [&](int k) { return eval(n.ch[std::size_t(k)]); };
        auto CB = [&](int k) -> const sid::IrNode& { return L.nodes[std::size_t(n.ch[std::size_t(k)])]; };
        switch(n.op) {
            case NodeOp::Arg: r = box[n.aux]; r.und = false; break;
            case NodeOp::Const: r = cval(int(n.aux)); break;
            case NodeOp::Neg: { auto a = C(0); r = {-a.hi, -a.lo, a.und}; break; }
            case NodeOp::Add: { auto a = C(0), b = C(1); r = {add_rd(a.lo, b.lo), add_ru(a.hi, b.hi), a.und || b.und}; break; }
            case NodeOp::Sub: { auto a = C(0), b = C(1); r = {sub_rd(a.lo, b.hi), sub_ru(a.hi, b.lo), a.und || b.und}; break; }
            case NodeOp::Mul: { auto a = C(0), b = C(1); r = mul(a, b, CB(0).lb, CB(0).ub, CB(1).lb, CB(1).ub); break; }
            case NodeOp::Div: { auto a = C(0), b = C(1); r = div(a, b, CB(0).lb, CB(0).ub, CB(1).lb, CB(1).ub); break; }
            case NodeOp::Sqrt: {
                auto x = C(0);
                T lo = x.lo, hi = x.hi;
                bool und = x.und;
                std::int64_t bl = CB(0).lb, bu = CB(0).ub;
                bool nonneg = bl >= 0 ? true : (bu <= 0 ? false : x.lo >= 0);
                if(!nonneg) {
                    if(hi < 0) { r = {-inf<T>(), inf<T>(), true}; break; }
                    lo = 0;
                    und = true;
                }
                r = {sqrt_rd(lo), sqrt_ru(hi), und};
                break;
            }
            case NodeOp::Pow: r = power(C(0), unsigned(n.aux)); break;
            case NodeOp::Min: case NodeOp::Max: {
                // n-ary forms evaluate as f(a1, f(a2, f(a3, ...)))
                std::size_t k = n.ch.size();
                Iv<T> acc = C(int(k - 1));
                for(std::size_t i = k - 1; i-- > 0;) {
                    Iv<T> a = C(int(i));
                    if(n.op == NodeOp::Min) {
                        acc = {a.lo < acc.lo ? a.lo : acc.lo, a.hi < acc.hi ? a.hi : acc.hi, a.und || acc.und};
                    } else {
                        acc = {acc.lo < a.lo ? a.lo : acc.lo, acc.hi < a.hi ? a.hi : acc.hi, a.und || acc.und};
                    }
                }
                r = acc;
                break;
            }
            case NodeOp::Acos: {
                Iv<T> x = C(0);
                bool und = x.und;
                if(CB(0).lb < -FX_ONE && x.lo < T(-1)) { und = true; x.lo = T(-1); }
                if(CB(0).ub > FX_ONE && T(1) < x.hi) { und = true; x.hi = T(1); }
                SIDO_COUNT(4);
                SIDO_COUNT(4);
                if(fast_acos) {
                    r = {T(acos_bound_f32(float(x.hi), false)), T(acos_bound_f32(float(x.lo), true)), und};
                } else {
                    r = {acos_rounded<T>(x.hi, false), acos_rounded<T>(x.lo, true), und};
                }
                break;
            }
            case NodeOp::Ite: {
                IB c = evalp(n.ch[0]);
                if(c.lb) r = C(1);
                else if(!c.ub) r = C(2);
                else {
                    r = C(1);
                    Iv<T> e = C(2);
                    if(e.lo < r.lo) r.lo = e.lo;
                    if(e.hi > r.hi) r.hi = e.hi;
                    r.und = r.und || e.und;
                }
                break;
            }
            default: throw std::logic_error("oracle: predicate node evaluated as expression");
        }
        val[std::size_t(id)] = r;
        stamp[std::size_t(id)] = epoch;
        return r;
    }

    static IB less(const Iv<T>& a, const Iv<T>& b) {
        return {!a.und && !b.und && a.hi < b.lo, a.und || b.und || a.lo < b.hi};
    }
    static IB notb(IB x) { return {!x.ub, !x.lb}; }

    IB evalp(int id) {
        const auto& n = L.nodes[std::size_t(id)];
        if(n.lb == n.ub) return {n.lb != 0, n.ub != 0};     // decided at compile time
        if(stamp[std::size_t(id)] == epoch) return pval[std::size_t(id)];
        IB r{false, true};
        switch(n.op) {
            case NodeOp::Lt: r = less(eval(n.ch[0]), eval(n.ch[1])); break;
            case NodeOp::Gt: r = less(eval(n.ch[1]), eval(n.ch[0])); break;
            case NodeOp::Le: r = notb(less(eval(n.ch[1]), eval(n.ch[0]))); break;
            case NodeOp::Ge: r = notb(less(eval(n.ch[0]), eval(n.ch[1]))); break;
            case NodeOp::Eq: case NodeOp::Ne: {
                Iv<T> a = eval(n.ch[0]), b = eval(n.ch[1]);
                bool ov = !(a.hi < b.lo) && !(b.hi < a.lo);
                r = {!a.und && !b.und && a.lo == a.hi && b.lo == b.hi && a.lo == b.lo, a.und || b.und || ov};
                if(n.op == NodeOp::Ne) r = notb(r);
                break;
            }
            case NodeOp::OrSeq: case NodeOp::Or: {
                r = {false, false};
                for(int c : n.ch) {
                    IB v = evalp(c);
                    if(n.op == NodeOp::OrSeq && v.lb) { r = {true, true}; break; }
                    r.lb = r.lb || v.lb; r.ub = r.ub || v.ub;
                }
                break;
            }
            case NodeOp::AndSeq: case NodeOp::And: {
                r = {true, true};
                for(int c : n.ch) {
                    IB v = evalp(c);
                    if(n.op == NodeOp::AndSeq && !v.ub) { r = {false, false}; break; }
                    r.lb = r.lb && v.lb; r.ub = r.ub && v.ub;
                }
                break;
            }
            case NodeOp::Not: r = notb(evalp(n.ch[0])); break;
            case NodeOp::BoolConst: r = {n.lb != 0, n.ub != 0}; break;
            default: throw std::logic_error("oracle: expression node evaluated as predicate");
        }
        pval[std::size_t(id)] = r;
        stamp[std::size_t(id)] = epoch;
        return r;
    }
};

enum BoundID { NONE = 0, LB = 1, UB = 2, BOTH = 3, EMPTY = 4 };

/// The constraints of each row in the engine's evaluation order (the code generator's row_order): repeatedly the
/// constraint whose not yet evaluated nodes weigh least (square root and quotient 12, arc cosine 40, product 2,
/// integer power 3, other operations 1, arguments and constants 0; ties in table order). A row holds iff every
/// constraint holds, so the order changes no result, only the work done before the first refuted constraint.
std::vector<std::vector<int>> device_row_order(const LemmaIR& L) {
    auto weight = [&](std::size_t nid) {
        switch(L.nodes[nid].op) {
            case NodeOp::Arg: case NodeOp::Const: case NodeOp::BoolConst: return 0;
            case NodeOp::Sqrt: case NodeOp::Div: return 12;
            case NodeOp::Acos: return 40;
            case NodeOp::Mul: return 2;
            case NodeOp::Pow: return 3;
            default: return 1;
        }
    };
    std::vector<std::vector<int>> out(L.rows.size());
    for(std::size_t r = 0; r < L.rows.size(); ++r) {
        const std::vector<int>& cons = L.rows[r];
        std::vector<std::vector<char>> in(cons.size(), std::vector<char>(L.nodes.size(), 0));
        for(std::size_t c = 0; c < cons.size(); ++c) {
            std::vector<int> stack{L.constraints[std::size_t(cons[c])]};
            while(!stack.empty()) {
                const int nid = stack.back();
                stack.pop_back();
                if(in[c][std::size_t(nid)]) continue;
                in[c][std::size_t(nid)] = 1;
                for(int ch : L.nodes[std::size_t(nid)].ch) stack.push_back(ch);
            }
        }
        std::vector<char> done(L.nodes.size(), 0), taken(cons.size(), 0);
        for(std::size_t k = 0; k < cons.size(); ++k) {
            std::size_t best = cons.size();
            long best_w = 0;
            for(std::size_t c = 0; c < cons.size(); ++c) {
                if(taken[c]) continue;
                long w = 0;
                for(std::size_t nid = 0; nid < L.nodes.size(); ++nid) if(in[c][nid] && !done[nid]) w += weight(nid);
                if(best == cons.size() || w < best_w) { best = c; best_w = w; }
            }
            taken[best] = 1;
            out[r].push_back(cons[best]);
            for(std::size_t nid = 0; nid < L.nodes.size(); ++nid) if(in[best][nid]) done[nid] = 1;
        }
    }
    return out;
}

// the oracle tests each row in the reference's table order unless set_device_row_order(true) selects the
// engine's order (the op-counting build uses it to count the engine's operations)
std::atomic<bool> g_device_row_order{false};

template<class T> struct Prover {
    const LemmaIR& L;
    Evaluator<T> ev;
    int nb;
    std::vector<std::vector<int>> rows;   // constraint ids of each row, in the order they are tested
    // propagation state (IndexQueueSet + IteratedRecursivePropInfo)
    std::vector<int> ring;
    std::vector<char> present, unstable;
    std::vector<std::uint8_t> rec;
    std::vector<int> unstable_list;
    std::size_t qb = 0, qe = 0, qn = 0;

    explicit Prover(const LemmaIR& l) : L(l), ev(l), nb(int(l.bounds.size())),
        rows(g_device_row_order.load() ? device_row_order(l) : l.rows),
        ring(std::size_t(std::max(nb, 1))), present(std::size_t(std::max(nb, 1)), 0),
        unstable(std::size_t(std::max(nb, 1)), 0), rec(std::size_t(std::max(nb, 1)), 0) {}

    int apply_bound(int k, Iv<T>* box) {
        const auto& b = L.bounds[std::size_t(k)];
        ev.begin(box);
        Iv<T> v = ev.eval(b.fn);
        if(!b.defined && v.und) return NONE;
        Iv<T>& t = box[b.target];
        if(b.dir == 1) {
            if(v.hi < t.hi) { t.hi = v.hi; return v.hi < t.lo ? EMPTY : UB; }
            return NONE;
        }
        if(b.dir == 2) {
            if(v.lo > t.lo) { t.lo = v.lo; return v.lo > t.hi ? EMPTY : LB; }
            return NONE;
        }
        int ch = NONE;
        if(v.hi < t.hi) { t.hi = v.hi; ch |= UB; }
        if(v.lo > t.lo) { t.lo = v.lo; ch |= LB; }
        if(t.hi < t.lo) return EMPTY;
        return ch;
    }

    bool enqueue(int a) {
        if(present[std::size_t(a)]) return false;
        present[std::size_t(a)] = 1;
        ring[qe] = a;
        if(++qe >= std::size_t(nb)) qe = 0;
        ++qn;
        return true;
    }
    int dequeue() {
        int a = ring[qb];
        present[std::size_t(a)] = 0;
        if(++qb >= std::size_t(nb)) qb = 0;
        --qn;
        return a;
    }
    void clear_info() {
        std::fill(rec.begin(), rec.end(), std::uint8_t(0));
        std::fill(unstable.begin(), unstable.end(), char(0));
        unstable_list.clear();
    }

    /// Returns true if the box became empty.
    bool propagate(int arg, Iv<T>* box, std::size_t it_limit, unsigned rec_limit) {
        if(nb == 0) return false;
        const auto& seed = L.upd_both[std::size_t(arg)];
        if(seed.empty()) return false;
        qb = qe = qn = 0;
        std::fill(present.begin(), present.end(), char(0));
        clear_info();
        for(int a : seed) enqueue(a);
        for(std::size_t i = 0; i < it_limit; ++i) {
            while(qn > 0) {
                int k = dequeue();
                int r = apply_bound(k, box);
                if(r == EMPTY) return true;
                const std::vector<int>* upd = nullptr;
                int tgt = L.bounds[std::size_t(k)].target;
                if(r == LB) upd = &L.upd_lb[std::size_t(tgt)];
                else if(r == UB) upd = &L.upd_ub[std::size_t(tgt)];
                else if(r == BOTH) upd = &L.upd_both[std::size_t(tgt)];
                if(!upd) continue;
                for(int a : *upd) {
                    if(rec[std::size_t(a)] >= rec_limit) {
                        if(!present[std::size_t(a)] && !unstable[std::size_t(a)]) {
                            unstable_list.push_back(a);
                            unstable[std::size_t(a)] = 1;
                        }
                    } else if(enqueue(a)) {
                        rec[std::size_t(a)] += 1;
                    }
                }
            }
            if(!unstable_list.empty()) {
                std::vector<int> u = unstable_list;
                for(int a : u) enqueue(a);
                clear_info();
            } else {
                break;
            }
        }
        return false;
    }

    /// True if every constraint of rows [r0, r1) is possibly satisfied.
    bool rows_ok(int r0, int r1, const Iv<T>* box) {
        ev.begin(box);
        for(int r = r0; r < r1; ++r) {
            for(int ci : rows[std::size_t(r)]) {
                if(!ev.evalp(L.constraints[std::size_t(ci)]).ub) return false;
            }
        }
        return true;
    }
    bool all_ok(const Iv<T>* box) { return rows_ok(L.nargs - 1, L.nargs, box); }
};

/// The provers one worker uses: the lemma's own number type, and for double lemmas in the precision form
/// a float prover that tries to refute each child first.
template<class T> struct Provers {
    Prover<T> P;
    std::unique_ptr<Prover<float>> F;
    Provers(const LemmaIR& l, bool fp32_first) : P(l) {
        if(fp32_first && std::is_same<T, double>::value) F.reset(new Prover<float>(l));
    }
};

template<class T> inline void split_point_pair(T lb, T ub, int n, int i, T& lo, T& hi) {
    T w = (ub - lb) / T(n);
    lo = (i >= n) ? ub : lb + T(i) * w;
    hi = (i + 1 >= n) ? ub : lb + T(i + 1) * w;
}

template<class T> struct Element {
    std::vector<Iv<T>> box;
    unsigned depth = 0;
};

template<class T> std::vector<Iv<T>> initial_box(const LemmaIR& L) {
    std::vector<Iv<T>> box(std::size_t(L.nargs));
    for(int i = 0; i < L.nargs; ++i) {
        std::int64_t l = L.ct_lb[std::size_t(i)], u = L.ct_ub[std::size_t(i)];
        // fixed point / 1e6, rounded outward (the ambient mode is round-down; casts round down too)
        double dl = l <= FXMIN ? -inf<double>() : double(l) / double(FX_ONE);
        double du = u >= FXMAX ? inf<double>() : -(double(-u) / double(FX_ONE));
        box[std::size_t(i)] = {T(dl), -T(-du), false};
    }
    Prover<T> P(L);
    for(int round = 0; round < 50 * L.nargs; ++round) {
        for(int k = 0; k < int(L.bounds.size()); ++k) {
            if(P.apply_bound(k, box.data()) == EMPTY) break;
        }
    }
    return box;
}

template<class T> struct Driver {
    const LemmaIR& L;
    ProveOptions opt;
    std::vector<sid::IrSplit> dyn, stat;
    std::vector<Element<T>> queue;
    std::mutex mtx;
    std::condition_variable cv;
    int busy = 0;
    Counts total;
    std::vector<double> criticals;
    std::exception_ptr error;

    Driver(const LemmaIR& l, const ProveOptions& o) : L(l), opt(o), dyn(l.dynamic_splits()), stat(l.static_splits()) {}

    void init(Provers<T>& S, Counts& c) {
        std::vector<Iv<T>> root = initial_box<T>(L);
        const std::size_t n = std::size_t(L.nargs);
        const unsigned rec_limit = unsigned(std::min<std::size_t>(n, 255));
        std::vector<Element<T>> out;
        std::vector<Iv<T>> cur = root;
        init_rec(S, c, 0, cur, rec_limit, out);
        queue = std::move(out);
    }

    /// Precision form: true if the float evaluation of child i of `parent` split n ways on `arg` already
    /// refutes it: the parent box rounded outward to float, the split variable's child range formed in
    /// float from RD(lb), RU(lb), RD(w), RU(w), RU(ub) with w = (ub - lb) / n in double (a float range
    /// that contains the double child range: lo = RD(RD(lb) + RD(i*RD(w))), hi = RU(RU(lb) + RU((i+1)*RU(w))),
    /// the last child ending at RU(ub)), then the same propagation and constraint rows as the double path.
    bool refuted_in_fp32(Provers<T>& S, Counts& c, const std::vector<Iv<T>>& parent, int arg, int i, int n,
                         std::size_t it, unsigned rec, int r0, int r1, std::size_t level) {
        if(!S.F) return false;
        if(level < 32 && !((opt.fp32_level_mask >> level) & 1u)) return false;   // level without the float pass
        std::vector<Iv<float>>& fb = fbox;
        fb.resize(parent.size());
        // the ambient rounding mode is downward: a cast rounds down, -cast(-x) rounds up
        for(std::size_t v = 0; v < parent.size(); ++v) {
            fb[v] = {static_cast<float>(parent[v].lo), -static_cast<float>(-parent[v].hi), false};
        }
        {
            const T lb = parent[std::size_t(arg)].lo, ub = parent[std::size_t(arg)].hi;
            const T w = (ub - lb) / T(n);
            const float lb_lo = static_cast<float>(lb), lb_hi = -static_cast<float>(-lb);
            const float w_lo = static_cast<float>(w), w_hi = -static_cast<float>(-w);
            const float ub_hi = -static_cast<float>(-ub);
            const float lo = lb_lo + float(i) * w_lo;
            const float hi = (i + 1 >= n) ? ub_hi : -((-lb_hi) - (-(-float(i + 1) * w_hi)));
            fb[std::size_t(arg)] = {lo, hi, false};
        }
        const bool noprop = level < 32 && ((opt.fp32_noprop_mask >> level) & 1u);
        bool refuted = (!noprop && S.F->propagate(arg, fb.data(), it, rec)) ||
                       (r1 > r0 && !S.F->rows_ok(r0, r1, fb.data()));
        if(refuted) ++c.fp32_refuted; else ++c.escalated;
        return refuted;
    }
    static thread_local std::vector<Iv<float>> fbox;

    void init_rec(Provers<T>& S, Counts& c, std::size_t d, const std::vector<Iv<T>>& box, unsigned rec_limit,
                  std::vector<Element<T>>& out) {
        Prover<T>& P = S.P;
        if(d == dyn.size()) {
            if(P.all_ok(box.data())) out.push_back({box, 0}); else ++c.leaves;
            return;
        }
        const auto& s = dyn[d];
        int m = int(s.initial);
        // sharding: the root's first split keeps only this part's children, and (as on the device) runs
        // without the float pass
        const bool sharded = d == 0 && opt.part_count > 1;
        for(int i = 0; i < m; ++i) {
            if(sharded && std::uint32_t(i) % opt.part_count != opt.part_index) continue;
            ++c.cuboids;
            std::vector<Iv<T>> child = box;
            T lo, hi;
            split_point_pair(box[std::size_t(s.arg)].lo, box[std::size_t(s.arg)].hi, m, i, lo, hi);
            child[std::size_t(s.arg)] = {lo, hi, false};
            if(!sharded && refuted_in_fp32(S, c, box, s.arg, i, m, 2 * std::size_t(L.nargs), rec_limit,
                               d + 1 == dyn.size() ? L.nargs - 1 : 0, d + 1 == dyn.size() ? L.nargs : 0, d)) {
                ++c.leaves;
                continue;
            }
            if(P.propagate(s.arg, child.data(), 2 * L.nargs, rec_limit)) { ++c.leaves; continue; }
            init_rec(S, c, d + 1, child, rec_limit, out);
        }
    }

    struct Hull {
        std::vector<Iv<T>> box;
        bool empty = true;
    };

    /// Static-split recursion (CPUProverCore::p_handle_cuboid).
    void handle(Provers<T>& S, Counts& c, std::size_t j, std::vector<Iv<T>>& box, Hull* hull) {
        Prover<T>& P = S.P;
        if(j == stat.size()) {
            ++c.leaves;
            if(hull) {
                if(hull->empty) { hull->box = box; hull->empty = false; }
                else {
                    for(std::size_t v = 0; v < box.size(); ++v) {
                        if(box[v].lo < hull->box[v].lo) hull->box[v].lo = box[v].lo;
                        if(box[v].hi > hull->box[v].hi) hull->box[v].hi = box[v].hi;
                    }
                }
            } else {
                ++c.criticals;
                std::lock_guard<std::mutex> g(crit_mtx);
                if(criticals.size() / (2 * box.size()) < opt.max_criticals) {
                    for(const auto& iv : box) { criticals.push_back(double(iv.lo)); criticals.push_back(double(iv.hi)); }
                }
            }
            return;
        }
        const auto& s = stat[j];
        int m = int(s.subdivisions);
        int r0 = s.arg;
        int r1 = (j + 1 < stat.size()) ? stat[j + 1].arg : L.nargs;
        T plo = box[std::size_t(s.arg)].lo, phi = box[std::size_t(s.arg)].hi;
        std::vector<Iv<T>> child;
        for(int i = 0; i < m; ++i) {
            child = box;
            T lo, hi;
            split_point_pair(plo, phi, m, i, lo, hi);
            child[std::size_t(s.arg)] = {lo, hi, false};
            if(refuted_in_fp32(S, c, box, s.arg, i, m, std::size_t(L.nargs), 4, r0, r1, dyn.size() + j)) {
                ++c.leaves;
                continue;
            }
            if(P.propagate(s.arg, child.data(), std::size_t(L.nargs), 4)) { ++c.leaves; continue; }
            if(!P.rows_ok(r0, r1, child.data())) { ++c.leaves; continue; }
            handle(S, c, j + 1, child, hull);
        }
        c.cuboids += std::uint64_t(m);
    }

    bool should_iterate(const std::vector<Iv<T>>& nw, const std::vector<Iv<T>>& old) const {
        const T single = T(opt.iteration_single), vol = T(opt.iteration_volume);
        for(std::size_t i = 0; i < nw.size(); ++i) {
            T mnw = nw[i].lo - nw[i].hi, mow = old[i].lo - old[i].hi;
            if(mow * single > mnw) return true;
        }
        T mnv = nw[0].lo - nw[0].hi, mov = old[0].lo - old[0].hi;
        for(std::size_t i = 1; i < nw.size(); ++i) {
            mnv *= (nw[i].hi - nw[i].lo);
            mov *= (old[i].hi - old[i].lo);
        }
        return mov * vol > mnv;
    }

    /// Dynamic re-split of a hull (SplitIntoImpl::perform_split).
    void split_rec(Provers<T>& S, Counts& c, std::size_t d, const std::vector<Iv<T>>& box, unsigned depth,
                   std::vector<Element<T>>& out) {
        Prover<T>& P = S.P;
        if(d == dyn.size()) {
            if(P.all_ok(box.data())) out.push_back({box, depth}); else ++c.leaves;
            return;
        }
        const auto& s = dyn[d];
        int m = int(s.subdivisions);
        const unsigned rec_limit = unsigned(std::min(L.nargs, 32));
        for(int i = 0; i < m; ++i) {
            ++c.cuboids;
            std::vector<Iv<T>> child = box;
            T lo, hi;
            split_point_pair(box[std::size_t(s.arg)].lo, box[std::size_t(s.arg)].hi, m, i, lo, hi);
            child[std::size_t(s.arg)] = {lo, hi, false};
            if(refuted_in_fp32(S, c, box, s.arg, i, m, 2 * std::size_t(L.nargs), rec_limit,
                               d + 1 == dyn.size() ? L.nargs - 1 : 0, d + 1 == dyn.size() ? L.nargs : 0, d)) {
                ++c.leaves;
                continue;
            }
            if(P.propagate(s.arg, child.data(), 2 * L.nargs, rec_limit)) { ++c.leaves; continue; }
            split_rec(S, c, d + 1, child, depth, out);
        }
    }

    void process(Provers<T>& S, Counts& c, Element<T> e, std::vector<Element<T>>& out) {
        int it = 0;
        for(;;) {
            Hull h;
            handle(S, c, 0, e.box, &h);
            if(h.empty) return;
            if(++it >= opt.max_iterations || !should_iterate(h.box, e.box)) {
                if(e.depth >= opt.generations) {
                    handle(S, c, 0, h.box, nullptr);
                } else {
                    split_rec(S, c, 0, h.box, e.depth + 1, out);
                }
                return;
            }
            ++c.repeated;
            ++c.cuboids;
            e.box = h.box;
        }
    }

    void worker() {
        try {
            RoundDownScope rd;
            Provers<T> S(L, opt.fp32_first);
            Counts c;
            std::vector<Element<T>> batch, out;
            for(;;) {
                {
                    std::unique_lock<std::mutex> lk(mtx);
                    cv.wait(lk, [&] { return !queue.empty() || busy == 0 || error; });
                    if(error || (queue.empty() && busy == 0)) break;
                    std::size_t take = std::min<std::size_t>(queue.size(), 32);
                    batch.assign(std::make_move_iterator(queue.end() - std::ptrdiff_t(take)), std::make_move_iterator(queue.end()));
                    queue.resize(queue.size() - take);
                    ++busy;
                }
                out.clear();
                for(auto& e : batch) process(S, c, std::move(e), out);
                {
                    std::lock_guard<std::mutex> lk(mtx);
                    for(auto& e : out) queue.push_back(std::move(e));
                    --busy;
                }
                cv.notify_all();
            }
            std::lock_guard<std::mutex> lk(mtx);
            total += c;
        } catch(...) {
            std::lock_guard<std::mutex> lk(mtx);
            if(!error) error = std::current_exception();
            cv.notify_all();
        }
    }

    ProveResult run() {
        auto t0 = std::chrono::steady_clock::now();
        {
            RoundDownScope rd;
            Provers<T> S(L, opt.fp32_first);
            Counts c;
            init(S, c);
            total += c;
        }
        int nt = opt.threads > 0 ? opt.threads : int(std::max(1u, std::thread::hardware_concurrency()));
        std::vector<std::thread> th;
        for(int i = 0; i < nt; ++i) th.emplace_back([this] { worker(); });
        for(auto& t : th) t.join();
        if(error) std::rethrow_exception(error);
        ProveResult r;
        r.counts = total;
        r.criticals = std::move(criticals);
        r.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        return r;
    }

    std::mutex crit_mtx;
};

template<class T> thread_local std::vector<Iv<float>> Driver<T>::fbox;

} // namespace

ProveResult prove(const std::string& ir, const ProveOptions& opt) {
    LemmaIR L = sid::parse_lemma_ir(ir);
    if(L.numtype == "f32") { Driver<float> d(L, opt); return d.run(); }
    Driver<double> d(L, opt);
    return d.run();
}

std::vector<double> root_box(const std::string& ir) {
    LemmaIR L = sid::parse_lemma_ir(ir);
    std::vector<double> r;
    RoundDownScope rd;
    if(L.numtype == "f32") {
        for(const auto& iv : initial_box<float>(L)) { r.push_back(iv.lo); r.push_back(iv.hi); }
    } else {
        for(const auto& iv : initial_box<double>(L)) { r.push_back(iv.lo); r.push_back(iv.hi); }
    }
    return r;
}

namespace {

/// The expressions compared by the constraints' comparison nodes that are not decided at compile time:
/// constraints in table order, each predicate tree in pre-order, (left, right) per comparison, every
/// comparison node once.
std::vector<int> comparison_operands(const LemmaIR& L) {
    std::vector<int> out;
    std::vector<char> seen(L.nodes.size(), 0);
    std::vector<int> stack;
    for(int root : L.constraints) {
        stack.assign(1, root);
        while(!stack.empty()) {
            const int id = stack.back();
            stack.pop_back();
            if(seen[std::size_t(id)]) continue;
            seen[std::size_t(id)] = 1;
            const auto& nd = L.nodes[std::size_t(id)];
            if(nd.lb == nd.ub) continue;   // decided at compile time
            switch(nd.op) {
                case NodeOp::Lt: case NodeOp::Le: case NodeOp::Gt: case NodeOp::Ge: case NodeOp::Eq: case NodeOp::Ne:
                    out.push_back(nd.ch[0]);
                    out.push_back(nd.ch[1]);
                    break;
                case NodeOp::OrSeq: case NodeOp::AndSeq: case NodeOp::Or: case NodeOp::And: case NodeOp::Not:
                    for(std::size_t k = nd.ch.size(); k-- > 0;) stack.push_back(nd.ch[k]);
                    break;
                default: break;
            }
        }
    }
    return out;
}

template<class T> void eval_operands_t(const LemmaIR& L, const std::vector<int>& ops, const double* lo, const double* hi,
                                       std::uint64_t n, double* out, std::int8_t* und, int threads) {
    int nt = threads > 0 ? threads : int(std::max(1u, std::thread::hardware_concurrency()));
    std::atomic<std::uint64_t> next{0};
    std::exception_ptr err;
    std::mutex em;
    const std::size_t k = ops.size();
    auto work = [&] {
        try {
            RoundDownScope rd;
            Evaluator<T> ev(L);
            std::vector<Iv<T>> box(std::size_t(L.nargs));
            for(;;) {
                std::uint64_t b = next.fetch_add(256);
                if(b >= n) break;
                for(std::uint64_t i = b; i < std::min<std::uint64_t>(n, b + 256); ++i) {
                    for(int v = 0; v < L.nargs; ++v) {
                        const double l = lo[std::uint64_t(v) * n + i], h = hi[std::uint64_t(v) * n + i];
                        box[std::size_t(v)] = {static_cast<T>(l), -static_cast<T>(-h), false};   // outward
                    }
                    ev.begin(box.data());
                    for(std::size_t j = 0; j < k; ++j) {
                        Iv<T> r = ev.eval(ops[j]);
                        out[(i * k + j) * 2] = double(r.lo);
                        out[(i * k + j) * 2 + 1] = double(r.hi);
                        und[i * k + j] = r.und ? 1 : 0;
                    }
                }
            }
        } catch(...) {
            std::lock_guard<std::mutex> g(em);
            if(!err) err = std::current_exception();
        }
    };
    std::vector<std::thread> th;
    for(int t = 0; t < nt; ++t) th.emplace_back(work);
    for(auto& t : th) t.join();
    if(err) std::rethrow_exception(err);
}

} // namespace

void count_ops(unsigned long long out[10]) {
#ifdef SIDO_COUNT_OPS
    for(int k = 0; k < 10; ++k) out[k] = g_ops[k].exchange(0);
#else
    throw std::runtime_error("oracle: built without SIDO_COUNT_OPS");
#endif
}

void set_device_row_order(bool on) { g_device_row_order.store(on); }

std::vector<std::vector<int>> device_row_order(const std::string& ir) {
    return device_row_order(sid::parse_lemma_ir(ir));
}

std::vector<int> operand_nodes(const std::string& ir) {
    return comparison_operands(sid::parse_lemma_ir(ir));
}

void eval_operands(const std::string& ir, const double* lo, const double* hi, std::uint64_t n, bool use_float,
                   double* out, std::int8_t* und, int threads) {
    LemmaIR L = sid::parse_lemma_ir(ir);
    const std::vector<int> ops = comparison_operands(L);
    if(use_float) eval_operands_t<float>(L, ops, lo, hi, n, out, und, threads);
    else eval_operands_t<double>(L, ops, lo, hi, n, out, und, threads);
}

void eval_batch(const std::string& ir, const double* lo, const double* hi, std::uint64_t n,
                double* out_lo, double* out_hi, std::int8_t* verdict, int threads, bool float_rows_first) {
    LemmaIR L = sid::parse_lemma_ir(ir);
    if(L.numtype != "f64") throw std::invalid_argument("oracle eval_batch supports f64 lemmas");
    int nt = threads > 0 ? threads : int(std::max(1u, std::thread::hardware_concurrency()));
    std::atomic<std::uint64_t> next{0};
    std::exception_ptr err;
    std::mutex em;
    auto work = [&] {
        try {
            RoundDownScope rd;
            Prover<double> P(L);
            Prover<float> F(L);
            std::vector<Iv<double>> box(std::size_t(L.nargs));
            std::vector<Iv<float>> fbox(std::size_t(L.nargs));
            const int last = L.nargs - 1;
            for(;;) {
                std::uint64_t b = next.fetch_add(4096);
                if(b >= n) break;
                std::uint64_t e = std::min<std::uint64_t>(n, b + 4096);
                for(std::uint64_t i = b; i < e; ++i) {
                    for(int v = 0; v < L.nargs; ++v) box[std::size_t(v)] = {lo[std::uint64_t(v) * n + i], hi[std::uint64_t(v) * n + i], false};
                    std::int8_t vd = 0;
                    if(P.propagate(last, box.data(), std::size_t(L.nargs), 4)) {
                        vd = 1;
                    } else if(float_rows_first) {
                        // the device's order: rows in float on the box rounded outward (round-down mode: a
                        // cast rounds down, -cast(-x) up), in double only where float does not refute
                        for(int v = 0; v < L.nargs; ++v) {
                            const auto& b = box[std::size_t(v)];
                            fbox[std::size_t(v)] = {static_cast<float>(b.lo), -static_cast<float>(-b.hi), false};
                        }
                        if(!F.all_ok(fbox.data()) || !P.all_ok(box.data())) vd = 2;
                    } else if(!P.all_ok(box.data())) {
                        vd = 2;
                    }
                    verdict[i] = vd;
                    for(int v = 0; v < L.nargs; ++v) {
                        out_lo[std::uint64_t(v) * n + i] = box[std::size_t(v)].lo;
                        out_hi[std::uint64_t(v) * n + i] = box[std::size_t(v)].hi;
                    }
                }
            }
        } catch(...) {
            std::lock_guard<std::mutex> g(em);
            if(!err) err = std::current_exception();
        }
    };
    std::vector<std::thread> th;
    for(int i = 0; i < nt; ++i) th.emplace_back(work);
    for(auto& t : th) t.join();
    if(err) std::rethrow_exception(err);
}

} // namespace sido
