// Compile-time bounds in fixed-point arithmetic (denominator 10^6).
//
// ivarp decides simplifications, pruned constraints, sign-specialised interval
// operations and the propagation update lists from conservative fixed-point
// bounds of every subexpression (ivarp/include/ivarp/number/fixed_point_bounds.hpp,
// fixed_point_bounds_impl.hpp, fixed_point_bounds_sqrt.hpp). Because these bounds
// change which cuboids are pruned, the same integer arithmetic (saturation,
// directed rounding, bisection square roots) is restated here so that the
// compiled tables are identical.
#pragma once

#include <cstdint>
#include <algorithm>

namespace ivarp {
namespace sid_fe {
namespace fxp {

using i64 = std::int64_t;
using u64 = std::uint64_t;

constexpr i64 denom = 1000000;
constexpr i64 max_bound = INT64_C(9223372036854775807);   // +inf
constexpr i64 min_bound = -max_bound;                     // -inf
constexpr i64 fp_maxint = INT64_C(9223372036854);

inline bool is_lb(i64 lb) { return lb > min_bound; }
inline bool is_ub(i64 ub) { return ub < max_bound; }
inline bool is_finite(i64 l, i64 u) { return l > min_bound && u < max_bound; }

/// Saturating unsigned addition (values are non-negative fixed-point numbers).
inline i64 uadd(u64 a, u64 b) {
    return (a + b >= u64(max_bound)) ? max_bound : i64(a + b);
}

inline i64 add(i64 a, i64 b) {
    if(a < 0 && b < 0) return -uadd(u64(-a), u64(-b));
    if(a > 0 && b > 0) return uadd(u64(a), u64(b));
    return a + b;
}

inline i64 add_rd(i64 a, i64 b) { return (a <= min_bound || b <= min_bound) ? min_bound : add(a, b); }
inline i64 add_ru(i64 a, i64 b) { return (a >= max_bound || b >= max_bound) ? max_bound : add(a, b); }

inline i64 sat_umul(u64 a, u64 b) {
    if(b == 0) return 0;
    if(a > u64(max_bound) / b) return max_bound;
    return i64(a * b);
}

inline i64 int_to_fp(i64 v) {
    return v < 0 ? -sat_umul(u64(-v), u64(denom)) : sat_umul(u64(v), u64(denom));
}

/// |a| * |b| with the fractional cross term rounded down (up=false) or up (up=true).
inline i64 do_mul(i64 a, i64 b, bool up) {
    i64 ia = a / denom, ib = b / denom, fa = a % denom, fb = b % denom;
    i64 ip = sat_umul(u64(sat_umul(u64(ia), u64(ib))), u64(denom));
    i64 f1 = uadd(u64(sat_umul(u64(ia), u64(fb))), u64(sat_umul(u64(ib), u64(fa))));
    i64 f2 = (fa * fb) / denom + ((up && (fa * fb) % denom != 0) ? 1 : 0);
    return uadd(u64(uadd(u64(ip), u64(f1))), u64(f2));
}

inline i64 iabs(i64 v) { return v < 0 ? -v : v; }

inline i64 mul_rd(i64 a, i64 b) {
    return ((a < 0) != (b < 0)) ? -do_mul(iabs(a), iabs(b), true) : do_mul(iabs(a), iabs(b), false);
}
inline i64 mul_ru(i64 a, i64 b) {
    return ((a < 0) != (b < 0)) ? -do_mul(iabs(a), iabs(b), false) : do_mul(iabs(a), iabs(b), true);
}

/// floor(a * 10^6 / b) (+1 if inexact and round_up), saturating at max_bound; a, b >= 0.
inline i64 long_div(u64 a, u64 b, bool round_up) {
    unsigned __int128 n = (unsigned __int128)a * (unsigned __int128)u64(denom);
    unsigned __int128 q = n / b;
    unsigned __int128 r = n % b;
    if(q >= (unsigned __int128)u64(max_bound)) return max_bound;
    return i64(u64(q)) + ((round_up && r != 0) ? 1 : 0);
}

inline i64 do_div_rd(i64 a, i64 b) { return (b >= max_bound) ? 0 : long_div(u64(a), u64(b), false); }
inline i64 do_div_ru(i64 a, i64 b) {
    return (b == 0 || a >= max_bound) ? max_bound : long_div(u64(a), u64(b), true);
}

inline i64 div_rd(i64 a, i64 b) {
    return ((a < 0) != (b < 0)) ? -do_div_ru(iabs(a), iabs(b)) : do_div_rd(iabs(a), iabs(b));
}
inline i64 div_ru(i64 a, i64 b) {
    return ((a < 0) != (b < 0)) ? -do_div_rd(iabs(a), iabs(b)) : do_div_ru(iabs(a), iabs(b));
}

inline i64 iv_mul_lb(i64 la, i64 ua, i64 lb, i64 ub) {
    if((!is_lb(la) && ub > 0) || (!is_lb(lb) && ua > 0)) return min_bound;
    if((!is_ub(ua) && lb < 0) || (!is_ub(ub) && la < 0)) return min_bound;
    i64 r1 = mul_rd(la, lb), r2 = mul_rd(la, ub), r3 = mul_rd(ua, lb), r4 = mul_rd(ua, ub);
    return std::min(std::min(r1, r2), std::min(r3, r4));
}

inline i64 iv_mul_ub(i64 la, i64 ua, i64 lb, i64 ub) {
    if((!is_ub(ua) && ub > 0) || (!is_ub(ub) && ua > 0)) return max_bound;
    if((!is_lb(la) && lb < 0) || (!is_lb(lb) && la < 0)) return max_bound;
    i64 r1 = mul_ru(la, lb), r2 = mul_ru(la, ub), r3 = mul_ru(ua, lb), r4 = mul_ru(ua, ub);
    return std::max(std::max(r1, r2), std::max(r3, r4));
}

inline i64 iv_div_lb(i64 la, i64 ua, i64 lb, i64 ub) {
    if((lb < 0 && ub > 0) || (lb == 0 && ub == 0)) return min_bound;
    if(la == 0 && ua == 0) return 0;
    if(lb == 0) return la < 0 ? min_bound : div_rd(la, ub);
    if(ub == 0) return ua > 0 ? min_bound : do_div_rd(-ua, -lb);
    if(lb > 0) return div_rd(la, la < 0 ? lb : ub);
    return div_rd(ua, ua > 0 ? ub : lb);
}

inline i64 iv_div_ub(i64 la, i64 ua, i64 lb, i64 ub) {
    if((lb < 0 && ub > 0) || (lb == 0 && ub == 0)) return max_bound;
    if(la == 0 && ua == 0) return 0;
    if(lb == 0) return ua > 0 ? max_bound : div_ru(ua, ub);
    if(ub == 0) return la < 0 ? max_bound : -do_div_ru(la, -lb);
    if(lb > 0) return div_ru(ua, ua < 0 ? ub : lb);
    return div_ru(la, la > 0 ? lb : ub);
}

inline i64 pow_lb(i64 lb, i64 ub, unsigned p) {
    if(!is_lb(lb) && !is_ub(ub)) return min_bound;
    if(p == 0) return int_to_fp(1);
    if(p % 2 == 1 && !is_lb(lb)) return min_bound;
    int sign = (p % 2 == 0) ? 1 : (lb < 0 ? -1 : 1);
    i64 op = (p % 2 == 0 && ub < 0) ? ub : ((p % 2 == 0 && lb < 0 && ub > 0) ? 0 : lb);
    op = op < 0 ? -op : op;
    i64 r = op;
    for(unsigned i = 1; i < p; ++i) r = sign > 0 ? mul_rd(r, op) : mul_ru(r, op);
    return r * sign;
}

inline i64 pow_ub(i64 lb, i64 ub, unsigned p) {
    if(!is_lb(lb) && !is_ub(ub)) return max_bound;
    if(p == 0) return int_to_fp(1);
    int sign = (p % 2 == 0) ? 1 : (ub < 0 ? -1 : 1);
    i64 op = (p % 2 == 0) ? std::max(-lb, ub) : ub;
    op = op < 0 ? -op : op;
    i64 r = op;
    for(unsigned i = 1; i < p; ++i) r = sign > 0 ? mul_ru(r, op) : mul_rd(r, op);
    return r * sign;
}

inline i64 sqrt_bisect_rd(i64 x, i64 lo, i64 hi) {
    while(hi - lo > 1) {
        i64 mid = (lo + hi) / 2;
        if(mul_ru(mid, mid) >= x) hi = mid; else lo = mid;
    }
    return mul_ru(hi, hi) == x ? hi : lo;
}

inline i64 sqrt_bisect_ru(i64 x, i64 lo, i64 hi) {
    while(hi - lo > 1) {
        i64 mid = (lo + hi) / 2;
        if(mul_rd(mid, mid) > x) hi = mid; else lo = mid;
    }
    return mul_rd(lo, lo) == x ? lo : hi;
}

inline i64 sqrt_rd(i64 x) {
    if(x == 0) return 0;
    if(x >= max_bound) return INT64_C(3037000499976);
    if(x < denom) return sqrt_bisect_rd(x, x, denom);
    if(x <= int_to_fp(16)) return sqrt_bisect_rd(x, x / 4, x);
    return sqrt_bisect_rd(x, 0, x / 4 + 1);
}

inline i64 sqrt_ru(i64 x) {
    if(x == 0) return 0;
    if(x >= max_bound) return max_bound;
    if(x < denom) return sqrt_bisect_ru(x, x, denom);
    if(x <= int_to_fp(16)) return sqrt_bisect_ru(x, x / 4, x);
    return sqrt_bisect_ru(x, 0, x / 4 + 1);
}

enum class Order { LT, LE, EQ, GE, GT, UNKNOWN };

inline Order iv_order(i64 la, i64 ua, i64 lb, i64 ub) {
    if(is_ub(ua) && is_lb(lb)) {
        if(ua < lb) return Order::LT;
        if(ua == lb) {
            if(is_ub(ub) && is_lb(la) && ub == la) return Order::EQ;
            return Order::LE;
        }
    }
    if(is_lb(la) && is_ub(ub)) {
        if(ub < la) return Order::GT;
        if(ub == la) return Order::GE;
    }
    return Order::UNKNOWN;
}

} // namespace fxp
} // namespace sid_fe
} // namespace ivarp
