// Outward-rounded interval arithmetic on the device (double and float).
//
// Every operation reproduces the reference's CPU results bit for bit: the
// reference runs in a global round-down FPU mode and obtains upper bounds with
// the sign trick, which equals IEEE round-up; here the directed-rounding
// intrinsics (__dadd_rd/__dadd_ru, __dmul_*, __ddiv_*, __dsqrt_* and the
// __f* counterparts) are used directly. The case analysis of multiplication,
// division and square root is selected by the operands' compile-time bounds,
// passed as template parameters by the generated lemma code:
//   NN = 1/0/-1: operand known non-negative / known not non-negative / test at run time,
//   NP likewise for non-positive, PS/NG for strictly positive/negative divisors.
// Reference: number/float_interval_addsub.hpp:53-102, float_interval_mul.hpp:55-164,
// float_interval_div.hpp:45-107, interval_div.hpp:113-288, math_fn/interval_sqrt.hpp:98-116,
// math_fn/fixed_pow.hpp:93-200, number/minmax.hpp:58-87, eval/if_then_else.hpp:64-81,
// number/interval_comparisons.hpp:32-119.
#pragma once

#include <cstdint>

namespace sid {

template<class T> struct Iv {
    T lo, hi;
    bool und;
};

struct IB {
    bool lb, ub;   // definitely, possibly
};

template<class T> struct Dir;

template<> struct Dir<double> {
    static __device__ __forceinline__ double add_rd(double a, double b) { return __dadd_rd(a, b); }
    static __device__ __forceinline__ double add_ru(double a, double b) { return __dadd_ru(a, b); }
    static __device__ __forceinline__ double sub_rd(double a, double b) { return __dsub_rd(a, b); }
    static __device__ __forceinline__ double sub_ru(double a, double b) { return __dsub_ru(a, b); }
    static __device__ __forceinline__ double mul_rd(double a, double b) { return __dmul_rd(a, b); }
    static __device__ __forceinline__ double mul_ru(double a, double b) { return __dmul_ru(a, b); }
    static __device__ __forceinline__ double div_rd(double a, double b) { return __ddiv_rd(a, b); }
    static __device__ __forceinline__ double div_ru(double a, double b) { return __ddiv_ru(a, b); }
    static __device__ __forceinline__ double sqrt_rd(double a) { return __dsqrt_rd(a); }
    static __device__ __forceinline__ double sqrt_ru(double a) { return __dsqrt_ru(a); }
    static __device__ __forceinline__ double inf() { return __longlong_as_double(0x7ff0000000000000ll); }
    static __device__ __forceinline__ bool signbit(double a) { return __double_as_longlong(a) < 0; }
    static __device__ __forceinline__ bool isfin(double a) { return (__double_as_longlong(a) & 0x7ff0000000000000ll) != 0x7ff0000000000000ll; }
};

template<> struct Dir<float> {
    static __device__ __forceinline__ float add_rd(float a, float b) { return __fadd_rd(a, b); }
    static __device__ __forceinline__ float add_ru(float a, float b) { return __fadd_ru(a, b); }
    static __device__ __forceinline__ float sub_rd(float a, float b) { return __fsub_rd(a, b); }
    static __device__ __forceinline__ float sub_ru(float a, float b) { return __fsub_ru(a, b); }
    static __device__ __forceinline__ float mul_rd(float a, float b) { return __fmul_rd(a, b); }
    static __device__ __forceinline__ float mul_ru(float a, float b) { return __fmul_ru(a, b); }
    static __device__ __forceinline__ float div_rd(float a, float b) { return __fdiv_rd(a, b); }
    static __device__ __forceinline__ float div_ru(float a, float b) { return __fdiv_ru(a, b); }
    static __device__ __forceinline__ float sqrt_rd(float a) { return __fsqrt_rd(a); }
    static __device__ __forceinline__ float sqrt_ru(float a) { return __fsqrt_ru(a); }
    static __device__ __forceinline__ float inf() { return __int_as_float(0x7f800000); }
    static __device__ __forceinline__ bool signbit(float a) { return __float_as_int(a) < 0; }
    static __device__ __forceinline__ bool isfin(float a) { return (__float_as_int(a) & 0x7f800000) != 0x7f800000; }
};

template<int K> __device__ __forceinline__ bool tri(bool runtime) { return K == 1 ? true : (K == 0 ? false : runtime); }

template<class T> __device__ __forceinline__ T nan0(T v, bool finite) { return (!finite && v != v) ? T(0) : v; }

template<class T> __device__ __forceinline__ Iv<T> iv_neg(const Iv<T>& a) { return {-a.hi, -a.lo, a.und}; }

template<class T> __device__ __forceinline__ Iv<T> iv_add(const Iv<T>& a, const Iv<T>& b) {
    return {Dir<T>::add_rd(a.lo, b.lo), Dir<T>::add_ru(a.hi, b.hi), a.und || b.und};
}

template<class T> __device__ __forceinline__ Iv<T> iv_sub(const Iv<T>& a, const Iv<T>& b) {
    return {Dir<T>::sub_rd(a.lo, b.hi), Dir<T>::sub_ru(a.hi, b.lo), a.und || b.und};
}

template<class T, bool FIN> __device__ __forceinline__ void do_mul(T l1, T l2, T u1, T u2, T& lo, T& hi) {
    lo = nan0(Dir<T>::mul_rd(l1, l2), FIN);
    hi = nan0(Dir<T>::mul_ru(u1, u2), FIN);
}

/// Product with the sign case analysis of ia_mul_check_signs.
template<class T, int NN1, int NP1, int NN2, int NP2, bool FIN>
__device__ __forceinline__ Iv<T> iv_mul(const Iv<T>& a, const Iv<T>& b) {
    T lo, hi;
    if(tri<NN1>(a.lo >= T(0))) {
        if(tri<NN2>(b.lo >= T(0))) do_mul<T, FIN>(a.lo, b.lo, a.hi, b.hi, lo, hi);
        else if(tri<NP2>(b.hi <= T(0))) do_mul<T, FIN>(a.hi, b.lo, a.lo, b.hi, lo, hi);
        else do_mul<T, FIN>(a.hi, b.lo, a.hi, b.hi, lo, hi);
    } else if(tri<NP1>(a.hi <= T(0))) {
        if(tri<NN2>(b.lo >= T(0))) do_mul<T, FIN>(a.lo, b.hi, a.hi, b.lo, lo, hi);
        else if(tri<NP2>(b.hi <= T(0))) do_mul<T, FIN>(a.hi, b.hi, a.lo, b.lo, lo, hi);
        else do_mul<T, FIN>(a.lo, b.hi, a.lo, b.lo, lo, hi);
    } else if(tri<NN2>(b.lo >= T(0))) {
        do_mul<T, FIN>(a.lo, b.hi, a.hi, b.hi, lo, hi);
    } else if(tri<NP2>(b.hi <= T(0))) {
        do_mul<T, FIN>(a.hi, b.lo, a.lo, b.lo, lo, hi);
    } else {
        T l1, h1, l2, h2;
        do_mul<T, FIN>(a.lo, b.hi, a.lo, b.lo, l1, h1);
        do_mul<T, FIN>(b.lo, a.hi, a.hi, b.hi, l2, h2);
        lo = (l2 <= l1) ? l2 : l1;
        hi = (h1 <= h2) ? h2 : h1;
    }
    return {lo, hi, a.und || b.und};
}

template<class T> __device__ __forceinline__ int sgnv(T v) { return (v > T(0)) - (v < T(0)); }

template<class T> __device__ __noinline__ void divide_by_zero(Iv<T>& num, const Iv<T>& den, int snl, int snu, int sds) {
    num.und = true;
    if(sds == 0 || snu - snl == 2) { num.lo = -Dir<T>::inf(); num.hi = Dir<T>::inf(); return; }
    if(sds > 0) {
        if(snl >= 0) { num.lo = Dir<T>::div_rd(num.lo, den.hi); num.hi = Dir<T>::inf(); }
        else { num.hi = Dir<T>::div_ru(num.hi, den.hi); num.lo = -Dir<T>::inf(); }
    } else {
        if(snl >= 0) { num.hi = Dir<T>::div_ru(num.lo, den.lo); num.lo = -Dir<T>::inf(); }
        else { num.lo = Dir<T>::div_rd(num.hi, den.lo); num.hi = Dir<T>::inf(); }
    }
}

template<class T> __device__ __forceinline__ T div_lb_inf(T n, int ni, T d, int di) {
    if(!ni && !di) return Dir<T>::div_rd(n, d);
    if(di != 0) return T(0);
    return -Dir<T>::inf();
}
template<class T> __device__ __forceinline__ T div_ub_inf(T n, int ni, T d, int di) {
    if(!ni && !di) return Dir<T>::div_ru(n, d);
    if(di != 0) return T(0);
    return Dir<T>::inf();
}

/// Division with infinite endpoints (divide_by_infinite of interval_div.hpp).
template<class T> __device__ __noinline__ Iv<T> divide_by_infinite(Iv<T> num, const Iv<T>& den) {
    int snl = sgnv(num.lo), snu = sgnv(num.hi), sdl = sgnv(den.lo), sdu = sgnv(den.hi);
    int inl = Dir<T>::isfin(num.lo) ? 0 : -1, inu = Dir<T>::isfin(num.hi) ? 0 : 1;
    int idl = Dir<T>::isfin(den.lo) ? 0 : -1, idu = Dir<T>::isfin(den.hi) ? 0 : 1;
    T nl = num.lo, nu = num.hi, dl = den.lo, du = den.hi;
    if(sdl > 0) {
        if(snl >= 0) { num.lo = div_lb_inf(nl, inl, du, idu); num.hi = div_ub_inf(nu, inu, dl, idl); }
        else if(snu <= 0) { num.lo = div_lb_inf(nl, inl, dl, idl); num.hi = div_ub_inf(nu, inu, du, idu); }
        else { num.lo = div_lb_inf(nl, inl, dl, idl); num.hi = div_ub_inf(nu, inu, dl, idl); }
    } else if(sdu < 0) {
        if(snl >= 0) { num.lo = div_lb_inf(nu, inu, du, idu); num.hi = div_ub_inf(nl, inl, dl, idl); }
        else if(snu <= 0) { num.lo = div_lb_inf(nu, inu, dl, idl); num.hi = div_ub_inf(nl, inl, du, idu); }
        else { num.lo = div_lb_inf(nu, inu, du, idu); num.hi = div_ub_inf(nl, inl, du, idu); }
    } else {
        divide_by_zero(num, den, snl, snu, sdl + sdu);
    }
    return num;
}

/// Quotient (ia_div with compile-time bounds of numerator and denominator).
template<class T, int NNn, int NPn, int PSd, int NGd, bool CTFIN>
__device__ __forceinline__ Iv<T> iv_div(Iv<T> num, const Iv<T>& den) {
    num.und = num.und || den.und;
    bool fin = CTFIN || (Dir<T>::isfin(num.lo) && Dir<T>::isfin(num.hi) && Dir<T>::isfin(den.lo) && Dir<T>::isfin(den.hi));
    if(!fin) return divide_by_infinite(num, den);
    T l, h;
    if(tri<PSd>(den.lo > T(0))) {
        if(tri<NNn>(num.lo >= T(0))) { l = Dir<T>::div_rd(num.lo, den.hi); h = Dir<T>::div_ru(num.hi, den.lo); }
        else if(tri<NPn>(num.hi <= T(0))) { l = Dir<T>::div_rd(num.lo, den.lo); h = Dir<T>::div_ru(num.hi, den.hi); }
        else { l = Dir<T>::div_rd(num.lo, den.lo); h = Dir<T>::div_ru(num.hi, den.lo); }
    } else if(tri<NGd>(den.hi < T(0))) {
        if(tri<NNn>(num.lo >= T(0))) { l = Dir<T>::div_rd(num.hi, den.hi); h = Dir<T>::div_ru(num.lo, den.lo); }
        else if(tri<NPn>(num.hi <= T(0))) { l = Dir<T>::div_rd(num.hi, den.lo); h = Dir<T>::div_ru(num.lo, den.hi); }
        else { l = Dir<T>::div_rd(num.hi, den.hi); h = Dir<T>::div_ru(num.lo, den.hi); }
    } else {
        divide_by_zero(num, den, sgnv(num.lo), sgnv(num.hi), sgnv(den.lo) + sgnv(den.hi));
        return num;
    }
    num.lo = l;
    num.hi = h;
    return num;
}

/// Square root with the reference's clamping of negative lower bounds.
template<class T, int NN> __device__ __forceinline__ Iv<T> iv_sqrt(const Iv<T>& x) {
    T lo = x.lo;
    bool und = x.und;
    if(!tri<NN>(x.lo >= T(0))) {
        if(x.hi < T(0)) return {-Dir<T>::inf(), Dir<T>::inf(), true};
        lo = T(0);
        und = true;
    }
    return {Dir<T>::sqrt_rd(lo), Dir<T>::sqrt_ru(x.hi), und};
}

/// square(x): general product (signs tested at run time) clamped below at 0.
template<class T> __device__ __forceinline__ Iv<T> iv_square(const Iv<T>& x) {
    Iv<T> r = iv_mul<T, -1, -1, -1, -1, false>(x, x);
    if(r.lo < T(0)) r.lo = T(0);
    return r;
}

/// Integer powers P >= 3 as computed by the reference's CPU path: two round-down lanes with the sign
/// bookkeeping of fixed_pow.hpp:93-126.
template<class T> __device__ __noinline__ Iv<T> pow_lanes(T lb, T ub, bool und, unsigned p, bool even) {
    T u = -ub;
    bool nl = Dir<T>::signbit(lb), nu = Dir<T>::signbit(u);
    T xl = lb, xu = u;
    T nxl = nl ? -xl : xl, nxu = nu ? -xu : xu;
    T yl = even ? T(1) : lb, yu = even ? T(-1) : u;
    for(p /= 2; p > 0; p /= 2) {
        xl = Dir<T>::mul_rd(xl, nxl);
        xu = Dir<T>::mul_rd(xu, nxu);
        nxl = nl ? -xl : xl;
        nxu = nu ? -xu : xu;
        if(p % 2) { yl = Dir<T>::mul_rd(yl, nxl); yu = Dir<T>::mul_rd(yu, nxu); }
    }
    return {yl, -yu, und};
}

template<class T, unsigned P> __device__ __forceinline__ Iv<T> iv_pow(const Iv<T>& x) {
    if(P == 0) return {T(1), T(1), x.und};
    if(P == 1) return x;
    if(P == 2) return iv_square(x);
    if(P % 2) return pow_lanes(x.lo, x.hi, x.und, P, false);
    if(x.hi < T(0)) return pow_lanes(-x.hi, -x.lo, x.und, P, true);
    if(x.lo < T(0)) {
        T a = fabs(x.lo), b = fabs(x.hi);
        return pow_lanes(T(0), a < b ? b : a, x.und, P, true);
    }
    return pow_lanes(x.lo, x.hi, x.und, P, true);
}

template<class T> __device__ __forceinline__ Iv<T> iv_min(const Iv<T>& a, const Iv<T>& b) {
    return {a.lo < b.lo ? a.lo : b.lo, a.hi < b.hi ? a.hi : b.hi, a.und || b.und};
}
template<class T> __device__ __forceinline__ Iv<T> iv_max(const Iv<T>& a, const Iv<T>& b) {
    return {b.lo < a.lo ? a.lo : b.lo, b.hi < a.hi ? a.hi : b.hi, a.und || b.und};
}

/// Join of both branches of an undecided if_then_else.
template<class T> __device__ __forceinline__ Iv<T> iv_join(Iv<T> t, const Iv<T>& e) {
    if(e.lo < t.lo) t.lo = e.lo;
    if(e.hi > t.hi) t.hi = e.hi;
    t.und = t.und || e.und;
    return t;
}

template<class T> __device__ __forceinline__ IB iv_less(const Iv<T>& a, const Iv<T>& b) {
    return {!a.und && !b.und && a.hi < b.lo, a.und || b.und || a.lo < b.hi};
}
__device__ __forceinline__ IB ib_not(IB x) { return {!x.ub, !x.lb}; }
template<class T> __device__ __forceinline__ IB iv_lt(const Iv<T>& a, const Iv<T>& b) { return iv_less(a, b); }
template<class T> __device__ __forceinline__ IB iv_gt(const Iv<T>& a, const Iv<T>& b) { return iv_less(b, a); }
template<class T> __device__ __forceinline__ IB iv_le(const Iv<T>& a, const Iv<T>& b) { return ib_not(iv_less(b, a)); }
template<class T> __device__ __forceinline__ IB iv_ge(const Iv<T>& a, const Iv<T>& b) { return ib_not(iv_less(a, b)); }
template<class T> __device__ __forceinline__ IB iv_eq(const Iv<T>& a, const Iv<T>& b) {
    bool ov = !(a.hi < b.lo) && !(b.hi < a.lo);
    return {!a.und && !b.und && a.lo == a.hi && b.lo == b.hi && a.lo == b.lo, a.und || b.und || ov};
}
template<class T> __device__ __forceinline__ IB iv_ne(const Iv<T>& a, const Iv<T>& b) { return ib_not(iv_eq(a, b)); }

} // namespace sid
