// CPU ORACLE -- test infrastructure only.
// Correctly rounded arc cosine in a given direction, as the reference computes it with MPFR at the
// number type's precision (ivarp/src/interval_acos.cpp:29-34,52-66): acos_rounded(x, up) is acos(x)
// rounded down (up = false) or up (up = true) to T; NaN outside [-1, 1]; acos(1) = +0.
//
// Independent of the device implementation: acos is taken from the C library in a wider format
// (x86-64: the 64-bit-significand long double, then __float128 from libquadmath where that does not
// decide the rounding; aarch64: the 113-bit long double), and the rounding to T is decided from an
// enclosure of 16 units in the last place of that format around it (the libraries are accurate to
// a few units). Since acos(x) is transcendental for x != 1, it never equals a T-number; if the
// enclosure still contains one, the oracle throws instead of guessing.
#pragma once

#include <cfenv>
#include <cmath>
#include <limits>
#include <stdexcept>

#if defined(__x86_64__)
#include <quadmath.h>
#endif

namespace sido {
namespace acos_detail {

// Largest T <= v (v finite, positive), computed without relying on the rounding mode.
template<class T, class Q> T floor_to(Q v) {
    T d = static_cast<T>(v);
    if(static_cast<Q>(d) > v) d = std::nextafter(d, -std::numeric_limits<T>::infinity());
    return d;
}

// Decide the downward rounding of a value known to lie in a (1 +- 2^-(digits-5)) band around a.
template<class T, class Q> bool decide(Q a, int digits, T& rd) {
    Q e = a;
    for(int i = 0; i < digits - 5; ++i) e = e / 2;
    T lo = floor_to<T>(a - e);
    T hi = floor_to<T>(a + e);
    rd = lo;
    return lo == hi;
}

struct NearestScope {
    int saved;
    NearestScope() : saved(std::fegetround()) { std::fesetround(FE_TONEAREST); }
    ~NearestScope() { std::fesetround(saved); }
};

} // namespace acos_detail

template<class T> T acos_rounded(T x, bool up) {
    using namespace acos_detail;
    if(!(x >= T(-1) && x <= T(1))) return std::numeric_limits<T>::quiet_NaN();
    if(x == T(1)) return T(0);
    NearestScope nearest;
    T rd;
    long double al = acosl(static_cast<long double>(x));
    bool ok = decide<T, long double>(al, std::numeric_limits<long double>::digits, rd);
#if defined(__x86_64__)
    if(!ok) {
        __float128 aq = acosq(static_cast<__float128>(x));
        ok = decide<T, __float128>(aq, 113, rd);
    }
#endif
    if(!ok) throw std::runtime_error("oracle: arc cosine rounding undecided");
    return up ? std::nextafter(rd, std::numeric_limits<T>::infinity()) : rd;
}

} // namespace sido
