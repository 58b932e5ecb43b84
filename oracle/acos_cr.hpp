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

/// The float pass's arc cosine bound (lower for up = false, upper for up = true) as the device computes it
/// for lemmas in double (squares-in-disk_gb300/csrc/acos.cuh, acos_bound_f32), restated: acos(x) = pi/2 -
/// asin(x) for |x| <= 1/2, 2 asin(r) for x > 1/2, pi - 2 asin(r) for x < -1/2 with r = sqrt((1 - |x|)/2);
/// asin(r) from the first 11 series terms with float coefficient bounds plus a remainder below r 2^-28.
/// Runs in the oracle's ambient round-down mode; upper bounds as minus the lower bound of the negation.
inline float acos_bound_f32(float x, bool up) {
    static const float lo_c[11] = {0x1p+0f, 0x1.555554p-3f, 0x1.333332p-4f, 0x1.6db6dap-5f, 0x1.f1c71cp-6f,
                                   0x1.6e8ba2p-6f, 0x1.1c4ec4p-6f, 0x1.c99998p-7f, 0x1.7a8786p-7f, 0x1.3fde50p-7f,
                                   0x1.12ef3cp-7f};
    static const float hi_c[11] = {0x1p+0f, 0x1.555556p-3f, 0x1.333334p-4f, 0x1.6db6dcp-5f, 0x1.f1c71ep-6f,
                                   0x1.6e8ba4p-6f, 0x1.1c4ec6p-6f, 0x1.c9999ap-7f, 0x1.7a8788p-7f, 0x1.3fde52p-7f,
                                   0x1.12ef3ep-7f};
    if(!(x >= -1.0f && x <= 1.0f)) return acos_rounded<float>(x, up);
    const bool negative = x < 0.0f;
    const float a = negative ? -x : x;
    const bool reduced = a > 0.5f;
    // the bound of asin needed: upper exactly when the result's direction and the formula's sign differ
    const bool want_upper = up != (reduced == negative);
    float r = a;
    if(reduced) {
        r = std::sqrt((1.0f - a) * 0.5f);
        if(want_upper) r = std::nextafter(r, std::numeric_limits<float>::infinity());
    }
    float r2, acc;
    if(want_upper) {
        r2 = -((-r) * r);
        acc = -hi_c[10];
        for(int k = 9; k >= 0; --k) acc = acc * r2 + (-hi_c[k]);
        acc = acc * r;
        acc = acc + (-r) * 0x1p-28f;
    } else {
        r2 = r * r;
        acc = lo_c[10];
        for(int k = 9; k >= 0; --k) acc = acc * r2 + lo_c[k];
        acc = acc * r;
    }
    const float pi_lo = 0x1.921fb4p+1f, pi_hi = 0x1.921fb6p+1f;
    float base;
    if(reduced) base = negative ? (up ? -pi_hi : pi_lo) : 0.0f;
    else base = up ? -pi_hi * 0.5f : pi_lo * 0.5f;
    const float v = base + (reduced ? 2.0f * acc : acc);
    return up ? -v : v;
}

} // namespace sido
