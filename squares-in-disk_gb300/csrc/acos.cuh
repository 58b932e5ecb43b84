// Correctly rounded arc cosine in a given direction, and the interval arc cosine built on it.
//
// The reference evaluates the interval arc cosine on the CPU with MPFR at the precision of the
// number type: [acos(x.ub) rounded down, acos(x.lb) rounded up], after clamping the argument to
// [-1, 1] when the compile-time bounds of the argument do not already guarantee the domain
// (ivarp/src/interval_acos.cpp:29-34,52-66, ivarp/include/ivarp/math_fn/interval_acos.hpp:19-28,
// interval_asin.hpp:14-32). The published cuboid counts of the lemmas that use acos depend on
// these endpoints, so they are reproduced exactly here, on the device, without MPFR.
//
// Method (this file's own design; runs on the integer pipe, which is far wider than the FP64
// pipe): acos(x) is evaluated in unsigned fixed point with NL 64-bit limbs and 64*NL-3
// fractional bits ("units" below are 2^-(64*NL-3)),
//   |x| <= 1/2 :  acos(x) = pi/2 - asin(x),
//   x > 1/2    :  acos(x) = 2 asin(sqrt((1-x)/2)),
//   x < -1/2   :  acos(x) = pi - 2 asin(sqrt((1+x)/2)),
// with asin(t) = t * sum C_k t^(2k) (t <= 1/2, Horner, exact rational coefficients rounded to the
// format) and sqrt(w) = w * y where y = 1/sqrt(w) is refined by Newton steps
// y <- y (3 - w y^2) / 2 from a float start value (the argument is first scaled by an even power
// of two into [1/4, 1)). (1-x)/2 and (1+x)/2 are exact in the format. Apart from that float start
// (rsqrtf) everything is integer arithmetic: GB300's FP64 pipe is not used at all.
//
// Error bound (all products truncated, each costs at most one unit): the series value is within
// 4.1 + 1.4 e_t units of the exact sum for an argument with error e_t, asin within 3.1 + 1.8 e_t,
// the square root within 3.5 units (the Newton steps from a start good to 2^-12 reach far below one
// unit), so the result is within 19 units of acos(x); kErrUnits = 64
// is used. The result is rounded to the target precision from the enclosure
// [R - 64 units, R + 64 units]: when both ends round down to the same floating-point number d,
// acos(x) lies strictly between d and its successor (acos(x) is transcendental for every
// floating-point x except 1, Lindemann-Weierstrass), so d is the downward and its successor the
// upward rounding. For float results one limb (61 fractional bits) decides all but a vanishing
// fraction of the arguments, for double results two limbs (125 bits); the rest are evaluated again
// with more limbs, up to four (253 fractional bits), which is more precision than any argument needs. If even that left the rounding undecided, the result
// would be the outward enclosure itself (still a valid bound).
//
// The same source compiles for the host (tests/acos_check.cpp checks it against 300-bit mpmath).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#include "acos_table.cuh"

#if defined(__CUDACC__)
#include "interval.cuh"
#endif

#if defined(__CUDACC__)
#define SID_ACOS_HD __host__ __device__
#define SID_ACOS_NOINLINE __noinline__
#define SID_ACOS_UNROLL _Pragma("unroll")
#else
#define SID_ACOS_HD
#define SID_ACOS_NOINLINE __attribute__((noinline))
#define SID_ACOS_UNROLL
#endif

namespace sid {
namespace acos_cr {

#if defined(__CUDACC__)
__constant__ const std::uint64_t kTableDev[SID_ACOS_TABLE_ROWS][4] = SID_ACOS_TABLE_INIT;
#endif
static const std::uint64_t kTableHost[SID_ACOS_TABLE_ROWS][4] = SID_ACOS_TABLE_INIT;

constexpr int kRowPiHalf = SID_ACOS_TABLE_TERMS;
constexpr int kRowPi = SID_ACOS_TABLE_TERMS + 1;
constexpr std::uint64_t kErrUnits = 64;

SID_ACOS_HD inline const std::uint64_t* table_row(int k) {
#if defined(__CUDA_ARCH__)
    return kTableDev[k];
#else
    return kTableHost[k];
#endif
}

SID_ACOS_HD inline std::uint64_t bits_of(double x) {
#if defined(__CUDA_ARCH__)
    return static_cast<std::uint64_t>(__double_as_longlong(x));
#else
    std::uint64_t b;
    std::memcpy(&b, &x, sizeof b);
    return b;
#endif
}

SID_ACOS_HD inline double double_of(std::uint64_t b) {
#if defined(__CUDA_ARCH__)
    return __longlong_as_double(static_cast<long long>(b));
#else
    double x;
    std::memcpy(&x, &b, sizeof x);
    return x;
#endif
}

SID_ACOS_HD inline float float_of(std::uint32_t b) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(b);
#else
    float x;
    std::memcpy(&x, &b, sizeof x);
    return x;
#endif
}

SID_ACOS_HD inline std::uint64_t mul_hi(std::uint64_t a, std::uint64_t b) {
#if defined(__CUDA_ARCH__)
    return __umul64hi(a, b);
#else
    return static_cast<std::uint64_t>((static_cast<unsigned __int128>(a) * b) >> 64);
#endif
}

SID_ACOS_HD inline int clz64(std::uint64_t v) {
#if defined(__CUDA_ARCH__)
    return __clzll(static_cast<long long>(v));
#else
    return __builtin_clzll(v);
#endif
}

// Unsigned fixed point: value = (sum w[i] 2^(64 i)) * 2^-(64 NL - 3), so values lie in [0, 8).
template<int NL> struct Fx {
    std::uint64_t w[NL];
};

template<int NL> SID_ACOS_HD inline Fx<NL> fx_zero() {
    Fx<NL> r;
SID_ACOS_UNROLL
    for(int i = 0; i < NL; ++i) r.w[i] = 0;
    return r;
}

template<int NL> SID_ACOS_HD inline Fx<NL> fx_row(int k) {
    const std::uint64_t* p = table_row(k);
    Fx<NL> r;
SID_ACOS_UNROLL
    for(int i = 0; i < NL; ++i) r.w[i] = p[4 - NL + i];
    return r;
}

template<int NL> SID_ACOS_HD inline Fx<NL> fx_units(std::uint64_t u) {
    Fx<NL> r = fx_zero<NL>();
    r.w[0] = u;
    return r;
}

template<int NL> SID_ACOS_HD inline Fx<NL> fx_int(std::uint64_t k) {   // k in [0, 8)
    Fx<NL> r = fx_zero<NL>();
    r.w[NL - 1] = k << 61;
    return r;
}

template<int NL> SID_ACOS_HD inline Fx<NL> fx_add(const Fx<NL>& a, const Fx<NL>& b) {
    Fx<NL> r;
    std::uint64_t c = 0;
SID_ACOS_UNROLL
    for(int i = 0; i < NL; ++i) {
        std::uint64_t s = a.w[i] + b.w[i];
        std::uint64_t c1 = s < a.w[i];
        r.w[i] = s + c;
        c = c1 | (r.w[i] < s);
    }
    return r;
}

template<int NL> SID_ACOS_HD inline Fx<NL> fx_sub(const Fx<NL>& a, const Fx<NL>& b) {   // requires a >= b
    Fx<NL> r;
    std::uint64_t br = 0;
SID_ACOS_UNROLL
    for(int i = 0; i < NL; ++i) {
        std::uint64_t d = a.w[i] - b.w[i];
        std::uint64_t b1 = a.w[i] < b.w[i];
        r.w[i] = d - br;
        br = b1 | (d < br);
    }
    return r;
}

template<int NL> SID_ACOS_HD inline bool fx_less(const Fx<NL>& a, const Fx<NL>& b) {
    bool less = false, decided = false;
SID_ACOS_UNROLL
    for(int i = NL - 1; i >= 0; --i) {
        if(!decided && a.w[i] != b.w[i]) {
            less = a.w[i] < b.w[i];
            decided = true;
        }
    }
    return less;
}

// Product truncated to the format (the exact 2NL-limb product shifted right by 64 NL - 3 bits);
// both factors' product must stay below 8.
template<int NL> SID_ACOS_HD inline Fx<NL> fx_mul(const Fx<NL>& a, const Fx<NL>& b) {
    std::uint64_t p[2 * NL];
SID_ACOS_UNROLL
    for(int i = 0; i < 2 * NL; ++i) p[i] = 0;
SID_ACOS_UNROLL
    for(int i = 0; i < NL; ++i) {
        std::uint64_t carry = 0;
SID_ACOS_UNROLL
        for(int j = 0; j < NL; ++j) {
            std::uint64_t lo = a.w[i] * b.w[j];
            std::uint64_t hi = mul_hi(a.w[i], b.w[j]);
            lo += p[i + j];
            hi += lo < p[i + j];
            lo += carry;
            hi += lo < carry;
            p[i + j] = lo;
            carry = hi;
        }
        p[i + NL] = carry;
    }
    Fx<NL> r;
SID_ACOS_UNROLL
    for(int k = 0; k < NL; ++k) r.w[k] = (p[NL - 1 + k] >> 61) | (p[NL + k] << 3);
    return r;
}

// Right shift by s bits, 0 < s < 64 (truncating).
template<int NL> SID_ACOS_HD inline Fx<NL> fx_shr(const Fx<NL>& a, int s) {
    Fx<NL> r;
SID_ACOS_UNROLL
    for(int i = 0; i < NL; ++i) {
        std::uint64_t hi = i + 1 < NL ? a.w[i + 1] : 0;
        r.w[i] = (a.w[i] >> s) | (hi << (64 - s));
    }
    return r;
}

template<int NL> SID_ACOS_HD inline Fx<NL> fx_shl1(const Fx<NL>& a) {
    Fx<NL> r;
SID_ACOS_UNROLL
    for(int i = 0; i < NL; ++i) r.w[i] = (a.w[i] << 1) | (i > 0 ? a.w[i - 1] >> 63 : 0);
    return r;
}

// A non-negative double (given by its bits) below 8, truncated to the format (exact when its last bit
// is >= 1 unit).
template<int NL> SID_ACOS_HD inline Fx<NL> fx_from_bits(std::uint64_t b) {
    int be = static_cast<int>((b >> 52) & 0x7ff);
    Fx<NL> r = fx_zero<NL>();
    if(be == 0) return r;   // zero or subnormal: below one unit
    std::uint64_t m = (b & ((std::uint64_t(1) << 52) - 1)) | (std::uint64_t(1) << 52);
    int s = be - 1075 + (64 * NL - 3);   // bit position of the mantissa's last bit
SID_ACOS_UNROLL
    for(int i = 0; i < NL; ++i) {
        int d = s - 64 * i;
        if(d >= 0) r.w[i] = d < 64 ? m << d : 0;
        else r.w[i] = d > -64 ? m >> -d : 0;
    }
    return r;
}

// A positive normal float (given by its bits) below 8, in the format (exact).
template<int NL> SID_ACOS_HD inline Fx<NL> fx_from_float_bits(std::uint32_t b) {
    const std::uint64_t m = std::uint64_t((b & 0x7fffffu) | 0x800000u);
    const int s = int((b >> 23) & 0xffu) - 150 + (64 * NL - 3);   // bit position of the last mantissa bit
    Fx<NL> r = fx_zero<NL>();
SID_ACOS_UNROLL
    for(int i = 0; i < NL; ++i) {
        int d = s - 64 * i;
        if(d >= 0) r.w[i] = d < 64 ? m << d : 0;
        else r.w[i] = d > -64 ? m >> -d : 0;
    }
    return r;
}

// Index of the highest set bit (-1 for zero).
template<int NL> SID_ACOS_HD inline int fx_top_bit(const Fx<NL>& v) {
    int p = -1;
SID_ACOS_UNROLL
    for(int i = NL - 1; i >= 0; --i) {
        if(p < 0 && v.w[i] != 0) p = 64 * i + 63 - clz64(v.w[i]);
    }
    return p;
}

// Left shift by s bits, 0 <= s < 64 NL (limbs selected with compile-time indices only).
template<int NL> SID_ACOS_HD inline Fx<NL> fx_shl(const Fx<NL>& a, int s) {
    const int q = s >> 6, b = s & 63;
    Fx<NL> r;
SID_ACOS_UNROLL
    for(int i = 0; i < NL; ++i) {
        std::uint64_t hi = 0, lo = 0;
SID_ACOS_UNROLL
        for(int k = 0; k < NL; ++k) {
            if(k == i - q) hi = a.w[k];
            if(k == i - q - 1) lo = a.w[k];
        }
        r.w[i] = (hi << b) | (b ? lo >> (64 - b) : 0);
    }
    return r;
}

SID_ACOS_HD inline float rsqrt_f32(float m) {
#if defined(__CUDA_ARCH__)
    return rsqrtf(m);
#else
    return 1.0f / __builtin_sqrtf(m);
#endif
}

SID_ACOS_HD inline std::uint32_t float_bits(float x) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(x);
#else
    std::uint32_t b;
    std::memcpy(&b, &x, sizeof b);
    return b;
#endif
}

// Series length (64 NL - 3 fractional bits need (1/4)^k below one unit) and Newton steps of the reciprocal
// square root (from a float start good to 2^-12 or better; each step squares the relative error).
template<int NL> struct Terms;
template<> struct Terms<1> { static constexpr int count = 32; static constexpr int newton = 3; };
template<> struct Terms<2> { static constexpr int count = 64; static constexpr int newton = 4; };
template<> struct Terms<4> { static constexpr int count = 128; static constexpr int newton = 5; };

// asin(t) for t <= 1/2 (plus rounding slack).
template<int NL> SID_ACOS_HD inline Fx<NL> fx_asin(const Fx<NL>& t) {
    Fx<NL> t2 = fx_mul(t, t);
    Fx<NL> s = fx_row<NL>(Terms<NL>::count - 1);
    for(int k = Terms<NL>::count - 2; k >= 0; --k) s = fx_add(fx_row<NL>(k), fx_mul(s, t2));
    return fx_mul(t, s);
}

// sqrt(w) for an exact w in [0, 1/4): w = m 4^-e with m in [1/4, 1), y = 1/sqrt(m) by Newton steps
// y <- y (3 - m y^2) / 2 from a float start, sqrt(w) = (m y) 2^-e.
template<int NL> SID_ACOS_HD inline Fx<NL> fx_sqrt_small(const Fx<NL>& w) {
    constexpr int F = 64 * NL - 3;
    const int p = fx_top_bit(w);
    if(p < 0) return fx_zero<NL>();
    const int e = (F - 1 - p) >> 1;                       // 1 <= e: the top bit of m is F-1 or F-2
    const Fx<NL> mm = fx_shl(w, 2 * e);
    const float mf = float(std::uint32_t(mm.w[NL - 1] >> 37)) * (1.0f / 16777216.0f);   // m to 24 bits
    Fx<NL> y = fx_from_float_bits<NL>(float_bits(rsqrt_f32(mf)));
    const Fx<NL> three = fx_int<NL>(3);
SID_ACOS_UNROLL
    for(int it = 0; it < Terms<NL>::newton; ++it) {
        Fx<NL> c = fx_mul(fx_mul(mm, y), y);
        y = fx_shr(fx_mul(y, fx_sub(three, c)), 1);
    }
    return fx_shr(fx_mul(mm, y), e);
}

// acos(x) for -1 <= x < 1 (x given by its double bits), within 19 units; integer arithmetic only.
template<int NL> SID_ACOS_HD inline Fx<NL> fx_acos(std::uint64_t xb) {
    const std::uint64_t ab = xb & ~(std::uint64_t(1) << 63);
    const bool neg = (xb >> 63) != 0;
    if(ab <= 0x3fe0000000000000ull) {                      // |x| <= 1/2
        Fx<NL> a = fx_asin(fx_from_bits<NL>(ab));
        Fx<NL> h = fx_row<NL>(kRowPiHalf);
        return neg ? fx_add(h, a) : fx_sub(h, a);
    }
    const Fx<NL> w = fx_shr(fx_sub(fx_int<NL>(1), fx_from_bits<NL>(ab)), 1);   // (1 - |x|) / 2, exact
    Fx<NL> a2 = fx_shl1(fx_asin(fx_sqrt_small(w)));
    return neg ? fx_sub(fx_row<NL>(kRowPi), a2) : a2;
}

// The largest floating-point number with `digits` significant bits that is <= v (v > 0), as
// (significand, exponent of its leading bit relative to the format's units).
template<int NL> SID_ACOS_HD inline void fx_floor_fp(const Fx<NL>& v, int digits, std::uint64_t& mant, int& lead) {
    const int p = fx_top_bit(v);
    int q = p - digits + 1;   // position of the last kept bit (>= 0: values here are >= 2^-31)
    std::uint64_t win = 0;
SID_ACOS_UNROLL
    for(int i = 0; i < NL; ++i) {
        int d = 64 * i - q;
        if(d >= 0) win |= d < 64 ? v.w[i] << d : 0;
        else win |= d > -64 ? v.w[i] >> -d : 0;
    }
    mant = win;
    lead = p;
}

// Downward rounding of acos(x) for -1 <= x < 1 at `digits` bits; false if NL limbs cannot decide
// it (then mant/lead describe the floor of the enclosure's lower end and mant_hi/lead_hi its upper).
template<int NL> SID_ACOS_HD inline bool acos_floor(std::uint64_t xb, int digits, std::uint64_t& mant, int& lead,
                                                    std::uint64_t& mant_hi, int& lead_hi) {
    Fx<NL> r = fx_acos<NL>(xb);
    Fx<NL> err = fx_units<NL>(kErrUnits);
    Fx<NL> lo = fx_less(err, r) ? fx_sub(r, err) : fx_units<NL>(1);
    Fx<NL> hi = fx_add(r, err);
    fx_floor_fp(lo, digits, mant, lead);
    fx_floor_fp(hi, digits, mant_hi, lead_hi);
    return mant == mant_hi && lead == lead_hi;
}

// acos(x) rounded down (up = false) or up (up = true) to double (digits 53) or float (digits 24), as bit
// patterns, for x given by its double bits. NaN and arguments outside [-1, 1] give NaN; acos(1) = +0.
// Float results try one limb first, double results two; undecided roundings retry with more limbs.
template<int DIGITS> SID_ACOS_HD SID_ACOS_NOINLINE std::uint64_t acos_rounded_bits(std::uint64_t xb, bool up) {
    constexpr int kBias = DIGITS == 53 ? 1023 : 127;
    constexpr std::uint64_t kNaN = DIGITS == 53 ? 0x7ff8000000000000ull : 0x7fc00000ull;
    const std::uint64_t ab = xb & ~(std::uint64_t(1) << 63);
    if(ab > 0x3ff0000000000000ull) return kNaN;             // |x| > 1 or NaN
    if(xb == 0x3ff0000000000000ull) return 0;              // acos(1) = +0
    std::uint64_t mant = 0, mant_hi = 0;
    int lead = 0, lead_hi = 0, frac = 64 * 4 - 3;
    bool done = false;
    if(DIGITS == 24 && acos_floor<1>(xb, DIGITS, mant, lead, mant_hi, lead_hi)) {
        frac = 64 - 3;
        done = true;
    }
    if(!done && acos_floor<2>(xb, DIGITS, mant, lead, mant_hi, lead_hi)) {
        frac = 64 * 2 - 3;
        done = true;
    }
    if(!done && !acos_floor<4>(xb, DIGITS, mant, lead, mant_hi, lead_hi) && up) {
        mant = mant_hi;   // undecided even with four limbs: outward enclosure
        lead = lead_hi;
    }
    std::uint64_t b = (static_cast<std::uint64_t>(lead - frac + kBias) << (DIGITS - 1)) |
                      (mant & ((std::uint64_t(1) << (DIGITS - 1)) - 1));
    return up ? b + 1 : b;   // the successor of a positive number: next bit pattern
}

// Double bits of a float, by integer operations (float subnormals, far below one unit, map to zero).
SID_ACOS_HD inline std::uint64_t f32_to_f64_bits(std::uint32_t f) {
    const std::uint64_t sign = std::uint64_t(f >> 31) << 63;
    const std::uint32_t e = (f >> 23) & 0xffu, m = f & 0x7fffffu;
    if(e == 0xffu) return sign | (std::uint64_t(0x7ff) << 52) | (std::uint64_t(m) << 29);
    if(e == 0) return sign;
    return sign | (std::uint64_t(e - 127 + 1023) << 52) | (std::uint64_t(m) << 29);
}

SID_ACOS_HD inline double acos_rd(double x) { return double_of(acos_rounded_bits<53>(bits_of(x), false)); }
SID_ACOS_HD inline double acos_ru(double x) { return double_of(acos_rounded_bits<53>(bits_of(x), true)); }
SID_ACOS_HD inline float acos_rd(float x) {
    return float_of(static_cast<std::uint32_t>(acos_rounded_bits<24>(f32_to_f64_bits(float_bits(x)), false)));
}
SID_ACOS_HD inline float acos_ru(float x) {
    return float_of(static_cast<std::uint32_t>(acos_rounded_bits<24>(f32_to_f64_bits(float_bits(x)), true)));
}

// Rounding toward -inf for acos_bound_f32: the directed-rounding intrinsics on the device; on the host the
// ambient rounding mode, which the caller must have set to FE_DOWNWARD (the CPU oracle runs in that mode).
struct RoundDownF32 {
    static SID_ACOS_HD inline float add(float a, float b) {
#if defined(__CUDA_ARCH__)
        return __fadd_rd(a, b);
#else
        return a + b;
#endif
    }
    static SID_ACOS_HD inline float mul(float a, float b) {
#if defined(__CUDA_ARCH__)
        return __fmul_rd(a, b);
#else
        return a * b;
#endif
    }
    static SID_ACOS_HD inline float sqrt(float a) {
#if defined(__CUDA_ARCH__)
        return __fsqrt_rd(a);
#else
        return std::sqrt(a);
#endif
    }
};

// Float bounds of the series coefficients c_k = binom(2k, k) / (4^k (2k + 1)) of asin(r) / r, k = 0..10,
// rounded down (hi = false) and up (c_0 = 1 is exact); a function of a constant index, so that unrolled
// device code sees immediates.
SID_ACOS_HD constexpr float asin_coef(int k, bool hi) {
    switch(k) {
        case 0: return 0x1p+0f;
        case 1: return hi ? 0x1.555556p-3f : 0x1.555554p-3f;
        case 2: return hi ? 0x1.333334p-4f : 0x1.333332p-4f;
        case 3: return hi ? 0x1.6db6dcp-5f : 0x1.6db6dap-5f;
        case 4: return hi ? 0x1.f1c71ep-6f : 0x1.f1c71cp-6f;
        case 5: return hi ? 0x1.6e8ba4p-6f : 0x1.6e8ba2p-6f;
        case 6: return hi ? 0x1.1c4ec6p-6f : 0x1.1c4ec4p-6f;
        case 7: return hi ? 0x1.c9999ap-7f : 0x1.c99998p-7f;
        case 8: return hi ? 0x1.7a8788p-7f : 0x1.7a8786p-7f;
        case 9: return hi ? 0x1.3fde52p-7f : 0x1.3fde50p-7f;
        default: return hi ? 0x1.12ef3ep-7f : 0x1.12ef3cp-7f;
    }
}
constexpr float kPiLoF = 0x1.921fb4p+1f, kPiHiF = 0x1.921fb6p+1f;
constexpr float kHalfPiLoF = 0x1.921fb4p+0f, kHalfPiHiF = 0x1.921fb6p+0f;

// A float bound of acos(x) for the precision form's float pass: lower (up = false) <= acos(x) <= upper
// (up = true), a few float units wide, not correctly rounded (the float pass only has to enclose the
// double evaluation, whose arc cosine is the correctly rounded one above).
//   |x| <= 1/2: acos(x) = pi/2 - asin(x) (asin is odd); x > 1/2: 2 asin(r); x < -1/2: pi - 2 asin(r),
//   r = sqrt((1 - |x|) / 2), where 1 - |x| and the halving are exact (Sterbenz);
//   asin(r) = r * sum_{k <= 10} c_k r^(2k) + R with 0 <= R <= r c_11 4^-11 / (1 - 1/4) < r 2^-28 for
//   0 <= r <= 1/2 (the c_k decrease).
// Every operation rounds toward -inf; an upper bound is computed as minus the lower bound of the negated
// quantity, so both directions run the same instructions on constants of the other rounding. The
// successor of sqrt rounded down bounds the square root from above. Arguments outside [-1, 1] and NaN
// give the correctly rounded function's result (NaN).
template<class Op = RoundDownF32> SID_ACOS_HD inline float acos_bound_f32(float x, bool up) {
    if(!(x >= -1.0f && x <= 1.0f)) return up ? acos_ru(x) : acos_rd(x);
    const bool pos = x >= 0.0f;
    const float ax = pos ? x : -x;
    const bool big = ax > 0.5f;
    const bool asin_up = up != (big != pos);       // which bound of asin the result needs
    float r = ax;
    if(big) {
        r = Op::sqrt(Op::mul(Op::add(1.0f, -ax), 0.5f));
        if(asin_up) r = float_of((float_bits(r) & 0x7fffffffu) + 1u);   // successor (1 - 1 is -0 rounding down)
    }
    // q: the lower bound of asin(r), or minus its upper bound
    const float s = asin_up ? -Op::mul(-r, r) : Op::mul(r, r);
    float q = asin_up ? -asin_coef(10, true) : asin_coef(10, false);
    SID_ACOS_UNROLL
    for(int k = 9; k >= 0; --k) q = Op::add(Op::mul(q, s), asin_up ? -asin_coef(k, true) : asin_coef(k, false));
    q = Op::mul(q, r);
    if(asin_up) q = Op::add(q, Op::mul(-r, 0x1p-28f));
    float k0;
    if(!up) k0 = big ? (pos ? 0.0f : kPiLoF) : kHalfPiLoF;
    else k0 = big ? (pos ? 0.0f : -kPiHiF) : -kHalfPiHiF;
    const float res = Op::add(k0, big ? Op::mul(2.0f, q) : q);
    return up ? -res : res;
}

} // namespace acos_cr

#if defined(__CUDACC__)
// Interval arc cosine: clamp to [-1, 1] (marking the result possibly undefined) only where the
// argument's compile-time bounds leave the domain, as the reference does.
template<class T, bool CLAMP_LO, bool CLAMP_HI> __device__ inline Iv<T> iv_acos(Iv<T> x) {
    bool und = x.und;
    if(CLAMP_LO && x.lo < T(-1)) {
        und = true;
        x.lo = T(-1);
    }
    if(CLAMP_HI && T(1) < x.hi) {
        und = true;
        x.hi = T(1);
    }
    return {acos_cr::acos_rd(x.hi), acos_cr::acos_ru(x.lo), und};
}

// Interval arc cosine of a lemma computed in double: double endpoints are the correctly rounded ones (the
// plain form and the precision form's escalation), float endpoints (the precision form's float pass) the
// cheaper enclosure acos_bound_f32.
template<class T, bool CLAMP_LO, bool CLAMP_HI> __device__ inline Iv<T> iv_acos_f64(Iv<T> x) {
    if constexpr(sizeof(T) == sizeof(double)) {
        return iv_acos<T, CLAMP_LO, CLAMP_HI>(x);
    } else {
        bool und = x.und;
        if(CLAMP_LO && x.lo < T(-1)) {
            und = true;
            x.lo = T(-1);
        }
        if(CLAMP_HI && T(1) < x.hi) {
            und = true;
            x.hi = T(1);
        }
        return {acos_cr::acos_bound_f32(x.hi, false), acos_cr::acos_bound_f32(x.lo, true), und};
    }
}
#endif

} // namespace sid
