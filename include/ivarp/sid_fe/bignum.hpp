// Exact integer / rational arithmetic used by the front end to fold constant
// subexpressions of a constraint system before they are rounded outward to
// double and float intervals.
//
// The reference folds constants with GMP rationals and evaluates irrational
// operations (square roots) with MPFR at 256 bits, rounding the operand to
// 256 bits and then the square root to 256 bits in the requested direction
// (ivarp/src/irational_sqrt.cpp:30-56, ivarp/include/ivarp/context.hpp:32-38).
// This header restates those semantics with a small self-contained big
// integer so that no GMP/MPFR headers are needed.
#pragma once

#include <cstdint>
#include <cmath>
#include <cfloat>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace ivarp {
namespace sid_fe {

/// Non-negative arbitrary precision integer (little-endian 32-bit limbs).
class BigNat {
public:
    BigNat() = default;
    explicit BigNat(std::uint64_t v) {
        while(v) { limbs.push_back(std::uint32_t(v)); v >>= 32; }
    }

    bool is_zero() const noexcept { return limbs.empty(); }
    bool is_odd() const noexcept { return !limbs.empty() && (limbs[0] & 1u); }

    std::size_t bit_length() const noexcept {
        if(limbs.empty()) return 0;
        std::uint32_t top = limbs.back();
        std::size_t n = 0;
        while(top) { ++n; top >>= 1; }
        return (limbs.size() - 1) * 32 + n;
    }

    bool bit(std::size_t i) const noexcept {
        std::size_t l = i / 32;
        if(l >= limbs.size()) return false;
        return (limbs[l] >> (i % 32)) & 1u;
    }

    static int cmp(const BigNat& a, const BigNat& b) noexcept {
        if(a.limbs.size() != b.limbs.size()) return a.limbs.size() < b.limbs.size() ? -1 : 1;
        for(std::size_t i = a.limbs.size(); i-- > 0;) {
            if(a.limbs[i] != b.limbs[i]) return a.limbs[i] < b.limbs[i] ? -1 : 1;
        }
        return 0;
    }

    friend bool operator==(const BigNat& a, const BigNat& b) noexcept { return cmp(a, b) == 0; }
    friend bool operator!=(const BigNat& a, const BigNat& b) noexcept { return cmp(a, b) != 0; }
    friend bool operator<(const BigNat& a, const BigNat& b) noexcept { return cmp(a, b) < 0; }
    friend bool operator<=(const BigNat& a, const BigNat& b) noexcept { return cmp(a, b) <= 0; }

    friend BigNat operator+(const BigNat& a, const BigNat& b) {
        BigNat r;
        std::size_t n = std::max(a.limbs.size(), b.limbs.size());
        r.limbs.resize(n);
        std::uint64_t carry = 0;
        for(std::size_t i = 0; i < n; ++i) {
            std::uint64_t s = carry;
            if(i < a.limbs.size()) s += a.limbs[i];
            if(i < b.limbs.size()) s += b.limbs[i];
            r.limbs[i] = std::uint32_t(s);
            carry = s >> 32;
        }
        if(carry) r.limbs.push_back(std::uint32_t(carry));
        return r;
    }

    /// a - b, requires a >= b.
    friend BigNat operator-(const BigNat& a, const BigNat& b) {
        if(a < b) throw std::logic_error("BigNat subtraction underflow");
        BigNat r;
        r.limbs.resize(a.limbs.size());
        std::int64_t borrow = 0;
        for(std::size_t i = 0; i < a.limbs.size(); ++i) {
            std::int64_t d = std::int64_t(a.limbs[i]) - borrow - (i < b.limbs.size() ? std::int64_t(b.limbs[i]) : 0);
            borrow = 0;
            if(d < 0) { d += (std::int64_t(1) << 32); borrow = 1; }
            r.limbs[i] = std::uint32_t(d);
        }
        r.trim();
        return r;
    }

    friend BigNat operator*(const BigNat& a, const BigNat& b) {
        if(a.is_zero() || b.is_zero()) return BigNat{};
        BigNat r;
        r.limbs.assign(a.limbs.size() + b.limbs.size(), 0u);
        for(std::size_t i = 0; i < a.limbs.size(); ++i) {
            std::uint64_t carry = 0;
            for(std::size_t j = 0; j < b.limbs.size(); ++j) {
                std::uint64_t t = std::uint64_t(a.limbs[i]) * b.limbs[j] + r.limbs[i + j] + carry;
                r.limbs[i + j] = std::uint32_t(t);
                carry = t >> 32;
            }
            std::size_t k = i + b.limbs.size();
            while(carry) {
                std::uint64_t t = std::uint64_t(r.limbs[k]) + carry;
                r.limbs[k] = std::uint32_t(t);
                carry = t >> 32;
                ++k;
            }
        }
        r.trim();
        return r;
    }

    BigNat shl(std::size_t s) const {
        if(is_zero()) return {};
        BigNat r;
        std::size_t ls = s / 32, bs = s % 32;
        r.limbs.assign(ls, 0u);
        std::uint32_t carry = 0;
        for(std::uint32_t l : limbs) {
            std::uint64_t v = (std::uint64_t(l) << bs) | carry;
            r.limbs.push_back(std::uint32_t(v));
            carry = bs ? std::uint32_t(std::uint64_t(l) >> (32 - bs)) : 0u;
        }
        if(carry) r.limbs.push_back(carry);
        r.trim();
        return r;
    }

    BigNat shr(std::size_t s) const {
        std::size_t ls = s / 32, bs = s % 32;
        if(ls >= limbs.size()) return {};
        BigNat r;
        for(std::size_t i = ls; i < limbs.size(); ++i) {
            std::uint64_t v = limbs[i] >> bs;
            if(bs && i + 1 < limbs.size()) v |= (std::uint64_t(limbs[i + 1]) << (32 - bs)) & 0xffffffffu;
            r.limbs.push_back(std::uint32_t(v));
        }
        r.trim();
        return r;
    }

    /// Schoolbook binary long division: returns quotient, remainder in *rem.
    static BigNat divmod(const BigNat& a, const BigNat& b, BigNat* rem) {
        if(b.is_zero()) throw std::domain_error("BigNat division by zero");
        if(a < b) { if(rem) *rem = a; return {}; }
        BigNat q, r;
        std::size_t n = a.bit_length();
        q.limbs.assign((n + 31) / 32, 0u);
        for(std::size_t i = n; i-- > 0;) {
            r = r.shl(1);
            if(a.bit(i)) {
                if(r.limbs.empty()) r.limbs.push_back(1u); else r.limbs[0] |= 1u;
            }
            if(!(r < b)) {
                r = r - b;
                q.limbs[i / 32] |= (1u << (i % 32));
            }
        }
        q.trim();
        if(rem) *rem = r;
        return q;
    }

    static BigNat gcd(BigNat a, BigNat b) {
        if(a.is_zero()) return b;
        if(b.is_zero()) return a;
        std::size_t shift = 0;
        while(!a.is_odd() && !b.is_odd()) { a = a.shr(1); b = b.shr(1); ++shift; }
        while(!a.is_odd()) a = a.shr(1);
        while(!b.is_zero()) {
            while(!b.is_odd()) b = b.shr(1);
            if(b < a) std::swap(a, b);
            b = b - a;
        }
        return a.shl(shift);
    }

    /// floor(sqrt(n)) by Newton iteration.
    static BigNat isqrt(const BigNat& n) {
        if(n.is_zero()) return {};
        BigNat x = BigNat(1).shl((n.bit_length() + 1) / 2 + 1);
        for(;;) {
            BigNat y = (x + divmod(n, x, nullptr)).shr(1);
            if(!(y < x)) return x;
            x = y;
        }
    }

    std::uint64_t to_u64() const noexcept {
        std::uint64_t v = 0;
        for(std::size_t i = std::min<std::size_t>(limbs.size(), 2); i-- > 0;) v = (v << 32) | limbs[i];
        return v;
    }

private:
    void trim() { while(!limbs.empty() && limbs.back() == 0u) limbs.pop_back(); }
    std::vector<std::uint32_t> limbs;
};

/// Exact rational number num/den with den > 0, kept in lowest terms.
class Rat {
public:
    Rat() : neg(false), num(), den(1) {}
    Rat(std::int64_t v) : neg(v < 0), num(v < 0 ? std::uint64_t(-(v + 1)) + 1u : std::uint64_t(v)), den(1) {} // NOLINT
    Rat(bool negative, BigNat n, BigNat d) : neg(negative), num(std::move(n)), den(std::move(d)) { normalize(); }

    static Rat ratio(std::int64_t n, std::int64_t d) {
        Rat a(n), b(d);
        return a / b;
    }

    /// Parse a non-negative decimal string "123.456" exactly.
    static Rat from_decimal(const std::string& s) {
        BigNat n, d(1);
        bool after = false;
        for(char c : s) {
            if(c == '.') { after = true; continue; }
            if(c < '0' || c > '9') throw std::invalid_argument("bad decimal literal: " + s);
            n = n * BigNat(10) + BigNat(std::uint64_t(c - '0'));
            if(after) d = d * BigNat(10);
        }
        return Rat(false, n, d);
    }

    /// Exact value of a finite double.
    static Rat from_double(double x) {
        if(!std::isfinite(x)) throw std::domain_error("non-finite double in exact constant");
        if(x == 0) return Rat{};
        int e;
        double m = std::frexp(std::fabs(x), &e);               // x = m * 2^e, m in [0.5,1)
        std::uint64_t mi = std::uint64_t(std::ldexp(m, 53));    // exact
        e -= 53;
        BigNat n(mi), d(1);
        if(e >= 0) n = n.shl(std::size_t(e)); else d = d.shl(std::size_t(-e));
        return Rat(x < 0, n, d);
    }

    bool is_zero() const noexcept { return num.is_zero(); }
    bool is_negative() const noexcept { return neg && !num.is_zero(); }

    friend Rat operator-(const Rat& a) { Rat r = a; if(!r.num.is_zero()) r.neg = !r.neg; return r; }
    friend Rat operator+(const Rat& a, const Rat& b) {
        BigNat x = a.num * b.den, y = b.num * a.den;
        if(a.neg == b.neg) return Rat(a.neg, x + y, a.den * b.den);
        if(y <= x) return Rat(a.neg, x - y, a.den * b.den);
        return Rat(b.neg, y - x, a.den * b.den);
    }
    friend Rat operator-(const Rat& a, const Rat& b) { return a + (-b); }
    friend Rat operator*(const Rat& a, const Rat& b) { return Rat(a.neg != b.neg, a.num * b.num, a.den * b.den); }
    friend Rat operator/(const Rat& a, const Rat& b) {
        if(b.num.is_zero()) throw std::domain_error("rational division by zero");
        return Rat(a.neg != b.neg, a.num * b.den, a.den * b.num);
    }

    static int cmp(const Rat& a, const Rat& b) {
        bool an = a.is_negative(), bn = b.is_negative();
        if(an != bn) return an ? -1 : 1;
        int c = BigNat::cmp(a.num * b.den, b.num * a.den);
        return an ? -c : c;
    }
    friend bool operator<(const Rat& a, const Rat& b) { return cmp(a, b) < 0; }
    friend bool operator<=(const Rat& a, const Rat& b) { return cmp(a, b) <= 0; }
    friend bool operator==(const Rat& a, const Rat& b) { return cmp(a, b) == 0; }

    /// Round |this| (non-zero) to a binary float with `prec` significant bits, towards zero (up=false)
    /// or away from zero (up=true), with an unbounded exponent: returns mantissa m and exponent e with value m*2^e.
    void round_magnitude(std::size_t prec, bool up, BigNat* m, long* e) const {
        // find k with 2^(prec-1) <= num*2^k/den < 2^prec
        long k = long(prec) - (long(num.bit_length()) - long(den.bit_length())) - 1;
        for(;;) {
            BigNat a = k >= 0 ? num.shl(std::size_t(k)) : num;
            BigNat b = k >= 0 ? den : den.shl(std::size_t(-k));
            BigNat r;
            BigNat q = BigNat::divmod(a, b, &r);
            std::size_t bl = q.bit_length();
            if(bl < prec) { ++k; continue; }
            if(bl > prec) { --k; continue; }
            if(up && !r.is_zero()) q = q + BigNat(1);
            *m = q;
            *e = -k;
            return;
        }
    }

    /// Directed rounding to an IEEE binary type with `prec` significand bits and minimum (subnormal) exponent
    /// `emin_sub` (value = m * 2^e with e >= emin_sub). down=true rounds towards -inf.
    double round_ieee(std::size_t prec, long emin_sub, bool down) const {
        if(num.is_zero()) return 0.0;
        bool toward_zero = (down != is_negative());   // rounding magnitude down?
        BigNat m; long e;
        round_magnitude(prec, !toward_zero, &m, &e);
        if(e < emin_sub) {
            // subnormal range: re-round on the fixed grid 2^emin_sub
            BigNat a = num, b = den;
            long sh = -emin_sub;
            if(sh >= 0) a = a.shl(std::size_t(sh)); else b = b.shl(std::size_t(-sh));
            BigNat r;
            BigNat q = BigNat::divmod(a, b, &r);
            if(!toward_zero && !r.is_zero()) q = q + BigNat(1);
            m = q; e = emin_sub;
        }
        double v = std::ldexp(double(m.to_u64()), int(e));
        return is_negative() ? -v : v;
    }

    double to_double_rd() const { return round_ieee(53, -1074, true); }
    double to_double_ru() const { return round_ieee(53, -1074, false); }
    float to_float_rd() const { return float(round_ieee(24, -149, true)); }
    float to_float_ru() const { return float(round_ieee(24, -149, false)); }

    /// Round to a `prec`-bit binary float in the given direction (MPFR mpfr_set_q semantics).
    Rat round_prec(std::size_t prec, bool down) const {
        if(num.is_zero()) return Rat{};
        bool toward_zero = (down != is_negative());
        BigNat m; long e;
        round_magnitude(prec, !toward_zero, &m, &e);
        BigNat n = m, d(1);
        if(e >= 0) n = n.shl(std::size_t(e)); else d = d.shl(std::size_t(-e));
        return Rat(is_negative(), n, d);
    }

    /// Square root of a non-negative rational: the operand is first rounded to `prec` bits and the result is
    /// rounded to `prec` bits, both in the same direction (MPFR-style directed square root).
    Rat sqrt_prec(std::size_t prec, bool down) const {
        if(is_negative()) throw std::domain_error("sqrt of negative constant");
        if(num.is_zero()) return Rat{};
        Rat x = round_prec(prec, down);       // x = m * 2^e exactly
        BigNat m; long e;
        x.round_magnitude(prec, false, &m, &e); // exact, recovers mantissa/exponent
        if(e & 1) { m = m.shl(1); e -= 1; }
        // sqrt(x) = sqrt(m) * 2^(e/2); find t = floor(sqrt(m * 4^k)) with exactly prec bits
        long k = long(prec) - long((m.bit_length() + 1) / 2);
        for(;;) {
            BigNat scaled = k >= 0 ? m.shl(std::size_t(2 * k)) : m.shr(std::size_t(-2 * k));
            if(k < 0) throw std::logic_error("sqrt_prec: negative scaling");
            BigNat t = BigNat::isqrt(scaled);
            std::size_t bl = t.bit_length();
            if(bl < prec) { ++k; continue; }
            if(bl > prec) { --k; continue; }
            bool exact = (t * t == scaled);
            if(!down && !exact) t = t + BigNat(1);
            long re = e / 2 - k;
            BigNat n = t, d(1);
            if(re >= 0) n = n.shl(std::size_t(re)); else d = d.shl(std::size_t(-re));
            return Rat(false, n, d);
        }
    }

    std::string debug() const {
        return (is_negative() ? "-" : "") + std::to_string(num.to_u64()) + "/" + std::to_string(den.to_u64());
    }

private:
    void normalize() {
        if(den.is_zero()) throw std::domain_error("zero denominator");
        if(num.is_zero()) { neg = false; den = BigNat(1); return; }
        BigNat g = BigNat::gcd(num, den);
        if(!(g == BigNat(1))) {
            num = BigNat::divmod(num, g, nullptr);
            den = BigNat::divmod(den, g, nullptr);
        }
    }

    bool neg;
    BigNat num, den;
};

/// Closed interval of exact rationals, used to fold constant subexpressions.
struct RatInterval {
    Rat lo, hi;
    bool undefined = false;
};

} // namespace sid_fe
} // namespace ivarp
