// A double that counts the FP64 operations performed on it (test
// infrastructure: the algorithmic FP64 cost of the reference's per-cell code).
// Counted: add/sub, mul, div, sqrt and other calls (pow with an exponent other
// than 1, 2 or -1, exp).  Not counted: comparisons, negation, fabs, copies.
// pow(x, 2) counts one mul, pow(x, -1) one div and pow(x, 1) nothing: what a
// compiler emits for those constant exponents.
#ifndef MFG_COUNT_DOUBLE_H_
#define MFG_COUNT_DOUBLE_H_
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <istream>

namespace mfg_count {

struct Counts {
    uint64_t add = 0, mul = 0, div = 0, sqrt = 0, other = 0;
};
inline Counts& counts() {
    static Counts c;
    return c;
}

struct CD {
    double v;
    constexpr CD() : v(0.0) {}
    constexpr CD(double x) : v(x) {}
    explicit operator double() const { return v; }
    explicit operator int() const { return (int)v; }
    CD& operator+=(const CD& o) { counts().add++; v += o.v; return *this; }
    CD& operator-=(const CD& o) { counts().add++; v -= o.v; return *this; }
    CD& operator*=(const CD& o) { counts().mul++; v *= o.v; return *this; }
    CD& operator/=(const CD& o) { counts().div++; v /= o.v; return *this; }
    CD operator-() const { return CD(-v); }
    CD operator+() const { return *this; }
};
static_assert(sizeof(CD) == sizeof(double), "CD must alias a double");

inline CD operator+(const CD& a, const CD& b) { counts().add++; return CD(a.v + b.v); }
inline CD operator-(const CD& a, const CD& b) { counts().add++; return CD(a.v - b.v); }
inline CD operator*(const CD& a, const CD& b) { counts().mul++; return CD(a.v * b.v); }
inline CD operator/(const CD& a, const CD& b) { counts().div++; return CD(a.v / b.v); }
inline bool operator<(const CD& a, const CD& b) { return a.v < b.v; }
inline bool operator>(const CD& a, const CD& b) { return a.v > b.v; }
inline bool operator<=(const CD& a, const CD& b) { return a.v <= b.v; }
inline bool operator>=(const CD& a, const CD& b) { return a.v >= b.v; }
inline bool operator==(const CD& a, const CD& b) { return a.v == b.v; }
inline bool operator!=(const CD& a, const CD& b) { return a.v != b.v; }

inline std::istream& operator>>(std::istream& is, CD& a) { return is >> a.v; }

inline CD fabs(const CD& a) { return CD(std::fabs(a.v)); }
inline CD abs(const CD& a) { return CD(std::fabs(a.v)); }
inline CD sqrt(const CD& a) { counts().sqrt++; return CD(std::sqrt(a.v)); }
inline CD exp(const CD& a) { counts().other++; return CD(std::exp(a.v)); }
inline CD pow(const CD& a, const CD& b) {
    if (b.v == 2.0) counts().mul++;
    else if (b.v == -1.0) counts().div++;
    else if (b.v != 1.0) counts().other++;
    return CD(std::pow(a.v, b.v));
}
inline CD pow(const CD& a, double b) { return pow(a, CD(b)); }
inline CD pow(const CD& a, int b) { return pow(a, CD((double)b)); }

}  // namespace mfg_count

namespace std {
// mixed double / CD arguments of std::min and std::max (flux_schemes.H,
// compute_flux_3d.H pass literals such as zeroval beside Real values)
inline mfg_count::CD min(double a, const mfg_count::CD& b) { return b.v < a ? b : mfg_count::CD(a); }
inline mfg_count::CD min(const mfg_count::CD& a, double b) { return b < a.v ? mfg_count::CD(b) : a; }
inline mfg_count::CD max(double a, const mfg_count::CD& b) { return a < b.v ? b : mfg_count::CD(a); }
inline mfg_count::CD max(const mfg_count::CD& a, double b) { return a.v < b ? mfg_count::CD(b) : a; }
using mfg_count::abs;
using mfg_count::exp;
using mfg_count::fabs;
using mfg_count::pow;
using mfg_count::sqrt;
}  // namespace std

#endif
