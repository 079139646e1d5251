// Double-double arithmetic (about 106 significant bits) for building the
// element tables on the host, then rounding each entry once to the run's
// type. The reference builds the same tables in 512-bit BigFloat and notes
// that Float64x2 (the same double-double representation) rounds to the same
// Float64/Float32 values (src/evolution.jl:811-842, "table_type"). Plain
// IEEE operations only, so x86 and Arm hosts give identical bits; requires
// that the compiler does not contract a*b+c into an FMA, which the build
// flags guarantee (-ffp-contract=off).
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

namespace twoldg {

struct dd {
    double hi, lo;
    dd() : hi(0), lo(0) {}
    dd(double h) : hi(h), lo(0) {}
    dd(double h, double l) : hi(h), lo(l) {}
};

inline dd two_sum(double a, double b) {
    double s = a + b;
    double bb = s - a;
    double e = (a - (s - bb)) + (b - bb);
    return dd(s, e);
}

inline dd quick_two_sum(double a, double b) {
    double s = a + b;
    double e = b - (s - a);
    return dd(s, e);
}

// Dekker's exact product by Veltkamp splitting (no FMA needed).
inline void split(double a, double& hi, double& lo) {
    const double c = 134217729.0;  // 2^27 + 1
    double t = c * a;
    hi = t - (t - a);
    lo = a - hi;
}

inline dd two_prod(double a, double b) {
    double p = a * b;
    double ah, al, bh, bl;
    split(a, ah, al);
    split(b, bh, bl);
    double e = ((ah * bh - p) + ah * bl + al * bh) + al * bl;
    return dd(p, e);
}

inline dd operator+(dd a, dd b) {
    dd s = two_sum(a.hi, b.hi);
    dd t = two_sum(a.lo, b.lo);
    s.lo += t.hi;
    s = quick_two_sum(s.hi, s.lo);
    s.lo += t.lo;
    return quick_two_sum(s.hi, s.lo);
}

inline dd operator-(dd a) { return dd(-a.hi, -a.lo); }
inline dd operator-(dd a, dd b) { return a + (-b); }

inline dd operator*(dd a, dd b) {
    dd p = two_prod(a.hi, b.hi);
    p.lo += a.hi * b.lo + a.lo * b.hi;
    return quick_two_sum(p.hi, p.lo);
}

inline dd operator/(dd a, dd b) {
    double q1 = a.hi / b.hi;
    dd r = a - b * dd(q1);
    double q2 = r.hi / b.hi;
    r = r - b * dd(q2);
    double q3 = r.hi / b.hi;
    dd q = quick_two_sum(q1, q2);
    return q + dd(q3);
}

inline dd& operator+=(dd& a, dd b) { a = a + b; return a; }
inline dd& operator-=(dd& a, dd b) { a = a - b; return a; }
inline dd& operator*=(dd& a, dd b) { a = a * b; return a; }

inline bool operator<(dd a, dd b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
inline dd dd_abs(dd a) { return a.hi < 0 ? -a : a; }

// Rounding of a normalised double-double (|lo| <= ulp(hi)/2) to double:
// hi is already the nearest double to hi + lo.
inline double to_double(dd a) { return a.hi; }

// Correct rounding to float. (float)hi is right unless hi sits exactly on
// the midpoint between two floats, where the sign of lo breaks the tie.
inline float to_float(dd a) {
    float f = (float)a.hi;
    double fd = (double)f;
    if (fd == a.hi || a.lo == 0.0) return f;
    float other = (a.hi > fd) ? std::nextafter(f, INFINITY) : std::nextafter(f, -INFINITY);
    double mid = 0.5 * (fd + (double)other);  // exact: both are floats
    if (a.hi != mid) return f;
    // hi is the midpoint: the true value lies on lo's side of it
    if (a.lo > 0) return (double)other > fd ? other : f;
    return (double)other < fd ? other : f;
}

}  // namespace twoldg
