// Oracle-side correctly rounded hypot (test infrastructure only; never linked into the product).
//
// The reference computes every 2-norm as a chain of std::hypot calls (src/spai.cpp:22-27,
// src/gmres.cpp:18-23, src/ir.cpp:166) and Givens radii with std::hypot (src/gmres.cpp:203).
// glibc's hypot is faithful but not correctly rounded, and its result differs between x86-64
// and aarch64 builds, so the reference's own bits are machine dependent. This oracle pins the
// ideal the reference approximates: hypot rounded to nearest-even from the exact value
// sqrt(a^2+b^2). The decision is made with exact arithmetic (Shewchuk-style expansion sums of
// error-free transformations), with no FMA and no long double, so it gives the same bits on
// every IEEE-754 machine. Compile with -ffp-contract=off.
#pragma once
#include <cmath>
#include <cstdint>
#include <utility>

namespace orc {

// Knuth two-sum: s + e == a + b exactly.
inline void o_two_sum(double a, double b, double &s, double &e) {
    s = a + b;
    const double bv = s - a;
    const double av = s - bv;
    e = (a - av) + (b - bv);
}
// Dekker split and product: p + e == a * b exactly (|a|,|b| well inside range).
inline void o_split(double a, double &hi, double &lo) {
    const double c = 134217729.0 * a;
    const double big = c - a;
    hi = c - big;
    lo = a - hi;
}
inline void o_two_prod(double a, double b, double &p, double &e) {
    p = a * b;
    double ah, al, bh, bl;
    o_split(a, ah, al);
    o_split(b, bh, bl);
    e = ((ah * bh - p) + ah * bl + al * bh) + al * bl;
}
// Exact sign of sum(t[0..n)) using a growing nonoverlapping expansion.
inline int o_exact_sign(const double *t, int n) {
    double e[32];
    int m = 0;
    for (int i = 0; i < n; ++i) {
        double q = t[i];
        for (int j = 0; j < m; ++j) {
            double s, h;
            o_two_sum(q, e[j], s, h);
            e[j] = h;
            q = s;
        }
        e[m++] = q;
    }
    for (int j = m - 1; j >= 0; --j)
        if (e[j] != 0)
            return e[j] > 0 ? 1 : -1;
    return 0;
}
// Sign of (c + sgn*half)^2 - (xx + xxe + yy + yye), everything exact. half is a power of two.
inline int o_midpoint_sign(double c, double half, int sgn, double xx, double xxe, double yy,
                           double yye) {
    double p, pe;
    o_two_prod(c, c, p, pe);
    const double cross = sgn * 2.0 * c * half; // exact: power-of-two scaling
    const double sq = half * half;             // exact
    const double t[8] = {p, pe, cross, sq, -xx, -xxe, -yy, -yye};
    return o_exact_sign(t, 8);
}

// Correctly rounded hypot for binary64. Inputs whose result is subnormal are outside the
// solver's range and are computed with a final ldexp (possible double rounding there only).
inline double cr_hypot(double a, double b) {
    double x = std::fabs(a), y = std::fabs(b);
    if (std::isinf(x) || std::isinf(y))
        return INFINITY;
    if (std::isnan(x) || std::isnan(y))
        return x + y;
    if (x < y)
        std::swap(x, y);
    if (y == 0)
        return x;
    const int ex = std::ilogb(x), ey = std::ilogb(y);
    if (ex - ey > 30)
        return x; // y/x < 2^-29: the exact value rounds to x
    const double xs = std::ldexp(x, -ex), ys = std::ldexp(y, -ex);
    double xx, xxe, yy, yye;
    o_two_prod(xs, xs, xx, xxe);
    o_two_prod(ys, ys, yy, yye);
    double c = std::sqrt(xx + yy);
    {
        // Filter: S - c^2 to ~2^-100 absolute (sh - p is exact by Sterbenz); if the implied
        // correction is clearly inside c's rounding interval, c is the correctly rounded root.
        double p, pe, sh, sl;
        o_two_prod(c, c, p, pe);
        o_two_sum(xx, yy, sh, sl);
        const double r = (sh - p) + ((sl - pe) + (xxe + yye));
        const double d = r / (c + c);
        const double hu = (std::nextafter(c, INFINITY) - c) * 0.5;
        const double hd = (c - std::nextafter(c, 0.0)) * 0.5;
        const double tol = 0x1p-80;
        if (d < hu - tol && d > -hd + tol)
            return std::ldexp(c, ex);
    }
    // Walk to the neighbour whose rounding interval holds the exact root. Each step decides with
    // exact signs only, so no tolerance is involved.
    for (int guard = 0; guard < 8; ++guard) {
        const double up = std::nextafter(c, INFINITY), dn = std::nextafter(c, 0.0);
        const double hu = (up - c) * 0.5, hd = (c - dn) * 0.5;
        const int su = o_midpoint_sign(c, hu, +1, xx, xxe, yy, yye);
        if (su < 0) { // exact root above upper midpoint
            c = up;
            continue;
        }
        const int sd = o_midpoint_sign(c, hd, -1, xx, xxe, yy, yye);
        if (sd > 0) { // exact root below lower midpoint
            c = dn;
            continue;
        }
        // Root inside [c - hd, c + hu]; ties go to the even neighbour.
        if (su == 0 || sd == 0) {
            const double other = su == 0 ? up : dn;
            std::uint64_t bc, bo;
            static_assert(sizeof(double) == 8, "binary64");
            __builtin_memcpy(&bc, &c, 8);
            __builtin_memcpy(&bo, &other, 8);
            if (bc & 1u)
                c = other;
        }
        break;
    }
    return std::ldexp(c, ex);
}

// Correctly rounded hypot for binary32: squares are exact in binary64; the binary64 root is
// rounded once to binary32 unless it lies within 2^-50 (relative) of a binary32 midpoint, where
// the exact midpoint comparison decides.
inline float cr_hypotf(float a, float b) {
    const double x = std::fabs(static_cast<double>(a)), y = std::fabs(static_cast<double>(b));
    if (std::isinf(x) || std::isinf(y))
        return INFINITY;
    if (std::isnan(x) || std::isnan(y))
        return static_cast<float>(x + y);
    const double xx = x * x, yy = y * y; // exact (24-bit significands)
    double s, se;
    o_two_sum(xx, yy, s, se);
    const double r = std::sqrt(s);
    float f = static_cast<float>(r);
    if (std::isinf(f))
        return f;
    const float fu = std::nextafter(f, INFINITY), fd = std::nextafter(f, 0.0f);
    // Binary32 midpoints are exact binary64 numbers (25 significant bits); their squares are too.
    const double mids[2] = {(static_cast<double>(f) + static_cast<double>(fu)) * 0.5,
                            (static_cast<double>(f) + static_cast<double>(fd)) * 0.5};
    for (int side = 0; side < 2; ++side) {
        const double m = mids[side];
        const double m2 = m * m; // exact: 50 significant bits
        const double t[3] = {m2, -s, -se};
        const int sg = o_exact_sign(t, 3); // sign of m^2 - (x^2 + y^2)
        if (side == 0 && sg < 0)
            return fu; // exact root above the upper midpoint
        if (side == 0 && sg == 0) {
            std::uint32_t bf;
            __builtin_memcpy(&bf, &f, 4);
            return (bf & 1u) ? fu : f;
        }
        if (side == 1 && sg > 0)
            return fd;
        if (side == 1 && sg == 0) {
            std::uint32_t bf;
            __builtin_memcpy(&bf, &f, 4);
            return (bf & 1u) ? fd : f;
        }
    }
    return f;
}

#ifdef ORACLE_PLATFORM_HYPOT
// Diagnostic build only: the platform's std::hypot, as the reference calls it. Used to show that
// oracle/reference differences come from hypot rounding alone.
inline double o_hypot(double a, double b) {
    return std::hypot(a, b);
}
inline float o_hypot(float a, float b) {
    return std::hypot(a, b);
}
#else
inline double o_hypot(double a, double b) {
    return cr_hypot(a, b);
}
inline float o_hypot(float a, float b) {
    return cr_hypotf(a, b);
}
#endif

} // namespace orc
