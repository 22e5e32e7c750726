// Correctly rounded hypot for the SPAI column fits, usable from device and host code.
//
// The reference forms every 2-norm of the SPAI least-squares fit as a left-to-right chain of
// hypot calls (src/spai.cpp:22-27): the Householder column length, the reflector norm and the
// fitted residual norm. Reproducing that chain with a correctly rounded hypot makes the device
// fit bit-identical to a CPU restatement of the same chain on any IEEE-754 machine; the choice
// of a correctly rounded hypot (rather than one platform's libm) is what makes this possible.
//
// Method: scale by a power of two, take the rounded square root of the rounded sum of squares,
// then check the candidate against the exact value with error-free transformations (Knuth
// two-sum; fma two-product on the device, Dekker's product on the host). A cheap double-length
// filter accepts almost every candidate; near a rounding midpoint the exact sign of
// (midpoint^2 - x^2 - y^2) is taken from a nonoverlapping expansion (Shewchuk 1997), so no
// tolerance decides the result. The binary32 version uses binary32 arithmetic only.
// Results in the subnormal range may carry one extra rounding in the final ldexp.
#pragma once

#ifdef __CUDACC__
#define SPAI_HD __host__ __device__ __forceinline__
#else
#define SPAI_HD inline
#endif

#include <cmath>
#include <cstdint>
#include <cstring>

namespace spai {

template <class T> SPAI_HD T em_fma(T a, T b, T c);
template <> SPAI_HD double em_fma<double>(double a, double b, double c) {
    return fma(a, b, c);
}
template <> SPAI_HD float em_fma<float>(float a, float b, float c) {
    return fmaf(a, b, c);
}

template <class T> SPAI_HD void em_two_sum(T a, T b, T &s, T &e) {
    s = a + b;
    const T bv = s - a;
    const T av = s - bv;
    e = (a - av) + (b - bv);
}

template <class T> SPAI_HD void em_two_prod(T a, T b, T &p, T &e) {
#ifdef __CUDA_ARCH__
    p = a * b;
    e = em_fma<T>(a, b, -p);
#else
    // Dekker/Veltkamp split: exact without a hardware fma (host builds use -ffp-contract=off).
    const T splitter = sizeof(T) == 8 ? T(134217729.0) : T(4097.0);
    p = a * b;
    T c = splitter * a, big = c - a, ah = c - big, al = a - ah;
    c = splitter * b;
    big = c - b;
    const T bh = c - big, bl = b - bh;
    e = ((ah * bh - p) + ah * bl + al * bh) + al * bl;
#endif
}

template <class T> SPAI_HD int em_exact_sign(const T *t, int n) {
    T e[12];
    int m = 0;
    for (int i = 0; i < n; ++i) {
        T q = t[i];
        for (int j = 0; j < m; ++j) {
            T s, h;
            em_two_sum(q, e[j], s, h);
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

template <class T> SPAI_HD T em_next_up(T x);
template <class T> SPAI_HD T em_next_down(T x);
template <> SPAI_HD double em_next_up<double>(double x) {
    uint64_t b;
    memcpy(&b, &x, 8);
    ++b; // x positive and finite here
    memcpy(&x, &b, 8);
    return x;
}
template <> SPAI_HD double em_next_down<double>(double x) {
    uint64_t b;
    memcpy(&b, &x, 8);
    --b;
    memcpy(&x, &b, 8);
    return x;
}
template <> SPAI_HD float em_next_up<float>(float x) {
    uint32_t b;
    memcpy(&b, &x, 4);
    ++b;
    memcpy(&x, &b, 4);
    return x;
}
template <> SPAI_HD float em_next_down<float>(float x) {
    uint32_t b;
    memcpy(&b, &x, 4);
    --b;
    memcpy(&x, &b, 4);
    return x;
}
template <class T> SPAI_HD bool em_odd(T x) {
    if (sizeof(T) == 8) {
        uint64_t b;
        memcpy(&b, &x, 8);
        return (b & 1u) != 0;
    }
    uint32_t b;
    memcpy(&b, &x, 4);
    return (b & 1u) != 0;
}

template <class T> SPAI_HD int em_ilogb(T x) {
    return std::ilogb(x);
}
template <class T> SPAI_HD T em_ldexp(T x, int e) {
    return std::ldexp(x, e);
}
template <class T> SPAI_HD T em_sqrt(T x) {
    return std::sqrt(x);
}
#ifdef __CUDA_ARCH__
template <> SPAI_HD int em_ilogb<float>(float x) {
    return ilogbf(x);
}
template <> SPAI_HD float em_ldexp<float>(float x, int e) {
    return ldexpf(x, e);
}
template <> SPAI_HD float em_sqrt<float>(float x) {
    return __fsqrt_rn(x);
}
template <> SPAI_HD double em_sqrt<double>(double x) {
    return __dsqrt_rn(x);
}
#endif

// Sign of (c + sgn*half)^2 - (xx + xxe + yy + yye); all terms exact.
template <class T>
SPAI_HD int em_midpoint_sign(T c, T half, int sgn, T xx, T xxe, T yy, T yye) {
    T p, pe;
    em_two_prod(c, c, p, pe);
    const T cross = T(sgn) * T(2) * c * half;
    const T sq = half * half;
    const T t[8] = {p, pe, cross, sq, -xx, -xxe, -yy, -yye};
    return em_exact_sign(t, 8);
}

// Correctly rounded (to nearest, ties to even) hypot in T = double or float.
template <class T> SPAI_HD T cr_hypot(T a, T b) {
    T x = std::fabs(a), y = std::fabs(b);
    if (std::isinf(x) || std::isinf(y))
        return T(INFINITY);
    if (std::isnan(x) || std::isnan(y))
        return x + y;
    if (x < y) {
        const T t = x;
        x = y;
        y = t;
    }
    if (y == 0)
        return x;
    const int ex = em_ilogb(x), ey = em_ilogb(y);
    // y/x below 2^-(p/2+2) with p the significand width: the exact value rounds to x.
    if (ex - ey > (sizeof(T) == 8 ? 30 : 14))
        return x;
    const T xs = em_ldexp(x, -ex), ys = em_ldexp(y, -ex);
    T xx, xxe, yy, yye;
    em_two_prod(xs, xs, xx, xxe);
    em_two_prod(ys, ys, yy, yye);
    T c = em_sqrt(xx + yy);
    {
        T p, pe, sh, sl;
        em_two_prod(c, c, p, pe);
        em_two_sum(xx, yy, sh, sl);
        const T r = (sh - p) + ((sl - pe) + (xxe + yye));
        const T d = r / (c + c);
        const T hu = (em_next_up(c) - c) * T(0.5);
        const T hd = (c - em_next_down(c)) * T(0.5);
        const T tol = sizeof(T) == 8 ? T(0x1p-80) : T(0x1p-40);
        if (d < hu - tol && d > -hd + tol)
            return em_ldexp(c, ex);
    }
    for (int guard = 0; guard < 8; ++guard) {
        const T up = em_next_up(c), dn = em_next_down(c);
        const T hu = (up - c) * T(0.5), hd = (c - dn) * T(0.5);
        const int su = em_midpoint_sign(c, hu, +1, xx, xxe, yy, yye);
        if (su < 0) {
            c = up;
            continue;
        }
        const int sd = em_midpoint_sign(c, hd, -1, xx, xxe, yy, yye);
        if (sd > 0) {
            c = dn;
            continue;
        }
        if ((su == 0 || sd == 0) && em_odd(c))
            c = su == 0 ? up : dn;
        break;
    }
    return em_ldexp(c, ex);
}

} // namespace spai
