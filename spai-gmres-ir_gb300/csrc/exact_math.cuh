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

#ifdef __CUDA_ARCH__
// Device fast path for normal operands: exponents and power-of-two scales from the bit fields,
// and a division-free acceptance test. With x >= y scaled to xs in [1, 2), the candidate
// c = fl(sqrt(fl(xs^2 + ys^2))) is the correctly rounded value iff |t - c| < h, t the exact
// value and h the distance from c to the nearer rounding midpoint (ulp(c)/2, or ulp(c)/4 below
// a power of two). Since |t - c| = |R| / (t + c) with R = xs^2 + ys^2 - c^2 (computed to within
// a few units of 2^-48 c^2 by error-free transformations), |R| < 2 c h (1 - 2^-16) is sufficient.
// Returns false (nothing decided) when an operand is subnormal or too large for the scaling, or
// when the test does not accept; the caller then takes the general path, so the result is the
// same correctly rounded value either way.
__device__ __forceinline__ bool cr_hypot_fast(float x, float y, float &out) {
    const unsigned bx = __float_as_uint(x), by = __float_as_uint(y);
    const int fx = static_cast<int>(bx >> 23), fy = static_cast<int>(by >> 23);
    if (fy == 0 || fx > 253)
        return false;
    if (fx - fy > 14) { // y/x < 2^-14: the exact value rounds to x
        out = x;
        return true;
    }
    const float scale = __uint_as_float(static_cast<unsigned>(254 - fx) << 23); // 2^(127 - fx)
    const float xs = x * scale, ys = y * scale;
    float xx, xxe, yy, yye, p, pe, sh, sl;
    em_two_prod(xs, xs, xx, xxe);
    em_two_prod(ys, ys, yy, yye);
    const float c = __fsqrt_rn(__fadd_rn(xx, yy));
    em_two_prod(c, c, p, pe);
    em_two_sum(xx, yy, sh, sl);
    const float r = __fadd_rn(__fsub_rn(sh, p), __fadd_rn(__fsub_rn(sl, pe), __fadd_rn(xxe, yye)));
    const unsigned bc = __float_as_uint(c);
    const unsigned hb = (bc & 0x7f800000u) - (24u << 23) - ((bc & 0x007fffffu) == 0 ? (1u << 23) : 0u);
    const float thr = __fmul_rn(__fmul_rn(__fadd_rn(c, c), __uint_as_float(hb)), 0.9999847412109375f);
    if (!(fabsf(r) < thr))
        return false;
    out = __fmul_rn(c, __uint_as_float(static_cast<unsigned>(fx) << 23)); // c * 2^(fx - 127), exact
    return true;
}
__device__ __forceinline__ bool cr_hypot_fast(double x, double y, double &out) {
    const unsigned long long bx = static_cast<unsigned long long>(__double_as_longlong(x));
    const unsigned long long by = static_cast<unsigned long long>(__double_as_longlong(y));
    const int fx = static_cast<int>(bx >> 52), fy = static_cast<int>(by >> 52);
    if (fy == 0 || fx > 2045)
        return false;
    if (fx - fy > 30) {
        out = x;
        return true;
    }
    const double scale = __longlong_as_double(static_cast<long long>(2046 - fx) << 52); // 2^(1023 - fx)
    const double xs = x * scale, ys = y * scale;
    double xx, xxe, yy, yye, p, pe, sh, sl;
    em_two_prod(xs, xs, xx, xxe);
    em_two_prod(ys, ys, yy, yye);
    const double c = __dsqrt_rn(__dadd_rn(xx, yy));
    em_two_prod(c, c, p, pe);
    em_two_sum(xx, yy, sh, sl);
    const double r = __dadd_rn(__dsub_rn(sh, p), __dadd_rn(__dsub_rn(sl, pe), __dadd_rn(xxe, yye)));
    const unsigned long long bc = static_cast<unsigned long long>(__double_as_longlong(c));
    const unsigned long long hb = (bc & 0x7ff0000000000000ull) - (53ull << 52) -
                                  ((bc & 0x000fffffffffffffull) == 0 ? (1ull << 52) : 0ull);
    const double thr = __dmul_rn(__dmul_rn(__dadd_rn(c, c), __longlong_as_double(static_cast<long long>(hb))),
                                 0.99999999999909050530);
    if (!(fabs(r) < thr))
        return false;
    out = __dmul_rn(c, __longlong_as_double(static_cast<long long>(fx) << 52)); // c * 2^(fx - 1023)
    return true;
}
#endif

#ifdef __CUDACC__
#define SPAI_HD_COLD __host__ __device__ __noinline__
#else
#define SPAI_HD_COLD inline
#endif

// General path for x >= y > 0 finite (out of line on the device: it runs rarely there, and
// keeping it out of the callers keeps the fit kernels' hot code small).
template <class T> SPAI_HD_COLD T cr_hypot_general(T x, T y) {
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
#ifdef __CUDA_ARCH__
    {
        T fast;
        if (cr_hypot_fast(x, y, fast))
            return fast;
    }
#endif
    return cr_hypot_general(x, y);
}

#ifdef __CUDACC__
// One step of a norm chain, c <- cr_hypot(c, a) with c >= 0, carrying c's square as the
// unevaluated exact sum cc + cce (error-free product). The square of the new value is exactly the
// product the acceptance test of the step forms anyway, so the next step starts from the sum of
// squares directly: the chain's dependency path is one addition, one square root, one exact
// product and the test, with no ordering, scaling or unscaling of the operands.
//
// The test is the one of cr_hypot_fast on unscaled operands. Both c and |a| lie in
// [2^-40, 2^40] on the fast path, so every square and every product error term is a normal
// number (no bits lost), and the computed remainder R of (c^2 + a^2) - c'^2 is within about
// 2^-48 c'^2 of the exact one, far inside the 2^-16 margin of the threshold. Outside that range,
// and when the test rejects, the step calls cr_hypot; when |a| < 2^-14 c the correctly rounded
// value is c itself (the rule cr_hypot applies too). Every step therefore returns exactly
// cr_hypot(c, a), bit for bit, for every input including zeros, subnormals, infinities and NaNs.
template <class T> struct NormChain {
    T c = 0, cc = 0, cce = 0;
};
__device__ __forceinline__ void norm_chain_step(NormChain<float> &st, float a) {
    const float y = fabsf(a);
    const int fy = static_cast<int>(__float_as_uint(y) >> 23);
    const int fc = static_cast<int>(__float_as_uint(st.c) >> 23);
    if (fc - fy > 14)
        return;
    if (static_cast<unsigned>(fc - 87) <= 80u && static_cast<unsigned>(fy - 87) <= 80u) {
        const float yy = __fmul_rn(y, y), yye = __fmaf_rn(y, y, -yy);
        const float s = __fadd_rn(st.cc, yy);
        const float c = __fsqrt_rn(s);
        const float p = __fmul_rn(c, c), pe = __fmaf_rn(c, c, -p);
        const float bv = __fsub_rn(s, st.cc), av = __fsub_rn(s, bv);
        const float sl = __fadd_rn(__fsub_rn(st.cc, av), __fsub_rn(yy, bv));
        const float r = __fadd_rn(__fsub_rn(s, p), __fadd_rn(__fsub_rn(sl, pe), __fadd_rn(st.cce, yye)));
        const unsigned bc = __float_as_uint(c);
        const unsigned hb = (bc & 0x7f800000u) - (24u << 23) - ((bc & 0x007fffffu) == 0 ? (1u << 23) : 0u);
        const float thr = __fmul_rn(__fmul_rn(__fadd_rn(c, c), __uint_as_float(hb)), 0.9999847412109375f);
        if (fabsf(r) < thr) {
            st.c = c;
            st.cc = p;
            st.cce = pe;
            return;
        }
    }
    st.c = cr_hypot<float>(st.c, y);
    st.cc = __fmul_rn(st.c, st.c);
    st.cce = __fmaf_rn(st.c, st.c, -st.cc);
}
__device__ __forceinline__ void norm_chain_step(NormChain<double> &st, double a) {
    const double y = fabs(a);
    const int fy = static_cast<int>(static_cast<unsigned long long>(__double_as_longlong(y)) >> 52);
    const int fc = static_cast<int>(static_cast<unsigned long long>(__double_as_longlong(st.c)) >> 52);
    if (fc - fy > 30)
        return;
    if (static_cast<unsigned>(fc - 623) <= 800u && static_cast<unsigned>(fy - 623) <= 800u) {
        const double yy = __dmul_rn(y, y), yye = __fma_rn(y, y, -yy);
        const double s = __dadd_rn(st.cc, yy);
        const double c = __dsqrt_rn(s);
        const double p = __dmul_rn(c, c), pe = __fma_rn(c, c, -p);
        const double bv = __dsub_rn(s, st.cc), av = __dsub_rn(s, bv);
        const double sl = __dadd_rn(__dsub_rn(st.cc, av), __dsub_rn(yy, bv));
        const double r = __dadd_rn(__dsub_rn(s, p), __dadd_rn(__dsub_rn(sl, pe), __dadd_rn(st.cce, yye)));
        const unsigned long long bc = static_cast<unsigned long long>(__double_as_longlong(c));
        const unsigned long long hb = (bc & 0x7ff0000000000000ull) - (53ull << 52) -
                                      ((bc & 0x000fffffffffffffull) == 0 ? (1ull << 52) : 0ull);
        const double thr = __dmul_rn(__dmul_rn(__dadd_rn(c, c), __longlong_as_double(static_cast<long long>(hb))),
                                     0.99999999999909050530);
        if (fabs(r) < thr) {
            st.c = c;
            st.cc = p;
            st.cce = pe;
            return;
        }
    }
    st.c = cr_hypot<double>(st.c, y);
    st.cc = __dmul_rn(st.c, st.c);
    st.cce = __fma_rn(st.c, st.c, -st.cc);
}
// The chain step from a running norm c >= 0 (its square formed here), for tests.
template <class T> __device__ __forceinline__ T norm_chain_step_from(T c, T a) {
    NormChain<T> st;
    st.c = c;
    em_two_prod(c, c, st.cc, st.cce);
    norm_chain_step(st, a);
    return st.c;
}
#endif



} // namespace spai
