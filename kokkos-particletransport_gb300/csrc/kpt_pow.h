/* kpt_pow: the FP64 power function of the plain FP64 push, one
 * implementation for the GPU (CUDA device code), the host library and the
 * CPU oracle (C and C++), so that all of them round every power the same way.
 *
 * Why a project pow.  The plain FP64 push is checked against the reference's
 * own code to 1e-10 over a whole MHD interval.  The focused push's
 * pitch-angle dynamics amplify last-bit differences over thousands of
 * substeps, and CUDA's pow and the host C library's pow, each accurate to
 * about an ulp, do not round alike.  Every caller here therefore computes
 * x^y with this function, built only from operations that IEEE 754 rounds
 * exactly once on every platform (add, subtract, multiply, divide, fused
 * multiply-add), each written as an explicit call so no compiler can contract
 * or reorder them: the result is the same bit pattern on the host and on the
 * GPU.
 *
 * Method (exp(y ln x) with double-double intermediates, as in the classical
 * argument-reduction schemes, e.g. J.-M. Muller, "Elementary Functions:
 * Algorithms and Implementation", chapters on logarithm and exponential):
 *  - ln x: x = 2^e m with m in [sqrt(1/2), sqrt(2)); s = (m - 1)/(m + 1) to
 *    double-double accuracy; ln m = 2 atanh(s) = 2s + s^3 P(s^2) with
 *    P(z) = sum_{k=1..12} 2/(2k+1) z^(k-1) (|s| <= 0.1716, truncation below
 *    2^-62 of 2s); ln x = e ln2 + ln m with ln2 split into a 42-bit head (e ln2_hi
 *    exact for every binary64 exponent) and a tail.
 *  - t = y ln x as a double-double (head y ln x_hi, exact product error by
 *    fma, plus y ln x_lo).
 *  - exp t: k = nearest integer to t / ln2, r = t - k ln2 (the head
 *    subtraction exact), exp r = 1 + r + r^2/2 (exact square by fma)
 *    + r^3 Q(r), Q(r) = sum_{n=3..15} r^(n-3)/n! (|r| <= 0.347, truncation
 *    below 2^-62), then the scale 2^k.
 * Error below 0.52 ulp for |y ln x| up to tens (the single rounding of the
 * final sum plus ~2^-58 relative from the truncated series and the
 * double-double tails), pinned against 80-digit evaluations and against the
 * host C library's pow by the tests.
 *
 * Special values follow C99 Annex F (F.9.4.4) for pow.
 *
 * Host code that includes this header must be compiled without floating
 * point contraction (-ffp-contract=off), as the library's host code and the
 * oracle are; device code uses the rounding intrinsics and is immune.
 */
#ifndef KPT_POW_H
#define KPT_POW_H

#include <stdint.h>
#include <string.h>
#ifndef __CUDA_ARCH__
#include <math.h>
#endif

#if defined(__CUDACC__)
#define KPT_POW_FN __host__ __device__ static inline
#else
#define KPT_POW_FN static inline
#endif

#if defined(__CUDA_ARCH__)
#define KPT_P_ADD(a, b) __dadd_rn((a), (b))
#define KPT_P_SUB(a, b) __dsub_rn((a), (b))
#define KPT_P_MUL(a, b) __dmul_rn((a), (b))
#define KPT_P_DIV(a, b) __ddiv_rn((a), (b))
#define KPT_P_FMA(a, b, c) __fma_rn((a), (b), (c))
#define KPT_P_FLOOR(a) floor(a)
#else
#define KPT_P_ADD(a, b) ((a) + (b))
#define KPT_P_SUB(a, b) ((a) - (b))
#define KPT_P_MUL(a, b) ((a) * (b))
#define KPT_P_DIV(a, b) ((a) / (b))
#define KPT_P_FMA(a, b, c) fma((a), (b), (c))
#define KPT_P_FLOOR(a) floor(a)
#endif

KPT_POW_FN uint64_t kpt_pow_bits(double x) {
    uint64_t u;
    memcpy(&u, &x, sizeof(u));
    return u;
}

KPT_POW_FN double kpt_pow_from_bits(uint64_t u) {
    double x;
    memcpy(&x, &u, sizeof(x));
    return x;
}

/* 2^k for -1022 <= k <= 1023 */
KPT_POW_FN double kpt_pow_two(int k) {
    return kpt_pow_from_bits((uint64_t)(k + 1023) << 52);
}

/* ln(x) as hi + lo for finite x > 0 (subnormals included). */
KPT_POW_FN void kpt_pow_log(double x, double* hi, double* lo) {
    /* ln 2 = LN2_HI + LN2_LO, LN2_HI with 42 significant bits */
    const double LN2_HI = 0x1.62e42fefa3800p-1;
    const double LN2_LO = 0x1.ef35793c76730p-45;
    const double SQRT2 = 0x1.6a09e667f3bcdp+0;
    uint64_t u = kpt_pow_bits(x);
    int e = (int)((u >> 52) & 0x7ff);
    if (e == 0) { /* subnormal: scale into the normal range (exact) */
        u = kpt_pow_bits(KPT_P_MUL(x, 0x1p54));
        e = (int)((u >> 52) & 0x7ff) - 54;
    }
    e -= 1023;
    double m = kpt_pow_from_bits((u & 0x000fffffffffffffULL) | 0x3ff0000000000000ULL);
    if (m > SQRT2) {
        m = KPT_P_MUL(m, 0.5);
        e += 1;
    }
    const double f = KPT_P_SUB(m, 1.0); /* exact (Sterbenz) */
    /* d = m + 1 as a double-double (two-sum) */
    const double d_hi = KPT_P_ADD(m, 1.0);
    const double bv = KPT_P_SUB(d_hi, m);
    const double d_lo = KPT_P_ADD(KPT_P_SUB(m, KPT_P_SUB(d_hi, bv)), KPT_P_SUB(1.0, bv));
    /* s = f / d to double-double accuracy */
    const double s_hi = KPT_P_DIV(f, d_hi);
    double rem = KPT_P_FMA(-s_hi, d_hi, f); /* exact */
    rem = KPT_P_SUB(rem, KPT_P_MUL(s_hi, d_lo));
    const double s_lo = KPT_P_DIV(rem, d_hi);
    /* P(z) = sum_{k=1..12} 2/(2k+1) z^(k-1), z = s^2 */
    const double z = KPT_P_MUL(s_hi, s_hi);
    double p = 0x1.47ae147ae147bp-4;       /* 2/25 */
    p = KPT_P_FMA(p, z, 0x1.642c8590b2164p-4); /* 2/23 */
    p = KPT_P_FMA(p, z, 0x1.8618618618618p-4); /* 2/21 */
    p = KPT_P_FMA(p, z, 0x1.af286bca1af28p-4); /* 2/19 */
    p = KPT_P_FMA(p, z, 0x1.e1e1e1e1e1e1ep-4); /* 2/17 */
    p = KPT_P_FMA(p, z, 0x1.1111111111111p-3); /* 2/15 */
    p = KPT_P_FMA(p, z, 0x1.3b13b13b13b14p-3); /* 2/13 */
    p = KPT_P_FMA(p, z, 0x1.745d1745d1746p-3); /* 2/11 */
    p = KPT_P_FMA(p, z, 0x1.c71c71c71c71cp-3); /* 2/9 */
    p = KPT_P_FMA(p, z, 0x1.2492492492492p-2); /* 2/7 */
    p = KPT_P_FMA(p, z, 0x1.999999999999ap-2); /* 2/5 */
    p = KPT_P_FMA(p, z, 0x1.5555555555555p-1); /* 2/3 */
    const double tail = KPT_P_MUL(KPT_P_MUL(s_hi, z), p);
    /* ln m = 2 s_hi + (2 s_lo + tail), |2 s_hi| >= |rest| */
    const double lm_hi0 = KPT_P_MUL(2.0, s_hi);
    const double lm_rest = KPT_P_ADD(KPT_P_MUL(2.0, s_lo), tail);
    const double lm_hi = KPT_P_ADD(lm_hi0, lm_rest);
    const double lm_lo = KPT_P_SUB(lm_rest, KPT_P_SUB(lm_hi, lm_hi0));
    /* + e ln2 (e * LN2_HI exact) */
    const double ed = (double)e;
    const double a = KPT_P_MUL(ed, LN2_HI);
    const double sum = KPT_P_ADD(a, lm_hi);
    const double bb = KPT_P_SUB(sum, a);
    const double err = KPT_P_ADD(KPT_P_SUB(a, KPT_P_SUB(sum, bb)), KPT_P_SUB(lm_hi, bb));
    const double low = KPT_P_ADD(KPT_P_ADD(err, lm_lo), KPT_P_MUL(ed, LN2_LO));
    const double h = KPT_P_ADD(sum, low);
    *hi = h;
    *lo = KPT_P_SUB(low, KPT_P_SUB(h, sum));
}

/* exp(hi + lo) for a double-double argument; hi within the finite range. */
KPT_POW_FN double kpt_pow_exp(double hi, double lo) {
    const double LN2_HI = 0x1.62e42fefa3800p-1;
    const double LN2_LO = 0x1.ef35793c76730p-45;
    const double INV_LN2 = 0x1.71547652b82fep+0;
    const double SHIFTER = 0x1.8p52; /* round to nearest integer by addition */
    if (hi > 709.8) {
        return kpt_pow_from_bits(0x7ff0000000000000ULL);
    }
    if (hi < -745.2) {
        return 0.0;
    }
    const double kd = KPT_P_SUB(KPT_P_ADD(KPT_P_MUL(hi, INV_LN2), SHIFTER), SHIFTER);
    const int k = (int)kd;
    /* r = hi - k ln2 + lo; the head subtraction is exact */
    const double r_head = KPT_P_SUB(hi, KPT_P_MUL(kd, LN2_HI));
    const double r_tail = KPT_P_SUB(lo, KPT_P_MUL(kd, LN2_LO));
    const double r_hi = KPT_P_ADD(r_head, r_tail);
    const double bv = KPT_P_SUB(r_hi, r_head);
    const double r_lo =
        KPT_P_ADD(KPT_P_SUB(r_head, KPT_P_SUB(r_hi, bv)), KPT_P_SUB(r_tail, bv));
    /* Q(r) = sum_{n=3..15} r^(n-3)/n! */
    double q = 0x1.ae7f3e733b81fp-41;           /* 1/15! */
    q = KPT_P_FMA(q, r_hi, 0x1.93974a8c07c9dp-37); /* 1/14! */
    q = KPT_P_FMA(q, r_hi, 0x1.6124613a86d09p-33); /* 1/13! */
    q = KPT_P_FMA(q, r_hi, 0x1.1eed8eff8d898p-29); /* 1/12! */
    q = KPT_P_FMA(q, r_hi, 0x1.ae64567f544e4p-26); /* 1/11! */
    q = KPT_P_FMA(q, r_hi, 0x1.27e4fb7789f5cp-22); /* 1/10! */
    q = KPT_P_FMA(q, r_hi, 0x1.71de3a556c734p-19); /* 1/9! */
    q = KPT_P_FMA(q, r_hi, 0x1.a01a01a01a01ap-16); /* 1/8! */
    q = KPT_P_FMA(q, r_hi, 0x1.a01a01a01a01ap-13); /* 1/7! */
    q = KPT_P_FMA(q, r_hi, 0x1.6c16c16c16c17p-10); /* 1/6! */
    q = KPT_P_FMA(q, r_hi, 0x1.1111111111111p-7);  /* 1/5! */
    q = KPT_P_FMA(q, r_hi, 0x1.5555555555555p-5);  /* 1/4! */
    q = KPT_P_FMA(q, r_hi, 0x1.5555555555555p-3);  /* 1/3! */
    /* r^2 / 2 exactly (fma product error), scaled by 1/2 exactly */
    const double sq = KPT_P_MUL(r_hi, r_hi);
    const double sq_err = KPT_P_FMA(r_hi, r_hi, -sq);
    const double half_sq = KPT_P_MUL(sq, 0.5);
    const double half_sq_err = KPT_P_MUL(sq_err, 0.5);
    const double cube_q = KPT_P_MUL(KPT_P_MUL(sq, r_hi), q);
    /* 1 + r_hi (|1| >= |r_hi|), then + r^2/2 */
    const double a_hi = KPT_P_ADD(1.0, r_hi);
    const double a_lo = KPT_P_SUB(r_hi, KPT_P_SUB(a_hi, 1.0));
    const double b_hi = KPT_P_ADD(a_hi, half_sq);
    const double bb = KPT_P_SUB(b_hi, a_hi);
    const double b_lo =
        KPT_P_ADD(KPT_P_SUB(a_hi, KPT_P_SUB(b_hi, bb)), KPT_P_SUB(half_sq, bb));
    /* the small terms; r_lo enters as exp(r_hi) r_lo ~ (1 + r_hi) r_lo */
    double low = KPT_P_ADD(a_lo, b_lo);
    low = KPT_P_ADD(low, half_sq_err);
    low = KPT_P_ADD(low, KPT_P_FMA(r_lo, r_hi, r_lo));
    low = KPT_P_ADD(low, cube_q);
    const double e = KPT_P_ADD(b_hi, low); /* the one rounding of the result */
    if (k >= -1021 && k <= 1023) {
        return KPT_P_MUL(e, kpt_pow_two(k));
    }
    /* near the ends of the range: scale in two exact-or-final steps */
    const int k1 = k / 2;
    return KPT_P_MUL(KPT_P_MUL(e, kpt_pow_two(k1)), kpt_pow_two(k - k1));
}

KPT_POW_FN int kpt_pow_isnan(double x) {
    return (kpt_pow_bits(x) & 0x7fffffffffffffffULL) > 0x7ff0000000000000ULL;
}

KPT_POW_FN int kpt_pow_isinf(double x) {
    return (kpt_pow_bits(x) & 0x7fffffffffffffffULL) == 0x7ff0000000000000ULL;
}

/* 0 = not an integer, 1 = even integer, 2 = odd integer (y finite) */
KPT_POW_FN int kpt_pow_integer_kind(double y) {
    if (KPT_P_FLOOR(y) != y) {
        return 0;
    }
    const double half = KPT_P_MUL(y, 0.5);
    return KPT_P_FLOOR(half) == half ? 1 : 2;
}

KPT_POW_FN double kpt_pow(double x, double y) {
    const double inf = kpt_pow_from_bits(0x7ff0000000000000ULL);
    const double nan = kpt_pow_from_bits(0x7ff8000000000000ULL);
    if (y == 0.0 || x == 1.0) {
        return 1.0;
    }
    if (kpt_pow_isnan(x) || kpt_pow_isnan(y)) {
        return nan;
    }
    const uint64_t xs = kpt_pow_bits(x) >> 63;
    const double ax = xs ? -x : x;
    if (kpt_pow_isinf(y)) {
        if (ax == 1.0) return 1.0; /* (-1)^(+-inf) */
        return ((ax < 1.0) == (y < 0.0)) ? inf : 0.0;
    }
    const int kind = kpt_pow_integer_kind(y);
    const int negative_result = xs && kind == 2;
    if (x == 0.0 || kpt_pow_isinf(x)) {
        /* |x|^y is 0 or inf; the sign is x's for odd integer y */
        const int big = (x == 0.0) == (y < 0.0);
        const double mag = big ? inf : 0.0;
        return negative_result ? -mag : mag;
    }
    if (xs && kind == 0) {
        return nan; /* negative base, non-integer exponent */
    }
    double lh, ll;
    kpt_pow_log(ax, &lh, &ll);
    const double t_hi = KPT_P_MUL(y, lh);
    const double t_lo = KPT_P_FMA(y, ll, KPT_P_FMA(y, lh, -t_hi));
    const double r = kpt_pow_exp(t_hi, t_lo);
    return negative_result ? -r : r;
}

#endif /* KPT_POW_H */
