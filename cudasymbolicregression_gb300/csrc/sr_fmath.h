/* sr_fmath.h -- the library's own float32 sin, cos, exp and log.
 *
 * Every float kernel of the library evaluates these four operators with the
 * functions below instead of the CUDA math library, and the CPU oracle's
 * kernel-arithmetic mode includes this same file: each function is a fixed
 * sequence of IEEE float32 operations (add, sub, mul, div and fused multiply-add,
 * each rounded once to nearest) plus integer and, on the rare huge-argument path of
 * sin/cos, double operations, so a GPU and a CPU compute the same bits.  That makes a
 * whole fit over tapes with these operators reproducible on the host, bit for bit.
 *
 * Methods (textbook; the coefficients of exp, sin and cos are the Taylor coefficients
 * rounded to float, those of log fitted here):
 *   exp  x = j ln2 + r with j = round(x / ln2) and r by a two-part Cody-Waite
 *        reduction (FMA), e^r by its degree-7 Taylor polynomial (|r| <= ln2/2),
 *        then 2^j applied as two exact powers of two (one rounding, correct into
 *        the subnormal range).
 *   log  x = m 2^e with m in [sqrt(1/2), sqrt(2)), f = m - 1 (exact), log(1 + f) =
 *        f - f^2/2 + f^3 h(f) with h a degree-8 polynomial fitted to the remainder
 *        (weighted least squares on Chebyshev nodes, iteratively reweighted towards
 *        the minimax error: sr_fmath_coefficients.py), plus e ln2 with ln2 split so
 *        that e ln2_hi is exact.  No division.
 *   sin, cos  x = q pi/2 + r: below 2^19 by a three-part Cody-Waite reduction with
 *        FMA (its first step is exact); above, by Payne and Hanek's method, the
 *        product of x's 24-bit significand with a 96-bit window of the bits of 2/pi
 *        in integer arithmetic.  Then the Taylor polynomials of sin and cos on
 *        |r| <= pi/4 (cos with the rounding error of 1 - r^2/2 carried), chosen and
 *        signed by q mod 4.
 * Accuracy, checked over every float32 input against a double-precision reference:
 * the maximum errors are stated in the test that checks them
 * (tests/test_fmath_cpu.py).  Domain rules (NaN for log of x <= 0 and so on) are
 * the callers'; these functions follow IEEE special values (log 0 = -inf, log of a
 * negative number or NaN = NaN, exp(+-inf) = inf / 0, sin and cos of +-inf = NaN).
 */
#ifndef SR_FMATH_H
#define SR_FMATH_H

#ifdef __CUDACC__
#define SRM_FN static __host__ __device__ __forceinline__
#define SRM_FN_COLD static __host__ __device__ __noinline__ /* rare path: kept out of the callers' registers */
#else
#define SRM_FN static inline
#define SRM_FN_COLD static
#endif

#include <stdint.h>
#if !defined(__CUDA_ARCH__)
#include <math.h>
#include <string.h>
#endif

#if defined(__CUDA_ARCH__)
#define SRM_ADD(a, b) __fadd_rn((a), (b))
#define SRM_SUB(a, b) __fsub_rn((a), (b))
#define SRM_MUL(a, b) __fmul_rn((a), (b))
#define SRM_DIV(a, b) __fdiv_rn((a), (b))
#define SRM_FMA(a, b, c) __fmaf_rn((a), (b), (c))
#define SRM_F2I(x) __float_as_int(x)
#define SRM_I2F(i) __int_as_float(i)
#define SRM_DMUL(a, b) __dmul_rn((a), (b))
#define SRM_D2F(d) __double2float_rn(d)
#define SRM_L2D(l) __ll2double_rn(l)
#else
/* host: plain IEEE operations; the including file is compiled without floating-point
 * contraction (-ffp-contract=off), so no multiply and add are fused implicitly */
#define SRM_ADD(a, b) ((a) + (b))
#define SRM_SUB(a, b) ((a) - (b))
#define SRM_MUL(a, b) ((a) * (b))
#define SRM_DIV(a, b) ((a) / (b))
#define SRM_FMA(a, b, c) fmaf((a), (b), (c))
SRM_FN int32_t srm_f2i(float x) { int32_t i; memcpy(&i, &x, sizeof i); return i; }
SRM_FN float srm_i2f(int32_t i) { float x; memcpy(&x, &i, sizeof x); return x; }
#define SRM_F2I(x) srm_f2i(x)
#define SRM_I2F(i) srm_i2f(i)
#define SRM_DMUL(a, b) ((a) * (b))
#define SRM_D2F(d) ((float)(d))
#define SRM_L2D(l) ((double)(l))
#endif

#define SRM_ROUNDER 12582912.0f /* 1.5 * 2^23: x + this, rounded, is an integer */

/* ---- exp --------------------------------------------------------------------- */
SRM_FN float sr_expf(float x)
{
    if (x != x) return SRM_ADD(x, x);
    if (x > 89.0f) return SRM_I2F(0x7f800000);   /* overflow (e^89 > FLT_MAX) */
    if (x < -104.0f) return 0.0f;                   /* below half the least subnormal */
    const float log2e = 1.44269502162933350f;       /* 1 / ln 2 */
    const float ln2_hi = 0.693147182464599609f;     /* ln 2 rounded */
    const float ln2_lo = -1.90465421212593e-09f;    /* ln 2 - ln2_hi */
    float j = SRM_SUB(SRM_FMA(x, log2e, SRM_ROUNDER), SRM_ROUNDER);
    float r = SRM_FMA(j, -ln2_hi, x);
    r = SRM_FMA(j, -ln2_lo, r);
    float p = 1.98412701138295e-04f;                /* 1/7! */
    p = SRM_FMA(p, r, 1.38888892251998e-03f);       /* 1/6! */
    p = SRM_FMA(p, r, 8.33333376795053e-03f);       /* 1/5! */
    p = SRM_FMA(p, r, 4.16666679084301e-02f);       /* 1/4! */
    p = SRM_FMA(p, r, 1.66666671633720e-01f);       /* 1/3! */
    p = SRM_FMA(p, r, 0.5f);
    p = SRM_FMA(p, r, 1.0f);
    p = SRM_FMA(p, r, 1.0f);
    int ji = (int)j;                                /* -151 .. 129 */
    int j1 = ji / 2, j2 = ji - j1;                  /* each -76 .. 65: normal powers of two */
    float s1 = SRM_I2F((j1 + 127) << 23), s2 = SRM_I2F((j2 + 127) << 23);
    return SRM_MUL(SRM_MUL(p, s1), s2);             /* p s1 is exact; one rounding */
}

/* ---- log --------------------------------------------------------------------- */
SRM_FN float sr_logf(float x)
{
    if (x != x) return SRM_ADD(x, x);
    if (x < 0.0f) return SRM_I2F(0x7fffffff);
    if (x == 0.0f) return SRM_I2F((int32_t)0xff800000u);
    int32_t ix = SRM_F2I(x);
    if (ix >= 0x7f800000) return x;                 /* +inf */
    int e = 0;
    if (ix < 0x00800000) {                          /* subnormal: scale by 2^23 */
        x = SRM_MUL(x, 8388608.0f);
        ix = SRM_F2I(x);
        e = -23;
    }
    e += (ix >> 23) - 127;
    ix = (ix & 0x007fffff) | 0x3f800000;            /* m in [1, 2) */
    if (ix > 0x3fb504f3) {                          /* m > sqrt(2): m / 2 */
        ix -= 0x00800000;
        e += 1;
    }
    float f = SRM_SUB(SRM_I2F(ix), 1.0f);           /* exact */
    /* log(1 + f) = f - f^2/2 + f^3 h(f), h a degree-8 polynomial fitted to
     * (log(1 + f) - f + f^2/2) / f^3 on [sqrt(1/2) - 1, sqrt(2) - 1]
     * (sr_fmath_coefficients.py; its own error is 0.06 ulp of the result) */
    float h = SRM_FMA(f, 0.054545700550079346f, -0.10845454782247543f);
    h = SRM_FMA(f, h, 0.12036514282226562f);
    h = SRM_FMA(f, h, -0.12560544908046722f);
    h = SRM_FMA(f, h, 0.14218197762966156f);
    h = SRM_FMA(f, h, -0.1665862649679184f);
    h = SRM_FMA(f, h, 0.20001961290836334f);
    h = SRM_FMA(f, h, -0.2500019073486328f);
    h = SRM_FMA(f, h, 0.3333331048488617f);
    float f2 = SRM_MUL(f, f);
    float hfsq = SRM_MUL(0.5f, f2);
    float lg = SRM_SUB(f, SRM_SUB(hfsq, SRM_MUL(SRM_MUL(f2, f), h)));
    const float ln2_hi = 0.693145751953125f;        /* ln 2 to 16 bits: e ln2_hi is exact */
    const float ln2_lo = 1.42860676533019e-06f;     /* ln 2 - ln2_hi */
    float fe = (float)e;
    return SRM_ADD(SRM_MUL(fe, ln2_hi), SRM_ADD(SRM_MUL(fe, ln2_lo), lg));
}

/* ---- sin and cos -------------------------------------------------------------- */

/* 32-bit word k of the binary fraction of 2/pi (bits 32k+1 .. 32k+32; zero before
 * the binary point and past the table). */
SRM_FN uint32_t srm_two_over_pi_word(int k)
{
    switch (k) {
    case 0: return 0xa2f9836eu;
    case 1: return 0x4e441529u;
    case 2: return 0xfc2757d1u;
    case 3: return 0xf534ddc0u;
    case 4: return 0xdb629599u;
    case 5: return 0x3c439041u;
    case 6: return 0xfe5163abu;
    case 7: return 0xdebbc561u;
    default: return 0u;
    }
}

/* 32 bits of 2/pi starting at fraction bit index s (0 = the 1/2 bit; s may be
 * negative: the integer part of 2/pi is 0). */
SRM_FN uint32_t srm_two_over_pi_bits(int s)
{
    int k = (s + 64) / 32 - 2;                      /* floor(s / 32) for s >= -64 */
    int sh = s - 32 * k;                            /* 0 .. 31 */
    uint64_t w = ((uint64_t)srm_two_over_pi_word(k) << 32) | srm_two_over_pi_word(k + 1);
    return (uint32_t)((w << sh) >> 32);
}

/* x = q pi/2 + r for |x| >= 2^19 (finite): Payne-Hanek.  Returns q mod 4 in *q. */
SRM_FN_COLD float srm_reduce_huge(float ax, int *q)
{
    int32_t ix = SRM_F2I(ax);
    int E = (ix >> 23) - 127;                       /* >= 19 */
    uint64_t m = (uint64_t)((ix & 0x007fffff) | 0x00800000);
    /* x 2/pi = m 2^(E-23) sum_i b_i 2^-i; the bits i <= E-25 add multiples of 4.  The
     * 96 bits from i0 = E-24 give x 2/pi = m C 2^-94 (mod 4), C their integer. */
    int s = E - 25;                                 /* 0-based index of bit i0 */
    uint64_t c2 = srm_two_over_pi_bits(s), c1 = srm_two_over_pi_bits(s + 32), c0 = srm_two_over_pi_bits(s + 64);
    uint64_t p0 = m * c0, p1 = m * c1, p2 = m * c2;
    uint64_t w0 = p0 & 0xffffffffu;
    uint64_t t1 = p1 + (p0 >> 32);
    uint64_t w1 = t1 & 0xffffffffu;
    uint64_t t2 = p2 + (t1 >> 32);
    uint64_t w2 = t2 & 0xffffffffu;
    int quad = (int)((w2 >> 30) & 3u);              /* bits 94, 95 of m C */
    uint64_t F = ((w2 & 0x3fffffffu) << 34) | (w1 << 2) | (w0 >> 30);  /* fraction, 2^-64 units */
    int64_t Fs = (int64_t)F;                        /* >= 1/2: take the next multiple */
    if (Fs < 0) quad = (quad + 1) & 3;
    *q = quad;
    const double pio2_2m64 = 8.515303950216386e-20; /* pi/2 * 2^-64 */
    return SRM_D2F(SRM_DMUL(SRM_L2D(Fs), pio2_2m64));
}

/* sin (odd = 0) or cos (odd = 1) of x */
SRM_FN float srm_sincos(float x, int odd)
{
    float ax = SRM_I2F(SRM_F2I(x) & 0x7fffffff);
    if (!(ax < SRM_I2F(0x7f800000))) return SRM_SUB(x, x);  /* NaN, +-inf */
    float r;
    int q;
    if (ax < 524288.0f) {                           /* 2^19 */
        const float two_over_pi = 0.636619746685028f;
        const float p1 = 1.57079637050628662f, p2 = -4.37113882867379e-08f, p3 = -1.71512451000588e-15f;
        float qf = SRM_SUB(SRM_FMA(x, two_over_pi, SRM_ROUNDER), SRM_ROUNDER);
        r = SRM_FMA(qf, -p1, x);
        r = SRM_FMA(qf, -p2, r);
        r = SRM_FMA(qf, -p3, r);
        q = (int)qf;
    } else {
        r = srm_reduce_huge(ax, &q);
        if (x < 0.0f) { r = -r; q = -q; }
    }
    q += odd;
    /* both polynomials, then a select: lanes in different quadrants do not diverge */
    float w = SRM_MUL(r, r);
    float c = SRM_FMA(w, -2.75573188446288e-07f, 2.48015876422869e-05f);  /* -1/10!, 1/8! */
    c = SRM_FMA(w, c, -1.38888892251998e-03f);                          /* -1/6! */
    c = SRM_FMA(w, c, 4.16666679084301e-02f);                           /* 1/4! */
    float hw = SRM_MUL(0.5f, w);
    float t = SRM_SUB(1.0f, hw);
    float cosr = SRM_ADD(t, SRM_FMA(SRM_MUL(w, w), c, SRM_SUB(SRM_SUB(1.0f, t), hw)));  /* 1 - w/2 + w^2 C(w) */
    float sp = SRM_FMA(w, 2.75573188446288e-06f, -1.98412701138295e-04f);  /* 1/9!, -1/7! */
    sp = SRM_FMA(w, sp, 8.33333376795053e-03f);                            /* 1/5! */
    sp = SRM_FMA(w, sp, -1.66666671633720e-01f);                           /* -1/3! */
    float sinr = SRM_FMA(SRM_MUL(r, w), sp, r);                          /* r + r^3 S(w) */
    float res = (q & 1) ? cosr : sinr;
    res = (q & 2) ? -res : res;
    return (!odd && ax < 2.44140625e-4f) ? x : res;  /* |x| < 2^-12: sin x rounds to x (keeps -0) */
}

SRM_FN float sr_sinf(float x) { return srm_sincos(x, 0); }
SRM_FN float sr_cosf(float x) { return srm_sincos(x, 1); }

#endif /* SR_FMATH_H */
