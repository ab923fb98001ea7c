/* Portable exp(t) and x**y for x >= 0, y > 0 (CPU oracle; test infrastructure).
 *
 * exp(y log x) from series, with IEEE +, -, *, /, fma, frexp/ldexp and rint only, so that
 * the oracles and the device code (gear.cuh: gpow, the same operations) give the same
 * bits on every platform.  libm's pow differs by ulps between platforms, and a single ulp
 * changes the step sequence of stiff cells in adaptive solvers (measured with SMVGEAR:
 * 830 vs 823 and 913 step attempts).
 * log: x = m 2^k, m in [sqrt(1/2), sqrt(2)), log m = 2 atanh(s), s = (m-1)/(m+1), series
 * to s^23; exp: t = n ln2 + r with a Cody-Waite split of ln2, |r| <= ln2/2, Taylor series
 * to r^13.  Relative error below 4e-16 x max(1, |y log x|) (about 4e-15 at x = 1e-30). */
#ifndef ORACLE_PORTABLE_POW_H
#define ORACLE_PORTABLE_POW_H
#include <math.h>

/* exp(t) by the series below: t = n ln2 + r with a Cody-Waite split of ln 2, |r| <= ln2/2,
 * Taylor series to r^13 (relative error below 3e-16). */
static double portable_exp(double t)
{
    const double ln2_hi = 0x1.62e42fee00000p-1, ln2_lo = 0x1.a39ef35793c76p-33;
    if (t > 709.0) return INFINITY;
    if (t < -745.0) return 0.0;
    const double n = rint(t * 0x1.71547652b82fep+0);   /* t / ln2 */
    const double r = fma(-n, ln2_lo, fma(-n, ln2_hi, t));
    double e = 0x1.6124613a86d09p-33;       /* 1/13! */
    e = fma(e, r, 0x1.1eed8eff8d898p-29);   /* 1/12! */
    e = fma(e, r, 0x1.ae64567f544e4p-26);   /* 1/11! */
    e = fma(e, r, 0x1.27e4fb7789f5cp-22);   /* 1/10! */
    e = fma(e, r, 0x1.71de3a556c734p-19);   /* 1/9! */
    e = fma(e, r, 0x1.a01a01a01a01ap-16);   /* 1/8! */
    e = fma(e, r, 0x1.a01a01a01a01ap-13);   /* 1/7! */
    e = fma(e, r, 0x1.6c16c16c16c17p-10);   /* 1/6! */
    e = fma(e, r, 0x1.1111111111111p-7);    /* 1/5! */
    e = fma(e, r, 0x1.5555555555555p-5);    /* 1/4! */
    e = fma(e, r, 0x1.5555555555555p-3);    /* 1/3! */
    e = fma(e, r, 0.5);
    e = fma(e, r, 1.0);
    e = fma(e, r, 1.0);
    return ldexp(e, (int)n);
}

static double portable_pow(double x, double y)
{
    if (!(x > 0.0)) return x == 0.0 ? 0.0 : x;
    if (isinf(x)) return x;
    int k;
    double m = frexp(x, &k);
    if (m < 0x1.6a09e667f3bcdp-1) {
        m = m * 2.0;
        k = k - 1;
    }
    const double s = (m - 1.0) / (m + 1.0);
    const double z = s * s;
    double p = 0x1.642c8590b2164p-5;        /* 1/23 */
    p = fma(p, z, 0x1.8618618618618p-5);    /* 1/21 */
    p = fma(p, z, 0x1.af286bca1af28p-5);    /* 1/19 */
    p = fma(p, z, 0x1.e1e1e1e1e1e1ep-5);    /* 1/17 */
    p = fma(p, z, 0x1.1111111111111p-4);    /* 1/15 */
    p = fma(p, z, 0x1.3b13b13b13b14p-4);    /* 1/13 */
    p = fma(p, z, 0x1.745d1745d1746p-4);    /* 1/11 */
    p = fma(p, z, 0x1.c71c71c71c71cp-4);    /* 1/9 */
    p = fma(p, z, 0x1.2492492492492p-3);    /* 1/7 */
    p = fma(p, z, 0x1.999999999999ap-3);    /* 1/5 */
    p = fma(p, z, 0x1.5555555555555p-2);    /* 1/3 */
    p = fma(p, z, 1.0);
    const double ln2_hi = 0x1.62e42fee00000p-1, ln2_lo = 0x1.a39ef35793c76p-33;
    const double lx = fma((double)k, ln2_hi, fma((double)k, ln2_lo, (2.0 * s) * p));
    const double t = y * lx;
    return portable_exp(t);
}

#endif
