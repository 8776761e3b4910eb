/*
 * cd_math.h -- float64 elementary functions shared by the device kernels and
 * the CPU oracle.
 *
 * The reference's step is chaotic: float64 rounding differences of one unit
 * in the last place grow about tenfold every two to three steps.  A device
 * path can only reproduce a multi-step rollout if every operation rounds
 * exactly as the oracle's does.  +, -, *, /, sqrt, fmod, floor, rint and
 * ldexp are correctly rounded (or exact) in both C and CUDA; the functions
 * below are built from those operations only, so the same source compiled
 * without fused multiply-add contraction gives identical bits on the host
 * and on the GPU.  Each one is accurate to about one unit in the last place
 * (checked against the C library by the tests).
 *
 * Methods (all published):
 *   hypot  : sqrt(x*x + y*y)  (no overflow scaling; |x|, |y| < 1e150)
 *   exp    : Cody & Waite (1980) reduction x = k ln2 + r, |r| <= ln2/2, with a
 *            two-part ln2, Taylor series to degree 13, scaling by ldexp
 *   sincos : Cody & Waite reduction by pi/2 with a three-part constant (exact
 *            products for |k| < 2^20), Taylor series to degree 17 / 18 on
 *            |r| <= pi/4; quadrant by k mod 4
 *   log    : x = m 2^e with m in [sqrt(1/2), sqrt(2)) (frexp, exact), then
 *            log m = 2 atanh(s), s = (m - 1) / (m + 1), |s| <= 3 - 2 sqrt(2),
 *            by the series 2 (s + s^3/3 + ... + s^25/25); e ln 2 with the
 *            two-part ln 2 of exp
 *   atan2  : reduction of t = min/max in [0, 1] by atan(t) = atan(c) +
 *            atan((t - c) / (1 + t c)) with c = tan(pi/8) or 1, Taylor series
 *            of atan to degree 23 on |u| <= tan(pi/16); quadrant and signed
 *            zero handling as in IEEE 754 / C99 atan2
 * Constants are correctly rounded values of the exact quantities (1/n!,
 * 1/n, pi/2, ln 2, atan(c) of the double c), computed to 80 digits.
 */
#ifndef CD_MATH_H
#define CD_MATH_H

#include <math.h>
#include <stdint.h>

#ifdef __CUDACC__
#define CDM_FN __host__ __device__ __forceinline__
#else
#define CDM_FN static inline
#endif

CDM_FN double cdm_hypot(double x, double y) { return sqrt(x * x + y * y); }

CDM_FN double cdm_exp(double x) {
    if (x != x) return x;
    if (x > 0x1.62e42fefa39efp+9) return INFINITY;
    if (x < -0x1.74910d52d3052p+9) return 0.0;
    const double k = rint(x * 0x1.71547652b82fep+0);
    const double r = (x - k * 0x1.62e42ff000000p-1) - k * (-0x1.718432a1b0e26p-35);
    double p = 0x1.6124613a86d09p-33;           /* 1/13! */
    p = p * r + 0x1.1eed8eff8d898p-29;          /* 1/12! */
    p = p * r + 0x1.ae64567f544e4p-26;          /* 1/11! */
    p = p * r + 0x1.27e4fb7789f5cp-22;          /* 1/10! */
    p = p * r + 0x1.71de3a556c734p-19;          /* 1/9!  */
    p = p * r + 0x1.a01a01a01a01ap-16;          /* 1/8!  */
    p = p * r + 0x1.a01a01a01a01ap-13;          /* 1/7!  */
    p = p * r + 0x1.6c16c16c16c17p-10;          /* 1/6!  */
    p = p * r + 0x1.1111111111111p-7;           /* 1/5!  */
    p = p * r + 0x1.5555555555555p-5;           /* 1/4!  */
    p = p * r + 0x1.5555555555555p-3;           /* 1/3!  */
    p = p * r + 0x1.0000000000000p-1;           /* 1/2!  */
    p = p * r + 1.0;
    p = p * r + 1.0;
    return ldexp(p, (int)k);
}

CDM_FN double cdm_log(double x) {
    if (!(x > 0)) return x == 0 ? -INFINITY : NAN;     /* NaN and negative: NaN */
    if (x == INFINITY) return x;
    int e;
    double m = frexp(x, &e);                            /* m in [1/2, 1) */
    if (m < 0x1.6a09e667f3bcdp-1) {                     /* sqrt(1/2) */
        m = m * 2.0;
        e -= 1;
    }
    const double s = (m - 1.0) / (m + 1.0);
    const double s2 = s * s;
    double p = 0x1.47ae147ae147bp-5;            /* 1/25 */
    p = p * s2 + 0x1.642c8590b2164p-5;          /* 1/23 */
    p = p * s2 + 0x1.8618618618618p-5;          /* 1/21 */
    p = p * s2 + 0x1.af286bca1af28p-5;          /* 1/19 */
    p = p * s2 + 0x1.e1e1e1e1e1e1ep-5;          /* 1/17 */
    p = p * s2 + 0x1.1111111111111p-4;          /* 1/15 */
    p = p * s2 + 0x1.3b13b13b13b14p-4;          /* 1/13 */
    p = p * s2 + 0x1.745d1745d1746p-4;          /* 1/11 */
    p = p * s2 + 0x1.c71c71c71c71cp-4;          /* 1/9  */
    p = p * s2 + 0x1.2492492492492p-3;          /* 1/7  */
    p = p * s2 + 0x1.999999999999ap-3;          /* 1/5  */
    p = p * s2 + 0x1.5555555555555p-2;          /* 1/3  */
    const double two_s = 2.0 * s;
    const double lm = two_s + two_s * (s2 * p);
    const double de = (double)e;
    return de * 0x1.62e42ff000000p-1 + (de * (-0x1.718432a1b0e26p-35) + lm);
}

CDM_FN void cdm_sincos(double x, double *s, double *c) {
    if (!(x - x == 0.0)) { *s = x - x; *c = x - x; return; }   /* inf, nan */
    double k, r;
    if (fabs(x) < 0x1.0p+20) {
        k = rint(x * 0x1.45f306dc9c883p-1);
        r = ((x - k * 0x1.921fb54400000p+0) - k * 0x1.0b4611a600000p-34) - k * 0x1.3198a2e037073p-69;
    } else {
        /* far outside the range the update produces: reduce by 2 pi first */
        double y = fmod(x, 2 * 0x1.921fb54442d18p+1);
        k = rint(y * 0x1.45f306dc9c883p-1);
        r = ((y - k * 0x1.921fb54400000p+0) - k * 0x1.0b4611a600000p-34) - k * 0x1.3198a2e037073p-69;
    }
    const double r2 = r * r;
    double ps = 0x1.952c77030ad4ap-49;          /* +1/17! */
    ps = ps * r2 - 0x1.ae7f3e733b81fp-41;       /* -1/15! */
    ps = ps * r2 + 0x1.6124613a86d09p-33;       /* +1/13! */
    ps = ps * r2 - 0x1.ae64567f544e4p-26;       /* -1/11! */
    ps = ps * r2 + 0x1.71de3a556c734p-19;       /* +1/9!  */
    ps = ps * r2 - 0x1.a01a01a01a01ap-13;       /* -1/7!  */
    ps = ps * r2 + 0x1.1111111111111p-7;        /* +1/5!  */
    ps = ps * r2 - 0x1.5555555555555p-3;        /* -1/3!  */
    const double sr = r + (r * r2) * ps;
    double pc = -0x1.6827863b97d97p-53;         /* -1/18! */
    pc = pc * r2 + 0x1.ae7f3e733b81fp-45;       /* +1/16! */
    pc = pc * r2 - 0x1.93974a8c07c9dp-37;       /* -1/14! */
    pc = pc * r2 + 0x1.1eed8eff8d898p-29;       /* +1/12! */
    pc = pc * r2 - 0x1.27e4fb7789f5cp-22;       /* -1/10! */
    pc = pc * r2 + 0x1.a01a01a01a01ap-16;       /* +1/8!  */
    pc = pc * r2 - 0x1.6c16c16c16c17p-10;       /* -1/6!  */
    pc = pc * r2 + 0x1.5555555555555p-5;        /* +1/4!  */
    pc = pc * r2 - 0x1.0000000000000p-1;        /* -1/2!  */
    const double cr = 1.0 + r2 * pc;
    const int q = (int)(((long long)k) & 3);
    if (q == 0) { *s = sr; *c = cr; }
    else if (q == 1) { *s = cr; *c = -sr; }
    else if (q == 2) { *s = -sr; *c = -cr; }
    else { *s = -cr; *c = sr; }
}

CDM_FN double cdm_sin(double x) { double s, c; cdm_sincos(x, &s, &c); return s; }
CDM_FN double cdm_cos(double x) { double s, c; cdm_sincos(x, &s, &c); return c; }

/* atan(t) for 0 <= t <= 1 */
CDM_FN double cdm_atan01(double t) {
    double base_hi = 0.0, base_lo = 0.0, u = t;
    if (t > 0x1.561b82ab7f990p-1) {              /* t > tan(3 pi / 16): c = 1 */
        u = (t - 1.0) / (1.0 + t);
        base_hi = 0x1.921fb54442d18p-1; base_lo = 0x1.1a62633145c07p-55;   /* pi/4 */
    } else if (t > 0x1.975f5e0553158p-3) {       /* t > tan(pi / 16): c = tan(pi/8) */
        const double c = 0x1.a827999fcef32p-2;
        u = (t - c) / (1.0 + t * c);
        base_hi = 0x1.921fb54442d18p-2; base_lo = 0x1.c398861b78b55p-59;   /* atan(c) */
    }
    const double u2 = u * u;
    double p = -0x1.642c8590b2164p-5;            /* -1/23 */
    p = p * u2 + 0x1.8618618618618p-5;           /* +1/21 */
    p = p * u2 - 0x1.af286bca1af28p-5;           /* -1/19 */
    p = p * u2 + 0x1.e1e1e1e1e1e1ep-5;           /* +1/17 */
    p = p * u2 - 0x1.1111111111111p-4;           /* -1/15 */
    p = p * u2 + 0x1.3b13b13b13b14p-4;           /* +1/13 */
    p = p * u2 - 0x1.745d1745d1746p-4;           /* -1/11 */
    p = p * u2 + 0x1.c71c71c71c71cp-4;           /* +1/9  */
    p = p * u2 - 0x1.2492492492492p-3;           /* -1/7  */
    p = p * u2 + 0x1.999999999999ap-3;           /* +1/5  */
    p = p * u2 - 0x1.5555555555555p-2;           /* -1/3  */
    const double au = u + (u * u2) * p;
    return base_hi + (base_lo + au);
}

CDM_FN double cdm_atan2(double y, double x) {
    const double PI_HI = 0x1.921fb54442d18p+1, PI_LO = 0x1.1a62633145c07p-53;
    const double PIO2_HI = 0x1.921fb54442d18p+0, PIO2_LO = 0x1.1a62633145c07p-54;
    if (x != x || y != y) return x + y;
    if (y == 0.0) {
        if (x > 0.0 || (x == 0.0 && !signbit(x))) return y;
        return signbit(y) ? -PI_HI : PI_HI;
    }
    if (x == 0.0) return y > 0 ? PIO2_HI : -PIO2_HI;
    const double ax = fabs(x), ay = fabs(y);
    double a;
    if (isinf(ax) || isinf(ay)) {
        if (isinf(ax) && isinf(ay)) a = 0x1.921fb54442d18p-1;       /* pi/4 */
        else if (isinf(ax)) a = 0.0;
        else a = PIO2_HI;
        if (x < 0) a = (isinf(ax) && isinf(ay)) ? 0x1.2d97c7f3321d2p+1 : (isinf(ax) ? PI_HI : a);
        return y < 0 ? -a : a;
    }
    if (ay > ax) a = (PIO2_HI - cdm_atan01(ax / ay)) + PIO2_LO;
    else a = cdm_atan01(ay / ax);
    if (x < 0) a = (PI_HI - a) + PI_LO;
    return y < 0 ? -a : a;
}

#endif /* CD_MATH_H */
