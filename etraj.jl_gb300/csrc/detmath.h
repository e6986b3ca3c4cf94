/*
 * detmath.h -- deterministic double-precision elementary functions.
 *
 * Every function here is written from the mathematics (Taylor series,
 * Cody-Waite additive range reduction, half-angle reduction for atan,
 * Kahan's log1p identity, Smith's complex division) and uses only
 * IEEE-754 operations that are correctly rounded on every target:
 * +, -, *, /, sqrt and explicit fma().  Compiled with FMA contraction
 * disabled (gcc -ffp-contract=off, nvcc --fmad=false), the same source
 * gives bit-identical results on an x86-64 host, an aarch64 host and an
 * sm_103a GPU.  That is what lets the FP64 device integrator match the
 * CPU oracle bit for bit: both evaluate sin, cos, exp, tanh, log, atan2,
 * asinh and pow through this file instead of through two different libms.
 *
 * Accuracy (checked against glibc by the test suite): a few ulp over the
 * argument ranges the trajectory code uses.  Domain notes: the sin/cos
 * reduction uses a three-part pi/2 and is accurate for |x| < 2^25; the
 * trajectory code evaluates phases of at most ~1e4 rad.
 *
 * The header compiles as C99 (oracle), C++ host code and CUDA device code.
 */
#ifndef ETRAJ_DETMATH_H
#define ETRAJ_DETMATH_H

#include <stdint.h>
#include <math.h>
#include <string.h>

#if defined(__CUDACC__)
#define DM_FN static __host__ __device__ __forceinline__
#else
#define DM_FN static inline
#endif

/* ---- constants (mathematical values split into double parts) ---------- */
#define DM_LN2_HI 0.6931471805599453
#define DM_LN2_LO 2.3190468138462996e-17
#define DM_LOG2E 1.4426950408889634
#define DM_PIO2_1 1.5707963267948966
#define DM_PIO2_2 6.123233995736766e-17
#define DM_PIO2_3 (-1.4973849048591698e-33)
#define DM_TWO_OVER_PI 0.6366197723675814
#define DM_PI_1 3.141592653589793
#define DM_PI_2 1.2246467991473532e-16
#define DM_PIO4_1 0.7853981633974483
#define DM_PIO4_2 3.061616997868383e-17
#define DM_LN10 2.302585092994046

/* ---- bit access ---------------------------------------------------------- */
DM_FN uint64_t dm_d2u(double x) {
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t u;
    memcpy(&u, &x, sizeof u);
    return u;
#endif
}

DM_FN double dm_u2d(uint64_t u) {
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)u);
#else
    double x;
    memcpy(&x, &u, sizeof x);
    return x;
#endif
}

DM_FN double dm_inf(void) { return dm_u2d(0x7ff0000000000000ull); }
DM_FN double dm_nan(void) { return dm_u2d(0x7ff8000000000000ull); }
DM_FN int dm_isnan(double x) { return !(x == x); }
DM_FN int dm_isinf(double x) { return fabs(x) == dm_inf(); }

/* 2^k for -1022 <= k <= 1023, exact. */
DM_FN double dm_pow2i(int k) { return dm_u2d((uint64_t)(k + 1023) << 52); }

/* p * 2^k with a single rounding (p normal, result may be subnormal). */
DM_FN double dm_scale(double p, int k) {
    if (k > 1023) return (p * dm_pow2i(1023)) * dm_pow2i(k - 1023);
    if (k < -1022) return (p * dm_pow2i(k + 54)) * dm_pow2i(-54);
    return p * dm_pow2i(k);
}

/* ---- exp / expm1 ------------------------------------------------------- */
/* Taylor series of e^r - 1 - r, divided by r^2, for |r| <= ln2/2
 * (truncation after the 1/13! term: relative error < 5e-18). */
DM_FN double dm_expm1_tail(double r) {
    double p = 1.0 / 6227020800.0;      /* 1/13! */
    p = fma(p, r, 1.0 / 479001600.0);   /* 1/12! */
    p = fma(p, r, 1.0 / 39916800.0);    /* 1/11! */
    p = fma(p, r, 1.0 / 3628800.0);     /* 1/10! */
    p = fma(p, r, 1.0 / 362880.0);      /* 1/9!  */
    p = fma(p, r, 1.0 / 40320.0);       /* 1/8!  */
    p = fma(p, r, 1.0 / 5040.0);        /* 1/7!  */
    p = fma(p, r, 1.0 / 720.0);         /* 1/6!  */
    p = fma(p, r, 1.0 / 120.0);         /* 1/5!  */
    p = fma(p, r, 1.0 / 24.0);          /* 1/4!  */
    p = fma(p, r, 1.0 / 6.0);           /* 1/3!  */
    p = fma(p, r, 0.5);                 /* 1/2!  */
    return p;
}

/* Cody-Waite reduction x = k*ln2 + r, |r| <= ~ln2/2. */
DM_FN double dm_reduce_ln2(double x, double* k) {
    double kk = rint(x * DM_LOG2E);
    double r = fma(-kk, DM_LN2_HI, x);
    r = fma(-kk, DM_LN2_LO, r);
    *k = kk;
    return r;
}

DM_FN double dm_exp(double x) {
    if (dm_isnan(x)) return x + x;
    if (x > 709.782712893384) return dm_inf();
    if (x < -745.1332191019412) return 0.0;
    double k;
    double r = dm_reduce_ln2(x, &k);
    double em1 = fma(r * r, dm_expm1_tail(r), r);
    return dm_scale(1.0 + em1, (int)k);
}

DM_FN double dm_expm1(double x) {
    if (dm_isnan(x)) return x + x;
    if (x > 709.782712893384) return dm_inf();
    if (x < -38.0) return -1.0;
    double k;
    double r = dm_reduce_ln2(x, &k);
    if (k == 0.0) return fma(x * x, dm_expm1_tail(x), x);
    double em = fma(r * r, dm_expm1_tail(r), r);
    int ik = (int)k;
    if (ik > 1000) return dm_scale(1.0 + em, ik);
    double tk = dm_pow2i(ik);
    /* e^x - 1 = 2^k * em + (2^k - 1); 2^k - 1 is exact for -53 <= k <= 53 */
    return fma(tk, em, tk - 1.0);
}

/* ---- log / log1p ------------------------------------------------------- */
DM_FN double dm_log(double x) {
    if (dm_isnan(x)) return x + x;
    if (x < 0.0) return dm_nan();
    if (x == 0.0) return -dm_inf();
    if (x == dm_inf()) return x;
    uint64_t u = dm_d2u(x);
    int e = 0;
    if (u < (1ull << 52)) { /* subnormal */
        x = x * dm_pow2i(54);
        u = dm_d2u(x);
        e = -54;
    }
    e += (int)(u >> 52) - 1023;
    double m = dm_u2d((u & 0x000fffffffffffffull) | 0x3ff0000000000000ull);
    if (m > 1.4142135623730951) {
        m = m * 0.5;
        e += 1;
    }
    /* log(m) = 2 atanh(s), s = (m-1)/(m+1), |s| <= 0.1716 */
    double f = m - 1.0;
    double s = f / (2.0 + f);
    double s2 = s * s;
    double p = 1.0 / 23.0;
    p = fma(p, s2, 1.0 / 21.0);
    p = fma(p, s2, 1.0 / 19.0);
    p = fma(p, s2, 1.0 / 17.0);
    p = fma(p, s2, 1.0 / 15.0);
    p = fma(p, s2, 1.0 / 13.0);
    p = fma(p, s2, 1.0 / 11.0);
    p = fma(p, s2, 1.0 / 9.0);
    p = fma(p, s2, 1.0 / 7.0);
    p = fma(p, s2, 1.0 / 5.0);
    p = fma(p, s2, 1.0 / 3.0);
    double two_s = 2.0 * s;
    double lm = fma(two_s * s2, p, two_s);
    double de = (double)e;
    return fma(de, DM_LN2_HI, fma(de, DM_LN2_LO, lm));
}

/* log(1+x) by Kahan's identity log1p(x) = log(u) * x / (u - 1), u = 1 + x. */
DM_FN double dm_log1p(double x) {
    double u = 1.0 + x;
    if (u == 1.0) return x;
    if (u == dm_inf()) return dm_log(x);
    return dm_log(u) * (x / (u - 1.0));
}

/* x^y for x > 0 (exp(y log x)); relative error grows like |y log x| ulp. */
DM_FN double dm_pow_pos(double x, double y) { return dm_exp(y * dm_log(x)); }

/* ---- sin / cos ----------------------------------------------------------- */
DM_FN void dm_sincos(double x, double* sp, double* cp) {
    if (!(fabs(x) < dm_inf())) {
        *sp = x - x;
        *cp = x - x;
        return;
    }
    double k = rint(x * DM_TWO_OVER_PI);
    double r = fma(-k, DM_PIO2_1, x);
    r = fma(-k, DM_PIO2_2, r);
    r = fma(-k, DM_PIO2_3, r);
    double r2 = r * r;
    /* sin r = r + r^3 * P(r^2), Taylor to r^19 */
    double ps = -1.0 / 121645100408832000.0; /* -1/19! */
    ps = fma(ps, r2, 1.0 / 355687428096000.0); /* 1/17! */
    ps = fma(ps, r2, -1.0 / 1307674368000.0);  /* -1/15! */
    ps = fma(ps, r2, 1.0 / 6227020800.0);      /* 1/13! */
    ps = fma(ps, r2, -1.0 / 39916800.0);       /* -1/11! */
    ps = fma(ps, r2, 1.0 / 362880.0);          /* 1/9! */
    ps = fma(ps, r2, -1.0 / 5040.0);           /* -1/7! */
    ps = fma(ps, r2, 1.0 / 120.0);             /* 1/5! */
    ps = fma(ps, r2, -1.0 / 6.0);              /* -1/3! */
    double sr = fma(r * r2, ps, r);
    /* cos r = (1 - r^2/2) + r^4 * Q(r^2), Taylor to r^18 */
    double pc = -1.0 / 6402373705728000.0;     /* -1/18! */
    pc = fma(pc, r2, 1.0 / 20922789888000.0);  /* 1/16! */
    pc = fma(pc, r2, -1.0 / 87178291200.0);    /* -1/14! */
    pc = fma(pc, r2, 1.0 / 479001600.0);       /* 1/12! */
    pc = fma(pc, r2, -1.0 / 3628800.0);        /* -1/10! */
    pc = fma(pc, r2, 1.0 / 40320.0);           /* 1/8! */
    pc = fma(pc, r2, -1.0 / 720.0);            /* -1/6! */
    pc = fma(pc, r2, 1.0 / 24.0);              /* 1/4! */
    double hr = 0.5 * r2;
    double w = 1.0 - hr;
    double cr = w + (((1.0 - w) - hr) + (r2 * r2) * pc);
    int q = (int)((long long)k & 3);
    if (q == 0) { *sp = sr; *cp = cr; }
    else if (q == 1) { *sp = cr; *cp = -sr; }
    else if (q == 2) { *sp = -sr; *cp = -cr; }
    else { *sp = -cr; *cp = sr; }
}

DM_FN double dm_sin(double x) { double s, c; dm_sincos(x, &s, &c); return s; }
DM_FN double dm_cos(double x) { double s, c; dm_sincos(x, &s, &c); return c; }

/* ---- tanh / sinh / cosh -------------------------------------------------- */
DM_FN double dm_tanh(double x) {
    double a = fabs(x);
    if (dm_isnan(a)) return x + x;
    double t;
    if (a >= 22.0) t = 1.0;
    else if (a < 1e-9) t = a;
    else {
        double em = dm_expm1(2.0 * a);
        t = em / (em + 2.0);
    }
    return copysign(t, x);
}

/* sinh and cosh of a real argument from one expm1. */
DM_FN void dm_sinhcosh(double x, double* shp, double* chp) {
    double a = fabs(x);
    double em = dm_expm1(a);
    double e = em + 1.0;
    double sh = 0.5 * (em + em / e);
    double ch = 0.5 * (e + 1.0 / e);
    *shp = copysign(sh, x);
    *chp = ch;
}

/* ---- atan / atan2 / asinh ------------------------------------------------ */
DM_FN double dm_atan(double x) {
    double a = fabs(x);
    if (dm_isnan(a)) return x + x;
    int inv = 0;
    if (a > 1.0) { a = 1.0 / a; inv = 1; }
    /* three half-angle steps atan(y) = 2 atan(y / (1 + sqrt(1 + y^2))) */
    double y = a;
    y = y / (1.0 + sqrt(fma(y, y, 1.0)));
    y = y / (1.0 + sqrt(fma(y, y, 1.0)));
    y = y / (1.0 + sqrt(fma(y, y, 1.0)));
    double y2 = y * y;
    double p = -1.0 / 19.0;
    p = fma(p, y2, 1.0 / 17.0);
    p = fma(p, y2, -1.0 / 15.0);
    p = fma(p, y2, 1.0 / 13.0);
    p = fma(p, y2, -1.0 / 11.0);
    p = fma(p, y2, 1.0 / 9.0);
    p = fma(p, y2, -1.0 / 7.0);
    p = fma(p, y2, 1.0 / 5.0);
    p = fma(p, y2, -1.0 / 3.0);
    double t = 8.0 * fma(y * y2, p, y);
    if (inv) t = (DM_PIO2_1 - t) + DM_PIO2_2;
    return copysign(t, x);
}

/* atan2 with the IEEE-754 / C99 conventions for signed zeros and infinities. */
DM_FN double dm_atan2(double y, double x) {
    if (dm_isnan(x) || dm_isnan(y)) return x + y;
    if (y == 0.0) {
        if (x > 0.0 || (x == 0.0 && !signbit(x))) return y;
        return copysign(DM_PI_1, y);
    }
    if (x == 0.0) return copysign(DM_PIO2_1, y);
    double ax = fabs(x), ay = fabs(y), t;
    if (dm_isinf(ax)) {
        if (dm_isinf(ay)) t = (x > 0.0) ? DM_PIO4_1 : 3.0 * DM_PIO4_1;
        else t = (x > 0.0) ? 0.0 : DM_PI_1;
        return copysign(t, y);
    }
    if (dm_isinf(ay)) return copysign(DM_PIO2_1, y);
    t = dm_atan(ay / ax);
    if (x < 0.0) t = (DM_PI_1 - t) + DM_PI_2;
    return copysign(t, y);
}

DM_FN double dm_asinh(double x) {
    double a = fabs(x);
    if (dm_isnan(a)) return x + x;
    double r;
    if (a > 268435456.0) r = dm_log(a) + DM_LN2_HI;
    else if (a > 2.0) r = dm_log(2.0 * a + 1.0 / (sqrt(fma(a, a, 1.0)) + a));
    else if (a < 3.7e-9) r = a;
    else {
        double a2 = a * a;
        r = dm_log1p(a + a2 / (1.0 + sqrt(1.0 + a2)));
    }
    return copysign(r, x);
}

DM_FN double dm_acos(double x) {
    /* acos x = atan2(sqrt((1-x)(1+x)), x) */
    return dm_atan2(sqrt((1.0 - x) * (1.0 + x)), x);
}

/* hypot without scaling: the arguments here are field strengths and momenta. */
DM_FN double dm_hypot(double x, double y) { return sqrt(x * x + y * y); }

/* ---- complex arithmetic ------------------------------------------------- */
typedef struct { double re, im; } dm_cplx;

DM_FN dm_cplx dm_c(double re, double im) { dm_cplx z; z.re = re; z.im = im; return z; }
DM_FN dm_cplx dm_cadd(dm_cplx a, dm_cplx b) { return dm_c(a.re + b.re, a.im + b.im); }
DM_FN dm_cplx dm_csub(dm_cplx a, dm_cplx b) { return dm_c(a.re - b.re, a.im - b.im); }
DM_FN dm_cplx dm_cneg(dm_cplx a) { return dm_c(-a.re, -a.im); }
DM_FN dm_cplx dm_cconj(dm_cplx a) { return dm_c(a.re, -a.im); }
DM_FN dm_cplx dm_cscale(dm_cplx a, double s) { return dm_c(a.re * s, a.im * s); }
DM_FN dm_cplx dm_caddr(dm_cplx a, double r) { return dm_c(a.re + r, a.im); }
DM_FN dm_cplx dm_cmul(dm_cplx a, dm_cplx b) {
    return dm_c(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
/* Smith's algorithm (1962). */
DM_FN dm_cplx dm_cdiv(dm_cplx a, dm_cplx b) {
    if (fabs(b.re) >= fabs(b.im)) {
        double r = b.im / b.re, d = b.re + b.im * r;
        return dm_c((a.re + a.im * r) / d, (a.im - a.re * r) / d);
    } else {
        double r = b.re / b.im, d = b.re * r + b.im;
        return dm_c((a.re * r + a.im) / d, (a.im * r - a.re) / d);
    }
}
DM_FN double dm_cabs2(dm_cplx a) { return a.re * a.re + a.im * a.im; }
DM_FN double dm_carg(dm_cplx a) { return dm_atan2(a.im, a.re); }
DM_FN dm_cplx dm_cexp(dm_cplx a) {
    double e = dm_exp(a.re), s, c;
    dm_sincos(a.im, &s, &c);
    return dm_c(e * c, e * s);
}
DM_FN dm_cplx dm_clog(dm_cplx a) {
    return dm_c(0.5 * dm_log(dm_cabs2(a)), dm_atan2(a.im, a.re));
}
/* principal z^p for real p; z^1 is returned unchanged */
DM_FN dm_cplx dm_cpow_real(dm_cplx z, double p) {
    if (p == 1.0) return z;
    if (z.re == 0.0 && z.im == 0.0) return dm_c(p == 0.0 ? 1.0 : 0.0, 0.0);
    dm_cplx l = dm_clog(z);
    return dm_cexp(dm_cscale(l, p));
}
/* z^n for a small non-negative integer n by repeated multiplication */
DM_FN dm_cplx dm_cpowi(dm_cplx z, int n) {
    dm_cplx r = dm_c(1.0, 0.0);
    for (int i = 0; i < n; ++i) r = dm_cmul(r, z);
    return r;
}
/* sin and cos of one complex argument from one sincos and one sinh/cosh
 * (the same values as dm_csin and dm_ccos) */
/* sin and cos of a + i im from s = sin(a), c = cos(a) */
DM_FN void dm_csincos_re(double s, double c, double im, dm_cplx* sn, dm_cplx* cs) {
    double sh, ch;
    dm_sinhcosh(im, &sh, &ch);
    *sn = dm_c(s * ch, c * sh);
    *cs = dm_c(c * ch, -(s * sh));
}
DM_FN void dm_csincos(dm_cplx a, dm_cplx* sn, dm_cplx* cs) {
    double s, c;
    dm_sincos(a.re, &s, &c);
    dm_csincos_re(s, c, a.im, sn, cs);
}
/* cos and sin of a complex argument */
DM_FN dm_cplx dm_ccos(dm_cplx a) {
    double s, c, sh, ch;
    dm_sincos(a.re, &s, &c);
    dm_sinhcosh(a.im, &sh, &ch);
    return dm_c(c * ch, -(s * sh));
}
DM_FN dm_cplx dm_csin(dm_cplx a) {
    double s, c, sh, ch;
    dm_sincos(a.re, &s, &c);
    dm_sinhcosh(a.im, &sh, &ch);
    return dm_c(s * ch, c * sh);
}

#endif /* ETRAJ_DETMATH_H */
