/* sae_skip.h -- when may exp(-b r) of the SAE potential be dropped exactly?
 *
 * The SAE potential and force (SAEAtom.jl:87-94, 102-181) evaluate three
 * sums, left to right:
 *   num = ((Z + a1 e1) + a2 r e2) + a3 e3
 *   br  = (Z + a1 (1 + b1 r) e1) + a3 (1 + b3 r) e3
 *   C   = br / (s sqrt(s)) + (a2 b2 / sqrt(s)) e2,   s = r^2 + sc,  e_i = exp(-b_i r).
 * Adding t to a nonzero double x returns x whenever |t| < 2^-55 |x|.  The
 * kernels replace e_i by 0 when b_i r > 60; this header decides, once per
 * target, whether that replacement leaves every sum bit-identical:
 *
 *  (1) partial sums stay >= Z/2 wherever some term is dropped: all b_i >= 0,
 *      every term with b_i = 0 has a_i >= 0, and the negative terms that may
 *      still be evaluated there (r >= r_min = 60 / max b_i) sum to at most
 *      Z/4 in magnitude;
 *  (2) each dropped term is below 2^-57 Z (a margin of 4 over what (1) needs):
 *      for x = b r > 60, |a| e^-x, |a| (1+x) e^-x, (|a2|/b2) x e^-x and, for
 *      C, |a2 b2| (r^2 + sc) e^-x <= ((|a2|/b2) x^2 + |a2 b2| sc) e^-x, all
 *      decreasing in x, are bounded at x = 60;
 *  (3) every b_i > 0 is >= 1e-6, so exp(-b r) already underflows to 0 before
 *      s sqrt(s) leaves the normal range.
 * The presets of AtomDatabase.jl (He, Ne, Ar, Xe, ...) all pass.  The
 * function is shared by the kernels' host setup and the CPU oracle so that
 * both make the same decision. */
#ifndef ETRAJ_SAE_SKIP_H
#define ETRAJ_SAE_SKIP_H

#include <math.h>

static inline int etraj_sae_skip_exact(double Z, const double a[3], const double b[3], double sc) {
    const double e60 = 8.7565107626965203e-27; /* e^-60, rounded up in the 17th digit */
    const double lim = 6.9388939039072284e-18; /* 2^-57 */
    double bmax = 0.0;
    int i;
    if (!(Z >= 1.0) || !(sc >= 0.0) || !(sc < 1e6)) return 0;
    for (i = 0; i < 3; ++i) {
        if (!(b[i] >= 0.0) || a[i] != a[i] || fabs(a[i]) > 1e12) return 0;
        if (b[i] == 0.0 && a[i] < 0.0) return 0;
        if (b[i] > 0.0 && b[i] < 1e-6) return 0;
        if (b[i] > bmax) bmax = b[i];
    }
    if (bmax == 0.0) return 1; /* nothing is ever dropped */
    /* (2) dropped terms */
    for (i = 0; i < 3; ++i) {
        double ai = fabs(a[i]);
        if (b[i] == 0.0) continue;
        if (ai * 61.0 * e60 >= lim * Z) return 0; /* |a| (1+x) e^-x >= |a| e^-x */
    }
    if (b[1] > 0.0) {
        double q = fabs(a[1]) / b[1];
        if (q * 60.0 * e60 >= lim * Z) return 0;
        if ((q * 3600.0 + fabs(a[1] * b[1]) * sc) * e60 >= 0.25 * lim * Z) return 0;
    }
    /* (1) negative terms still evaluated where r >= r_min */
    {
        const double rmin = 60.0 / bmax;
        double neg_num = 0.0, neg_br = 0.0;
        for (i = 0; i < 3; ++i) {
            if (!(a[i] < 0.0)) continue;
            if (i == 1) {
                double rs = (rmin > 1.0 / b[1]) ? rmin : 1.0 / b[1];
                neg_num += -a[1] * rs * dm_exp(-b[1] * rs);
            } else {
                neg_num += -a[i] * dm_exp(-b[i] * rmin);
                neg_br += -a[i] * (1.0 + b[i] * rmin) * dm_exp(-b[i] * rmin);
            }
        }
        if (neg_num > 0.25 * Z || neg_br > 0.25 * Z) return 0;
    }
    return 1;
}

#endif
