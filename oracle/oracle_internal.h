/* oracle_internal.h -- shared declarations of the CPU oracle (TEST
 * INFRASTRUCTURE ONLY; see oracle.h). */
#ifndef ETRAJ_ORACLE_INTERNAL_H
#define ETRAJ_ORACLE_INTERNAL_H

#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include "oracle.h"
#include "../etraj.jl_gb300/csrc/detmath.h"
#include "../etraj.jl_gb300/csrc/sae_skip.h"
#include "../etraj.jl_gb300/csrc/mol_check.h"

typedef struct {
    int kind;
    double omega, period, F0, A0, N, cep, t_shift, ellip, azi;
    int azi_zero;
    double cphi, sphi;
    double w2n, cN, k, Npiw;      /* cos^n envelopes */
    double sigma, inv_s2, inv_2s2; /* Gaussian envelope */
} o_mono;

typedef struct {
    int kind, nmono;
    o_mono m[2];
    double delay;
} o_laser;

typedef struct {
    int kind;
    int skip_ok; /* exp(-b r) terms with b r > 60 may be dropped exactly (o_sae_exp) */
    double Z, Ip, sc, a1, b1, a2, b2, a3, b3;
} o_target;

/* exp(-b r) of the SAE potential.  For targets that pass
 * etraj_sae_skip_exact, every term this factor enters when b r > 60 is too
 * small to change the sum it is added to, so returning 0 leaves every result
 * bit-identical and saves the evaluation. */
static inline double o_sae_exp(const o_target* T, double b, double r) {
    if (T->skip_ok && b * r > 60.0) return 0.0;
    return dm_exp(-b * r);
}

typedef struct {
    int dim, phase, n;  /* n = ODE state size */
    double rtol;
    o_laser laser;
    o_target target;
} o_sys;

void o_mono_prepare(const etraj_mono_laser* in, o_mono* L);
void o_laser_prepare(const etraj_laser* in, o_laser* L);
void o_mono_F(const o_mono* L, double t, double* Fx, double* Fy);
void o_mono_A(const o_mono* L, double t, double* Ax, double* Ay);
double o_mono_env(const o_mono* L, double t);
void o_mono_F_dual(const o_mono* L, double t, double* Fx, double* Fy, double* dFx, double* dFy);
void o_mono_AF_complex(const o_mono* L, dm_cplx t, dm_cplx* Ax, dm_cplx* Ay, dm_cplx* Fx,
                       dm_cplx* Fy);
void o_laser_F(const o_laser* L, double t, double* Fx, double* Fy);
void o_laser_F_dual(const o_laser* L, double t, double* Fx, double* Fy, double* dFx, double* dFy);
void o_laser_A(const o_laser* L, double t, double* Ax, double* Ay);
void o_laser_AF_complex(const o_laser* L, dm_cplx t, dm_cplx* Ax, dm_cplx* Ay, dm_cplx* Fx,
                        dm_cplx* Fy);
void o_laser_windows(const o_laser* L, double tre, double* win);
void o_laser_AF_complex_w(const o_laser* L, dm_cplx t, const double* win, dm_cplx* Ax, dm_cplx* Ay,
                          dm_cplx* Fx, dm_cplx* Fy);
void o_target_prepare(const etraj_target* in, o_target* T);
double o_target_V(const o_target* T, double x, double y, double z);
void o_target_F(const o_target* T, double x, double y, double z, double* F);
void o_rhs(const o_sys* S, double t, const double* u, double* du);
void o_sys_prepare(const etraj_job* job, o_sys* S);

/* the spacing of doubles at |x| (Julia's eps(x)) */
static inline double o_ulp(double x) {
    double a = fabs(x);
    uint64_t u = dm_d2u(a);
    int e = (int)(u >> 52);
    if (e == 0) return dm_u2d(1);            /* subnormal or zero: 2^-1074 */
    if (e >= 2046) return dm_inf();
    int p = e - 1023 - 52;
    if (p >= -1022) return dm_pow2i(p);
    return dm_u2d(1ull << (p + 1074));
}

/* Julia's NaN-propagating min / max */
static inline double o_jmin(double a, double b) { return (a != a || b != b) ? a + b : (a < b ? a : b); }
static inline double o_jmax(double a, double b) { return (a != a || b != b) ? a + b : (a > b ? a : b); }

#endif
