/* oracle_spa_ref.c -- an independent restatement of the SFA-SPA candidate, for
 * checking the SPA solver and quadratures the device kernel and the oracle's
 * bit-exact twin (oracle_sampler.c, o_candidate_spa) share.  TEST
 * INFRASTRUCTURE ONLY: nothing in the product includes or calls this file.
 *
 * It follows SPASampler.jl:150-431 with nothing of the shared code: C99
 * complex arithmetic and the C library's elementary functions, the laser's
 * vector potential and field at complex time written out from the reference's
 * formulas (Cos4Laser.jl:97-150, Cos2Laser.jl:97-151, GaussianLaser.jl:105-158,
 * BichromaticLaser.jl:59-85), and its own statements of the two third-party
 * algorithms the reference calls with their defaults:
 *   - NLsolve 4.5 `nlsolve(f, x0)`: the trust-region method (Nocedal & Wright,
 *     "Numerical Optimization", algorithm 4.1 with the dogleg step, the scaling
 *     d_j = column norms of J kept at >= 0.1 of their previous value; initial
 *     radius |d x0|, eta = 1e-4, ftol 1e-8, xtol 0, 1000 iterations) with a
 *     central finite-difference Jacobian (step max(r |x|, r), r = eps^(1/3)).
 *     In one unknown the dogleg path is the Newton step, cut back to the trust
 *     radius when it leaves it (the Cauchy point lies on the Newton step).
 *   - QuadGK 2.11 `quadgk(f, a, b)`: adaptive Gauss-Kronrod (7, 15) on the
 *     straight segment a -> b, bisecting the piece of largest |K15 - G7| until
 *     the summed estimate is <= sqrt(eps) |I|.
 * The results agree with the twin's to rounding, not to the bit (other
 * orders of operations, the C library's functions); the tests compare them at
 * a stated tolerance.  Atoms only (molecular SPA prefactors stay in the twin). */
#include <math.h>
#include <stdlib.h>

#include "oracle_sampler.h"

#include <complex.h>
#undef I /* the imaginary unit is IU here: I names arrays in the headers above */
#define IU _Complex_I

typedef double complex zc;

/* ---- laser at complex time -------------------------------------------------------- */
/* one monochromatic component at complex t: A and F = -dA/dt */
static void ref_mono_AF(const o_mono* M, zc t, zc* Ax, zc* Ay, zc* Fx, zc* Fy) {
    t -= M->t_shift;
    const double w = M->omega, eps = M->ellip;
    const double cphi = cos(M->azi), sphi = sin(M->azi);
    zc ua, va, uf, vf; /* A and F before the azimuthal rotation: (u, eps v) */
    const zc ph = w * t + M->cep;
    const zc cp = ccos(ph), sp = csin(ph);
    if (M->kind == ETRAJ_LASER_GAUSSIAN) {
        const double sig = M->sigma;
        const zc g = cexp(-(t * t) / 2.0 / (sig * sig));
        ua = M->A0 * g * cp;
        va = M->A0 * g * sp;
        uf = M->A0 * g * (t / (sig * sig) * cp + w * sp);
        vf = M->A0 * g * (t / (sig * sig) * sp - w * cp);
    } else {
        /* cos^4 (Cos4) or cos^2 (Cos2) envelope, with the reference's tanh windows
         * at +-N pi / omega (k = 200 / period) applied to Re t */
        const double N = M->N, tr = creal(t), k = 200.0 / M->period;
        const double win = (0.5 + 0.5 * tanh(k * (tr + N * M_PI / w))) * (0.5 + 0.5 * tanh(-k * (tr - N * M_PI / w)));
        const zc ce = ccos(w * t / (2.0 * N)), se = csin(w * t / (2.0 * N));
        const int four = (M->kind == ETRAJ_LASER_COS4);
        const zc envA = four ? (ce * ce) * (ce * ce) : ce * ce;
        const zc envF = four ? ce * ce * ce : ce;
        const double q = four ? 2.0 / N : 1.0 / N;
        ua = M->A0 * envA * win * cp;
        va = M->A0 * envA * win * sp;
        uf = M->F0 * envF * win * (ce * sp + q * se * cp);
        vf = M->F0 * envF * win * (-ce * cp + q * se * sp);
    }
    *Ax = ua * cphi + eps * va * sphi;
    *Ay = -ua * sphi + eps * va * cphi;
    *Fx = uf * cphi + eps * vf * sphi;
    *Fy = -uf * sphi + eps * vf * cphi;
}

static void ref_laser_AF(const o_laser* L, zc t, zc* Ax, zc* Ay, zc* Fx, zc* Fy) {
    ref_mono_AF(&L->m[0], t, Ax, Ay, Fx, Fy);
    if (L->nmono == 2) {
        zc ax, ay, fx, fy;
        ref_mono_AF(&L->m[1], t - L->delay, &ax, &ay, &fx, &fy);
        *Ax += ax;
        *Ay += ay;
        *Fx += fx;
        *Fy += fy;
    }
}

static void ref_A(const o_laser* L, zc t, zc* Ax, zc* Ay) {
    zc fx, fy;
    ref_laser_AF(L, t, Ax, Ay, &fx, &fy);
}

/* ---- saddle-point equation and its solve ----------------------------------------- */
typedef struct {
    const o_laser* L;
    double tr, kd, kz, Ip;
} ref_spe_par;

/* px_, py_ (SPASampler.jl:231-232) */
static void ref_pxy(double kd, zc Ax, zc Ay, double* px, double* py) {
    const double n = sqrt(cimag(Ax) * cimag(Ax) + cimag(Ay) * cimag(Ay));
    *px = kd * cimag(Ay) / n - creal(Ax);
    *py = -kd * cimag(Ax) / n - creal(Ay);
}

/* saddle_point_equation (SPASampler.jl:233-239) */
static double ref_spe(const ref_spe_par* P, double ti) {
    zc Ax, Ay;
    ref_A(P->L, P->tr + IU * ti, &Ax, &Ay);
    double px, py;
    ref_pxy(P->kd, Ax, Ay, &px, &py);
    const zc s = ((px + Ax) * (px + Ax) + (py + Ay) * (py + Ay) + P->kz * P->kz) / 2.0 + P->Ip;
    return creal(s);
}

static double ref_jacobian(const ref_spe_par* P, double x) {
    const double r = cbrt(2.220446049250313e-16);
    const double h = fmax(r * fabs(x), r);
    return (ref_spe(P, x + h) - ref_spe(P, x - h)) / (2.0 * h);
}

/* solve_spe (SPASampler.jl:240-250): t_i > 0 of a converged solve, else 0 */
static double ref_solve_ti(const ref_spe_par* P, double x0) {
    const double ftol = 1e-8, eta = 1e-4;
    double x = x0, f = ref_spe(P, x);
    if (!isfinite(f)) return 0.0;
    double J = ref_jacobian(P, x);
    double d = fabs(J) > 0.0 ? fabs(J) : 1.0;
    double radius = fabs(d * x) > 0.0 ? fabs(d * x) : 1.0;
    int conv = fabs(f) <= ftol;
    for (int it = 0; it < 1000 && !conv; ++it) {
        if (J == 0.0) return 0.0; /* no Newton direction: the solve stalls */
        double p = -f / J;
        if (fabs(d * p) > radius) p = copysign(radius / d, p);
        const double xn = x + p, fn = ref_spe(P, xn);
        const double fpred = f + J * p;
        const double rho = (f * f - fn * fn) / (f * f - fpred * fpred);
        if (rho > eta) {
            const double xold = x;
            x = xn;
            f = fn;
            J = ref_jacobian(P, x);
            d = fmax(0.1 * d, fabs(J));
            conv = (x == xold) || (fabs(f) <= ftol);
        }
        if (rho < 0.1) radius /= 2.0;
        else if (rho >= 0.9) radius = 2.0 * fabs(d * p);
        else if (rho >= 0.5) radius = fmax(radius, 2.0 * fabs(d * p));
        if (isnan(x) || isnan(fn)) break;
    }
    return (conv && x > 0.0) ? x : 0.0;
}

/* ---- adaptive Gauss-Kronrod on a complex segment ------------------------------------ */
/* the (7, 15) rule: abscissae and weights of the published Gauss-Kronrod pair
 * (QUADPACK's qk15), positive half, the last abscissa the centre */
static const double GK_X[8] = {0.991455371120812639206854697526329, 0.949107912342758524526189684047851,
                               0.864864423359769072789712788640926, 0.741531185599394439863864773280788,
                               0.586087235467691130294144845693013, 0.405845151377397166906606412076961,
                               0.207784955007898467600689403773245, 0.0};
static const double GK_WK[8] = {0.022935322010529224963732008058970, 0.063092092629978553290700663189204,
                                0.104790010322250183839876322541518, 0.140653259715525918745189590510238,
                                0.169004726639267902826583426598550, 0.190350578064785409913256402421014,
                                0.204432940075298892414161999234649, 0.209482141084727828012999174891714};
/* Gauss weights of the abscissae GK_X[1], [3], [5], [7] */
static const double GK_WG[4] = {0.129484966168869693270611432679082, 0.279705391489276667901467771423780,
                                0.381830050505118944950369775488975, 0.417959183673469387755102040816327};

typedef zc (*ref_fn)(const void* ctx, zc t);
typedef struct {
    zc a, b, I;
    double E;
} ref_piece;

static ref_piece ref_rule(ref_fn f, const void* ctx, zc a, zc b) {
    const zc c = (a + b) / 2.0, h = (b - a) / 2.0;
    zc k = 0.0, g = 0.0;
    for (int i = 0; i < 7; ++i) {
        const zc v = f(ctx, c - h * GK_X[i]) + f(ctx, c + h * GK_X[i]);
        k += GK_WK[i] * v;
        if (i & 1) g += GK_WG[i / 2] * v;
    }
    const zc v0 = f(ctx, c);
    k += GK_WK[7] * v0;
    g += GK_WG[3] * v0;
    ref_piece p = {a, b, k * h, cabs((k - g) * h)};
    return p;
}

/* integral of f from a to b; *ok = 0 when an estimate is not finite or the
 * pieces run out (QuadGK's evaluation limit is 1e7, ~6.7e5 pieces) */
static zc ref_quadgk(ref_fn f, const void* ctx, zc a, zc b, int* ok) {
    const double rtol = sqrt(2.220446049250313e-16);
    enum { CAP = 4096 };
    ref_piece* P = (ref_piece*)malloc(sizeof(ref_piece) * CAP);
    int n = 1;
    P[0] = ref_rule(f, ctx, a, b);
    zc Itot = P[0].I;
    double Etot = P[0].E;
    *ok = isfinite(Etot);
    while (*ok && Etot > 0.0 && Etot > rtol * cabs(Itot)) {
        if (n + 1 > CAP) {
            *ok = 0;
            break;
        }
        int w = 0;
        for (int i = 1; i < n; ++i)
            if (P[i].E > P[w].E) w = i;
        const ref_piece s = P[w];
        const zc mid = (s.a + s.b) / 2.0;
        P[w] = ref_rule(f, ctx, s.a, mid);
        P[n] = ref_rule(f, ctx, mid, s.b);
        if (!isfinite(P[w].E) || !isfinite(P[n].E)) *ok = 0;
        ++n;
        Itot = 0.0;
        Etot = 0.0;
        for (int i = 0; i < n; ++i) {
            Itot += P[i].I;
            Etot += P[i].E;
        }
    }
    free(P);
    return Itot;
}

typedef struct {
    const o_laser* L;
    double tr, px, py, kz, Ip;
    int comp; /* 0: Im A_x, 1: Im A_y at t_r + i tau; 2: the action integrand */
} ref_quad_par;

static zc ref_integrand(const void* ctx, zc t) {
    const ref_quad_par* Q = (const ref_quad_par*)ctx;
    zc Ax, Ay;
    if (Q->comp < 2) {
        ref_A(Q->L, Q->tr + IU * creal(t), &Ax, &Ay);
        return cimag(Q->comp == 0 ? Ax : Ay);
    }
    ref_A(Q->L, t, &Ax, &Ay);
    return ((Q->px + Ax) * (Q->px + Ax) + (Q->py + Ay) * (Q->py + Ay) + Q->kz * Q->kz) / 2.0 + Q->Ip;
}

/* ---- the candidate ------------------------------------------------------------------- */
static dm_cplx to_dm(zc z) { return dm_c(creal(z), cimag(z)); }
static zc from_dm(dm_cplx z) { return z.re + IU * z.im; }

/* jac(kd, kz) (SPASampler.jl:280-292) */
static double ref_jac(const o_laser* L, double tr, double kd, double kz, double Ip, double omega, double F) {
    const double dtr = 0.01, dkd = 0.01;
    double ti[4], pxv[4], pyv[4];
    const double trs[4] = {tr + dtr, tr - dtr, tr, tr}, kds[4] = {kd, kd, kd + dkd, kd - dkd};
    for (int j = 0; j < 4; ++j) {
        const ref_spe_par P = {L, trs[j], kds[j], kz, Ip};
        ti[j] = ref_solve_ti(&P, asinh(omega / F * sqrt(kds[j] * kds[j] + kz * kz + 2.0 * Ip)) / omega);
        zc Ax, Ay;
        ref_A(L, trs[j] + IU * ti[j], &Ax, &Ay);
        ref_pxy(kds[j], Ax, Ay, &pxv[j], &pyv[j]);
    }
    const double dpxdtr = pxv[0] - pxv[1], dpydtr = pyv[0] - pyv[1];
    const double dpxdkd = pxv[2] - pxv[3], dpydkd = pyv[2] - pyv[3];
    return fabs(dpxdtr * dpydkd - dpxdkd * dpydtr) / (4.0 * dtr * dkd);
}

/* One SPA candidate of an atomic target (SPASampler.jl:320-347 for the grid,
 * :364-391 for Monte-Carlo); the batch is skipped before this when F(t_r) <= 1e-3. */
int o_candidate_spa_ref(const o_sampler* S, const o_batch* B, double kd0, double kz0, double* row) {
    if (S->mol) return o_candidate_spa(S, B, kd0, kz0, row);
    if (fabs(kd0) < 1e-4) return 0;
    const o_laser* L = &S->laser;
    const double tr = B->tr, Ip = S->Ip, w = S->spa_omega;
    const ref_spe_par SP = {L, tr, kd0, kz0, Ip};
    const double ti = ref_solve_ti(&SP, asinh(w / B->F * sqrt(kd0 * kd0 + kz0 * kz0 + 2.0 * Ip)) / w);
    if (ti == 0.0) return 0;
    const zc ts = tr + IU * ti;
    zc Ax, Ay, Fx, Fy;
    ref_laser_AF(L, ts, &Ax, &Ay, &Fx, &Fy);
    double px, py;
    ref_pxy(kd0, Ax, Ay, &px, &py);
    int ok1, ok2, ok3;
    ref_quad_par Q = {L, tr, px, py, kz0, Ip, 0};
    const double x0 = creal(ref_quadgk(ref_integrand, &Q, 0.0, ti, &ok1));
    Q.comp = 1;
    const double y0 = creal(ref_quadgk(ref_integrand, &Q, 0.0, ti, &ok2));
    zc Ar, Ayr, Fr, Fyr;
    ref_laser_AF(L, tr, &Ar, &Ayr, &Fr, &Fyr);
    const double kx0 = px + creal(Ar), ky0 = py + creal(Ayr);
    Q.comp = 2;
    const zc S_tun = -ref_quadgk(ref_integrand, &Q, ts, tr, &ok3);
    if (!(ok1 && ok2 && ok3)) return 0;
    zc amp = sqrt(S->dkdt) * cexp(IU * S_tun);
    if (S->prefix & (ETRAJ_PREFIX_PRE | ETRAJ_PREFIX_PRECC)) {
        const zc kx = px + Ax, ky = py + Ay, kz = kz0;
        const zc num = from_dm(o_pre_numerator(S, B, to_dm(kx), to_dm(ky), to_dm(kz)));
        const double c = (S->prefix & ETRAJ_PREFIX_PRE) ? S->c : B->c_cc;
        amp *= c * num / cpow(kx * Fx + ky * Fy + kz * 0.0, (S->n + 1.0) / 2.0);
    }
    if (S->prefix & ETRAJ_PREFIX_JAC) amp *= sqrt(ref_jac(L, tr, kd0, kz0, Ip, w, B->F));
    const double rate = creal(amp) * creal(amp) + cimag(amp) * cimag(amp);
    if (isnan(rate) || rate < S->cutoff) return 0;
    int k = 0;
    row[k++] = x0;
    row[k++] = y0;
    if (S->dim == 3) row[k++] = 0.0;
    row[k++] = kx0;
    row[k++] = ky0;
    if (S->dim == 3) row[k++] = kz0;
    row[k++] = tr;
    row[k++] = rate;
    if (S->phase != ETRAJ_PHASE_CTMC) row[k++] = carg(amp);
    return 1;
}
