/* spa.h -- the numerical pieces of the SFA saddle-point (SPA) sampler, shared
 * by the device kernel (sampler.cu) and the CPU oracle (oracle_sampler.c) so
 * both evaluate one sequence of floating-point operations.
 *
 * SPASampler.jl:150-431 builds every electron from
 *   - the imaginary part t_i of the saddle-point time t_s = t_r + i t_i, the
 *     root of Re[((p_x+A_x(t_s))^2 + (p_y+A_y(t_s))^2 + k_z^2)/2 + I_p] with
 *     p from px_/py_ (:230-240), solved by NLsolve's `nlsolve` with its
 *     defaults (:241-249);
 *   - the tunnel exit x0 = int_0^{t_i} Im A_x(t_r + i tau) dtau (and y0),
 *     and the tunnelling action S = -int_{t_s}^{t_r} (...) dt, all by
 *     QuadGK's `quadgk` with its defaults (:279, :355-356);
 *   - a finite-difference Jacobian from four further saddle-point solves
 *     (:280-292).
 * NLsolve 4.5.1 and QuadGK 2.11.1 are not part of the reference's sources;
 * what follows restates their published default algorithms:
 *
 *   spa_solve_ti: NLsolve's default `trust_region` method (dogleg step with
 *     autoscaling, Nocedal & Wright ch. 4 and 11; factor 1, eta 1e-4,
 *     ftol 1e-8, xtol 0, at most 1000 iterations), with the Jacobian by
 *     central finite differences (FiniteDiff: step max(r|x|, r),
 *     r = cbrt(eps)).  In one dimension the dogleg reduces to the Newton
 *     step clipped to the trust radius; the general formulas are kept.
 *   spa_quadgk: adaptive Gauss-Kronrod (7, 15) quadrature on a straight
 *     complex segment, splitting the interval of largest error estimate
 *     |K15 - G7| until it is <= rtol |I| (rtol = sqrt(eps), atol 0), with a
 *     binary max-heap of intervals and a final re-summation in heap order.
 *
 * The including file defines
 *   SPA_LASER_T                       the laser description type,
 *   SPA_WIN(L, tre, w)                what A at complex time needs of its
 *                                     real part tre alone (the tanh window
 *                                     factors, and whatever else the includer
 *                                     caches; double w[12] at most), and
 *   SPA_AW(L, t, w, ax, ay)           A_x, A_y at complex time t (dm_cplx*)
 *                                     from those values w at Re t.
 * Re t is the same for all but a few evaluations of one electron (every
 * quadrature node and every iterate of a solve share t_r), so those values
 * are cached per thread in a spa_win keyed by Re t.
 */
#ifndef ETRAJ_SPA_H
#define ETRAJ_SPA_H

#ifndef SPA_LASER_T
#error "spa.h: define SPA_LASER_T, SPA_WIN and SPA_AW before including"
#endif

/* The heavy pieces are real functions on the device: inlined at every call
 * site they made the sampler's compilation take minutes.  With contraction
 * off the results do not depend on inlining. */
#ifdef __CUDACC__
#define SPA_HEAVY static __host__ __device__ __noinline__
#else
#define SPA_HEAVY static
#endif

typedef struct {
    double key; /* Re t of w[] (NaN: empty) */
    double w[12]; /* what the including file caches per Re t (SPA_WIN), at most 6 per laser */
} spa_win;

DM_FN void spa_win_init(spa_win* W) { W->key = dm_u2d(0x7ff8000000000000ull); }

SPA_HEAVY void spa_A(const SPA_LASER_T* L, spa_win* W, dm_cplx t, dm_cplx* ax, dm_cplx* ay) {
    if (!(W->key == t.re)) {
        SPA_WIN(L, t.re, W->w);
        W->key = t.re;
    }
    SPA_AW(L, t, W->w, ax, ay);
}

/* momenta of the saddle-point solution (px_, py_, SPASampler.jl:230-231) */
DM_FN void spa_pxy(double kd, dm_cplx Ax, dm_cplx Ay, double* px, double* py) {
    const double den = sqrt(Ax.im * Ax.im + Ay.im * Ay.im);
    *px = (kd * Ay.im) / den - Ax.re;
    *py = ((-kd) * Ax.im) / den - Ay.re;
}

/* saddle_point_equation (SPASampler.jl:233-239) */
DM_FN double spa_spe(const SPA_LASER_T* L, spa_win* W, double tr, double ti, double kd, double kz, double Ip) {
    dm_cplx Ax, Ay;
    spa_A(L, W, dm_c(tr, ti), &Ax, &Ay);
    double px, py;
    spa_pxy(kd, Ax, Ay, &px, &py);
    const double ur = px + Ax.re, ui = Ax.im, vr = py + Ay.re, vi = Ay.im;
    const double u2 = ur * ur - ui * ui, v2 = vr * vr - vi * vi;
    return ((u2 + v2) + kz * kz) / 2.0 + Ip;
}

/* central-difference derivative of spa_spe in t_i (FiniteDiff defaults) */
DM_FN double spa_dspe(const SPA_LASER_T* L, spa_win* W, double tr, double x, double kd, double kz, double Ip) {
    const double rel = 6.0554544523933395e-06; /* cbrt(eps(Float64)) */
    const double ax = fabs(x);
    const double e = (rel * ax > rel) ? rel * ax : rel;
    const double f1 = spa_spe(L, W, tr, x + e, kd, kz, Ip);
    const double f0 = spa_spe(L, W, tr, x - e, kd, kz, Ip);
    return (f1 - f0) / (2.0 * e);
}

/* t_i of the saddle point from the initial guess x0; returns 0 when the
 * solve does not converge or t_i <= 0 (solve_spe, SPASampler.jl:241-249). */
SPA_HEAVY double spa_solve_ti(const SPA_LASER_T* L, spa_win* W, double tr, double kd, double kz, double Ip,
                          double x0) {
    const double ftol = 1e-8, eta = 1e-4;
    double x = x0;
    double r = spa_spe(L, W, tr, x, kd, kz, Ip);
    if (dm_isnan(r) || dm_isinf(r)) return 0.0; /* NLsolve rejects a non-finite f(x0) */
    int converged = (fabs(r) <= ftol);
    if (dm_isnan(x)) return 0.0;
    if (converged) return (x > 0.0) ? x : 0.0;
    /* the Jacobian is only needed for a further step: it is evaluated after
     * the convergence test, which changes no iterate */
    double J = spa_dspe(L, W, tr, x, kd, kz, Ip);
    double d = fabs(J);
    if (d == 0.0) d = 1.0;
    double delta = fabs(d * x);
    if (delta == 0.0) delta = 1.0;
    for (int it = 0; it < 1000 && !converged; ++it) {
        /* dogleg step */
        double p;
        if (J == 0.0) {
            /* singular Jacobian: the least-squares step is 0, which repeats
             * until the iteration limit, i.e. no convergence */
            return 0.0;
        }
        const double pn = -(r / J);
        if (fabs(d * pn) <= delta) {
            p = pn;
        } else {
            const double g = (J * r) / (d * d);
            const double wg = fabs(d * g);
            const double Jg = J * g;
            const double pc = ((-(wg * wg)) / (Jg * Jg)) * g;
            if (fabs(d * pc) >= delta) {
                p = g * (-delta / wg);
            } else {
                const double df = pn - pc;
                const double b = 2.0 * ((d * pc) * (d * df));
                const double a = (d * df) * (d * df);
                const double wc = fabs(d * pc);
                const double tau = (-b + sqrt(b * b - (4.0 * a) * (wc * wc - delta * delta))) / (2.0 * a);
                p = pc + tau * df;
            }
        }
        const double xold = x;
        x = x + p;
        const double fn = spa_spe(L, W, tr, x, kd, kz, Ip);
        const double rp = J * p + r;
        const double rho = (r * r - fn * fn) / (r * r - rp * rp);
        if (rho > eta) {
            r = fn;
            converged = (fabs(x - xold) <= 0.0) || (fabs(r) <= ftol);
            if (converged) break;
            J = spa_dspe(L, W, tr, x, kd, kz, Ip);
            const double dj = fabs(J), d1 = 0.1 * d;
            d = (d1 > dj) ? d1 : dj;
        } else {
            x = x - p;
        }
        if (rho < 0.1) {
            delta = delta / 2.0;
        } else if (rho >= 0.9) {
            delta = 2.0 * fabs(d * p);
        } else if (rho >= 0.5) {
            const double dd = 2.0 * fabs(d * p);
            delta = (delta > dd) ? delta : dd;
        }
        if (dm_isnan(x) || dm_isnan(fn)) break;
    }
    if (!converged || !(x > 0.0)) return 0.0;
    return x;
}

/* ---- quadrature ---------------------------------------------------------- */
/* SPA_INT_IM_AXY evaluates the first two together (one A per node) */
enum { SPA_INT_IM_AX = 0, SPA_INT_IM_AY = 1, SPA_INT_ACTION = 2, SPA_INT_IM_AXY = 3 };

typedef struct {
    const SPA_LASER_T* L;
    spa_win* W;
    double tr, px, py, kz, Ip;
} spa_quad_par;

/* integrands: Im A_x(t_r + i tau), Im A_y(t_r + i tau) (tau = Re t) and
 * ((p_x+A_x(t))^2 + (p_y+A_y(t))^2 + k_z^2)/2 + I_p at complex t; v1 is the
 * second integrand of SPA_INT_IM_AXY */
DM_FN dm_cplx spa_integrand(int kind, const spa_quad_par* P, dm_cplx t, dm_cplx* v1) {
    dm_cplx Ax, Ay;
    if (kind != SPA_INT_ACTION) {
        spa_A(P->L, P->W, dm_c(P->tr, t.re), &Ax, &Ay);
        *v1 = dm_c(Ay.im, 0.0);
        return dm_c(kind == SPA_INT_IM_AY ? Ay.im : Ax.im, 0.0);
    }
    spa_A(P->L, P->W, t, &Ax, &Ay);
    const dm_cplx u = dm_c(P->px + Ax.re, Ax.im), v = dm_c(P->py + Ay.re, Ay.im);
    dm_cplx s = dm_cadd(dm_cmul(u, u), dm_cmul(v, v));
    s = dm_caddr(s, P->kz * P->kz);
    s = dm_c(s.re / 2.0, s.im / 2.0);
    *v1 = dm_c(0.0, 0.0);
    return dm_caddr(s, P->Ip);
}

typedef struct {
    dm_cplx a, b, I;
    double E;
} spa_seg;

DM_FN double spa_norm(dm_cplx z) { return (z.im == 0.0) ? fabs(z.re) : dm_hypot(z.re, z.im); }

/* Gauss-Kronrod (7, 15) rule on [a, b] (nodes and weights of the 15-point
 * Kronrod extension of the 7-point Gauss rule, Kronrod 1965).  g1 receives
 * the rule of the second integrand of SPA_INT_IM_AXY (same arithmetic as a
 * separate pass; may be NULL otherwise). */
SPA_HEAVY spa_seg spa_evalrule2(int kind, const spa_quad_par* P, dm_cplx a, dm_cplx b, spa_seg* g1) {
    const double x[8] = {-0.991455371120812639206854697526329, -0.949107912342758524526189684047851,
                         -0.864864423359769072789712788640926, -0.741531185599394439863864773280788,
                         -0.586087235467691130294144845693013, -0.405845151377397166906606412076961,
                         -0.207784955007898467600689403773245, 0.0};
    const double w[8] = {0.022935322010529224963732008058970, 0.063092092629978553290700663189204,
                         0.104790010322250183839876322541518, 0.140653259715525918745189590510238,
                         0.169004726639267902826583426598550, 0.190350578064785409913256402421014,
                         0.204432940075298892414161999234649, 0.209482141084727828012999174891714};
    const double gw[4] = {0.129484966168869693270611432679082, 0.279705391489276667901467771423780,
                          0.381830050505118944950369775488975, 0.417959183673469387755102040816327};
    const dm_cplx s = dm_cscale(dm_csub(b, a), 0.5);
    dm_cplx u1, u2, fg, fk, hg, hk, Ig, Ik, Jg, Jk;
#define SPA_F2(i, f, h)                                                                  \
    do {                                                                                 \
        const dm_cplx p_ = spa_integrand(kind, P, dm_cadd(a, dm_cscale(s, 1.0 + x[i])), &u1); \
        const dm_cplx q_ = spa_integrand(kind, P, dm_cadd(a, dm_cscale(s, 1.0 - x[i])), &u2); \
        f = dm_cadd(p_, q_);                                                             \
        h = dm_cadd(u1, u2);                                                             \
    } while (0)
    SPA_F2(1, fg, hg);
    SPA_F2(0, fk, hk);
    Ig = dm_cscale(fg, gw[0]);
    Ik = dm_cadd(dm_cscale(fg, w[1]), dm_cscale(fk, w[0]));
    Jg = dm_cscale(hg, gw[0]);
    Jk = dm_cadd(dm_cscale(hg, w[1]), dm_cscale(hk, w[0]));
    for (int i = 2; i <= 3; ++i) {
        SPA_F2(2 * i - 1, fg, hg);
        SPA_F2(2 * i - 2, fk, hk);
        Ig = dm_cadd(Ig, dm_cscale(fg, gw[i - 1]));
        Ik = dm_cadd(Ik, dm_cadd(dm_cscale(fg, w[2 * i - 1]), dm_cscale(fk, w[2 * i - 2])));
        Jg = dm_cadd(Jg, dm_cscale(hg, gw[i - 1]));
        Jk = dm_cadd(Jk, dm_cadd(dm_cscale(hg, w[2 * i - 1]), dm_cscale(hk, w[2 * i - 2])));
    }
    const dm_cplx f0 = spa_integrand(kind, P, dm_cadd(a, s), &u1);
    const dm_cplx h0 = u1;
    SPA_F2(6, fg, hg);
    Ig = dm_cadd(Ig, dm_cscale(f0, gw[3]));
    Ik = dm_cadd(Ik, dm_cadd(dm_cscale(f0, w[7]), dm_cscale(fg, w[6])));
    Jg = dm_cadd(Jg, dm_cscale(h0, gw[3]));
    Jk = dm_cadd(Jk, dm_cadd(dm_cscale(h0, w[7]), dm_cscale(hg, w[6])));
#undef SPA_F2
    spa_seg g;
    g.a = a;
    g.b = b;
    g.I = dm_cmul(Ik, s);
    g.E = spa_norm(dm_csub(g.I, dm_cmul(Ig, s)));
    if (g1) {
        g1->a = a;
        g1->b = b;
        g1->I = dm_cmul(Jk, s);
        g1->E = spa_norm(dm_csub(g1->I, dm_cmul(Jg, s)));
    }
    return g;
}

DM_FN spa_seg spa_evalrule(int kind, const spa_quad_par* P, dm_cplx a, dm_cplx b) {
    return spa_evalrule2(kind, P, a, b, (spa_seg*)0);
}

#define SPA_MAX_SEGS 48

DM_FN void spa_heap_up(spa_seg* h, int i) {
    const spa_seg x = h[i];
    while (i > 0) {
        const int p = (i - 1) / 2;
        if (!(h[p].E < x.E)) break;
        h[i] = h[p];
        i = p;
    }
    h[i] = x;
}

DM_FN void spa_heap_down(spa_seg* h, int n, int i) {
    const spa_seg x = h[i];
    for (;;) {
        const int l = 2 * i + 1;
        if (l >= n) break;
        const int r = l + 1;
        const int j = (r >= n || h[r].E < h[l].E) ? l : r; /* ties go right, as in DataStructures */
        if (!(x.E < h[j].E)) break;
        h[i] = h[j];
        i = j;
    }
    h[i] = x;
}

/* integral of `kind` whose first Kronrod pass over the whole segment is
 * `first`; *ok = 0 when the estimate is not finite or the interval budget
 * runs out before the tolerance is met */
SPA_HEAVY dm_cplx spa_quadgk_from(int kind, const spa_quad_par* P, spa_seg first, int* ok) {
    const double rtol = 1.4901161193847656e-08; /* sqrt(eps(Float64)) */
    spa_seg h[SPA_MAX_SEGS];
    h[0] = first;
    dm_cplx I = h[0].I;
    double E = h[0].E;
    *ok = !(dm_isnan(E) || dm_isinf(E));
    if (!*ok) return I;
    if (E <= 0.0 || E <= rtol * spa_norm(I)) return I;
    int n = 1;
    while (rtol * spa_norm(I) < E) {
        if (n + 1 > SPA_MAX_SEGS) {
            *ok = 0;
            break;
        }
        /* pop the interval of largest error */
        const spa_seg s = h[0];
        h[0] = h[n - 1];
        --n;
        if (n > 0) spa_heap_down(h, n, 0);
        const dm_cplx mid = dm_cscale(dm_cadd(s.a, s.b), 0.5);
        const spa_seg s1 = spa_evalrule(kind, P, s.a, mid);
        const spa_seg s2 = spa_evalrule(kind, P, mid, s.b);
        if (dm_isnan(s1.E) || dm_isnan(s2.E) || dm_isinf(s1.E) || dm_isinf(s2.E)) {
            *ok = 0;
            return I;
        }
        I = dm_cadd(dm_cadd(dm_csub(I, s.I), s1.I), s2.I);
        E = ((E - s.E) + s1.E) + s2.E;
        h[n] = s1;
        spa_heap_up(h, n);
        ++n;
        h[n] = s2;
        spa_heap_up(h, n);
        ++n;
    }
    I = h[0].I;
    for (int i = 1; i < n; ++i) I = dm_cadd(I, h[i].I);
    return I;
}

DM_FN dm_cplx spa_quadgk(int kind, const spa_quad_par* P, dm_cplx a, dm_cplx b, int* ok) {
    return spa_quadgk_from(kind, P, spa_evalrule(kind, P, a, b), ok);
}

/* x0 and y0 (SPASampler.jl:355-356): both integrals from one first pass */
DM_FN void spa_exit(const spa_quad_par* P, double ti, double* x0, double* y0, int* ok) {
    spa_seg sy;
    const spa_seg sx = spa_evalrule2(SPA_INT_IM_AXY, P, dm_c(0.0, 0.0), dm_c(ti, 0.0), &sy);
    int okx, oky;
    *x0 = spa_quadgk_from(SPA_INT_IM_AX, P, sx, &okx).re;
    *y0 = spa_quadgk_from(SPA_INT_IM_AY, P, sy, &oky).re;
    *ok = okx && oky;
}

/* jac(kd, kz) (SPASampler.jl:280-292): |d(px,py)/d(tr,kd)| by central
 * differences of four saddle-point solves (a failed solve enters as t_i = 0). */
SPA_HEAVY double spa_jac(const SPA_LASER_T* L, spa_win* W, double tr, double kd, double kz, double Ip,
                     double omega_over_F, double omega) {
    const double dtr = 0.01, dkd = 0.01;
#define SPA_GUESS(k) (dm_asinh(omega_over_F * sqrt(((k) * (k) + kz * kz) + 2.0 * Ip)) / omega)
    const double ti_tp = spa_solve_ti(L, W, tr + dtr, kd, kz, Ip, SPA_GUESS(kd));
    const double ti_tm = spa_solve_ti(L, W, tr - dtr, kd, kz, Ip, SPA_GUESS(kd));
    const double ti_kp = spa_solve_ti(L, W, tr, kd + dkd, kz, Ip, SPA_GUESS(kd + dkd));
    const double ti_km = spa_solve_ti(L, W, tr, kd - dkd, kz, Ip, SPA_GUESS(kd - dkd));
#undef SPA_GUESS
    dm_cplx ax, ay;
    double pxa, pya, pxb, pyb;
    spa_A(L, W, dm_c(tr + dtr, ti_tp), &ax, &ay);
    spa_pxy(kd, ax, ay, &pxa, &pya);
    spa_A(L, W, dm_c(tr - dtr, ti_tm), &ax, &ay);
    spa_pxy(kd, ax, ay, &pxb, &pyb);
    const double dpxdtr = pxa - pxb, dpydtr = pya - pyb;
    spa_A(L, W, dm_c(tr, ti_kp), &ax, &ay);
    spa_pxy(kd + dkd, ax, ay, &pxa, &pya);
    spa_A(L, W, dm_c(tr, ti_km), &ax, &ay);
    spa_pxy(kd - dkd, ax, ay, &pxb, &pyb);
    const double dpxdkd = pxa - pxb, dpydkd = pya - pyb;
    return fabs(dpxdtr * dpydkd - dpxdkd * dpydtr) / ((4.0 * dtr) * dkd);
}

/* principal z^p of a complex z and real p (Julia's Complex ^ Real: |z|^p cis(p arg z)) */
DM_FN dm_cplx spa_cpow(dm_cplx z, double p) {
    if (p == 1.0) return z;
    const double az = dm_hypot(z.re, z.im);
    if (az == 0.0) return dm_c(0.0, 0.0);
    const double r = dm_pow_pos(az, p);
    double s, c;
    dm_sincos(p * dm_atan2(z.im, z.re), &s, &c);
    return dm_c(r * c, r * s);
}

#endif /* ETRAJ_SPA_H */
