/*
 * oracle_physics.c -- lasers and targets of the CPU oracle (TEST INFRASTRUCTURE
 * ONLY; see oracle.h).
 *
 * Restates:
 *   src/Lasers/Cos4Laser.jl:81-152, Cos2Laser.jl:81-152,
 *   GaussianLaser.jl:85-160, BichromaticLaser.jl:59-85
 *   src/Targets/HydrogenLikeAtom.jl:66-159, SAEAtom.jl:84-186,
 *   SAEAtomBase_shared.jl:3-11
 *
 * Canonical arithmetic: every expression keeps the reference's
 * left-to-right association; three places replace an operation by an
 * equal one that is cheaper on the device and are used identically by the
 * device kernels: omega*t/(2N) is t*(omega/(2N)); s^(-1.5) is
 * 1/(s*sqrt(s)); s^(-0.5) is 1/sqrt(s); X^1.5 is X*sqrt(X).
 */
#include "oracle_internal.h"

/* ---- lasers ------------------------------------------------------------------ */

void o_mono_prepare(const etraj_mono_laser* in, o_mono* L) {
    memset(L, 0, sizeof *L);
    L->kind = in->kind;
    /* AngFreq = 45.563352525 / wave_len (Cos4Laser.jl:81) */
    L->omega = 45.563352525 / in->wave_len;
    L->period = 6.283185307179586 / L->omega; /* 2pi/omega */
    /* LaserF0 = sqrt(peak_int/(1+ellip^2)/3.50944521e16) (Cos4Laser.jl:85) */
    L->F0 = sqrt((in->peak_int / (1.0 + in->ellip * in->ellip)) / 3.50944521e16);
    L->A0 = L->F0 / L->omega;
    L->N = in->cyc_num;
    L->cep = in->cep;
    L->t_shift = in->t_shift;
    L->ellip = in->ellip;
    L->azi = in->azi;
    L->azi_zero = (in->azi == 0.0);
    dm_sincos(in->azi, &L->sphi, &L->cphi);
    if (L->kind == ETRAJ_LASER_GAUSSIAN) {
        /* SpreadDuration = spread_cyc_num * Period (GaussianLaser.jl:85) */
        L->sigma = in->cyc_num * L->period;
        L->inv_s2 = 1.0 / (L->sigma * L->sigma);
        L->inv_2s2 = 1.0 / (2.0 * (L->sigma * L->sigma));
    } else {
        L->w2n = L->omega / (2.0 * L->N);
        L->cN = (L->kind == ETRAJ_LASER_COS4) ? 2.0 / L->N : 1.0 / L->N;
        L->k = 200.0 / L->period;                    /* k = 200/Period */
        L->Npiw = (L->N * 3.141592653589793) / L->omega; /* N*pi/omega */
    }
}

void o_laser_prepare(const etraj_laser* in, o_laser* L) {
    memset(L, 0, sizeof *L);
    L->kind = in->kind;
    o_mono_prepare(&in->mono[0], &L->m[0]);
    if (in->kind == ETRAJ_LASER_BICHROMATIC) {
        o_mono_prepare(&in->mono[1], &L->m[1]);
        L->delay = in->delay;
        L->nmono = 2;
    } else {
        L->nmono = 1;
    }
}

/* tanh window factors 0.5+0.5*tanh(k*(t+N*pi/omega)) and
 * 0.5+0.5*tanh(-k*(t-N*pi/omega)), Cos4Laser.jl:93 */
static void o_window(const o_mono* L, double tt, double* w1, double* w2) {
    *w1 = 0.5 + 0.5 * dm_tanh(L->k * (tt + L->Npiw));
    *w2 = 0.5 + 0.5 * dm_tanh(-L->k * (tt - L->Npiw));
}

/* LaserFx / LaserFy of one monochromatic laser (Cos4Laser.jl:125-152,
 * Cos2Laser.jl:125-152, GaussianLaser.jl:133-160). */
void o_mono_F(const o_mono* L, double t, double* Fx, double* Fy) {
    double tt = t - L->t_shift;
    double sth, cth, pre, cx, cy;
    dm_sincos(L->omega * tt + L->cep, &sth, &cth);
    if (L->kind == ETRAJ_LASER_GAUSSIAN) {
        double g = dm_exp(-(tt * tt) * L->inv_2s2);
        double a = tt * L->inv_s2;
        pre = L->A0 * g;
        cx = a * cth + L->omega * sth;
        cy = a * sth - L->omega * cth;
    } else {
        double s, c, w1, w2;
        dm_sincos(tt * L->w2n, &s, &c);
        o_window(L, tt, &w1, &w2);
        double env = (L->kind == ETRAJ_LASER_COS4) ? (c * c) * c : c;
        pre = ((L->F0 * env) * w1) * w2;
        double b = L->cN * s;
        cx = c * sth + b * cth;
        cy = (-c) * cth + b * sth;
    }
    if (L->azi_zero) {
        *Fx = pre * cx;
        *Fy = (pre * cy) * L->ellip;
    } else {
        double cye = cy * L->ellip;
        *Fx = pre * (cx * L->cphi + cye * L->sphi);
        *Fy = pre * (cx * (-L->sphi) + cye * L->cphi);
    }
}

/* LaserAx / LaserAy (Cos4Laser.jl:97-124, GaussianLaser.jl:105-132). */
void o_mono_A(const o_mono* L, double t, double* Ax, double* Ay) {
    double tt = t - L->t_shift;
    double sth, cth, pre;
    dm_sincos(L->omega * tt + L->cep, &sth, &cth);
    if (L->kind == ETRAJ_LASER_GAUSSIAN) {
        pre = L->A0 * dm_exp(-(tt * tt) * L->inv_2s2);
    } else {
        double s, c, w1, w2;
        dm_sincos(tt * L->w2n, &s, &c);
        o_window(L, tt, &w1, &w2);
        double env = (L->kind == ETRAJ_LASER_COS4) ? (c * c) * (c * c) : c * c;
        pre = ((L->A0 * env) * w1) * w2;
    }
    if (L->azi_zero) {
        *Ax = pre * cth;
        *Ay = (pre * sth) * L->ellip;
    } else {
        double se = sth * L->ellip;
        *Ax = pre * (cth * L->cphi + se * L->sphi);
        *Ay = pre * (cth * (-L->sphi) + se * L->cphi);
    }
}

/* UnitEnvelope (Cos4Laser.jl:89-95, GaussianLaser.jl:97-103). */
double o_mono_env(const o_mono* L, double t) {
    double tt = t - L->t_shift;
    if (L->kind == ETRAJ_LASER_GAUSSIAN) return dm_exp(-(tt * tt) * L->inv_2s2);
    double s, c, w1, w2;
    dm_sincos(tt * L->w2n, &s, &c);
    o_window(L, tt, &w1, &w2);
    double env = (L->kind == ETRAJ_LASER_COS4) ? (c * c) * (c * c) : c * c;
    return (env * w1) * w2;
}

/* ---- forward-mode derivative of F (SPANESampler.jl:168-169 uses ForwardDiff) */
typedef struct { double v, d; } o_dual;
static o_dual dv(double v, double d) { o_dual r; r.v = v; r.d = d; return r; }
static o_dual dmul(o_dual a, o_dual b) { return dv(a.v * b.v, a.v * b.d + a.d * b.v); }
static o_dual dadd(o_dual a, o_dual b) { return dv(a.v + b.v, a.d + b.d); }
static o_dual dsub(o_dual a, o_dual b) { return dv(a.v - b.v, a.d - b.d); }
static o_dual dscale(o_dual a, double s) { return dv(a.v * s, a.d * s); }
static o_dual dneg(o_dual a) { return dv(-a.v, -a.d); }
static void dsincos(o_dual a, o_dual* s, o_dual* c) {
    double sv, cv;
    dm_sincos(a.v, &sv, &cv);
    *s = dv(sv, cv * a.d);
    *c = dv(cv, -sv * a.d);
}
static o_dual dtanh(o_dual a) {
    double t = dm_tanh(a.v);
    return dv(t, (1.0 - t * t) * a.d);
}
static o_dual dexp(o_dual a) {
    double e = dm_exp(a.v);
    return dv(e, e * a.d);
}

void o_mono_F_dual(const o_mono* L, double t, double* Fx, double* Fy, double* dFx, double* dFy) {
    o_dual tt = dv(t - L->t_shift, 1.0);
    o_dual th = dadd(dscale(tt, L->omega), dv(L->cep, 0.0));
    o_dual sth, cth, pre, cx, cy;
    dsincos(th, &sth, &cth);
    if (L->kind == ETRAJ_LASER_GAUSSIAN) {
        o_dual g = dexp(dscale(dneg(dmul(tt, tt)), L->inv_2s2));
        o_dual a = dscale(tt, L->inv_s2);
        pre = dscale(g, L->A0);
        cx = dadd(dmul(a, cth), dscale(sth, L->omega));
        cy = dsub(dmul(a, sth), dscale(cth, L->omega));
    } else {
        o_dual s, c;
        dsincos(dscale(tt, L->w2n), &s, &c);
        o_dual w1 = dadd(dv(0.5, 0.0), dscale(dtanh(dscale(dadd(tt, dv(L->Npiw, 0.0)), L->k)), 0.5));
        o_dual w2 = dadd(dv(0.5, 0.0), dscale(dtanh(dscale(dsub(tt, dv(L->Npiw, 0.0)), -L->k)), 0.5));
        o_dual env = (L->kind == ETRAJ_LASER_COS4) ? dmul(dmul(c, c), c) : c;
        pre = dmul(dmul(dscale(env, L->F0), w1), w2);
        o_dual b = dscale(s, L->cN);
        cx = dadd(dmul(c, sth), dmul(b, cth));
        cy = dadd(dmul(dneg(c), cth), dmul(b, sth));
    }
    o_dual fx, fy;
    if (L->azi_zero) {
        fx = dmul(pre, cx);
        fy = dscale(dmul(pre, cy), L->ellip);
    } else {
        o_dual cye = dscale(cy, L->ellip);
        fx = dmul(pre, dadd(dscale(cx, L->cphi), dscale(cye, L->sphi)));
        fy = dmul(pre, dadd(dscale(cx, -L->sphi), dscale(cye, L->cphi)));
    }
    *Fx = fx.v; *Fy = fy.v; *dFx = fx.d; *dFy = fy.d;
}

/* ---- complex time (SPASampler.jl evaluates A and F at t_r + i t_i) ----------- */
static void o_window_c(const o_mono* L, double tt_re, double* w1, double* w2) {
    /* the windows use real(t) (Cos4Laser.jl:93) */
    o_window(L, tt_re, w1, w2);
}

/* win: the window factors (w1, w2) at Re t when the caller holds them, else NULL */
static void o_mono_AF_complex_w(const o_mono* L, dm_cplx t, const double* win, dm_cplx* Ax, dm_cplx* Ay,
                                dm_cplx* Fx, dm_cplx* Fy) {
    dm_cplx tt = dm_c(t.re - L->t_shift, t.im);
    dm_cplx th = dm_caddr(dm_cscale(tt, L->omega), L->cep);
    dm_cplx sth = dm_csin(th), cth = dm_ccos(th);
    dm_cplx preA, preF, cx, cy;
    if (L->kind == ETRAJ_LASER_GAUSSIAN) {
        dm_cplx g = dm_cexp(dm_cscale(dm_cneg(dm_cmul(tt, tt)), L->inv_2s2));
        dm_cplx a = dm_cscale(tt, L->inv_s2);
        preA = dm_cscale(g, L->A0);
        preF = preA;
        cx = dm_cadd(dm_cmul(a, cth), dm_cscale(sth, L->omega));
        cy = dm_csub(dm_cmul(a, sth), dm_cscale(cth, L->omega));
    } else {
        double w1, w2;
        dm_cplx u = dm_cscale(tt, L->w2n);
        dm_cplx s = dm_csin(u), c = dm_ccos(u);
        if (win) {
            w1 = win[0];
            w2 = win[1];
        } else {
            o_window_c(L, tt.re, &w1, &w2);
        }
        dm_cplx c2 = dm_cmul(c, c);
        dm_cplx envA = (L->kind == ETRAJ_LASER_COS4) ? dm_cmul(c2, c2) : c2;
        dm_cplx envF = (L->kind == ETRAJ_LASER_COS4) ? dm_cmul(c2, c) : c;
        preA = dm_cscale(dm_cscale(dm_cscale(envA, L->A0), w1), w2);
        preF = dm_cscale(dm_cscale(dm_cscale(envF, L->F0), w1), w2);
        dm_cplx b = dm_cscale(s, L->cN);
        cx = dm_cadd(dm_cmul(c, sth), dm_cmul(b, cth));
        cy = dm_cadd(dm_cmul(dm_cneg(c), cth), dm_cmul(b, sth));
    }
    if (L->azi_zero) {
        *Ax = dm_cmul(preA, cth);
        *Ay = dm_cscale(dm_cmul(preA, sth), L->ellip);
        *Fx = dm_cmul(preF, cx);
        *Fy = dm_cscale(dm_cmul(preF, cy), L->ellip);
    } else {
        dm_cplx se = dm_cscale(sth, L->ellip);
        dm_cplx cye = dm_cscale(cy, L->ellip);
        *Ax = dm_cmul(preA, dm_cadd(dm_cscale(cth, L->cphi), dm_cscale(se, L->sphi)));
        *Ay = dm_cmul(preA, dm_cadd(dm_cscale(cth, -L->sphi), dm_cscale(se, L->cphi)));
        *Fx = dm_cmul(preF, dm_cadd(dm_cscale(cx, L->cphi), dm_cscale(cye, L->sphi)));
        *Fy = dm_cmul(preF, dm_cadd(dm_cscale(cx, -L->sphi), dm_cscale(cye, L->cphi)));
    }
}

void o_mono_AF_complex(const o_mono* L, dm_cplx t, dm_cplx* Ax, dm_cplx* Ay, dm_cplx* Fx,
                       dm_cplx* Fy) {
    o_mono_AF_complex_w(L, t, NULL, Ax, Ay, Fx, Fy);
}

/* ---- whole laser (bichromatic = sum, laser 2 delayed: BichromaticLaser.jl:73-85) */
void o_laser_F(const o_laser* L, double t, double* Fx, double* Fy) {
    o_mono_F(&L->m[0], t, Fx, Fy);
    if (L->nmono == 2) {
        double fx2, fy2;
        o_mono_F(&L->m[1], t - L->delay, &fx2, &fy2);
        *Fx = *Fx + fx2;
        *Fy = *Fy + fy2;
    }
}

void o_laser_F_dual(const o_laser* L, double t, double* Fx, double* Fy, double* dFx, double* dFy) {
    o_mono_F_dual(&L->m[0], t, Fx, Fy, dFx, dFy);
    if (L->nmono == 2) {
        double fx2, fy2, dfx2, dfy2;
        o_mono_F_dual(&L->m[1], t - L->delay, &fx2, &fy2, &dfx2, &dfy2);
        *Fx = *Fx + fx2; *Fy = *Fy + fy2; *dFx = *dFx + dfx2; *dFy = *dFy + dfy2;
    }
}

void o_laser_A(const o_laser* L, double t, double* Ax, double* Ay) {
    o_mono_A(&L->m[0], t, Ax, Ay);
    if (L->nmono == 2) {
        double ax2, ay2;
        o_mono_A(&L->m[1], t - L->delay, &ax2, &ay2);
        *Ax = *Ax + ax2;
        *Ay = *Ay + ay2;
    }
}

void o_laser_windows(const o_laser* L, double tre, double* win) {
    o_window(&L->m[0], tre - L->m[0].t_shift, &win[0], &win[1]);
    if (L->nmono == 2) o_window(&L->m[1], (tre - L->delay) - L->m[1].t_shift, &win[2], &win[3]);
}

void o_laser_AF_complex_w(const o_laser* L, dm_cplx t, const double* win, dm_cplx* Ax, dm_cplx* Ay,
                          dm_cplx* Fx, dm_cplx* Fy) {
    o_mono_AF_complex_w(&L->m[0], t, win, Ax, Ay, Fx, Fy);
    if (L->nmono == 2) {
        dm_cplx ax2, ay2, fx2, fy2;
        o_mono_AF_complex_w(&L->m[1], dm_c(t.re - L->delay, t.im), win ? win + 2 : NULL, &ax2, &ay2, &fx2,
                            &fy2);
        *Ax = dm_cadd(*Ax, ax2); *Ay = dm_cadd(*Ay, ay2);
        *Fx = dm_cadd(*Fx, fx2); *Fy = dm_cadd(*Fy, fy2);
    }
}

void o_laser_AF_complex(const o_laser* L, dm_cplx t, dm_cplx* Ax, dm_cplx* Ay, dm_cplx* Fx,
                        dm_cplx* Fy) {
    o_laser_AF_complex_w(L, t, NULL, Ax, Ay, Fx, Fy);
}

/* ---- targets ---------------------------------------------------------------- */

/* 0 disables the exp(-b r) skip everywhere (tests compare both settings) */
static int g_sae_skip = 1;
void oracle_set_sae_skip(int enable) { g_sae_skip = enable; }
int oracle_sae_skip_exact(const etraj_target* in) {
    double a[3] = {in->a1, in->a2, in->a3}, b[3] = {in->b1, in->b2, in->b3};
    return etraj_sae_skip_exact((double)in->Z, a, b, in->soft_core);
}

void o_target_prepare(const etraj_target* in, o_target* T) {
    memset(T, 0, sizeof *T);
    if (in->kind == ETRAJ_TARGET_MOLECULE) {
        /* GenericMolecule's trajectories: -Z (r^2+1)^(-1/2) with Z = charge + 1
         * and the phase's Ip = IonPotential(mol) (GenericMolecule.jl:438-445) --
         * the hydrogen-like equations with soft core 1.0 */
        T->kind = ETRAJ_TARGET_HYDROGEN_LIKE;
        T->Z = (double)in->Z;
        T->Ip = in->mol_Ip_traj;
        T->sc = 1.0;
        return;
    }
    T->kind = in->kind;
    T->Z = (double)in->Z;
    T->Ip = in->Ip;
    T->sc = in->soft_core;
    T->a1 = in->a1; T->b1 = in->b1;
    T->a2 = in->a2; T->b2 = in->b2;
    T->a3 = in->a3; T->b3 = in->b3;
    {
        double a[3] = {in->a1, in->a2, in->a3}, b[3] = {in->b1, in->b2, in->b3};
        T->skip_ok = g_sae_skip && etraj_sae_skip_exact((double)in->Z, a, b, in->soft_core);
    }
}

/* TargetPotential (HydrogenLikeAtom.jl:75, SAEAtom.jl:84-89) */
double o_target_V(const o_target* T, double x, double y, double z) {
    if (T->kind == ETRAJ_TARGET_HYDROGEN_LIKE) {
        double s = ((x * x + y * y) + z * z) + T->sc;
        return (-T->Z) * (1.0 / sqrt(s));
    }
    double r = sqrt((x * x + y * y) + z * z);
    double num = ((T->Z + T->a1 * o_sae_exp(T, T->b1, r)) + (T->a2 * r) * o_sae_exp(T, T->b2, r)) +
                 T->a3 * o_sae_exp(T, T->b3, r);
    return -num / sqrt(r * r + T->sc);
}

/* TargetForce (HydrogenLikeAtom.jl:76, SAEAtom.jl:91-96) */
void o_target_F(const o_target* T, double x, double y, double z, double* F) {
    if (T->kind == ETRAJ_TARGET_HYDROGEN_LIKE) {
        double s = ((x * x + y * y) + z * z) + T->sc;
        double f = (-T->Z) * (1.0 / (s * sqrt(s)));
        F[0] = f * x; F[1] = f * y; F[2] = f * z;
        return;
    }
    double r = sqrt((x * x + y * y) + z * z);
    double s = r * r + T->sc, rs = sqrt(s);
    double br = (T->Z + (T->a1 * (1.0 + T->b1 * r)) * o_sae_exp(T, T->b1, r)) +
                (T->a3 * (1.0 + T->b3 * r)) * o_sae_exp(T, T->b3, r);
    double coef = -((1.0 / (s * rs)) * br + ((T->a2 * T->b2) / rs) * o_sae_exp(T, T->b2, r));
    F[0] = x * coef; F[1] = y * coef; F[2] = z * coef;
}

/* Hartree formula C_kl = 2^(n*-1)/sqrt(n* Gamma(n*+l+1) Gamma(n*-l)),
 * falling back to l = 0 when n* <= l (SAEAtomBase_shared.jl:3-11). */
double oracle_hartree_asymp_coeff(int Z, double Ip, int l) {
    double n = (double)Z / sqrt(2.0 * Ip);
    if (n <= (double)l) l = 0;
    return pow(2.0, n - 1.0) / sqrt(n * tgamma(n + l + 1.0) * tgamma(n - l));
}

/* ODE right-hand sides: HydrogenLikeAtom.jl:78-159 and SAEAtom.jl:98-186. */
void o_rhs(const o_sys* S, double t, const double* u, double* du) {
    const o_target* T = &S->target;
    double Fx, Fy;
    o_laser_F(&S->laser, t, &Fx, &Fy);
    if (S->dim == 2) {
        double x = u[0], y = u[1], px = u[2], py = u[3];
        double tFx, tFy, Vphase = 0.0, s = 0.0, rs = 0.0;
        if (T->kind == ETRAJ_TARGET_HYDROGEN_LIKE) {
            s = (x * x + y * y) + T->sc;
            rs = sqrt(s);
            double f = (-T->Z) * (1.0 / (s * rs));
            tFx = f * x; tFy = f * y;
            Vphase = T->Z * (1.0 / rs);
        } else {
            double r = sqrt(x * x + y * y);
            s = r * r + T->sc;
            rs = sqrt(s);
            double e1 = o_sae_exp(T, T->b1, r), e2 = o_sae_exp(T, T->b2, r), e3 = o_sae_exp(T, T->b3, r);
            double br = (T->Z + (T->a1 * (1.0 + T->b1 * r)) * e1) + (T->a3 * (1.0 + T->b3 * r)) * e3;
            double coef = -((1.0 / (s * rs)) * br + ((T->a2 * T->b2) / rs) * e2);
            tFx = x * coef; tFy = y * coef;
            double num = ((T->Z + T->a1 * e1) + (T->a2 * r) * e2) + T->a3 * e3;
            /* SCTS 2D divides by r^2+sc, not its square root (SAEAtom.jl:136) */
            Vphase = (S->phase == ETRAJ_PHASE_SCTS) ? num / s : num / rs;
        }
        du[0] = px;
        du[1] = py;
        du[2] = tFx - Fx;
        du[3] = tFy - Fy;
        if (S->phase == ETRAJ_PHASE_QTMC) {
            du[4] = -((T->Ip + (px * px + py * py) / 2.0) - Vphase);
        } else if (S->phase == ETRAJ_PHASE_SCTS) {
            du[4] = -(((px * px + py * py) / 2.0 - Vphase) + (x * tFx + y * tFy));
        }
    } else {
        double x = u[0], y = u[1], z = u[2], px = u[3], py = u[4], pz = u[5];
        double tFx, tFy, tFz, Vphase = 0.0;
        if (T->kind == ETRAJ_TARGET_HYDROGEN_LIKE) {
            double s = ((x * x + y * y) + z * z) + T->sc;
            double rs = sqrt(s);
            double f = (-T->Z) * (1.0 / (s * rs));
            tFx = f * x; tFy = f * y; tFz = f * z;
            Vphase = T->Z * (1.0 / rs);
        } else {
            double r = sqrt((x * x + y * y) + z * z);
            double s = r * r + T->sc, rs = sqrt(s);
            double e1 = o_sae_exp(T, T->b1, r), e2 = o_sae_exp(T, T->b2, r), e3 = o_sae_exp(T, T->b3, r);
            double br = (T->Z + (T->a1 * (1.0 + T->b1 * r)) * e1) + (T->a3 * (1.0 + T->b3 * r)) * e3;
            double coef = -((1.0 / (s * rs)) * br + ((T->a2 * T->b2) / rs) * e2);
            tFx = x * coef; tFy = y * coef; tFz = z * coef;
            double num = ((T->Z + T->a1 * e1) + (T->a2 * r) * e2) + T->a3 * e3;
            Vphase = num / rs;
        }
        du[0] = px;
        du[1] = py;
        du[2] = pz;
        du[3] = tFx - Fx;
        du[4] = tFy - Fy;
        du[5] = tFz;
        double K = ((px * px + py * py) + pz * pz) / 2.0;
        if (S->phase == ETRAJ_PHASE_QTMC) {
            du[6] = -((T->Ip + K) - Vphase);
        } else if (S->phase == ETRAJ_PHASE_SCTS) {
            du[6] = -((K - Vphase) + ((x * tFx + y * tFy) + z * tFz));
        }
    }
}
