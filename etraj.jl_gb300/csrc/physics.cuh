// physics.cuh -- FP64 device evaluation of the lasers, targets and ODE
// right-hand sides.
//
// Reference: src/Lasers/Cos4Laser.jl:89-152, Cos2Laser.jl:89-152,
// GaussianLaser.jl:97-160, BichromaticLaser.jl:59-85;
// src/Targets/HydrogenLikeAtom.jl:75-159, SAEAtom.jl:84-186.
//
// Every expression keeps the reference's left-to-right association and uses
// detmath for transcendentals, so with --fmad=false the results are
// bit-identical to the CPU oracle.  Shared sub-expressions (the two sincos
// of the carrier and envelope, the window factors, exp(-b r)) are computed
// once per right-hand side and used for both field components, where the
// reference's closures recompute them.  Three operations are replaced by
// equal ones: omega*t/(2N) -> t*(omega/(2N)), s^(-3/2) -> 1/(s*sqrt(s)),
// s^(-1/2) -> 1/sqrt(s).
#pragma once

#include "engine.h"

namespace etraj {

__host__ __device__ __forceinline__ void window(const DMono& L, double tt, double& w1, double& w2) {
    w1 = 0.5 + 0.5 * dm_tanh(L.k * (tt + L.Npiw));
    w2 = 0.5 + 0.5 * dm_tanh(-L.k * (tt - L.Npiw));
}

// LaserFx / LaserFy of one monochromatic laser.
__host__ __device__ __forceinline__ void mono_F(const DMono& L, double t, double& Fx, double& Fy) {
    double tt = t - L.t_shift;
    double sth, cth, pre, cx, cy;
    dm_sincos(L.omega * tt + L.cep, &sth, &cth);
    if (L.kind == ETRAJ_LASER_GAUSSIAN) {
        double g = dm_exp(-(tt * tt) * L.inv_2s2);
        double a = tt * L.inv_s2;
        pre = L.A0 * g;
        cx = a * cth + L.omega * sth;
        cy = a * sth - L.omega * cth;
    } else {
        double s, c, w1, w2;
        dm_sincos(tt * L.w2n, &s, &c);
        window(L, tt, w1, w2);
        double env = (L.kind == ETRAJ_LASER_COS4) ? (c * c) * c : c;
        pre = ((L.F0 * env) * w1) * w2;
        double b = L.cN * s;
        cx = c * sth + b * cth;
        cy = (-c) * cth + b * sth;
    }
    if (L.azi_zero) {
        Fx = pre * cx;
        Fy = (pre * cy) * L.ellip;
    } else {
        double cye = cy * L.ellip;
        Fx = pre * (cx * L.cphi + cye * L.sphi);
        Fy = pre * (cx * (-L.sphi) + cye * L.cphi);
    }
}

__host__ __device__ __forceinline__ void laser_F(const DLaser& L, double t, double& Fx, double& Fy) {
    mono_F(L.m[0], t, Fx, Fy);
    if (L.nmono == 2) {
        double fx2, fy2;
        mono_F(L.m[1], t - L.delay, fx2, fy2);
        Fx = Fx + fx2;
        Fy = Fy + fy2;
    }
}

// UnitEnvelope (Cos4Laser.jl:89-95, GaussianLaser.jl:97-103)
__host__ __device__ __forceinline__ double mono_env(const DMono& L, double t) {
    double tt = t - L.t_shift;
    if (L.kind == ETRAJ_LASER_GAUSSIAN) return dm_exp(-(tt * tt) * L.inv_2s2);
    double s, c, w1, w2;
    dm_sincos(tt * L.w2n, &s, &c);
    window(L, tt, w1, w2);
    double env = (L.kind == ETRAJ_LASER_COS4) ? (c * c) * (c * c) : c * c;
    return (env * w1) * w2;
}

// LaserAx / LaserAy (Cos4Laser.jl:97-124, GaussianLaser.jl:105-132).
__host__ __device__ __forceinline__ void mono_A(const DMono& L, double t, double& Ax, double& Ay) {
    double tt = t - L.t_shift;
    double sth, cth, pre;
    dm_sincos(L.omega * tt + L.cep, &sth, &cth);
    if (L.kind == ETRAJ_LASER_GAUSSIAN) {
        pre = L.A0 * dm_exp(-(tt * tt) * L.inv_2s2);
    } else {
        double s, c, w1, w2;
        dm_sincos(tt * L.w2n, &s, &c);
        window(L, tt, w1, w2);
        double env = (L.kind == ETRAJ_LASER_COS4) ? (c * c) * (c * c) : c * c;
        pre = ((L.A0 * env) * w1) * w2;
    }
    if (L.azi_zero) {
        Ax = pre * cth;
        Ay = (pre * sth) * L.ellip;
    } else {
        double se = sth * L.ellip;
        Ax = pre * (cth * L.cphi + se * L.sphi);
        Ay = pre * (cth * (-L.sphi) + se * L.cphi);
    }
}

__host__ __device__ __forceinline__ void laser_A(const DLaser& L, double t, double& Ax, double& Ay) {
    mono_A(L.m[0], t, Ax, Ay);
    if (L.nmono == 2) {
        double ax2, ay2;
        mono_A(L.m[1], t - L.delay, ax2, ay2);
        Ax = Ax + ax2;
        Ay = Ay + ay2;
    }
}

// A and (optionally) F at complex time t_r + i t_i, as SPASampler.jl evaluates
// them; the tanh windows take real(t) (Cos4Laser.jl:93), so callers that hold
// Re t fixed pass them precomputed in `win` (w1, w2), or nullptr.
// doubles per laser in the `win` cache of the complex-time evaluations (laser_windows)
constexpr int kWinPerMono = 6;

__host__ __device__ __forceinline__ void mono_AF_complex(const DMono& L, dm_cplx t, dm_cplx& Ax, dm_cplx& Ay,
                                                         dm_cplx* Fx, dm_cplx* Fy, const double* win = nullptr) {
    const dm_cplx tt = dm_c(t.re - L.t_shift, t.im);
    const dm_cplx th = dm_caddr(dm_cscale(tt, L.omega), L.cep);
    dm_cplx sth, cth;
    if (win) dm_csincos_re(win[2], win[3], th.im, &sth, &cth);
    else dm_csincos(th, &sth, &cth);
    dm_cplx preA, preF, cx, cy;
    if (L.kind == ETRAJ_LASER_GAUSSIAN) {
        const dm_cplx g = dm_cexp(dm_cscale(dm_cneg(dm_cmul(tt, tt)), L.inv_2s2));
        const dm_cplx a = dm_cscale(tt, L.inv_s2);
        preA = dm_cscale(g, L.A0);
        preF = preA;
        cx = dm_cadd(dm_cmul(a, cth), dm_cscale(sth, L.omega));
        cy = dm_csub(dm_cmul(a, sth), dm_cscale(cth, L.omega));
    } else {
        double w1, w2;
        const dm_cplx u = dm_cscale(tt, L.w2n);
        dm_cplx s, c;
        if (win) dm_csincos_re(win[4], win[5], u.im, &s, &c);
        else dm_csincos(u, &s, &c);
        if (win) {
            w1 = win[0];
            w2 = win[1];
        } else {
            window(L, tt.re, w1, w2);
        }
        const dm_cplx c2 = dm_cmul(c, c);
        const dm_cplx envA = (L.kind == ETRAJ_LASER_COS4) ? dm_cmul(c2, c2) : c2;
        const dm_cplx envF = (L.kind == ETRAJ_LASER_COS4) ? dm_cmul(c2, c) : c;
        preA = dm_cscale(dm_cscale(dm_cscale(envA, L.A0), w1), w2);
        preF = dm_cscale(dm_cscale(dm_cscale(envF, L.F0), w1), w2);
        const dm_cplx b = dm_cscale(s, L.cN);
        cx = dm_cadd(dm_cmul(c, sth), dm_cmul(b, cth));
        cy = dm_cadd(dm_cmul(dm_cneg(c), cth), dm_cmul(b, sth));
    }
    if (L.azi_zero) {
        Ax = dm_cmul(preA, cth);
        Ay = dm_cscale(dm_cmul(preA, sth), L.ellip);
        if (Fx) {
            *Fx = dm_cmul(preF, cx);
            *Fy = dm_cscale(dm_cmul(preF, cy), L.ellip);
        }
    } else {
        const dm_cplx se = dm_cscale(sth, L.ellip);
        Ax = dm_cmul(preA, dm_cadd(dm_cscale(cth, L.cphi), dm_cscale(se, L.sphi)));
        Ay = dm_cmul(preA, dm_cadd(dm_cscale(cth, -L.sphi), dm_cscale(se, L.cphi)));
        if (Fx) {
            const dm_cplx cye = dm_cscale(cy, L.ellip);
            *Fx = dm_cmul(preF, dm_cadd(dm_cscale(cx, L.cphi), dm_cscale(cye, L.sphi)));
            *Fy = dm_cmul(preF, dm_cadd(dm_cscale(cx, -L.sphi), dm_cscale(cye, L.cphi)));
        }
    }
}

__host__ __device__ __forceinline__ void laser_AF_complex(const DLaser& L, dm_cplx t, dm_cplx& Ax, dm_cplx& Ay,
                                                          dm_cplx* Fx, dm_cplx* Fy, const double* win = nullptr) {
    mono_AF_complex(L.m[0], t, Ax, Ay, Fx, Fy, win);
    if (L.nmono == 2) {
        dm_cplx ax2, ay2, fx2, fy2;
        mono_AF_complex(L.m[1], dm_c(t.re - L.delay, t.im), ax2, ay2, Fx ? &fx2 : nullptr, Fx ? &fy2 : nullptr,
                        win ? win + kWinPerMono : nullptr);
        Ax = dm_cadd(Ax, ax2);
        Ay = dm_cadd(Ay, ay2);
        if (Fx) {
            *Fx = dm_cadd(*Fx, fx2);
            *Fy = dm_cadd(*Fy, fy2);
        }
    }
}

// What a complex-time evaluation at Re t = tre needs of each laser that depends
// on tre only, computed with the expressions mono_AF_complex uses, so a cache
// of them keyed by tre changes no bit: the window factors (w1, w2), then sin
// and cos of Re(theta) (carrier) and of Re(u) (envelope).
__host__ __device__ __forceinline__ void laser_windows(const DLaser& L, double tre, double* win) {
    for (int k = 0; k < L.nmono; ++k) {
        const DMono& M = L.m[k];
        double* w = win + kWinPerMono * k;
        const double ttre = ((k == 0) ? tre : tre - L.delay) - M.t_shift;
        window(M, ttre, w[0], w[1]);
        dm_sincos(ttre * M.omega + M.cep, &w[2], &w[3]);
        if (M.kind != ETRAJ_LASER_GAUSSIAN) dm_sincos(ttre * M.w2n, &w[4], &w[5]);
    }
}

__host__ __device__ __forceinline__ void laser_A_complex(const DLaser& L, dm_cplx t, const double* win, dm_cplx* Ax,
                                                         dm_cplx* Ay) {
    laser_AF_complex(L, t, *Ax, *Ay, nullptr, nullptr, win);
}

// ---- forward-mode derivative (SPANESampler.jl:168-169 differentiates F with ForwardDiff)
struct Dual {
    double v, d;
};
__host__ __device__ __forceinline__ Dual dv(double v, double d) { return Dual{v, d}; }
__host__ __device__ __forceinline__ Dual dmul(Dual a, Dual b) { return dv(a.v * b.v, a.v * b.d + a.d * b.v); }
__host__ __device__ __forceinline__ Dual dadd(Dual a, Dual b) { return dv(a.v + b.v, a.d + b.d); }
__host__ __device__ __forceinline__ Dual dsub(Dual a, Dual b) { return dv(a.v - b.v, a.d - b.d); }
__host__ __device__ __forceinline__ Dual dscale(Dual a, double s) { return dv(a.v * s, a.d * s); }
__host__ __device__ __forceinline__ Dual dneg(Dual a) { return dv(-a.v, -a.d); }
__host__ __device__ __forceinline__ void dsincos(Dual a, Dual& s, Dual& c) {
    double sv, cv;
    dm_sincos(a.v, &sv, &cv);
    s = dv(sv, cv * a.d);
    c = dv(cv, -sv * a.d);
}
__host__ __device__ __forceinline__ Dual dtanh(Dual a) {
    double t = dm_tanh(a.v);
    return dv(t, (1.0 - t * t) * a.d);
}
__host__ __device__ __forceinline__ Dual dexp(Dual a) {
    double e = dm_exp(a.v);
    return dv(e, e * a.d);
}

__host__ __device__ __forceinline__ void mono_F_dual(const DMono& L, double t, double& Fx, double& Fy,
                                                     double& dFx, double& dFy) {
    Dual tt = dv(t - L.t_shift, 1.0);
    Dual th = dadd(dscale(tt, L.omega), dv(L.cep, 0.0));
    Dual sth, cth, pre, cx, cy;
    dsincos(th, sth, cth);
    if (L.kind == ETRAJ_LASER_GAUSSIAN) {
        Dual g = dexp(dscale(dneg(dmul(tt, tt)), L.inv_2s2));
        Dual a = dscale(tt, L.inv_s2);
        pre = dscale(g, L.A0);
        cx = dadd(dmul(a, cth), dscale(sth, L.omega));
        cy = dsub(dmul(a, sth), dscale(cth, L.omega));
    } else {
        Dual s, c;
        dsincos(dscale(tt, L.w2n), s, c);
        Dual w1 = dadd(dv(0.5, 0.0), dscale(dtanh(dscale(dadd(tt, dv(L.Npiw, 0.0)), L.k)), 0.5));
        Dual w2 = dadd(dv(0.5, 0.0), dscale(dtanh(dscale(dsub(tt, dv(L.Npiw, 0.0)), -L.k)), 0.5));
        Dual env = (L.kind == ETRAJ_LASER_COS4) ? dmul(dmul(c, c), c) : c;
        pre = dmul(dmul(dscale(env, L.F0), w1), w2);
        Dual b = dscale(s, L.cN);
        cx = dadd(dmul(c, sth), dmul(b, cth));
        cy = dadd(dmul(dneg(c), cth), dmul(b, sth));
    }
    Dual fx, fy;
    if (L.azi_zero) {
        fx = dmul(pre, cx);
        fy = dscale(dmul(pre, cy), L.ellip);
    } else {
        Dual cye = dscale(cy, L.ellip);
        fx = dmul(pre, dadd(dscale(cx, L.cphi), dscale(cye, L.sphi)));
        fy = dmul(pre, dadd(dscale(cx, -L.sphi), dscale(cye, L.cphi)));
    }
    Fx = fx.v;
    Fy = fy.v;
    dFx = fx.d;
    dFy = fy.d;
}

__host__ __device__ __forceinline__ void laser_F_dual(const DLaser& L, double t, double& Fx, double& Fy,
                                                      double& dFx, double& dFy) {
    mono_F_dual(L.m[0], t, Fx, Fy, dFx, dFy);
    if (L.nmono == 2) {
        double fx2, fy2, dfx2, dfy2;
        mono_F_dual(L.m[1], t - L.delay, fx2, fy2, dfx2, dfy2);
        Fx = Fx + fx2;
        Fy = Fy + fy2;
        dFx = dFx + dfx2;
        dFy = dFy + dfy2;
    }
}

// ---- targets -----------------------------------------------------------------------
// exp(-b r) of the SAE potential.  For targets that pass etraj_sae_skip_exact
// (sae_skip.h, checked on the host), every term this factor enters when
// b r > 60 is too small to change the sum it is added to, so returning 0
// leaves every result bit-identical and saves the evaluation at large r,
// where trajectories spend most of their steps.
__host__ __device__ __forceinline__ double sae_exp(const DTarget& T, double b, double r) {
    if (T.skip_ok && b * r > 60.0) return 0.0;
    return dm_exp(-b * r);
}

// TargetPotential (HydrogenLikeAtom.jl:75, SAEAtom.jl:84-89)
__host__ __device__ __forceinline__ double target_V(const DTarget& T, double x, double y, double z) {
    if (T.kind == ETRAJ_TARGET_HYDROGEN_LIKE) {
        double s = ((x * x + y * y) + z * z) + T.sc;
        return (-T.Z) * (1.0 / sqrt(s));
    }
    double r = sqrt((x * x + y * y) + z * z);
    double num = ((T.Z + T.a1 * sae_exp(T, T.b1, r)) + (T.a2 * r) * sae_exp(T, T.b2, r)) +
                 T.a3 * sae_exp(T, T.b3, r);
    return -num / sqrt(r * r + T.sc);
}

// ODE right-hand side (TrajectoryFunction, HydrogenLikeAtom.jl:78-159, SAEAtom.jl:98-186).
// DIM: 2 or 3; PHASE: ETRAJ_PHASE_*; TGT: ETRAJ_TARGET_*.
template <int DIM, int PHASE, int TGT>
__host__ __device__ __forceinline__ void rhs(const DJob& J, double t, const double* u, double* du) {
    const DTarget& T = J.target;
    double Fx, Fy;
    laser_F(J.laser, t, Fx, Fy);
    if (DIM == 2) {
        double x = u[0], y = u[1], px = u[2], py = u[3];
        double tFx, tFy, Vphase;
        if (TGT == ETRAJ_TARGET_HYDROGEN_LIKE) {
            double s = (x * x + y * y) + T.sc;
            double rs = sqrt(s);
            double f = (-T.Z) * (1.0 / (s * rs));
            tFx = f * x;
            tFy = f * y;
            Vphase = T.Z * (1.0 / rs);
        } else {
            double r = sqrt(x * x + y * y);
            double s = r * r + T.sc, rs = sqrt(s);
            double e1 = sae_exp(T, T.b1, r), e2 = sae_exp(T, T.b2, r), e3 = sae_exp(T, T.b3, r);
            double br = (T.Z + (T.a1 * (1.0 + T.b1 * r)) * e1) + (T.a3 * (1.0 + T.b3 * r)) * e3;
            double coef = -((1.0 / (s * rs)) * br + ((T.a2 * T.b2) / rs) * e2);
            tFx = x * coef;
            tFy = y * coef;
            if (PHASE != ETRAJ_PHASE_CTMC) {
                double num = ((T.Z + T.a1 * e1) + (T.a2 * r) * e2) + T.a3 * e3;
                // the 2D SCTS reference divides by r^2+sc, not its square root (SAEAtom.jl:136)
                Vphase = (PHASE == ETRAJ_PHASE_SCTS) ? num / s : num / rs;
            } else {
                Vphase = 0.0;
            }
        }
        du[0] = px;
        du[1] = py;
        du[2] = tFx - Fx;
        du[3] = tFy - Fy;
        if (PHASE == ETRAJ_PHASE_QTMC) du[4] = -((T.Ip + (px * px + py * py) / 2.0) - Vphase);
        if (PHASE == ETRAJ_PHASE_SCTS) du[4] = -(((px * px + py * py) / 2.0 - Vphase) + (x * tFx + y * tFy));
    } else {
        double x = u[0], y = u[1], z = u[2], px = u[3], py = u[4], pz = u[5];
        double tFx, tFy, tFz, Vphase;
        if (TGT == ETRAJ_TARGET_HYDROGEN_LIKE) {
            double s = ((x * x + y * y) + z * z) + T.sc;
            double rs = sqrt(s);
            double f = (-T.Z) * (1.0 / (s * rs));
            tFx = f * x;
            tFy = f * y;
            tFz = f * z;
            Vphase = T.Z * (1.0 / rs);
        } else {
            double r = sqrt((x * x + y * y) + z * z);
            double s = r * r + T.sc, rs = sqrt(s);
            double e1 = sae_exp(T, T.b1, r), e2 = sae_exp(T, T.b2, r), e3 = sae_exp(T, T.b3, r);
            double br = (T.Z + (T.a1 * (1.0 + T.b1 * r)) * e1) + (T.a3 * (1.0 + T.b3 * r)) * e3;
            double coef = -((1.0 / (s * rs)) * br + ((T.a2 * T.b2) / rs) * e2);
            tFx = x * coef;
            tFy = y * coef;
            tFz = z * coef;
            Vphase = (PHASE != ETRAJ_PHASE_CTMC) ? (((T.Z + T.a1 * e1) + (T.a2 * r) * e2) + T.a3 * e3) / rs : 0.0;
        }
        du[0] = px;
        du[1] = py;
        du[2] = pz;
        du[3] = tFx - Fx;
        du[4] = tFy - Fy;
        du[5] = tFz;
        if (PHASE != ETRAJ_PHASE_CTMC) {
            double K = ((px * px + py * py) + pz * pz) / 2.0;
            if (PHASE == ETRAJ_PHASE_QTMC) du[6] = -((T.Ip + K) - Vphase);
            else du[6] = -((K - Vphase) + ((x * tFx + y * tFy) + z * tFz));
        }
    }
}

}  // namespace etraj
