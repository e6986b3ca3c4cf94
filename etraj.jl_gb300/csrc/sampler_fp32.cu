// sampler_fp32.cu -- FP32 candidate kernel of the ADK and SPANE samplers for
// the bulk path.
//
// Same algorithm, loop order and Philox draws as k_sample in sampler.cu
// (ADKSampler.jl:318-391, SPANESampler.jl:320-398), evaluated in FP32 on the
// CUDA cores instead of in FP64: on GB300 the FP64 pipe made sampling the
// largest cost of a bulk job.  Per-batch constants (field, derivative,
// Wigner-D row, Coulomb-corrected constant) still come from the FP64
// k_batch_prepare, which also stores their FP32 copies.  Grid values are
// rounded once to FP32 and Monte-Carlo draws keep the leading 24 bits of the
// FP64 sampler's uniforms, so the bulk path samples the same electrons as the
// FP64 path to ~1e-7 relative; a candidate whose rate lies within that
// distance of the cutoff may be kept by one path and dropped by the other.  Output layout is the
// FP64 kernel's (candidate-indexed SoA of doubles and a keep flag).

#include "physics.cuh"

namespace etraj {
namespace {

struct cf {
    float re, im;
};
__device__ __forceinline__ cf cmk(float r, float i) { return cf{r, i}; }
__device__ __forceinline__ cf cadd(cf a, cf b) { return cmk(a.re + b.re, a.im + b.im); }
__device__ __forceinline__ cf cmul(cf a, cf b) {
    return cmk(fmaf(a.re, b.re, -a.im * b.im), fmaf(a.re, b.im, a.im * b.re));
}
__device__ __forceinline__ cf cscale(cf a, float s) { return cmk(a.re * s, a.im * s); }
__device__ __forceinline__ cf cconj(cf a) { return cmk(a.re, -a.im); }
__device__ __forceinline__ cf cpowi(cf z, int n) {
    cf r = cmk(1.0f, 0.0f);
    for (int i = 0; i < n; ++i) r = cmul(r, z);
    return r;
}

// Coefficients (-1)^k / (2^(2k+m) (k+m)! k! (l-m-2k)!) of the solid harmonic's
// k-sum for l <= 6, m = -l..l, k = max(0, -m) + j (j < 4), rounded once at
// compile time: every factor and product is an integer below 2^24, so the only
// rounding is the one correctly rounded division a kernel would do.
struct SphCoef {
    float c[MOL_MAX_L + 1][2 * MOL_MAX_L + 1][4];
};
constexpr float sph_fact(int n) { return n <= 1 ? 1.0f : (float)n * sph_fact(n - 1); }
constexpr SphCoef sph_coef_table() {
    SphCoef t{};
    for (int l = 0; l <= MOL_MAX_L; ++l)
        for (int m = -l; m <= l; ++m) {
            const int kmin = (m < 0) ? -m : 0, kmax = (l - m) / 2;
            for (int k = kmin; k <= kmax && k - kmin < 4; ++k) {
                float p2 = 1.0f;
                for (int i = 0; i < 2 * k + m; ++i) p2 *= 2.0f;
                t.c[l][m + l][k - kmin] =
                    ((k & 1) ? -1.0f : 1.0f) / (p2 * sph_fact(k + m) * sph_fact(k) * sph_fact(l - m - 2 * k));
            }
        }
    return t;
}
__constant__ SphCoef kSph = sph_coef_table();

__device__ __forceinline__ void philox4x32(uint32_t c[4], uint64_t seed) {
    uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0 = __umulhi(0xD2511F53u, c[0]), lo0 = 0xD2511F53u * c[0];
        uint32_t hi1 = __umulhi(0xCD9E8D57u, c[2]), lo1 = 0xCD9E8D57u * c[2];
        uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0;
        c[1] = lo1;
        c[2] = n2;
        c[3] = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}

// the FP64 sampler's 53-bit uniform in [0, 1) from two draws (sampler.cu), for the
// pre-pass that must see the FP64 sampler's own momenta
__device__ __forceinline__ double u53(uint32_t a, uint32_t b) {
    return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) * (1.0 / 9007199254740992.0);
}

// k-sum of the solid harmonic (shared_methods.jl:21) at complex (x, y, z).
__device__ cf sph_sum(int l, int m, cf x, cf y, cf z) {
    const cf xp = cmk(x.re - y.im, x.im + y.re);
    const cf xm = cmk(x.re + y.im, x.im - y.re);
    const int kmin = (m < 0) ? -m : 0, kmax = (l - m) / 2;
    cf acc = cmk(0.0f, 0.0f);
    for (int k = kmin; k <= kmax; ++k) {
        const float coef = kSph.c[l][m + l][k - kmin];
        cf tt = cscale(cpowi(xp, k + m), coef);
        tt = cmul(tt, cpowi(xm, k));
        tt = cmul(tt, cpowi(z, l - m - 2 * k));
        acc = cadd(acc, tt);
    }
    return acc;
}

// ---- FP32 SPA candidate (SPASampler.jl:150-431) -------------------------------------
// Every complex time the SPA candidate evaluates, except the four solves of its
// finite-difference Jacobian, has Re t = t_r: the saddle-point iterates
// t_r + i t_i and the quadrature paths from t_r to t_r + i t_i.  The laser's
// phases at t_r (up to ~1e3 rad) are therefore reduced once in FP64, and
// A(t_r + i tau), F(t_r + i tau) follow in FP32 from cosh/sinh of the
// imaginary parts.  The solve and the quadratures are the algorithms of spa.h
// (NLsolve's trust-region dogleg with a central-difference derivative, which
// a cold solve replaces by the secant of its last two iterates after an
// accepted step; QuadGK's adaptive Gauss-Kronrod (7,15) with an interval heap)
// at FP32's tolerances: ftol 1e-5 on the saddle-point residual, derivative
// step cbrt(eps(Float32)), quadrature rtol sqrt(eps(Float32)), which is the
// tolerance QuadGK picks for Float32 integrands.
enum { Q_IM_AX = 0, Q_IM_AY = 1, Q_ACTION = 2, Q_IM_AXY = 3 };
constexpr int kSegs32 = 48;  // interval budget of one quadrature

__device__ void spa32_base(const DLaser& L, double tr, SpaBase32& S) {
    S.n = L.nmono;
    for (int k = 0; k < L.nmono; ++k) {
        const DMono& M = L.m[k];
        SpaMono32& m = S.m[k];
        const double tt = ((k == 0) ? tr : tr - L.delay) - M.t_shift;
        double th = M.omega * tt + M.cep;
        th = th - 6.283185307179586 * rint(th * 0.15915494309189535);
        double sn, cs;
        sincos(th, &sn, &cs);
        m.cth = (float)cs;
        m.sth = (float)sn;
        m.om = (float)M.omega;
        m.kind = M.kind;
        m.azi0 = M.azi_zero;
        m.ellip = (float)M.ellip;
        m.cphi = (float)M.cphi;
        m.sphi = (float)M.sphi;
        if (M.kind == ETRAJ_LASER_GAUSSIAN) {
            m.gt = (float)tt;
            m.gi = (float)M.inv_2s2;
            m.inv_s2 = (float)M.inv_s2;
            const double g0 = exp(-(tt * tt) * M.inv_2s2) * M.A0;
            m.preA = (float)g0;
            m.preF = (float)g0;
            m.cu = m.su = m.w2n = m.cN = 0.0f;
        } else {
            double su, cu;
            sincos(M.w2n * tt, &su, &cu);
            m.cu = (float)cu;
            m.su = (float)su;
            m.w2n = (float)M.w2n;
            m.cN = (float)M.cN;
            double w1, w2;
            window(M, tt, w1, w2);
            m.preA = (float)((M.A0 * w1) * w2);
            m.preF = (float)((M.F0 * w1) * w2);
            m.gt = m.gi = m.inv_s2 = 0.0f;
        }
    }
}

// cosh x and sinh x from one exponential e = e^x and its reciprocal.  Below
// |x| = 0.5, where e - 1/e would lose bits to cancellation, sinh is its Taylor
// series x (1 + x^2/3! + x^4/5! + x^6/7!), whose truncation (x^8/9! relative)
// is under 1.1e-8 there.
__device__ __forceinline__ void csh32(float x, float& ch, float& sh) {
    const float e = expf(x), ei = __frcp_rn(e);
    ch = 0.5f * (e + ei);
    const float x2 = x * x;
    const float ps = x * fmaf(x2, fmaf(x2, fmaf(x2, 1.0f / 5040.0f, 1.0f / 120.0f), 1.0f / 6.0f), 1.0f);
    sh = (fabsf(x) < 0.5f) ? ps : 0.5f * (e - ei);
}

// A (and F when fx != nullptr) at t_r + i tau
__device__ void spa32_AF(const SpaBase32& S, float tau, cf& ax, cf& ay, cf* fx, cf* fy) {
    ax = ay = cmk(0.0f, 0.0f);
    if (fx) *fx = *fy = cmk(0.0f, 0.0f);
    for (int k = 0; k < S.n; ++k) {
        const SpaMono32& m = S.m[k];
        float ch, sh;
        csh32(m.om * tau, ch, sh);
        const cf sth = cmk(m.sth * ch, m.cth * sh), cth = cmk(m.cth * ch, -(m.sth * sh));
        cf preA, preF, cx, cy;
        if (m.kind == ETRAJ_LASER_GAUSSIAN) {
            float sa, ca;
            sincosf(-2.0f * m.gt * tau * m.gi, &sa, &ca);
            const float e = expf(tau * tau * m.gi);
            preA = cmk(m.preA * e * ca, m.preA * e * sa);
            preF = preA;
            const cf a = cmk(m.gt * m.inv_s2, tau * m.inv_s2);
            cx = cadd(cmul(a, cth), cscale(sth, m.om));
            cy = cadd(cmul(a, sth), cscale(cth, -m.om));
        } else {
            float chu, shu;
            csh32(m.w2n * tau, chu, shu);
            const cf c = cmk(m.cu * chu, -(m.su * shu)), sv = cmk(m.su * chu, m.cu * shu);
            const cf c2 = cmul(c, c);
            const bool c4 = (m.kind == ETRAJ_LASER_COS4);
            preA = cscale(c4 ? cmul(c2, c2) : c2, m.preA);
            preF = cscale(c4 ? cmul(c2, c) : c, m.preF);
            const cf b = cscale(sv, m.cN);
            cx = cadd(cmul(c, sth), cmul(b, cth));
            cy = cadd(cmul(cmk(-c.re, -c.im), cth), cmul(b, sth));
        }
        if (m.azi0) {
            ax = cadd(ax, cmul(preA, cth));
            ay = cadd(ay, cscale(cmul(preA, sth), m.ellip));
            if (fx) {
                *fx = cadd(*fx, cmul(preF, cx));
                *fy = cadd(*fy, cscale(cmul(preF, cy), m.ellip));
            }
        } else {
            const cf se = cscale(sth, m.ellip);
            ax = cadd(ax, cmul(preA, cadd(cscale(cth, m.cphi), cscale(se, m.sphi))));
            ay = cadd(ay, cmul(preA, cadd(cscale(cth, -m.sphi), cscale(se, m.cphi))));
            if (fx) {
                const cf cye = cscale(cy, m.ellip);
                *fx = cadd(*fx, cmul(preF, cadd(cscale(cx, m.cphi), cscale(cye, m.sphi))));
                *fy = cadd(*fy, cmul(preF, cadd(cscale(cx, -m.sphi), cscale(cye, m.cphi))));
            }
        }
    }
}

// px_, py_ of SPASampler.jl:230-231
__device__ __forceinline__ void spa32_pxy(float kd, cf Ax, cf Ay, float& px, float& py) {
    const float den = sqrtf(fmaf(Ax.im, Ax.im, Ay.im * Ay.im));
    px = (kd * Ay.im) / den - Ax.re;
    py = (-kd * Ax.im) / den - Ay.re;
}

// saddle_point_equation (SPASampler.jl:233-239) at t_r + i x
__device__ float spa32_spe(const SpaBase32& S, float x, float kd, float kz, float Ip) {
    cf Ax, Ay;
    spa32_AF(S, x, Ax, Ay, nullptr, nullptr);
    float px, py;
    spa32_pxy(kd, Ax, Ay, px, py);
    const float ur = px + Ax.re, ui = Ax.im, vr = py + Ay.re, vi = Ay.im;
    const float u2 = fmaf(ur, ur, -ui * ui), v2 = fmaf(vr, vr, -vi * vi);
    return fmaf(0.5f, fmaf(kz, kz, u2 + v2), Ip);
}

__device__ float spa32_dspe(const SpaBase32& S, float x, float kd, float kz, float Ip) {
    const float e = 4.9215667e-3f * fmaxf(fabsf(x), 1.0f);  // cbrt(eps(Float32))
    return (spa32_spe(S, x + e, kd, kz, Ip) - spa32_spe(S, x - e, kd, kz, Ip)) / (2.0f * e);
}

// t_i of the saddle point (0: not converged or t_i <= 0); spa_solve_ti in FP32.
// warm: x0 is the root of a neighbouring equation (the Jacobian's solves at
// t_r +- 0.01 and k_d +- 0.01 start from the candidate's own t_i instead of
// the asinh guess).  Its residual is often already inside ftol, and a root
// accepted there would carry up to ftol / |J| of error into the Jacobian's
// finite differences, so a warm start is accepted only at |r| <= ftol / 10
// (ten times the FP32 rounding of the residual); otherwise one Newton step
// takes it to rounding level.
__device__ __noinline__ float spa32_solve(const SpaBase32& S, float kd, float kz, float Ip, float x0,
                                          bool warm = false) {
    const float ftol = 1e-5f, eta = 1e-4f;
    float x = x0;
    float r = spa32_spe(S, x, kd, kz, Ip);
    if (!isfinite(r) || !isfinite(x)) return 0.0f;
    bool converged = (fabsf(r) <= (warm ? 0.1f * ftol : ftol));
    if (converged) return (x > 0.0f) ? x : 0.0f;
    // the Jacobian is only needed for a further step
    float J = spa32_dspe(S, x, kd, kz, Ip);
    float d = fabsf(J);
    if (d == 0.0f) d = 1.0f;
    float delta = fabsf(d * x);
    if (delta == 0.0f) delta = 1.0f;
    for (int it = 0; it < 200 && !converged; ++it) {
        if (J == 0.0f) return 0.0f;
        float p;
        const float pn = -(r / J);
        if (fabsf(d * pn) <= delta) {
            p = pn;
        } else {
            const float g = (J * r) / (d * d);
            const float wg = fabsf(d * g), Jg = J * g;
            const float pc = ((-(wg * wg)) / (Jg * Jg)) * g;
            if (fabsf(d * pc) >= delta) {
                p = g * (-delta / wg);
            } else {
                const float df = pn - pc;
                const float b = 2.0f * ((d * pc) * (d * df));
                const float a = (d * df) * (d * df);
                const float wc = fabsf(d * pc);
                const float tau = (-b + sqrtf(b * b - (4.0f * a) * (wc * wc - delta * delta))) / (2.0f * a);
                p = pc + tau * df;
            }
        }
        const float xold = x;
        x = x + p;
        const float fn = spa32_spe(S, x, kd, kz, Ip);
        const float rp = J * p + r;
        const float rho = (r * r - fn * fn) / (r * r - rp * rp);
        if (rho > eta) {
            const float rold = r;
            r = fn;
            converged = (fabsf(x - xold) <= 0.0f) || (fabsf(r) <= ftol);
            if (converged) break;
            // a cold solve takes the secant through its last two iterates as the
            // derivative, which costs no evaluation; a step too short for FP32 to
            // resolve the difference, and the warm solves' one step, take the
            // central difference
            const float dx = x - xold;
            if (!warm && fabsf(dx) > 1e-3f * fmaxf(fabsf(x), 1.0f)) J = (fn - rold) / dx;
            else J = spa32_dspe(S, x, kd, kz, Ip);
            d = fmaxf(0.1f * d, fabsf(J));
        } else {
            x = x - p;
        }
        if (rho < 0.1f) delta = 0.5f * delta;
        else if (rho >= 0.9f) delta = 2.0f * fabsf(d * p);
        else if (rho >= 0.5f) delta = fmaxf(delta, 2.0f * fabsf(d * p));
        if (isnan(x) || isnan(fn)) break;
    }
    return (converged && x > 0.0f) ? x : 0.0f;
}

// integrands over tau at t = t_r + i tau: Im A_x, Im A_y (kind 3: both), or the
// action's ((p_x+A_x)^2 + (p_y+A_y)^2 + k_z^2)/2 + I_p (kind 2)
struct SpaQ32 {
    const SpaBase32* S;
    float px, py, kz, Ip;
};
__device__ __forceinline__ cf spa32_f(int kind, const SpaQ32& Q, float tau, float& v1) {
    cf Ax, Ay;
    spa32_AF(*Q.S, tau, Ax, Ay, nullptr, nullptr);
    if (kind != Q_ACTION) {
        v1 = Ay.im;
        return cmk(kind == Q_IM_AY ? Ay.im : Ax.im, 0.0f);
    }
    v1 = 0.0f;
    const cf u = cmk(Q.px + Ax.re, Ax.im), v = cmk(Q.py + Ay.re, Ay.im);
    const cf sq = cadd(cmul(u, u), cmul(v, v));
    return cmk(fmaf(0.5f, sq.re + Q.kz * Q.kz, Q.Ip), 0.5f * sq.im);
}

struct Seg32 {
    float a, b, E;
    cf I;
};

__device__ __forceinline__ float cabsf(cf z) { return (z.im == 0.0f) ? fabsf(z.re) : hypotf(z.re, z.im); }

// Gauss-Kronrod (7, 15) on [a, b]; g1: the second integrand of kind 3
__device__ __noinline__ Seg32 spa32_rule(int kind, const SpaQ32& Q, float a, float b, Seg32* g1) {
    const float x[8] = {-0.991455371120812639f, -0.949107912342758525f, -0.864864423359769073f,
                        -0.741531185599394440f, -0.586087235467691130f, -0.405845151377397167f,
                        -0.207784955007898468f, 0.0f};
    const float w[8] = {0.022935322010529225f, 0.063092092629978553f, 0.104790010322250184f,
                        0.140653259715525919f, 0.169004726639267903f, 0.190350578064785410f,
                        0.204432940075298892f, 0.209482141084727828f};
    const float gw[4] = {0.129484966168869693f, 0.279705391489276668f, 0.381830050505118945f,
                         0.417959183673469388f};
    const float h = 0.5f * (b - a), c = 0.5f * (a + b);
    cf Ig = cmk(0.0f, 0.0f), Ik = Ig;
    float Jg = 0.0f, Jk = 0.0f;
    for (int i = 0; i < 8; ++i) {
        float u1 = 0.0f, u2 = 0.0f;
        cf f;
        float fh;
        if (i < 7) {
            const cf p = spa32_f(kind, Q, fmaf(h, x[i], c), u1);
            const cf q = spa32_f(kind, Q, fmaf(-h, x[i], c), u2);
            f = cadd(p, q);
            fh = u1 + u2;
        } else {
            f = spa32_f(kind, Q, c, u1);
            fh = u1;
        }
        Ik = cadd(Ik, cscale(f, w[i]));
        Jk = fmaf(fh, w[i], Jk);
        if (i & 1) {  // the Gauss nodes are the odd Kronrod nodes, the centre (i = 7) included
            Ig = cadd(Ig, cscale(f, gw[i >> 1]));
            Jg = fmaf(fh, gw[i >> 1], Jg);
        }
    }
    Seg32 sg;
    sg.a = a;
    sg.b = b;
    sg.I = cscale(Ik, h);
    sg.E = cabsf(cadd(sg.I, cscale(Ig, -h)));
    if (g1) {
        g1->a = a;
        g1->b = b;
        g1->I = cmk(Jk * h, 0.0f);
        g1->E = fabsf(Jk * h - Jg * h);
    }
    return sg;
}

__device__ __noinline__ cf spa32_quad_from(int kind, const SpaQ32& Q, Seg32 first, bool& ok) {
    const float rtol = 3.4526698e-4f;  // sqrt(eps(Float32))
    Seg32 hp[kSegs32];
    hp[0] = first;
    cf I = first.I;
    float E = first.E;
    ok = isfinite(E);
    if (!ok || E <= rtol * cabsf(I)) return I;
    int n = 1;
    while (rtol * cabsf(I) < E) {
        if (n + 1 > kSegs32) {
            ok = false;
            break;
        }
        const Seg32 sg = hp[0];
        hp[0] = hp[n - 1];
        --n;
        {  // sift down
            int i = 0;
            const Seg32 xx = hp[0];
            for (;;) {
                const int l = 2 * i + 1;
                if (l >= n) break;
                const int rr = l + 1;
                const int j = (rr >= n || hp[rr].E < hp[l].E) ? l : rr;
                if (!(xx.E < hp[j].E)) break;
                hp[i] = hp[j];
                i = j;
            }
            if (n > 0) hp[i] = xx;
        }
        const float mid = 0.5f * (sg.a + sg.b);
        const Seg32 s1 = spa32_rule(kind, Q, sg.a, mid, nullptr);
        const Seg32 s2 = spa32_rule(kind, Q, mid, sg.b, nullptr);
        if (!isfinite(s1.E) || !isfinite(s2.E)) {
            ok = false;
            return I;
        }
        I = cadd(cadd(cadd(I, cscale(sg.I, -1.0f)), s1.I), s2.I);
        E = ((E - sg.E) + s1.E) + s2.E;
        for (int t = 0; t < 2; ++t) {  // sift up
            int i = n;
            const Seg32 xx = t ? s2 : s1;
            while (i > 0) {
                const int pp = (i - 1) / 2;
                if (!(hp[pp].E < xx.E)) break;
                hp[i] = hp[pp];
                i = pp;
            }
            hp[i] = xx;
            ++n;
        }
    }
    I = hp[0].I;
    for (int i = 1; i < n; ++i) I = cadd(I, hp[i].I);
    return I;
}

// jac(kd, kz) of SPASampler.jl:280-292 from four saddle-point solves
__device__ __noinline__ float spa32_jac(const SpaBase32& S0, const SpaBase32& Sp, const SpaBase32& Sm, float kd,
                                        float kz, float Ip, float ti) {
    const float dtr = 0.01f, dkd = 0.01f;
    const float ti_tp = spa32_solve(Sp, kd, kz, Ip, ti, true);
    const float ti_tm = spa32_solve(Sm, kd, kz, Ip, ti, true);
    const float ti_kp = spa32_solve(S0, kd + dkd, kz, Ip, ti, true);
    const float ti_km = spa32_solve(S0, kd - dkd, kz, Ip, ti, true);
    cf ax, ay;
    float pxa, pya, pxb, pyb;
    spa32_AF(Sp, ti_tp, ax, ay, nullptr, nullptr);
    spa32_pxy(kd, ax, ay, pxa, pya);
    spa32_AF(Sm, ti_tm, ax, ay, nullptr, nullptr);
    spa32_pxy(kd, ax, ay, pxb, pyb);
    const float dpxdtr = pxa - pxb, dpydtr = pya - pyb;
    spa32_AF(S0, ti_kp, ax, ay, nullptr, nullptr);
    spa32_pxy(kd + dkd, ax, ay, pxa, pya);
    spa32_AF(S0, ti_km, ax, ay, nullptr, nullptr);
    spa32_pxy(kd - dkd, ax, ay, pxb, pyb);
    const float dpxdkd = pxa - pxb, dpydkd = pya - pyb;
    return fabsf(dpxdtr * dpydkd - dpxdkd * dpydtr) / ((4.0f * dtr) * dkd);
}

// sum over m' of C D^l_{m' m} Y_{l m'} of conj(k) in the field frame (ADKSampler.jl:243-265)
__device__ cf num32(const DJob& J, const FBatch& B, cf kx, cf ky, float kz0) {
    const cf nkx = cmk(kz0, 0.0f);
    const cf nky = cadd(cscale(cconj(kx), B.ny0), cscale(cconj(ky), B.ny1));
    const cf nkz = cadd(cscale(cconj(kx), B.nz0), cscale(cconj(ky), B.nz1));
    cf num = cmk(0.0f, 0.0f);
    for (int mp = -J.l; mp <= J.l; ++mp) {
        const int ii = mp + J.l;
        const cf Y = cmul(cmk(J.fPlm[2 * ii], J.fPlm[2 * ii + 1]), sph_sum(J.l, mp, nkx, nky, nkz));
        num = cadd(num, cmul(cmk(B.CD[2 * ii], B.CD[2 * ii + 1]), Y));
    }
    return num;
}

// batches[b].spa of the sampled batches: one thread per (time sample, t_r + {0, 0.01, -0.01})
__global__ void k_spa32_bases(const __grid_constant__ DJob J, int64_t b0, int64_t nb, DBatch* __restrict__ batches) {
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < 3 * nb;
         q += (int64_t)gridDim.x * blockDim.x) {
        DBatch& DB = batches[b0 + q / 3];
        const int w = (int)(q % 3);
        const double tr = DB.tr;
        spa32_base(J.laser, (w == 0) ? tr : (w == 1) ? tr + 0.01 : tr - 0.01, DB.spa[w]);
    }
}

// The rate part of one SPA candidate in FP32 (the steps of SPASampler.jl:320-347):
// the saddle point t_i, the momenta p, the action's quadrature, the prefactor and
// the Jacobian, as the log-rate lr = log |amp|^2 and the phase arg.  Returns false
// when the solve or the action's quadrature fails (the candidate is dropped).
struct Spa32Rate {
    float ti, px, py, lr, arg;
};
__device__ __forceinline__ bool spa32_rate(const DJob& J, const DBatch& DB, const SpaBase32& S, float kd0, float kz0,
                                           Spa32Rate& R) {
    const FBatch& B = DB.f;
    const float Ip = J.fc.Ip, w = J.fc.spa_omega, e_half = J.fc.e_half;
    const float wF = w / B.F;
    const float guess = asinhf(wF * sqrtf(fmaf(kd0, kd0, kz0 * kz0) + 2.0f * Ip)) / w;
    const float ti = spa32_solve(S, kd0, kz0, Ip, guess);
    if (ti == 0.0f) return false;
    cf Ax, Ay, Fx, Fy;
    spa32_AF(S, ti, Ax, Ay, &Fx, &Fy);
    float px, py;
    spa32_pxy(kd0, Ax, Ay, px, py);
    SpaQ32 Q{&S, px, py, kz0, Ip};
    bool oks;
    // S_tun = -int_{t_s}^{t_r} f dt = i int_0^{t_i} f(t_r + i tau) dtau
    const cf Qs = spa32_quad_from(Q_ACTION, Q, spa32_rule(Q_ACTION, Q, 0.0f, ti, nullptr), oks);
    if (!oks) return false;
    // amplitude sqrt(dkdt) exp(i S_tun) [pre] [sqrt(jac)] = sqrt(dkdt) exp(-Q) [...],
    // kept as its log-rate lr = log |amp|^2 - log dkdt and phase arg
    float lr = -2.0f * Qs.re, arg = -Qs.im;
    if (J.prefix & (ETRAJ_PREFIX_PRE | ETRAJ_PREFIX_PRECC)) {
        const cf kx = cmk(px + Ax.re, Ax.im), ky = cmk(py + Ay.re, Ay.im);
        const cf num = num32(J, B, kx, ky, kz0);
        const float cpre = (J.prefix & ETRAJ_PREFIX_PRE) ? J.fc.c : B.c_cc;
        const cf kF = cadd(cmul(kx, Fx), cmul(ky, Fy));
        // (k_ts . F(t_s))^((n*+1)/2) as |z|^p cis(p arg z)
        const float mag = powf(hypotf(kF.re, kF.im), e_half);
        float sn, cs;
        sincosf(e_half * atan2f(kF.im, kF.re), &sn, &cs);
        const cf den = cmk(mag * cs, mag * sn);
        const float dd = fmaf(den.re, den.re, den.im * den.im);
        const cf nd = cscale(cmul(num, cconj(den)), cpre / dd);
        lr += 2.0f * logf(hypotf(nd.re, nd.im));
        arg += atan2f(nd.im, nd.re);
    }
    if (J.prefix & ETRAJ_PREFIX_JAC) lr += logf(spa32_jac(S, DB.spa[1], DB.spa[2], kd0, kz0, Ip, ti));
    R.ti = ti;
    R.px = px;
    R.py = py;
    R.lr = lr + J.fc.log_dkdt;
    R.arg = arg;
    return true;
}

__global__ void __launch_bounds__(128)
k_sample_spa32(const __grid_constant__ DJob J, int64_t b0, int64_t nb, const double* __restrict__ kdv,
               const double* __restrict__ kzv, const DBatch* __restrict__ batches, InitSoA soa,
               uint8_t* __restrict__ flag) {
    const int64_t total = nb * J.n_cand;
    const float Ip = J.fc.Ip, kd_max = J.fc.kd_max, kz_max = J.fc.kz_max;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < total;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t bl = q / J.n_cand, i = q - bl * J.n_cand, b = b0 + bl;
        const DBatch& DB = batches[b];
        const FBatch& B = DB.f;
        float kd0, kz0;
        if (!J.mc) {
            kd0 = (float)kdv[i / J.n_kz];
            kz0 = (float)kzv[i % J.n_kz];
        } else {
            uint32_t c[4] = {(uint32_t)i, (uint32_t)((uint64_t)i >> 32), (uint32_t)b, 0x4B445A00u};
            philox4x32(c, J.seed);
            const float ua = (float)(c[0] >> 8) * 5.9604644775390625e-8f;
            const float ub = (float)(c[2] >> 8) * 5.9604644775390625e-8f;
            kd0 = ((ua - 0.5f) * 2.0f) * kd_max;
            if (J.dim == 3) {
                kz0 = ((ub - 0.5f) * 2.0f) * kz_max;
                if (J.fc.kd_zero) kd0 = 0.0f;
                else if (J.fc.kz_zero) kz0 = 0.0f;
            } else {
                kz0 = 0.0f;
            }
        }
        uint8_t keep = 0;
        double x0 = 0.0, y0 = 0.0, kx0 = 0.0, ky0 = 0.0, rate = 0.0, ph = 0.0;
        // the batch is skipped when F(t_r) <= 1e-3 (SPASampler.jl:167-169)
        if (!(fabsf(kd0) < 1e-4f) && B.spa_on) {
            const SpaBase32 S = DB.spa[0];
            Spa32Rate R;
            if (spa32_rate(J, DB, S, kd0, kz0, R)) {
                // FP32's exp down to its normal range, FP64 below
                rate = (R.lr >= -87.0f) ? (double)expf(R.lr) : exp((double)R.lr);
                keep = (!(rate != rate) && !(rate < J.cutoff)) ? 1 : 0;
                if (keep) {
                    // the exit position's two quadratures, for the candidates the rate
                    // keeps only (a failed quadrature drops the candidate)
                    SpaQ32 Q{&S, R.px, R.py, kz0, Ip};
                    Seg32 sy;
                    const Seg32 sx = spa32_rule(Q_IM_AXY, Q, 0.0f, R.ti, &sy);
                    bool okx, oky;
                    x0 = spa32_quad_from(Q_IM_AX, Q, sx, okx).re;
                    y0 = spa32_quad_from(Q_IM_AY, Q, sy, oky).re;
                    keep = (okx && oky) ? 1 : 0;
                    cf A0x, A0y;
                    spa32_AF(S, 0.0f, A0x, A0y, nullptr, nullptr);
                    kx0 = (double)(R.px + A0x.re);
                    ky0 = (double)(R.py + A0y.re);
                }
                if (keep && J.phase != ETRAJ_PHASE_CTMC) {
                    // arg reduced to [-pi, pi]: k 2 pi subtracted with 2 pi split in two
                    // floats (Cody and Waite's reduction)
                    const float k = rintf(R.arg * 0.159154943f);
                    const float r = fmaf(-k, -1.7484556e-7f, fmaf(-k, 6.28318548f, R.arg));
                    ph = (double)r;
                }
            }
        }
        const int64_t g = b * J.n_cand + i;
        flag[g] = keep;
        if (keep) {
            soa.x[g] = x0;
            soa.y[g] = y0;
            soa.kx[g] = kx0;
            soa.ky[g] = ky0;
            soa.kz[g] = kz0;
            soa.rate[g] = rate;
            if (soa.phase) soa.phase[g] = ph;
            soa.batch[g] = (int32_t)b;
        }
    }
}

// Molecules (mol.h layouts; the per-time-sample tables are FP64): the MO-ADK
// numerator sum over (l, m, m') of C_lm D^l_{m' m} Y_{l m'}, in FP32.
__device__ cf mol_num32(const DJob& J, const float* __restrict__ cd, cf nkx, cf nky, cf nkz) {
    const mol_terms& T = J.mol.T;
    cf acc = cmk(0.0f, 0.0f), Y[2 * MOL_MAX_L + 1];
    int e = 0, ycur = -1;
    for (int k = 0; k < T.n; ++k) {
        const int l = T.l[k];
        if (l != ycur) {
            for (int mp = -l; mp <= l; ++mp) {
                const int pi = l * l + l + mp;
                Y[mp + l] = cmul(cmk(J.mol.Pf[2 * pi], J.mol.Pf[2 * pi + 1]), sph_sum(l, mp, nkx, nky, nkz));
            }
            ycur = l;
        }
        for (int mp = -l; mp <= l; ++mp, ++e) acc = cadd(acc, cmul(cmk(cd[2 * e], cd[2 * e + 1]), Y[mp + l]));
    }
    return acc;
}

// The WFAT rate (WFATSampler.jl:169) in FP32: channels n_xi fastest; each
// channel's W as (A E) K, so the time-sample factor A (up to F^-7) never
// meets K before the exponential has scaled it.
__device__ float wfat_rate32(const DJob& J, const float* __restrict__ tb, float F, float kd, float kz) {
    const int nxi = J.mol.nxi, mmax = J.mol.mmax;
    const float* g2 = tb;
    const float* A = tb + (nxi + 1) * (2 * mmax + 1);
    const float k2 = fmaf(kd, kd, kz * kz);
    const float X = J.fc.kap2 + k2;
    const float E = expf((-2.0f * (X * sqrtf(X))) / (3.0f * F));
    float K[MOL_MAX_L + 1];
    K[0] = 1.0f;
    for (int a = 1; a <= mmax; ++a) K[a] = K[a - 1] * k2;
    float sum = 0.0f;
    for (int m = -mmax; m <= mmax; ++m) {
        const int am = m < 0 ? -m : m;
        for (int n = 0; n <= nxi; ++n)
            sum = fmaf(g2[n + (m + mmax) * (nxi + 1)], (A[n + am * (nxi + 1)] * E) * K[am], sum);
    }
    return sum * J.fc.dkdt;
}

// Stores float f as the double of equal value without the FP64 pipe (which on
// GB300 also executes conversions, at 1/64 of the FP32 rate): IEEE 754 gives a
// normal float and its double the same sign and significand, with the exponent
// rebiased from 127 to 1023, and zeros, infinities and NaNs (payload kept) map
// field by field.  The two 32-bit halves are stored directly.  Subnormal
// floats take the conversion instruction.
__device__ __forceinline__ void store_f2d(double* dst, float f) {
    const uint32_t u = __float_as_uint(f);
    const uint32_t e = (u >> 23) & 0xFFu, m = u & 0x7FFFFFu;
    if (e == 0u && m != 0u) {
        *dst = (double)f;
        return;
    }
    const uint32_t ed = (e == 0u) ? 0u : (e == 0xFFu) ? 0x7FFu : e + 896u;
    *reinterpret_cast<uint2*>(dst) = make_uint2(m << 29, (u & 0x80000000u) | (ed << 20) | (m >> 3));
}

// x 2^-24 for an integer 0 <= x < 2^24, exactly and without a conversion
// instruction: 1 + (x >> 1) 2^-23 is built from its bits, 1 subtracted
// (exact), and the low bit of x added back (the sum has at most 24
// significant bits, so it is exact too).
__device__ __forceinline__ float u24_unit(uint32_t x) {
    const float a = __uint_as_float(0x3F800000u | (x >> 1)) - 1.0f;
    return a + (float)(x & 1u) * 5.9604644775390625e-8f;
}

// One candidate per thread.  A thread's (time sample, candidate) pair advances
// by the grid's stride without dividing, so the 64-bit divisions that split a
// flat candidate index run once per thread instead of once per candidate.
__global__ void __launch_bounds__(256)
k_sample32(const __grid_constant__ DJob J, int64_t b0, int64_t nb, const double* __restrict__ kdv,
           const double* __restrict__ kzv, const DBatch* __restrict__ batches, InitSoA soa,
           uint8_t* __restrict__ flag) {
    const float Ip = J.fc.Ip, kap2 = J.fc.kap2, sqdkdt = J.fc.sqdkdt;
    const float inv_dkdt = J.fc.inv_dkdt, cutoff = J.fc.cutoff, e_pre = J.fc.e_pre;
    const float c_pre = J.fc.c, kd_max = J.fc.kd_max, kz_max = J.fc.kz_max;
    const float spane_lim = J.mc ? 0.04f : 0.111111111f;  // 1/25, 1/9
    const bool spane = (J.method == ETRAJ_SAMPLER_SPANE);
    const int64_t n = J.n_cand, stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t step_b = stride / n, step_i = stride - step_b * n;
    const int64_t q0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t bl = q0 / n, i = q0 - bl * n;
    for (; bl < nb; bl += step_b, i += step_i, bl += (i >= n) ? 1 : 0, i -= (i >= n) ? n : 0) {
        const int64_t b = b0 + bl;
        const FBatch& B = batches[b].f;
        float kd0, kz0;
        if (!J.mc) {
            const int64_t ik = i / J.n_kz;
            kd0 = (float)kdv[ik];
            kz0 = (float)kzv[i - ik * J.n_kz];
        } else {
            uint32_t c[4] = {(uint32_t)i, (uint32_t)((uint64_t)i >> 32), (uint32_t)b, 0x4B445A00u};
            philox4x32(c, J.seed);
            // the leading 24 bits of the FP64 sampler's 53-bit uniforms
            const float ua = u24_unit(c[0] >> 8);
            const float ub = u24_unit(c[2] >> 8);
            kd0 = ((ua - 0.5f) * 2.0f) * kd_max;
            if (J.dim == 3) {
                kz0 = ((ub - 0.5f) * 2.0f) * kz_max;
                if (J.fc.kd_zero) kd0 = 0.0f;
                else if (J.fc.kz_zero) kz0 = 0.0f;
            } else {
                kz0 = 0.0f;
            }
        }
        uint8_t keep = 0;
        float x0 = 0.0f, y0 = 0.0f, kx0 = 0.0f, ky0 = 0.0f, rate = 0.0f, ph = 0.0f;
        if (J.method == ETRAJ_SAMPLER_WFAT) {
            // WFATSampler.jl:173-240: ADK's exit point, the WFAT rate, CTMC rows
            if (!(fmaf(kd0, kd0, kz0 * kz0) < 1e-8f)) {
                const float F = B.F;
                kx0 = kd0 * (-B.sphi);
                ky0 = kd0 * B.cphi;
                const float r0 = fmaf(0.5f, fmaf(kd0, kd0, kz0 * kz0), Ip) / F;
                x0 = r0 * B.cphi;
                y0 = r0 * B.sphi;
                rate = wfat_rate32(J, J.mol.tabf + b * (int64_t)J.mol.stride, F, kd0, kz0);
                keep = (!(rate != rate) && !(rate < cutoff)) ? 1 : 0;
            }
        } else if (!(fabsf(kd0) < 1e-4f)) {
            const float F = B.F;
            kx0 = kd0 * (-B.sphi);
            ky0 = kd0 * B.cphi;
            const float k2 = fmaf(kd0, kd0, kz0 * kz0);
            const float Xk = k2 + 2.0f * Ip;
            float ti, X2, Fexp;
            bool skip = false;
            if (!spane) {
                const float r0 = fmaf(0.5f, k2, Ip) / F;
                x0 = r0 * B.cphi;
                y0 = r0 * B.sphi;
                ti = sqrtf(kap2 + k2) / F;
                X2 = Xk * (F * F);
                Fexp = F;
            } else {
                const float F2eff = fmaf(F, F, -fmaf(kx0, B.dFx, ky0 * B.dFy));
                const float r0 = ((0.5f * F) * Xk) / F2eff;
                x0 = r0 * B.cphi;
                y0 = r0 * B.sphi;
                skip = (F2eff <= (F * F) * spane_lim);
                ti = sqrtf((kap2 + k2) / F2eff);
                X2 = Xk * F2eff;
                Fexp = sqrtf(F2eff);
            }
            if (!skip) {
                const float E = expf(-(Xk * sqrtf(Xk)) / (3.0f * Fexp));
                const float r1 = sqdkdt * E;
                cf amp;
                if (J.prefix & (ETRAJ_PREFIX_PRE | ETRAJ_PREFIX_PRECC)) {
                    cf kx, ky;
                    if (!spane) {
                        kx = cmk(kx0, -(ti * B.Fx));
                        ky = cmk(ky0, -(ti * B.Fy));
                    } else {
                        const float h = 0.5f * ti * ti;
                        kx = cmk(fmaf(h, B.dFx, kx0), -(ti * B.Fx));
                        ky = cmk(fmaf(h, B.dFy, ky0), -(ti * B.Fy));
                    }
                    // rotate conj(k_ts) into the field frame (ADKSampler.jl:247-249)
                    const cf nkx = cmk(kz0, 0.0f);
                    const cf nky = cadd(cscale(cconj(kx), B.ny0), cscale(cconj(ky), B.ny1));
                    const cf nkz = cadd(cscale(cconj(kx), B.nz0), cscale(cconj(ky), B.nz1));
                    cf num = cmk(0.0f, 0.0f);
                    if (J.mol.on) {
                        num = mol_num32(J, J.mol.tabf + b * (int64_t)J.mol.stride, nkx, nky, nkz);
                    } else {
                        for (int mp = -J.l; mp <= J.l; ++mp) {
                            const int ii = mp + J.l;
                            const cf Y = cmul(cmk(J.fPlm[2 * ii], J.fPlm[2 * ii + 1]), sph_sum(J.l, mp, nkx, nky, nkz));
                            num = cadd(num, cmul(cmk(B.CD[2 * ii], B.CD[2 * ii + 1]), Y));
                        }
                    }
                    const float cpre = (J.prefix & ETRAJ_PREFIX_PRE) ? c_pre : B.c_cc;
                    const float den = (e_pre == 0.5f) ? sqrtf(X2) : exp2f(e_pre * log2f(X2));
                    amp = cscale(num, (cpre / den) * r1);
                } else {
                    amp = cmk(r1, 0.0f);
                }
                if (J.prefix & ETRAJ_PREFIX_JAC) {
                    const float jac = spane ? fabsf(fmaf(sqrtf(k2) / (F * F), B.W, F)) : F;
                    amp = cscale(amp, sqrtf(jac));
                }
                rate = fmaf(amp.re, amp.re, amp.im * amp.im);
                const float crit = spane ? rate * inv_dkdt : rate;
                keep = (!(rate != rate) && !(crit < cutoff)) ? 1 : 0;
                if (keep && J.phase != ETRAJ_PHASE_CTMC) ph = atan2f(amp.im, amp.re);
            }
        }
        const int64_t g = b * J.n_cand + i;
        flag[g] = keep;
        if (keep) {
            store_f2d(soa.x + g, x0);
            store_f2d(soa.y + g, y0);
            store_f2d(soa.kx + g, kx0);
            store_f2d(soa.ky + g, ky0);
            store_f2d(soa.kz + g, kz0);
            store_f2d(soa.rate + g, rate);
            if (soa.phase) store_f2d(soa.phase + g, ph);
            soa.batch[g] = (int32_t)b;
        }
    }
}

// The FP64 SPA sampler's pre-pass (atoms): each candidate's rate in FP32 at the FP64
// sampler's own (kd, kz) draws, and flag[g] = 0 where its FP32 solve succeeds and
// that rate is below exp(log_margin) x the cutoff, else 1.  The FP64 path uses a
// margin of 1/100: a candidate so far below is one the FP64 rate cannot keep
// (FP32's rate is within 3e-3 of FP64's where both solve, and the FP32 sampler
// keeps the FP64 sampler's electrons but for a few in 1e6, at the cutoff), so its
// survivors and their values do not change.  Double-float jobs use 0.8: a
// candidate dropped then that FP64 would keep weighs about the cutoff (1e-16 of a
// rate on the headline jobs).  k_sample_spa then computes every candidate marked
// 1 in FP64 as before.
__global__ void __launch_bounds__(128)
k_spa_prefilter(const __grid_constant__ DJob J, int64_t b0, int64_t nb, const double* __restrict__ kdv,
                const double* __restrict__ kzv, const DBatch* __restrict__ batches, float log_margin,
                uint8_t* __restrict__ flag) {
    const int64_t total = nb * J.n_cand;
    const float lr_drop = logf(J.fc.cutoff) + log_margin;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < total;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t bl = q / J.n_cand, i = q - bl * J.n_cand, b = b0 + bl;
        const DBatch& DB = batches[b];
        double kd0, kz0;
        if (!J.mc) {
            kd0 = kdv[i / J.n_kz];
            kz0 = kzv[i % J.n_kz];
        } else {
            uint32_t c[4] = {(uint32_t)i, (uint32_t)((uint64_t)i >> 32), (uint32_t)b, 0x4B445A00u};
            philox4x32(c, J.seed);
            const double ua = u53(c[0], c[1]), ub = u53(c[2], c[3]);
            kd0 = ((ua - 0.5) * 2.0) * J.mc_kd_max;
            if (J.dim == 3) {
                kz0 = ((ub - 0.5) * 2.0) * J.mc_kz_max;
                if (J.mc_kd_max == 0.0) kd0 = 0.0;
                else if (J.mc_kz_max == 0.0) kz0 = 0.0;
            } else {
                kz0 = 0.0;
            }
        }
        uint8_t maybe = 1;
        if (!(fabs(kd0) < 1e-4) && DB.f.spa_on) {
            Spa32Rate R;
            if (spa32_rate(J, DB, DB.spa[0], (float)kd0, (float)kz0, R) && R.lr < lr_drop) maybe = 0;
        }
        flag[b * J.n_cand + i] = maybe;
    }
}

}  // namespace

int launch_spa_prefilter(const DJob& J, int64_t b0, int64_t nb, const double* kd, const double* kz,
                         DBatch* batches, float log_margin, uint8_t* flag, int sm_count, cudaStream_t s) {
    const int64_t bb = (3 * nb + 127) / 128;
    k_spa32_bases<<<(int)(bb > 0 ? bb : 1), 128, 0, s>>>(J, b0, nb, batches);
    const int threads = 128;
    const int64_t want = (nb * J.n_cand + threads - 1) / threads;
    const int64_t cap = (int64_t)sm_count * 64;
    const int blocks = (int)(want < cap ? (want > 0 ? want : 1) : cap);
    k_spa_prefilter<<<blocks, threads, 0, s>>>(J, b0, nb, kd, kz, batches, log_margin, flag);
    return 2;
}

int launch_sample32_range(const DJob& J, int64_t b0, int64_t nb, const double* kd, const double* kz,
                          DBatch* batches, InitSoA soa, uint8_t* flag, int sm_count,
                          cudaStream_t s) {
    if (J.method == ETRAJ_SAMPLER_SPA) {
        const int64_t bb = (3 * nb + 127) / 128;
        k_spa32_bases<<<(int)(bb > 0 ? bb : 1), 128, 0, s>>>(J, b0, nb, batches);
        const int threads = 128;
        const int64_t want = (nb * J.n_cand + threads - 1) / threads;
        const int64_t cap = (int64_t)sm_count * 64;
        const int blocks = (int)(want < cap ? (want > 0 ? want : 1) : cap);
        k_sample_spa32<<<blocks, threads, 0, s>>>(J, b0, nb, kd, kz, batches, soa, flag);
        return 2;
    }
    const int threads = 256;
    const int64_t want = (nb * J.n_cand + threads - 1) / threads;
    const int64_t cap = (int64_t)sm_count * 32;
    const int blocks = (int)(want < cap ? (want > 0 ? want : 1) : cap);
    k_sample32<<<blocks, threads, 0, s>>>(J, b0, nb, kd, kz, batches, soa, flag);
    return 1;
}

}  // namespace etraj
