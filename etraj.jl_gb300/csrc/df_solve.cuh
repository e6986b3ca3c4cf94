// df_solve.cuh -- one electron's double-float Tsit5 solve, cut into the
// operations the kernel of integrate_df.cu interleaves across a warp: load,
// the two evaluations of the starting step, and per step attempt a prologue,
// six stage inputs (each followed by one right-hand side) and an epilogue.
//
// It restates solve() and initdt() of integrate_fp64.cu (OrdinaryDiffEq's
// Tsit5 with its default controller) with every quantity a double-float pair
// (dfloat.h): stage values and sums, the RMS error estimate, the controller's
// powers EEst^(7/50) and qold^(2/25) (double-float log2 and exp2) and Hairer's
// starting step.
//
// Differences from the accepted state.  In an electron's first steps the
// error estimate is a weighted sum of the stage derivatives that cancels to
// ~1e-10 of them, so a rounding of 2^-48 in a stage value moves it by ~1e-5
// and the step sizes off the FP64 path's (by 2^-53, FP64 moves it ~30x less).
// So every stage is formed relative to the accepted state (x0, p0, K0): its
// increments dX = X_l - x0 and dP = P_l - p0 are double-float sums of small
// terms, the laser's change is an exact table difference F(t_l) - F(t0), and
// the target's change is written algebraically in dX, e.g. with
// b = sqrt(s_l/s_0): s_l^(-1/2) - s_0^(-1/2) = -s_0^(-1/2) (b - 1)/b and
// b - 1 = (ds/s_0)/(1 + b), so each difference carries a 2^-48 error of itself,
// not of the value.  Tsit5's weights satisfy sum bt = 0 and sum bt c = 0, so the
// error estimate is a sum over the differences dK_l = K_l - K_0 alone, and the
// stage sums are (row sum) K_0 + sum a dK.  Only the accepted state itself is
// rounded to double-float once per step (harmless: it is where the next step
// starts, not an error the controller sees).  The target's terms at each newly
// accepted state are evaluated directly (stage 6 always is), not carried as sums
// of differences: those keep absolute errors of the largest r^2 they saw, which
// relative to r^2 grow without bound as an electron falls to the core.
//
// Differences are needed only where the error estimate cancels that far: in an
// electron's first attempts, while the last accepted error estimate is below 1e-6
// (the "start-up" attempts, ~5% of all on the argon jobs of the tests).  There
// the stages are differences; from the first attempt that follows an estimate
// above 1e-6 on, each stage's target terms are evaluated directly at x0 + dX, and
// the sixth stage's direct terms are the new accepted state's.  On the jobs of the
// tests, ending the start-up at 1e-3, 1e-4, 1e-6 or 1e-8, or taking the later
// attempts with small estimates (where qmax holds the controller back) directly,
// changed no status and no step count; differences in the first attempt alone
// were not enough (the median asymptotic momentum moved by 1.6e-9).
//
// The code compiles for the device and, unchanged, for the host (the CPU tests
// run it against the FP64 oracle).
#pragma once

#include "dfloat.h"
#include "physics.cuh"
#include "tsit5.h"

namespace etraj {
namespace dfs {

#if defined(__CUDACC__)
#define DFS_HD __host__ __device__ __forceinline__
#else
#define DFS_HD inline
#endif

// double-float constant of an FP64 value (folded at compile time)
DFS_HD constexpr df dfc(double v) { return df{(float)v, (float)(v - (double)(float)v)}; }
DFS_HD df d2(float2 v) { return df{v.x, v.y}; }

// The Tsit5 coefficients as double-float pairs: a __constant__ copy for the device
// and a static one for the host build (stage indices are compile-time constants
// where they are read, so the device reads them as constant-bank operands).
#define DFS_ROW(f, i) {f(i, 0), f(i, 1), f(i, 2), f(i, 3), f(i, 4), f(i, 5), f(i, 6)}
#define DFS_A(i, l) dfc(tsit5::kA[i][l])
#define DFS_AA(i, l) dfc(tsit5::aa(i, l))
#define DFS_V7(f) {dfc(f(0)), dfc(f(1)), dfc(f(2)), dfc(f(3)), dfc(f(4)), dfc(f(5)), dfc(f(6))}
#define DFS_C(i) tsit5::kC[i]
#define DFS_BT(i) tsit5::kBT[i]
#define DFS_TABLES(Q)                                                                                   \
    Q df A[7][7] = {DFS_ROW(DFS_A, 0), DFS_ROW(DFS_A, 1), DFS_ROW(DFS_A, 2), DFS_ROW(DFS_A, 3),          \
                    DFS_ROW(DFS_A, 4), DFS_ROW(DFS_A, 5), DFS_ROW(DFS_A, 6)};                           \
    Q df AA[7][7] = {DFS_ROW(DFS_AA, 0), DFS_ROW(DFS_AA, 1), DFS_ROW(DFS_AA, 2), DFS_ROW(DFS_AA, 3),     \
                     DFS_ROW(DFS_AA, 4), DFS_ROW(DFS_AA, 5), DFS_ROW(DFS_AA, 6)};                       \
    Q df C[7] = DFS_V7(DFS_C);                                                                          \
    Q df BT[7] = DFS_V7(DFS_BT);                                                                        \
    Q df BTA[7] = DFS_V7(tsit5::bta);                                                                   \
    Q df RA[7] = DFS_V7(tsit5::rowsum_a);                                                               \
    Q df RAA[7] = DFS_V7(tsit5::rowsum_aa);
#if defined(__CUDACC__)
namespace dev {
DFS_TABLES(__constant__)
}
#endif
namespace host {
DFS_TABLES(static const)
}
#undef DFS_TABLES
#undef DFS_BT
#undef DFS_C
#undef DFS_V7
#undef DFS_AA
#undef DFS_A
#undef DFS_ROW
#if defined(__CUDA_ARCH__)
#define DFS_T dev::
#else
#define DFS_T host::
#endif

constexpr double kAbstol = 1e-6, kBeta1 = 0.14, kBeta2 = 0.08, kQminInv = 5.0, kQmaxInv = 0.1, kGamma = 0.9,
                 kQoldInit = 1e-4, kLog2QoldInit = -13.287712379549449;
constexpr float kPreciseBelow = 1e-6f;  // the start-up ends after an accepted error estimate above this
constexpr float kSaeSkip = 50.0f;      // exp(-b r) with b r > 50 (< 2e-22 of the sum it joins) is dropped
constexpr float kExpm1Small = 1.4e-3f;  // below this |x| exp(x) - 1 is taken from its series

// the lookup tables of the elementary functions (ETRAJ_DF_* tables of dfloat.h)
struct Tabs {
    const float* exp2;
    const float* log2c;
    const float* rcpc;
};

// The differences dK_l (and of the phase rate) of stages l = 1..6 of the attempt,
// as float pairs at p[((l - 1) * KW + 2 c) * stride] (hi) and one stride further (lo).
template <int KW>
struct Slots {
    float* p;
    int stride;
    DFS_HD df get(int l, int c) const {
        const int i = ((l - 1) * KW + 2 * c) * stride;
        return df{p[i], p[i + stride]};
    }
    DFS_HD void set(int l, int c, df v) const {
        const int i = ((l - 1) * KW + 2 * c) * stride;
        p[i] = v.hi;
        p[i + stride] = v.lo;
    }
};

// ---- field table ------------------------------------------------------------------
// Piece k of the table: the degree-7 polynomial interpolating F at the Chebyshev
// nodes of [T0 + k h, T0 + (k+1) h], as monomial coefficients in the piece's local
// variable u in [-1, 1].  Per component (kDfTableF4 = 7 float4 per piece, x then y):
// c0 as the three-float split of its FP64 value (exact), c1..c3 as double-float
// pairs, c4..c7 as floats.  F(t) = c0 + q(u) with |q| <= ~3e-3 |F| at this spacing,
// so a difference F(t_a) - F(t_b) = (c0_a - c0_b) + (q_a - q_b) is exact to ~2^-56 of F.
DFS_HD void split3(double v, float& a, float& b, float& c) {
    a = (float)v;
    const double r = v - (double)a;
    b = (float)r;
    c = (float)(r - (double)b);
}

DFS_HD void table_piece(const DLaser& L, double T0, double h, int k, const DfTableNodes& N, float4* o) {
    constexpr double kMono[8][8] = {{1, 0, 0, 0, 0, 0, 0, 0},       {0, 1, 0, 0, 0, 0, 0, 0},
                                    {-1, 0, 2, 0, 0, 0, 0, 0},      {0, -3, 0, 4, 0, 0, 0, 0},
                                    {1, 0, -8, 0, 8, 0, 0, 0},      {0, 5, 0, -20, 0, 16, 0, 0},
                                    {-1, 0, 18, 0, -48, 0, 32, 0}, {0, -7, 0, 56, 0, -112, 0, 64}};
    double fx[8], fy[8];
    for (int j = 0; j < 8; ++j) laser_F(L, T0 + h * ((double)k + 0.5 * (N.u[j] + 1.0)), fx[j], fy[j]);
    double cx[8] = {0, 0, 0, 0, 0, 0, 0, 0}, cy[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int m = 0; m < 8; ++m) {
        double ax = 0.0, ay = 0.0;
        for (int j = 0; j < 8; ++j) {
            ax = ax + fx[j] * N.Tm[m][j];
            ay = ay + fy[j] * N.Tm[m][j];
        }
        const double w = (m == 0) ? 0.125 : 0.25;
        ax = ax * w;
        ay = ay * w;
        for (int i = 0; i < 8; ++i) {
            cx[i] = cx[i] + ax * kMono[m][i];
            cy[i] = cy[i] + ay * kMono[m][i];
        }
    }
    // 28 floats: x at [0, 13), y at [13, 26), 2 spare
    float w[28];
    const double* cc[2] = {cx, cy};
    for (int q = 0; q < 2; ++q) {
        const double* c = cc[q];
        float* o13 = w + 13 * q;
        split3(c[0], o13[0], o13[1], o13[2]);
        for (int i = 0; i < 3; ++i) {
            const float hi = (float)c[i + 1];
            o13[3 + 2 * i] = hi;
            o13[4 + 2 * i] = (float)(c[i + 1] - (double)hi);
        }
        for (int i = 0; i < 4; ++i) o13[9 + i] = (float)c[4 + i];
    }
    w[26] = w[27] = 0.0f;
    for (int i = 0; i < kDfTableF4; ++i) o[i] = make_float4(w[4 * i], w[4 * i + 1], w[4 * i + 2], w[4 * i + 3]);
}

// The laser table at one time: the exact c0 of each component (three floats) and
// q(u) = u (c1 + u (c2 + u (c3 + u (c4 + ...)))) in double-float.
struct FieldAt {
    float c0x[3], c0y[3];
    df qx, qy;
};

DFS_HD df q_of(const float* c, df u) {
    const float t = fmaf(fmaf(fmaf(c[12], u.hi, c[11]), u.hi, c[10]), u.hi, c[9]);
    df s = df_fma_f(t, u, df{c[7], c[8]});
    s = df_fma(s, u, df{c[5], c[6]});
    s = df_fma(s, u, df{c[3], c[4]});
    return df_mul(s, u);
}

DFS_HD void field_at(const DFParams& P, int n, df f, FieldAt& F) {
    n = n < 0 ? 0 : (n > P.n_int - 1 ? P.n_int - 1 : n);
    const df u = df_add_f(df{f.hi * 2.0f, f.lo * 2.0f}, -1.0f);
    const float4* p = P.table + kDfTableF4 * (size_t)n;
    float w[28];
    for (int i = 0; i < kDfTableF4; ++i) {
#if defined(__CUDA_ARCH__)
        const float4 v = __ldg(p + i);
#else
        const float4 v = p[i];
#endif
        w[4 * i] = v.x;
        w[4 * i + 1] = v.y;
        w[4 * i + 2] = v.z;
        w[4 * i + 3] = v.w;
    }
    for (int i = 0; i < 3; ++i) {
        F.c0x[i] = w[i];
        F.c0y[i] = w[13 + i];
    }
    F.qx = q_of(w, u);
    F.qy = q_of(w + 13, u);
}

// c0 (three floats) as a double-float
DFS_HD df c0_df(const float* c) { return quick_two_sum(c[0], c[1] + c[2]); }
// a - b of two exact three-float values, as a double-float
DFS_HD df diff3(const float* a, const float* b) {
    const df s = df_add(two_sum(a[0], -b[0]), two_sum(a[1], -b[1]));
    return df_add_f(s, a[2] - b[2]);
}

// clock (n, f) advanced by d >= 0 table intervals; the fraction stays in [0, 1)
DFS_HD void clk_adv(int n, df f, df d, int& no, df& fo) {
    df g = df_add(f, d);
    float k = floorf(g.hi);
    g = quick_two_sum(g.hi - k, g.lo);  // g.hi - k is exact
    if (g.hi < 0.0f) {
        g = df_add_f(g, 1.0f);
        k -= 1.0f;
    } else if (g.hi >= 1.0f) {
        g = df_add_f(g, -1.0f);
        k += 1.0f;
    }
    no = n + (int)k;
    fo = g;
}

// ---- target ---------------------------------------------------------------------------
// exp(-b r) of the SAE potential; a lane with b r > 50 takes exactly 0, and on the
// device a warp whose active lanes all do skips the evaluation: no lane's result
// depends on the electrons that share its warp.
DFO df sae_exp(df b, df r, const float* exptab) {
    const df br = df_mul(b, r);
    const bool far = br.hi > kSaeSkip;
#if defined(__CUDA_ARCH__)
    if (__all_sync(__activemask(), far)) return df{0.0f, 0.0f};
#endif
    if (far) return df{0.0f, 0.0f};
    return df_exp_neg(df_neg(br), exptab);
}

// The target's terms at one state (TargetPotential / TargetForce / TrajectoryFunction,
// HydrogenLikeAtom.jl:78-159, SAEAtom.jl:84-186): r^2 = x.x, y = (r^2 + sc)^(-1/2),
// y^3, the force coefficient coef (F_target = coef x) and the potential term V of the
// phase rate; for SAE targets also r, the three exp(-b_i r) and the two brackets
// br = Z + a1 (1 + b1 r) e1 + a3 (1 + b3 r) e3 and num = Z + a1 e1 + a2 r e2 + a3 e3.
struct TAt {
    df r2, y, y3, coef, V;
    df r, e1, e2, e3, br, num;
};

// the potential term: Z y (hydrogen-like), num y, or num y^2 for the 2D SCTS SAE
// reference, which divides by r^2+sc instead of its square root (SAEAtom.jl:136)
template <int DIM, int PHASE, int TGT>
DFS_HD df potential_of(const DFParams& P, const TAt& T) {
    if (TGT == ETRAJ_TARGET_HYDROGEN_LIKE) return df_mul(d2(P.Z), T.y);
    return (DIM == 2 && PHASE == ETRAJ_PHASE_SCTS) ? df_mul(T.num, df_sqr(T.y)) : df_mul(T.num, T.y);
}

// phase rate from the kinetic energy and the target's terms
template <int PHASE>
DFS_HD df phase_rate(const DFParams& P, df KE, df V, df coef_r2) {
    if (PHASE == ETRAJ_PHASE_QTMC) return df_neg(df_sub(df_add(d2(P.Ip), KE), V));
    return df_neg(df_add(df_sub(KE, V), coef_r2));
}

template <int DIM>
DFS_HD df half_sq(const df* p) {
    df s = df_add(df_sqr(p[0]), df_sqr(p[1]));
    if (DIM == 3) s = df_add(s, df_sqr(p[2]));
    return df{s.hi * 0.5f, s.lo * 0.5f};
}

// The target's terms evaluated directly at state (X, Pm); KT = coef X; kph the phase rate.
// Beyond r2_far (an SAE electron far from the core) every exp(-b_i r) is exactly
// 0, so br = num = Z and coef = -y^3 Z: the same bits the full formulas give
// there (adding an exact zero to a normalized pair changes nothing), without r
// and the brackets -- unless NEED_R (the start-up pass, whose differences read r).
template <int DIM, int PHASE, int TGT, bool NEED_R = true>
DFS_HD void target_at(const DFParams& P, const float* exptab, const df* X, const df* Pm, TAt& T, df* KT, df& kph) {
    T.r2 = df_add(df_sqr(X[0]), df_sqr(X[1]));
    if (DIM == 3) T.r2 = df_add(T.r2, df_sqr(X[2]));
    T.y = df_rsqrt(df_add(T.r2, d2(P.sc)));
    T.y3 = df_mul(df_sqr(T.y), T.y);
    if (TGT == ETRAJ_TARGET_HYDROGEN_LIKE) {
        T.coef = df_neg(df_mul(d2(P.Z), T.y3));
    } else if (!NEED_R && T.r2.hi > P.r2_far) {
        T.e1 = T.e2 = T.e3 = df{0.0f, 0.0f};
        T.br = T.num = d2(P.Z);
        T.coef = df_neg(df_mul(T.y3, T.br));
    } else {
        T.r = df_sqrt(T.r2);
        T.e1 = sae_exp(d2(P.b1), T.r, exptab);
        T.e2 = sae_exp(d2(P.b2), T.r, exptab);
        T.e3 = sae_exp(d2(P.b3), T.r, exptab);
        T.br = df_add(df_add(d2(P.Z), df_mul(df_mul(d2(P.a1), df_add_f(df_mul(d2(P.b1), T.r), 1.0f)), T.e1)),
                      df_mul(df_mul(d2(P.a3), df_add_f(df_mul(d2(P.b3), T.r), 1.0f)), T.e3));
        T.num = df_add(df_add(df_add(d2(P.Z), df_mul(d2(P.a1), T.e1)), df_mul(df_mul(d2(P.a2), T.r), T.e2)),
                       df_mul(d2(P.a3), T.e3));
        T.coef = df_neg(df_add(df_mul(T.y3, T.br), df_mul(df_mul(d2(P.a2b2), T.y), T.e2)));
    }
    for (int d = 0; d < DIM; ++d) KT[d] = df_mul(T.coef, X[d]);
    if (PHASE != ETRAJ_PHASE_CTMC) {
        T.V = potential_of<DIM, PHASE, TGT>(P, T);
        kph = phase_rate<PHASE>(P, half_sq<DIM>(Pm), T.V, df_mul(T.coef, T.r2));
    } else {
        kph = df{0.0f, 0.0f};
    }
}

// exp(-b r_l) and its change from exp(-b r_0) = e0, given dr = r_l - r_0
DFS_HD void exp_step(df b, df r_l, df dr, df e0, const float* exptab, df& el, df& de) {
    const df x = df_neg(df_mul(b, dr));
    const bool small = e0.hi != 0.0f && fabsf(x.hi) < kExpm1Small;
    if (small) {
        de = df_mul(e0, df_expm1_small(x));
        el = df_add(e0, de);
    } else {
        el = sae_exp(b, r_l, exptab);
        de = df_sub(el, e0);
    }
}

// The changes dKT of the target's force and dkph of the phase rate from x0 (terms B)
// to x0 + dX (P0 + dP the stage momentum), written as differences.  Returns false,
// leaving them to a direct evaluation, when s = r^2 + sc is not within a factor 2
// of s_0 (a pass near the core, where r changes by orders of magnitude within a
// step): there y_l = y_0 / b and its kin would be small remainders of cancelling
// terms, while such a step's error estimate needs no differences.
template <int DIM, int PHASE, int TGT>
DFS_HD bool target_diff(const DFParams& P, const float* exptab, const df* X0, const df* P0, const TAt& B,
                        const df* dX, const df* dP, df* dKT, df& dkph) {
    TAt T;
    // ds = r_l^2 - r_0^2 = 2 x0.dX + dX.dX,  delta = ds / s_0,  b = sqrt(1 + delta)
    df ds = df_add(df_mul(df_f(2.0f), df_mul(X0[0], dX[0])), df_sqr(dX[0]));
    for (int d = 1; d < DIM; ++d) ds = df_add(ds, df_add(df_mul(df_f(2.0f), df_mul(X0[d], dX[d])), df_sqr(dX[d])));
    const df y02 = df_sqr(B.y);
    const df delta = df_mul(ds, y02);
    if (!(delta.hi >= -0.5f && delta.hi <= 1.0f)) return false;
    const df opd = df_add_f(delta, 1.0f);
    const df b = df_sqrt(opd);
    const df bm1 = df_div(delta, df_add_f(b, 1.0f));  // b - 1
    const df ib = df_rcp(b);
    T.r2 = df_add(B.r2, ds);
    T.y = df_mul(B.y, ib);
    const df dy = df_neg(df_mul(df_mul(B.y, bm1), ib));
    // b^3 - 1 = (b - 1)(b^2 + b + 1), b^2 = 1 + delta
    const df ib3 = df_mul(df_sqr(ib), ib);
    const df dy3 = df_neg(df_mul(df_mul(B.y3, df_mul(bm1, df_add(df_add_f(opd, 1.0f), b))), ib3));
    T.y3 = df_add(B.y3, dy3);
    df dcoef, dV = df{0.0f, 0.0f};
    if (TGT == ETRAJ_TARGET_HYDROGEN_LIKE) {
        dcoef = df_neg(df_mul(d2(P.Z), dy3));
        if (PHASE != ETRAJ_PHASE_CTMC) dV = df_mul(d2(P.Z), dy);
    } else {
        T.r = df_sqrt(T.r2);
        const df dr = df_div(ds, df_add(T.r, B.r));
        df de1, de2, de3;
        exp_step(d2(P.b1), T.r, dr, B.e1, exptab, T.e1, de1);
        exp_step(d2(P.b2), T.r, dr, B.e2, exptab, T.e2, de2);
        exp_step(d2(P.b3), T.r, dr, B.e3, exptab, T.e3, de3);
        // d(br) = a1 ((1 + b1 r_l) de1 + b1 dr e1_0) + a3 ((1 + b3 r_l) de3 + b3 dr e3_0)
        const df dbr = df_add(
            df_mul(d2(P.a1), df_add(df_mul(df_add_f(df_mul(d2(P.b1), T.r), 1.0f), de1),
                                    df_mul(df_mul(d2(P.b1), dr), B.e1))),
            df_mul(d2(P.a3), df_add(df_mul(df_add_f(df_mul(d2(P.b3), T.r), 1.0f), de3),
                                    df_mul(df_mul(d2(P.b3), dr), B.e3))));
        T.br = df_add(B.br, dbr);
        // coef = -(y^3 br + a2 b2 y e2)
        dcoef = df_neg(df_add(df_add(df_mul(dy3, B.br), df_mul(T.y3, dbr)),
                              df_mul(d2(P.a2b2), df_add(df_mul(dy, B.e2), df_mul(T.y, de2)))));
        if (PHASE != ETRAJ_PHASE_CTMC) {
            // d(num) = a1 de1 + a2 (r_l de2 + dr e2_0) + a3 de3
            const df dnum = df_add(df_add(df_mul(d2(P.a1), de1),
                                          df_mul(d2(P.a2), df_add(df_mul(T.r, de2), df_mul(dr, B.e2)))),
                                   df_mul(d2(P.a3), de3));
            T.num = df_add(B.num, dnum);
            if (DIM == 2 && PHASE == ETRAJ_PHASE_SCTS) {
                // d(y^2) = -y0^2 delta / (1 + delta)
                const df dy2 = df_neg(df_mul(y02, df_div(delta, opd)));
                dV = df_add(df_mul(dnum, df_add(y02, dy2)), df_mul(B.num, dy2));
            } else {
                dV = df_add(df_mul(dnum, T.y), df_mul(B.num, dy));
            }
        }
    }
    T.coef = df_add(B.coef, dcoef);
    for (int d = 0; d < DIM; ++d) dKT[d] = df_add(df_mul(T.coef, dX[d]), df_mul(dcoef, X0[d]));
    if (PHASE != ETRAJ_PHASE_CTMC) {
        T.V = df_add(B.V, dV);
        // dKE = dP . (p0 + dP/2)
        df dKE = df_mul(dP[0], df_add(P0[0], df{dP[0].hi * 0.5f, dP[0].lo * 0.5f}));
        for (int d = 1; d < DIM; ++d) dKE = df_add(dKE, df_mul(dP[d], df_add(P0[d], df{dP[d].hi * 0.5f, dP[d].lo * 0.5f})));
        if (PHASE == ETRAJ_PHASE_QTMC) {
            dkph = df_neg(df_sub(dKE, dV));
        } else {
            // d(coef r^2) = coef_l ds + dcoef r_0^2
            const df dcr2 = df_add(df_mul(T.coef, ds), df_mul(dcoef, B.r2));
            dkph = df_neg(df_add(df_sub(dKE, dV), dcr2));
        }
    } else {
        dkph = df{0.0f, 0.0f};
    }
    return true;
}

// ---- one electron ---------------------------------------------------------------------
template <int DIM, int PHASE>
struct Lane {
    static constexpr bool HASPH = (PHASE != ETRAJ_PHASE_CTMC);
    static constexpr int N = 2 * DIM + (HASPH ? 1 : 0);   // ODE state size
    static constexpr int KW = 2 * DIM + (HASPH ? 2 : 0);  // floats of one stage slot (dK, dkph)
    df X[DIM], Pv[DIM], PH;   // accepted state (position, momentum, phase)
    df K0[DIM], kph0;         // derivative at the accepted state (momentum rows), phase rate
    df KT0[DIM];              // the target's force there (coef x)
    FieldAt F0;               // laser table at the accepted state's time
    df dX[DIM], dP[DIM];      // increments of the state to evaluate next
    df dt, dth, dt2, dtprop, dtmax, lqold, q11;
    df tfr, f1, fi;           // clock fractions: accepted state, end of the attempt, evaluation
    FieldAt F5;               // laser table at the end of the attempt (stage 5), for stage 6
    df d1;                    // starting step: |f0 / sk|
    float dtmin;
    int tn, n1, ni;           // clock intervals: accepted state, end of the attempt, evaluation
    int iter, attempts;
    float elast;              // the last accepted error estimate (0 before the first)
    bool accept, last;
};

DFS_HD double ulp_of(double x) {
    double a = x < 0 ? -x : x;
    uint64_t u;
    std::memcpy(&u, &a, sizeof u);
    ++u;
    double b;
    std::memcpy(&b, &u, sizeof b);
    return b - a;
}

template <int DIM, int PHASE>
DFS_HD void load(Lane<DIM, PHASE>& L, const DFParams& P, const double* x0, const double* p0, double ph0,
                 double t0) {
    for (int d = 0; d < DIM; ++d) {
        L.X[d] = df_from_double(x0[d]);
        L.Pv[d] = df_from_double(p0[d]);
        L.dX[d] = df_f(0.0f);
        L.dP[d] = df_f(0.0f);
    }
    L.PH = df_from_double(ph0);
    const double q0 = (t0 - P.T0) * P.inv_h_d;
    const double fl = floor(q0);
    L.tn = L.ni = (int)fl;
    L.tfr = L.fi = df_from_double(q0 - fl);
    L.dtmax = df_from_double(P.t_final - t0);
    const double ua = ulp_of(t0), ub = ulp_of(P.t_final);
    L.dtmin = (float)(ua > ub ? ua : ub);
    L.iter = 0;
    L.attempts = 0;
    L.elast = 0.0f;
    L.accept = false;
    L.last = false;
    L.lqold = dfc(kLog2QoldInit);
    L.q11 = df_f(1.0f);
}

// The accepted state's derivative from its target force KT = coef X, phase rate kph
// and laser table F.
template <int DIM, int PHASE>
DFS_HD void set_base(Lane<DIM, PHASE>& L, const FieldAt& F, const df* KT, df kph) {
    L.F0 = F;
    L.kph0 = kph;
    for (int d = 0; d < DIM; ++d) L.K0[d] = L.KT0[d] = KT[d];
    L.K0[0] = df_sub(L.K0[0], df_add(c0_df(F.c0x), F.qx));
    L.K0[1] = df_sub(L.K0[1], df_add(c0_df(F.c0y), F.qy));
}

// dK = K - K_0 of an evaluation (target change dKT, dkph; laser table F), into slot l (1..6)
template <int DIM, int PHASE, int KW>
DFS_HD void set_diff(const Lane<DIM, PHASE>& L, const Slots<KW>& k, int l, const FieldAt& F, const df* dKT,
                     df dkph) {
    const df dFx = df_add(diff3(F.c0x, L.F0.c0x), df_sub(F.qx, L.F0.qx));
    const df dFy = df_add(diff3(F.c0y, L.F0.c0y), df_sub(F.qy, L.F0.qy));
    k.set(l, 0, df_sub(dKT[0], dFx));
    k.set(l, 1, df_sub(dKT[1], dFy));
    if (DIM == 3) k.set(l, 2, dKT[2]);
    if (Lane<DIM, PHASE>::HASPH) k.set(l, DIM, dkph);
}

// The main pass keeps each stage's whole derivative instead: K_l = KT - F (the
// momentum rows, formed as set_base forms K_0) and the phase rate, into slot l.
template <int DIM, int PHASE, int KW>
DFS_HD void set_full(const Lane<DIM, PHASE>& L, const Slots<KW>& k, int l, const FieldAt& F, const df* KT,
                     df kph) {
    k.set(l, 0, df_sub(KT[0], df_add(c0_df(F.c0x), F.qx)));
    k.set(l, 1, df_sub(KT[1], df_add(c0_df(F.c0y), F.qy)));
    if (DIM == 3) k.set(l, 2, KT[2]);
    if (Lane<DIM, PHASE>::HASPH) k.set(l, DIM, kph);
}

// sqrt(sum_j (v_j / sk_j)^2 / N)
template <int N>
DFS_HD df rms_ratio(const df* v, const df* sk) {
    df acc = df{0.0f, 0.0f};
    for (int j = 0; j < N; ++j) {
        const df q = df_div(v[j], sk[j]);
        acc = df_fma(q, q, acc);
    }
    return df_sqrt(df_div(acc, df_f((float)N)));
}

template <int DIM, int PHASE>
DFS_HD void scales(const Lane<DIM, PHASE>& L, const DFParams& P, df* sk) {
    constexpr int N = Lane<DIM, PHASE>::N;
    for (int d = 0; d < DIM; ++d) {
        sk[d] = df_fma(df_abs(L.X[d]), d2(P.rtol), dfc(kAbstol));
        sk[DIM + d] = df_fma(df_abs(L.Pv[d]), d2(P.rtol), dfc(kAbstol));
    }
    if (Lane<DIM, PHASE>::HASPH) sk[N - 1] = df_fma(df_abs(L.PH), d2(P.rtol), dfc(kAbstol));
}

// After set_base at the initial state: d0, d1 and dt0 of Hairer's starting step
// (initdt of integrate_fp64.cu), and the increments of u1 = u0 + dt0 f0 to
// evaluate next.  Returns false when the step is decided already (dt0 below 10 eps).
template <int DIM, int PHASE>
DFS_HD bool init_first(Lane<DIM, PHASE>& L, const DFParams& P) {
    constexpr int N = Lane<DIM, PHASE>::N;
    df sk[N], u0[N], f0[N];
    scales(L, P, sk);
    for (int d = 0; d < DIM; ++d) {
        u0[d] = L.X[d];
        u0[DIM + d] = L.Pv[d];
        f0[d] = L.Pv[d];
        f0[DIM + d] = L.K0[d];
    }
    if (Lane<DIM, PHASE>::HASPH) {
        u0[N - 1] = L.PH;
        f0[N - 1] = L.kph0;
    }
    const df d0 = rms_ratio<N>(u0, sk);
    L.d1 = rms_ratio<N>(f0, sk);
    df dt0 = (d0.hi < 1e-5f || L.d1.hi < 1e-5f) ? dfc(1e-6) : df_div(df_div(d0, L.d1), df_f(100.0f));
    dt0 = df_min(dt0, L.dtmax);
    if (dt0.hi < 2.220446049250313e-15f) {
        L.dt = L.dtprop = dfc(1e-6);
        return false;
    }
    for (int d = 0; d < DIM; ++d) {
        L.dX[d] = df_mul(dt0, L.Pv[d]);
        L.dP[d] = df_mul(dt0, L.K0[d]);
    }
    clk_adv(L.tn, L.tfr, df_mul(dt0, d2(P.inv_h)), L.ni, L.fi);
    L.dth = dt0;
    return true;
}

// After the evaluation at u1 (its differences in slot 1): d2 and the starting step.
template <int DIM, int PHASE, int KW>
DFS_HD void init_second(Lane<DIM, PHASE>& L, const DFParams& P, const Slots<KW>& k, const Tabs& T) {
    constexpr int N = Lane<DIM, PHASE>::N;
    df sk[N], dfv[N];
    scales(L, P, sk);
    const df dt0 = L.dth;
    for (int d = 0; d < DIM; ++d) {
        dfv[d] = L.dP[d];  // f1 - f0 of a position row: (p + dt0 K0) - p
        dfv[DIM + d] = k.get(1, d);
    }
    if (Lane<DIM, PHASE>::HASPH) dfv[N - 1] = k.get(1, DIM);
    const df dd2 = df_div(rms_ratio<N>(dfv, sk), dt0);
    const df md = df_max(L.d1, dd2);
    df dt1;
    if (md.hi <= 1e-15f) {
        dt1 = df_max(dfc(1e-6), df_mul(dt0, dfc(1e-3)));
    } else {
        // 10^(-(2 + log10 md)/5) = 2^(-(2 log2 10 + log2 md)/5)
        const df e = df_add(df_mul(df_f(2.0f), kDfLog2Of10), df_log2(md, T.log2c, T.rcpc));
        dt1 = df_exp2(df_mul(e, dfc(-0.2)), T.exp2);
    }
    L.dt = df_max(df_f(L.dtmin), df_min(df_min(df_mul(dt0, df_f(100.0f)), dt1), L.dtmax));
    L.dtprop = L.dt;
}

// Start of a step attempt (the top of solve()'s loop).  Returns a status > 0 when
// the solve ends before the attempt (1 MaxIters, 2 DtLessThanMin, 4 DtNaN).
template <int DIM, int PHASE>
DFS_HD int prologue(Lane<DIM, PHASE>& L, const DFParams& P) {
    if (L.iter > 0) {
        if (!L.accept) L.dt = df_div(L.dt, df_min(dfc(kQminInv), df_div(L.q11, dfc(kGamma))));
        else L.dt = L.dtprop;
    }
    ++L.iter;
    L.dt = df_max(df_min(L.dtmax, L.dt), df_f(L.dtmin));
    const df rem = df_mul(df_add(df_f((float)(P.nf - L.tn)), df_sub(d2(P.ff), L.tfr)), d2(P.h));
    L.last = !df_lt(L.dt, rem);
    if (L.last) L.dt = rem;
    if (!(L.dt.hi == L.dt.hi)) return 4;
    if (L.iter > P.max_iters) return 1;
    if (L.dt.hi <= L.dtmin && (!L.accept || !L.last)) return 2;
    L.dth = df_mul(L.dt, d2(P.inv_h));
    L.dt2 = df_sqr(L.dt);
    if (L.last) {
        L.n1 = P.nf;
        L.f1 = d2(P.ff);
    } else {
        clk_adv(L.tn, L.tfr, L.dth, L.n1, L.f1);
    }
    return 0;
}

// Sum of products c_l v_l: one TwoSum per term, the rounding errors gathered in a
// float and normalized at the end; it may start from a double-float value.
struct Acc {
    float s = 0.0f, e = 0.0f;
    DFS_HD Acc() {}
    DFS_HD explicit Acc(df v) : s(v.hi), e(v.lo) {}
    DFS_HD void add(df c, df v) {
        const df p = two_prod(c.hi, v.hi);
        const float pe = fmaf(c.hi, v.lo, fmaf(c.lo, v.hi, p.lo));
        const df t = two_sum(s, p.hi);
        s = t.hi;
        e += t.lo + pe;
    }
    DFS_HD df get() const { return two_sum(s, e); }
};

// The increments and clock of stage st (1..6; 6 is the new state):
// dP = dt ((sum_l A_l) K_0 + sum_l A_l dK_l) and
// dX = (sum_l A_l) dt p0 + dt^2 ((sum_l (A A)_l) K_0 + sum_l (A A)_l dK_l);
// with FULL slots (the main pass) the same sums over K_0 .. K_{st-1}.
// st is the same for every stepping lane of a warp, so the coefficients are
// uniform constant-memory reads and one copy of the code serves all stages.
template <bool FULL, int DIM, int PHASE, int KW>
DFS_HD void stage_in(Lane<DIM, PHASE>& L, const Slots<KW>& k, int st) {
    const df adt = df_mul(DFS_T RA[st], L.dt);
    for (int d = 0; d < DIM; ++d) {
        Acc sa(df_mul(FULL ? DFS_T A[st][0] : DFS_T RA[st], L.K0[d])),
            saa(df_mul(FULL ? DFS_T AA[st][0] : DFS_T RAA[st], L.K0[d]));
        for (int l = 1; l < st; ++l) {
            const df kl = k.get(l, d);
            sa.add(DFS_T A[st][l], kl);
            if (l + 1 < st) saa.add(DFS_T AA[st][l], kl);  // (A A)[st][st-1] = 0
        }
        L.dP[d] = df_mul(L.dt, sa.get());
        L.dX[d] = df_fma(adt, L.Pv[d], df_mul(L.dt2, saa.get()));
    }
    if (st < 5) {
        clk_adv(L.tn, L.tfr, df_mul(DFS_T C[st], L.dth), L.ni, L.fi);
    } else {
        L.ni = L.n1;
        L.fi = L.f1;
    }
}

// Whether the coming start-up attempt forms its stages as differences (the last
// accepted error estimate was below 1e-6); the first attempt for which it does
// not ends the start-up.
template <int DIM, int PHASE>
DFS_HD bool precise(const Lane<DIM, PHASE>& L) {
    return L.elast < kPreciseBelow;
}

// One evaluation of the target at x0 + (dX, dP): the change of its terms from the
// accepted state (dKT, dkph), as differences from its terms B there when wanted
// (DIFF and diff) and possible, and with direct terms T, KT = coef x and kph at
// the new point when wanted (direct) or when the difference was not formed.
template <int DIM, int PHASE, int TGT, bool DIFF>
DFS_HD void target_eval(const DFParams& P, const float* exptab, const Lane<DIM, PHASE>& L, const TAt& B, bool diff,
                        bool direct, TAt& T, df* KT, df* dKT, df& dkph, df& kph) {
    bool ok = false;
    if (DIFF && diff) ok = target_diff<DIM, PHASE, TGT>(P, exptab, L.X, L.Pv, B, L.dX, L.dP, dKT, dkph);
    if (direct || !ok) {
        df Xl[DIM], Pl[DIM];
        for (int d = 0; d < DIM; ++d) {
            Xl[d] = df_add(L.X[d], L.dX[d]);
            Pl[d] = df_add(L.Pv[d], L.dP[d]);
        }
        target_at<DIM, PHASE, TGT, DIFF>(P, exptab, Xl, Pl, T, KT, kph);
        if (!ok && DIFF) {  // (the main pass keeps whole derivatives, set_full)
            for (int d = 0; d < DIM; ++d) dKT[d] = df_sub(KT[d], L.KT0[d]);
            dkph = df_sub(kph, L.kph0);
        }
    }
}

// After the evaluation of stage 6 (slot 6): error estimate, controller and the
// decision (the bottom of solve()'s loop).  Returns -1 when t_final is reached, a
// status > 0 on failure (3 Unstable, 4 DtNaN), 0 to go on; after an accepted step
// that goes on (L.accept) the caller makes stage 6's direct target terms the new
// state's (set_base with the laser table L.F5).
template <bool FULL, int DIM, int PHASE, int KW>
DFS_HD int epilogue(Lane<DIM, PHASE>& L, const DFParams& P, const Slots<KW>& k, const Tabs& T) {
    constexpr bool HASPH = Lane<DIM, PHASE>::HASPH;
    constexpr int N = Lane<DIM, PHASE>::N;
    df dPH = df{0.0f, 0.0f};
    if (HASPH) {
        Acc a(df_mul(FULL ? DFS_T A[6][0] : DFS_T RA[6], L.kph0));
#pragma unroll
        for (int l = 1; l < 6; ++l) a.add(DFS_T A[6][l], k.get(l, DIM));
        dPH = df_mul(L.dt, a.get());
    }
    const df PHn = df_add(L.PH, dPH);
    // RMS of the error estimate over the scales abstol + rtol max(|u_prev|, |u_new|);
    // the weights of K_0 (sum bt, sum bt A) are 0 on differences
    df acc = df{0.0f, 0.0f};
    df Xn[DIM], Pn[DIM];
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        Acc ex, ep;
        if (FULL) {
            ex = Acc(df_mul(DFS_T BTA[0], L.K0[d]));
            ep = Acc(df_mul(DFS_T BT[0], L.K0[d]));
        }
#pragma unroll
        for (int l = 1; l < 7; ++l) {
            const df kl = k.get(l, d);
            if (l < 6) ex.add(DFS_T BTA[l], kl);  // (bt A)[6] = 0
            ep.add(DFS_T BT[l], kl);
        }
        Xn[d] = df_add(L.X[d], L.dX[d]);
        Pn[d] = df_add(L.Pv[d], L.dP[d]);
        const df scx = df_fma(df_max(df_abs(L.X[d]), df_abs(Xn[d])), d2(P.rtol), dfc(kAbstol));
        const df scp = df_fma(df_max(df_abs(L.Pv[d]), df_abs(Pn[d])), d2(P.rtol), dfc(kAbstol));
        const df rx = df_div(df_mul(L.dt2, ex.get()), scx);
        const df rp = df_div(df_mul(L.dt, ep.get()), scp);
        acc = df_fma(rx, rx, df_fma(rp, rp, acc));
    }
    if (HASPH) {
        Acc ef;
        if (FULL) ef = Acc(df_mul(DFS_T BT[0], L.kph0));
#pragma unroll
        for (int l = 1; l < 7; ++l) ef.add(DFS_T BT[l], k.get(l, DIM));
        const df scf = df_fma(df_max(df_abs(L.PH), df_abs(PHn)), d2(P.rtol), dfc(kAbstol));
        const df rf = df_div(df_mul(L.dt, ef.get()), scf);
        acc = df_fma(rf, rf, acc);
    }
    const df EEst = df_sqrt(df_div(acc, df_f((float)N)));
    ++L.attempts;
    if (!(EEst.hi == EEst.hi)) return 4;
    L.accept = !df_lt(df_f(1.0f), EEst);
    // log2 EEst (EEst below 1e-30 gives the same clamped q as its exact value)
    const df l2e = df_log2(df_max(EEst, df_f(1e-30f)), T.log2c, T.rcpc);
    if (!L.accept) {
        L.q11 = df_exp2(df_mul(dfc(kBeta1), l2e), T.exp2);
        return 0;
    }
    df q;
    if (EEst.hi == 0.0f) {
        q = dfc(kQmaxInv);
    } else {
        // q = EEst^beta1 / qold^beta2 / gamma, clamped to [1/qmax, 1/qmin]
        q = df_exp2(df_sub(df_mul(dfc(kBeta1), l2e), df_mul(dfc(kBeta2), L.lqold)), T.exp2);
        q = df_max(dfc(kQmaxInv), df_min(dfc(kQminInv), df_div(q, dfc(kGamma))));
    }
    L.lqold = df_lt(EEst, dfc(kQoldInit)) ? dfc(kLog2QoldInit) : l2e;
    L.elast = EEst.hi;
    L.dtprop = df_max(df_min(L.dtmax, df_div(L.dt, q)), df_f(L.dtmin));
    bool bad = false;
    for (int d = 0; d < DIM; ++d) {
        L.X[d] = Xn[d];
        L.Pv[d] = Pn[d];
        bad |= !(Xn[d].hi == Xn[d].hi) || !(Pn[d].hi == Pn[d].hi);
    }
    L.PH = PHn;
    L.tn = L.n1;
    L.tfr = L.f1;
    if (L.last) return -1;
    // within 100 ulp of t_final the FP64 solve takes t = t_final and stops
    const df rem = df_mul(df_add(df_f((float)(P.nf - L.tn)), df_sub(d2(P.ff), L.tfr)), d2(P.h));
    if (rem.hi < P.t_snap) return -1;
    return bad ? 3 : 0;
}

// ---- the start-up pass's hand-over -----------------------------------------------------
// An electron leaves the start-up pass at the first attempt boundary where its
// last accepted error estimate is not below 1e-6 (always right after an accepted
// step): word w of carried electron k at c[w * cap + k].  What it carries is what
// the next attempt reads; the main pass evaluates the target and the laser at the
// state again, which gives the bits stage 6 gave (x + 0 is x).
struct Carry {
    float* c;
    int64_t cap;
    DFS_HD float& w(int i, int64_t k) const { return c[(int64_t)i * cap + k]; }
    DFS_HD void put(int& i, int64_t k, df v) const {
        w(i++, k) = v.hi;
        w(i++, k) = v.lo;
    }
    DFS_HD df take(int& i, int64_t k) const {
        const df v{w(i, k), w(i + 1, k)};
        i += 2;
        return v;
    }
    DFS_HD void put_i(int& i, int64_t k, uint32_t v) const {
        uint32_t* u = reinterpret_cast<uint32_t*>(c);
        u[(int64_t)(i++) * cap + k] = v;
    }
    DFS_HD uint32_t take_i(int& i, int64_t k) const {
        const uint32_t* u = reinterpret_cast<const uint32_t*>(c);
        return u[(int64_t)(i++) * cap + k];
    }
};

template <int DIM, int PHASE>
DFS_HD void save_carry(const Lane<DIM, PHASE>& L, const Carry& C, int64_t k, uint64_t s) {
    int i = 0;
    for (int d = 0; d < DIM; ++d) {
        C.put(i, k, L.X[d]);
        C.put(i, k, L.Pv[d]);
    }
    C.put(i, k, L.PH);
    C.put(i, k, L.tfr);
    C.put(i, k, L.dtprop);
    C.put(i, k, L.dtmax);
    C.put(i, k, L.lqold);
    C.w(i++, k) = L.dtmin;
    C.put_i(i, k, (uint32_t)L.tn);
    C.put_i(i, k, (uint32_t)L.iter);
    C.put_i(i, k, (uint32_t)L.attempts);
    C.put_i(i, k, (uint32_t)s);
    C.put_i(i, k, (uint32_t)(s >> 32));
}

// Restores carried electron k; returns its index.  The target and laser at the
// state are evaluated next (dX = dP = 0 at clock tn + tfr).
template <int DIM, int PHASE>
DFS_HD uint64_t restore_carry(Lane<DIM, PHASE>& L, const Carry& C, int64_t k) {
    int i = 0;
    for (int d = 0; d < DIM; ++d) {
        L.X[d] = C.take(i, k);
        L.Pv[d] = C.take(i, k);
        L.dX[d] = df_f(0.0f);
        L.dP[d] = df_f(0.0f);
    }
    L.PH = C.take(i, k);
    L.tfr = L.fi = C.take(i, k);
    L.dtprop = L.dt = C.take(i, k);
    L.dtmax = C.take(i, k);
    L.lqold = C.take(i, k);
    L.dtmin = C.w(i++, k);
    L.tn = L.ni = (int)C.take_i(i, k);
    L.iter = (int)C.take_i(i, k);
    L.attempts = (int)C.take_i(i, k);
    const uint64_t lo = C.take_i(i, k);
    const uint64_t hi = C.take_i(i, k);
    L.accept = true;
    L.last = false;
    L.q11 = df_f(1.0f);
    return lo | (hi << 32);
}

template <int DIM, int PHASE>
DFS_HD void final_state(const Lane<DIM, PHASE>& L, double* fs) {
    for (int d = 0; d < DIM; ++d) {
        fs[d] = df_to_double(L.X[d]);
        fs[DIM + d] = df_to_double(L.Pv[d]);
    }
    if (Lane<DIM, PHASE>::HASPH) fs[2 * DIM] = df_to_double(L.PH);
}

}  // namespace dfs
}  // namespace etraj
