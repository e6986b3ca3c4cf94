// integrate_fp32.cu -- the bulk integrator: persistent, warp-cooperative,
// work-stealing Tsit5 with FP32 stages and compensated state.
//
// Same method and step controller as the plain FP64 path (Tsit5, abstol 1e-6,
// RMS error norm, PI control with beta1 = 7/50, beta2 = 2/25; see
// integrate_fp64.cu), re-cast for GB300's FP32 CUDA cores:
//
//  * Field table.  F(t) is one function of time shared by every trajectory,
//    so it is tabulated once per job in FP64 (cubic Hermite pieces from the
//    exact F and its forward-mode derivative, spacing h = T_min/512; largest
//    error ~1e-6 F0 at the steep tanh window edges, ~1e-8 F0 elsewhere) and
//    stored as FP32 polynomial coefficients, in shared memory when it fits.
//    A right-hand side then costs 6 FFMA for the field instead of two sincos
//    and two tanh, for every laser kind alike.
//  * Fixed-point time.  t = T0 + h (n + f) with an integer interval n and an
//    FP32 fraction f, i.e. ~1e-7 a.u. resolution over any time span, without
//    FP64 arithmetic in the step loop.
//  * Second-order form.  For the position rows (x' = p) the stage values and
//    the update are evaluated as x + c_i dt p + dt^2 (A A)_i . K, with K the
//    momentum derivatives: algebraically the same Tsit5 step, but the
//    position error estimate dt^2 (b~ A) . K no longer cancels large stage
//    momenta, which in FP32 put a noise floor of ~3e-5 under EEst.
//  * Compensated state.  Positions, momenta and the QTMC/SCTS phase are
//    double-float pairs (hi + lo, Knuth's TwoSum), so 1e3 steps add no
//    rounding drift; stage values and the error estimate are plain FP32.
//  * Work stealing.  One lane owns one trajectory; when it finishes, the lane
//    takes the next one from a global queue (warp-aggregated atomicAdd), so
//    step counts that differ 100x between trajectories do not idle the warp.
//    `refill_min` lanes must be free before a warp refills (autotuned).
//
// The kernel writes the final state in FP64 (hi + lo); the Kepler asymptote,
// SCTS correction and deposit contribution are then computed in FP64 by the
// collection kernel of integrate_fp64.cu, exactly as on the plain path.
//
// Roofline: FP32 issue bound, MUFU for rsqrt/exp2/log2; no tensor cores.

#include "physics.cuh"

namespace etraj {

namespace {

// Tsit5 tableau (Tsitouras 2011); row 6 of A is the solution weights b.
constexpr double kC[7] = {0.0, 0.161, 0.327, 0.9, 0.9800255409045097, 1.0, 1.0};
constexpr double kA[7][7] = {
    {0, 0, 0, 0, 0, 0, 0},
    {0.161, 0, 0, 0, 0, 0, 0},
    {-0.008480655492356989, 0.335480655492357, 0, 0, 0, 0, 0},
    {2.897153057105493, -6.359448489975075, 4.3622954328695815, 0, 0, 0, 0},
    {5.325864828439257, -11.748883564062828, 7.4955393428898365, -0.09249506636175525, 0, 0, 0},
    {5.86145544294642, -12.92096931784711, 8.159367898576159, -0.071584973281401, -0.028269050394068383, 0, 0},
    {0.09646076681806523, 0.01, 0.4798896504144996, 1.379008574103742, -3.290069515436081, 2.324710524099774, 0}};
constexpr double kBT[7] = {-0.00178001105222577714, -0.0008164344596567469, 0.007880878010261995,
                           -0.1447110071732629, 0.5823571654525552, -0.45808210592918697,
                           0.015151515151515152};
constexpr double aa(int i, int l) {
    double s = 0.0;
    for (int j = 0; j < 7; ++j) s += kA[i][j] * kA[j][l];
    return s;
}
constexpr double bta(int l) {
    double s = 0.0;
    for (int i = 0; i < 7; ++i) s += kBT[i] * kA[i][l];
    return s;
}

#define ETRAJ_ROW(f, i) {(float)f(i, 0), (float)f(i, 1), (float)f(i, 2), (float)f(i, 3), (float)f(i, 4), (float)f(i, 5), (float)f(i, 6)}
#define ETRAJ_A(i, l) kA[i][l]
__constant__ float cA[7][7] = {ETRAJ_ROW(ETRAJ_A, 0), ETRAJ_ROW(ETRAJ_A, 1), ETRAJ_ROW(ETRAJ_A, 2),
                               ETRAJ_ROW(ETRAJ_A, 3), ETRAJ_ROW(ETRAJ_A, 4), ETRAJ_ROW(ETRAJ_A, 5),
                               ETRAJ_ROW(ETRAJ_A, 6)};
__constant__ float cAA[7][7] = {ETRAJ_ROW(aa, 0), ETRAJ_ROW(aa, 1), ETRAJ_ROW(aa, 2), ETRAJ_ROW(aa, 3),
                                ETRAJ_ROW(aa, 4), ETRAJ_ROW(aa, 5), ETRAJ_ROW(aa, 6)};
#undef ETRAJ_A
#undef ETRAJ_ROW
__constant__ float cC[7] = {(float)kC[0], (float)kC[1], (float)kC[2], (float)kC[3], (float)kC[4], (float)kC[5], (float)kC[6]};
__constant__ float cBT[7] = {(float)kBT[0], (float)kBT[1], (float)kBT[2], (float)kBT[3], (float)kBT[4], (float)kBT[5], (float)kBT[6]};
__constant__ float cBTA[7] = {(float)bta(0), (float)bta(1), (float)bta(2), (float)bta(3), (float)bta(4), (float)bta(5), (float)bta(6)};

constexpr float ABSTOL = 1e-6f, BETA1 = 0.14f, BETA2 = 0.08f, QMIN_INV = 5.0f, QMAX_INV = 0.1f,
                GAMMA = 0.9f, QOLDINIT = 1e-4f;
constexpr int MAXITERS = 1000000;
constexpr float kDthMin = 2.4e-7f;  // smallest step (in table intervals) the FP32 clock resolves

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// (hi, lo) += d
__device__ __forceinline__ void df_add(float& hi, float& lo, float d) {
    float s, e;
    two_sum(hi, d, s, e);
    e = e + lo;
    hi = s + e;
    lo = e - (hi - s);
}

__device__ __forceinline__ float rsqrt_nr(float s) {
    float r = rsqrtf(s);
    return r * fmaf(-0.5f * s, r * r, 1.5f);
}

__device__ __forceinline__ void field(const float4* __restrict__ tab, int n_int, int ni, float fi,
                                      float& Fx, float& Fy) {
    ni = min(max(ni, 0), n_int - 1);
    const float4 a = tab[2 * ni], b = tab[2 * ni + 1];
    Fx = fmaf(fmaf(fmaf(a.w, fi, a.z), fi, a.y), fi, a.x);
    Fy = fmaf(fmaf(fmaf(b.w, fi, b.z), fi, b.y), fi, b.x);
}

// Momentum derivatives K = F_target(X) - F_laser(t) and the phase rate
// (HydrogenLikeAtom.jl:78-159, SAEAtom.jl:278-366); x . F_target = coef r^2.
template <int DIM, int PHASE, int TGT>
__device__ __forceinline__ void accel(const BulkParams& P, const float4* __restrict__ tab, int ni, float fi,
                                      const float* X, const float* Pm, float* K, float& kph) {
    float Fx, Fy;
    field(tab, P.n_int, ni, fi, Fx, Fy);
    const float r2 = (DIM == 3) ? fmaf(X[0], X[0], fmaf(X[1], X[1], X[2] * X[2])) : fmaf(X[0], X[0], X[1] * X[1]);
    float coef, V = 0.0f;
    if (TGT == ETRAJ_TARGET_HYDROGEN_LIKE) {
        const float ri = rsqrt_nr(r2 + P.sc);
        coef = -P.Z * (ri * ri * ri);
        V = P.Z * ri;
    } else {
        const float r = r2 * rsqrt_nr(fmaxf(r2, 1e-30f));
        const float ris = rsqrt_nr(r2 + P.sc);
        const float e1 = __expf(-P.b1 * r), e2 = __expf(-P.b2 * r), e3 = __expf(-P.b3 * r);
        const float br = fmaf(P.a3 * fmaf(P.b3, r, 1.0f), e3, fmaf(P.a1 * fmaf(P.b1, r, 1.0f), e1, P.Z));
        coef = -fmaf(ris * ris * ris, br, P.a2b2 * ris * e2);
        if (PHASE != ETRAJ_PHASE_CTMC) {
            const float num = fmaf(P.a3, e3, fmaf(P.a2 * r, e2, fmaf(P.a1, e1, P.Z)));
            // the 2D SCTS reference divides by r^2+sc, not its square root (SAEAtom.jl:316)
            V = (DIM == 2 && PHASE == ETRAJ_PHASE_SCTS) ? num * (ris * ris) : num * ris;
        }
    }
    K[0] = fmaf(coef, X[0], -Fx);
    K[1] = fmaf(coef, X[1], -Fy);
    if (DIM == 3) K[2] = coef * X[2];
    if (PHASE != ETRAJ_PHASE_CTMC) {
        const float KE = 0.5f * ((DIM == 3) ? fmaf(Pm[0], Pm[0], fmaf(Pm[1], Pm[1], Pm[2] * Pm[2]))
                                            : fmaf(Pm[0], Pm[0], Pm[1] * Pm[1]));
        kph = (PHASE == ETRAJ_PHASE_QTMC) ? -((P.Ip + KE) - V) : -((KE - V) + coef * r2);
    } else {
        kph = 0.0f;
    }
}

__device__ __forceinline__ void advance(int n, float f, float dth, int& no, float& fo) {
    float g = f + dth;
    float fl = floorf(g);
    no = n + (int)fl;
    fo = g - fl;
}

template <int DIM, int PHASE, int TGT>
__global__ void __launch_bounds__(256, 2)
k_integrate_bulk(const __grid_constant__ BulkParams P, InitSoA soa, const double* __restrict__ tsamp,
                 const int64_t* __restrict__ idx, const unsigned long long* __restrict__ count,
                 unsigned long long* __restrict__ queue, TrajOut out) {
    constexpr bool HASPH = (PHASE != ETRAJ_PHASE_CTMC);
    constexpr int N = 2 * DIM + (HASPH ? 1 : 0);
    extern __shared__ float4 s_tab[];
    const float4* tab = P.table;
    if (P.table_in_smem) {
        for (int i = threadIdx.x; i < 2 * P.n_int; i += blockDim.x) s_tab[i] = P.table[i];
        __syncthreads();
        tab = s_tab;
    }
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned lt_mask = (1u << lane) - 1u;
    const unsigned long long n_traj = *count;

    // state (hi, lo): x[DIM], p[DIM], phase
    float xh[DIM], xl[DIM], ph[DIM], pl[DIM], fh = 0.0f, flo = 0.0f;
    float K1[DIM], kph1 = 0.0f;  // FSAL derivatives
    int tn = 0, iter = 0, attempts = 0;
    float tfr = 0.0f, dth = 0.0f, dthp = 0.0f, dthmax = 0.0f, qold = QOLDINIT, q11 = 1.0f;
    bool accept = false, active = false, need = true;
    unsigned long long s = 0;

    while (true) {
        // ---- work stealing: refill free lanes from the queue -----------------------
        const unsigned needm = __ballot_sync(FULL, need);
        const unsigned actm = __ballot_sync(FULL, active);
        if (needm && (__popc(needm) >= P.refill_min || actm == 0u)) {
            const int leader = __ffs(needm) - 1;
            unsigned long long base = 0ull;
            if (lane == leader) base = atomicAdd(queue, (unsigned long long)__popc(needm));
            base = __shfl_sync(FULL, base, leader);
            if (need) {
                need = false;
                s = base + __popc(needm & lt_mask);
                if (s < n_traj) {
                    // load the electron and pick the first step (Hairer's starting step)
                    const int64_t g = idx ? idx[s] : (int64_t)s;
                    double u0x[DIM], u0p[DIM];
                    u0x[0] = soa.x[g];
                    u0x[1] = soa.y[g];
                    if (DIM == 3) u0x[2] = 0.0;
                    u0p[0] = soa.kx[g];
                    u0p[1] = soa.ky[g];
                    if (DIM == 3) u0p[2] = soa.kz[g];
#pragma unroll
                    for (int d = 0; d < DIM; ++d) {
                        xh[d] = (float)u0x[d];
                        xl[d] = (float)(u0x[d] - (double)xh[d]);
                        ph[d] = (float)u0p[d];
                        pl[d] = (float)(u0p[d] - (double)ph[d]);
                    }
                    if (HASPH) {
                        const double f0 = soa.phase[g];
                        fh = (float)f0;
                        flo = (float)(f0 - (double)fh);
                    }
                    const double t0 = tsamp[soa.batch[g]];
                    const double q0 = (t0 - P.T0) * P.inv_h_d;
                    const double fl = floor(q0);
                    tn = (int)fl;
                    tfr = (float)(q0 - fl);
                    dthmax = (float)((P.t_final - t0) * P.inv_h_d);
                    accel<DIM, PHASE, TGT>(P, tab, tn, tfr, xh, ph, K1, kph1);
                    // d0 = |u0/sk|, d1 = |f0/sk| (f0 = (p, K, phase rate))
                    float skx[DIM], skp[DIM], skf = 0.0f, a0 = 0.0f, a1 = 0.0f;
#pragma unroll
                    for (int d = 0; d < DIM; ++d) {
                        skx[d] = fmaf(fabsf(xh[d]), P.rtol, ABSTOL);
                        skp[d] = fmaf(fabsf(ph[d]), P.rtol, ABSTOL);
                        float q = xh[d] / skx[d], r = ph[d] / skp[d];
                        a0 = fmaf(q, q, fmaf(r, r, a0));
                        q = ph[d] / skx[d];
                        r = K1[d] / skp[d];
                        a1 = fmaf(q, q, fmaf(r, r, a1));
                    }
                    if (HASPH) {
                        skf = fmaf(fabsf(fh), P.rtol, ABSTOL);
                        const float q = fh / skf, r = kph1 / skf;
                        a0 = fmaf(q, q, a0);
                        a1 = fmaf(r, r, a1);
                    }
                    const float d0 = sqrtf(a0 * (1.0f / N)), d1 = sqrtf(a1 * (1.0f / N));
                    float dt0 = (d0 < 1e-5f || d1 < 1e-5f) ? 1e-6f : (d0 / d1) * 0.01f;
                    dt0 = fminf(dt0, dthmax * P.h);
                    // f1 at u1 = u0 + dt0 f0; f1 - f0 for the position rows is dt0 K exactly
                    float X1[DIM], P1[DIM], K1b[DIM], kph1b;
#pragma unroll
                    for (int d = 0; d < DIM; ++d) {
                        X1[d] = fmaf(dt0, ph[d], xh[d]);
                        P1[d] = fmaf(dt0, K1[d], ph[d]);
                    }
                    int n1;
                    float f1r;
                    advance(tn, tfr, dt0 * P.inv_h, n1, f1r);
                    accel<DIM, PHASE, TGT>(P, tab, n1, f1r, X1, P1, K1b, kph1b);
                    float a2 = 0.0f;
#pragma unroll
                    for (int d = 0; d < DIM; ++d) {
                        const float q = (dt0 * K1[d]) / skx[d], r = (K1b[d] - K1[d]) / skp[d];
                        a2 = fmaf(q, q, fmaf(r, r, a2));
                    }
                    if (HASPH) {
                        const float r = (kph1b - kph1) / skf;
                        a2 = fmaf(r, r, a2);
                    }
                    const float d2 = sqrtf(a2 * (1.0f / N)) / dt0;
                    const float md = fmaxf(d1, d2);
                    const float dt1 = (md <= 1e-15f) ? fmaxf(1e-6f, dt0 * 1e-3f)
                                                     : exp2f(-(2.0f + log10f(md)) * (3.321928094887362f / 5.0f));
                    dth = fminf(fminf(100.0f * dt0, dt1), dthmax * P.h) * P.inv_h;
                    dthp = dth;
                    qold = QOLDINIT;
                    q11 = 1.0f;
                    accept = false;
                    iter = 0;
                    attempts = 0;
                    active = true;
                }
            }
        }
        if (__ballot_sync(FULL, active) == 0u) break;
        if (active) {
            // ---- one Tsit5 step attempt (lanes without work idle; every lane returns to
            //      the ballots above, so the *_sync calls always see the full warp) -----------
            if (iter > 0) {
                if (!accept) dth = dth / fminf(QMIN_INV, q11 / GAMMA);
                else dth = dthp;
            }
            ++iter;
            dth = fminf(dth, dthmax);
            const float remaining = (float)(P.nf - tn) + (P.ff - tfr);
            const bool last = dth >= remaining;
            if (last) dth = remaining;
            int status = 0;
            if (!(dth == dth)) status = 4;
            else if (iter > MAXITERS) status = 1;
            else if (dth < kDthMin && !last) status = 2;
            if (status == 0) {
                const float dt = dth * P.h, dt2 = dt * dt;
                float K[7][DIM], kph[7], X[DIM], Pm[DIM];
                int n1 = 0;
                float f1 = 0.0f;
                if (last) {
                    n1 = P.nf;
                    f1 = P.ff;
                } else {
                    advance(tn, tfr, dth, n1, f1);
                }
#pragma unroll
                for (int d = 0; d < DIM; ++d) K[0][d] = K1[d];
                kph[0] = kph1;
#pragma unroll
                for (int st = 1; st < 7; ++st) {
#pragma unroll
                    for (int d = 0; d < DIM; ++d) {
                        float ap = 0.0f, aq = 0.0f;
#pragma unroll
                        for (int l = 0; l < st; ++l) {
                            ap = fmaf(cA[st][l], K[l][d], ap);
                            aq = fmaf(cAA[st][l], K[l][d], aq);
                        }
                        Pm[d] = fmaf(dt, ap, ph[d]);
                        X[d] = fmaf(dt2, aq, fmaf(cC[st] * dt, ph[d], xh[d]));
                    }
                    int ni = n1;
                    float fi = f1;
                    if (st < 5) advance(tn, tfr, cC[st] * dth, ni, fi);
                    accel<DIM, PHASE, TGT>(P, tab, ni, fi, X, Pm, K[st], kph[st]);
                }
                // X, Pm now hold the new position and momentum (stage 7 = solution)
                float incf = 0.0f, phnew = 0.0f;
                if (HASPH) {
                    float a = 0.0f;
#pragma unroll
                    for (int l = 0; l < 6; ++l) a = fmaf(cA[6][l], kph[l], a);
                    incf = dt * a;
                    phnew = fh + incf;
                }
                float acc = 0.0f;
#pragma unroll
                for (int d = 0; d < DIM; ++d) {
                    float ex = 0.0f, ep = 0.0f;
#pragma unroll
                    for (int l = 0; l < 7; ++l) {
                        ex = fmaf(cBTA[l], K[l][d], ex);
                        ep = fmaf(cBT[l], K[l][d], ep);
                    }
                    const float scx = fmaf(fmaxf(fabsf(xh[d]), fabsf(X[d])), P.rtol, ABSTOL);
                    const float scp = fmaf(fmaxf(fabsf(ph[d]), fabsf(Pm[d])), P.rtol, ABSTOL);
                    const float rx = (dt2 * ex) / scx, rp = (dt * ep) / scp;
                    acc = fmaf(rx, rx, fmaf(rp, rp, acc));
                }
                if (HASPH) {
                    float ef = 0.0f;
#pragma unroll
                    for (int l = 0; l < 7; ++l) ef = fmaf(cBT[l], kph[l], ef);
                    const float scf = fmaf(fmaxf(fabsf(fh), fabsf(phnew)), P.rtol, ABSTOL);
                    const float rf = (dt * ef) / scf;
                    acc = fmaf(rf, rf, acc);
                }
                const float EEst = sqrtf(acc * (1.0f / N));
                ++attempts;
                float q;
                if (EEst == 0.0f) {
                    q = QMAX_INV;
                } else {
                    q11 = exp2f(BETA1 * __log2f(EEst));
                    q = q11 * exp2f(-BETA2 * __log2f(qold));
                    q = fmaxf(QMAX_INV, fminf(QMIN_INV, q / GAMMA));
                }
                accept = (EEst <= 1.0f);
                if (!(EEst == EEst)) status = 4;
                if (accept && status == 0) {
                    qold = fmaxf(EEst, QOLDINIT);
                    dthp = fminf(dthmax, dth / q);
#pragma unroll
                    for (int d = 0; d < DIM; ++d) {
                        float a = 0.0f, b = 0.0f;
#pragma unroll
                        for (int l = 0; l < 6; ++l) {
                            a = fmaf(cAA[6][l], K[l][d], a);
                            b = fmaf(cA[6][l], K[l][d], b);
                        }
                        df_add(xh[d], xl[d], fmaf(dt, ph[d], fmaf(dt, pl[d], dt2 * a)));
                        df_add(ph[d], pl[d], dt * b);
                        K1[d] = K[6][d];
                    }
                    if (HASPH) df_add(fh, flo, incf);
                    kph1 = kph[6];
                    tn = n1;
                    tfr = f1;
                    if (last) {
                        status = -1;  // reached t_final
                    } else {
                        bool bad = false;
#pragma unroll
                        for (int d = 0; d < DIM; ++d) bad |= !(xh[d] == xh[d]) || !(ph[d] == ph[d]);
                        if (bad) status = 3;
                    }
                }
            }
            if (status != 0) {
                // finished (status -1 = Success) or failed: write the FP64 state and free the lane
                const int code = (status < 0) ? 0 : status;
                out.status[s] = code;
                out.steps[s] = attempts;
                double* fs = out.final_state + s * N;
#pragma unroll
                for (int d = 0; d < DIM; ++d) {
                    fs[d] = (double)xh[d] + (double)xl[d];
                    fs[DIM + d] = (double)ph[d] + (double)pl[d];
                }
                if (HASPH) fs[2 * DIM] = (double)fh + (double)flo;
                active = false;
                need = true;
            }
        }  // active
    }
}

__global__ void k_field_table(const __grid_constant__ DJob J, double T0, double h, int n_int,
                              float4* __restrict__ tab) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_int) return;
    const double ta = T0 + (double)k * h, tb = T0 + (double)(k + 1) * h;
    double fxa, fya, dfxa, dfya, fxb, fyb, dfxb, dfyb;
    laser_F_dual(J.laser, ta, fxa, fya, dfxa, dfya);
    laser_F_dual(J.laser, tb, fxb, fyb, dfxb, dfyb);
    auto herm = [h](double fa, double fb, double da, double db) {
        const double ma = h * da, mb = h * db;
        return make_float4((float)fa, (float)ma, (float)(3.0 * (fb - fa) - 2.0 * ma - mb),
                           (float)(2.0 * (fa - fb) + ma + mb));
    };
    tab[2 * k] = herm(fxa, fxb, dfxa, dfxb);
    tab[2 * k + 1] = herm(fya, fyb, dfya, dfyb);
}

template <int DIM, int PHASE, int TGT>
int launch_bulk_t(const BulkParams& P, InitSoA soa, const double* t, const int64_t* idx,
                  const unsigned long long* count, unsigned long long* queue, TrajOut out, int sm_count,
                  cudaStream_t s) {
    const size_t smem = P.table_in_smem ? (size_t)P.n_int * 2 * sizeof(float4) : 0;
    auto kern = k_integrate_bulk<DIM, PHASE, TGT>;
    if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const int blocks = sm_count * P.blocks_per_sm;
    kern<<<blocks, P.threads, smem, s>>>(P, soa, t, idx, count, queue, out);
    return 1;
}

}  // namespace

int launch_field_table(const DJob& J, double T0, double h, int n_int, float4* tab, cudaStream_t s) {
    k_field_table<<<(n_int + 127) / 128, 128, 0, s>>>(J, T0, h, n_int, tab);
    return 1;
}

int launch_integrate_bulk(const BulkParams& P, InitSoA soa, const double* t, const int64_t* idx,
                          const unsigned long long* count, unsigned long long* queue, TrajOut out,
                          int sm_count, cudaStream_t s) {
#define ETRAJ_BULK_TGT(D, PH)                                                                       \
    return (P.tgt == ETRAJ_TARGET_HYDROGEN_LIKE)                                                    \
               ? launch_bulk_t<D, PH, ETRAJ_TARGET_HYDROGEN_LIKE>(P, soa, t, idx, count, queue, out, \
                                                                  sm_count, s)                      \
               : launch_bulk_t<D, PH, ETRAJ_TARGET_SAE>(P, soa, t, idx, count, queue, out, sm_count, s);
    if (P.dim == 2) {
        if (P.phase == ETRAJ_PHASE_CTMC) { ETRAJ_BULK_TGT(2, ETRAJ_PHASE_CTMC) }
        if (P.phase == ETRAJ_PHASE_QTMC) { ETRAJ_BULK_TGT(2, ETRAJ_PHASE_QTMC) }
        ETRAJ_BULK_TGT(2, ETRAJ_PHASE_SCTS)
    } else {
        if (P.phase == ETRAJ_PHASE_CTMC) { ETRAJ_BULK_TGT(3, ETRAJ_PHASE_CTMC) }
        if (P.phase == ETRAJ_PHASE_QTMC) { ETRAJ_BULK_TGT(3, ETRAJ_PHASE_QTMC) }
        ETRAJ_BULK_TGT(3, ETRAJ_PHASE_SCTS)
    }
#undef ETRAJ_BULK_TGT
}

}  // namespace etraj
