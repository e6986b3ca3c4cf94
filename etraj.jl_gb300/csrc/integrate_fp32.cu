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
//  * Noise-aware error estimate.  Each FP32 stage value carries ~1 ulp of
//    the magnitude of the terms summed into it; the error sums cancel those
//    values to ~dt^5, so the estimate is taken less a bound on that noise
//    (2 ulp x the sum of |weights|).  Without it, EEst would not fall below
//    ~1e-5 and a trajectory starting with a tiny step would grow it by ~2x per
//    step instead of 10x: 15-20% more steps than the FP64 path for the same
//    tolerance.  Near EEst ~ 1 the bound is ~1e-5 of the tolerance.
//  * Compensated state.  Positions, momenta and the QTMC/SCTS phase are
//    double-float pairs (hi + lo, Knuth's TwoSum), so 1e3 steps add no
//    rounding drift; stage values and the error estimate are plain FP32.
//  * Work stealing.  One lane owns one trajectory; when it finishes, the lane
//    takes the next one from a global queue (warp-aggregated atomicAdd), so
//    step counts that differ 100x between trajectories do not idle the warp.
//    `refill_min` lanes must be free before a warp refills (autotuned).
//
// The kernel writes the final state in FP64 (hi + lo); k_collect_bulk then
// computes the Kepler asymptote, SCTS correction and deposit contribution of
// every electron in FP32 (the phase sum and its reduction in FP64).
//
// Roofline: FP32 issue bound, MUFU for rsqrt/exp2/log2; no tensor cores.

#include <climits>

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
constexpr double cabs_(double x) { return x < 0 ? -x : x; }
constexpr double sum_abs_bt() {
    double s = 0.0;
    for (int l = 0; l < 7; ++l) s += cabs_(kBT[l]);
    return s;
}
constexpr double sum_abs_bta() {
    double s = 0.0;
    for (int l = 0; l < 7; ++l) s += cabs_(bta(l));
    return s;
}
// Rounding-noise bound of one FP32 stage value of magnitude M: 2 M 2^-24.
constexpr float kNoiseUlp = 1.1920928955078125e-7f;
constexpr float kSumAbsBT = (float)sum_abs_bt(), kSumAbsBTA = (float)sum_abs_bta();

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
                INV_GAMMA = 1.0f / 0.9f, LOG2_QOLDINIT = -13.287712379549449f;  // log2(1e-4)
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
// (HydrogenLikeAtom.jl:78-159, SAEAtom.jl:98-186); x . F_target = coef r^2.
// mK and mph are the magnitudes of the terms summed into K and the phase rate
// (for the rounding-noise bound of the error estimate; unused outputs of the
// inlined call are removed by the compiler).
template <int DIM, int PHASE, int TGT>
__device__ __forceinline__ void accel(const BulkParams& P, const float4* __restrict__ tab, int n_int, int ni,
                                      float fi, const float* X, const float* Pm, float* K, float& kph, float& mK,
                                      float& mph) {
    float Fx, Fy;
    field(tab, n_int, ni, fi, Fx, Fy);
    const float r2 = (DIM == 3) ? fmaf(X[0], X[0], fmaf(X[1], X[1], X[2] * X[2])) : fmaf(X[0], X[0], X[1] * X[1]);
    float coef, V = 0.0f;
    if (TGT == ETRAJ_TARGET_HYDROGEN_LIKE) {
        const float ri = rsqrt_nr(r2 + P.sc);
        coef = -P.Z * (ri * ri * ri);
        V = P.Z * ri;
    } else {
        const float r = r2 * rsqrt_nr(fmaxf(r2, 1e-30f));
        const float ris = rsqrt_nr(r2 + P.sc);
        // Beyond r_far (host: every exp(-b r) term below 2^-26 of the sum it
        // joins) each lane takes its exponentials as exactly 0.  fmaf(x, 0, y) is
        // y, so when all active lanes are that far the short form below gives
        // the same bits as the full one: a lane's result never depends on which
        // electrons share its warp.
        const bool far = r > P.r_far;
        float br, num;
        if (__all_sync(__activemask(), far)) {
            br = P.Z;
            coef = -((ris * ris * ris) * br);
            num = P.Z;
        } else {
            float e1 = 0.0f, e2 = 0.0f, e3 = 0.0f;
            if (!far) {
                e1 = __expf(-P.b1 * r);
                e2 = __expf(-P.b2 * r);
                e3 = __expf(-P.b3 * r);
            }
            br = fmaf(P.a3 * fmaf(P.b3, r, 1.0f), e3, fmaf(P.a1 * fmaf(P.b1, r, 1.0f), e1, P.Z));
            coef = -fmaf(ris * ris * ris, br, P.a2b2 * ris * e2);
            num = fmaf(P.a3, e3, fmaf(P.a2 * r, e2, fmaf(P.a1, e1, P.Z)));
        }
        if (PHASE != ETRAJ_PHASE_CTMC) {
            // the 2D SCTS reference divides by r^2+sc, not its square root (SAEAtom.jl:136)
            V = (DIM == 2 && PHASE == ETRAJ_PHASE_SCTS) ? num * (ris * ris) : num * ris;
        }
    }
    K[0] = fmaf(coef, X[0], -Fx);
    K[1] = fmaf(coef, X[1], -Fy);
    if (DIM == 3) K[2] = coef * X[2];
    const float ax = fmaxf(fabsf(X[0]), fabsf(X[1]));
    mK = fmaf(fabsf(coef), (DIM == 3) ? fmaxf(ax, fabsf(X[2])) : ax, fmaxf(fabsf(Fx), fabsf(Fy)));
    if (PHASE != ETRAJ_PHASE_CTMC) {
        const float KE = 0.5f * ((DIM == 3) ? fmaf(Pm[0], Pm[0], fmaf(Pm[1], Pm[1], Pm[2] * Pm[2]))
                                            : fmaf(Pm[0], Pm[0], Pm[1] * Pm[1]));
        kph = (PHASE == ETRAJ_PHASE_QTMC) ? -((P.Ip + KE) - V) : -((KE - V) + coef * r2);
        mph = (P.Ip + KE) + fabsf(V) + ((PHASE == ETRAJ_PHASE_SCTS) ? fabsf(coef * r2) : 0.0f);
    } else {
        kph = 0.0f;
        mph = 0.0f;
    }
}

// Fixed-point clock: t = T0 + h (n + f), 0 <= f < 1.  Adding kMagic = 1.5 * 2^23
// with round-down leaves floor(g) in the low mantissa bits for 0 <= g < 2^22
// (the host keeps every job below 2^21 intervals), so the split costs two FP32
// adds and an integer subtract instead of floor and float-int conversions.
constexpr float kMagic = 12582912.0f;
__device__ __forceinline__ void advance(int n, float f, float dth, int& no, float& fo) {
    const float g = f + dth;
    const float r = __fadd_rd(g, kMagic);
    no = n + (__float_as_int(r) - __float_as_int(kMagic));
    fo = g - (r - kMagic);  // exact: g and floor(g) are within a factor of 2, or floor(g) = 0
}
// (float)k for 0 <= k < 2^22, without a conversion instruction
__device__ __forceinline__ float small_int_to_float(int k) {
    return __int_as_float(__float_as_int(kMagic) + k) - kMagic;
}

// MULTI: one launch over the electrons of P.n_inst instances (different
// lasers, same target, dimension, phase and tolerance).  Each lane finds its
// electron's instance when it loads it (binary search of the candidate index
// over the instances' ranges, held in shared memory) and reads that instance's
// table and clock there, so one warp may integrate electrons of several
// instances at once: the work stealing spans all of them.
// OCC: resident 256-thread blocks per SM the build is held to (2: <= 128
// registers per thread, 16 warps per SM; 3: <= 85 registers, 24 warps).
template <int DIM, int PHASE, int TGT, bool MULTI, int OCC>
__global__ void __launch_bounds__(256, OCC)
k_integrate_bulk(const __grid_constant__ BulkParams P, InitSoA soa, const double* __restrict__ tsamp,
                 const int64_t* __restrict__ idx, const unsigned long long* __restrict__ count,
                 unsigned long long* __restrict__ queue, TrajOut out) {
    constexpr bool HASPH = (PHASE != ETRAJ_PHASE_CTMC);
    constexpr int N = 2 * DIM + (HASPH ? 1 : 0);
    extern __shared__ float4 s_tab[];
    __shared__ BulkInst s_inst[MULTI ? kMaxInstances : 1];
    // a resume round launches a full grid; blocks past the parked electrons exit
    // at once, so a job's later rounds hold only the SMs their electrons need
    if (P.park_in && (unsigned long long)blockIdx.x * blockDim.x >=
                         min(*P.park_in_count, (unsigned long long)P.park_cap))
        return;
    const float4* tab = P.table;
    if (MULTI) {
        for (int i = threadIdx.x; i < P.n_inst; i += blockDim.x) s_inst[i] = P.inst[i];
        __syncthreads();
    } else if (P.table_in_smem) {
        for (int i = threadIdx.x; i < 2 * P.n_int; i += blockDim.x) s_tab[i] = P.table[i];
        __syncthreads();
        tab = s_tab;
    }
    int my = 0;  // the lane's instance (MULTI)
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned lt_mask = (1u << lane) - 1u;
    const bool resume = (P.park_in != nullptr);
    const unsigned long long n_traj = resume ? min(*P.park_in_count, (unsigned long long)P.park_cap) : *count;

    // state (hi, lo): x[DIM], p[DIM], phase
    float xh[DIM], xl[DIM], ph[DIM], pl[DIM], fh = 0.0f, flo = 0.0f;
    float K1[DIM], kph1 = 0.0f;  // FSAL derivatives
    float mK1 = 0.0f, mph1 = 0.0f;  // and their term magnitudes
    int tn = 0, iter = 0, attempts = 0, rs = 0;  // rs: step attempts in this round
    bool drained = false;                         // the queue was found empty
    bool taken = false;                           // static assignment: the lane's electron was taken
    float tfr = 0.0f, dth = 0.0f, dthp = 0.0f, dthmax = 0.0f, lqold = LOG2_QOLDINIT, q11 = 1.0f;
    bool accept = false, active = false, need = true;
    unsigned long long s = 0;

    while (true) {
        // ---- work stealing: refill free lanes from the queue -----------------------
        const unsigned needm = __ballot_sync(FULL, need);
        const unsigned actm = __ballot_sync(FULL, active);
        if (needm && (__popc(needm) >= P.refill_min || actm == 0u)) {
            const int leader = __ffs(needm) - 1;
            unsigned long long base = 0ull;
            if (P.static_assign) {
                // electron blockIdx.x * blockDim.x + threadIdx.x, then nothing more
                base = taken ? n_traj : (unsigned long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31u);
                taken = true;
            } else {
                if (lane == leader) base = atomicAdd(queue, (unsigned long long)__popc(needm));
                base = __shfl_sync(FULL, base, leader);
            }
            drained = drained || (base + (unsigned long long)__popc(needm) > n_traj);
            if (need) {
                need = false;
                s = base + __popc(needm & lt_mask);
                rs = 0;
                if (s < n_traj && resume) {
                    // a parked electron: its whole state, in the order the parking wrote it
                    const uint32_t* b = P.park_in + s;
                    const size_t cs = (size_t)P.park_cap;
                    int k = 0;
                    auto gf = [&]() { return __uint_as_float(b[cs * (size_t)(k++)]); };
                    auto gi = [&]() { return (int)b[cs * (size_t)(k++)]; };
                    const unsigned long long lo = (unsigned)gi(), hi = (unsigned)gi();
                    s = lo | (hi << 32);
#pragma unroll
                    for (int d = 0; d < DIM; ++d) {
                        xh[d] = gf();
                        xl[d] = gf();
                        ph[d] = gf();
                        pl[d] = gf();
                        K1[d] = gf();
                    }
                    fh = gf();
                    flo = gf();
                    kph1 = gf();
                    mK1 = gf();
                    mph1 = gf();
                    tn = gi();
                    iter = gi();
                    attempts = gi();
                    tfr = gf();
                    dth = gf();
                    dthp = gf();
                    dthmax = gf();
                    lqold = gf();
                    q11 = gf();
                    accept = gi() != 0;
                    my = gi();
                    active = true;
                } else if (s < n_traj) {
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
                    double T0 = P.T0, inv_h_d = P.inv_h_d, t_final = P.t_final;
                    int toff = 0;
                    if (MULTI) {
                        int lo = 0, hi = P.n_inst - 1;
                        while (lo < hi) {
                            const int mid = (lo + hi) >> 1;
                            if (g < s_inst[mid].cand_end) hi = mid;
                            else lo = mid + 1;
                        }
                        my = lo;
                        T0 = s_inst[my].T0;
                        inv_h_d = s_inst[my].inv_h_d;
                        t_final = s_inst[my].t_final;
                        toff = s_inst[my].t_off;
                    }
                    const float4* tabi = MULTI ? s_inst[my].table : tab;
                    const int nint = MULTI ? s_inst[my].n_int : P.n_int;
                    const float hh = MULTI ? s_inst[my].h : P.h, ihh = MULTI ? s_inst[my].inv_h : P.inv_h;
                    const double t0 = tsamp[toff + soa.batch[g]];
                    const double q0 = (t0 - T0) * inv_h_d;
                    const double fl = floor(q0);
                    tn = (int)fl;
                    tfr = (float)(q0 - fl);
                    dthmax = (float)((t_final - t0) * inv_h_d);
                    accel<DIM, PHASE, TGT>(P, tabi, nint, tn, tfr, xh, ph, K1, kph1, mK1, mph1);
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
                    dt0 = fminf(dt0, dthmax * hh);
                    // f1 at u1 = u0 + dt0 f0; f1 - f0 for the position rows is dt0 K exactly
                    float X1[DIM], P1[DIM], K1b[DIM], kph1b;
#pragma unroll
                    for (int d = 0; d < DIM; ++d) {
                        X1[d] = fmaf(dt0, ph[d], xh[d]);
                        P1[d] = fmaf(dt0, K1[d], ph[d]);
                    }
                    int n1;
                    float f1r;
                    advance(tn, tfr, dt0 * ihh, n1, f1r);
                    float unused_m, unused_p;
                    accel<DIM, PHASE, TGT>(P, tabi, nint, n1, f1r, X1, P1, K1b, kph1b, unused_m, unused_p);
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
                    dth = fminf(fminf(100.0f * dt0, dt1), dthmax * hh) * ihh;
                    dthp = dth;
                    lqold = LOG2_QOLDINIT;
                    q11 = 1.0f;
                    accept = false;
                    iter = 0;
                    attempts = 0;
                    active = true;
                }
            }
        }
        if (__ballot_sync(FULL, active) == 0u) break;
        if (P.park_out) {
            // park the electrons that used up this round's step budget, once the
            // queue is empty: while it holds work they keep their lanes, so they
            // overlap the rest of the job instead of waiting for the next round
            bool want = active && rs >= P.park_budget;
            if (__any_sync(FULL, want) && !drained) {
                unsigned long long q = 0ull;
                if (lane == 0) q = atomicAdd(queue, 0ull);
                drained = __shfl_sync(FULL, q, 0) >= n_traj;
            }
            want = want && drained;
            const unsigned pm = __ballot_sync(FULL, want);
            if (pm) {
                const int leader = __ffs(pm) - 1;
                unsigned long long base = 0ull;
                if (lane == leader) base = atomicAdd(P.park_out_count, (unsigned long long)__popc(pm));
                base = __shfl_sync(FULL, base, leader);
                const unsigned long long e = base + __popc(pm & lt_mask);
                if (want && e < (unsigned long long)P.park_cap) {
                    uint32_t* b = P.park_out + e;
                    const size_t cs = (size_t)P.park_cap;
                    int k = 0;
                    auto pf = [&](float v) { b[cs * (size_t)(k++)] = __float_as_uint(v); };
                    auto pi = [&](int v) { b[cs * (size_t)(k++)] = (uint32_t)v; };
                    pi((int)(uint32_t)s);
                    pi((int)(uint32_t)(s >> 32));
#pragma unroll
                    for (int d = 0; d < DIM; ++d) {
                        pf(xh[d]);
                        pf(xl[d]);
                        pf(ph[d]);
                        pf(pl[d]);
                        pf(K1[d]);
                    }
                    pf(fh);
                    pf(flo);
                    pf(kph1);
                    pf(mK1);
                    pf(mph1);
                    pi(tn);
                    pi(iter);
                    pi(attempts);
                    pf(tfr);
                    pf(dth);
                    pf(dthp);
                    pf(dthmax);
                    pf(lqold);
                    pf(q11);
                    pi(accept ? 1 : 0);
                    pi(my);
                    active = false;
                    need = true;  // the lane takes the next queued electron
                } else if (want) {
                    rs = INT_MIN;  // park buffer full: finish the electron in this round
                }
                if (__ballot_sync(FULL, active) == 0u) continue;
            }
        }
        if (active) {
            // ---- one Tsit5 step attempt (lanes without work idle; every lane returns to
            //      the ballots above, so the *_sync calls always see the full warp) -----------
            if (iter > 0) {
                if (!accept) dth = __fdividef(dth, fminf(QMIN_INV, q11 * INV_GAMMA));
                else dth = dthp;
            }
            ++iter;
            dth = fminf(dth, dthmax);
            const float4* tabi = MULTI ? s_inst[my].table : tab;
            const int nint = MULTI ? s_inst[my].n_int : P.n_int;
            const int nfi = MULTI ? s_inst[my].nf : P.nf;
            const float ffi = MULTI ? s_inst[my].ff : P.ff;
            const float hh = MULTI ? s_inst[my].h : P.h;
            const float remaining = small_int_to_float(nfi - tn) + (ffi - tfr);
            const bool last = dth >= remaining;
            if (last) dth = remaining;
            int status = 0;
            if (!(dth == dth)) status = 4;
            else if (iter > P.max_iters) status = 1;
            else if (dth < kDthMin && !last) status = 2;
            if (status == 0) {
                const float dt = dth * hh, dt2 = dt * dt;
                float K[7][DIM], kph[7], X[DIM], Pm[DIM], mK7 = 0.0f, mph7 = 0.0f;
                int n1 = 0;
                float f1 = 0.0f;
                if (last) {
                    n1 = nfi;
                    f1 = ffi;
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
                    accel<DIM, PHASE, TGT>(P, tabi, nint, ni, fi, X, Pm, K[st], kph[st], mK7, mph7);
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
                // Error estimate less its own FP32 rounding noise: the weighted sums
                // below cancel to ~dt^5 while each stage value carries ~1 ulp of the
                // magnitude of its terms, which would otherwise put a floor of
                // ~1e-5 under EEst and hold the step growth of well-resolved
                // trajectories to ~2x per step instead of the controller's 10x.
                const float mk = fmaxf(mK1, mK7) * kNoiseUlp;
                const float nx = dt2 * kSumAbsBTA * mk, np = dt * kSumAbsBT * mk;
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
                    const float rx = __fdividef(fmaxf(fabsf(dt2 * ex) - nx, 0.0f), scx);
                    const float rp = __fdividef(fmaxf(fabsf(dt * ep) - np, 0.0f), scp);
                    acc = fmaf(rx, rx, fmaf(rp, rp, acc));
                }
                if (HASPH) {
                    float ef = 0.0f;
#pragma unroll
                    for (int l = 0; l < 7; ++l) ef = fmaf(cBT[l], kph[l], ef);
                    const float scf = fmaf(fmaxf(fabsf(fh), fabsf(phnew)), P.rtol, ABSTOL);
                    const float nf = dt * kSumAbsBT * (fmaxf(mph1, mph7) * kNoiseUlp);
                    const float rf = __fdividef(fmaxf(fabsf(dt * ef) - nf, 0.0f), scf);
                    acc = fmaf(rf, rf, acc);
                }
                // EEst^2 and half its log2: the controller needs only powers of EEst
                const float ms = acc * (1.0f / N);
                const float lh = 0.5f * __log2f(ms);  // log2 EEst
                ++attempts;
                ++rs;
                float q;
                if (ms == 0.0f) {
                    q = QMAX_INV;
                } else {
                    q11 = exp2f(BETA1 * lh);
                    q = q11 * exp2f(-BETA2 * lqold);
                    q = fmaxf(QMAX_INV, fminf(QMIN_INV, q * INV_GAMMA));
                }
                accept = (ms <= 1.0f);
                if (!(ms == ms)) status = 4;
                if (accept && status == 0) {
                    lqold = fmaxf(lh, LOG2_QOLDINIT);
                    dthp = fminf(dthmax, __fdividef(dth, q));
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
                    mK1 = mK7;
                    mph1 = mph7;
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

// FP32 collection of the bulk path's final states (TrajectorySimulation.jl:356-393,
// 3D :451-493): the same Kepler asymptote, SCTS phase correction, binning and
// contributions as collect() in integrate_fp64.cu, in FP32 except for the phase
// sum and its reduction mod 2 pi (FP64, a few operations per electron), so the
// absolute phase error stays ~1e-6 rad for phases of 1e3 rad.  A separate
// kernel rather than an epilogue of k_integrate_bulk: there, each finishing
// lane would stall its warp for the whole collection.
template <int DIM, int PHASE>
__global__ void __launch_bounds__(256)
k_collect_bulk(const __grid_constant__ DJob J, InitSoA soa, const double* __restrict__ tsamp,
               const int64_t* __restrict__ idx, const unsigned long long* __restrict__ count,
               TrajOut out, const BulkInst* __restrict__ inst, int n_inst) {
    constexpr int N = 2 * DIM + (PHASE != ETRAJ_PHASE_CTMC ? 1 : 0);
    __shared__ int64_t s_end[kMaxInstances];
    __shared__ int s_toff[kMaxInstances];
    for (int i = threadIdx.x; i < n_inst; i += blockDim.x) {
        s_end[i] = inst[i].cand_end;
        s_toff[i] = inst[i].t_off;
    }
    __syncthreads();
    const int64_t n = (int64_t)(*count);
    const float Z = (float)J.target.Z, sc = (float)J.target.sc;
    const uint32_t sentinel = (uint32_t)(n_inst > 0 ? (int64_t)n_inst * J.grid : J.grid);
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n;
         s += (int64_t)gridDim.x * blockDim.x) {
        const int st = out.status[s] & 0xff;
        const int64_t g = idx ? idx[s] : s;
        int my = 0;
        if (n_inst > 0) {
            int lo = 0, hi = n_inst - 1;
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (g < s_end[mid]) hi = mid;
                else lo = mid + 1;
            }
            my = lo;
        }
        const double prob = soa.rate[g];
        uint32_t key = sentinel;
        double cre = 0.0, cim = 0.0, wion = 0.0, wunc = 0.0;
        float pin[3] = {0.0f, 0.0f, 0.0f};
        double phase_out = 0.0;
        bool ionized = false;
        if (st == 0) {
            const double* f = out.final_state + s * N;
            float rv[3], pv[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                rv[d] = (d < DIM) ? (float)f[d] : 0.0f;
                pv[d] = (d < DIM) ? (float)f[DIM + d] : 0.0f;
            }
            const float r2 = fmaf(rv[0], rv[0], fmaf(rv[1], rv[1], rv[2] * rv[2]));
            const float K = 0.5f * fmaf(pv[0], pv[0], fmaf(pv[1], pv[1], pv[2] * pv[2]));
            float V;
            if (J.target.kind == ETRAJ_TARGET_HYDROGEN_LIKE) {
                V = -Z * rsqrt_nr(r2 + sc);
            } else {
                const DTarget& T = J.target;
                const float r = sqrtf(r2);
                const float num = fmaf((float)T.a3, __expf(-(float)T.b3 * r),
                                       fmaf((float)T.a2 * r, __expf(-(float)T.b2 * r),
                                            fmaf((float)T.a1, __expf(-(float)T.b1 * r), Z)));
                V = -num * rsqrt_nr(r2 + sc);
            }
            const float E = K + V;
            const float L[3] = {rv[1] * pv[2] - rv[2] * pv[1], rv[2] * pv[0] - rv[0] * pv[2],
                                rv[0] * pv[1] - rv[1] * pv[0]};
            const float L2 = fmaf(L[0], L[0], fmaf(L[1], L[1], L[2] * L[2]));
            double phase = 0.0;
            if (PHASE != ETRAJ_PHASE_CTMC) phase = f[N - 1];
            if (PHASE == ETRAJ_PHASE_SCTS && E > 0.0f) {
                const float sqrtb = rsqrtf(2.0f * E);
                const float gg = sqrtf(fmaf(2.0f * E, L2, 1.0f));
                // the 3D reference uses x*py where x*px is meant (TrajectorySimulation.jl:463)
                const float rp = (DIM == 2) ? fmaf(rv[0], pv[0], rv[1] * pv[1])
                                            : fmaf(rv[0], pv[1], fmaf(rv[1], pv[1], rv[2] * pv[2]));
                const float corr = (Z * sqrtb) * (logf(gg) + asinhf(rp / (gg * sqrtb)));
                const int toff = (n_inst > 0) ? s_toff[my] : 0;
                phase = (phase + J.target.Ip * tsamp[toff + soa.batch[g]]) - (double)corr;
            }
            phase_out = phase;
            if (E >= 0.0f) {
                ionized = true;
                wion = prob;
                const float pinf = sqrtf(2.0f * E);
                const float inr = rsqrt_nr(fmaxf(r2, 1e-30f));
                const float pL[3] = {pv[1] * L[2] - pv[2] * L[1], pv[2] * L[0] - pv[0] * L[2],
                                     pv[0] * L[1] - pv[1] * L[0]};
                float a[3];
#pragma unroll
                for (int i = 0; i < 3; ++i) a[i] = pL[i] - Z * rv[i] * inr;
                const float La[3] = {L[1] * a[2] - L[2] * a[1], L[2] * a[0] - L[0] * a[2],
                                     L[0] * a[1] - L[1] * a[0]};
                const float fac = pinf / fmaf(pinf * pinf, L2, 1.0f);
#pragma unroll
                for (int i = 0; i < 3; ++i) pin[i] = fac * fmaf(pinf, La[i], -a[i]);
                int64_t lin = 0, stride = 1;
                bool ok = true;
#pragma unroll
                for (int d = 0; d < DIM; ++d) {
                    const int64_t num = J.pnum[d];
                    int64_t ix = 1;
                    if (num > 1) {
                        const float v = rintf((pin[d] + (float)J.pmax[d]) / (float)J.binw[d]);
                        if (!(v >= 1.0f && v <= (float)num)) ok = false;
                        else ix = (int64_t)v;
                    }
                    lin += (ix - 1) * stride;
                    stride *= num;
                }
                if (ok) {
                    key = (uint32_t)((int64_t)my * J.grid + lin);
                    if (PHASE == ETRAJ_PHASE_CTMC) {
                        cre = prob;
                    } else {
                        // reduce mod 2 pi in FP64 (2 pi split in two parts), then FP32 sincos
                        const double kq = rint(phase * 0.15915494309189535);
                        const double red = fma(-kq, 1.2246467991473532e-16, fma(-kq, 6.283185307179586, phase));
                        float sn, cs;
                        sincosf((float)red, &sn, &cs);
                        const float sp = sqrtf((float)prob);
                        cre = (double)(sp * cs);
                        cim = (double)(sp * sn);
                    }
                } else {
                    wunc = prob;
                }
            }
        }
        out.key[s] = key;
        out.c_re[s] = cre;
        out.c_im[s] = cim;
        out.w_ion[s] = wion;
        out.w_unc[s] = wunc;
        if (out.p_inf) {
            out.p_inf[3 * s] = pin[0];
            out.p_inf[3 * s + 1] = pin[1];
            out.p_inf[3 * s + 2] = pin[2];
        }
        if (out.fphase) out.fphase[s] = phase_out;
        out.status[s] = st | (ionized ? 0x100 : 0);
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

template <int DIM, int PHASE, int TGT, bool MULTI>
int launch_bulk_t(const BulkParams& P, InitSoA soa, const double* t, const int64_t* idx,
                  const unsigned long long* count, unsigned long long* queue, TrajOut out, int sm_count,
                  cudaStream_t s) {
    const size_t smem = (!MULTI && P.table_in_smem) ? (size_t)P.n_int * 2 * sizeof(float4) : 0;
    auto kern = (P.occ == 3) ? k_integrate_bulk<DIM, PHASE, TGT, MULTI, 3> : k_integrate_bulk<DIM, PHASE, TGT, MULTI, 2>;
    if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    // persistent grid, but no more blocks than the job can keep busy (at least ~4
    // electrons per lane): a block holds its SM's registers until its last warp
    // exits, so an oversized grid for a small job would fence off the whole GPU
    // from concurrent jobs for as long as its slowest trajectory runs
    const int64_t lanes_per_block = (int64_t)P.threads * 4;
    const int64_t want = (P.max_n + lanes_per_block - 1) / lanes_per_block;
    const int64_t cap = (int64_t)sm_count * P.blocks_per_sm;
    int blocks = (int)(want < 1 ? 1 : (want < cap ? want : cap));
    if (P.static_assign) {
        // one electron per lane: a grid over all of them, one launch
        const int64_t nb = (P.max_n + P.threads - 1) / P.threads;
        blocks = (int)(nb < 1 ? 1 : nb);
        cudaMemsetAsync(queue, 0, sizeof(unsigned long long) * 2, s);
        BulkParams Q = P;
        Q.park_buf = nullptr;
        Q.park_in = nullptr;
        Q.park_out = nullptr;
        Q.park_budget = 0;
        Q.park_out_count = queue + 1;
        kern<<<blocks, P.threads, smem, s>>>(Q, soa, t, idx, count, queue, out);
        return 1;
    }
    // queue[2r]: the work counter of round r; queue[2r+1]: electrons parked in round r
    const int rounds = P.park_buf ? kBulkRounds : 1;
    cudaMemsetAsync(queue, 0, sizeof(unsigned long long) * 2 * rounds, s);
    for (int r = 0; r < rounds; ++r) {
        BulkParams Q = P;
        const size_t half = (size_t)P.park_cap * kParkWords;
        // the step chunk of round r: chunk0 16^r steps (1024, 16384, 262144 for the
        // default chunk0 = 1024); the last round has none
        Q.park_budget = (r + 1 < rounds) ? (P.chunk0 > 0 ? P.chunk0 : 1024) << (4 * r) : 0;
        Q.park_in = (r > 0) ? P.park_buf + (size_t)((r - 1) & 1) * half : nullptr;
        Q.park_in_count = (r > 0) ? queue + 2 * (r - 1) + 1 : nullptr;
        Q.park_out = (P.park_buf && r + 1 < rounds) ? P.park_buf + (size_t)(r & 1) * half : nullptr;
        Q.park_out_count = queue + 2 * r + 1;
        kern<<<(r == 0) ? blocks : (int)cap, P.threads, smem, s>>>(Q, soa, t, idx, count, queue + 2 * r, out);
    }
    return rounds;
}

}  // namespace

int launch_collect_bulk(const DJob& J, InitSoA soa, const double* t, const int64_t* idx,
                        const unsigned long long* count, TrajOut out, int64_t max_n, int sm_count,
                        cudaStream_t s, const BulkInst* inst, int n_inst) {
    const int threads = 256;
    const int64_t want = (max_n + threads - 1) / threads;
    const int64_t cap = (int64_t)sm_count * 8;
    const int blocks = (int)(want < cap ? (want > 0 ? want : 1) : cap);
#define ETRAJ_COLLECT(D, P) k_collect_bulk<D, P><<<blocks, threads, 0, s>>>(J, soa, t, idx, count, out, inst, n_inst)
    if (J.dim == 2) {
        if (J.phase == ETRAJ_PHASE_CTMC) ETRAJ_COLLECT(2, ETRAJ_PHASE_CTMC);
        else if (J.phase == ETRAJ_PHASE_QTMC) ETRAJ_COLLECT(2, ETRAJ_PHASE_QTMC);
        else ETRAJ_COLLECT(2, ETRAJ_PHASE_SCTS);
    } else {
        if (J.phase == ETRAJ_PHASE_CTMC) ETRAJ_COLLECT(3, ETRAJ_PHASE_CTMC);
        else if (J.phase == ETRAJ_PHASE_QTMC) ETRAJ_COLLECT(3, ETRAJ_PHASE_QTMC);
        else ETRAJ_COLLECT(3, ETRAJ_PHASE_SCTS);
    }
#undef ETRAJ_COLLECT
    return 1;
}

namespace {
__global__ void k_clamp_count(const unsigned long long* __restrict__ count, unsigned long long cap,
                              unsigned long long* __restrict__ out) {
    const unsigned long long c = *count;
    *out = c < cap ? c : cap;
}
}  // namespace

int launch_clamp_count(const unsigned long long* count, unsigned long long cap, unsigned long long* out,
                       cudaStream_t s) {
    k_clamp_count<<<1, 1, 0, s>>>(count, cap, out);
    return 1;
}

int launch_field_table(const DJob& J, double T0, double h, int n_int, float4* tab, cudaStream_t s) {
    k_field_table<<<(n_int + 127) / 128, 128, 0, s>>>(J, T0, h, n_int, tab);
    return 1;
}

int launch_integrate_bulk(const BulkParams& P, InitSoA soa, const double* t, const int64_t* idx,
                          const unsigned long long* count, unsigned long long* queue, TrajOut out,
                          int sm_count, cudaStream_t s) {
#define ETRAJ_BULK_M(D, PH, TG)                                                                    \
    return (P.n_inst > 0) ? launch_bulk_t<D, PH, TG, true>(P, soa, t, idx, count, queue, out, sm_count, s) \
                          : launch_bulk_t<D, PH, TG, false>(P, soa, t, idx, count, queue, out, sm_count, s);
#define ETRAJ_BULK_TGT(D, PH)                                      \
    if (P.tgt == ETRAJ_TARGET_HYDROGEN_LIKE) {                     \
        ETRAJ_BULK_M(D, PH, ETRAJ_TARGET_HYDROGEN_LIKE)            \
    }                                                              \
    ETRAJ_BULK_M(D, PH, ETRAJ_TARGET_SAE)
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
#undef ETRAJ_BULK_M
}

}  // namespace etraj
