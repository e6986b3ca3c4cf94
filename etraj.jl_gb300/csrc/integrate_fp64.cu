// integrate_fp64.cu -- the plain FP64 integrator (one thread per trajectory,
// static grid-stride assignment) with the collection fused into its epilogue.
//
// Replaces, per electron, the ensemble solve
//   solve(EnsembleProblem(...), Tsit5(), EnsembleSerial(), reltol=traj_rtol)
// (src/TrajectorySimulation.jl:334-342, 3D :429-437) and the collection loop
// body (:344-397, 3D :439-497): retcode check, E_inf, SCTS post-pulse
// phase, Kepler asymptote, bin index and the deposit contribution.
//
// Tsit5 with OrdinaryDiffEq's defaults for `solve(prob, Tsit5(), reltol)`:
// abstol 1e-6, RMS error norm, PI controller (beta1 = 7/50, beta2 = 2/25,
// qmin = 1/5, qmax = 10, gamma = 9/10, qoldinit = 1e-4), Hairer's starting
// step, FSAL, t_final hit exactly.  Compiled with --fmad=false: every
// fused multiply-add is an explicit fma(), so the results are bit-identical
// to the CPU oracle's.
//
// Roofline: FP64-pipe bound (about 600 DFMA-equivalent per step for
// hydrogen + Cos4); no tensor cores (not a contraction).

#include "physics.cuh"

namespace etraj {
namespace {

constexpr double C2 = 0.161, C3 = 0.327, C4 = 0.9, C5 = 0.9800255409045097;
constexpr double A21 = 0.161;
constexpr double A31 = -0.008480655492356989, A32 = 0.335480655492357;
constexpr double A41 = 2.897153057105493, A42 = -6.359448489975075, A43 = 4.3622954328695815;
constexpr double A51 = 5.325864828439257, A52 = -11.748883564062828, A53 = 7.4955393428898365,
                 A54 = -0.09249506636175525;
constexpr double A61 = 5.86145544294642, A62 = -12.92096931784711, A63 = 8.159367898576159,
                 A64 = -0.071584973281401, A65 = -0.028269050394068383;
constexpr double A71 = 0.09646076681806523, A72 = 0.01, A73 = 0.4798896504144996,
                 A74 = 1.379008574103742, A75 = -3.290069515436081, A76 = 2.324710524099774;
constexpr double BT1 = -0.00178001105222577714, BT2 = -0.0008164344596567469,
                 BT3 = 0.007880878010261995, BT4 = -0.1447110071732629, BT5 = 0.5823571654525552,
                 BT6 = -0.45808210592918697, BT7 = 0.015151515151515152;
constexpr double ABSTOL = 1e-6, BETA1 = 0.14, BETA2 = 0.08, QMIN_INV = 5.0, QMAX_INV = 0.1,
                 GAMMA = 0.9, QOLDINIT = 1e-4;
constexpr long MAXITERS = 1000000L;

__device__ __forceinline__ double d_ulp(double x) {
    double a = fabs(x);
    uint64_t u = dm_d2u(a);
    int e = (int)(u >> 52);
    if (e == 0) return dm_u2d(1);
    if (e >= 2046) return dm_inf();
    int p = e - 1023 - 52;
    if (p >= -1022) return dm_pow2i(p);
    return dm_u2d(1ull << (p + 1074));
}
__device__ __forceinline__ double jmin(double a, double b) {
    return (a != a || b != b) ? a + b : (a < b ? a : b);
}
__device__ __forceinline__ double jmax(double a, double b) {
    return (a != a || b != b) ? a + b : (a > b ? a : b);
}

template <int N>
__device__ __forceinline__ double rms_ratio(const double* v, const double* sk) {
    double acc = 0.0;
#pragma unroll
    for (int j = 0; j < N; ++j) {
        double q = v[j] / sk[j];
        acc = fma(q, q, acc);
    }
    return sqrt(acc / (double)N);
}

template <int DIM, int PHASE, int TGT, int N>
__device__ double initdt(const DJob& J, double t, const double* u0, const double* f0, double dtmax,
                         double dtmin) {
    double sk[N], u1[N], f1[N], df[N];
#pragma unroll
    for (int j = 0; j < N; ++j) sk[j] = fma(fabs(u0[j]), J.rtol, ABSTOL);
    double d0 = rms_ratio<N>(u0, sk);
    double d1 = rms_ratio<N>(f0, sk);
    double dt0 = (d0 < 1e-5 || d1 < 1e-5) ? 1e-6 : (d0 / d1) / 100.0;
    dt0 = jmin(dt0, dtmax);
    if (dt0 < 10.0 * 2.220446049250313e-16) return 1e-6;
#pragma unroll
    for (int j = 0; j < N; ++j) u1[j] = fma(dt0, f0[j], u0[j]);
    rhs<DIM, PHASE, TGT>(J, t + dt0, u1, f1);
#pragma unroll
    for (int j = 0; j < N; ++j) df[j] = f1[j] - f0[j];
    double d2 = rms_ratio<N>(df, sk) / dt0;
    double md = jmax(d1, d2);
    double dt1;
    if (md <= 1e-15) dt1 = jmax(1e-6, dt0 * 1e-3);
    else dt1 = dm_pow_pos(10.0, -(2.0 + dm_log(md) / DM_LN10) / 5.0);
    return jmax(dtmin, jmin(jmin(100.0 * dt0, dt1), dtmax));
}

// r^2 of a state, summed left to right
template <int DIM>
__device__ __forceinline__ double radius2(const double* u) {
    double r2 = u[0] * u[0] + u[1] * u[1];
    if (DIM == 3) r2 = r2 + u[2] * u[2];
    return r2;
}

// One adaptive Tsit5 solve; returns the status (0 Success).  rmin (optional):
// the least |r| of the initial state and of the end of every accepted step.
template <int DIM, int PHASE, int TGT, int N>
__device__ int solve(const DJob& J, double t0, double tf, const double* u0, double* uout,
                     int32_t& attempts, double* rmin = nullptr) {
    double uprev[N], u[N], tmp[N];
    double k1[N], k2[N], k3[N], k4[N], k5[N], k6[N], k7[N];
    double t = t0;
#pragma unroll
    for (int j = 0; j < N; ++j) uprev[j] = u[j] = u0[j];
    const double dtmax = tf - t0;
    const double dtmin = jmax(d_ulp(t0), d_ulp(tf));
    rhs<DIM, PHASE, TGT>(J, t, uprev, k1);
    double dt = initdt<DIM, PHASE, TGT, N>(J, t, uprev, k1, dtmax, dtmin);
    double dtpropose = dt, qold = QOLDINIT, q11 = 1.0;
    double r2min = rmin ? radius2<DIM>(uprev) : 0.0;
    bool accept = false;
    int status = 0;
    long iter = 0;
    attempts = 0;
    while (t < tf) {
        if (iter > 0) {
            if (!accept) {
                dt = dt / jmin(QMIN_INV, q11 / GAMMA);
            } else {
#pragma unroll
                for (int j = 0; j < N; ++j) {
                    uprev[j] = u[j];
                    k1[j] = k7[j];
                }
                dt = dtpropose;
            }
        }
        ++iter;
        dt = jmin(dtmax, dt);
        dt = jmax(dt, jmax(dtmin, d_ulp(t)));
        dt = jmin(dt, tf - t);
        if (dt != dt) { status = 4; break; }
        if (iter > MAXITERS) { status = 1; break; }
        if (dt <= dtmin && (!accept || t + dt < tf)) { status = 2; break; }
        if (accept) {
            bool bad = false;
#pragma unroll
            for (int j = 0; j < N; ++j) bad |= (u[j] != u[j]);
            if (bad) { status = 3; break; }
        }
        // stages 2..7 (perform_step! of Tsit5); every sum is built left to right
#pragma unroll
        for (int j = 0; j < N; ++j) tmp[j] = fma(dt, A21 * k1[j], uprev[j]);
        rhs<DIM, PHASE, TGT>(J, fma(C2, dt, t), tmp, k2);
#pragma unroll
        for (int j = 0; j < N; ++j) {
            double s = A31 * k1[j];
            s = fma(A32, k2[j], s);
            tmp[j] = fma(dt, s, uprev[j]);
        }
        rhs<DIM, PHASE, TGT>(J, fma(C3, dt, t), tmp, k3);
#pragma unroll
        for (int j = 0; j < N; ++j) {
            double s = A41 * k1[j];
            s = fma(A42, k2[j], s);
            s = fma(A43, k3[j], s);
            tmp[j] = fma(dt, s, uprev[j]);
        }
        rhs<DIM, PHASE, TGT>(J, fma(C4, dt, t), tmp, k4);
#pragma unroll
        for (int j = 0; j < N; ++j) {
            double s = A51 * k1[j];
            s = fma(A52, k2[j], s);
            s = fma(A53, k3[j], s);
            s = fma(A54, k4[j], s);
            tmp[j] = fma(dt, s, uprev[j]);
        }
        rhs<DIM, PHASE, TGT>(J, fma(C5, dt, t), tmp, k5);
#pragma unroll
        for (int j = 0; j < N; ++j) {
            double s = A61 * k1[j];
            s = fma(A62, k2[j], s);
            s = fma(A63, k3[j], s);
            s = fma(A64, k4[j], s);
            s = fma(A65, k5[j], s);
            tmp[j] = fma(dt, s, uprev[j]);
        }
        const double t1 = t + dt;
        rhs<DIM, PHASE, TGT>(J, t1, tmp, k6);
#pragma unroll
        for (int j = 0; j < N; ++j) {
            double s = A71 * k1[j];
            s = fma(A72, k2[j], s);
            s = fma(A73, k3[j], s);
            s = fma(A74, k4[j], s);
            s = fma(A75, k5[j], s);
            s = fma(A76, k6[j], s);
            u[j] = fma(dt, s, uprev[j]);
        }
        rhs<DIM, PHASE, TGT>(J, t1, u, k7);
        double acc = 0.0;
#pragma unroll
        for (int j = 0; j < N; ++j) {
            double s = BT1 * k1[j];
            s = fma(BT2, k2[j], s);
            s = fma(BT3, k3[j], s);
            s = fma(BT4, k4[j], s);
            s = fma(BT5, k5[j], s);
            s = fma(BT6, k6[j], s);
            s = fma(BT7, k7[j], s);
            double ut = dt * s;
            double sc = fma(jmax(fabs(uprev[j]), fabs(u[j])), J.rtol, ABSTOL);
            double r = ut / sc;
            acc = fma(r, r, acc);
        }
        const double EEst = sqrt(acc / (double)N);
        ++attempts;
        double q;
        if (EEst == 0.0) {
            q = QMAX_INV;
        } else {
            q11 = dm_pow_pos(EEst, BETA1);
            q = q11 / dm_pow_pos(qold, BETA2);
            q = jmax(QMAX_INV, jmin(QMIN_INV, q / GAMMA));
        }
        accept = (EEst <= 1.0);
        if (accept) {
            if (q >= 1.0 && q <= 1.0) q = 1.0;
            qold = jmax(EEst, QOLDINIT);
            double dtnew = dt / q;
            t = (fabs(t1 - tf) < 100.0 * d_ulp(jmax(t, tf))) ? tf : t1;
            dtpropose = jmax(jmin(dtmax, dtnew), dtmin);
            if (rmin) r2min = jmin(r2min, radius2<DIM>(u));
        }
    }
    if (rmin) *rmin = sqrt(r2min);
#pragma unroll
    for (int j = 0; j < N; ++j) uout[j] = (status == 0) ? u[j] : uprev[j];
    return status;
}

__device__ __forceinline__ void cross3(const double* a, const double* b, double* c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

// Collection of one electron (TrajectorySimulation.jl:356-393, 3D :451-493).
// Returns true when the electron is finally ionized (E_inf >= 0).
template <int DIM, int PHASE, int N>
__device__ __forceinline__ bool collect(const DJob& J, int status, const double* f, double tr,
                                        double prob, const TrajOut& out, int64_t s) {
    uint32_t key = (uint32_t)J.grid;
    double cre = 0.0, cim = 0.0, wion = 0.0, wunc = 0.0;
    double pin[3] = {0.0, 0.0, 0.0};
    double phase_out = 0.0;
    bool ionized = false;
    if (status == 0) {
        double x, y, z, px, py, pz, K;
        if (DIM == 2) {
            x = f[0]; y = f[1]; z = 0.0; px = f[2]; py = f[3]; pz = 0.0;
            K = (px * px + py * py) / 2.0;
        } else {
            x = f[0]; y = f[1]; z = f[2]; px = f[3]; py = f[4]; pz = f[5];
            K = ((px * px + py * py) + pz * pz) / 2.0;
        }
        double phase = (PHASE == ETRAJ_PHASE_CTMC) ? 0.0 : f[N - 1];
        double E = K + target_V(J.target, x, y, z);
        double rv[3] = {x, y, z}, pv[3] = {px, py, pz}, L[3];
        cross3(rv, pv, L);
        double L2 = (L[0] * L[0] + L[1] * L[1]) + L[2] * L[2];
        const double Z = J.target.Z;
        if (PHASE == ETRAJ_PHASE_SCTS && E > 0.0) {
            phase = phase + J.target.Ip * tr;
            double sqrtb = 1.0 / sqrt(2.0 * E);
            double g = sqrt(1.0 + (2.0 * E) * L2);
            // the 3D reference uses x*py where x*px is meant (TrajectorySimulation.jl:463)
            double rp = (DIM == 2) ? (x * px + y * py) : ((x * py + y * py) + z * pz);
            phase = phase - (Z * sqrtb) * (dm_log(g) + dm_asinh(rp / (g * sqrtb)));
        }
        phase_out = phase;
        if (E >= 0.0) {
            ionized = true;
            wion = prob;
            double pinf = sqrt(2.0 * E);
            double nr = sqrt((x * x + y * y) + z * z);
            double pL[3], a[3], La[3];
            cross3(pv, L, pL);
#pragma unroll
            for (int i = 0; i < 3; ++i) a[i] = pL[i] - (Z * rv[i]) / nr;
            cross3(L, a, La);
            double fac = pinf / (1.0 + (pinf * pinf) * L2);
#pragma unroll
            for (int i = 0; i < 3; ++i) pin[i] = fac * (pinf * La[i] - a[i]);
            int64_t lin = 0, stride = 1;
            bool ok = true;
#pragma unroll
            for (int d = 0; d < DIM; ++d) {
                int64_t num = J.pnum[d], ix = 1;
                if (num > 1) {
                    double pm = J.pmax[d];
                    double v = rint((pin[d] + pm) / J.binw[d]);
                    if (!(v >= 1.0 && v <= (double)num)) ok = false;
                    else ix = (int64_t)v;
                }
                lin += (ix - 1) * stride;
                stride *= num;
            }
            if (ok) {
                key = (uint32_t)lin;
                if (PHASE == ETRAJ_PHASE_CTMC) {
                    cre = prob;
                } else {
                    double sp = sqrt(prob), sn, cs;
                    dm_sincos(phase, &sn, &cs);
                    cre = sp * cs;
                    cim = sp * sn;
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
    return ionized;
}

template <int DIM, int PHASE, int TGT>
__global__ void __launch_bounds__(128)
k_integrate_fp64(const __grid_constant__ DJob J, InitSoA soa, const double* __restrict__ tsamp,
                 const int64_t* __restrict__ idx, const unsigned long long* __restrict__ count,
                 TrajOut out) {
    constexpr int N = (DIM == 3 ? 6 : 4) + (PHASE != ETRAJ_PHASE_CTMC ? 1 : 0);
    const int64_t n = (int64_t)(*count);
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n; s += stride) {
        const int64_t g = idx ? idx[s] : s;
        double u0[N], uf[N];
        u0[0] = soa.x[g];
        u0[1] = soa.y[g];
        if (DIM == 2) {
            u0[2] = soa.kx[g];
            u0[3] = soa.ky[g];
        } else {
            u0[2] = 0.0;
            u0[3] = soa.kx[g];
            u0[4] = soa.ky[g];
            u0[5] = soa.kz[g];
        }
        if (PHASE != ETRAJ_PHASE_CTMC) u0[N - 1] = soa.phase[g];
        const double t0 = tsamp[soa.batch[g]];
        int32_t attempts = 0;
        double rmin = 0.0;
        int st = solve<DIM, PHASE, TGT, N>(J, t0, J.t_final, u0, uf, attempts, out.rmin ? &rmin : nullptr);
        out.steps[s] = attempts;
        if (out.rmin) out.rmin[s] = rmin;
        if (out.final_state) {
#pragma unroll
            for (int j = 0; j < N; ++j) out.final_state[s * N + j] = uf[j];
        }
        const bool ion = collect<DIM, PHASE, N>(J, st, uf, t0, soa.rate[g], out, s);
        out.status[s] = st | (ion ? 0x100 : 0);
    }
}

// Collection of final states computed elsewhere (the FP32 bulk integrator).
template <int DIM, int PHASE>
__global__ void __launch_bounds__(128)
k_collect_fp64(const __grid_constant__ DJob J, InitSoA soa, const double* __restrict__ tsamp,
               const int64_t* __restrict__ idx, const unsigned long long* __restrict__ count,
               TrajOut out) {
    constexpr int N = (DIM == 3 ? 6 : 4) + (PHASE != ETRAJ_PHASE_CTMC ? 1 : 0);
    const int64_t n = (int64_t)(*count);
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n;
         s += (int64_t)gridDim.x * blockDim.x) {
        const int64_t g = idx ? idx[s] : s;
        double f[N];
#pragma unroll
        for (int j = 0; j < N; ++j) f[j] = out.final_state[s * N + j];
        const int st = out.status[s] & 0xff;
        const bool ion = collect<DIM, PHASE, N>(J, st, f, tsamp[soa.batch[g]], soa.rate[g], out, s);
        out.status[s] = st | (ion ? 0x100 : 0);
    }
}

template <int DIM, int PHASE, int TGT>
int launch_t(const DJob& J, InitSoA soa, const double* t, const int64_t* idx,
             const unsigned long long* count, TrajOut out, int64_t max_n, int sm_count,
             cudaStream_t s) {
    const int threads = 128;
    int64_t want = (max_n + threads - 1) / threads;
    int64_t cap = (int64_t)sm_count * 16;  // grid-stride beyond 16 blocks per SM
    int blocks = (int)(want < cap ? (want > 0 ? want : 1) : cap);
    k_integrate_fp64<DIM, PHASE, TGT><<<blocks, threads, 0, s>>>(J, soa, t, idx, count, out);
    return 1;
}

}  // namespace

int launch_integrate_fp64(const DJob& J, InitSoA soa, const double* t, const int64_t* idx,
                          const unsigned long long* count, TrajOut out, int64_t max_n,
                          int sm_count, cudaStream_t s) {
#define ETRAJ_DISPATCH_TGT(D, P)                                                               \
    return (J.target.kind == ETRAJ_TARGET_HYDROGEN_LIKE)                                       \
               ? launch_t<D, P, ETRAJ_TARGET_HYDROGEN_LIKE>(J, soa, t, idx, count, out, max_n, \
                                                            sm_count, s)                       \
               : launch_t<D, P, ETRAJ_TARGET_SAE>(J, soa, t, idx, count, out, max_n, sm_count, s);
    if (J.dim == 2) {
        if (J.phase == ETRAJ_PHASE_CTMC) { ETRAJ_DISPATCH_TGT(2, ETRAJ_PHASE_CTMC) }
        if (J.phase == ETRAJ_PHASE_QTMC) { ETRAJ_DISPATCH_TGT(2, ETRAJ_PHASE_QTMC) }
        ETRAJ_DISPATCH_TGT(2, ETRAJ_PHASE_SCTS)
    } else {
        if (J.phase == ETRAJ_PHASE_CTMC) { ETRAJ_DISPATCH_TGT(3, ETRAJ_PHASE_CTMC) }
        if (J.phase == ETRAJ_PHASE_QTMC) { ETRAJ_DISPATCH_TGT(3, ETRAJ_PHASE_QTMC) }
        ETRAJ_DISPATCH_TGT(3, ETRAJ_PHASE_SCTS)
    }
#undef ETRAJ_DISPATCH_TGT
}

int launch_collect_fp64(const DJob& J, InitSoA soa, const double* t, const int64_t* idx,
                        const unsigned long long* count, TrajOut out, int64_t max_n, int sm_count,
                        cudaStream_t s) {
    const int threads = 128;
    int64_t want = (max_n + threads - 1) / threads;
    int64_t cap = (int64_t)sm_count * 16;
    int blocks = (int)(want < cap ? (want > 0 ? want : 1) : cap);
#define ETRAJ_COLLECT(D, P) k_collect_fp64<D, P><<<blocks, threads, 0, s>>>(J, soa, t, idx, count, out)
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

}  // namespace etraj
