// integrate_fp32.cu -- the bulk integrator: persistent, warp-cooperative,
// work-stealing Tsit5 with FP32 stages and compensated state.
//
// Same method and step controller as the plain FP64 path (Tsit5, abstol 1e-6,
// RMS error norm, PI control with beta1 = 7/50, beta2 = 2/25; see
// integrate_fp64.cu), re-cast for GB300's FP32 CUDA cores:
//
//  * Field table.  F(t) is one function of time shared by every trajectory,
//    so it is tabulated once per job in FP64 (cubic Hermite pieces from the
//    exact F and its forward-mode derivative, spacing h = T_min/128, relative
//    interpolation error ~1e-8) and stored as FP32 polynomial coefficients in
//    shared memory.  A right-hand side then costs 6 FFMA for the field instead
//    of two sincos and two tanh, for every laser kind alike.
//  * Fixed-point time.  t = T0 + h (n + f) with an integer interval n and an
//    FP32 fraction f, i.e. ~1e-7 a.u. resolution over any time span, without
//    FP64 arithmetic in the step loop.
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
// Roofline: FP32 issue bound (~450 FP32 instructions per Tsit5 step for
// hydrogen in 2D), MUFU for rsqrt/exp2/log2; no tensor cores.

#include "physics.cuh"

namespace etraj {

namespace {

constexpr float C2 = 0.161f, C3 = 0.327f, C4 = 0.9f, C5 = 0.9800255409045097f;
constexpr float A21 = 0.161f;
constexpr float A31 = -0.008480655492356989f, A32 = 0.335480655492357f;
constexpr float A41 = 2.897153057105493f, A42 = -6.359448489975075f, A43 = 4.3622954328695815f;
constexpr float A51 = 5.325864828439257f, A52 = -11.748883564062828f, A53 = 7.4955393428898365f,
                A54 = -0.09249506636175525f;
constexpr float A61 = 5.86145544294642f, A62 = -12.92096931784711f, A63 = 8.159367898576159f,
                A64 = -0.071584973281401f, A65 = -0.028269050394068383f;
constexpr float A71 = 0.09646076681806523f, A72 = 0.01f, A73 = 0.4798896504144996f,
                A74 = 1.379008574103742f, A75 = -3.290069515436081f, A76 = 2.324710524099774f;
constexpr float BT1 = -0.00178001105222577714f, BT2 = -0.0008164344596567469f,
                BT3 = 0.007880878010261995f, BT4 = -0.1447110071732629f, BT5 = 0.5823571654525552f,
                BT6 = -0.45808210592918697f, BT7 = 0.015151515151515152f;
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

template <int DIM, int PHASE, int TGT>
__device__ __forceinline__ void rhs32(const BulkParams& P, const float4* __restrict__ tab, int ni,
                                      float fi, const float* u, float* du) {
    float Fx, Fy;
    field(tab, P.n_int, ni, fi, Fx, Fy);
    const float x = u[0], y = u[1];
    const float z = (DIM == 3) ? u[2] : 0.0f;
    const float px = u[DIM], py = u[DIM + 1];
    const float pz = (DIM == 3) ? u[5] : 0.0f;
    const float r2 = (DIM == 3) ? fmaf(x, x, fmaf(y, y, z * z)) : fmaf(x, x, y * y);
    float coef, Vphase = 0.0f;
    if (TGT == ETRAJ_TARGET_HYDROGEN_LIKE) {
        const float ri = rsqrt_nr(r2 + P.sc);
        coef = -P.Z * (ri * ri * ri);
        Vphase = P.Z * ri;
    } else {
        const float r = r2 * rsqrt_nr(fmaxf(r2, 1e-30f));
        const float ris = rsqrt_nr(r2 + P.sc);
        const float e1 = __expf(-P.b1 * r), e2 = __expf(-P.b2 * r), e3 = __expf(-P.b3 * r);
        const float br = fmaf(P.a3 * fmaf(P.b3, r, 1.0f), e3, fmaf(P.a1 * fmaf(P.b1, r, 1.0f), e1, P.Z));
        coef = -fmaf(ris * ris * ris, br, P.a2b2 * ris * e2);
        if (PHASE != ETRAJ_PHASE_CTMC) {
            const float num = fmaf(P.a3, e3, fmaf(P.a2 * r, e2, fmaf(P.a1, e1, P.Z)));
            Vphase = (DIM == 2 && PHASE == ETRAJ_PHASE_SCTS) ? num * (ris * ris) : num * ris;
        }
    }
    const float tFx = coef * x, tFy = coef * y, tFz = coef * z;
    du[0] = px;
    du[1] = py;
    if (DIM == 3) du[2] = pz;
    du[DIM] = tFx - Fx;
    du[DIM + 1] = tFy - Fy;
    if (DIM == 3) du[5] = tFz;
    if (PHASE != ETRAJ_PHASE_CTMC) {
        const float K = 0.5f * ((DIM == 3) ? fmaf(px, px, fmaf(py, py, pz * pz)) : fmaf(px, px, py * py));
        const float rF = (DIM == 3) ? fmaf(x, tFx, fmaf(y, tFy, z * tFz)) : fmaf(x, tFx, y * tFy);
        du[2 * DIM] = (PHASE == ETRAJ_PHASE_QTMC) ? -((P.Ip + K) - Vphase) : -((K - Vphase) + rF);
    }
}

__device__ __forceinline__ void advance(int n, float f, float dth, int& no, float& fo) {
    float g = f + dth;
    float fl = floorf(g);
    no = n + (int)fl;
    fo = g - fl;
}

template <int N>
__device__ __forceinline__ float rms_ratio(const float* v, const float* sk) {
    float acc = 0.0f;
#pragma unroll
    for (int j = 0; j < N; ++j) {
        float q = v[j] / sk[j];
        acc = fmaf(q, q, acc);
    }
    return sqrtf(acc * (1.0f / N));
}

template <int DIM, int PHASE, int TGT>
__global__ void __launch_bounds__(256, 2)
k_integrate_bulk(const __grid_constant__ BulkParams P, InitSoA soa, const double* __restrict__ tsamp,
                 const int64_t* __restrict__ idx, const unsigned long long* __restrict__ count,
                 unsigned long long* __restrict__ queue, TrajOut out) {
    constexpr int N = 2 * DIM + (PHASE != ETRAJ_PHASE_CTMC ? 1 : 0);
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

    float uh[N], ul[N], k1[N], k7[N];
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
                    double u0d[N];
                    u0d[0] = soa.x[g];
                    u0d[1] = soa.y[g];
                    if (DIM == 2) {
                        u0d[2] = soa.kx[g];
                        u0d[3] = soa.ky[g];
                    } else {
                        u0d[2] = 0.0;
                        u0d[3] = soa.kx[g];
                        u0d[4] = soa.ky[g];
                        u0d[5] = soa.kz[g];
                    }
                    if (PHASE != ETRAJ_PHASE_CTMC) u0d[N - 1] = soa.phase[g];
#pragma unroll
                    for (int j = 0; j < N; ++j) {
                        uh[j] = (float)u0d[j];
                        ul[j] = (float)(u0d[j] - (double)uh[j]);
                    }
                    const double t0 = tsamp[soa.batch[g]];
                    const double q0 = (t0 - P.T0) * P.inv_h_d;
                    const double fl = floor(q0);
                    tn = (int)fl;
                    tfr = (float)(q0 - fl);
                    dthmax = (float)((P.t_final - t0) * P.inv_h_d);
                    rhs32<DIM, PHASE, TGT>(P, tab, tn, tfr, uh, k1);
                    float sk[N], u1[N], f1[N], df[N];
#pragma unroll
                    for (int j = 0; j < N; ++j) sk[j] = fmaf(fabsf(uh[j]), P.rtol, ABSTOL);
                    const float d0 = rms_ratio<N>(uh, sk), d1 = rms_ratio<N>(k1, sk);
                    float dt0 = (d0 < 1e-5f || d1 < 1e-5f) ? 1e-6f : (d0 / d1) * 0.01f;
                    dt0 = fminf(dt0, dthmax * P.h);
#pragma unroll
                    for (int j = 0; j < N; ++j) u1[j] = fmaf(dt0, k1[j], uh[j]);
                    int n1;
                    float f1r;
                    advance(tn, tfr, dt0 * P.inv_h, n1, f1r);
                    rhs32<DIM, PHASE, TGT>(P, tab, n1, f1r, u1, f1);
#pragma unroll
                    for (int j = 0; j < N; ++j) df[j] = f1[j] - k1[j];
                    const float d2 = rms_ratio<N>(df, sk) / dt0;
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
            const float dt = dth * P.h;
            float tmp[N], k2[N], k3[N], k4[N], k5[N], k6[N], inc[N];
            int ni;
            float fi;
#pragma unroll
            for (int j = 0; j < N; ++j) tmp[j] = fmaf(dt, A21 * k1[j], uh[j]);
            advance(tn, tfr, C2 * dth, ni, fi);
            rhs32<DIM, PHASE, TGT>(P, tab, ni, fi, tmp, k2);
#pragma unroll
            for (int j = 0; j < N; ++j) tmp[j] = fmaf(dt, fmaf(A32, k2[j], A31 * k1[j]), uh[j]);
            advance(tn, tfr, C3 * dth, ni, fi);
            rhs32<DIM, PHASE, TGT>(P, tab, ni, fi, tmp, k3);
#pragma unroll
            for (int j = 0; j < N; ++j)
                tmp[j] = fmaf(dt, fmaf(A43, k3[j], fmaf(A42, k2[j], A41 * k1[j])), uh[j]);
            advance(tn, tfr, C4 * dth, ni, fi);
            rhs32<DIM, PHASE, TGT>(P, tab, ni, fi, tmp, k4);
#pragma unroll
            for (int j = 0; j < N; ++j)
                tmp[j] = fmaf(dt, fmaf(A54, k4[j], fmaf(A53, k3[j], fmaf(A52, k2[j], A51 * k1[j]))), uh[j]);
            advance(tn, tfr, C5 * dth, ni, fi);
            rhs32<DIM, PHASE, TGT>(P, tab, ni, fi, tmp, k5);
#pragma unroll
            for (int j = 0; j < N; ++j)
                tmp[j] = fmaf(dt, fmaf(A65, k5[j], fmaf(A64, k4[j], fmaf(A63, k3[j], fmaf(A62, k2[j], A61 * k1[j])))),
                              uh[j]);
            int n1;
            float f1;
            if (last) {
                n1 = P.nf;
                f1 = P.ff;
            } else {
                advance(tn, tfr, dth, n1, f1);
            }
            rhs32<DIM, PHASE, TGT>(P, tab, n1, f1, tmp, k6);
#pragma unroll
            for (int j = 0; j < N; ++j) {
                inc[j] = dt * fmaf(A76, k6[j], fmaf(A75, k5[j], fmaf(A74, k4[j], fmaf(A73, k3[j], fmaf(A72, k2[j], A71 * k1[j])))));
                tmp[j] = uh[j] + inc[j];
            }
            rhs32<DIM, PHASE, TGT>(P, tab, n1, f1, tmp, k7);
            float acc = 0.0f;
#pragma unroll
            for (int j = 0; j < N; ++j) {
                const float ut = dt * fmaf(BT7, k7[j], fmaf(BT6, k6[j], fmaf(BT5, k5[j], fmaf(BT4, k4[j],
                                     fmaf(BT3, k3[j], fmaf(BT2, k2[j], BT1 * k1[j]))))));
                const float sc = fmaf(fmaxf(fabsf(uh[j]), fabsf(tmp[j])), P.rtol, ABSTOL);
                const float r = ut / sc;
                acc = fmaf(r, r, acc);
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
                if (q == 1.0f) q = 1.0f;
                qold = fmaxf(EEst, QOLDINIT);
                dthp = fminf(dthmax, dth / q);
#pragma unroll
                for (int j = 0; j < N; ++j) {
                    df_add(uh[j], ul[j], inc[j]);
                    k1[j] = k7[j];
                }
                tn = n1;
                tfr = f1;
                if (last) status = -1;  // reached t_final
                else {
                    bool bad = false;
#pragma unroll
                    for (int j = 0; j < N; ++j) bad |= !(uh[j] == uh[j]);
                    if (bad) status = 3;
                }
            }
        }
        if (status != 0) {
            // finished (status -1 = Success) or failed: write the FP64 state and free the lane
            const int code = (status < 0) ? 0 : status;
            out.status[s] = code;
            out.steps[s] = attempts;
#pragma unroll
            for (int j = 0; j < N; ++j) out.final_state[s * N + j] = (double)uh[j] + (double)ul[j];
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
