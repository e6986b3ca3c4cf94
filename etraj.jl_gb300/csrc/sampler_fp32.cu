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

#include "engine.h"

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

__device__ __forceinline__ float factf(int n) {
    float f = 1.0f;
    for (int i = 2; i <= n; ++i) f *= (float)i;
    return f;
}

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

// k-sum of the solid harmonic (shared_methods.jl:21) at complex (x, y, z).
__device__ cf sph_sum(int l, int m, cf x, cf y, cf z) {
    const cf xp = cmk(x.re - y.im, x.im + y.re);
    const cf xm = cmk(x.re + y.im, x.im - y.re);
    const int kmin = (m < 0) ? -m : 0, kmax = (l - m) / 2;
    cf acc = cmk(0.0f, 0.0f);
    for (int k = kmin; k <= kmax; ++k) {
        float p2 = 1.0f;
        for (int i = 0; i < 2 * k + m; ++i) p2 *= 2.0f;
        const float coef = ((k & 1) ? -1.0f : 1.0f) / (p2 * factf(k + m) * factf(k) * factf(l - m - 2 * k));
        cf tt = cscale(cpowi(xp, k + m), coef);
        tt = cmul(tt, cpowi(xm, k));
        tt = cmul(tt, cpowi(z, l - m - 2 * k));
        acc = cadd(acc, tt);
    }
    return acc;
}

__global__ void __launch_bounds__(256)
k_sample32(const __grid_constant__ DJob J, int64_t b0, int64_t nb, const double* __restrict__ kdv,
           const double* __restrict__ kzv, const DBatch* __restrict__ batches, InitSoA soa,
           uint8_t* __restrict__ flag) {
    const int64_t total = nb * J.n_cand;
    const float Ip = (float)J.Ip, kap2 = (float)(J.kappa * J.kappa), sqdkdt = (float)sqrt(J.dkdt);
    const float inv_dkdt = (float)(1.0 / J.dkdt), cutoff = (float)J.cutoff, e_pre = (float)J.e_pre;
    const float c_pre = (float)J.c, kd_max = (float)J.mc_kd_max, kz_max = (float)J.mc_kz_max;
    const float spane_lim = J.mc ? 0.04f : (float)(1.0 / 9.0);
    const bool spane = (J.method == ETRAJ_SAMPLER_SPANE);
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < total;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t bl = q / J.n_cand, i = q - bl * J.n_cand, b = b0 + bl;
        const FBatch& B = batches[b].f;
        float kd0, kz0;
        if (!J.mc) {
            kd0 = (float)kdv[i / J.n_kz];
            kz0 = (float)kzv[i % J.n_kz];
        } else {
            uint32_t c[4] = {(uint32_t)i, (uint32_t)((uint64_t)i >> 32), (uint32_t)b, 0x4B445A00u};
            philox4x32(c, J.seed);
            // the leading 24 bits of the FP64 sampler's 53-bit uniforms
            const float ua = (float)(c[0] >> 8) * 5.9604644775390625e-8f;
            const float ub = (float)(c[2] >> 8) * 5.9604644775390625e-8f;
            kd0 = ((ua - 0.5f) * 2.0f) * kd_max;
            if (J.dim == 3) {
                kz0 = ((ub - 0.5f) * 2.0f) * kz_max;
                if (J.mc_kd_max == 0.0) kd0 = 0.0f;
                else if (J.mc_kz_max == 0.0) kz0 = 0.0f;
            } else {
                kz0 = 0.0f;
            }
        }
        uint8_t keep = 0;
        float x0 = 0.0f, y0 = 0.0f, kx0 = 0.0f, ky0 = 0.0f, rate = 0.0f, ph = 0.0f;
        if (!(fabsf(kd0) < 1e-4f)) {
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
                    for (int mp = -J.l; mp <= J.l; ++mp) {
                        const int ii = mp + J.l;
                        const cf Y = cmul(cmk(J.fPlm[2 * ii], J.fPlm[2 * ii + 1]), sph_sum(J.l, mp, nkx, nky, nkz));
                        num = cadd(num, cmul(cmk(B.CD[2 * ii], B.CD[2 * ii + 1]), Y));
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

}  // namespace

int launch_sample32_range(const DJob& J, int64_t b0, int64_t nb, const double* kd, const double* kz,
                          const DBatch* batches, InitSoA soa, uint8_t* flag, int sm_count,
                          cudaStream_t s) {
    const int threads = 256;
    const int64_t want = (nb * J.n_cand + threads - 1) / threads;
    const int64_t cap = (int64_t)sm_count * 32;
    const int blocks = (int)(want < cap ? (want > 0 ? want : 1) : cap);
    k_sample32<<<blocks, threads, 0, s>>>(J, b0, nb, kd, kz, batches, soa, flag);
    return 1;
}

}  // namespace etraj
