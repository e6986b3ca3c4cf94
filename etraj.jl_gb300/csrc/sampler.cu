// sampler.cu -- ADK, SPANE, SPA and WFAT initial-condition sampling on the device.
//
// Reference: gen_electron_batch in src/ElectronSamplers/ADKSampler.jl:167-396,
// SPANESampler.jl:163-404, SPASampler.jl:150-431 and WFATSampler.jl:129-249,
// with the helpers of shared_methods.jl:4-47.  The SPA saddle-point solve and
// quadratures are in spa.h, the molecular prefactor and the WFAT rate in
// mol.h, both shared with the CPU oracle.
//
// Layout: one thread per candidate (time sample b, transverse-momentum
// sample i), candidates in the reference's loop order (kd outer, kz inner;
// Monte-Carlo index i).  k_sample writes the candidate-indexed structure of
// arrays and a keep flag; the compaction kernels turn the flags into the
// ordered survivor list, so survivor k is the reference's k-th column of the
// concatenated `init` matrices.  The per-batch prologue (field at t_r, its
// derivative, Keldysh parameter, Coulomb-corrected prefactor constant and
// the Wigner-D row) runs once per time sample in k_batch_prepare.
//
// Monte-Carlo draws come from Philox4x32-10 (Salmon et al., SC'11), counter
// (i, batch, 0x4B445A00) keyed by the job seed: kd from output words 0,1 and
// kz from words 2,3, each mapped to [0,1) with 53 bits.
//
// Roofline: memory bound on the SoA writes (about 61 B per candidate).

#include "physics.cuh"

#define SPA_LASER_T etraj::DLaser
#define SPA_WIN(L, tre, w) etraj::laser_windows(*(L), (tre), (w))
#define SPA_AW(L, t, w, ax, ay) etraj::laser_A_complex(*(L), (t), (w), (ax), (ay))
#include "spa.h"

namespace etraj {
namespace {

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

__device__ __forceinline__ double u53(uint32_t a, uint32_t b) {
    return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) * (1.0 / 9007199254740992.0);
}

__device__ __forceinline__ double fact(int n) {
    double f = 1.0;
    for (int i = 2; i <= n; ++i) f *= (double)i;
    return f;
}

// Wigner small-d d^j_{m'm}(beta), explicit sum (standard convention).
__device__ double wigner_d(int j, int mp, int m, double beta) {
    double sh, ch;
    dm_sincos(0.5 * beta, &sh, &ch);
    double pref = sqrt(fact(j + mp) * fact(j - mp) * fact(j + m) * fact(j - m));
    double sum = 0.0;
    for (int s = 0; s <= 2 * j; ++s) {
        int a1 = j + m - s, a3 = mp - m + s, a4 = j - mp - s;
        if (a1 < 0 || a3 < 0 || a4 < 0) continue;
        double den = fact(a1) * fact(s) * fact(a3) * fact(a4);
        double sign = ((mp - m + s) & 1) ? -1.0 : 1.0;
        int pc = 2 * j + m - mp - 2 * s, ps = mp - m + 2 * s;
        double cpow = 1.0, spow = 1.0;
        for (int i = 0; i < pc; ++i) cpow *= ch;
        for (int i = 0; i < ps; ++i) spow *= sh;
        sum = sum + ((sign * pref / den) * cpow) * spow;
    }
    return sum;
}

__device__ void rotzyz(double a, double b, double g, double R[3][3]) {
    double sa, ca, sb, cb, sg, cg;
    dm_sincos(a, &sa, &ca);
    dm_sincos(b, &sb, &cb);
    dm_sincos(g, &sg, &cg);
    R[0][0] = ca * cb * cg - sa * sg; R[0][1] = -(ca * cb * sg) - sa * cg; R[0][2] = ca * sb;
    R[1][0] = sa * cb * cg + ca * sg; R[1][1] = -(sa * cb * sg) + ca * cg; R[1][2] = sa * sb;
    R[2][0] = -(sb * cg);             R[2][1] = sb * sg;                   R[2][2] = cb;
}

// gen_electron_batch prologue (ADKSampler.jl:168-235, SPANESampler.jl:164-235).
__global__ void k_batch_prepare(const __grid_constant__ DJob J, const double* __restrict__ t,
                                DBatch* __restrict__ out) {
    int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= J.n_t) return;
    DBatch B;
    double tr = t[b];
    B.tr = tr;
    if (J.method == ETRAJ_SAMPLER_SPANE) {
        laser_F_dual(J.laser, tr, B.Fx, B.Fy, B.dFx, B.dFy);
    } else {
        laser_F(J.laser, tr, B.Fx, B.Fy);
        B.dFx = 0.0;
        B.dFy = 0.0;
    }
    B.F = dm_hypot(B.Fx, B.Fy);
    double phi = dm_atan2(-B.Fy, -B.Fx);
    dm_sincos(phi, &B.sphi, &B.cphi);
    double gamma = 0.0;
    if (J.mono) {
        const DMono& M = J.laser.m[0];
        gamma = (M.omega * J.kappa) / (M.F0 * mono_env(M, tr));
    }
    B.c_cc = (J.cc_base * dm_pow_pos(B.F, -J.nstar)) *
             dm_pow_pos(1.0 + (2.0 * gamma) / 2.718281828459045, -J.nstar);
    B.W = B.Fx * B.dFy - B.dFx * B.Fy;
    B.ny0 = B.Fy / B.F;
    B.ny1 = -B.Fx / B.F;
    B.nz0 = B.Fx / B.F;
    B.nz1 = B.Fy / B.F;
    // Euler angles FF -> MF (shared_methods.jl:31-38), MF = RotZYZ(phi_q, theta_q, 0)
    double FF[3][3] = {{0.0, B.Fy / B.F, B.Fx / B.F}, {0.0, -B.Fx / B.F, B.Fy / B.F}, {1.0, 0.0, 0.0}};
    double MF[3][3], M[3][3];
    rotzyz(J.q_phi, J.q_theta, 0.0, MF);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            M[i][j] = (MF[0][i] * FF[0][j] + MF[1][i] * FF[1][j]) + MF[2][i] * FF[2][j];
    double t1 = dm_atan2(M[1][2], M[0][2]);
    double st1, ct1;
    dm_sincos(t1, &st1, &ct1);
    double t2 = dm_atan2(M[0][2] * ct1 + M[1][2] * st1, M[2][2]);
    double t3 = dm_atan2(M[1][0] * ct1 - M[0][0] * st1, M[1][1] * ct1 - M[0][1] * st1);
    for (int mp = -J.l; mp <= J.l; ++mp) {
        double s1, c1, s3, c3;
        dm_sincos(-((double)mp * t1), &s1, &c1);
        dm_sincos(-((double)J.m * t3), &s3, &c3);
        double d = wigner_d(J.l, mp, J.m, t2);
        dm_cplx D = dm_cmul(dm_cscale(dm_c(c1, s1), d), dm_c(c3, s3));
        B.D[2 * (mp + J.l)] = D.re;
        B.D[2 * (mp + J.l) + 1] = D.im;
    }
    B.f.Fx = (float)B.Fx;
    B.f.Fy = (float)B.Fy;
    B.f.dFx = (float)B.dFx;
    B.f.dFy = (float)B.dFy;
    B.f.F = (float)B.F;
    B.f.spa_on = (B.F > 1e-3) ? 1 : 0;
    B.f.sphi = (float)B.sphi;
    B.f.cphi = (float)B.cphi;
    B.f.c_cc = (float)B.c_cc;
    B.f.W = (float)B.W;
    B.f.ny0 = (float)B.ny0;
    B.f.ny1 = (float)B.ny1;
    B.f.nz0 = (float)B.nz0;
    B.f.nz1 = (float)B.nz1;
    for (int i = 0; i < 2 * 9; ++i) B.f.CD[i] = (i < 2 * (2 * J.l + 1)) ? (float)(J.C * B.D[i]) : 0.0f;
    out[b] = B;
}

// Per-time-sample tables of a molecular target: one block per time sample,
// threads over the table's entries (MO-ADK: C_lm D^l_{m' m}; WFAT: |G|^2 of
// each channel and the time-sample factors of W).
// WFAT: the Wigner d values and phase factors of a time sample are computed
// once into shared memory and shared by its channels (G of every n_xi uses the
// same d^l_{m m'}(beta)).
__global__ void __launch_bounds__(128) k_mol_prepare(const __grid_constant__ DJob J, const DBatch* __restrict__ batches) {
    constexpr int L = MOL_MAX_L, W = 2 * MOL_MAX_L + 1;
    __shared__ double s_d[(MOL_MAX_L + 1) * W * W];
    __shared__ double s_cs[2 * W];
    const DMol& M = J.mol;
    for (int64_t b = blockIdx.x; b < J.n_t; b += gridDim.x) {
        const DBatch& B = batches[b];
        double a, be, g;
        mol_euler(M.rot, B.Fx, B.Fy, B.F, &a, &be, &g);
        double* out = M.tab + b * (int64_t)M.stride;
        float* outf = M.tabf + b * (int64_t)M.stride;
        if (M.wfat) {
            __syncthreads();  // the previous time sample's tables are no longer read
            double shb, chb;
            dm_sincos(0.5 * be, &shb, &chb);
            for (int q = threadIdx.x; q < (M.wl + 1) * W * W; q += blockDim.x) {
                const int l = q / (W * W), m = (q / W) % W - L, mp = q % W - L;
                const int am = m < 0 ? -m : m, amp = mp < 0 ? -mp : mp;
                if (am <= l && amp <= l && am <= M.mmax) s_d[q] = mol_wigner_d_sc(l, m, mp, shb, chb);
            }
            for (int q = threadIdx.x; q < W; q += blockDim.x) {
                double sn, cn;
                dm_sincos(-((double)(q - L)) * g, &sn, &cn);
                s_cs[2 * q] = cn;
                s_cs[2 * q + 1] = sn;
            }
            __syncthreads();
            const int nch = (M.nxi + 1) * (2 * M.mmax + 1), na = (M.nxi + 1) * (M.mmax + 1);
            for (int c = threadIdx.x; c < nch + na; c += blockDim.x) {
                if (c < nch) {
                    const int nxi = c % (M.nxi + 1), m = c / (M.nxi + 1) - M.mmax;
                    const dm_cplx G = mol_wfat_G_tab(nxi, m, M.nxi, M.mmax, M.wl, M.wint, M.mu, J.kappa, be, g, s_d, s_cs);
                    out[c] = G.re * G.re + G.im * G.im;
                } else {
                    out[c] = mol_wfat_A(c - nch, M.nxi, J.kappa, J.nstar, B.F);
                }
                outf[c] = (float)out[c];
            }
        } else {
            for (int e = threadIdx.x; e < M.T.ncd; e += blockDim.x) {
                const dm_cplx v = mol_cd_entry(&M.T, M.clm, e, a, be, g);
                out[2 * e] = v.re;
                out[2 * e + 1] = v.im;
                outf[2 * e] = (float)v.re;
                outf[2 * e + 1] = (float)v.im;
            }
        }
    }
}

// Coefficients (-1)^k / (2^(2k+m) (k+m)! k! (l-m-2k)!) of the k-sum below for
// l <= kMaxL, k = max(0, -m) + j (j < 3), rounded at compile time: every factor
// and product is an exact integer, so the one rounding is the correctly
// rounded division the loop used to do per candidate.
struct SphCoef64 {
    double c[kMaxL + 1][2 * kMaxL + 1][3];
};
constexpr double sph_fact64(int n) { return n <= 1 ? 1.0 : (double)n * sph_fact64(n - 1); }
constexpr SphCoef64 sph_coef64_table() {
    SphCoef64 t{};
    for (int l = 0; l <= kMaxL; ++l)
        for (int m = -l; m <= l; ++m) {
            const int kmin = (m < 0) ? -m : 0, kmax = (l - m) / 2;
            for (int k = kmin; k <= kmax && k - kmin < 3; ++k) {
                double p2 = 1.0;
                for (int i = 0; i < 2 * k + m; ++i) p2 *= 2.0;
                t.c[l][m + l][k - kmin] =
                    ((k & 1) ? -1.0 : 1.0) / (p2 * (sph_fact64(k + m) * sph_fact64(k) * sph_fact64(l - m - 2 * k)));
            }
        }
    return t;
}
__constant__ SphCoef64 kSph64 = sph_coef64_table();

// The k-sum of the solid harmonic (shared_methods.jl:21).
__device__ dm_cplx sph_sum(int l, int m, dm_cplx x, dm_cplx y, dm_cplx z) {
    dm_cplx xp = dm_c(x.re - y.im, x.im + y.re);
    dm_cplx xm = dm_c(x.re + y.im, x.im - y.re);
    int kmin = (m < 0) ? -m : 0, kmax = (l - m) / 2;
    dm_cplx acc = dm_c(0.0, 0.0);
    for (int k = kmin; k <= kmax; ++k) {
        const double coef = kSph64.c[l][m + l][k - kmin];
        dm_cplx tt = dm_cscale(dm_cpowi(xp, k + m), coef);
        tt = dm_cmul(tt, dm_cpowi(xm, k));
        tt = dm_cmul(tt, dm_cpowi(z, l - m - 2 * k));
        acc = (k == kmin) ? tt : dm_cadd(acc, tt);
    }
    return acc;
}

// Sum over m' of C D^l_{m' m} Y_{l m'} (ADKSampler.jl:243-265).
// Molecules: sum over (l, m, m') of C_lm D^l_{m' m} Y_{l m'} (mol.h), with
// the time sample's C D table.
__device__ dm_cplx pre_numerator(const DJob& J, const DBatch& B, int64_t b, dm_cplx kx, dm_cplx ky, dm_cplx kz) {
    dm_cplx ckx = dm_cconj(kx), cky = dm_cconj(ky), ckz = dm_cconj(kz);
    dm_cplx nkx = dm_cadd(dm_cadd(dm_cscale(ckx, 0.0), dm_cscale(cky, 0.0)), dm_cscale(ckz, 1.0));
    dm_cplx nky = dm_cadd(dm_cadd(dm_cscale(ckx, B.ny0), dm_cscale(cky, B.ny1)), dm_cscale(ckz, 0.0));
    dm_cplx nkz = dm_cadd(dm_cadd(dm_cscale(ckx, B.nz0), dm_cscale(cky, B.nz1)), dm_cscale(ckz, 0.0));
    if (J.mol.on) return mol_numerator(&J.mol.T, J.mol.tab + b * (int64_t)J.mol.stride, J.mol.P, nkx, nky, nkz);
    dm_cplx acc = dm_c(0.0, 0.0);
    for (int mp = -J.l; mp <= J.l; ++mp) {
        int i = mp + J.l;
        dm_cplx P = dm_c(J.Plm[2 * i], J.Plm[2 * i + 1]);
        dm_cplx Y = dm_cmul(P, sph_sum(J.l, mp, nkx, nky, nkz));
        dm_cplx term = dm_cmul(dm_cscale(dm_c(B.D[2 * i], B.D[2 * i + 1]), J.C), Y);
        acc = (mp == -J.l) ? term : dm_cadd(acc, term);
    }
    return acc;
}

// A Gaussian-proposal Monte-Carlo point (etraj_mc_proposal ADK_GAUSS): kd (and, in
// 3D, kz) normal with the ADK width sigma^2 = F / (2 kappa) at field strength F, by
// Box-Muller from the candidate's two uniforms, and its weight dkdt = dkdt_base /
// pdf(kd) [/ pdf(kz)].  The oracle's o_mc_point evaluates the same expressions.
__device__ __forceinline__ void mc_gauss_point(const DJob& J, double F, double ua, double ub, double* kd0,
                                               double* kz0, double* dkdt) {
    const double sig = sqrt(F / (2.0 * J.kappa));
    const double r = sqrt(-2.0 * dm_log(1.0 - ua));
    double sn, cs;
    dm_sincos(6.283185307179586 * ub, &sn, &cs);
    const double z1 = r * cs, z2 = r * sn;
    const double norm = sig * 2.5066282746310002;  // sigma sqrt(2 pi)
    const double inv2s2 = 1.0 / (2.0 * (sig * sig));
    double w = J.dkdt_base;
    *kd0 = 0.0;
    *kz0 = 0.0;
    if (J.dim != 3 || J.mc_kd_max != 0.0) {
        *kd0 = sig * z1;
        w = w * (norm * dm_exp((*kd0 * *kd0) * inv2s2));
    }
    if (J.dim == 3 && J.mc_kz_max != 0.0) {
        *kz0 = sig * z2;
        w = w * (norm * dm_exp((*kz0 * *kz0) * inv2s2));
    }
    *dkdt = w;
}

__global__ void __launch_bounds__(256)
k_sample(const __grid_constant__ DJob J, int64_t b0, int64_t nb, const double* __restrict__ kdv,
         const double* __restrict__ kzv, const DBatch* __restrict__ batches, InitSoA soa,
         uint8_t* __restrict__ flag) {
    const int64_t total = nb * J.n_cand;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < total;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t bl = q / J.n_cand, i = q - bl * J.n_cand, b = b0 + bl;
        const DBatch& B = batches[b];
        double kd0, kz0, dkdt = J.dkdt;
        if (!J.mc) {
            kd0 = kdv[i / J.n_kz];
            kz0 = kzv[i % J.n_kz];
        } else {
            uint32_t c[4] = {(uint32_t)i, (uint32_t)((uint64_t)i >> 32), (uint32_t)b, 0x4B445A00u};
            philox4x32(c, J.seed);
            double ua = u53(c[0], c[1]), ub = u53(c[2], c[3]);
            if (J.gauss) {
                mc_gauss_point(J, B.F, ua, ub, &kd0, &kz0, &dkdt);
            } else {
                kd0 = ((ua - 0.5) * 2.0) * J.mc_kd_max;
                if (J.dim == 3) {
                    kz0 = ((ub - 0.5) * 2.0) * J.mc_kz_max;
                    if (J.mc_kd_max == 0.0) kd0 = 0.0;
                    else if (J.mc_kz_max == 0.0) kz0 = 0.0;
                } else {
                    kz0 = 0.0;
                }
            }
        }
        uint8_t keep = 0;
        double x0 = 0.0, y0 = 0.0, kx0 = 0.0, ky0 = 0.0, rate = 0.0, ph = 0.0;
        if (J.method == ETRAJ_SAMPLER_WFAT) {
            // WFATSampler.jl:173-240: ADK's exit point, the WFAT rate, CTMC rows
            if (!(kd0 * kd0 + kz0 * kz0 < 1e-4 * 1e-4)) {
                const double F = B.F;
                kx0 = kd0 * (-B.sphi);
                ky0 = kd0 * B.cphi;
                const double r0 = (J.Ip + (kd0 * kd0 + kz0 * kz0) / 2.0) / F;
                x0 = r0 * B.cphi;
                y0 = r0 * B.sphi;
                const double* tb = J.mol.tab + b * (int64_t)J.mol.stride;
                const int nch = (J.mol.nxi + 1) * (2 * J.mol.mmax + 1);
                rate = mol_wfat_rate(J.mol.nxi, J.mol.mmax, tb, tb + nch, J.kappa, F, kd0, kz0, J.dkdt);
                keep = (!(rate != rate) && !(rate < J.cutoff)) ? 1 : 0;
            }
        } else if (!(fabs(kd0) < 1e-4) && !(fabs(kd0) > J.mc_kd_max && J.gauss) &&
                   !(J.gauss && J.dim == 3 && fabs(kz0) > J.mc_kz_max)) {
            // (a Gaussian draw outside +-mc_kd_max, +-mc_kz_max is dropped)
            const double Ip = J.Ip, F = B.F;
            kx0 = kd0 * (-B.sphi);
            ky0 = kd0 * B.cphi;
            const bool spane = (J.method == ETRAJ_SAMPLER_SPANE);
            double F2eff = 0.0, ti, X2, Fexp;
            bool skip = false;
            if (!spane) {
                double r0 = (Ip + (kd0 * kd0 + kz0 * kz0) / 2.0) / F;
                x0 = r0 * B.cphi;
                y0 = r0 * B.sphi;
                ti = sqrt((J.kappa * J.kappa + kd0 * kd0) + kz0 * kz0) / F;
                X2 = (((kx0 * kx0 + ky0 * ky0) + kz0 * kz0) + 2.0 * Ip) * (F * F);
                Fexp = F;
            } else {
                F2eff = F * F - (kx0 * B.dFx + ky0 * B.dFy);
                double Xk = ((kx0 * kx0 + ky0 * ky0) + kz0 * kz0) + 2.0 * Ip;
                double r0 = ((F / 2.0) * Xk) / F2eff;
                x0 = r0 * B.cphi;
                y0 = r0 * B.sphi;
                double lim = J.mc ? (F * F) / 25.0 : (F * F) / 9.0;
                skip = (F2eff <= lim);
                ti = sqrt(((J.kappa * J.kappa + kd0 * kd0) + kz0 * kz0) / F2eff);
                X2 = Xk * F2eff;
                Fexp = sqrt(F2eff);
            }
            if (!skip) {
                double Xe = (kd0 * kd0 + kz0 * kz0) + 2.0 * Ip;
                double E = dm_exp(-(Xe * sqrt(Xe)) / (3.0 * Fexp));
                double r1 = sqrt(dkdt) * E;
                dm_cplx amp;
                if (J.prefix & (ETRAJ_PREFIX_PRE | ETRAJ_PREFIX_PRECC)) {
                    dm_cplx kx, ky, kz = dm_c(kz0, 0.0);
                    if (!spane) {
                        kx = dm_c(kx0, -(ti * B.Fx));
                        ky = dm_c(ky0, -(ti * B.Fy));
                    } else {
                        double h = (ti * ti) / 2.0;
                        kx = dm_c(kx0 + h * B.dFx, -(ti * B.Fx));
                        ky = dm_c(ky0 + h * B.dFy, -(ti * B.Fy));
                    }
                    dm_cplx num = pre_numerator(J, B, b, kx, ky, kz);
                    double cpre = (J.prefix & ETRAJ_PREFIX_PRE) ? J.c : B.c_cc;
                    double den = (J.e_pre == 0.5) ? sqrt(X2) : dm_pow_pos(X2, J.e_pre);
                    dm_cplx pre = dm_cscale(num, cpre);
                    pre = dm_c(pre.re / den, pre.im / den);
                    amp = dm_cscale(pre, r1);
                } else {
                    amp = dm_c(r1, 0.0);
                }
                if (J.prefix & ETRAJ_PREFIX_JAC) {
                    double jac = spane ? fabs(F + (sqrt(kd0 * kd0 + kz0 * kz0) / (F * F)) * B.W) : F;
                    amp = dm_cscale(amp, sqrt(jac));
                }
                rate = amp.re * amp.re + amp.im * amp.im;
                double crit = spane ? rate / dkdt : rate;
                keep = (!(rate != rate) && !(crit < J.cutoff)) ? 1 : 0;
                if (keep && J.phase != ETRAJ_PHASE_CTMC) ph = dm_carg(amp);
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

// ---- order-preserving compaction -------------------------------------------------
constexpr int kCompactThreads = 256;
constexpr int kCompactItems = 8;
constexpr int kCompactChunk = kCompactThreads * kCompactItems;

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* total) {
    __shared__ uint32_t warp_sums[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = (lane < nw) ? warp_sums[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < nw) warp_sums[lane] = w;
    }
    __syncthreads();
    uint32_t base = (warp > 0) ? warp_sums[warp - 1] : 0u;
    if (total) *total = warp_sums[nw - 1];
    uint32_t r = base + x - v;
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(kCompactThreads)
k_compact_count(const uint8_t* __restrict__ flag, int64_t n, uint32_t* __restrict__ block_sums) {
    const int64_t base = (int64_t)blockIdx.x * kCompactChunk + (int64_t)threadIdx.x * kCompactItems;
    uint32_t c = 0;
#pragma unroll
    for (int k = 0; k < kCompactItems; ++k) c += (base + k < n && flag[base + k]) ? 1u : 0u;
    c = __reduce_add_sync(0xffffffffu, c);
    __shared__ uint32_t ws[kCompactThreads / 32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t s = 0;
        for (int w = 0; w < kCompactThreads / 32; ++w) s += ws[w];
        block_sums[blockIdx.x] = s;
    }
}

// Exclusive scan of block_sums in place (one block), total to *count.
__global__ void __launch_bounds__(1024)
k_compact_scan(uint32_t* __restrict__ block_sums, int64_t nblocks, unsigned long long* __restrict__ count) {
    __shared__ unsigned long long carry;
    if (threadIdx.x == 0) carry = 0ull;
    __syncthreads();
    for (int64_t off = 0; off < nblocks; off += blockDim.x) {
        int64_t i = off + threadIdx.x;
        uint32_t v = (i < nblocks) ? block_sums[i] : 0u;
        uint32_t tot;
        uint32_t ex = block_exclusive_scan(v, &tot);
        if (i < nblocks) block_sums[i] = (uint32_t)(carry + ex);
        __syncthreads();
        if (threadIdx.x == 0) carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) *count = carry;
}

__global__ void __launch_bounds__(kCompactThreads)
k_compact_scatter(const uint8_t* __restrict__ flag, int64_t n, const uint32_t* __restrict__ block_off,
                  int64_t* __restrict__ idx) {
    const int64_t base = (int64_t)blockIdx.x * kCompactChunk + (int64_t)threadIdx.x * kCompactItems;
    uint8_t f[kCompactItems];
    uint32_t c = 0;
#pragma unroll
    for (int k = 0; k < kCompactItems; ++k) {
        f[k] = (base + k < n) ? flag[base + k] : 0;
        c += f[k] ? 1u : 0u;
    }
    uint32_t ex = block_exclusive_scan(c, nullptr);
    int64_t pos = (int64_t)block_off[blockIdx.x] + ex;
#pragma unroll
    for (int k = 0; k < kCompactItems; ++k)
        if (f[k]) idx[pos++] = base + k;
}

// One thread per SPA candidate (SPASampler.jl:318-391): the same steps as the
// CPU oracle's o_candidate_spa, in the same order.
__global__ void __launch_bounds__(128)
k_sample_spa(const __grid_constant__ DJob J, int64_t b0, int64_t nb, const double* __restrict__ kdv,
             const double* __restrict__ kzv, const DBatch* __restrict__ batches, InitSoA soa,
             uint8_t* __restrict__ flag, int prefiltered, const int64_t* __restrict__ list,
             const unsigned long long* __restrict__ lcount) {
    // every candidate of the range, or (list) the *lcount candidates it names
    const int64_t total = list ? (int64_t)*lcount : nb * J.n_cand;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < total;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c = list ? list[q] : q;
        const int64_t bl = c / J.n_cand, i = c - bl * J.n_cand, b = b0 + bl;
        // a candidate the FP32 pre-pass dropped (flag 0) keeps flag 0
        if (!list && prefiltered && flag[b * J.n_cand + i] == 0) continue;
        const DBatch& B = batches[b];
        double kd0, kz0;
        if (!J.mc) {
            kd0 = kdv[i / J.n_kz];
            kz0 = kzv[i % J.n_kz];
        } else {
            uint32_t c[4] = {(uint32_t)i, (uint32_t)((uint64_t)i >> 32), (uint32_t)b, 0x4B445A00u};
            philox4x32(c, J.seed);
            double ua = u53(c[0], c[1]), ub = u53(c[2], c[3]);
            kd0 = ((ua - 0.5) * 2.0) * J.mc_kd_max;
            if (J.dim == 3) {
                kz0 = ((ub - 0.5) * 2.0) * J.mc_kz_max;
                if (J.mc_kd_max == 0.0) kd0 = 0.0;
                else if (J.mc_kz_max == 0.0) kz0 = 0.0;
            } else {
                kz0 = 0.0;
            }
        }
        uint8_t keep = 0;
        double x0 = 0.0, y0 = 0.0, kx0 = 0.0, ky0 = 0.0, rate = 0.0, ph = 0.0;
        const double tr = B.tr, Ip = J.Ip;
        if (B.F > 1e-3 && !(fabs(kd0) < 1e-4)) {
            const double w = J.spa_omega, wF = w / B.F;
            const double guess = dm_asinh(wF * sqrt((kd0 * kd0 + kz0 * kz0) + 2.0 * Ip)) / w;
            spa_win W;
            spa_win_init(&W);
            const double ti = spa_solve_ti(&J.laser, &W, tr, kd0, kz0, Ip, guess);
            if (ti != 0.0) {
                dm_cplx Ax, Ay, Fx, Fy;
                laser_AF_complex(J.laser, dm_c(tr, ti), Ax, Ay, &Fx, &Fy);
                double px, py;
                spa_pxy(kd0, Ax, Ay, &px, &py);
                spa_quad_par Q;
                Q.L = &J.laser;
                Q.W = &W;
                Q.tr = tr;
                Q.px = px;
                Q.py = py;
                Q.kz = kz0;
                Q.Ip = Ip;
                int ok2;
                const dm_cplx Si = spa_quadgk(SPA_INT_ACTION, &Q, dm_c(tr, ti), dm_c(tr, 0.0), &ok2);
                // the exit position (two quadratures) is computed after the rate, for
                // the candidates it keeps only; a failed quadrature drops the candidate
                // as before, and no value changes
                if (ok2) {
                    const dm_cplx St = dm_cneg(Si);
                    const dm_cplx iS = dm_c(0.0 * St.re - 1.0 * St.im, 0.0 * St.im + 1.0 * St.re);
                    dm_cplx amp = dm_cscale(dm_cexp(iS), sqrt(J.dkdt));
                    if (J.prefix & (ETRAJ_PREFIX_PRE | ETRAJ_PREFIX_PRECC)) {
                        const dm_cplx kx = dm_c(px + Ax.re, Ax.im), ky = dm_c(py + Ay.re, Ay.im);
                        const dm_cplx num = pre_numerator(J, B, b, kx, ky, dm_c(kz0, 0.0));
                        const double cpre = (J.prefix & ETRAJ_PREFIX_PRE) ? J.c : B.c_cc;
                        const dm_cplx kF = dm_caddr(dm_cadd(dm_cmul(kx, Fx), dm_cmul(ky, Fy)), kz0 * 0.0);
                        const dm_cplx den = spa_cpow(kF, (J.nstar + 1.0) / 2.0);
                        amp = dm_cmul(amp, dm_cdiv(dm_cscale(num, cpre), den));
                    }
                    if (J.prefix & ETRAJ_PREFIX_JAC) amp = dm_cscale(amp, sqrt(spa_jac(&J.laser, &W, tr, kd0, kz0, Ip, wF, w)));
                    rate = amp.re * amp.re + amp.im * amp.im;
                    keep = (!(rate != rate) && !(rate < J.cutoff)) ? 1 : 0;
                    if (keep) {
                        int ok01;
                        spa_exit(&Q, ti, &x0, &y0, &ok01);
                        keep = ok01 ? 1 : 0;
                        double axr, ayr;
                        laser_A(J.laser, tr, axr, ayr);
                        kx0 = px + axr;
                        ky0 = py + ayr;
                    }
                    if (keep && J.phase != ETRAJ_PHASE_CTMC) ph = dm_carg(amp);
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

}  // namespace

int launch_batch_prepare(const DJob& J, const double* t, DBatch* batches, cudaStream_t s) {
    int threads = 64;  // few, FP64-heavy threads: spread them over every SM
    int blocks = (int)((J.n_t + threads - 1) / threads);
    k_batch_prepare<<<blocks, threads, 0, s>>>(J, t, batches);
    if (!J.mol.on) return 1;
    const int64_t mb = J.n_t < ((int64_t)1 << 20) ? J.n_t : ((int64_t)1 << 20);
    k_mol_prepare<<<(unsigned)(mb > 0 ? mb : 1), 128, 0, s>>>(J, batches);
    return 2;
}

int launch_sample_range(const DJob& J, int64_t b0, int64_t nb, const double* kd, const double* kz,
                        DBatch* batches, InitSoA soa, uint8_t* flag, int sm_count,
                        cudaStream_t s, const SampleScratch* scr) {
    if (J.method == ETRAJ_SAMPLER_SPA) {
        // atoms: an FP32 pre-pass marks the candidates below the cutoff (by the
        // margin scr gives, else 100 times below), and a compaction lists the
        // others (with scr), so the FP64 kernel's warps hold only candidates it may
        // keep; without a list it skips the marked ones in place (molecules: every
        // candidate in FP64)
        const int pre = J.mol.on ? 0 : 1;
        const bool listed = pre && scr && compact_blocks(nb * J.n_cand) + 1 <= scr->block_cap;
        const float log_margin = scr ? scr->log_margin : -4.6051702f;  // log(1/100)
        int launches = pre ? launch_spa_prefilter(J, b0, nb, kd, kz, batches, log_margin, flag, sm_count, s) : 0;
        if (listed)
            launches += launch_compact(flag + b0 * J.n_cand, nb * J.n_cand, scr->list, scr->block_sums,
                                       scr->block_cap, scr->count, s);
        const int threads = 128;
        const int64_t want = (nb * J.n_cand + threads - 1) / threads;
        const int64_t cap = (int64_t)sm_count * 64;
        const int blocks = (int)(want < cap ? (want > 0 ? want : 1) : cap);
        k_sample_spa<<<blocks, threads, 0, s>>>(J, b0, nb, kd, kz, batches, soa, flag, pre,
                                                 listed ? scr->list : nullptr, listed ? scr->count : nullptr);
        return launches + 1;
    }
    int threads = 256;
    int64_t want = (nb * J.n_cand + threads - 1) / threads;
    int64_t cap = (int64_t)sm_count * 32;
    int blocks = (int)(want < cap ? (want > 0 ? want : 1) : cap);
    k_sample<<<blocks, threads, 0, s>>>(J, b0, nb, kd, kz, batches, soa, flag);
    return 1;
}

int64_t compact_blocks(int64_t n) { return (n + kCompactChunk - 1) / kCompactChunk; }

int launch_compact(const uint8_t* flag, int64_t n, int64_t* idx, uint32_t* block_sums,
                   int64_t nblocks_cap, unsigned long long* count, cudaStream_t s) {
    int64_t nb = compact_blocks(n);
    if (nb > nblocks_cap || nb == 0) {
        cudaMemsetAsync(count, 0, sizeof(unsigned long long), s);
        return 0;
    }
    k_compact_count<<<(unsigned)nb, kCompactThreads, 0, s>>>(flag, n, block_sums);
    k_compact_scan<<<1, 1024, 0, s>>>(block_sums, nb, count);
    k_compact_scatter<<<(unsigned)nb, kCompactThreads, 0, s>>>(flag, n, block_sums, idx);
    return 3;
}

}  // namespace etraj
