// api.cu -- the C ABI of include/etraj.h: contexts, validation, host-side job
// set-up and the orchestration of the device pipeline.
//
// Pipeline of etraj_run (all launches on the context's stream, one host
// synchronization at the end):
//   k_batch_prepare  per time sample   (gen_electron_batch prologue)
//   k_sample         per candidate     (gen_electron_batch loop body)
//   compaction       order-preserving survivor list
//   k_integrate_*    per survivor      (Tsit5 solve + collection)
//   deposit          radix sort + segmented sums + canonical reductions
// This replaces the `@threads for i in 1:batch_num` loop of
// src/TrajectorySimulation.jl:154-157 and the reduction of write_output!
// (:521-543).

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <chrono>
#include <deque>
#include <mutex>
#include <thread>
#include <string>
#include <vector>

#include "engine.h"
#include "integrate_setup.h"
#include "mol_check.h"

using namespace etraj;

#define ETRAJ_VERSION_STRING "etraj-gb300 1.0 (sm_103a)"

namespace {

constexpr bool kHaveFp32Bulk = true;

// ---- host-side job set-up (same expressions as the reference's getters) ----------
double fact(int n) {
    double f = 1.0;
    for (int i = 2; i <= n; ++i) f *= (double)i;
    return f;
}

// Prefactor of the solid harmonic Y_{l m} of shared_methods.jl:21.
dm_cplx sph_prefactor(int l, int m, double kappa) {
    double A = (m & 1) ? -1.0 : 1.0;
    double B = std::sqrt((((2.0 * l + 1.0) / 12.566370614359172) * fact(l - m)) / fact(l + m));
    dm_cplx C = dm_cpowi(dm_c(0.0, -kappa), l);
    dm_cplx P = dm_cdiv(dm_c(A * B, 0.0), C);
    return dm_cscale(P, fact(l + m));
}

void two_sum(double a, double b, double* s, double* e) {
    double ss = a + b, bb = ss - a;
    *s = ss;
    *e = (a - (ss - bb)) + (b - bb);
}

// Element i (0-based) of Julia's range(a, b; length=n).
double linrange(double a, double b, int64_t n, int64_t i) {
    if (n == 1 || i == 0) return a;
    if (i == n - 1) return b;
    double lim = 4503599627370496.0 / (double)n;
    if (a == std::rint(a) && b == std::rint(b) && std::fabs(a) < lim && std::fabs(b) < lim)
        return (a * (double)(n - 1 - i) + b * (double)i) / (double)(n - 1);
    double dh, dl, m = (double)(n - 1), fi = (double)i;
    two_sum(b, -a, &dh, &dl);
    double q1 = dh / m;
    double r = std::fma(-q1, m, dh) + dl;
    double q2 = r / m;
    double p1 = fi * q1, p1e = std::fma(fi, q1, -p1);
    double p2 = fi * q2;
    double s, se;
    two_sum(a, p1, &s, &se);
    return s + (se + (p1e + p2));
}

void philox_host(uint32_t c[4], uint64_t seed) {
    uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0;
        uint32_t n1 = (uint32_t)p1;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
        uint32_t n3 = (uint32_t)p0;
        c[0] = n0; c[1] = n1; c[2] = n2; c[3] = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}

double u53_host(uint32_t a, uint32_t b) {
    return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) * (1.0 / 9007199254740992.0);
}

struct HostJob {
    DJob J;
    std::vector<double> t, kd, kz;
    std::vector<double> mol_clm, mol_wint;  // molecular target: copies of the caller's tables
};

// The sampler's name as the reference's messages carry it (ADKSampler.jl:79-102,
// SPANESampler.jl:101-124, SPASampler.jl:79-102 share their checks).
const char* sampler_tag(int method) {
    switch (method) {
        case ETRAJ_SAMPLER_SPANE: return "[SPANESampler]";
        case ETRAJ_SAMPLER_SPA: return "[SPASampler]";
        case ETRAJ_SAMPLER_WFAT: return "[WFATSampler]";
        default: return "[ADKSampler]";
    }
}

int validate_job(const etraj_job* job, std::string& err) {
    auto fail = [&](const char* m) {
        err = m;
        if (job && err.compare(0, 12, "[ADKSampler]") == 0) err.replace(0, 12, sampler_tag(job->init_cond_method));
        return (int)ETRAJ_ERR_INVALID_ARGUMENT;
    };
    if (!job) return fail("job is NULL");
    if (!(job->sample_t_intv[0] < job->sample_t_intv[1]))
        return fail("[TrajectorySimulationJob] `sample_t_intv` must be a valid interval.");
    if (!(job->traj_t_final > job->sample_t_intv[1]))
        return fail("[TrajectorySimulationJob] `traj_t_final` must be greater than the last time point of `sample_t_intv`.");
    if (job->dimension != 2 && job->dimension != 3)
        return fail("[TrajectorySimulationJob] `dimension` must be either 2 or 3.");
    if (job->init_cond_method != ETRAJ_SAMPLER_ADK && job->init_cond_method != ETRAJ_SAMPLER_SPANE &&
        job->init_cond_method != ETRAJ_SAMPLER_SPA && job->init_cond_method != ETRAJ_SAMPLER_WFAT)
        return fail("[ElectronSamplers] Undefined initial condition method.");
    if (job->traj_phase_method < 0 || job->traj_phase_method > 2)
        return fail("[ADKSampler] Undefined phase method.");
    if (job->precision == ETRAJ_PRECISION_FP32_BULK && !kHaveFp32Bulk) {
        err = "the FP32-bulk integrator is not built in this library.";
        return ETRAJ_ERR_UNSUPPORTED;
    }
    if (job->precision != ETRAJ_PRECISION_FP64 && job->precision != ETRAJ_PRECISION_FP32_BULK &&
        job->precision != ETRAJ_PRECISION_FP32_DF)
        return fail("unknown precision.");
    if (job->mc_kt_proposal != ETRAJ_PROPOSAL_UNIFORM && job->mc_kt_proposal != ETRAJ_PROPOSAL_ADK_GAUSS)
        return fail("unknown mc_kt_proposal.");
    if (job->mc_kt_proposal == ETRAJ_PROPOSAL_ADK_GAUSS &&
        (!job->sample_monte_carlo ||
         (job->init_cond_method != ETRAJ_SAMPLER_ADK && job->init_cond_method != ETRAJ_SAMPLER_SPANE)))
        return fail("mc_kt_proposal ADK_GAUSS applies to Monte-Carlo ADK and SPANE sampling only.");
    if (job->rate_prefix & ~7) return fail("[ADKSampler] Undefined tunneling rate prefix.");
    if ((job->rate_prefix & ETRAJ_PREFIX_PRE) && (job->rate_prefix & ETRAJ_PREFIX_PRECC))
        return fail("[ADKSampler] Rate prefixes [Pre] & [PreCC] conflict.");
    if (!(job->sample_t_num > 0)) return fail("[ADKSampler] Invalid time sample number.");
    if (!(job->sample_cutoff_limit >= 0)) return fail("[ADKSampler] Invalid cut-off limit.");
    if (!job->sample_monte_carlo) {
        if (job->dimension == 3) {
            if (!(job->ss_kd_num > 0 && job->ss_kz_num > 0)) return fail("[ADKSampler] Invalid kd,kz sample number.");
            if (!(job->ss_kd_max > 0 || job->ss_kz_max > 0))
                return fail("[ADKSampler] Invalid kd,kz sample boundaries (cannot be zero simultaneously).");
            if (job->ss_kz_num == 1 && job->ss_kz_max != 0)
                return fail("range(-abs(ss_kz_max), abs(ss_kz_max); length=1): endpoints differ.");
        } else {
            if (!(job->ss_kd_num > 0)) return fail("[ADKSampler] Invalid kd sample number.");
            if (!(job->ss_kd_max > 0)) return fail("[ADKSampler] Invalid kd sample boundaries.");
        }
        // Julia's range(a, b; length=1) needs a == b (ADKSampler.jl:85,97)
        if (job->ss_kd_num == 1 && job->ss_kd_max != 0)
            return fail("range(-abs(ss_kd_max), abs(ss_kd_max); length=1): endpoints differ.");
    } else {
        if (!(job->mc_kt_num > 0)) return fail("[ADKSampler] Invalid sampling kt_num.");
        if (job->dimension == 3) {
            if (!(job->mc_kd_max > 0 || job->mc_kz_max > 0))
                return fail("[ADKSampler] Invalid kd,kz sample boundaries (cannot be zero simultaneously).");
        } else if (!(job->mc_kd_max > 0)) {
            return fail("[ADKSampler] Invalid kd sample boundaries.");
        }
    }
    int64_t grid = 1;
    for (int d = 0; d < job->dimension; ++d) {
        if (job->final_p_num[d] < 1) return fail("[TrajectorySimulationJob] `final_p_num` must be positive.");
        if (job->final_p_num[d] > 1 && !(job->final_p_max[d] > 0))
            return fail("[TrajectorySimulationJob] `final_p_max` must be positive.");
        grid *= job->final_p_num[d];
    }
    if (grid >= (int64_t)0xFFFFFFFFll) return fail("momentum grid too large (>= 2^32 bins).");
    const etraj_target& T = job->target;
    const char* mmsg = nullptr;
    const int mst = etraj_mol_check(job, &mmsg);
    if (mst > 0) {
        err = mmsg;
        return mst;
    }
    if (mst < 0) {
        if (!(T.Ip > 0)) return fail("[SAEAtom] Ip should be positive.");
        if (!(T.l >= 0 && T.l >= std::abs(T.m))) return fail("[SAEAtom] Invalid (l,m).");
        if (T.l > kMaxL) {
            err = "angular quantum number l > 4 is not supported.";
            return ETRAJ_ERR_UNSUPPORTED;
        }
        if (!(T.asymp_coeff > 0))
            return fail("[SAEAtom] asymp_coeff should be either `:hartree` or a positive number.");
    }
    if (T.kind == ETRAJ_TARGET_MOLECULE) {
        // trajectories: Coulomb tail with soft core 1.0 (GenericMolecule.jl:444-445)
    } else if (T.kind == ETRAJ_TARGET_SAE) {
        if (!(T.b1 >= 0 && T.b2 >= 0 && T.b3 >= 0)) return fail("[SAEAtom] b1,b2,b3 should be non-negative.");
        if (!(T.soft_core > 0)) return fail("[SAEAtom] soft_core should be positive.");
    } else if (T.kind == ETRAJ_TARGET_HYDROGEN_LIKE) {
        if (!(T.soft_core >= 0)) return fail("[HydrogenLikeAtom] `soft_core` should be non-negative.");
    } else {
        return fail("Unknown target kind.");
    }
    if (job->laser.kind < 0 || job->laser.kind > 3) return fail("Unknown laser kind.");
    int nm = (job->laser.kind == ETRAJ_LASER_BICHROMATIC) ? 2 : 1;
    for (int i = 0; i < nm; ++i) {
        const etraj_mono_laser& L = job->laser.mono[i];
        if (L.kind < 0 || L.kind > 2) return fail("Unknown monochromatic laser kind.");
        if (!(L.wave_len > 0)) return fail("[Cos4Laser] Must specify either `wave_len` or `ang_freq`.");
        if (!(L.cyc_num > 0)) return fail("[Cos4Laser] Must specify either `cyc_num` or `duration`.");
    }
    if (!(job->traj_rtol > 0)) return fail("`traj_rtol` must be positive.");
    int64_t ncand = job->sample_monte_carlo ? job->mc_kt_num
                                            : job->ss_kd_num * ((job->dimension == 3) ? job->ss_kz_num : 1);
    if ((double)ncand * (double)job->sample_t_num >= 4.0e9)
        return fail("more than 4e9 candidate electrons in one job; split the job.");
    if (job->precision == ETRAJ_PRECISION_FP32_BULK) {
        // the bulk integrator's clock counts field-table intervals of T/512 in FP32
        double T = 6.283185307179586 * job->laser.mono[0].wave_len / 45.563352525;
        if (nm == 2) T = std::min(T, 6.283185307179586 * job->laser.mono[1].wave_len / 45.563352525);
        const double span = (job->traj_t_final - job->sample_t_intv[0]) / (T / 512.0);
        if (!(span < (double)(1 << 21) - 8.0)) {
            err = "the FP32-bulk integrator covers at most 4096 laser periods from the first time sample "
                  "to traj_t_final; use FP64 precision.";
            return ETRAJ_ERR_UNSUPPORTED;
        }
    }
    if (job->precision == ETRAJ_PRECISION_FP32_DF) {
        // the double-float integrator's clock counts field-table intervals of T/1024 below 2^24
        double T = 6.283185307179586 * job->laser.mono[0].wave_len / 45.563352525;
        if (nm == 2) T = std::min(T, 6.283185307179586 * job->laser.mono[1].wave_len / 45.563352525);
        const double span = (job->traj_t_final - job->sample_t_intv[0]) / (T / (double)kDfTablePerPeriod);
        if (!(span < (double)(1 << 24) - 8.0)) {
            err = "the double-float integrator covers at most 16000 laser periods from the first time sample "
                  "to traj_t_final; use FP64 precision.";
            return ETRAJ_ERR_UNSUPPORTED;
        }
    }
    return ETRAJ_OK;
}

void prepare_job(const etraj_job* job, HostJob& H) {
    DJob& J = H.J;
    std::memset(&J, 0, sizeof J);
    J.method = job->init_cond_method;
    J.dim = job->dimension;
    J.mc = job->sample_monte_carlo ? 1 : 0;
    int p = job->rate_prefix;
    if ((p & ETRAJ_PREFIX_PRECC) && job->laser.kind == ETRAJ_LASER_BICHROMATIC)
        p = (p & ~ETRAJ_PREFIX_PRECC) | ETRAJ_PREFIX_PRE;  // ADKSampler.jl:72-77
    J.prefix = p;
    J.phase = job->traj_phase_method;
    J.rows = (J.dim == 3) ? ((J.phase == ETRAJ_PHASE_CTMC) ? 8 : 9) : ((J.phase == ETRAJ_PHASE_CTMC) ? 6 : 7);
    J.n_state = (J.dim == 3 ? 6 : 4) + (J.phase != ETRAJ_PHASE_CTMC ? 1 : 0);
    J.mono = (job->laser.kind != ETRAJ_LASER_BICHROMATIC) ? 1 : 0;
    J.cutoff = job->sample_cutoff_limit;
    J.seed = job->seed;
    prepare_integration(job, J);  // laser, target, rtol, t_final
    // the SPA initial guess uses the laser's omega, or the mean of the two (SPASampler.jl:160-166)
    J.spa_omega = (J.laser.nmono == 2) ? (J.laser.m[0].omega + J.laser.m[1].omega) / 2.0 : J.laser.m[0].omega;
    const etraj_target& T = job->target;
    J.Ip = T.Ip;
    J.Z = (double)T.Z;
    J.l = T.l;
    J.m = T.m;
    J.C = T.asymp_coeff;
    if (T.kind == ETRAJ_TARGET_MOLECULE) {
        // GenericMolecule's trajectories are the hydrogen-like equations with
        // Z = charge + 1, soft core 1.0 and the phase's Ip = IonPotential(mol)
        // (GenericMolecule.jl:438-445); the sampler uses the orbital's Ip (J.Ip)
        // (the trajectories' target is set by prepare_integration)
        J.l = 0;
        J.m = 0;
        J.C = 0.0;
        DMol& M = J.mol;
        M.on = 1;
        M.wfat = (J.method == ETRAJ_SAMPLER_WFAT) ? 1 : 0;
        for (int i = 0; i < 3; ++i) {
            M.rot[i] = T.mol_rot[i];
            M.mu[i] = T.wfat_mu[i];
        }
        const double kap = std::sqrt(2.0 * T.Ip);
        if (M.wfat) {
            M.nxi = T.wfat_nxi_max;
            M.mmax = T.wfat_m_max;
            M.wl = T.wfat_lmax;
            const size_t n = (size_t)(M.nxi + 1) * (size_t)(2 * M.mmax + 1) * (size_t)(M.wl + 1) * (size_t)(2 * M.wl + 1);
            H.mol_wint.assign(T.wfat_intdata, T.wfat_intdata + 2 * n);
            M.stride = (M.nxi + 1) * (2 * M.mmax + 1) + (M.nxi + 1) * (M.mmax + 1);
        } else {
            const int L = T.asymp_lmax;
            H.mol_clm.assign(T.asymp_coeff_lm, T.asymp_coeff_lm + 2 * (size_t)(L + 1) * (size_t)(2 * L + 1));
            mol_terms_build(L, H.mol_clm.data(), &M.T);
            for (int l = 0; l <= L; ++l)
                for (int mp = -l; mp <= l; ++mp) {
                    const dm_cplx P = mol_sph_prefactor(l, mp, kap);
                    M.P[2 * (l * l + l + mp)] = P.re;
                    M.P[2 * (l * l + l + mp) + 1] = P.im;
                    M.Pf[2 * (l * l + l + mp)] = (float)P.re;
                    M.Pf[2 * (l * l + l + mp) + 1] = (float)P.im;
                }
            M.stride = std::max(2 * M.T.ncd, 2);
        }
    }
    J.q_theta = T.quan_ax_theta;
    J.q_phi = T.quan_ax_phi;
    J.kappa = std::sqrt(2.0 * J.Ip);
    J.nstar = J.Z / J.kappa;
    const double n = J.nstar;
    J.c = (dm_pow_pos(2.0, n / 2.0 + 1.0) * dm_pow_pos(J.kappa, 2.0 * n + 0.5)) * std::tgamma(n / 2.0 + 1.0);
    J.cc_base = dm_pow_pos(2.0, (3.0 * n) / 2.0 + 1.0) * dm_pow_pos(J.kappa, 5.0 * n + 0.5);
    J.e_pre = (n + 1.0) / 4.0;
    for (int mp = -J.l; mp <= J.l; ++mp) {
        dm_cplx P = sph_prefactor(J.l, mp, J.kappa);
        J.Plm[2 * (mp + J.l)] = P.re;
        J.Plm[2 * (mp + J.l) + 1] = P.im;
        J.fPlm[2 * (mp + J.l)] = (float)P.re;
        J.fPlm[2 * (mp + J.l) + 1] = (float)P.im;
    }
    // time samples: range(t1, t2; length=n) or sort!(rand(n)*(t2-t1) .+ t1)  (ADKSampler.jl:136,141)
    J.n_t = job->sample_t_num;
    H.t.resize((size_t)J.n_t);
    const double t1 = job->sample_t_intv[0], t2 = job->sample_t_intv[1];
    if (!J.mc) {
        for (int64_t j = 0; j < J.n_t; ++j) H.t[(size_t)j] = linrange(t1, t2, J.n_t, j);
    } else {
        const double span = t2 - t1;
        for (int64_t j = 0; j < J.n_t; ++j) {
            uint32_t c[4] = {(uint32_t)j, (uint32_t)((uint64_t)j >> 32), 0u, 0x54494D45u};
            philox_host(c, job->seed);
            H.t[(size_t)j] = u53_host(c[0], c[1]) * span + t1;
        }
        std::sort(H.t.begin(), H.t.end());
    }
    const double t_step = (H.t.back() - H.t.front()) / (double)J.n_t;  // ADKSampler.jl:267
    if (!J.mc) {
        int64_t nkd = job->ss_kd_num, nkz = (J.dim == 3) ? job->ss_kz_num : 1;
        double kdm = std::fabs(job->ss_kd_max), kzm = (J.dim == 3) ? std::fabs(job->ss_kz_max) : 0.0;
        J.n_kd = nkd;
        J.n_kz = nkz;
        H.kd.resize((size_t)nkd);
        H.kz.resize((size_t)nkz);
        for (int64_t i = 0; i < nkd; ++i) H.kd[(size_t)i] = linrange(-kdm, kdm, nkd, i);
        for (int64_t i = 0; i < nkz; ++i) H.kz[(size_t)i] = linrange(-kzm, kzm, nkz, i);
        double kd_step = (nkd > 1) ? (kdm - (-kdm)) / (double)nkd : 1.0;
        double kz_step = (J.dim == 3 && nkz > 1) ? (kzm - (-kzm)) / (double)nkz : 1.0;
        J.dkdt = (t_step * kd_step) * kz_step;
        J.n_cand = nkd * nkz;
    } else {
        J.mc_kd_max = job->mc_kd_max;
        J.mc_kz_max = job->mc_kz_max;
        double kd_span = (job->mc_kd_max > 0.0) ? 2.0 * job->mc_kd_max : 1.0;
        double kz_span = (job->mc_kz_max > 0.0) ? 2.0 * job->mc_kz_max : 1.0;
        J.dkdt = ((t_step * kd_span) * kz_span) / (double)job->mc_kt_num;
        J.gauss = (job->mc_kt_proposal == ETRAJ_PROPOSAL_ADK_GAUSS) ? 1 : 0;
        J.dkdt_base = (J.dim == 3 ? t_step : t_step * kz_span) / (double)job->mc_kt_num;
        J.n_cand = job->mc_kt_num;
        J.n_kd = 1;
        J.n_kz = 1;
        H.kd.assign(1, 0.0);
        H.kz.assign(1, 0.0);
    }
    J.n_total = J.n_t * J.n_cand;
    FJobConst& fc = J.fc;
    fc.Ip = (float)J.Ip;
    fc.kap2 = (float)(J.kappa * J.kappa);
    fc.dkdt = (float)J.dkdt;
    fc.sqdkdt = (float)std::sqrt(J.dkdt);
    fc.inv_dkdt = (float)(1.0 / J.dkdt);
    fc.log_dkdt = (float)std::log(J.dkdt);
    fc.cutoff = (float)J.cutoff;
    fc.e_pre = (float)J.e_pre;
    fc.c = (float)J.c;
    fc.e_half = (float)((J.nstar + 1.0) / 2.0);
    fc.spa_omega = (float)J.spa_omega;
    fc.kd_max = (float)J.mc_kd_max;
    fc.kz_max = (float)J.mc_kz_max;
    fc.kd_zero = (J.mc_kd_max == 0.0) ? 1 : 0;
    fc.kz_zero = (J.mc_kz_max == 0.0) ? 1 : 0;
    J.grid = 1;
    for (int d = 0; d < 3; ++d) {
        if (d < J.dim) {
            J.pmax[d] = job->final_p_max[d];
            J.pnum[d] = job->final_p_num[d];
            J.binw[d] = (J.pmax[d] / (double)J.pnum[d]) * 2.0;
            J.grid *= J.pnum[d];
        } else {
            J.pnum[d] = 1;
        }
    }
}

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
};

// One enqueued job.  Its results land either straight in the caller's
// buffers (synchronous etraj_run) or in a pinned staging block that is copied
// out when the job completes (asynchronous submit and the server).
struct JobRec {
    uint64_t ticket = 0;         // 0: etraj_run's job
    int status = ETRAJ_OK;       // enqueue status; an error completes the job at once
    std::string error;
    etraj_result res{};          // the caller's output pointers; scalars filled at completion
    int64_t grid = 0;
    bool coherent = false;
    int launches = 0;
    bool staged = false;
    void* pinned = nullptr;      // staged: sums[2] | Counters | mspec[grid] | amplitude[2 grid]
    size_t pinned_bytes = 0;
    cudaEvent_t ev_start = nullptr, ev_done = nullptr;
    double direct_sums[2] = {0.0, 0.0};
    Counters direct_cnt{};
};

struct PinnedBlock {
    void* p = nullptr;
    size_t bytes = 0;
};

// Launch shape of the bulk integrator.
struct BulkTile {
    int threads, blocks_per_sm, refill_min, occ;
    int chunk;  // step chunk: round 0's step budget per electron (round r: chunk 16^r)
};

}  // namespace

struct etraj_ctx {
    int device = 0;
    int sm_count = 152;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    size_t budget = 0;
    size_t used = 0;
    std::string err;
    std::map<std::string, DevBuf> bufs;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // stage boundaries of the last etraj_run: sample | compact | field table |
    // integrate | collect | deposit
    static constexpr int kStages = 6;
    cudaEvent_t stage_ev[kStages + 1] = {};
    bool stage_valid = false;
    uint64_t next_ticket = 1;
    std::map<uint64_t, JobRec> jobs;       // asynchronous tickets of this context
    // per-survivor final states of the last job, kept with etraj_set_keep_final_states
    bool keep_states = false;
    bool dump_valid = false;
    uint64_t dump_ticket = 0;
    TrajOut dump_out{};
    const unsigned long long* dump_count = nullptr;
    std::vector<PinnedBlock> pinned_pool;  // staging blocks for reuse
    std::vector<cudaEvent_t> event_pool;
    // CUDA-graph replay of the per-job kernel sequence (opt-in): the graph of
    // the last captured job and the launch parameters it was captured with
    bool graphs = true;   // CUDA-graph replay of kernel sequences that repeat
    bool capturing = false;
    cudaGraphExec_t gexec = nullptr;
    std::vector<unsigned char> gkey;
    int glaunches = 0;
    cudaGraphExec_t bgexec = nullptr;  // the last multi-instance batch's graph
    std::vector<unsigned char> bgkey;
    int bglaunches = 0;
    std::vector<unsigned char> gseen, bgseen;  // the last keys run without a graph
    // bulk-integrator launch shapes chosen by the autotuner, per kernel variant
    bool autotune = true;
    bool repack = true;  // the bulk integrator's rounds with parking of long-running electrons
    bool static_assign = false;  // the bulk integrator with one electron per lane, no work stealing
    std::map<int, BulkTile> tiles;
    // sizing without allocating: ensure() only adds up the growth
    bool dry = false;
    size_t dry_bytes = 0;
    std::mutex mu;
};

namespace {

int set_err(etraj_ctx* ctx, int code, const std::string& msg) {
    if (ctx) ctx->err = msg;
    return code;
}

int cuda_err(etraj_ctx* ctx, cudaError_t e, const char* where) {
    return set_err(ctx, ETRAJ_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

// Grow-only named device buffer, counted against the context's HBM budget.
int ensure(etraj_ctx* ctx, const char* name, size_t bytes, void** out) {
    if (bytes == 0) bytes = 256;
    if (ctx->dry) {
        auto it = ctx->bufs.find(name);
        const size_t have = (it == ctx->bufs.end()) ? 0 : it->second.bytes;
        if (have < bytes) ctx->dry_bytes += (bytes + bytes / 8) - have;
        *out = nullptr;
        return ETRAJ_OK;
    }
    DevBuf& b = ctx->bufs[name];
    if (b.bytes >= bytes) {
        *out = b.p;
        return ETRAJ_OK;
    }
    size_t grow = bytes + bytes / 8;
    if (ctx->used - b.bytes + grow > ctx->budget) {
        grow = bytes;
        if (ctx->used - b.bytes + grow > ctx->budget)
            return set_err(ctx, ETRAJ_ERR_OUT_OF_MEMORY,
                           std::string("HBM budget exceeded allocating ") + name + " (" +
                               std::to_string(bytes) + " bytes; budget " + std::to_string(ctx->budget) +
                               ", in use " + std::to_string(ctx->used) + ")");
    }
    // stream-ordered (de)allocation: a context's growth never waits for the
    // work of other contexts (cudaFree would synchronize the whole device)
    if (b.p) {
        cudaFreeAsync(b.p, ctx->stream);
        ctx->used -= b.bytes;
        b.p = nullptr;
        b.bytes = 0;
    }
    cudaError_t e = cudaMallocAsync(&b.p, grow, ctx->stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_err(ctx, ETRAJ_ERR_OUT_OF_MEMORY, std::string("cudaMalloc ") + name + ": " + cudaGetErrorString(e));
    }
    b.bytes = grow;
    ctx->used += grow;
    *out = b.p;
    return ETRAJ_OK;
}

template <typename T>
int ensure_t(etraj_ctx* ctx, const char* name, size_t count, T** out) {
    void* p = nullptr;
    int st = ensure(ctx, name, count * sizeof(T), &p);
    *out = (T*)p;
    return st;
}

struct Pipeline {
    double* t = nullptr;
    double* kd = nullptr;
    double* kz = nullptr;
    DBatch* batches = nullptr;
    InitSoA soa{};
    uint8_t* flag = nullptr;
    int64_t* idx = nullptr;
    uint32_t* block_sums = nullptr;
    unsigned long long* count = nullptr;
    TrajOut out{};
    DepositScratch dep{};
    double* spec_re = nullptr;
    double* spec_im = nullptr;
    double* mspec = nullptr;
    double* sums = nullptr;
    Counters* counters = nullptr;
    unsigned long long* work = nullptr;
};

#define ETRAJ_TRY(x)                 \
    do {                             \
        int _st = (x);               \
        if (_st != ETRAJ_OK) return _st; \
    } while (0)

int alloc_sampling(etraj_ctx* ctx, HostJob& H, Pipeline& P) {
    const DJob& J = H.J;
    const size_t n = (size_t)J.n_total;
    if (J.mol.on) {
        // the molecular tables; their addresses go into the device job
        double *clm = nullptr, *wint = nullptr, *tab = nullptr;
        float* tabf = nullptr;
        if (!H.mol_clm.empty()) ETRAJ_TRY(ensure_t(ctx, "mol.clm", H.mol_clm.size(), &clm));
        if (!H.mol_wint.empty()) ETRAJ_TRY(ensure_t(ctx, "mol.wint", H.mol_wint.size(), &wint));
        ETRAJ_TRY(ensure_t(ctx, "mol.tab", (size_t)J.n_t * (size_t)J.mol.stride, &tab));
        ETRAJ_TRY(ensure_t(ctx, "mol.tabf", (size_t)J.n_t * (size_t)J.mol.stride, &tabf));
        H.J.mol.clm = clm;
        H.J.mol.wint = wint;
        H.J.mol.tab = tab;
        H.J.mol.tabf = tabf;
    }
    ETRAJ_TRY(ensure_t(ctx, "t", H.t.size(), &P.t));
    ETRAJ_TRY(ensure_t(ctx, "kd", H.kd.size(), &P.kd));
    ETRAJ_TRY(ensure_t(ctx, "kz", H.kz.size(), &P.kz));
    ETRAJ_TRY(ensure_t(ctx, "batches", (size_t)J.n_t, &P.batches));
    ETRAJ_TRY(ensure_t(ctx, "soa.x", n, &P.soa.x));
    ETRAJ_TRY(ensure_t(ctx, "soa.y", n, &P.soa.y));
    ETRAJ_TRY(ensure_t(ctx, "soa.kx", n, &P.soa.kx));
    ETRAJ_TRY(ensure_t(ctx, "soa.ky", n, &P.soa.ky));
    ETRAJ_TRY(ensure_t(ctx, "soa.kz", n, &P.soa.kz));
    ETRAJ_TRY(ensure_t(ctx, "soa.rate", n, &P.soa.rate));
    if (J.phase != ETRAJ_PHASE_CTMC) ETRAJ_TRY(ensure_t(ctx, "soa.phase", n, &P.soa.phase));
    else P.soa.phase = nullptr;
    ETRAJ_TRY(ensure_t(ctx, "soa.batch", n, &P.soa.batch));
    ETRAJ_TRY(ensure_t(ctx, "flag", n, &P.flag));
    ETRAJ_TRY(ensure_t(ctx, "idx", n, &P.idx));
    ETRAJ_TRY(ensure_t(ctx, "block_sums", (size_t)compact_blocks((int64_t)n) + 1, &P.block_sums));
    ETRAJ_TRY(ensure_t(ctx, "count", 4, &P.count));
    return ETRAJ_OK;
}

int alloc_outputs(etraj_ctx* ctx, const DJob& J, int64_t max_n, bool with_state, Pipeline& P) {
    const size_t n = (size_t)(max_n > 0 ? max_n : 1);
    if (!ctx->dry) ctx->dump_valid = false;  // the buffers now belong to a new job
    ETRAJ_TRY(ensure_t(ctx, "out.key", n, &P.out.key));
    ETRAJ_TRY(ensure_t(ctx, "out.c_re", n, &P.out.c_re));
    ETRAJ_TRY(ensure_t(ctx, "out.c_im", n, &P.out.c_im));
    ETRAJ_TRY(ensure_t(ctx, "out.w_ion", n, &P.out.w_ion));
    ETRAJ_TRY(ensure_t(ctx, "out.w_unc", n, &P.out.w_unc));
    ETRAJ_TRY(ensure_t(ctx, "out.status", n, &P.out.status));
    ETRAJ_TRY(ensure_t(ctx, "out.steps", n, &P.out.steps));
    if (with_state) ETRAJ_TRY(ensure_t(ctx, "out.final_state", n * (size_t)J.n_state, &P.out.final_state));
    else P.out.final_state = nullptr;
    if (ctx->keep_states) {
        ETRAJ_TRY(ensure_t(ctx, "out.p_inf", 3 * n, &P.out.p_inf));
        ETRAJ_TRY(ensure_t(ctx, "out.fphase", n, &P.out.fphase));
        ETRAJ_TRY(ensure_t(ctx, "out.rmin", n, &P.out.rmin));
    } else {
        P.out.p_inf = nullptr;
        P.out.fphase = nullptr;
        P.out.rmin = nullptr;
    }
    void* dep = nullptr;
    ETRAJ_TRY(ensure(ctx, "deposit", deposit_scratch_bytes(max_n), &dep));
    deposit_scratch_carve(dep, max_n, &P.dep);
    ETRAJ_TRY(ensure_t(ctx, "spec_re", (size_t)J.grid, &P.spec_re));
    ETRAJ_TRY(ensure_t(ctx, "spec_im", (size_t)J.grid, &P.spec_im));
    ETRAJ_TRY(ensure_t(ctx, "mspec", (size_t)J.grid, &P.mspec));
    ETRAJ_TRY(ensure_t(ctx, "sums", 2, &P.sums));
    ETRAJ_TRY(ensure_t(ctx, "counters", 1, &P.counters));
    ETRAJ_TRY(ensure_t(ctx, "work", kBulkCounters, &P.work));
    return ETRAJ_OK;
}

// The candidate kernel of a job: the bulk path samples in FP32 (ADK, SPANE and
// WFAT, atoms and molecules, while every kept rate stays in FP32's normal
// range; SPA for atoms), the FP64 path and molecular SPA in FP64.
int launch_sampler(int precision, const DJob& J, int64_t b0, int64_t nb, const double* kd, const double* kz,
                   DBatch* batches, InitSoA soa, uint8_t* flag, int sm_count, cudaStream_t s,
                   const SampleScratch* scr) {
    // (a Gaussian-proposal job samples in FP64 on every path)
    const bool fp32 = precision == ETRAJ_PRECISION_FP32_BULK && !J.gauss &&
                      (J.method == ETRAJ_SAMPLER_SPA ? !J.mol.on : J.cutoff >= kSample32MinCutoff);
    return fp32 ? launch_sample32_range(J, b0, nb, kd, kz, batches, soa, flag, sm_count, s)
                : launch_sample_range(J, b0, nb, kd, kz, batches, soa, flag, sm_count, s, scr);
}

// The FP64 SPA sampler's list and margin: double-float jobs drop candidates whose
// FP32 rate is below 0.8 x the cutoff (the same electrons survive: FP32's SPA rate
// is within 3e-3 of FP64's where both solve); FP64 jobs only those 100 times
// below, which keeps the oracle's sampler exactly.
SampleScratch sample_scratch(const Pipeline& P, int64_t n, int precision) {
    const float log_margin = (precision == ETRAJ_PRECISION_FP32_DF) ? -0.22314355f : -4.6051702f;
    return SampleScratch{P.idx, P.block_sums, compact_blocks(n) + 1, P.count, log_margin};
}

// Copies a job's host inputs (time and momentum samples, molecular tables) to the device.
void upload_inputs(const HostJob& H, const Pipeline& P, cudaStream_t s) {
    cudaMemcpyAsync(P.t, H.t.data(), H.t.size() * sizeof(double), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(P.kd, H.kd.data(), H.kd.size() * sizeof(double), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(P.kz, H.kz.data(), H.kz.size() * sizeof(double), cudaMemcpyHostToDevice, s);
    if (!H.mol_clm.empty())
        cudaMemcpyAsync((void*)H.J.mol.clm, H.mol_clm.data(), H.mol_clm.size() * sizeof(double),
                        cudaMemcpyHostToDevice, s);
    if (!H.mol_wint.empty())
        cudaMemcpyAsync((void*)H.J.mol.wint, H.mol_wint.data(), H.mol_wint.size() * sizeof(double),
                        cudaMemcpyHostToDevice, s);
}

// Smallest radius beyond which every exp(-b r) term of the SAE potential and
// force is below 2^-26 Z: |a| (1 + b r) e^{-b r} (potential and force
// brackets), |a2| r e^{-b2 r} (potential) and |a2 b2| (r^2 + sc) e^{-b2 r}
// (force, relative to Z / r^2).  Each is decreasing beyond its maximum, so the
// first radius past all maxima where all hold is returned (1e30: never).
float sae_far_radius(const DTarget& T) {
    if (T.kind != ETRAJ_TARGET_SAE) return 1e30f;
    const double eps = std::ldexp(1.0, -26) * T.Z;
    const double a[3] = {T.a1, T.a2, T.a3}, b[3] = {T.b1, T.b2, T.b3};
    double rmin = 0.0;
    for (int i = 0; i < 3; ++i) {
        if (a[i] == 0.0) continue;
        if (!(b[i] > 0.0)) return 1e30f;
        rmin = std::max(rmin, 2.0 / b[i]);
    }
    auto ok = [&](double r) {
        for (int i = 0; i < 3; ++i) {
            if (a[i] == 0.0) continue;
            const double e = std::exp(-b[i] * r);
            if (std::fabs(a[i]) * (1.0 + b[i] * r) * e >= eps) return false;
            if (i == 1 && std::fabs(a[i]) * r * e >= eps) return false;
            if (i == 1 && std::fabs(a[i] * b[i]) * (r * r + T.sc) * e >= eps) return false;
        }
        return true;
    };
    double r = rmin;
    while (!ok(r)) {
        r *= 1.01;
        r += 0.01;
        if (r > 1e6) return 1e30f;
    }
    return (float)(r * 1.01);
}

// Bulk-integrator parameters: field table spanning [tmin, t_final] with
// spacing T_min/512 (T_min the shortest laser period).
void prepare_bulk(const DJob& J, double tmin, BulkParams& B) {
    std::memset(&B, 0, sizeof B);
    B.dim = J.dim;
    B.phase = J.phase;
    B.tgt = J.target.kind;
    double T = J.laser.m[0].period;
    if (J.laser.nmono == 2) T = std::min(T, J.laser.m[1].period);
    const double h = T / 512.0;
    B.T0 = tmin - h;
    B.n_int = (int)std::ceil((J.t_final - B.T0) / h) + 2;
    B.inv_h_d = 1.0 / h;
    B.max_iters = kBulkMaxIters;
    B.h = (float)h;
    B.inv_h = (float)(1.0 / h);
    B.t_final = J.t_final;
    const double q = (J.t_final - B.T0) / h;
    const double fl = std::floor(q);
    B.nf = (int)fl;
    B.ff = (float)(q - fl);
    B.rtol = (float)J.rtol;
    B.table_in_smem = ((size_t)B.n_int * 2 * sizeof(float4) <= (size_t)96 * 1024) ? 1 : 0;
    B.threads = 256;
    B.blocks_per_sm = 2;
    B.refill_min = 4;
    B.occ = 2;
    const DTarget& T_ = J.target;
    B.Z = (float)T_.Z;
    B.Ip = (float)T_.Ip;
    B.sc = (float)T_.sc;
    B.a1 = (float)T_.a1; B.b1 = (float)T_.b1;
    B.a2 = (float)T_.a2; B.b2 = (float)T_.b2;
    B.a3 = (float)T_.a3; B.b3 = (float)T_.b3;
    B.a2b2 = (float)(T_.a2 * T_.b2);
    B.r_far = sae_far_radius(T_);
}

// Double-float integrator parameters (integrate_setup.h) and its launch shapes:
// persistent grids, as many blocks as are resident, and no more than the job
// keeps busy (~4 electrons per lane).
void prepare_df(const DJob& J, double tmin, int64_t max_n, int sm_count, DFParams& D) {
    prepare_df_params(J, tmin, max_n, D);
    D.threads = df_threads(false);
    D.threads_main = df_threads(true);
    for (int main = 0; main < 2; ++main) {
        const int th = main ? D.threads_main : D.threads;
        const int64_t lanes_per_block = (int64_t)th * 4;
        const int64_t want = (max_n + lanes_per_block - 1) / lanes_per_block;
        const int64_t cap = (int64_t)sm_count * df_blocks_per_sm(D.dim, D.phase, D.tgt, main != 0, th);
        (main ? D.blocks_main : D.blocks) = (int)(want < 1 ? 1 : (want < cap ? want : cap));
    }
}

// The double-float integrator's buffers: the field table and the carried electrons
// (kDfCarryWords x max_n words).
int attach_df(etraj_ctx* ctx, DFParams& D) {
    float4* tab = nullptr;
    ETRAJ_TRY(ensure_t(ctx, "field_table_df", (size_t)D.n_int * kDfTableF4, &tab));
    ETRAJ_TRY(ensure_t(ctx, "df_carry", (size_t)kDfCarryWords * (size_t)(D.max_n > 0 ? D.max_n : 1), &D.carry));
    D.table = tab;
    return ETRAJ_OK;
}

// ---- autotuner of the bulk integrator's launch shape ----------------------------------
// Candidates: threads per block x blocks per SM x the register budget of the
// build (<= 128 registers: 16 warps per SM; <= 85: 24 warps) x the number of
// free lanes a warp waits for before it refills.  Each variant (dimension,
// phase, target, single/multi-instance) is tuned once per device and process,
// on the first 2^18 electrons of its first job with enough work, each electron
// capped at kTuneMaxIters steps (a job's slowest trajectory would otherwise set
// the time of every candidate), by timing every candidate twice with events.
// The choice is kept process-wide, so the contexts of a server tune a variant
// once between them.  Results do not depend on the launch shape (one electron
// per lane, deterministic deposit).
cudaEvent_t get_event(etraj_ctx* ctx);
constexpr int kTuneMaxIters = 4096;

std::mutex g_tile_mu;                             // guards g_tiles; held across a tuning run
std::map<std::pair<int, int>, BulkTile> g_tiles;  // (device, variant) -> launch shape

// The context's launch shape for a variant: its own choice, else the process-wide one.
bool find_tile(etraj_ctx* ctx, int key, BulkTile* t) {
    auto it = ctx->tiles.find(key);
    if (it == ctx->tiles.end()) {
        if (!ctx->autotune) return false;
        std::lock_guard<std::mutex> lk(g_tile_mu);
        auto g = g_tiles.find({ctx->device, key});
        if (g == g_tiles.end()) return false;
        it = ctx->tiles.emplace(key, g->second).first;
    }
    if (t) *t = it->second;
    return true;
}

constexpr BulkTile kTileCandidates[] = {{256, 2, 4, 2, 1024}, {256, 2, 8, 2, 1024}, {256, 2, 2, 2, 1024},
                                        {256, 2, 16, 2, 1024}, {128, 4, 4, 2, 1024}, {128, 4, 8, 2, 1024},
                                        {128, 3, 4, 2, 1024}, {64, 8, 4, 2, 1024},   {256, 3, 4, 3, 1024},
                                        {256, 3, 8, 3, 1024}, {128, 6, 4, 3, 1024}, {128, 6, 8, 3, 1024}};
// step chunks the tuner tries once the shape is chosen (with rounds on)
constexpr int kChunkCandidates[] = {256, 4096};
constexpr BulkTile kTileDefault = {256, 2, 4, 2, 1024};

// Stage events: inside a stream capture they become event-record nodes of the graph.
void rec(etraj_ctx* ctx, cudaEvent_t e, cudaStream_t s) {
    if (ctx->capturing) cudaEventRecordWithFlags(e, s, cudaEventRecordExternal);
    else cudaEventRecord(e, s);
}

int tile_key(const BulkParams& B) { return ((B.n_inst > 0) ? 1000 : 0) + B.dim * 100 + B.phase * 10 + B.tgt; }

void apply_tile(BulkParams& B, const BulkTile& t) {
    B.threads = t.threads;
    B.blocks_per_sm = t.blocks_per_sm;
    B.refill_min = t.refill_min;
    B.occ = t.occ;
    B.chunk0 = t.chunk > 0 ? t.chunk : 1024;
    const size_t tb = (size_t)B.n_int * 2 * sizeof(float4);
    B.table_in_smem = (B.n_inst == 0 && tb <= (size_t)96 * 1024 && tb * (size_t)t.blocks_per_sm <= (size_t)200 * 1024)
                          ? 1 : 0;
}

int tuned_bulk_launch(etraj_ctx* ctx, BulkParams& B, const InitSoA& soa, const double* t, const int64_t* idx,
                      const unsigned long long* count, unsigned long long* work, const TrajOut& out,
                      int* launches, cudaEvent_t* ev) {
    cudaStream_t s = ctx->stream;
    const int key = tile_key(B);
    BulkTile chosen = kTileDefault;
    bool have = find_tile(ctx, key, &chosen);
    if (B.static_assign) {
        // the plain schedule: the tuned (or default) block shape, no tuning run
        apply_tile(B, chosen);
        if (ev) rec(ctx, ev[0], s);
        *launches += launch_integrate_bulk(B, soa, t, idx, count, work, out, ctx->sm_count, s);
        if (ev) rec(ctx, ev[1], s);
        return ETRAJ_OK;
    }
    std::unique_lock<std::mutex> tune_lk(g_tile_mu, std::defer_lock);
    if (!have && ctx->autotune && B.max_n >= ((int64_t)1 << 18)) {
        tune_lk.lock();  // one tuning run at a time; another context may have finished it meanwhile
        auto g = g_tiles.find({ctx->device, key});
        if (g != g_tiles.end()) {
            chosen = g->second;
            have = true;
            ctx->tiles[key] = chosen;
        }
    }
    if (!have && ctx->autotune && B.max_n >= ((int64_t)1 << 18)) {
        unsigned long long* sub = nullptr;
        ETRAJ_TRY(ensure_t(ctx, "tune.count", 1, &sub));
        *launches += launch_clamp_count(count, 1ull << 18, sub, s);
        const int nc = (int)(sizeof kTileCandidates / sizeof kTileCandidates[0]);
        std::vector<cudaEvent_t> evs((size_t)4 * nc);
        for (auto& e : evs) e = get_event(ctx);
        for (int rep = 0; rep < 2; ++rep) {
            for (int c = 0; c < nc; ++c) {
                BulkParams Bc = B;
                Bc.max_iters = kTuneMaxIters;
                apply_tile(Bc, kTileCandidates[c]);
                cudaEventRecord(evs[(size_t)(4 * c + 2 * rep)], s);
                *launches += launch_integrate_bulk(Bc, soa, t, idx, sub, work, out, ctx->sm_count, s);
                cudaEventRecord(evs[(size_t)(4 * c + 2 * rep + 1)], s);
            }
        }
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return cuda_err(ctx, e, "autotune");
        float best = 1e30f;
        BulkTile bt = kTileDefault;
        for (int c = 0; c < nc; ++c) {
            float m0 = 0.f, m1 = 0.f;
            cudaEventElapsedTime(&m0, evs[(size_t)(4 * c)], evs[(size_t)(4 * c + 1)]);
            cudaEventElapsedTime(&m1, evs[(size_t)(4 * c + 2)], evs[(size_t)(4 * c + 3)]);
            const float m = m0 < m1 ? m0 : m1;
            if (m < best) {
                best = m;
                bt = kTileCandidates[c];
            }
        }
        // second stage: the step chunk of the rounds, with the chosen shape
        if (B.park_buf) {
            const int nk = (int)(sizeof kChunkCandidates / sizeof kChunkCandidates[0]);
            for (int rep = 0; rep < 2; ++rep)
                for (int c = 0; c < nk; ++c) {
                    BulkParams Bc = B;
                    Bc.max_iters = kTuneMaxIters;
                    BulkTile tc = bt;
                    tc.chunk = kChunkCandidates[c];
                    apply_tile(Bc, tc);
                    cudaEventRecord(evs[(size_t)(4 * c + 2 * rep)], s);
                    *launches += launch_integrate_bulk(Bc, soa, t, idx, sub, work, out, ctx->sm_count, s);
                    cudaEventRecord(evs[(size_t)(4 * c + 2 * rep + 1)], s);
                }
            e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) return cuda_err(ctx, e, "autotune");
            const BulkTile shape = bt;
            for (int c = 0; c < nk; ++c) {
                float m0 = 0.f, m1 = 0.f;
                cudaEventElapsedTime(&m0, evs[(size_t)(4 * c)], evs[(size_t)(4 * c + 1)]);
                cudaEventElapsedTime(&m1, evs[(size_t)(4 * c + 2)], evs[(size_t)(4 * c + 3)]);
                const float m = m0 < m1 ? m0 : m1;
                if (m < best) {
                    best = m;
                    bt = shape;
                    bt.chunk = kChunkCandidates[c];
                }
            }
        }
        for (auto& ev_ : evs) ctx->event_pool.push_back(ev_);
        ctx->tiles[key] = bt;
        g_tiles[{ctx->device, key}] = bt;
        chosen = bt;
    }
    if (tune_lk.owns_lock()) tune_lk.unlock();
    apply_tile(B, chosen);
    if (ev) rec(ctx, ev[0], s);
    *launches += launch_integrate_bulk(B, soa, t, idx, count, work, out, ctx->sm_count, s);
    if (ev) rec(ctx, ev[1], s);
    return ETRAJ_OK;
}

// The park buffer of the bulk integrator's rounds: two halves of max_n/16 +
// 4096 entries (at most 2^20) of kParkWords words.  An electron that finds
// the buffer full finishes in its current round, so the size only bounds how
// much the later rounds can repack.
int attach_park(etraj_ctx* ctx, BulkParams& B) {
    B.park_buf = nullptr;
    B.park_cap = 0;
    if (!ctx->repack) return ETRAJ_OK;
    const int cap = (int)std::min<int64_t>(B.max_n / 16 + 4096, (int64_t)1 << 20);
    uint32_t* buf = nullptr;
    ETRAJ_TRY(ensure_t(ctx, "park", (size_t)2 * (size_t)cap * kParkWords, &buf));
    B.park_buf = buf;
    B.park_cap = cap;
    return ETRAJ_OK;
}

int launch_integrate(etraj_ctx* ctx, const DJob& J, const InitSoA& soa, const double* t, const int64_t* idx,
                     const unsigned long long* count, const TrajOut& out, int64_t max_n, unsigned long long* work,
                     int precision, double tmin, int* launches, cudaEvent_t* ev = nullptr) {
    // ev (optional): events recorded after the field table [0] and the integrator [1]
    cudaStream_t s = ctx->stream;
    if (precision == ETRAJ_PRECISION_FP32_DF) {
        DFParams D;
        prepare_df(J, tmin, max_n, ctx->sm_count, D);
        ETRAJ_TRY(attach_df(ctx, D));
        DfTableNodes nodes;
        df_table_nodes(nodes);
        *launches += launch_field_table_df(J, D.T0, D.h_d, D.n_int, nodes, (float4*)D.table, s);
        if (ev) rec(ctx, ev[0], s);
        *launches += launch_integrate_df(D, soa, t, idx, count, work, out, s);
        if (ev) rec(ctx, ev[1], s);
        *launches += launch_collect_fp64(J, soa, t, idx, count, out, max_n, ctx->sm_count, s);
        return ETRAJ_OK;
    }
    if (precision != ETRAJ_PRECISION_FP32_BULK) {
        if (ev) rec(ctx, ev[0], s);
        *launches += launch_integrate_fp64(J, soa, t, idx, count, out, max_n, ctx->sm_count, s);
        if (ev) rec(ctx, ev[1], s);
        return ETRAJ_OK;
    }
    BulkParams B;
    prepare_bulk(J, tmin, B);
    B.max_n = max_n;
    float4* tab = nullptr;
    ETRAJ_TRY(ensure_t(ctx, "field_table", (size_t)B.n_int * 2, &tab));
    B.table = tab;
    B.static_assign = ctx->static_assign ? 1 : 0;
    if (!B.static_assign) ETRAJ_TRY(attach_park(ctx, B));
    *launches += launch_field_table(J, B.T0, (double)1.0 / B.inv_h_d, B.n_int, tab, s);
    ETRAJ_TRY(tuned_bulk_launch(ctx, B, soa, t, idx, count, work, out, launches, ev));
    *launches += launch_collect_bulk(J, soa, t, idx, count, out, max_n, ctx->sm_count, s);
    return ETRAJ_OK;
}

// ---- pinned staging and events, pooled per context ---------------------------------
int get_pinned(etraj_ctx* ctx, size_t bytes, PinnedBlock* out) {
    for (size_t i = 0; i < ctx->pinned_pool.size(); ++i) {
        if (ctx->pinned_pool[i].bytes >= bytes) {
            *out = ctx->pinned_pool[i];
            ctx->pinned_pool.erase(ctx->pinned_pool.begin() + (long)i);
            return ETRAJ_OK;
        }
    }
    void* p = nullptr;
    cudaError_t e = cudaMallocHost(&p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_err(ctx, ETRAJ_ERR_OUT_OF_MEMORY, std::string("cudaMallocHost: ") + cudaGetErrorString(e));
    }
    out->p = p;
    out->bytes = bytes;
    return ETRAJ_OK;
}

void put_pinned(etraj_ctx* ctx, void* p, size_t bytes) {
    if (!p) return;
    if (ctx->pinned_pool.size() < 64) ctx->pinned_pool.push_back(PinnedBlock{p, bytes});
    else cudaFreeHost(p);
}

cudaEvent_t get_event(etraj_ctx* ctx) {
    if (!ctx->event_pool.empty()) {
        cudaEvent_t e = ctx->event_pool.back();
        ctx->event_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return e;
}

void release_job(etraj_ctx* ctx, JobRec& r) {
    if (r.staged) {
        put_pinned(ctx, r.pinned, r.pinned_bytes);
        if (r.ev_start) ctx->event_pool.push_back(r.ev_start);
        if (r.ev_done) ctx->event_pool.push_back(r.ev_done);
    }
    r.pinned = nullptr;
    r.ev_start = r.ev_done = nullptr;
}

// Device bytes a job would add to this context's buffers (0 for an invalid job,
// whose error comes at enqueue).
size_t plan_growth(etraj_ctx* ctx, const etraj_job* job) {
    std::string err;
    if (validate_job(job, err) != ETRAJ_OK) return 0;
    HostJob H;
    prepare_job(job, H);
    Pipeline P;
    ctx->dry = true;
    ctx->dry_bytes = 0;
    alloc_sampling(ctx, H, P);
    const bool bulk = (job->precision == ETRAJ_PRECISION_FP32_BULK);
    alloc_outputs(ctx, H.J, H.J.n_total, job->precision != ETRAJ_PRECISION_FP64, P);
    if (job->precision == ETRAJ_PRECISION_FP32_DF) {
        DFParams D;
        prepare_df_params(H.J, H.t.front(), H.J.n_total, D);
        attach_df(ctx, D);
    }
    if (bulk) {
        BulkParams B;
        prepare_bulk(H.J, H.t.front(), B);
        float4* tab = nullptr;
        ensure_t(ctx, "field_table", (size_t)B.n_int * 2, &tab);
        B.max_n = H.J.n_total;
        attach_park(ctx, B);
    }
    ctx->dry = false;
    return ctx->dry_bytes;
}

// The device work of one job, from the per-batch prologue to the deposit.
int enqueue_kernels(etraj_ctx* ctx, const etraj_job* job, const HostJob& H, const Pipeline& P, int* nl) {
    const DJob& J = H.J;
    cudaStream_t s = ctx->stream;
    int launches = 0;
    rec(ctx, ctx->stage_ev[0], s);
    launches += launch_batch_prepare(J, P.t, P.batches, s);
    const SampleScratch scr = sample_scratch(P, J.n_total, job->precision);
    launches += launch_sampler(job->precision, J, 0, J.n_t, P.kd, P.kz, P.batches, P.soa, P.flag, ctx->sm_count, s,
                               &scr);
    rec(ctx, ctx->stage_ev[1], s);
    launches += launch_compact(P.flag, J.n_total, P.idx, P.block_sums, compact_blocks(J.n_total) + 1, P.count, s);
    rec(ctx, ctx->stage_ev[2], s);
    ETRAJ_TRY(launch_integrate(ctx, J, P.soa, P.t, P.idx, P.count, P.out, J.n_total, P.work, job->precision,
                               H.t.front(), &launches, ctx->stage_ev + 3));
    rec(ctx, ctx->stage_ev[5], s);
    launches += launch_deposit(J, P.out, P.count, J.n_total, P.dep, P.spec_re, P.spec_im, P.mspec, P.sums,
                               P.counters, s);
    rec(ctx, ctx->stage_ev[6], s);
    ctx->stage_valid = true;
    *nl = launches;
    return ETRAJ_OK;
}

// With ctx->graphs the kernel sequence is captured once into a CUDA graph and
// replayed while the launch parameters (device job, buffer addresses, bulk
// launch shape, table size) stay the same; a job that needs an autotuning pass
// first runs without a graph.
int enqueue_kernels_maybe_graph(etraj_ctx* ctx, const etraj_job* job, const HostJob& H, const Pipeline& P,
                                int* launches) {
    const DJob& J = H.J;
    bool use_graph = ctx->graphs;
    int tile_k = -1;
    size_t n_int = 0;
    if (use_graph && job->precision == ETRAJ_PRECISION_FP32_BULK) {
        BulkParams B;
        prepare_bulk(J, H.t.front(), B);
        B.max_n = J.n_total;
        n_int = (size_t)B.n_int;
        tile_k = tile_key(B);
        if (ctx->autotune && !find_tile(ctx, tile_k, nullptr) && B.max_n >= ((int64_t)1 << 18)) use_graph = false;
        float4* tab = nullptr;  // allocate the field table and the park buffer outside the capture
        ETRAJ_TRY(ensure_t(ctx, "field_table", n_int * 2, &tab));
        ETRAJ_TRY(attach_park(ctx, B));
    }
    if (use_graph && job->precision == ETRAJ_PRECISION_FP32_DF) {
        DFParams D;  // allocate the field table and the carry buffer outside the capture
        prepare_df_params(J, H.t.front(), J.n_total, D);
        n_int = (size_t)D.n_int;
        ETRAJ_TRY(attach_df(ctx, D));
    }
    if (!use_graph) return enqueue_kernels(ctx, job, H, P, launches);
    const char* tab_name = (job->precision == ETRAJ_PRECISION_FP32_DF) ? "field_table_df" : "field_table";
    const char* aux_name = (job->precision == ETRAJ_PRECISION_FP32_DF) ? "df_carry" : "park";
    void* ptrs[2] = {ctx->bufs.count(tab_name) ? ctx->bufs[tab_name].p : nullptr,
                     ctx->bufs.count(aux_name) ? ctx->bufs[aux_name].p : nullptr};
    std::vector<unsigned char> key(sizeof J + sizeof P + sizeof(int) * 3 + sizeof(size_t) + sizeof ptrs);
    unsigned char* k = key.data();
    std::memcpy(k, &J, sizeof J);
    k += sizeof J;
    std::memcpy(k, &P, sizeof P);
    k += sizeof P;
    BulkTile t = kTileDefault;
    find_tile(ctx, tile_k, &t);
    const int extra[3] = {job->precision, t.threads * 1000 + t.blocks_per_sm * 10 + t.occ,
                          (t.refill_min * 4 + (ctx->repack ? 1 : 0) + (ctx->static_assign ? 2 : 0)) * 65536 +
                              t.chunk};
    std::memcpy(k, extra, sizeof extra);
    k += sizeof extra;
    std::memcpy(k, &n_int, sizeof n_int);
    k += sizeof n_int;
    std::memcpy(k, ptrs, sizeof ptrs);
    cudaStream_t s = ctx->stream;
    if (ctx->gexec && key == ctx->gkey) {
        cudaError_t e = cudaGraphLaunch(ctx->gexec, s);
        if (e != cudaSuccess) return cuda_err(ctx, e, "cudaGraphLaunch");
        *launches = ctx->glaunches;
        ctx->stage_valid = true;
        return ETRAJ_OK;
    }
    if (key != ctx->gseen) {
        // first sighting: run directly; the same launch parameters again are captured
        ctx->gseen = key;
        return enqueue_kernels(ctx, job, H, P, launches);
    }
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        return enqueue_kernels(ctx, job, H, P, launches);
    }
    ctx->capturing = true;
    const int st = enqueue_kernels(ctx, job, H, P, launches);
    ctx->capturing = false;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(s, &g);
    cudaGraphExec_t ex = nullptr;
    if (st == ETRAJ_OK && e == cudaSuccess && g && cudaGraphInstantiate(&ex, g, 0) == cudaSuccess) {
        cudaGraphDestroy(g);
        if (ctx->gexec) cudaGraphExecDestroy(ctx->gexec);
        ctx->gexec = ex;
        ctx->gkey = key;
        ctx->glaunches = *launches;
        e = cudaGraphLaunch(ex, s);
        if (e != cudaSuccess) return cuda_err(ctx, e, "cudaGraphLaunch");
        return ETRAJ_OK;
    }
    // capture failed: run the sequence directly
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    if (st != ETRAJ_OK) return st;
    return enqueue_kernels(ctx, job, H, P, launches);
}

// Enqueues one whole job on the context's stream: host set-up, copies of the
// time and momentum samples, every kernel, and the copies of the results.  With
// r.staged the results go to a pinned block and r.ev_done marks completion;
// otherwise they go straight to the caller's buffers.
int enqueue_job(etraj_ctx* ctx, const etraj_job* job, JobRec& r) {
    std::string err;
    int st = validate_job(job, err);
    if (st != ETRAJ_OK) return set_err(ctx, st, err);
    HostJob H;
    prepare_job(job, H);
    const DJob& J = H.J;
    Pipeline P;
    ETRAJ_TRY(alloc_sampling(ctx, H, P));
    ETRAJ_TRY(alloc_outputs(ctx, J, J.n_total, job->precision != ETRAJ_PRECISION_FP64, P));
    r.grid = J.grid;
    r.coherent = (J.phase != ETRAJ_PHASE_CTMC);
    const bool want_spec = r.res.momentum_spec != nullptr;
    const bool want_amp = r.res.amplitude != nullptr && r.coherent;
    double* dst_sums = r.direct_sums;
    Counters* dst_cnt = &r.direct_cnt;
    double* dst_spec = r.res.momentum_spec;
    double* dst_amp = r.res.amplitude;
    if (r.staged) {
        const size_t bytes = 2 * sizeof(double) + sizeof(Counters) + (want_spec ? (size_t)J.grid * 8 : 0) +
                             (want_amp ? (size_t)J.grid * 16 : 0);
        PinnedBlock blk;
        ETRAJ_TRY(get_pinned(ctx, bytes, &blk));
        r.pinned = blk.p;
        r.pinned_bytes = blk.bytes;
        char* base = (char*)blk.p;
        dst_sums = (double*)base;
        dst_cnt = (Counters*)(base + 2 * sizeof(double));
        char* rest = base + 2 * sizeof(double) + sizeof(Counters);
        dst_spec = want_spec ? (double*)rest : nullptr;
        dst_amp = want_amp ? (double*)(rest + (want_spec ? (size_t)J.grid * 8 : 0)) : nullptr;
        r.ev_start = get_event(ctx);
        r.ev_done = get_event(ctx);
        if (!r.ev_start || !r.ev_done) return set_err(ctx, ETRAJ_ERR_CUDA, "cudaEventCreate failed");
    } else {
        r.ev_start = ctx->ev0;
        r.ev_done = ctx->ev1;
    }
    cudaStream_t s = ctx->stream;
    upload_inputs(H, P, s);
    cudaEventRecord(r.ev_start, s);
    int launches = 0;
    ETRAJ_TRY(enqueue_kernels_maybe_graph(ctx, job, H, P, &launches));
    cudaMemcpyAsync(dst_sums, P.sums, 2 * sizeof(double), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(dst_cnt, P.counters, sizeof(Counters), cudaMemcpyDeviceToHost, s);
    if (dst_spec) cudaMemcpyAsync(dst_spec, P.mspec, (size_t)J.grid * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (dst_amp) {
        cudaMemcpy2DAsync(dst_amp, 2 * sizeof(double), P.spec_re, sizeof(double), sizeof(double), (size_t)J.grid,
                          cudaMemcpyDeviceToHost, s);
        cudaMemcpy2DAsync(dst_amp + 1, 2 * sizeof(double), P.spec_im, sizeof(double), sizeof(double), (size_t)J.grid,
                          cudaMemcpyDeviceToHost, s);
    }
    cudaEventRecord(r.ev_done, s);
    r.launches = launches;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_err(ctx, e, "kernel launch");
    ctx->dump_valid = ctx->keep_states;
    ctx->dump_ticket = r.ticket;
    ctx->dump_out = P.out;
    if (job->precision != ETRAJ_PRECISION_FP64) ctx->dump_out.rmin = nullptr;  // filled by the FP64 path only
    ctx->dump_count = P.count;
    return ETRAJ_OK;
}

// Completes a job whose ev_done has been reached: fills the caller's result.
int finish_job(etraj_ctx* ctx, JobRec& r) {
    const double* sums = r.direct_sums;
    const Counters* cnt = &r.direct_cnt;
    if (r.staged) {
        const char* base = (const char*)r.pinned;
        sums = (const double*)base;
        cnt = (const Counters*)(base + 2 * sizeof(double));
        const char* rest = base + 2 * sizeof(double) + sizeof(Counters);
        if (r.res.momentum_spec) {
            std::memcpy(r.res.momentum_spec, rest, (size_t)r.grid * 8);
            rest += (size_t)r.grid * 8;
        }
        if (r.res.amplitude && r.coherent) std::memcpy(r.res.amplitude, rest, (size_t)r.grid * 16);
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, r.ev_start, r.ev_done);
    r.res.ion_prob = sums[0];
    r.res.ion_prob_uncollected = sums[1];
    r.res.num_effective_traj = (int64_t)cnt->n_eff;
    r.res.num_failed_traj = (int64_t)cnt->n_failed;
    r.res.num_ionized_traj = (int64_t)cnt->n_ionized;
    r.res.num_steps = (int64_t)cnt->n_steps;
    r.res.num_kernel_launches = r.launches;
    r.res.elapsed_ms = ms;
    const bool sort_failed = cnt->sort_err != 0;
    release_job(ctx, r);
    if (sort_failed) return set_err(ctx, ETRAJ_ERR_CUDA, "deposit: a look-back wait of the radix sort gave up");
    return ETRAJ_OK;
}

int run_job(etraj_ctx* ctx, const etraj_job* job, etraj_result* res) {
    JobRec r;
    r.res = *res;
    r.staged = false;
    ETRAJ_TRY(enqueue_job(ctx, job, r));
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_err(ctx, e, "etraj_run");
    ETRAJ_TRY(finish_job(ctx, r));
    *res = r.res;
    return ETRAJ_OK;
}

// ---- multi-instance batch: many jobs in one integrator launch ------------------------
// The instances' time samples, candidates and field tables are concatenated;
// sampling runs per instance, then one compaction, one bulk-integrator launch
// whose work stealing spans every instance, one collection, one deposit into
// an instance-major grid, and per-instance reductions.  Every per-instance
// result equals that of the same job run alone.
int run_batch(etraj_ctx* ctx, const etraj_job* jobs, int n, etraj_result* res, const double* weights,
              double* wspec) {
    if (!jobs || !res || n < 1 || n > kMaxInstances)
        return set_err(ctx, ETRAJ_ERR_INVALID_ARGUMENT, "etraj_run_batch: 1 to 64 jobs");
    if ((weights == nullptr) != (wspec == nullptr))
        return set_err(ctx, ETRAJ_ERR_INVALID_ARGUMENT, "etraj_run_batch: weights and weighted_spec go together");
    const etraj_job& j0 = jobs[0];
    for (int i = 0; i < n; ++i) {
        std::string err;
        const int st = validate_job(&jobs[i], err);
        if (st != ETRAJ_OK) return set_err(ctx, st, "job " + std::to_string(i) + ": " + err);
        const etraj_job& ji = jobs[i];
        if (ji.target.kind == ETRAJ_TARGET_MOLECULE)
            return set_err(ctx, ETRAJ_ERR_UNSUPPORTED,
                           "etraj_run_batch: molecular targets are run one job at a time (etraj_run, etraj_submit)");
        bool same = ji.precision == ETRAJ_PRECISION_FP32_BULK && ji.dimension == j0.dimension &&
                    ji.traj_phase_method == j0.traj_phase_method && ji.traj_rtol == j0.traj_rtol &&
                    std::memcmp(&ji.target, &j0.target, sizeof ji.target) == 0;
        for (int d = 0; d < 3; ++d)
            same = same && ji.final_p_num[d] == j0.final_p_num[d] && ji.final_p_max[d] == j0.final_p_max[d];
        if (!same)
            return set_err(ctx, ETRAJ_ERR_INVALID_ARGUMENT,
                           "etraj_run_batch: job " + std::to_string(i) +
                               " differs from job 0 in precision (must be FP32_BULK), dimension, phase method, "
                               "rtol, target or momentum grid");
    }
    std::vector<HostJob> H((size_t)n);
    for (int i = 0; i < n; ++i) prepare_job(&jobs[i], H[(size_t)i]);
    const int64_t grid1 = H[0].J.grid;
    if ((int64_t)n * grid1 >= (int64_t)0xFFFFFFFFll)
        return set_err(ctx, ETRAJ_ERR_INVALID_ARGUMENT, "etraj_run_batch: instances x grid >= 2^32 bins");
    std::vector<int64_t> toff(n + 1, 0), koff(n + 1, 0), zoff(n + 1, 0), coff(n + 1, 0), tab_off(n + 1, 0);
    std::vector<BulkParams> B((size_t)n);
    for (int i = 0; i < n; ++i) {
        const HostJob& h = H[(size_t)i];
        toff[i + 1] = toff[i] + (int64_t)h.t.size();
        koff[i + 1] = koff[i] + (int64_t)h.kd.size();
        zoff[i + 1] = zoff[i] + (int64_t)h.kz.size();
        coff[i + 1] = coff[i] + h.J.n_total;
        prepare_bulk(h.J, h.t.front(), B[(size_t)i]);
        tab_off[i + 1] = tab_off[i] + 2 * (int64_t)B[(size_t)i].n_int;
    }
    const int64_t N = coff[n];
    if (toff[n] >= (int64_t)1 << 31)
        return set_err(ctx, ETRAJ_ERR_INVALID_ARGUMENT, "etraj_run_batch: more than 2^31 time samples");
    std::vector<double> t_all((size_t)toff[n]), kd_all((size_t)koff[n]), kz_all((size_t)zoff[n]);
    for (int i = 0; i < n; ++i) {
        const HostJob& h = H[(size_t)i];
        std::copy(h.t.begin(), h.t.end(), t_all.begin() + toff[i]);
        std::copy(h.kd.begin(), h.kd.end(), kd_all.begin() + koff[i]);
        std::copy(h.kz.begin(), h.kz.end(), kz_all.begin() + zoff[i]);
    }
    // buffers (the single-job names, sized for the whole batch)
    Pipeline P;
    DJob Jgrid = H[0].J;
    Jgrid.grid = (int64_t)n * grid1;
    HostJob Hsz;
    Hsz.J = Jgrid;
    Hsz.J.n_total = N;
    Hsz.J.n_t = toff[n];
    Hsz.t = t_all;
    Hsz.kd = kd_all;
    Hsz.kz = kz_all;
    ETRAJ_TRY(alloc_sampling(ctx, Hsz, P));
    ETRAJ_TRY(alloc_outputs(ctx, Jgrid, N, true, P));
    float4* tab = nullptr;
    BulkInst* d_inst = nullptr;
    int64_t* d_seg = nullptr;
    double *d_scr = nullptr, *d_isums = nullptr, *d_w = nullptr, *d_wout = nullptr;
    Counters* d_icnt = nullptr;
    ETRAJ_TRY(ensure_t(ctx, "field_table", (size_t)tab_off[n], &tab));
    ETRAJ_TRY(ensure_t(ctx, "batch.inst", (size_t)n, &d_inst));
    ETRAJ_TRY(ensure_t(ctx, "batch.seg", (size_t)n + 1, &d_seg));
    ETRAJ_TRY(ensure_t(ctx, "batch.scratch", instance_scratch_doubles(N, n), &d_scr));
    ETRAJ_TRY(ensure_t(ctx, "batch.sums", (size_t)2 * n, &d_isums));
    ETRAJ_TRY(ensure_t(ctx, "batch.counters", (size_t)n, &d_icnt));
    if (weights) {
        ETRAJ_TRY(ensure_t(ctx, "batch.w", (size_t)n, &d_w));
        ETRAJ_TRY(ensure_t(ctx, "batch.wout", (size_t)grid1, &d_wout));
    }
    std::vector<BulkInst> inst((size_t)n);
    for (int i = 0; i < n; ++i) {
        const BulkParams& b = B[(size_t)i];
        BulkInst& q = inst[(size_t)i];
        q.table = tab + tab_off[i];
        q.cand_end = coff[i + 1];
        q.T0 = b.T0;
        q.inv_h_d = b.inv_h_d;
        q.t_final = b.t_final;
        q.t_off = (int)toff[i];
        q.n_int = b.n_int;
        q.nf = b.nf;
        q.ff = b.ff;
        q.h = b.h;
        q.inv_h = b.inv_h;
    }
    cudaStream_t s = ctx->stream;
    cudaMemcpyAsync(P.t, t_all.data(), t_all.size() * 8, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(P.kd, kd_all.data(), kd_all.size() * 8, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(P.kz, kz_all.data(), kz_all.size() * 8, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(d_inst, inst.data(), inst.size() * sizeof(BulkInst), cudaMemcpyHostToDevice, s);
    if (weights) cudaMemcpyAsync(d_w, weights, (size_t)n * 8, cudaMemcpyHostToDevice, s);
    BulkParams M = B[0];
    M.table = nullptr;
    M.table_in_smem = 0;
    M.max_n = N;
    M.inst = d_inst;
    M.n_inst = n;
    // a batch runs as one launch (no rounds): it is throughput work, and its
    // resume rounds would run the parked electrons on a few SMs while no other
    // job waits for the rest (measured 140 ms against 121 ms for 64 instances)
    M.park_buf = nullptr;
    M.park_cap = 0;
    // the device work of the batch, from the first sampling launch to the weighted sum
    auto enqueue = [&](int* nl) -> int {
        int launches = 0;
        rec(ctx, ctx->ev0, s);
        rec(ctx, ctx->stage_ev[0], s);
        for (int i = 0; i < n; ++i) {
            const DJob& J = H[(size_t)i].J;
            DBatch* bat = P.batches + toff[i];
            launches += launch_batch_prepare(J, P.t + toff[i], bat, s);
            InitSoA so = P.soa;
            const int64_t c = coff[i];
            so.x += c; so.y += c; so.kx += c; so.ky += c; so.kz += c; so.rate += c; so.batch += c;
            if (so.phase) so.phase += c;
            launches += launch_sampler(ETRAJ_PRECISION_FP32_BULK, J, 0, J.n_t, P.kd + koff[i], P.kz + zoff[i], bat, so,
                                       P.flag + c, ctx->sm_count, s, nullptr);
        }
        rec(ctx, ctx->stage_ev[1], s);
        launches += launch_compact(P.flag, N, P.idx, P.block_sums, compact_blocks(N) + 1, P.count, s);
        rec(ctx, ctx->stage_ev[2], s);
        for (int i = 0; i < n; ++i) {
            const BulkParams& b = B[(size_t)i];
            launches += launch_field_table(H[(size_t)i].J, b.T0, 1.0 / b.inv_h_d, b.n_int, tab + tab_off[i], s);
        }
        ETRAJ_TRY(tuned_bulk_launch(ctx, M, P.soa, P.t, P.idx, P.count, P.work, P.out, &launches, ctx->stage_ev + 3));
        launches += launch_collect_bulk(H[0].J, P.soa, P.t, P.idx, P.count, P.out, N, ctx->sm_count, s, d_inst, n);
        rec(ctx, ctx->stage_ev[5], s);
        launches += launch_deposit(Jgrid, P.out, P.count, N, P.dep, P.spec_re, P.spec_im, P.mspec, P.sums, P.counters, s);
        launches += launch_instance_reductions(P.out, P.idx, P.count, d_inst, n, d_seg, d_scr, d_isums, d_icnt, s);
        if (weights) launches += launch_weighted_sum(P.mspec, n, grid1, d_w, d_wout, s);
        rec(ctx, ctx->stage_ev[6], s);
        rec(ctx, ctx->ev1, s);
        *nl = launches;
        return ETRAJ_OK;
    };
    int launches = 0;
    BulkTile tile;
    const bool tuned = !ctx->autotune || N < ((int64_t)1 << 18) || find_tile(ctx, tile_key(M), &tile);
    if (ctx->graphs && tuned) {
        // replayed when the same batch runs again on the same buffers and launch shape
        // (the inputs above are copied before and the results read after the graph)
        std::vector<unsigned char> key(1 + (size_t)n * sizeof(etraj_job) + sizeof P + 10 * sizeof(void*) +
                                       3 * sizeof(int));
        unsigned char* k = key.data();
        *k++ = 'B';
        std::memcpy(k, jobs, (size_t)n * sizeof(etraj_job));
        k += (size_t)n * sizeof(etraj_job);
        std::memcpy(k, &P, sizeof P);
        k += sizeof P;
        const void* ptrs[10] = {tab, d_inst, d_seg, d_scr, d_isums, d_icnt, d_w, d_wout, P.work, nullptr};
        std::memcpy(k, ptrs, sizeof ptrs);
        k += sizeof ptrs;
        BulkTile t = kTileDefault;
        find_tile(ctx, tile_key(M), &t);
        const int extra[3] = {t.threads * 1000 + t.blocks_per_sm * 10 + t.occ, t.refill_min * 65536 + t.chunk,
                              (ctx->static_assign ? 1 : 0) + (weights ? 2 : 0)};
        std::memcpy(k, extra, sizeof extra);
        if (ctx->bgexec && key == ctx->bgkey) {
            cudaError_t e = cudaGraphLaunch(ctx->bgexec, s);
            if (e != cudaSuccess) return cuda_err(ctx, e, "cudaGraphLaunch (batch)");
            launches = ctx->bglaunches;
        } else if (key != ctx->bgseen) {
            ctx->bgseen = key;  // first sighting: direct; the same batch again is captured
            ETRAJ_TRY(enqueue(&launches));
        } else if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
            ctx->capturing = true;
            const int st = enqueue(&launches);
            ctx->capturing = false;
            cudaGraph_t g = nullptr;
            cudaError_t e = cudaStreamEndCapture(s, &g);
            cudaGraphExec_t ex = nullptr;
            if (st == ETRAJ_OK && e == cudaSuccess && g && cudaGraphInstantiate(&ex, g, 0) == cudaSuccess) {
                cudaGraphDestroy(g);
                if (ctx->bgexec) cudaGraphExecDestroy(ctx->bgexec);
                ctx->bgexec = ex;
                ctx->bgkey = key;
                ctx->bglaunches = launches;
                e = cudaGraphLaunch(ex, s);
                if (e != cudaSuccess) return cuda_err(ctx, e, "cudaGraphLaunch (batch)");
            } else {
                if (g) cudaGraphDestroy(g);
                cudaGetLastError();
                if (st != ETRAJ_OK) return st;
                ETRAJ_TRY(enqueue(&launches));
            }
        } else {
            cudaGetLastError();
            ETRAJ_TRY(enqueue(&launches));
        }
    } else {
        ETRAJ_TRY(enqueue(&launches));
    }
    ctx->stage_valid = true;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_err(ctx, e, "batch launch");
    std::vector<double> isums((size_t)2 * n);
    std::vector<Counters> icnt((size_t)n);
    unsigned long long sort_err = 0ull;
    cudaMemcpyAsync(&sort_err, &P.counters->sort_err, sizeof sort_err, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(isums.data(), d_isums, isums.size() * 8, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(icnt.data(), d_icnt, icnt.size() * sizeof(Counters), cudaMemcpyDeviceToHost, s);
    const bool coherent = (H[0].J.phase != ETRAJ_PHASE_CTMC);
    for (int i = 0; i < n; ++i) {
        const int64_t o = (int64_t)i * grid1;
        if (res[i].momentum_spec)
            cudaMemcpyAsync(res[i].momentum_spec, P.mspec + o, (size_t)grid1 * 8, cudaMemcpyDeviceToHost, s);
        if (res[i].amplitude && coherent) {
            cudaMemcpy2DAsync(res[i].amplitude, 16, P.spec_re + o, 8, 8, (size_t)grid1, cudaMemcpyDeviceToHost, s);
            cudaMemcpy2DAsync(res[i].amplitude + 1, 16, P.spec_im + o, 8, 8, (size_t)grid1, cudaMemcpyDeviceToHost, s);
        }
    }
    if (weights) cudaMemcpyAsync(wspec, d_wout, (size_t)grid1 * 8, cudaMemcpyDeviceToHost, s);
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_err(ctx, e, "etraj_run_batch");
    if (sort_err) return set_err(ctx, ETRAJ_ERR_CUDA, "deposit: a look-back wait of the radix sort gave up");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    for (int i = 0; i < n; ++i) {
        etraj_result& r = res[i];
        r.ion_prob = isums[(size_t)2 * i];
        r.ion_prob_uncollected = isums[(size_t)2 * i + 1];
        r.num_effective_traj = (int64_t)icnt[(size_t)i].n_eff;
        r.num_failed_traj = (int64_t)icnt[(size_t)i].n_failed;
        r.num_ionized_traj = (int64_t)icnt[(size_t)i].n_ionized;
        r.num_steps = (int64_t)icnt[(size_t)i].n_steps;
        r.num_kernel_launches = launches;
        r.elapsed_ms = ms;
    }
    return ETRAJ_OK;
}

// Copies sampled candidates back and assembles the reference's `init` columns.
int gather_rows(etraj_ctx* ctx, const HostJob& H, const Pipeline& P, int64_t g0, int64_t ng, double* init,
                int64_t capacity, int64_t* count) {
    const DJob& J = H.J;
    cudaStream_t s = ctx->stream;
    std::vector<uint8_t> flag((size_t)ng);
    std::vector<double> x((size_t)ng), y((size_t)ng), kx((size_t)ng), ky((size_t)ng), kz((size_t)ng),
        rate((size_t)ng), ph((size_t)ng);
    std::vector<int32_t> batch((size_t)ng);
    cudaMemcpyAsync(flag.data(), P.flag + g0, (size_t)ng, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(x.data(), P.soa.x + g0, (size_t)ng * 8, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(y.data(), P.soa.y + g0, (size_t)ng * 8, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(kx.data(), P.soa.kx + g0, (size_t)ng * 8, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(ky.data(), P.soa.ky + g0, (size_t)ng * 8, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(kz.data(), P.soa.kz + g0, (size_t)ng * 8, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(rate.data(), P.soa.rate + g0, (size_t)ng * 8, cudaMemcpyDeviceToHost, s);
    if (P.soa.phase) cudaMemcpyAsync(ph.data(), P.soa.phase + g0, (size_t)ng * 8, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(batch.data(), P.soa.batch + g0, (size_t)ng * 4, cudaMemcpyDeviceToHost, s);
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_err(ctx, e, "sample copy-back");
    int64_t c = 0;
    for (int64_t i = 0; i < ng; ++i) {
        if (!flag[(size_t)i]) continue;
        if (c < capacity) {
            double* r = init + c * J.rows;
            int k = 0;
            r[k++] = x[(size_t)i];
            r[k++] = y[(size_t)i];
            if (J.dim == 3) r[k++] = 0.0;
            r[k++] = kx[(size_t)i];
            r[k++] = ky[(size_t)i];
            if (J.dim == 3) r[k++] = kz[(size_t)i];
            r[k++] = H.t[(size_t)batch[(size_t)i]];
            r[k++] = rate[(size_t)i];
            if (J.phase != ETRAJ_PHASE_CTMC) r[k++] = ph[(size_t)i];
        }
        ++c;
    }
    *count = c;
    return ETRAJ_OK;
}

int sample_range(etraj_ctx* ctx, const etraj_job* job, int64_t b0, int64_t nb, double* init, int64_t capacity,
                 int64_t* count) {
    std::string err;
    int st = validate_job(job, err);
    if (st != ETRAJ_OK) return set_err(ctx, st, err);
    HostJob H;
    prepare_job(job, H);
    Pipeline P;
    ETRAJ_TRY(alloc_sampling(ctx, H, P));
    cudaStream_t s = ctx->stream;
    upload_inputs(H, P, s);
    launch_batch_prepare(H.J, P.t, P.batches, s);
    const SampleScratch scr = sample_scratch(P, H.J.n_total, job->precision);
    launch_sampler(job->precision, H.J, b0, nb, P.kd, P.kz, P.batches, P.soa, P.flag, ctx->sm_count, s, &scr);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_err(ctx, e, "sample launch");
    return gather_rows(ctx, H, P, b0 * H.J.n_cand, nb * H.J.n_cand, init, capacity, count);
}

}  // namespace

// ---- exported entry points --------------------------------------------------------
extern "C" {

const char* etraj_version(void) { return ETRAJ_VERSION_STRING; }

int etraj_create(etraj_ctx** out, int device, size_t hbm_budget_bytes) {
    if (!out) return ETRAJ_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || device < 0 || device >= ndev) {
        cudaGetLastError();
        return ETRAJ_ERR_CUDA;
    }
    e = cudaSetDevice(device);
    if (e != cudaSuccess) return ETRAJ_ERR_CUDA;
    etraj_ctx* ctx = new etraj_ctx();
    ctx->device = device;
    cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
    {
        // keep freed stream-ordered memory in this process's pool instead of
        // returning it at every synchronization (process-local setting)
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
            uint64_t keep = ~0ull;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
        cudaGetLastError();
    }
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    const size_t reserve = (size_t)1 << 30;
    ctx->budget = hbm_budget_bytes ? hbm_budget_bytes : (free_b > reserve ? free_b - reserve : free_b / 2);
    if (cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&ctx->ev0) != cudaSuccess || cudaEventCreate(&ctx->ev1) != cudaSuccess) {
        delete ctx;
        return ETRAJ_ERR_CUDA;
    }
    for (int i = 0; i <= etraj_ctx::kStages; ++i) {
        if (cudaEventCreate(&ctx->stage_ev[i]) == cudaSuccess) continue;
        delete ctx;
        return ETRAJ_ERR_CUDA;
    }
    ctx->stream = ctx->own_stream;
    *out = ctx;
    return ETRAJ_OK;
}

void etraj_destroy(etraj_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    for (auto& kv : ctx->jobs) release_job(ctx, kv.second);
    for (auto& b : ctx->pinned_pool) cudaFreeHost(b.p);
    for (cudaEvent_t e : ctx->event_pool) cudaEventDestroy(e);
    for (auto& kv : ctx->bufs)
        if (kv.second.p) cudaFreeAsync(kv.second.p, ctx->stream);
    cudaStreamSynchronize(ctx->stream);
    if (ctx->gexec) cudaGraphExecDestroy(ctx->gexec);
    if (ctx->bgexec) cudaGraphExecDestroy(ctx->bgexec);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    for (int i = 0; i <= etraj_ctx::kStages; ++i)
        if (ctx->stage_ev[i]) cudaEventDestroy(ctx->stage_ev[i]);
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    delete ctx;
}

const char* etraj_last_error(const etraj_ctx* ctx) { return ctx ? ctx->err.c_str() : "no context"; }

int etraj_set_stream(etraj_ctx* ctx, void* cuda_stream) {
    if (!ctx) return ETRAJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    // buffers are stream-ordered allocations: finish everything queued on the
    // old stream before the new one may touch them
    cudaStreamSynchronize(ctx->stream);
    ctx->stream = cuda_stream ? (cudaStream_t)cuda_stream : ctx->own_stream;
    return ETRAJ_OK;
}

int etraj_validate(const etraj_job* job, char* msg, size_t msg_len) {
    std::string err;
    int st = validate_job(job, err);
    if (msg && msg_len > 0) {
        std::strncpy(msg, err.c_str(), msg_len - 1);
        msg[msg_len - 1] = 0;
    }
    return st;
}

int etraj_batch_info(const etraj_job* job, int64_t* batch_num, int64_t* batch_max_size) {
    if (!job) return ETRAJ_ERR_INVALID_ARGUMENT;
    if (batch_num) *batch_num = job->sample_t_num;
    if (batch_max_size)
        *batch_max_size = job->sample_monte_carlo ? job->mc_kt_num
                                                  : job->ss_kd_num * ((job->dimension == 3) ? job->ss_kz_num : 1);
    return ETRAJ_OK;
}

int etraj_run(etraj_ctx* ctx, const etraj_job* job, etraj_result* out) {
    if (!ctx || !job || !out) return ETRAJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    return run_job(ctx, job, out);
}

int etraj_sample_batch(etraj_ctx* ctx, const etraj_job* job, int64_t batch_id, double* init, int64_t capacity,
                       int64_t* count) {
    if (!ctx || !job || !count) return ETRAJ_ERR_INVALID_ARGUMENT;
    if (batch_id < 1 || batch_id > job->sample_t_num)
        return set_err(ctx, ETRAJ_ERR_INVALID_ARGUMENT, "batch_id out of range");
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    return sample_range(ctx, job, batch_id - 1, 1, init, capacity, count);
}

int etraj_sample_all(etraj_ctx* ctx, const etraj_job* job, double* init, int64_t capacity, int64_t* count) {
    if (!ctx || !job || !count) return ETRAJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    return sample_range(ctx, job, 0, job->sample_t_num, init, capacity, count);
}

int etraj_integrate(etraj_ctx* ctx, const etraj_job* job, int64_t n, const double* init, double* final_state,
                    int32_t* status, int32_t* steps) {
    if (!ctx || !job || (n > 0 && !init) || n < 0) return ETRAJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    std::string err;
    int st = validate_job(job, err);
    if (st != ETRAJ_OK) return set_err(ctx, st, err);
    if (n == 0) return ETRAJ_OK;
    if (n >= ((int64_t)1 << 31)) return set_err(ctx, ETRAJ_ERR_INVALID_ARGUMENT, "n too large");
    HostJob H;
    prepare_job(job, H);
    const DJob& J = H.J;
    // unpack the reference `init` columns into a structure of arrays
    std::vector<double> x((size_t)n), y((size_t)n), kx((size_t)n), ky((size_t)n), kz((size_t)n, 0.0),
        rate((size_t)n), ph((size_t)n, 0.0), t0((size_t)n);
    std::vector<int32_t> batch((size_t)n);
    for (int64_t i = 0; i < n; ++i) {
        const double* r = init + i * J.rows;
        size_t u = (size_t)i;
        x[u] = r[0];
        y[u] = r[1];
        if (J.dim == 2) {
            kx[u] = r[2]; ky[u] = r[3]; t0[u] = r[4]; rate[u] = r[5];
        } else {
            kx[u] = r[3]; ky[u] = r[4]; kz[u] = r[5]; t0[u] = r[6]; rate[u] = r[7];
        }
        if (J.phase != ETRAJ_PHASE_CTMC) ph[u] = r[J.rows - 1];
        batch[u] = (int32_t)i;
    }
    Pipeline P;
    ETRAJ_TRY(ensure_t(ctx, "soa.x", (size_t)n, &P.soa.x));
    ETRAJ_TRY(ensure_t(ctx, "soa.y", (size_t)n, &P.soa.y));
    ETRAJ_TRY(ensure_t(ctx, "soa.kx", (size_t)n, &P.soa.kx));
    ETRAJ_TRY(ensure_t(ctx, "soa.ky", (size_t)n, &P.soa.ky));
    ETRAJ_TRY(ensure_t(ctx, "soa.kz", (size_t)n, &P.soa.kz));
    ETRAJ_TRY(ensure_t(ctx, "soa.rate", (size_t)n, &P.soa.rate));
    ETRAJ_TRY(ensure_t(ctx, "soa.phase", (size_t)n, &P.soa.phase));
    ETRAJ_TRY(ensure_t(ctx, "soa.batch", (size_t)n, &P.soa.batch));
    ETRAJ_TRY(ensure_t(ctx, "t", (size_t)n, &P.t));
    ETRAJ_TRY(ensure_t(ctx, "count", 4, &P.count));
    ETRAJ_TRY(alloc_outputs(ctx, J, n, true, P));
    cudaStream_t s = ctx->stream;
    auto up = [&](void* d, const void* h, size_t b) { cudaMemcpyAsync(d, h, b, cudaMemcpyHostToDevice, s); };
    up(P.soa.x, x.data(), (size_t)n * 8);
    up(P.soa.y, y.data(), (size_t)n * 8);
    up(P.soa.kx, kx.data(), (size_t)n * 8);
    up(P.soa.ky, ky.data(), (size_t)n * 8);
    up(P.soa.kz, kz.data(), (size_t)n * 8);
    up(P.soa.rate, rate.data(), (size_t)n * 8);
    up(P.soa.phase, ph.data(), (size_t)n * 8);
    up(P.soa.batch, batch.data(), (size_t)n * 4);
    up(P.t, t0.data(), (size_t)n * 8);
    unsigned long long cn = (unsigned long long)n;
    up(P.count, &cn, sizeof cn);
    int nl = 0;
    ETRAJ_TRY(launch_integrate(ctx, J, P.soa, P.t, nullptr, P.count, P.out, n, P.work, job->precision,
                               *std::min_element(t0.begin(), t0.end()), &nl));
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_err(ctx, e, "integrate launch");
    std::vector<int32_t> stv((size_t)n);
    if (final_state)
        cudaMemcpyAsync(final_state, P.out.final_state, (size_t)n * J.n_state * 8, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(stv.data(), P.out.status, (size_t)n * 4, cudaMemcpyDeviceToHost, s);
    if (steps) cudaMemcpyAsync(steps, P.out.steps, (size_t)n * 4, cudaMemcpyDeviceToHost, s);
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_err(ctx, e, "etraj_integrate");
    if (status)
        for (int64_t i = 0; i < n; ++i) status[i] = stv[(size_t)i] & 0xff;
    return ETRAJ_OK;
}

// Asynchronous jobs on one context: enqueued on its stream in submission order
// (the host set-up of the next job overlaps the device work of the previous
// one); results are staged in pinned memory and copied out at poll/wait.
int etraj_submit(etraj_ctx* ctx, const etraj_job* job, etraj_result* out, uint64_t* ticket) {
    if (!ctx || !job || !ticket || !out) return ETRAJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    const uint64_t tk = ctx->next_ticket++;
    JobRec& r = ctx->jobs[tk];
    r.ticket = tk;
    r.res = *out;
    r.staged = true;
    r.status = enqueue_job(ctx, job, r);
    if (r.status != ETRAJ_OK) {
        r.error = ctx->err;
        release_job(ctx, r);
    }
    *ticket = tk;
    return ETRAJ_OK;
}

namespace {
// Completes ticket tk of ctx if it is done (blocking when `block`).
int poll_locked(etraj_ctx* ctx, uint64_t tk, etraj_result* out, bool block) {
    auto it = ctx->jobs.find(tk);
    if (it == ctx->jobs.end()) return set_err(ctx, ETRAJ_ERR_NOT_FOUND, "unknown ticket");
    JobRec& r = it->second;
    int st = r.status;
    if (st == ETRAJ_OK) {
        cudaError_t e = block ? cudaEventSynchronize(r.ev_done) : cudaEventQuery(r.ev_done);
        if (e == cudaErrorNotReady) {
            cudaGetLastError();
            return ETRAJ_ERR_NOT_READY;
        }
        if (e != cudaSuccess) {
            st = cuda_err(ctx, e, "etraj_poll");
            release_job(ctx, r);
        } else {
            st = finish_job(ctx, r);
        }
    } else {
        ctx->err = r.error;
    }
    double* ms = out->momentum_spec;
    double* amp = out->amplitude;
    *out = r.res;
    out->momentum_spec = ms;
    out->amplitude = amp;
    ctx->jobs.erase(it);
    return st;
}
}  // namespace

int etraj_poll(etraj_ctx* ctx, uint64_t ticket, etraj_result* out) {
    if (!ctx || !out) return ETRAJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    return poll_locked(ctx, ticket, out, false);
}

int etraj_wait(etraj_ctx* ctx, uint64_t ticket, etraj_result* out) {
    if (!ctx || !out) return ETRAJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    return poll_locked(ctx, ticket, out, true);
}

// ---- server: continuous batching of many jobs on one GPU -----------------------------
// `slots` contexts, each with its own stream and buffers.  A submitted job waits
// in a FIFO queue until a slot is free and the device bytes it would add fit in
// the server's HBM budget; it is then enqueued on that slot and overlaps on the
// device with the jobs of the other slots.  A job's result depends on nothing
// but the job: no state is shared between slots.
}  // extern "C"

struct etraj_server {
    int device = 0;
    size_t budget = 0;
    std::vector<etraj_ctx*> slot;
    std::vector<uint64_t> slot_ticket;  // 0: free
    struct Req {
        etraj_job job;
        etraj_result res;
        uint64_t ticket;
    };
    std::deque<Req> queue;
    std::map<uint64_t, JobRec> running;
    std::map<uint64_t, int> running_slot;
    struct Done {
        int status;
        std::string error;
        etraj_result res;
    };
    std::map<uint64_t, Done> done;
    uint64_t next_ticket = 1;
    std::string err;
    std::mutex mu;
};

namespace {

size_t server_used(const etraj_server* srv) {
    size_t u = 0;
    for (const etraj_ctx* c : srv->slot) u += c->used;
    return u;
}

void free_ctx_buffers(etraj_ctx* ctx) {
    for (auto& kv : ctx->bufs)
        if (kv.second.p) cudaFreeAsync(kv.second.p, ctx->stream);
    ctx->bufs.clear();
    ctx->used = 0;
}

// Retires finished jobs and admits queued ones (server lock held).
void server_progress(etraj_server* srv) {
    cudaSetDevice(srv->device);
    for (size_t i = 0; i < srv->slot.size(); ++i) {
        const uint64_t tk = srv->slot_ticket[i];
        if (!tk) continue;
        etraj_ctx* ctx = srv->slot[i];
        JobRec& r = srv->running[tk];
        cudaError_t e = cudaEventQuery(r.ev_done);
        if (e == cudaErrorNotReady) {
            cudaGetLastError();
            continue;
        }
        etraj_server::Done d;
        if (e == cudaSuccess) {
            d.status = finish_job(ctx, r);
        } else {
            d.status = cuda_err(ctx, e, "server job");
            release_job(ctx, r);
        }
        d.error = (d.status == ETRAJ_OK) ? std::string() : ctx->err;
        d.res = r.res;
        srv->done[tk] = d;
        srv->running.erase(tk);
        srv->running_slot.erase(tk);
        srv->slot_ticket[i] = 0;
    }
    while (!srv->queue.empty()) {
        int free_slot = -1;
        for (size_t i = 0; i < srv->slot.size(); ++i)
            if (!srv->slot_ticket[i]) {
                free_slot = (int)i;
                break;
            }
        if (free_slot < 0) return;
        etraj_server::Req& q = srv->queue.front();
        etraj_ctx* ctx = srv->slot[(size_t)free_slot];
        size_t growth = plan_growth(ctx, &q.job);
        if (server_used(srv) + growth > srv->budget) {
            // give back the buffers of idle slots, then re-plan
            for (size_t i = 0; i < srv->slot.size(); ++i)
                if (!srv->slot_ticket[i] && (int)i != free_slot) free_ctx_buffers(srv->slot[i]);
            growth = plan_growth(ctx, &q.job);
            if (server_used(srv) + growth > srv->budget) {
                free_ctx_buffers(ctx);
                growth = plan_growth(ctx, &q.job);
            }
            if (server_used(srv) + growth > srv->budget) {
                if (!srv->running.empty()) return;  // wait for memory
                etraj_server::Done d;
                d.status = ETRAJ_ERR_OUT_OF_MEMORY;
                d.error = "job needs " + std::to_string(growth) + " device bytes; server budget " +
                          std::to_string(srv->budget);
                d.res = q.res;
                srv->done[q.ticket] = d;
                srv->queue.pop_front();
                continue;
            }
        }
        JobRec r;
        r.res = q.res;
        r.staged = true;
        const int st = enqueue_job(ctx, &q.job, r);
        if (st != ETRAJ_OK) {
            release_job(ctx, r);
            etraj_server::Done d;
            d.status = st;
            d.error = ctx->err;
            d.res = q.res;
            srv->done[q.ticket] = d;
        } else {
            srv->running[q.ticket] = r;
            srv->running_slot[q.ticket] = free_slot;
            srv->slot_ticket[(size_t)free_slot] = q.ticket;
        }
        srv->queue.pop_front();
    }
}

// Takes a finished ticket's result (server lock held); NOT_READY while queued or running.
int server_take(etraj_server* srv, uint64_t tk, etraj_result* out) {
    auto it = srv->done.find(tk);
    if (it == srv->done.end()) {
        if (srv->running.count(tk)) return ETRAJ_ERR_NOT_READY;
        for (const auto& q : srv->queue)
            if (q.ticket == tk) return ETRAJ_ERR_NOT_READY;
        srv->err = "unknown ticket";
        return ETRAJ_ERR_NOT_FOUND;
    }
    double* ms = out->momentum_spec;
    double* amp = out->amplitude;
    *out = it->second.res;
    out->momentum_spec = ms;
    out->amplitude = amp;
    const int st = it->second.status;
    if (st != ETRAJ_OK) srv->err = it->second.error;
    srv->done.erase(it);
    return st;
}

}  // namespace

extern "C" {

int etraj_server_create(etraj_server** out, int device, int slots, size_t hbm_budget_bytes) {
    if (!out || slots < 1 || slots > 64) return ETRAJ_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    etraj_server* srv = new etraj_server();
    srv->device = device;
    for (int i = 0; i < slots; ++i) {
        etraj_ctx* c = nullptr;
        const int st = etraj_create(&c, device, hbm_budget_bytes);
        if (st != ETRAJ_OK) {
            for (etraj_ctx* d : srv->slot) etraj_destroy(d);
            delete srv;
            return st;
        }
        srv->slot.push_back(c);
        srv->slot_ticket.push_back(0);
    }
    // the server enforces one budget over all slots
    srv->budget = srv->slot[0]->budget;
    for (etraj_ctx* c : srv->slot) c->budget = (size_t)-1 / 2;
    *out = srv;
    return ETRAJ_OK;
}

void etraj_server_destroy(etraj_server* srv) {
    if (!srv) return;
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        cudaSetDevice(srv->device);
        for (size_t i = 0; i < srv->slot.size(); ++i) {
            const uint64_t tk = srv->slot_ticket[i];
            if (!tk) continue;
            cudaEventSynchronize(srv->running[tk].ev_done);
            release_job(srv->slot[i], srv->running[tk]);
        }
    }
    for (etraj_ctx* c : srv->slot) etraj_destroy(c);
    delete srv;
}

int etraj_server_submit(etraj_server* srv, const etraj_job* job, etraj_result* out, uint64_t* ticket) {
    if (!srv || !job || !out || !ticket) return ETRAJ_ERR_INVALID_ARGUMENT;
    std::string err;
    const int st = validate_job(job, err);
    if (st != ETRAJ_OK) {
        std::lock_guard<std::mutex> lk(srv->mu);
        srv->err = err;
        return st;
    }
    std::lock_guard<std::mutex> lk(srv->mu);
    const uint64_t tk = srv->next_ticket++;
    srv->queue.push_back(etraj_server::Req{*job, *out, tk});
    server_progress(srv);
    *ticket = tk;
    return ETRAJ_OK;
}

int etraj_server_poll(etraj_server* srv, uint64_t ticket, etraj_result* out) {
    if (!srv || !out) return ETRAJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(srv->mu);
    server_progress(srv);
    return server_take(srv, ticket, out);
}

int etraj_server_wait(etraj_server* srv, uint64_t ticket, etraj_result* out, double timeout_s) {
    if (!srv || !out) return ETRAJ_ERR_INVALID_ARGUMENT;
    const auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        {
            std::lock_guard<std::mutex> lk(srv->mu);
            server_progress(srv);
            const int st = server_take(srv, ticket, out);
            if (st != ETRAJ_ERR_NOT_READY) return st;
        }
        const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (timeout_s >= 0.0 && el > timeout_s) {
            std::lock_guard<std::mutex> lk(srv->mu);
            srv->err = "etraj_server_wait: timed out";
            return ETRAJ_ERR_TIMEOUT;
        }
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
}

int etraj_server_stats(etraj_server* srv, int64_t* running, int64_t* queued, size_t* hbm_in_use) {
    if (!srv) return ETRAJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(srv->mu);
    server_progress(srv);
    if (running) *running = (int64_t)srv->running.size();
    if (queued) *queued = (int64_t)srv->queue.size();
    if (hbm_in_use) *hbm_in_use = server_used(srv);
    return ETRAJ_OK;
}

const char* etraj_server_last_error(const etraj_server* srv) { return srv ? srv->err.c_str() : "no server"; }

int etraj_run_batch(etraj_ctx* ctx, const etraj_job* jobs, int n_jobs, etraj_result* results,
                    const double* weights, double* weighted_spec) {
    if (!ctx) return ETRAJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    return run_batch(ctx, jobs, n_jobs, results, weights, weighted_spec);
}

int etraj_set_graphs(etraj_ctx* ctx, int enable) {
    if (!ctx) return ETRAJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->graphs = (enable != 0);
    if (!enable && (ctx->gexec || ctx->bgexec)) {
        cudaStreamSynchronize(ctx->stream);
        if (ctx->gexec) cudaGraphExecDestroy(ctx->gexec);
        if (ctx->bgexec) cudaGraphExecDestroy(ctx->bgexec);
        ctx->gexec = ctx->bgexec = nullptr;
        ctx->gkey.clear();
        ctx->bgkey.clear();
    }
    return ETRAJ_OK;
}

int etraj_set_autotune(etraj_ctx* ctx, int enable) {
    if (!ctx) return ETRAJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->autotune = (enable != 0);
    if (!enable) ctx->tiles.clear();
    return ETRAJ_OK;
}

int etraj_bulk_tile(etraj_ctx* ctx, int dimension, int phase, int target, int multi, int* threads,
                    int* blocks_per_sm, int* refill_min) {
    if (!ctx) return ETRAJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    const int key = (multi ? 1000 : 0) + dimension * 100 + phase * 10 + target;
    BulkTile t = kTileDefault;
    const bool found = find_tile(ctx, key, &t);
    if (threads) *threads = t.threads;
    if (blocks_per_sm) *blocks_per_sm = t.blocks_per_sm;
    if (refill_min) *refill_min = t.refill_min;
    return found ? ETRAJ_OK : ETRAJ_ERR_NOT_FOUND;
}

int etraj_set_bulk_tile(etraj_ctx* ctx, int dimension, int phase, int target, int multi, int threads,
                        int blocks_per_sm, int refill_min) {
    if (!ctx) return ETRAJ_ERR_INVALID_ARGUMENT;
    const int warps = (threads / 32) * blocks_per_sm;
    if ((threads != 64 && threads != 128 && threads != 256) || blocks_per_sm < 1 || warps > 24 ||
        refill_min < 1 || refill_min > 32)
        return ETRAJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    const int key = (multi ? 1000 : 0) + dimension * 100 + phase * 10 + target;
    BulkTile old = kTileDefault;
    find_tile(ctx, key, &old);
    ctx->tiles[key] = BulkTile{threads, blocks_per_sm, refill_min, warps > 16 ? 3 : 2, old.chunk};
    return ETRAJ_OK;
}

int etraj_bulk_step_chunk(etraj_ctx* ctx, int dimension, int phase, int target, int multi, int* steps) {
    if (!ctx) return ETRAJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    const int key = (multi ? 1000 : 0) + dimension * 100 + phase * 10 + target;
    BulkTile t = kTileDefault;
    const bool found = find_tile(ctx, key, &t);
    if (steps) *steps = t.chunk;
    return found ? ETRAJ_OK : ETRAJ_ERR_NOT_FOUND;
}

int etraj_set_bulk_step_chunk(etraj_ctx* ctx, int dimension, int phase, int target, int multi, int steps) {
    if (!ctx || steps < 16 || steps > (1 << 16)) return ETRAJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    const int key = (multi ? 1000 : 0) + dimension * 100 + phase * 10 + target;
    BulkTile t = kTileDefault;
    find_tile(ctx, key, &t);
    t.chunk = steps;
    ctx->tiles[key] = t;
    return ETRAJ_OK;
}

int etraj_set_straggler_repack(etraj_ctx* ctx, int enable) {
    if (!ctx) return ETRAJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->repack = (enable != 0);
    return ETRAJ_OK;
}

int etraj_set_static_assignment(etraj_ctx* ctx, int enable) {
    if (!ctx) return ETRAJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->static_assign = (enable != 0);
    return ETRAJ_OK;
}

int etraj_set_keep_final_states(etraj_ctx* ctx, int enable) {
    if (!ctx) return ETRAJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->keep_states = (enable != 0);
    return ETRAJ_OK;
}

namespace {
// Number of survivors of the kept job, after it has finished (ticket 0: the last job).
int dump_prepare(etraj_ctx* ctx, uint64_t ticket, int64_t* n) {
    if (!ctx->dump_valid || (ticket != 0 && ticket != ctx->dump_ticket))
        return set_err(ctx, ETRAJ_ERR_NOT_FOUND,
                       "final states are kept only for the context's last job, and only when "
                       "etraj_set_keep_final_states was on when it was enqueued");
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    unsigned long long c = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&c, ctx->dump_count, sizeof c, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_err(ctx, e, "final states");
    *n = (int64_t)c;
    return ETRAJ_OK;
}
}  // namespace

int etraj_dump_final_states(etraj_ctx* ctx, uint64_t ticket, double* p_inf, double* phase, int32_t* status) {
    if (!ctx) return ETRAJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    int64_t n = 0;
    ETRAJ_TRY(dump_prepare(ctx, ticket, &n));
    if (n == 0) return ETRAJ_OK;
    const TrajOut& o = ctx->dump_out;
    cudaError_t e = cudaSuccess;
    if (p_inf && e == cudaSuccess) e = cudaMemcpy(p_inf, o.p_inf, (size_t)n * 3 * 8, cudaMemcpyDeviceToHost);
    if (phase && e == cudaSuccess) e = cudaMemcpy(phase, o.fphase, (size_t)n * 8, cudaMemcpyDeviceToHost);
    if (status && e == cudaSuccess) e = cudaMemcpy(status, o.status, (size_t)n * 4, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_err(ctx, e, "final states");
    return ETRAJ_OK;
}

int etraj_dump_step_counts(etraj_ctx* ctx, uint64_t ticket, int32_t* steps) {
    if (!ctx || !steps) return ETRAJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    int64_t n = 0;
    ETRAJ_TRY(dump_prepare(ctx, ticket, &n));
    if (n == 0) return ETRAJ_OK;
    cudaError_t e = cudaMemcpy(steps, ctx->dump_out.steps, (size_t)n * 4, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_err(ctx, e, "step counts");
    return ETRAJ_OK;
}

int etraj_dump_min_radius(etraj_ctx* ctx, uint64_t ticket, double* rmin) {
    if (!ctx || !rmin) return ETRAJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    int64_t n = 0;
    ETRAJ_TRY(dump_prepare(ctx, ticket, &n));
    if (!ctx->dump_out.rmin)
        return set_err(ctx, ETRAJ_ERR_UNSUPPORTED, "the least radius is tracked by the FP64 path only");
    if (n == 0) return ETRAJ_OK;
    cudaError_t e = cudaMemcpy(rmin, ctx->dump_out.rmin, (size_t)n * 8, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_err(ctx, e, "least radius");
    return ETRAJ_OK;
}

int etraj_stage_times(etraj_ctx* ctx, double* ms, int n) {
    if (!ctx || !ms) return 0;
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (!ctx->stage_valid) return 0;
    if (cudaEventSynchronize(ctx->stage_ev[etraj_ctx::kStages]) != cudaSuccess) return 0;
    int k = 0;
    for (; k < etraj_ctx::kStages && k < n; ++k) {
        float f = 0.f;
        cudaEventElapsedTime(&f, ctx->stage_ev[k], ctx->stage_ev[k + 1]);
        ms[k] = f;
    }
    return k;
}

}  // extern "C"
