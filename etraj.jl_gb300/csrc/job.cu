// job.cu -- the checks of a job (the reference's constructor assertions and
// messages) and its host-side set-up: time and momentum samples, the sampler's
// per-job constants, the target and the grid, in the reference's expressions.
#include "host.h"

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

}  // namespace

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

