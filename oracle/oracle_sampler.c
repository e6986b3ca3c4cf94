/*
 * oracle_sampler.c -- initial-condition sampling of the CPU oracle (TEST
 * INFRASTRUCTURE ONLY; see oracle.h).
 *
 * Restates:
 *   src/ElectronSamplers/ADKSampler.jl:19-396   (ctor checks, gen_electron_batch)
 *   src/ElectronSamplers/SPANESampler.jl:19-404
 *   src/ElectronSamplers/SPASampler.jl:19-431 (with the shared spa.h)
 *   src/ElectronSamplers/shared_methods.jl:4-47 (random points, solid
 *     harmonics, FF->MF Euler angles, field-frame axes)
 *   src/ElectronSamplers/WFATSampler.jl:129-249 and the molecular branches of
 *     the ADK, SPANE and SPA prefactors (the shared mol.h)
 *
 * Monte-Carlo draws: the reference uses Julia's unseeded global RNG
 * (shared_methods.jl:4-12, ADKSampler.jl:141).  Here every draw comes from a
 * counter-based Philox4x32-10 stream (Salmon et al., SC'11) keyed by the
 * job's seed, so the device and the oracle draw identical numbers:
 *   time samples:  counter (j, 0, 0x54494D45), u53 from words 0,1
 *   kd, kz:        counter (i, batch, 0x4B445A00), kd from words 0,1, kz from 2,3
 * u53(a,b) = ((a>>5)*2^26 + (b>>6)) * 2^-53 (uniform on [0,1)).
 */
#include "oracle_internal.h"
#include "oracle_sampler.h"

/* ---- Philox4x32-10 ---------------------------------------------------------- */
void o_philox4x32(uint32_t c[4], uint64_t seed) {
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

double o_u53(uint32_t a, uint32_t b) {
    return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) * (1.0 / 9007199254740992.0);
}

/* ---- Julia range(a, b; length=n), element i (0-based) ------------------------ */
static void two_sum(double a, double b, double* s, double* e) {
    double ss = a + b, bb = ss - a;
    *s = ss;
    *e = (a - (ss - bb)) + (b - bb);
}

double o_linrange(double a, double b, int64_t n, int64_t i) {
    if (n == 1 || i == 0) return a;
    if (i == n - 1) return b;
    double lim = 4503599627370496.0 / (double)n; /* 2^52 / n */
    if (a == rint(a) && b == rint(b) && fabs(a) < lim && fabs(b) < lim) {
        /* integer end points: the exact rational value, rounded once (what
         * Julia's rational-endpoint path produces) */
        return (a * (double)(n - 1 - i) + b * (double)i) / (double)(n - 1);
    }
    /* double-double a + i*(b-a)/(n-1), rounded once */
    double dh, dl, m = (double)(n - 1), fi = (double)i;
    two_sum(b, -a, &dh, &dl);
    double q1 = dh / m;
    double r = fma(-q1, m, dh) + dl;
    double q2 = r / m;
    double p1 = fi * q1, p1e = fma(fi, q1, -p1);
    double p2 = fi * q2;
    double s, se;
    two_sum(a, p1, &s, &se);
    return s + (se + (p1e + p2));
}

/* ---- Wigner small-d and solid harmonics ---------------------------------------- */
static double o_fact(int n) {
    double f = 1.0;
    for (int i = 2; i <= n; ++i) f *= (double)i;
    return f;
}

/* d^j_{m'm}(beta) by Wigner's explicit sum (standard convention). */
static double o_wigner_d(int j, int mp, int m, double beta) {
    double sh, ch;
    dm_sincos(0.5 * beta, &sh, &ch);
    double pref = sqrt(o_fact(j + mp) * o_fact(j - mp) * o_fact(j + m) * o_fact(j - m));
    double sum = 0.0;
    for (int s = 0; s <= 2 * j; ++s) {
        int a1 = j + m - s, a3 = mp - m + s, a4 = j - mp - s;
        if (a1 < 0 || a3 < 0 || a4 < 0) continue;
        double den = o_fact(a1) * o_fact(s) * o_fact(a3) * o_fact(a4);
        double sign = ((mp - m + s) & 1) ? -1.0 : 1.0;
        int pc = 2 * j + m - mp - 2 * s, ps = mp - m + 2 * s;
        double cpow = 1.0, spow = 1.0;
        for (int i = 0; i < pc; ++i) cpow *= ch;
        for (int i = 0; i < ps; ++i) spow *= sh;
        sum = sum + ((sign * pref / den) * cpow) * spow;
    }
    return sum;
}

/* Prefactor of the solid harmonic Y_{l m}(x,y,z) of shared_methods.jl:21:
 * (-1)^m sqrt((2l+1)/4pi (l-m)!/(l+m)!) / (-i kappa)^l * (l+m)!. */
static dm_cplx o_sph_prefactor(int l, int m, double kappa) {
    double A = (m & 1) ? -1.0 : 1.0;
    double B = sqrt((((2.0 * l + 1.0) / 12.566370614359172) * o_fact(l - m)) / o_fact(l + m));
    dm_cplx C = dm_cpowi(dm_c(0.0, -kappa), l);
    dm_cplx P = dm_cdiv(dm_c(A * B, 0.0), C);
    return dm_cscale(P, o_fact(l + m));
}

/* The k-sum of shared_methods.jl:21 at complex (x, y, z). */
static dm_cplx o_sph_sum(int l, int m, dm_cplx x, dm_cplx y, dm_cplx z) {
    dm_cplx xp = dm_c(x.re - y.im, x.im + y.re); /* x + i y */
    dm_cplx xm = dm_c(x.re + y.im, x.im - y.re); /* x - i y */
    int kmin = (m < 0) ? -m : 0, kmax = (l - m) / 2;
    dm_cplx acc = dm_c(0.0, 0.0);
    for (int k = kmin; k <= kmax; ++k) {
        double den = o_fact(k + m) * o_fact(k) * o_fact(l - m - 2 * k);
        double p2 = 1.0;
        for (int i = 0; i < 2 * k + m; ++i) p2 *= 2.0;
        double coef = ((k & 1) ? -1.0 : 1.0) / (p2 * den);
        dm_cplx t = dm_cscale(dm_cpowi(xp, k + m), coef);
        t = dm_cmul(t, dm_cpowi(xm, k));
        t = dm_cmul(t, dm_cpowi(z, l - m - 2 * k));
        acc = (k == kmin) ? t : dm_cadd(acc, t);
    }
    return acc;
}

/* ---- job-level sampler set-up (ADKSampler.jl:19-149) --------------------------- */
static int o_prefix_normalize(const etraj_job* job) {
    int p = job->rate_prefix;
    /* :PreCC is replaced by :Pre for non-monochromatic lasers (ADKSampler.jl:72-77) */
    if ((p & ETRAJ_PREFIX_PRECC) && job->laser.kind == ETRAJ_LASER_BICHROMATIC) {
        p = (p & ~ETRAJ_PREFIX_PRECC) | ETRAJ_PREFIX_PRE;
    }
    return p;
}

int o_sampler_init(const etraj_job* job, o_sampler* S) {
    memset(S, 0, sizeof *S);
    S->method = job->init_cond_method;
    S->dim = job->dimension;
    S->mc = job->sample_monte_carlo;
    S->prefix = o_prefix_normalize(job);
    S->phase = job->traj_phase_method;
    S->rows = (S->dim == 3) ? ((S->phase == ETRAJ_PHASE_CTMC) ? 8 : 9)
                            : ((S->phase == ETRAJ_PHASE_CTMC) ? 6 : 7);
    S->cutoff = job->sample_cutoff_limit;
    S->seed = job->seed;
    o_laser_prepare(&job->laser, &S->laser);
    S->mono = (job->laser.kind != ETRAJ_LASER_BICHROMATIC);
    /* SPA's omega: the laser's, or the mean of the two for a bichromatic one */
    S->spa_omega = S->mono ? S->laser.m[0].omega : (S->laser.m[0].omega + S->laser.m[1].omega) / 2.0;
    const etraj_target* T = &job->target;
    S->Ip = T->Ip;
    S->Z = (double)T->Z;
    S->l = T->l;
    S->m = T->m;
    S->C = T->asymp_coeff;
    S->q_theta = T->quan_ax_theta;
    S->q_phi = T->quan_ax_phi;
    S->kappa = sqrt(2.0 * S->Ip);
    S->n = S->Z / S->kappa;
    double n = S->n;
    S->c = (dm_pow_pos(2.0, n / 2.0 + 1.0) * dm_pow_pos(S->kappa, 2.0 * n + 0.5)) * tgamma(n / 2.0 + 1.0);
    S->cc_base = dm_pow_pos(2.0, (3.0 * n) / 2.0 + 1.0) * dm_pow_pos(S->kappa, 5.0 * n + 0.5);
    S->e_pre = (n + 1.0) / 4.0;
    for (int mp = -S->l; mp <= S->l; ++mp) S->Plm[mp + S->l] = o_sph_prefactor(S->l, mp, S->kappa);
    if (T->kind == ETRAJ_TARGET_MOLECULE) {
        S->mol = 1;
        S->wfat = (S->method == ETRAJ_SAMPLER_WFAT);
        for (int i = 0; i < 3; ++i) S->mol_rot[i] = T->mol_rot[i];
        if (S->wfat) {
            S->nxi = T->wfat_nxi_max;
            S->mmax = T->wfat_m_max;
            S->wl = T->wfat_lmax;
            S->wint = T->wfat_intdata;
            for (int i = 0; i < 3; ++i) S->mu[i] = T->wfat_mu[i];
        } else {
            S->clm = T->asymp_coeff_lm;
            mol_terms_build(T->asymp_lmax, S->clm, &S->T);
            for (int l = 0; l <= T->asymp_lmax; ++l)
                for (int mp = -l; mp <= l; ++mp) {
                    const dm_cplx P = mol_sph_prefactor(l, mp, S->kappa);
                    S->Pmol[2 * (l * l + l + mp)] = P.re;
                    S->Pmol[2 * (l * l + l + mp) + 1] = P.im;
                }
        }
    }

    S->n_t = job->sample_t_num;
    S->t = (double*)malloc(sizeof(double) * (size_t)S->n_t);
    if (!S->t) return -1;
    oracle_t_samples(job, S->t);
    double t_step = (S->t[S->n_t - 1] - S->t[0]) / (double)S->n_t; /* step(range) of ADKSampler.jl:267 */
    if (!S->mc) {
        int64_t nkd = job->ss_kd_num, nkz = (S->dim == 3) ? job->ss_kz_num : 1;
        double kdm = fabs(job->ss_kd_max), kzm = (S->dim == 3) ? fabs(job->ss_kz_max) : 0.0;
        S->n_kd = nkd;
        S->n_kz = nkz;
        S->kd = (double*)malloc(sizeof(double) * (size_t)nkd);
        S->kz = (double*)malloc(sizeof(double) * (size_t)nkz);
        for (int64_t i = 0; i < nkd; ++i) S->kd[i] = o_linrange(-kdm, kdm, nkd, i);
        for (int64_t i = 0; i < nkz; ++i) S->kz[i] = o_linrange(-kzm, kzm, nkz, i);
        double kd_step = (nkd > 1) ? (kdm - (-kdm)) / (double)nkd : 1.0;
        double kz_step = (S->dim == 3 && nkz > 1) ? (kzm - (-kzm)) / (double)nkz : 1.0;
        S->dkdt = (t_step * kd_step) * kz_step;
        S->n_cand = nkd * nkz;
    } else {
        S->mc_kd_max = job->mc_kd_max;
        S->mc_kz_max = job->mc_kz_max;
        double kd_span = (job->mc_kd_max > 0.0) ? 2.0 * job->mc_kd_max : 1.0;
        double kz_span = (job->mc_kz_max > 0.0) ? 2.0 * job->mc_kz_max : 1.0;
        S->dkdt = ((t_step * kd_span) * kz_span) / (double)job->mc_kt_num;
        S->gauss = (job->mc_kt_proposal == ETRAJ_PROPOSAL_ADK_GAUSS) ? 1 : 0;
        S->dkdt_base = (S->dim == 3 ? t_step : t_step * kz_span) / (double)job->mc_kt_num;
        S->n_cand = job->mc_kt_num;
    }
    return 0;
}

void o_sampler_free(o_sampler* S) {
    free(S->t);
    free(S->kd);
    free(S->kz);
    memset(S, 0, sizeof *S);
}

/* ---- per-batch constants (gen_electron_batch prologue, ADKSampler.jl:168-296) --- */
static void o_rotzyz(double a, double b, double g, double R[3][3]) {
    double sa, ca, sb, cb, sg, cg;
    dm_sincos(a, &sa, &ca);
    dm_sincos(b, &sb, &cb);
    dm_sincos(g, &sg, &cg);
    /* Rz(a) Ry(b) Rz(g) */
    R[0][0] = ca * cb * cg - sa * sg; R[0][1] = -(ca * cb * sg) - sa * cg; R[0][2] = ca * sb;
    R[1][0] = sa * cb * cg + ca * sg; R[1][1] = -(sa * cb * sg) + ca * cg; R[1][2] = sa * sb;
    R[2][0] = -(sb * cg);             R[2][1] = sb * sg;                   R[2][2] = cb;
}

void o_batch_prepare(const o_sampler* S, int64_t b, o_batch* B) {
    memset(B, 0, sizeof *B);
    double tr = S->t[b];
    B->tr = tr;
    if (S->method == ETRAJ_SAMPLER_SPANE) {
        o_laser_F_dual(&S->laser, tr, &B->Fx, &B->Fy, &B->dFx, &B->dFy);
    } else {
        o_laser_F(&S->laser, tr, &B->Fx, &B->Fy);
    }
    B->F = dm_hypot(B->Fx, B->Fy);
    B->phi = dm_atan2(-B->Fy, -B->Fx);
    dm_sincos(B->phi, &B->sphi, &B->cphi);
    if (S->mono) {
        const o_mono* M = &S->laser.m[0];
        B->gamma = (M->omega * S->kappa) / (M->F0 * o_mono_env(M, tr));
    } else {
        B->gamma = 0.0;
    }
    B->c_cc = (S->cc_base * dm_pow_pos(B->F, -S->n)) * dm_pow_pos(1.0 + (2.0 * B->gamma) / 2.718281828459045, -S->n);
    B->W = B->Fx * B->dFy - B->dFx * B->Fy;
    /* field-frame axes in the lab frame (shared_methods.jl:42-47) */
    B->ny[0] = B->Fy / B->F; B->ny[1] = -B->Fx / B->F; B->ny[2] = 0.0;
    B->nz[0] = B->Fx / B->F; B->nz[1] = B->Fy / B->F; B->nz[2] = 0.0;
    /* Euler angles FF -> MF (shared_methods.jl:31-38) with MF = RotZYZ(phi, theta, 0) */
    double FF[3][3] = {{0.0, B->Fy / B->F, B->Fx / B->F},
                       {0.0, -B->Fx / B->F, B->Fy / B->F},
                       {1.0, 0.0, 0.0}};
    double MF[3][3], M[3][3];
    o_rotzyz(S->q_phi, S->q_theta, 0.0, MF);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            M[i][j] = (MF[0][i] * FF[0][j] + MF[1][i] * FF[1][j]) + MF[2][i] * FF[2][j];
    double t1 = dm_atan2(M[1][2], M[0][2]);
    double st1, ct1;
    dm_sincos(t1, &st1, &ct1);
    double t2 = dm_atan2(M[0][2] * ct1 + M[1][2] * st1, M[2][2]);
    double t3 = dm_atan2(M[1][0] * ct1 - M[0][0] * st1, M[1][1] * ct1 - M[0][1] * st1);
    if (S->mol) {
        /* molecular frame RotZYZ(MolRotation) instead of the quantization axis */
        double a, b_, g;
        mol_euler(S->mol_rot, B->Fx, B->Fy, B->F, &a, &b_, &g);
        if (S->wfat) {
            const int nch = (S->nxi + 1) * (2 * S->mmax + 1), na = (S->nxi + 1) * (S->mmax + 1);
            for (int c = 0; c < nch; ++c) B->g2[c] = mol_wfat_g2(c, S->nxi, S->mmax, S->wl, S->wint, S->mu, S->kappa, b_, g);
            for (int e = 0; e < na; ++e) B->A[e] = mol_wfat_A(e, S->nxi, S->kappa, S->n, B->F);
        } else {
            for (int e = 0; e < S->T.ncd; ++e) {
                const dm_cplx v = mol_cd_entry(&S->T, S->clm, e, a, b_, g);
                B->cd[2 * e] = v.re;
                B->cd[2 * e + 1] = v.im;
            }
        }
        return;
    }
    /* D^l_{m' m}(a,b,g) = e^{-i m' a} d^l_{m' m}(b) e^{-i m g} for m' = -l..l */
    for (int mp = -S->l; mp <= S->l; ++mp) {
        double s1, c1, s3, c3;
        dm_sincos(-((double)mp * t1), &s1, &c1);
        dm_sincos(-((double)S->m * t3), &s3, &c3);
        double d = o_wigner_d(S->l, mp, S->m, t2);
        B->D[mp + S->l] = dm_cmul(dm_cscale(dm_c(c1, s1), d), dm_c(c3, s3));
    }
}

/* Sum over m' of C * D^l_{m' m} * Y_{l m'}(k_ts rotated to the field frame),
 * the numerator of pre() (ADKSampler.jl:243-265). */
/* which molecular rate pieces the sampler runs: the twin of the device's
 * (mol.h, 0) or the independent restatement of oracle_mol_ref.c (1) */
static int g_mol_independent = 0;
void oracle_set_mol_independent(int on) { g_mol_independent = on; }

dm_cplx o_pre_numerator(const o_sampler* S, const o_batch* B, dm_cplx kx, dm_cplx ky, dm_cplx kz) {
    /* new_k = conj(k_ts) . axis (LinearAlgebra.dot conjugates its first argument) */
    dm_cplx ckx = dm_cconj(kx), cky = dm_cconj(ky), ckz = dm_cconj(kz);
    dm_cplx nkx = dm_cadd(dm_cadd(dm_cscale(ckx, 0.0), dm_cscale(cky, 0.0)), dm_cscale(ckz, 1.0));
    dm_cplx nky = dm_cadd(dm_cadd(dm_cscale(ckx, B->ny[0]), dm_cscale(cky, B->ny[1])), dm_cscale(ckz, B->ny[2]));
    dm_cplx nkz = dm_cadd(dm_cadd(dm_cscale(ckx, B->nz[0]), dm_cscale(cky, B->nz[1])), dm_cscale(ckz, B->nz[2]));
    if (S->mol)
        return g_mol_independent ? o_mol_numerator_ref(S, B, nkx, nky, nkz)
                                 : mol_numerator(&S->T, B->cd, S->Pmol, nkx, nky, nkz);
    dm_cplx acc = dm_c(0.0, 0.0);
    for (int mp = -S->l; mp <= S->l; ++mp) {
        dm_cplx Y = dm_cmul(S->Plm[mp + S->l], o_sph_sum(S->l, mp, nkx, nky, nkz));
        dm_cplx term = dm_cmul(dm_cscale(B->D[mp + S->l], S->C), Y);
        acc = (mp == -S->l) ? term : dm_cadd(acc, term);
    }
    return acc;
}

/* One ADK / SPANE candidate (ADKSampler.jl:318-347, SPANESampler.jl:320-352).
 * Returns 1 and fills row[] when the electron survives the cutoff. */
int o_candidate(const o_sampler* S, const o_batch* B, double kd0, double kz0, double dkdt, double* row) {
    if (fabs(kd0) < 1e-4) return 0;
    /* a Gaussian draw outside +-mc_kd_max (+-mc_kz_max) is dropped */
    if (S->gauss && (fabs(kd0) > S->mc_kd_max || (S->dim == 3 && fabs(kz0) > S->mc_kz_max))) return 0;
    double Ip = S->Ip, F = B->F;
    double kx0 = kd0 * (-B->sphi);
    double ky0 = kd0 * B->cphi;
    double x0, y0, F2eff = 0.0, ti, X2, Fexp;
    int spane = (S->method == ETRAJ_SAMPLER_SPANE);
    if (!spane) {
        double r0 = (Ip + (kd0 * kd0 + kz0 * kz0) / 2.0) / F;
        x0 = r0 * B->cphi;
        y0 = r0 * B->sphi;
        ti = sqrt((S->kappa * S->kappa + kd0 * kd0) + kz0 * kz0) / F;
        X2 = (((kx0 * kx0 + ky0 * ky0) + kz0 * kz0) + 2.0 * Ip) * (F * F);
        Fexp = F;
    } else {
        F2eff = F * F - (kx0 * B->dFx + ky0 * B->dFy);
        double Xk = ((kx0 * kx0 + ky0 * ky0) + kz0 * kz0) + 2.0 * Ip;
        double r0 = ((F / 2.0) * Xk) / F2eff;
        x0 = r0 * B->cphi;
        y0 = r0 * B->sphi;
        double lim = S->mc ? (F * F) / 25.0 : (F * F) / 9.0;
        if (F2eff <= lim) return 0;
        ti = sqrt(((S->kappa * S->kappa + kd0 * kd0) + kz0 * kz0) / F2eff);
        X2 = Xk * F2eff;
        Fexp = sqrt(F2eff);
    }
    /* ADKAmpExp(F, Ip, kd, kz) = exp(-(kd^2+kz^2+2Ip)^1.5/3F) */
    double Xe = (kd0 * kd0 + kz0 * kz0) + 2.0 * Ip;
    double E = dm_exp(-(Xe * sqrt(Xe)) / (3.0 * Fexp));
    double r1 = sqrt(dkdt) * E;
    dm_cplx amp;
    if (S->prefix & (ETRAJ_PREFIX_PRE | ETRAJ_PREFIX_PRECC)) {
        dm_cplx kx, ky, kz = dm_c(kz0, 0.0);
        if (!spane) {
            kx = dm_c(kx0, -(ti * B->Fx));
            ky = dm_c(ky0, -(ti * B->Fy));
        } else {
            double h = (ti * ti) / 2.0;
            kx = dm_c(kx0 + h * B->dFx, -(ti * B->Fx));
            ky = dm_c(ky0 + h * B->dFy, -(ti * B->Fy));
        }
        dm_cplx num = o_pre_numerator(S, B, kx, ky, kz);
        double cpre = (S->prefix & ETRAJ_PREFIX_PRE) ? S->c : B->c_cc;
        double den = (S->e_pre == 0.5) ? sqrt(X2) : dm_pow_pos(X2, S->e_pre);
        dm_cplx pre = dm_cscale(num, cpre);
        pre = dm_c(pre.re / den, pre.im / den);
        amp = dm_cscale(pre, r1);
    } else {
        amp = dm_c(r1, 0.0);
    }
    if (S->prefix & ETRAJ_PREFIX_JAC) {
        double jac = spane ? fabs(F + (sqrt(kd0 * kd0 + kz0 * kz0) / (F * F)) * B->W) : F;
        amp = dm_cscale(amp, sqrt(jac));
    }
    double rate = amp.re * amp.re + amp.im * amp.im;
    double crit = spane ? rate / dkdt : rate;
    if (dm_isnan(rate) || crit < S->cutoff) return 0;
    int k = 0;
    row[k++] = x0;
    row[k++] = y0;
    if (S->dim == 3) row[k++] = 0.0;
    row[k++] = kx0;
    row[k++] = ky0;
    if (S->dim == 3) row[k++] = kz0;
    row[k++] = B->tr;
    row[k++] = rate;
    if (S->phase != ETRAJ_PHASE_CTMC) row[k++] = dm_carg(amp);
    return 1;
}

/* ---- SPA ---------------------------------------------------------------------- */
static void o_spa_AW(const o_laser* L, dm_cplx t, const double* win, dm_cplx* Ax, dm_cplx* Ay) {
    dm_cplx fx, fy;
    o_laser_AF_complex_w(L, t, win, Ax, Ay, &fx, &fy);
}
#define SPA_LASER_T o_laser
#define SPA_WIN(L, tre, w) o_laser_windows((L), (tre), (w))
#define SPA_AW(L, t, w, ax, ay) o_spa_AW((L), (t), (w), (ax), (ay))
#include "../etraj.jl_gb300/csrc/spa.h"

/* One SPA candidate (SPASampler.jl:320-347 for the grid, :364-391 for
 * Monte-Carlo); the batch is skipped before this when F(t_r) <= 1e-3 (:167-169). */
int o_candidate_spa(const o_sampler* S, const o_batch* B, double kd0, double kz0, double* row) {
    if (fabs(kd0) < 1e-4) return 0;
    const o_laser* L = &S->laser;
    const double tr = B->tr, Ip = S->Ip, w = S->spa_omega, wF = w / B->F;
    /* initial guess asinh(omega/F sqrt(kd^2+kz^2+2Ip))/omega (:242) */
    const double guess = dm_asinh(wF * sqrt((kd0 * kd0 + kz0 * kz0) + 2.0 * Ip)) / w;
    spa_win W;
    spa_win_init(&W);
    const double ti = spa_solve_ti(L, &W, tr, kd0, kz0, Ip, guess);
    if (ti == 0.0) return 0;
    dm_cplx Ax, Ay, Fx, Fy;
    o_laser_AF_complex(L, dm_c(tr, ti), &Ax, &Ay, &Fx, &Fy);
    double px, py;
    spa_pxy(kd0, Ax, Ay, &px, &py);
    spa_quad_par Q;
    Q.L = L; Q.W = &W; Q.tr = tr; Q.px = px; Q.py = py; Q.kz = kz0; Q.Ip = Ip;
    int ok01, ok2;
    double x0, y0;
    spa_exit(&Q, ti, &x0, &y0, &ok01);
    double axr, ayr;
    o_laser_A(L, tr, &axr, &ayr);
    const double kx0 = px + axr, ky0 = py + ayr;
    /* S_tun = -quadgk(..., t_r + i t_i, t_r) (:279); amplitude = sqrt(dkdt) exp(i S_tun) [pre] [sqrt(jac)] */
    const dm_cplx Si = spa_quadgk(SPA_INT_ACTION, &Q, dm_c(tr, ti), dm_c(tr, 0.0), &ok2);
    if (!(ok01 && ok2)) return 0;
    const dm_cplx St = dm_cneg(Si);
    const dm_cplx iS = dm_c(0.0 * St.re - 1.0 * St.im, 0.0 * St.im + 1.0 * St.re);
    dm_cplx amp = dm_cscale(dm_cexp(iS), sqrt(S->dkdt));
    if (S->prefix & (ETRAJ_PREFIX_PRE | ETRAJ_PREFIX_PRECC)) {
        const dm_cplx kx = dm_c(px + Ax.re, Ax.im), ky = dm_c(py + Ay.re, Ay.im), kz = dm_c(kz0, 0.0);
        const dm_cplx num = o_pre_numerator(S, B, kx, ky, kz);
        const double cpre = (S->prefix & ETRAJ_PREFIX_PRE) ? S->c : B->c_cc;
        /* (k_ts . F(t_s))^((n*+1)/2) (:257-262) */
        const dm_cplx kF = dm_caddr(dm_cadd(dm_cmul(kx, Fx), dm_cmul(ky, Fy)), kz0 * 0.0);
        const dm_cplx den = spa_cpow(kF, (S->n + 1.0) / 2.0);
        amp = dm_cmul(amp, dm_cdiv(dm_cscale(num, cpre), den));
    }
    if (S->prefix & ETRAJ_PREFIX_JAC) amp = dm_cscale(amp, sqrt(spa_jac(L, &W, tr, kd0, kz0, Ip, wF, w)));
    const double rate = amp.re * amp.re + amp.im * amp.im;
    if (dm_isnan(rate) || rate < S->cutoff) return 0;
    int k = 0;
    row[k++] = x0;
    row[k++] = y0;
    if (S->dim == 3) row[k++] = 0.0;
    row[k++] = kx0;
    row[k++] = ky0;
    if (S->dim == 3) row[k++] = kz0;
    row[k++] = tr;
    row[k++] = rate;
    if (S->phase != ETRAJ_PHASE_CTMC) row[k++] = dm_carg(amp);
    return 1;
}

/* One WFAT candidate (WFATSampler.jl:173-198 for the grid, :200-240 for
 * Monte-Carlo): ADK's exit point and momentum, the WFAT rate, CTMC rows. */
int o_candidate_wfat(const o_sampler* S, const o_batch* B, double kd0, double kz0, double* row) {
    if (kd0 * kd0 + kz0 * kz0 < 1e-4 * 1e-4) return 0;
    const double F = B->F;
    const double kx0 = kd0 * (-B->sphi);
    const double ky0 = kd0 * B->cphi;
    const double r0 = (S->Ip + (kd0 * kd0 + kz0 * kz0) / 2.0) / F;
    const double x0 = r0 * B->cphi;
    const double y0 = r0 * B->sphi;
    const double rate = g_mol_independent ? o_wfat_rate_ref(S, B, kd0, kz0)
                                          : mol_wfat_rate(S->nxi, S->mmax, B->g2, B->A, S->kappa, F, kd0, kz0, S->dkdt);
    if (dm_isnan(rate) || rate < S->cutoff) return 0;
    int k = 0;
    row[k++] = x0;
    row[k++] = y0;
    if (S->dim == 3) row[k++] = 0.0;
    row[k++] = kx0;
    row[k++] = ky0;
    if (S->dim == 3) row[k++] = kz0;
    row[k++] = B->tr;
    row[k++] = rate;
    return 1;
}

/* (kd0, kz0) of Monte-Carlo candidate i of batch b (shared_methods.jl:4-12,
 * ADKSampler.jl:350-363). */
/* A Monte-Carlo point and its weight dkdt: gen_rand_pt (shared_methods.jl:3-12,
 * weight S->dkdt), or with the Gaussian proposal (etraj_mc_proposal ADK_GAUSS, not
 * in the reference) kd (and kz in 3D) normal of variance F / (2 kappa), by
 * Box-Muller from the same two uniforms, weighted by dkdt_base / pdf. */
void o_mc_point(const o_sampler* S, int64_t b, int64_t i, double F, double* kd0, double* kz0, double* dkdt) {
    uint32_t c[4] = {(uint32_t)i, (uint32_t)((uint64_t)i >> 32), (uint32_t)b, 0x4B445A00u};
    o_philox4x32(c, S->seed);
    double u1 = o_u53(c[0], c[1]), u2 = o_u53(c[2], c[3]);
    *dkdt = S->dkdt;
    if (S->gauss) {
        const double sig = sqrt(F / (2.0 * S->kappa));
        const double r = sqrt(-2.0 * dm_log(1.0 - u1));
        double sn, cs;
        dm_sincos(6.283185307179586 * u2, &sn, &cs);
        const double z1 = r * cs, z2 = r * sn;
        const double norm = sig * 2.5066282746310002; /* sigma sqrt(2 pi) */
        const double inv2s2 = 1.0 / (2.0 * (sig * sig));
        double w = S->dkdt_base;
        *kd0 = 0.0;
        *kz0 = 0.0;
        if (S->dim != 3 || S->mc_kd_max != 0.0) {
            *kd0 = sig * z1;
            w = w * (norm * dm_exp((*kd0 * *kd0) * inv2s2));
        }
        if (S->dim == 3 && S->mc_kz_max != 0.0) {
            *kz0 = sig * z2;
            w = w * (norm * dm_exp((*kz0 * *kz0) * inv2s2));
        }
        *dkdt = w;
        return;
    }
    if (S->dim == 3) {
        *kd0 = ((u1 - 0.5) * 2.0) * S->mc_kd_max;
        *kz0 = ((u2 - 0.5) * 2.0) * S->mc_kz_max;
        if (S->mc_kd_max == 0.0) *kd0 = 0.0;
        else if (S->mc_kz_max == 0.0) *kz0 = 0.0;
    } else {
        *kd0 = ((u1 - 0.5) * 2.0) * S->mc_kd_max;
        *kz0 = 0.0;
    }
}

/* which SPA candidate the sampler runs: the twin of the device's (spa.h, 0) or
 * the independent restatement of oracle_spa_ref.c (1) */
static int g_spa_independent = 0;
void oracle_set_spa_independent(int on) { g_spa_independent = on; }

int64_t o_sample_batch(const o_sampler* S, int64_t b, double* init, int64_t capacity) {
    static __thread o_batch B;  /* about 8 KB with the molecular tables: off the stack */
    o_batch_prepare(S, b, &B);
    int64_t count = 0;
    double row[9];
    const int spa = (S->method == ETRAJ_SAMPLER_SPA);
    if (spa && B.F <= 1e-3) return 0; /* SPASampler.jl:167-169 */
    for (int64_t i = 0; i < S->n_cand; ++i) {
        double kd0, kz0, dkdt = S->dkdt;
        if (!S->mc) {
            kd0 = S->kd[i / S->n_kz];
            kz0 = S->kz[i % S->n_kz];
        } else {
            o_mc_point(S, b, i, B.F, &kd0, &kz0, &dkdt);
        }
        const int kept = spa ? (g_spa_independent ? o_candidate_spa_ref(S, &B, kd0, kz0, row)
                                                  : o_candidate_spa(S, &B, kd0, kz0, row))
                             : S->wfat ? o_candidate_wfat(S, &B, kd0, kz0, row) : o_candidate(S, &B, kd0, kz0, dkdt, row);
        if (kept) {
            if (count < capacity) memcpy(init + count * S->rows, row, sizeof(double) * (size_t)S->rows);
            ++count;
        }
    }
    return count;
}

/* ---- public entry points --------------------------------------------------------- */
static int cmp_double(const void* a, const void* b) {
    double x = *(const double*)a, y = *(const double*)b;
    return (x > y) - (x < y);
}

int oracle_t_samples(const etraj_job* job, double* t) {
    int64_t n = job->sample_t_num;
    double t1 = job->sample_t_intv[0], t2 = job->sample_t_intv[1];
    if (!job->sample_monte_carlo) {
        for (int64_t j = 0; j < n; ++j) t[j] = o_linrange(t1, t2, n, j);
    } else {
        double span = t2 - t1;
        for (int64_t j = 0; j < n; ++j) {
            uint32_t c[4] = {(uint32_t)j, (uint32_t)((uint64_t)j >> 32), 0u, 0x54494D45u};
            o_philox4x32(c, job->seed);
            t[j] = o_u53(c[0], c[1]) * span + t1;
        }
        qsort(t, (size_t)n, sizeof(double), cmp_double);
    }
    return 0;
}

int oracle_batch_info(const etraj_job* job, int64_t* batch_num, int64_t* batch_max_size) {
    if (batch_num) *batch_num = job->sample_t_num;
    if (batch_max_size) {
        if (job->sample_monte_carlo) *batch_max_size = job->mc_kt_num;
        else *batch_max_size = job->ss_kd_num * ((job->dimension == 3) ? job->ss_kz_num : 1);
    }
    return 0;
}

int oracle_sample_batch(const etraj_job* job, int64_t batch_id, double* init, int64_t capacity,
                        int64_t* count) {
    char msg[256];
    int st = oracle_validate(job, msg, sizeof msg);
    if (st) return st;
    if (batch_id < 1 || batch_id > job->sample_t_num) return ETRAJ_ERR_INVALID_ARGUMENT;
    o_sampler S;
    if (o_sampler_init(job, &S)) return ETRAJ_ERR_OUT_OF_MEMORY;
    *count = o_sample_batch(&S, batch_id - 1, init, capacity);
    o_sampler_free(&S);
    return 0;
}

int oracle_sample_all(const etraj_job* job, double* init, int64_t capacity, int64_t* count,
                      int nthreads) {
    char msg[256];
    int st = oracle_validate(job, msg, sizeof msg);
    if (st) return st;
    o_sampler S;
    if (o_sampler_init(job, &S)) return ETRAJ_ERR_OUT_OF_MEMORY;
    int64_t nb = S.n_t, maxb = S.n_cand;
    int64_t* counts = (int64_t*)calloc((size_t)nb, sizeof(int64_t));
    double** bufs = (double**)calloc((size_t)nb, sizeof(double*));
    if (nthreads <= 0) nthreads = 1;
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 1)
    for (int64_t b = 0; b < nb; ++b) {
        double* buf = (double*)malloc(sizeof(double) * (size_t)(maxb * S.rows + 1));
        counts[b] = o_sample_batch(&S, b, buf, maxb);
        bufs[b] = buf;
    }
    int64_t total = 0;
    for (int64_t b = 0; b < nb; ++b) {
        for (int64_t i = 0; i < counts[b]; ++i) {
            if (total < capacity)
                memcpy(init + total * S.rows, bufs[b] + i * S.rows, sizeof(double) * (size_t)S.rows);
            ++total;
        }
        free(bufs[b]);
    }
    free(bufs);
    free(counts);
    *count = total;
    o_sampler_free(&S);
    return 0;
}

/* G_{nxi m}(theta, chi) of a molecular target's WFAT data (mol.h), for the
 * structure-factor pins (GenericMolecule.jl:236-259); out = (re, im). */
void oracle_mol_wfat_G(const etraj_target* T, int nxi, int m, double theta, double chi, double* out) {
    const dm_cplx G = mol_wfat_G(nxi, m, T->wfat_nxi_max, T->wfat_m_max, T->wfat_lmax, T->wfat_intdata, T->wfat_mu,
                                 sqrt(2.0 * T->Ip), theta, chi);
    out[0] = G.re;
    out[1] = G.im;
}
