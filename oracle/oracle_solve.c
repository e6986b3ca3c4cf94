/*
 * oracle_solve.c -- ODE solve, collection, deposit and entry points of the CPU
 * oracle (TEST INFRASTRUCTURE ONLY; see oracle.h).
 *
 * Integrator: Tsit5 (Tsitouras, Comput. Math. Appl. 62 (2011) 770) with the
 * defaults OrdinaryDiffEq applies to `solve(prob, Tsit5(), reltol=rtol)`
 * (OrdinaryDiffEq 6.66 / OrdinaryDiffEqTsit5 1.1, not vendored in the
 * reference -- parity unpinned): abstol 1e-6; error norm RMS of
 * utilde/(abstol + max(|uprev|,|u|)*reltol); PI step control with
 * beta1 = 7/50, beta2 = 2/25, qmin = 1/5, qmax = 10, gamma = 9/10,
 * qoldinit = 1e-4; initial step from Hairer-Norsett-Wanner's starting-step
 * algorithm with order 5; dtmax = t_final - t0; dtmin = eps(max(|t0|,|tf|));
 * maxiters = 1e6; t snapped to t_final within 100 eps; FSAL.
 * Call sites: src/TrajectorySimulation.jl:334-342 (2D), :429-437 (3D).
 *
 * Collection: src/TrajectorySimulation.jl:344-400 (2D), :439-499 (3D).
 * Deterministic reductions (the reference sums per Julia thread in a
 * schedule-dependent order; this is the fixed order the device reproduces):
 *   spectrum bin     -- 0.0 + contributions in trajectory order;
 *   ion_prob, ...    -- 256-ary tree over trajectory order; each node is a
 *                       binary tree over its 256 slots (absent slots +0.0),
 *                       so no chain of dependent additions exceeds 8.
 */
#include <stdio.h>

#include "oracle_internal.h"
#include "oracle_sampler.h"

#ifdef _OPENMP
#include <omp.h>
#endif

/* ---- Tsit5 tableau --------------------------------------------------------------- */
static const double TS_C[7] = {0.0, 0.161, 0.327, 0.9, 0.9800255409045097, 1.0, 1.0};
static const double TS_A[7][6] = {
    {0, 0, 0, 0, 0, 0},
    {0.161, 0, 0, 0, 0, 0},
    {-0.008480655492356989, 0.335480655492357, 0, 0, 0, 0},
    {2.897153057105493, -6.359448489975075, 4.3622954328695815, 0, 0, 0},
    {5.325864828439257, -11.748883564062828, 7.4955393428898365, -0.09249506636175525, 0, 0},
    {5.86145544294642, -12.92096931784711, 8.159367898576159, -0.071584973281401, -0.028269050394068383, 0},
    {0.09646076681806523, 0.01, 0.4798896504144996, 1.379008574103742, -3.290069515436081, 2.324710524099774}};
static const double TS_BT[7] = {-0.00178001105222577714, -0.0008164344596567469, 0.007880878010261995,
                                -0.1447110071732629, 0.5823571654525552, -0.45808210592918697,
                                0.015151515151515152};

#define TS_ABSTOL 1e-6
#define TS_BETA1 0.14
#define TS_BETA2 0.08
#define TS_QMIN_INV 5.0
#define TS_QMAX_INV 0.1
#define TS_GAMMA 0.9
#define TS_QOLDINIT 1e-4
#define TS_MAXITERS 1000000L

enum { ST_SUCCESS = 0, ST_MAXITERS = 1, ST_DTMIN = 2, ST_UNSTABLE = 3, ST_DTNAN = 4 };

void oracle_tsit5_tableau(double* c, double* a, double* btilde) {
    for (int i = 0; i < 7; ++i) {
        c[i] = TS_C[i];
        btilde[i] = TS_BT[i];
        for (int j = 0; j < 6; ++j) a[i * 6 + j] = TS_A[i][j];
    }
}

void o_sys_prepare(const etraj_job* job, o_sys* S) {
    memset(S, 0, sizeof *S);
    S->dim = job->dimension;
    S->phase = job->traj_phase_method;
    S->n = (S->dim == 3 ? 6 : 4) + (S->phase != ETRAJ_PHASE_CTMC ? 1 : 0);
    S->rtol = job->traj_rtol;
    o_laser_prepare(&job->laser, &S->laser);
    o_target_prepare(&job->target, &S->target);
}

/* RMS norm of v[j]/sk[j] */
static double o_rms_ratio(const double* v, const double* sk, int n) {
    double acc = 0.0;
    for (int j = 0; j < n; ++j) {
        double q = v[j] / sk[j];
        acc = fma(q, q, acc);
    }
    return sqrt(acc / (double)n);
}

/* Starting step size (Hairer, Norsett & Wanner, Solving ODEs I, II.4). */
static double o_initdt(const o_sys* S, double t, const double* u0, const double* f0, double dtmax,
                       double dtmin) {
    int n = S->n;
    double sk[7], u1[7], f1[7], df[7];
    for (int j = 0; j < n; ++j) sk[j] = fma(fabs(u0[j]), S->rtol, TS_ABSTOL);
    double d0 = o_rms_ratio(u0, sk, n);
    double d1 = o_rms_ratio(f0, sk, n);
    double dt0 = (d0 < 1e-5 || d1 < 1e-5) ? 1e-6 : (d0 / d1) / 100.0;
    dt0 = o_jmin(dt0, dtmax);
    if (dt0 < 10.0 * 2.220446049250313e-16) return 1e-6;
    for (int j = 0; j < n; ++j) u1[j] = fma(dt0, f0[j], u0[j]);
    o_rhs(S, t + dt0, u1, f1);
    for (int j = 0; j < n; ++j) df[j] = f1[j] - f0[j];
    double d2 = o_rms_ratio(df, sk, n) / dt0;
    double md = o_jmax(d1, d2);
    double dt1;
    if (md <= 1e-15) dt1 = o_jmax(1e-6, dt0 * 1e-3);
    else dt1 = dm_pow_pos(10.0, -(2.0 + dm_log(md) / DM_LN10) / 5.0);
    return o_jmax(dtmin, o_jmin(o_jmin(100.0 * dt0, dt1), dtmax));
}

/* r^2 of a state, summed left to right */
static double o_radius2(const o_sys* S, const double* u) {
    double r2 = u[0] * u[0] + u[1] * u[1];
    if (S->dim == 3) r2 = r2 + u[2] * u[2];
    return r2;
}

/* Integrates one trajectory from (t0, u0) to tf.  Returns the status code.
 * rmin (optional): the least |r| of the initial state and of the end of every
 * accepted step. */
static int o_solve(const o_sys* S, double t0, double tf, const double* u0, double* u_out,
                   int32_t* nsteps, double* rmin) {
    const int n = S->n;
    double uprev[7], u[7], k[7][7], tmp[7], s;
    double t = t0;
    for (int j = 0; j < n; ++j) uprev[j] = u[j] = u0[j];
    double dtmax = tf - t0;
    double dtmin = o_jmax(o_ulp(t0), o_ulp(tf));
    o_rhs(S, t, uprev, k[0]);
    double dt = o_initdt(S, t, uprev, k[0], dtmax, dtmin);
    double dtpropose = dt, qold = TS_QOLDINIT, q11 = 1.0;
    double r2min = rmin ? o_radius2(S, uprev) : 0.0;
    int accept = 0, status = ST_SUCCESS;
    long iter = 0;
    int32_t attempts = 0;
    while (t < tf) {
        /* loopheader!: apply the previous step's decision */
        if (iter > 0) {
            if (!accept) {
                dt = dt / o_jmin(TS_QMIN_INV, q11 / TS_GAMMA);
            } else {
                for (int j = 0; j < n; ++j) { uprev[j] = u[j]; k[0][j] = k[6][j]; }
                dt = dtpropose;
            }
        }
        ++iter;
        /* fix_dt_at_bounds! and modify_dt_for_tstops! */
        dt = o_jmin(dtmax, dt);
        dt = o_jmax(dt, o_jmax(dtmin, o_ulp(t)));
        dt = o_jmin(dt, tf - t);
        /* check_error! */
        if (dm_isnan(dt)) { status = ST_DTNAN; break; }
        if (iter > TS_MAXITERS) { status = ST_MAXITERS; break; }
        if (dt <= dtmin && (!accept || t + dt < tf)) { status = ST_DTMIN; break; }
        if (accept) {
            int bad = 0;
            for (int j = 0; j < n; ++j) bad |= dm_isnan(u[j]);
            if (bad) { status = ST_UNSTABLE; break; }
        }
        /* perform_step! (Tsit5, FSAL) */
        for (int i = 1; i < 7; ++i) {
            for (int j = 0; j < n; ++j) {
                s = TS_A[i][0] * k[0][j];
                for (int q = 1; q < i; ++q) s = fma(TS_A[i][q], k[q][j], s);
                tmp[j] = fma(dt, s, uprev[j]);
            }
            double ti = (i >= 5) ? t + dt : fma(TS_C[i], dt, t);
            if (i == 6) for (int j = 0; j < n; ++j) u[j] = tmp[j];
            o_rhs(S, ti, tmp, k[i]);
        }
        double acc = 0.0;
        for (int j = 0; j < n; ++j) {
            s = TS_BT[0] * k[0][j];
            for (int q = 1; q < 7; ++q) s = fma(TS_BT[q], k[q][j], s);
            double ut = dt * s;
            double sc = fma(o_jmax(fabs(uprev[j]), fabs(u[j])), S->rtol, TS_ABSTOL);
            double r = ut / sc;
            acc = fma(r, r, acc);
        }
        double EEst = sqrt(acc / (double)n);
        ++attempts;
        /* loopfooter!: PI controller */
        double ttmp = t + dt, q;
        if (EEst == 0.0) {
            q = TS_QMAX_INV;
        } else {
            q11 = dm_pow_pos(EEst, TS_BETA1);
            q = q11 / dm_pow_pos(qold, TS_BETA2);
            q = o_jmax(TS_QMAX_INV, o_jmin(TS_QMIN_INV, q / TS_GAMMA));
        }
        accept = (EEst <= 1.0);
        if (accept) {
            if (q >= 1.0 && q <= 1.0) q = 1.0;
            qold = o_jmax(EEst, TS_QOLDINIT);
            double dtnew = dt / q;
            t = (fabs(ttmp - tf) < 100.0 * o_ulp(o_jmax(t, tf))) ? tf : ttmp;
            dtpropose = o_jmax(o_jmin(dtmax, dtnew), dtmin);
            if (rmin) r2min = o_jmin(r2min, o_radius2(S, u));
        }
    }
    for (int j = 0; j < n; ++j) u_out[j] = (status == ST_SUCCESS) ? u[j] : uprev[j];
    if (nsteps) *nsteps = attempts;
    if (rmin) *rmin = sqrt(r2min);
    return status;
}

/* ---- validation (TrajectorySimulation.jl:178-186, ADKSampler.jl:43-105,
 *      HydrogenLikeAtom.jl:53-56, SAEAtom.jl:60-64, Cos4Laser.jl:57-58) ----------- */
/* the sampler of the job being validated: its name replaces "[ADKSampler]" in the
 * shared checks, as the reference's SPANE / SPA / WFAT samplers word them */
static __thread int o_method = ETRAJ_SAMPLER_ADK;

static int o_fail(char* msg, int len, const char* text) {
    if (msg && len > 0) {
        const char* tag = (o_method == ETRAJ_SAMPLER_SPANE) ? "[SPANESampler]"
                          : (o_method == ETRAJ_SAMPLER_SPA) ? "[SPASampler]"
                          : (o_method == ETRAJ_SAMPLER_WFAT) ? "[WFATSampler]" : "[ADKSampler]";
        if (strncmp(text, "[ADKSampler]", 12) == 0)
            snprintf(msg, (size_t)len, "%s%s", tag, text + 12);
        else
            snprintf(msg, (size_t)len, "%s", text);
    }
    return ETRAJ_ERR_INVALID_ARGUMENT;
}

int oracle_validate(const etraj_job* job, char* msg, int len) {
    o_method = job ? job->init_cond_method : ETRAJ_SAMPLER_ADK;
    if (msg && len > 0) msg[0] = 0;
    if (!(job->sample_t_intv[0] < job->sample_t_intv[1]))
        return o_fail(msg, len, "[TrajectorySimulationJob] `sample_t_intv` must be a valid interval.");
    if (!(job->traj_t_final > job->sample_t_intv[1]))
        return o_fail(msg, len, "[TrajectorySimulationJob] `traj_t_final` must be greater than the last time point of `sample_t_intv`.");
    if (job->mc_kt_proposal != ETRAJ_PROPOSAL_UNIFORM && job->mc_kt_proposal != ETRAJ_PROPOSAL_ADK_GAUSS)
        return o_fail(msg, len, "unknown mc_kt_proposal.");
    if (job->mc_kt_proposal == ETRAJ_PROPOSAL_ADK_GAUSS &&
        (!job->sample_monte_carlo ||
         (job->init_cond_method != ETRAJ_SAMPLER_ADK && job->init_cond_method != ETRAJ_SAMPLER_SPANE)))
        return o_fail(msg, len, "mc_kt_proposal ADK_GAUSS applies to Monte-Carlo ADK and SPANE sampling only.");
    if (job->dimension != 2 && job->dimension != 3)
        return o_fail(msg, len, "[TrajectorySimulationJob] `dimension` must be either 2 or 3.");
    if (job->init_cond_method != ETRAJ_SAMPLER_ADK && job->init_cond_method != ETRAJ_SAMPLER_SPANE &&
        job->init_cond_method != ETRAJ_SAMPLER_SPA && job->init_cond_method != ETRAJ_SAMPLER_WFAT)
        return o_fail(msg, len, "[ElectronSamplers] Undefined initial condition method.");
    if (job->traj_phase_method < 0 || job->traj_phase_method > 2)
        return o_fail(msg, len, "[ADKSampler] Undefined phase method.");
    if (job->rate_prefix & ~7) return o_fail(msg, len, "[ADKSampler] Undefined tunneling rate prefix.");
    if ((job->rate_prefix & ETRAJ_PREFIX_PRE) && (job->rate_prefix & ETRAJ_PREFIX_PRECC))
        return o_fail(msg, len, "[ADKSampler] Rate prefixes [Pre] & [PreCC] conflict.");
    if (!(job->sample_t_num > 0)) return o_fail(msg, len, "[ADKSampler] Invalid time sample number.");
    if (!(job->sample_cutoff_limit >= 0)) return o_fail(msg, len, "[ADKSampler] Invalid cut-off limit.");
    if (!job->sample_monte_carlo) {
        if (job->dimension == 3) {
            if (!(job->ss_kd_num > 0 && job->ss_kz_num > 0))
                return o_fail(msg, len, "[ADKSampler] Invalid kd,kz sample number.");
            if (!(job->ss_kd_max > 0 || job->ss_kz_max > 0))
                return o_fail(msg, len, "[ADKSampler] Invalid kd,kz sample boundaries (cannot be zero simultaneously).");
            if (job->ss_kz_num == 1 && job->ss_kz_max != 0)
                return o_fail(msg, len, "range(-abs(ss_kz_max), abs(ss_kz_max); length=1): endpoints differ.");
        } else {
            if (!(job->ss_kd_num > 0)) return o_fail(msg, len, "[ADKSampler] Invalid kd sample number.");
            if (!(job->ss_kd_max > 0)) return o_fail(msg, len, "[ADKSampler] Invalid kd sample boundaries.");
        }
        // Julia's range(a, b; length=1) needs a == b (ADKSampler.jl:85,97)
        if (job->ss_kd_num == 1 && job->ss_kd_max != 0)
            return o_fail(msg, len, "range(-abs(ss_kd_max), abs(ss_kd_max); length=1): endpoints differ.");
    } else {
        if (!(job->mc_kt_num > 0)) return o_fail(msg, len, "[ADKSampler] Invalid sampling kt_num.");
        if (job->dimension == 3) {
            if (!(job->mc_kd_max > 0 || job->mc_kz_max > 0))
                return o_fail(msg, len, "[ADKSampler] Invalid kd,kz sample boundaries (cannot be zero simultaneously).");
        } else if (!(job->mc_kd_max > 0)) {
            return o_fail(msg, len, "[ADKSampler] Invalid kd sample boundaries.");
        }
    }
    for (int d = 0; d < job->dimension; ++d) {
        if (job->final_p_num[d] < 1) return o_fail(msg, len, "[TrajectorySimulationJob] `final_p_num` must be positive.");
        if (job->final_p_num[d] > 1 && !(job->final_p_max[d] > 0))
            return o_fail(msg, len, "[TrajectorySimulationJob] `final_p_max` must be positive.");
    }
    const etraj_target* T = &job->target;
    const char* mmsg = 0;
    int mst = etraj_mol_check(job, &mmsg);
    if (mst > 0) {
        o_fail(msg, len, mmsg);
        return mst;
    }
    if (mst == 0) {
        /* molecular target: checked above */
    } else if (!(T->Ip > 0)) return o_fail(msg, len, "[SAEAtom] Ip should be positive.");
    else if (!(T->l >= 0 && T->l >= abs(T->m))) return o_fail(msg, len, "[SAEAtom] Invalid (l,m).");
    else if (T->l > 4) return ETRAJ_ERR_UNSUPPORTED;
    else if (!(T->asymp_coeff > 0)) return o_fail(msg, len, "[SAEAtom] asymp_coeff should be either `:hartree` or a positive number.");
    if (T->kind == ETRAJ_TARGET_MOLECULE) {
        /* trajectories: Coulomb tail with soft core 1.0 (GenericMolecule.jl:444-445) */
    } else if (T->kind == ETRAJ_TARGET_SAE) {
        if (!(T->b1 >= 0 && T->b2 >= 0 && T->b3 >= 0)) return o_fail(msg, len, "[SAEAtom] b1,b2,b3 should be non-negative.");
        if (!(T->soft_core > 0)) return o_fail(msg, len, "[SAEAtom] soft_core should be positive.");
    } else if (T->kind == ETRAJ_TARGET_HYDROGEN_LIKE) {
        if (!(T->soft_core >= 0)) return o_fail(msg, len, "[HydrogenLikeAtom] `soft_core` should be non-negative.");
    } else {
        return o_fail(msg, len, "Unknown target kind.");
    }
    int nm = (job->laser.kind == ETRAJ_LASER_BICHROMATIC) ? 2 : 1;
    if (job->laser.kind < 0 || job->laser.kind > 3) return o_fail(msg, len, "Unknown laser kind.");
    for (int i = 0; i < nm; ++i) {
        const etraj_mono_laser* L = &job->laser.mono[i];
        if (L->kind < 0 || L->kind > 2) return o_fail(msg, len, "Unknown monochromatic laser kind.");
        if (!(L->wave_len > 0)) return o_fail(msg, len, "[Cos4Laser] Must specify either `wave_len` or `ang_freq`.");
        if (!(L->cyc_num > 0)) return o_fail(msg, len, "[Cos4Laser] Must specify either `cyc_num` or `duration`.");
    }
    if (!(job->traj_rtol > 0)) return o_fail(msg, len, "`traj_rtol` must be positive.");
    return ETRAJ_OK;
}

/* ---- integrate ------------------------------------------------------------------------ */
int oracle_integrate(const etraj_job* job, int64_t n, const double* init, double* final_state,
                     int32_t* status, int32_t* steps, int nthreads) {
    return oracle_integrate_rmin(job, n, init, final_state, status, steps, NULL, nthreads);
}

int oracle_integrate_rmin(const etraj_job* job, int64_t n, const double* init, double* final_state,
                          int32_t* status, int32_t* steps, double* rmin, int nthreads) {
    o_sys S;
    o_sys_prepare(job, &S);
    int rows = (S.dim == 3) ? ((S.phase == ETRAJ_PHASE_CTMC) ? 8 : 9) : ((S.phase == ETRAJ_PHASE_CTMC) ? 6 : 7);
    int tcol = (S.dim == 3) ? 6 : 4;
    if (nthreads <= 0) nthreads = 1;
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 64)
    for (int64_t i = 0; i < n; ++i) {
        const double* r = init + i * rows;
        double u0[7], uf[7];
        int nq = S.dim == 3 ? 6 : 4;
        for (int j = 0; j < nq; ++j) u0[j] = r[j];
        if (S.phase != ETRAJ_PHASE_CTMC) u0[nq] = r[rows - 1];
        int32_t ns = 0;
        int st = o_solve(&S, r[tcol], job->traj_t_final, u0, uf, &ns, rmin ? rmin + i : NULL);
        if (final_state)
            for (int j = 0; j < S.n; ++j) final_state[i * S.n + j] = uf[j];
        if (status) status[i] = st;
        if (steps) steps[i] = ns;
    }
    return 0;
}

/* ---- collect --------------------------------------------------------------------------- */
typedef struct {
    int ionized, in_grid;
    int64_t bin;
    double prob, are, aim;
    double pinf[3];
} o_coll;

static void o_cross(const double a[3], const double b[3], double c[3]) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

static void o_collect_one(const etraj_job* job, const o_sys* S, const double* r, const double* f,
                          o_coll* C) {
    memset(C, 0, sizeof *C);
    C->bin = -1;
    int dim = S->dim, rows = (dim == 3) ? ((S->phase == ETRAJ_PHASE_CTMC) ? 8 : 9) : ((S->phase == ETRAJ_PHASE_CTMC) ? 6 : 7);
    double x, y, z, px, py, pz, phase, K;
    if (dim == 2) {
        x = f[0]; y = f[1]; z = 0.0; px = f[2]; py = f[3]; pz = 0.0;
        K = (px * px + py * py) / 2.0;
    } else {
        x = f[0]; y = f[1]; z = f[2]; px = f[3]; py = f[4]; pz = f[5];
        K = ((px * px + py * py) + pz * pz) / 2.0;
    }
    phase = (S->phase == ETRAJ_PHASE_CTMC) ? 0.0 : f[S->n - 1];
    double prob = r[rows - ((S->phase == ETRAJ_PHASE_CTMC) ? 1 : 2)];
    double tr = r[rows - ((S->phase == ETRAJ_PHASE_CTMC) ? 2 : 3)];
    double E = K + o_target_V(&S->target, x, y, z);
    double rv[3] = {x, y, z}, pv[3] = {px, py, pz}, L[3];
    o_cross(rv, pv, L);
    double L2 = (L[0] * L[0] + L[1] * L[1]) + L[2] * L[2];
    double Z = S->target.Z;
    if (E > 0.0 && S->phase == ETRAJ_PHASE_SCTS) {
        phase = phase + S->target.Ip * tr;
        double sqrtb = 1.0 / sqrt(2.0 * E);
        double g = sqrt(1.0 + (2.0 * E) * L2);
        /* the 3D reference uses x*py where x*px is meant (TrajectorySimulation.jl:463) */
        double rp = (dim == 2) ? (x * px + y * py) : ((x * py + y * py) + z * pz);
        phase = phase - (Z * sqrtb) * (dm_log(g) + dm_asinh(rp / (g * sqrtb)));
    }
    if (!(E >= 0.0)) return;
    C->ionized = 1;
    C->prob = prob;
    double pinf = sqrt(2.0 * E);
    double nr = sqrt((x * x + y * y) + z * z);
    double pL[3], a[3], La[3];
    o_cross(pv, L, pL);
    for (int i = 0; i < 3; ++i) a[i] = pL[i] - (Z * rv[i]) / nr;
    o_cross(L, a, La);
    double fac = pinf / (1.0 + (pinf * pinf) * L2);
    for (int i = 0; i < 3; ++i) C->pinf[i] = fac * (pinf * La[i] - a[i]);
    int64_t idx[3] = {1, 1, 1}, stride = 1, lin = 0;
    int ok = 1;
    for (int d = 0; d < dim; ++d) {
        int64_t num = job->final_p_num[d];
        if (num > 1) {
            double pm = job->final_p_max[d];
            double v = rint((C->pinf[d] + pm) / ((pm / (double)num) * 2.0));
            if (!(v >= 1.0 && v <= (double)num)) ok = 0;
            else idx[d] = (int64_t)v;
        }
        lin += (idx[d] - 1) * stride;
        stride *= num;
    }
    if (!ok) return;
    C->in_grid = 1;
    C->bin = lin;
    if (S->phase == ETRAJ_PHASE_CTMC) {
        C->are = prob;
        C->aim = 0.0;
    } else {
        double sp = sqrt(prob), s, c;
        dm_sincos(phase, &s, &c);
        C->are = sp * c;
        C->aim = sp * s;
    }
}

/* Per-electron deposit inputs: bin key (grid when not deposited) and the
 * contribution w or sqrt(w) e^{i phi}, as the deposit consumes them. */
int oracle_contributions(const etraj_job* job, int64_t n, const double* init, const double* final_state,
                         const int32_t* status, uint32_t* key, double* c_re, double* c_im) {
    o_sys S;
    o_sys_prepare(job, &S);
    int rows = (S.dim == 3) ? ((S.phase == ETRAJ_PHASE_CTMC) ? 8 : 9) : ((S.phase == ETRAJ_PHASE_CTMC) ? 6 : 7);
    int64_t G = 1;
    for (int d = 0; d < job->dimension; ++d) G *= job->final_p_num[d];
    for (int64_t i = 0; i < n; ++i) {
        o_coll C;
        key[i] = (uint32_t)G;
        c_re[i] = 0.0;
        c_im[i] = 0.0;
        if (status && status[i] != 0) continue;
        o_collect_one(job, &S, init + i * rows, final_state + i * S.n, &C);
        if (C.ionized && C.in_grid) {
            key[i] = (uint32_t)C.bin;
            c_re[i] = C.are;
            c_im[i] = C.aim;
        }
    }
    return 0;
}

/* one node of the canonical tree: v[0..len) (len <= 256) in 256 slots, absent
 * slots +0.0, summed as a binary tree over consecutive pairs */
static double o_node_sum(const double* v, int64_t len) {
    double t[256];
    for (int i = 0; i < 256; ++i) t[i] = (i < len) ? v[i] : 0.0;
    for (int w = 128; w >= 1; w >>= 1)
        for (int i = 0; i < w; ++i) t[i] = t[2 * i] + t[2 * i + 1];
    return t[0];
}

/* 256-ary tree over v[0..n) whose nodes are o_node_sum */
static double o_canon_sum(const double* v, int64_t n) {
    if (n == 0) return 0.0;
    double* cur = (double*)malloc(sizeof(double) * (size_t)n);
    memcpy(cur, v, sizeof(double) * (size_t)n);
    int64_t m = n;
    do {
        int64_t nb = (m + 255) / 256;
        for (int64_t b = 0; b < nb; ++b) {
            int64_t e = (b + 1) * 256 < m ? (b + 1) * 256 : m;
            cur[b] = o_node_sum(cur + b * 256, e - b * 256);
        }
        m = nb;
    } while (m > 1);
    double r = cur[0];
    free(cur);
    return r;
}

static int64_t o_grid_size(const etraj_job* job) {
    int64_t g = 1;
    for (int d = 0; d < job->dimension; ++d) g *= job->final_p_num[d];
    return g;
}

int oracle_collect(const etraj_job* job, int64_t n, const double* init, const double* final_state,
                   const int32_t* status, const int32_t* steps, double* spec, double* amp,
                   double* scalars, double* p_inf, int32_t* bin) {
    o_sys S;
    o_sys_prepare(job, &S);
    int rows = (S.dim == 3) ? ((S.phase == ETRAJ_PHASE_CTMC) ? 8 : 9) : ((S.phase == ETRAJ_PHASE_CTMC) ? 6 : 7);
    int64_t G = o_grid_size(job);
    double* are = (double*)calloc((size_t)G, sizeof(double));
    double* aim = (double*)calloc((size_t)G, sizeof(double));
    double* w_ion = (double*)calloc((size_t)(n > 0 ? n : 1), sizeof(double));
    double* w_unc = (double*)calloc((size_t)(n > 0 ? n : 1), sizeof(double));
    int64_t failed = 0, ionized = 0, nsteps = 0;
    for (int64_t i = 0; i < n; ++i) {
        o_coll C;
        if (steps) nsteps += steps[i];
        if (status && status[i] != 0) {
            ++failed;
            if (p_inf) p_inf[3 * i] = p_inf[3 * i + 1] = p_inf[3 * i + 2] = 0.0;
            if (bin) bin[i] = -2;
            continue;
        }
        o_collect_one(job, &S, init + i * rows, final_state + i * S.n, &C);
        if (p_inf) { p_inf[3 * i] = C.pinf[0]; p_inf[3 * i + 1] = C.pinf[1]; p_inf[3 * i + 2] = C.pinf[2]; }
        if (bin) bin[i] = C.ionized ? (C.in_grid ? (int32_t)C.bin : -1) : -3;
        if (!C.ionized) continue;
        ++ionized;
        w_ion[i] = C.prob;
        if (C.in_grid) {
            are[C.bin] = are[C.bin] + C.are;
            aim[C.bin] = aim[C.bin] + C.aim;
        } else {
            w_unc[i] = C.prob;
        }
    }
    for (int64_t g = 0; g < G; ++g) {
        if (S.phase == ETRAJ_PHASE_CTMC) {
            if (spec) spec[g] = are[g];
        } else {
            if (amp) { amp[2 * g] = are[g]; amp[2 * g + 1] = aim[g]; }
            if (spec) spec[g] = are[g] * are[g] + aim[g] * aim[g];
        }
    }
    if (scalars) {
        scalars[ORACLE_ION_PROB] = o_canon_sum(w_ion, n);
        scalars[ORACLE_ION_PROB_UNCOLLECTED] = o_canon_sum(w_unc, n);
        scalars[ORACLE_NUM_EFFECTIVE] = (double)n;
        scalars[ORACLE_NUM_FAILED] = (double)failed;
        scalars[ORACLE_NUM_IONIZED] = (double)ionized;
        scalars[ORACLE_NUM_STEPS] = (double)nsteps;
    }
    free(are); free(aim); free(w_ion); free(w_unc);
    return 0;
}

int oracle_run(const etraj_job* job, double* spec, double* amp, double* scalars, int nthreads) {
    char msg[256];
    int st = oracle_validate(job, msg, sizeof msg);
    if (st) return st;
    int64_t nb, maxb;
    oracle_batch_info(job, &nb, &maxb);
    int rows = (job->dimension == 3) ? ((job->traj_phase_method == ETRAJ_PHASE_CTMC) ? 8 : 9)
                                     : ((job->traj_phase_method == ETRAJ_PHASE_CTMC) ? 6 : 7);
    int64_t cap = nb * maxb, count = 0;
    double* init = (double*)malloc(sizeof(double) * (size_t)(cap * rows + 1));
    if (!init) return ETRAJ_ERR_OUT_OF_MEMORY;
    st = oracle_sample_all(job, init, cap, &count, nthreads);
    if (st) { free(init); return st; }
    int ns = (job->dimension == 3 ? 6 : 4) + (job->traj_phase_method != ETRAJ_PHASE_CTMC);
    double* fin = (double*)malloc(sizeof(double) * (size_t)(count * ns + 1));
    int32_t* status = (int32_t*)malloc(sizeof(int32_t) * (size_t)(count + 1));
    int32_t* steps = (int32_t*)malloc(sizeof(int32_t) * (size_t)(count + 1));
    oracle_integrate(job, count, init, fin, status, steps, nthreads);
    oracle_collect(job, count, init, fin, status, steps, spec, amp, scalars, NULL, NULL);
    free(init); free(fin); free(status); free(steps);
    return 0;
}

/* ---- probes for the known-answer tests ------------------------------------------------- */
void oracle_laser_eval(const etraj_laser* laser, int64_t n, const double* t, double* Fx, double* Fy,
                       double* Ax, double* Ay, double* dFx, double* dFy, double* env) {
    o_laser L;
    o_laser_prepare(laser, &L);
    for (int64_t i = 0; i < n; ++i) {
        double fx, fy, dfx, dfy, ax, ay;
        o_laser_F(&L, t[i], &fx, &fy);
        o_laser_F_dual(&L, t[i], &fx, &fy, &dfx, &dfy);
        o_laser_A(&L, t[i], &ax, &ay);
        if (Fx) Fx[i] = fx;
        if (Fy) Fy[i] = fy;
        if (dFx) dFx[i] = dfx;
        if (dFy) dFy[i] = dfy;
        if (Ax) Ax[i] = ax;
        if (Ay) Ay[i] = ay;
        if (env) env[i] = (L.nmono == 1) ? o_mono_env(&L.m[0], t[i]) : 0.0;
    }
}

void oracle_laser_eval_complex(const etraj_laser* laser, int64_t n, const double* t_re,
                               const double* t_im, double* Ax, double* Ay, double* Fx, double* Fy) {
    o_laser L;
    o_laser_prepare(laser, &L);
    for (int64_t i = 0; i < n; ++i) {
        dm_cplx ax, ay, fx, fy;
        o_laser_AF_complex(&L, dm_c(t_re[i], t_im[i]), &ax, &ay, &fx, &fy);
        Ax[2 * i] = ax.re; Ax[2 * i + 1] = ax.im;
        Ay[2 * i] = ay.re; Ay[2 * i + 1] = ay.im;
        Fx[2 * i] = fx.re; Fx[2 * i + 1] = fx.im;
        Fy[2 * i] = fy.re; Fy[2 * i + 1] = fy.im;
    }
}

void oracle_target_eval(const etraj_target* target, int64_t n, const double* xyz, double* V,
                        double* F) {
    o_target T;
    o_target_prepare(target, &T);
    for (int64_t i = 0; i < n; ++i) {
        const double* p = xyz + 3 * i;
        if (V) V[i] = o_target_V(&T, p[0], p[1], p[2]);
        if (F) o_target_F(&T, p[0], p[1], p[2], F + 3 * i);
    }
}

void oracle_rhs(const etraj_job* job, double t, const double* u, double* du) {
    o_sys S;
    o_sys_prepare(job, &S);
    o_rhs(&S, t, u, du);
}

/* detmath probes: 0 exp 1 expm1 2 log 3 log1p 4 sin 5 cos 6 tanh 7 atan
 * 8 atan2(x,y) 9 asinh 10 pow(x,y) */
void oracle_detmath(int fn, int64_t n, const double* x, const double* y, double* out) {
    for (int64_t i = 0; i < n; ++i) {
        double v = x[i], r = 0.0;
        switch (fn) {
        case 0: r = dm_exp(v); break;
        case 1: r = dm_expm1(v); break;
        case 2: r = dm_log(v); break;
        case 3: r = dm_log1p(v); break;
        case 4: r = dm_sin(v); break;
        case 5: r = dm_cos(v); break;
        case 6: r = dm_tanh(v); break;
        case 7: r = dm_atan(v); break;
        case 8: r = dm_atan2(v, y[i]); break;
        case 9: r = dm_asinh(v); break;
        case 10: r = dm_pow_pos(v, y[i]); break;
        default: r = dm_nan();
        }
        out[i] = r;
    }
}
