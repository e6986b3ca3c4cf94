/* oracle_sampler.h -- sampler state of the CPU oracle (TEST INFRASTRUCTURE ONLY). */
#ifndef ETRAJ_ORACLE_SAMPLER_H
#define ETRAJ_ORACLE_SAMPLER_H

#include "oracle_internal.h"
#include "../etraj.jl_gb300/csrc/mol.h"

typedef struct {
    int method, dim, mc, prefix, phase, rows, mono;
    double cutoff;
    uint64_t seed;
    o_laser laser;
    double Ip, Z, kappa, n, c, cc_base, e_pre, C, q_theta, q_phi;
    int l, m;
    dm_cplx Plm[9];
    int64_t n_t, n_kd, n_kz, n_cand;
    double *t, *kd, *kz;
    double mc_kd_max, mc_kz_max, dkdt;
    int gauss;          /* Monte-Carlo: the Gaussian proposal (etraj_mc_proposal ADK_GAUSS) */
    double dkdt_base;   /* gauss: step_t / mc_kt_num (times the kz span in 2D) */
    double spa_omega; /* the SPA initial guess' angular frequency (SPASampler.jl:160-166) */
    /* molecular targets (mol.h layouts) */
    int mol, wfat;
    mol_terms T;                  /* MO-ADK: (l, m) pairs with C_lm != 0 */
    double mol_rot[3];
    const double* clm;            /* C_lm (caller's array) */
    double Pmol[2 * MOL_NLM];     /* Y_{l m'} prefactors */
    int nxi, mmax, wl;            /* WFAT channel and integral sizes */
    const double* wint;           /* WFAT integrals (caller's array) */
    double mu[3];
} o_sampler;

typedef struct {
    double tr, Fx, Fy, dFx, dFy, F, phi, sphi, cphi, gamma, c_cc, W;
    double ny[3], nz[3];
    dm_cplx D[9];
    double cd[2 * MOL_NCD];       /* MO-ADK: C_lm D^l_{m' m} */
    double g2[MOL_NCH], A[MOL_NA]; /* WFAT: |G|^2 per channel, time-sample factors of W */
} o_batch;

void o_philox4x32(uint32_t c[4], uint64_t seed);
double o_u53(uint32_t a, uint32_t b);
double o_linrange(double a, double b, int64_t n, int64_t i);
int o_sampler_init(const etraj_job* job, o_sampler* S);
void o_sampler_free(o_sampler* S);
void o_batch_prepare(const o_sampler* S, int64_t b, o_batch* B);
int o_candidate(const o_sampler* S, const o_batch* B, double kd0, double kz0, double dkdt, double* row);
int o_candidate_spa(const o_sampler* S, const o_batch* B, double kd0, double kz0, double* row);
int o_candidate_spa_ref(const o_sampler* S, const o_batch* B, double kd0, double kz0, double* row);
dm_cplx o_pre_numerator(const o_sampler* S, const o_batch* B, dm_cplx kx, dm_cplx ky, dm_cplx kz);
dm_cplx o_mol_numerator_ref(const o_sampler* S, const o_batch* B, dm_cplx nkx, dm_cplx nky, dm_cplx nkz);
double o_wfat_rate_ref(const o_sampler* S, const o_batch* B, double kd, double kz);
int o_candidate_wfat(const o_sampler* S, const o_batch* B, double kd0, double kz0, double* row);
void o_mc_point(const o_sampler* S, int64_t b, int64_t i, double F, double* kd0, double* kz0, double* dkdt);
int64_t o_sample_batch(const o_sampler* S, int64_t b, double* init, int64_t capacity);

#endif
