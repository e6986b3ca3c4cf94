/*
 * oracle.h -- CPU FP64 restatement of eTraj.jl's ensemble-trajectory path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (the CUDA library and
 * its Python host side) may call, link or load this code; it exists so the
 * tests, smoke() and the CPU-baseline leg of bench.py can check the device
 * results.  It takes the same etraj_job description as the C ABI.
 *
 * Parity status: the reference (Julia) cannot run in this environment.  The
 * oracle is pinned against every numeric known-answer test the reference's
 * own suite holds for this path (sampler survivor counts,
 * test/ElectronSamplers_test.jl:53-292; A' = -F, test/Lasers_test.jl;
 * F = -grad V and the He asymptotic coefficient, test/Targets_test.jl).
 * The ODE integrator follows OrdinaryDiffEq's documented Tsit5 defaults
 * (a third-party dependency not vendored in the reference): that part is
 * parity unpinned against the real reference.
 */
#ifndef ETRAJ_ORACLE_H
#define ETRAJ_ORACLE_H

#include <stdint.h>
#include "../include/etraj.h"

#ifdef __cplusplus
extern "C" {
#endif

/* scalars[] layout returned by oracle_collect / oracle_run */
enum {
    ORACLE_ION_PROB = 0,
    ORACLE_ION_PROB_UNCOLLECTED = 1,
    ORACLE_NUM_EFFECTIVE = 2,
    ORACLE_NUM_FAILED = 3,
    ORACLE_NUM_IONIZED = 4,
    ORACLE_NUM_STEPS = 5,
    ORACLE_NUM_SCALARS = 6
};

int oracle_validate(const etraj_job* job, char* msg, int msg_len);
int oracle_batch_info(const etraj_job* job, int64_t* batch_num, int64_t* batch_max_size);
int oracle_t_samples(const etraj_job* job, double* t);
int oracle_sample_batch(const etraj_job* job, int64_t batch_id, double* init,
                        int64_t capacity, int64_t* count);
int oracle_sample_all(const etraj_job* job, double* init, int64_t capacity,
                      int64_t* count, int nthreads);
int oracle_integrate(const etraj_job* job, int64_t n, const double* init, double* final_state,
                     int32_t* status, int32_t* steps, int nthreads);
/* oracle_integrate with each trajectory's least |r| (the initial state and the
 * end of every accepted step) in rmin[i] (may be NULL). */
int oracle_integrate_rmin(const etraj_job* job, int64_t n, const double* init, double* final_state,
                          int32_t* status, int32_t* steps, double* rmin, int nthreads);
int oracle_collect(const etraj_job* job, int64_t n, const double* init, const double* final_state,
                   const int32_t* status, const int32_t* steps, double* spec, double* amp,
                   double* scalars, double* p_inf, int32_t* bin);
int oracle_run(const etraj_job* job, double* spec, double* amp, double* scalars, int nthreads);
int oracle_contributions(const etraj_job* job, int64_t n, const double* init, const double* final_state,
                         const int32_t* status, uint32_t* key, double* c_re, double* c_im);

/* physics probes used by the known-answer tests */
void oracle_laser_eval(const etraj_laser* laser, int64_t n, const double* t, double* Fx,
                       double* Fy, double* Ax, double* Ay, double* dFx, double* dFy,
                       double* env);
void oracle_laser_eval_complex(const etraj_laser* laser, int64_t n, const double* t_re,
                               const double* t_im, double* Ax, double* Ay, double* Fx,
                               double* Fy);
void oracle_target_eval(const etraj_target* target, int64_t n, const double* xyz, double* V,
                        double* F);
/* G_{nxi m}(theta, chi) of a molecular target's WFAT data; out = (re, im). */
void oracle_mol_wfat_G(const etraj_target* T, int nxi, int m, double theta, double chi, double* out);
double oracle_hartree_asymp_coeff(int Z, double Ip, int l);
/* exp(-b r) skip of the SAE terms: the per-target exactness check and a
 * process-wide switch (default on) used to show the skip changes nothing */
int oracle_sae_skip_exact(const etraj_target* target);
void oracle_set_sae_skip(int enable);
/* SPA candidates from the independent restatement (oracle_spa_ref.c: C library
 * functions, its own solver and quadrature) instead of the device's twin */
void oracle_set_spa_independent(int on);
/* molecular prefactor numerators and WFAT rates from the independent
 * restatement (oracle_mol_ref.c) instead of the device's twin (mol.h) */
void oracle_set_mol_independent(int on);
void oracle_mol_wfat_G_ref(const etraj_target* T, int nxi, int m, double theta, double chi, double* out);
void oracle_rhs(const etraj_job* job, double t, const double* u, double* du);
void oracle_detmath(int fn, int64_t n, const double* x, const double* y, double* out);
void oracle_tsit5_tableau(double* c, double* a, double* btilde);

#ifdef __cplusplus
}
#endif

#endif
