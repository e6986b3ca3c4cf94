// engine.h -- device-side job description and the kernel launchers shared by
// the translation units of libetraj_gb300.
//
// Every field is derived on the host from an etraj_job (setup.cpp) with the
// same expressions the reference uses (src/Lasers/*.jl getters,
// src/ElectronSamplers/ADKSampler.jl:226-276), then passed to kernels by
// value as a __grid_constant__ parameter.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/etraj.h"
#include "detmath.h"
#include "mol.h"
#include "sae_skip.h"

namespace etraj {

struct DMono {
    int kind;
    int azi_zero;
    double omega, period, F0, A0, N, cep, t_shift, ellip;
    double cphi, sphi;        // cos/sin of the azimuth
    double w2n, cN, k, Npiw;  // cos^n envelope: omega/(2N), 2/N or 1/N, 200/T, N*pi/omega
    double sigma, inv_s2, inv_2s2;  // Gaussian envelope
};

struct DLaser {
    int nmono;
    int kind;
    DMono m[2];
    double delay;
};

struct DTarget {
    int kind;
    int skip_ok;  // exp(-b r) with b r > 60 may be dropped exactly (sae_exp in physics.cuh)
    double Z, Ip, sc, a1, b1, a2, b2, a3, b3;
};

// Per-time-sample constants of the ADK/SPANE samplers (the prologue of
// gen_electron_batch, ADKSampler.jl:168-296).
// FP32 copies read by the bulk path's sampler (CD = C * D).
struct FBatch {
    float Fx, Fy, dFx, dFy, F, sphi, cphi, c_cc, W;
    int spa_on;  // SPA: F(t_r) > 1e-3 (decided in FP64)
    float ny0, ny1, nz0, nz1;
    float CD[2 * 9];
};

// The laser of one time sample in the form the FP32 SPA sampler evaluates it
// at complex times t_r + i tau (sampler_fp32.cu, spa32_base and spa32_AF).
struct SpaMono32 {
    float cth, sth, cu, su;   // cos, sin of the carrier and envelope phases at t_r
    float om, w2n, cN;        // carrier and envelope angular frequencies, envelope factor
    float preA, preF;         // A0 (F0) times the tanh windows (Cos) or the Gaussian at t_r
    float gt, gi, inv_s2;     // Gaussian: t_r - t_shift, 1/(2 sigma^2), 1/sigma^2
    float ellip, cphi, sphi;
    int kind, azi0;
};
struct SpaBase32 {
    int n;
    SpaMono32 m[2];
};

struct DBatch {
    double tr, Fx, Fy, dFx, dFy, F, sphi, cphi, c_cc, W;
    double ny0, ny1, nz0, nz1;
    double D[2 * 9];  // D^l_{m' m}, m' = -l..l, interleaved (re, im)
    FBatch f;
    SpaBase32 spa[3];  // FP32 SPA sampler: the laser at t_r, t_r + 0.01, t_r - 0.01
};

constexpr int kMaxL = 4;

// Molecular targets (mol.h): the ionizing orbital's tables on the device.
struct DMol {
    int on;              // molecular target
    int wfat;            // WFAT sampler (else the MO-ADK prefix of ADK/SPANE/SPA)
    mol_terms T;         // MO-ADK: (l, m) pairs with C_lm != 0
    int nxi, mmax, wl;   // WFAT: channels n_xi <= nxi, |m| <= mmax; integrals l <= wl
    int stride;          // doubles per time sample in tab
    double rot[3];       // MolRotation
    double mu[3];        // WFAT orbital dipole
    double P[2 * MOL_NLM];   // Y_{l m'} prefactors (complex)
    float Pf[2 * MOL_NLM];   // the same in FP32 (the bulk path's sampler)
    const double* clm;   // C_lm (device copy)
    const double* wint;  // WFAT integrals (device copy)
    double* tab;         // per time sample: C D (MO-ADK) or |G|^2 and the W factors (WFAT)
    float* tabf;         // the same table in FP32 (read by the bulk path's sampler)
};

// Job constants in FP32 for the bulk path's candidate kernels, rounded once on
// the host (each is the float nearest the FP64 value, or of the FP64 expression
// named), so the kernels do no FP64 work to set up.
struct FJobConst {
    float Ip, kap2, dkdt, sqdkdt, inv_dkdt, log_dkdt;  // kappa^2, sqrt(dkdt), 1/dkdt, log(dkdt)
    float cutoff, e_pre, c, e_half, spa_omega;   // e_half = (n* + 1)/2
    float kd_max, kz_max;                        // Monte-Carlo half-widths
    int kd_zero, kz_zero;                        // mc_kd_max == 0, mc_kz_max == 0
};

struct DJob {
    // sampling
    int method, dim, mc, prefix, phase, rows, mono, l, m;
    int n_state;
    int64_t n_t, n_kd, n_kz, n_cand, n_total;  // n_total = n_t * n_cand
    double Ip, Z, kappa, nstar, c, cc_base, e_pre, C, q_theta, q_phi;
    double cutoff, dkdt, mc_kd_max, mc_kz_max;
    int gauss;         // Monte-Carlo ADK / SPANE: transverse momenta normal of the ADK width
    double dkdt_base;  // gauss: step_t / mc_kt_num (times the kz span in 2D); dkdt = that / pdf
    double spa_omega;  // SPA initial guess' angular frequency (SPASampler.jl:160-166)
    uint64_t seed;
    double Plm[2 * (2 * kMaxL + 1)];
    float fPlm[2 * (2 * kMaxL + 1)];  // FP32 copy for the bulk path's sampler
    FJobConst fc;
    // integration
    double rtol, t_final;
    // collection
    double pmax[3], binw[3];
    int64_t pnum[3];
    int64_t grid;
    DLaser laser;
    DTarget target;
    DMol mol;
};

// Sampled electrons, candidate-indexed structure of arrays.
struct InitSoA {
    double *x, *y, *kx, *ky, *kz, *rate, *phase;
    int32_t* batch;   // time-sample index (t0 = t_samples[batch])
};

// Per-survivor outputs of the integrate+collect kernel.
struct TrajOut {
    uint32_t* key;       // bin (0..grid-1) or grid for "not deposited"
    double* c_re;        // contribution: w (CTMC) or sqrt(w)cos(phi)
    double* c_im;        // sqrt(w) sin(phi) (QTMC/SCTS)
    double* w_ion;       // w if ionized, else 0
    double* w_unc;       // w if ionized and outside the grid, else 0
    int32_t* status;     // 0 Success, 1 MaxIters, 2 DtLessThanMin, 3 Unstable, 4 DtNaN
    int32_t* steps;      // step attempts
    double* final_state; // optional: n_state doubles per survivor (row-major)
    double* p_inf;       // optional: 3 doubles per survivor
    double* fphase;      // optional: final phase per survivor (0 for CTMC)
    double* rmin;        // optional, FP64 path: least |r| over the accepted steps
};

struct Counters {
    unsigned long long n_eff;
    unsigned long long n_failed;
    unsigned long long n_ionized;
    unsigned long long n_steps;
    unsigned long long sort_err;  // nonzero: a look-back wait of the deposit's sort gave up
};

// ---- launchers (all stream-ordered; each returns the number of kernel launches) ----
int launch_batch_prepare(const DJob& J, const double* t, DBatch* batches, cudaStream_t s);
// Samples the candidates of time samples [b0, b0+nb) (flag and SoA indexed by
// b * n_cand + i).
// The FP64 SPA sampler's list (the candidates its FP32 pre-pass may keep), in the
// survivors' compaction buffers, which are free until that compaction runs, and
// the pre-pass's margin: it drops candidates whose FP32 rate is below
// exp(log_margin) x the cutoff.
struct SampleScratch {
    int64_t* list;
    uint32_t* block_sums;
    int64_t block_cap;
    unsigned long long* count;
    float log_margin;
};
int launch_sample_range(const DJob& J, int64_t b0, int64_t nb, const double* kd, const double* kz,
                        DBatch* batches, InitSoA soa, uint8_t* flag, int sm_count,
                        cudaStream_t s, const SampleScratch* scr);
// The FP64 SPA sampler's FP32 pre-pass (atoms): fills batches[b].spa and sets
// flag = 0 for the candidates whose FP32 rate is more than 100 times below the cutoff.
int launch_spa_prefilter(const DJob& J, int64_t b0, int64_t nb, const double* kd, const double* kz,
                         DBatch* batches, float log_margin, uint8_t* flag, int sm_count, cudaStream_t s);
// FP32 variant of the same kernel for the bulk path (sampler_fp32.cu); used
// when the rate cutoff keeps every kept rate in FP32's normal range.
// Its SPA variant first fills batches[b].spa of the batches it samples.
int launch_sample32_range(const DJob& J, int64_t b0, int64_t nb, const double* kd, const double* kz,
                          DBatch* batches, InitSoA soa, uint8_t* flag, int sm_count,
                          cudaStream_t s);
constexpr double kSample32MinCutoff = 1e-30;
// Order-preserving compaction: idx[k] = k-th i with flag[i] != 0; *count = total.
int launch_compact(const uint8_t* flag, int64_t n, int64_t* idx, uint32_t* block_sums,
                   int64_t nblocks_cap, unsigned long long* count, cudaStream_t s);
int64_t compact_blocks(int64_t n);
int launch_integrate_fp64(const DJob& J, InitSoA soa, const double* t, const int64_t* idx,
                          const unsigned long long* count, TrajOut out, int64_t max_n,
                          int sm_count, cudaStream_t s);
// FP64 collection of final states written by the bulk integrator (same code as
// the epilogue of the plain kernel).
int launch_collect_fp64(const DJob& J, InitSoA soa, const double* t, const int64_t* idx,
                        const unsigned long long* count, TrajOut out, int64_t max_n, int sm_count,
                        cudaStream_t s);

// One instance of a multi-instance bulk launch: its field table and clock, and
// where its candidates and time samples sit in the concatenated arrays.
struct BulkInst {
    const float4* table;
    int64_t cand_end;  // the instance owns candidates [cand_end of the one before, cand_end)
    double T0, inv_h_d, t_final;
    int t_off;         // its first time sample in the concatenated array
    int n_int, nf;
    float ff, h, inv_h;
};
constexpr int kMaxInstances = 64;

// Parameters of the FP32 bulk integrator (integrate_fp32.cu).
struct BulkParams {
    int dim, phase, tgt;
    int n_int;          // field-table intervals
    int table_in_smem;  // 1: stage the table in shared memory
    int threads, blocks_per_sm, refill_min;
    int chunk0;         // round 0's step budget per electron; round r's is chunk0 16^r (last: none)
    int static_assign;  // 1: one electron per lane, no queue, no rounds (the plain kernel's schedule)
    int occ;            // register budget of the build: 2 (<= 128 per thread) or 3 (<= 85)
    int64_t max_n;      // upper bound of the electron count (grid sizing)
    const BulkInst* inst;  // multi-instance launch: n_inst instances (else nullptr, 0)
    int n_inst;
    const float4* table;
    double T0, inv_h_d, t_final;
    float h, inv_h, rtol;
    int nf;             // t_final = T0 + h (nf + ff)
    float ff;
    float Z, Ip, sc, a1, b1, a2, b2, a3, b3, a2b2;
    float r_far;        // SAE: radius beyond which the exp(-b r) terms are dropped
    int max_iters;      // steps before an electron is given up (status 1)
    // Rounds: the integrator runs as kBulkRounds launches.  In round r, once
    // the round's queue is empty, an electron that has taken the round's step
    // chunk (chunk0 16^r steps; the last round has none; 1024, 16384, 262144 by
    // default) in the round writes its whole state to the park buffer and frees
    // its lane; round r+1 resumes the parked electrons packed densely (blocks
    // without parked work exit at once).  park_buf == nullptr: one launch.
    uint32_t* park_buf;   // 2 halves x park_cap entries x kParkWords words (word-major)
    int park_cap;         // entries per half
    // set per round by the launcher
    int park_budget;      // steps per electron in this round (0: no limit)
    const uint32_t* park_in;                    // rounds >= 1: resume from here
    const unsigned long long* park_in_count;
    uint32_t* park_out;                         // all rounds but the last: park into here
    unsigned long long* park_out_count;
};
constexpr int kParkWords = 33;   // words of one parked electron (3D with phase)
constexpr int kBulkRounds = 4;
constexpr int kBulkCounters = 2 * kBulkRounds;  // work counter and park count per round
constexpr int kBulkMaxIters = 1000000;  // OrdinaryDiffEq's default maxiters
int launch_field_table(const DJob& J, double T0, double h, int n_int, float4* tab, cudaStream_t s);
// *out = min(*count, cap) (the autotuner's sample of the electrons)
int launch_clamp_count(const unsigned long long* count, unsigned long long cap, unsigned long long* out,
                       cudaStream_t s);
// FP32 collection of the bulk integrator's final states.  With inst (n_inst
// instances of one grid J.grid) the keys are instance * J.grid + bin and the
// "not deposited" key is n_inst * J.grid.
int launch_collect_bulk(const DJob& J, InitSoA soa, const double* t, const int64_t* idx,
                        const unsigned long long* count, TrajOut out, int64_t max_n, int sm_count,
                        cudaStream_t s, const BulkInst* inst = nullptr, int n_inst = 0);
// Per-instance results of a multi-instance launch (deposit.cu): survivor
// segments, canonical ion_prob sums, counters, and the weighted sum of spectra.
int launch_instance_reductions(const TrajOut& out, const int64_t* idx, const unsigned long long* count,
                               const BulkInst* inst, int n_inst, int64_t* seg, double* scratch,
                               double* sums /* 2 per instance */, Counters* counters, cudaStream_t s);
size_t instance_scratch_doubles(int64_t max_n, int n_inst);
int launch_weighted_sum(const double* mspec, int n_inst, int64_t grid, const double* w, double* out,
                        cudaStream_t s);
int launch_integrate_bulk(const BulkParams& P, InitSoA soa, const double* t, const int64_t* idx,
                          const unsigned long long* count, unsigned long long* queue, TrajOut out,
                          int sm_count, cudaStream_t s);

// Parameters of the double-float integrator (integrate_df.cu).  float2 values are
// double-float pairs (x = high float, y = low float), rounded on the host.
struct DFParams {
    int dim, phase, tgt;
    int n_int;            // field-table intervals (kDfTableF4 float4 each: degree-7 pieces of Fx, Fy)
    const float4* table;
    double T0, h_d, inv_h_d, t_final;
    float2 h, inv_h;      // table spacing and its inverse
    int nf;               // t_final = T0 + h (nf + ff)
    float2 ff;
    float2 rtol;
    float t_snap;         // 100 ulp of t_final: a step ending closer than this ends the solve
    float2 Z, Ip, sc, a1, b1, a2, b2, a3, b3, a2b2;
    float r2_far;         // SAE: r^2 beyond which every exp(-b_i r) of the potential is 0
    int max_iters;
    int threads, blocks;    // launch shape of the start-up pass (persistent grid)
    int threads_main, blocks_main;  // and of the main pass
    int64_t max_n;
    float* carry;           // kDfCarryWords x max_n words: electrons passed to the main pass
};
constexpr int kDfCarryWords = 32;        // words of one carried electron (at most 29 used)
constexpr int kDfTablePerPeriod = 1024;  // table intervals per shortest laser period
constexpr int kDfTableF4 = 7;            // float4 per table interval
// Chebyshev nodes of a field-table piece and the values of T_0..T_7 there
struct DfTableNodes {
    double u[8];
    double Tm[8][8];
};
int launch_field_table_df(const DJob& J, double T0, double h, int n_int, const DfTableNodes& nodes, float4* tab,
                          cudaStream_t s);
// Work-stealing double-float Tsit5 solve of the survivors in two passes (an
// electron's first steps, whose error estimates need stage differences, then the
// rest); writes out.final_state (FP64), out.status and out.steps, for
// launch_collect_fp64.  work: three counters (start-up queue, carried electrons,
// main-pass queue).
int launch_integrate_df(const DFParams& P, InitSoA soa, const double* t, const int64_t* idx,
                        const unsigned long long* count, unsigned long long* work, TrajOut out,
                        cudaStream_t s);
// Resident blocks per SM of a double-float integrator pass (main: the main pass).
int df_blocks_per_sm(int dim, int phase, int tgt, bool main, int threads);
// threads per block of the double-float integrator's passes (their launch bounds)
int df_threads(bool main);

// Deterministic deposit: stable radix sort of (key, survivor) and segmented sums.
struct DepositScratch {
    uint32_t *keys_a, *keys_b, *vals_a, *vals_b;
    unsigned long long* post;  // the sort's look-back posts: 512 per tile of 4096 keys
    uint32_t* aux;             // digit counts, digit offsets, tile counters
    double* tree_a;            // canonical-sum partials
    double* tree_b;
};
size_t deposit_scratch_bytes(int64_t max_n);
void deposit_scratch_carve(void* base, int64_t max_n, DepositScratch* d);
int launch_deposit(const DJob& J, const TrajOut& out, const unsigned long long* count,
                   int64_t max_n, DepositScratch d, double* spec_re, double* spec_im,
                   double* momentum_spec, double* sums /* [2]: ion, unc */,
                   Counters* counters, cudaStream_t s);

}  // namespace etraj
