/*
 * etraj.h -- C ABI of the GB300 ensemble-trajectory engine.
 *
 * This library replaces the batch loop of eTraj.jl's trajectory simulation
 * (src/TrajectorySimulation.jl:154-157, `@threads for i in 1:batch_num
 * launch_and_collect!(job, i)`) with one call that runs every stage on one
 * GPU: initial-condition sampling (gen_electron_batch in
 * src/ElectronSamplers/ADKSampler.jl, SPANESampler.jl, SPASampler.jl), the adaptive Tsit5 ensemble solve
 * (src/TrajectorySimulation.jl:334-342 / 429-437), the asymptotic Kepler
 * step and SCTS phase correction (:356-374 / :451-469) and the spectrum
 * collection (:375-393 / :470-493, reduced as in write_output! :521-543).
 *
 * Conventions
 *  - All physical quantities are in atomic units, except the laser's peak
 *    intensity (W/cm^2) and wavelength (nm), as in the reference's laser
 *    constructors (src/Lasers/Cos4Laser.jl:44-74).
 *  - Plain C types only; every array is caller-owned host memory unless an
 *    entry point says otherwise.  No exceptions cross the ABI: every entry
 *    point returns an etraj_status and etraj_last_error() explains it.
 *  - Spectra are laid out in Julia column-major order (px fastest), so a
 *    Julia caller can pass pointer(Array) under GC.@preserve.
 *  - Sample matrices use the reference's `init` layout (ADKSampler.jl:299-303):
 *    one column per electron, rows x,y[,z],kx,ky[,kz],t0,rate[,phase],
 *    stored column-major (the rows of one electron are contiguous).
 */
#ifndef ETRAJ_H
#define ETRAJ_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ETRAJ_ABI_VERSION 1

typedef enum etraj_status {
    ETRAJ_OK = 0,
    ETRAJ_ERR_INVALID_ARGUMENT = 1, /* a check the reference makes with @assert / error() */
    ETRAJ_ERR_UNSUPPORTED = 2,      /* valid in the reference, not built here */
    ETRAJ_ERR_CUDA = 3,             /* a CUDA runtime call failed */
    ETRAJ_ERR_OUT_OF_MEMORY = 4,    /* the job does not fit the context's HBM budget */
    ETRAJ_ERR_TIMEOUT = 5,          /* a device work budget ran out */
    ETRAJ_ERR_NOT_READY = 6,        /* etraj_poll: the job is still running */
    ETRAJ_ERR_NOT_FOUND = 7         /* unknown ticket */
} etraj_status;

/* ---- lasers: src/Lasers/{Cos4,Cos2,Gaussian,Bichromatic}Laser.jl ---------- */
typedef enum etraj_laser_kind {
    ETRAJ_LASER_COS4 = 0,        /* Cos4Laser.jl:7 */
    ETRAJ_LASER_COS2 = 1,        /* Cos2Laser.jl:7 */
    ETRAJ_LASER_GAUSSIAN = 2,    /* GaussianLaser.jl:7 */
    ETRAJ_LASER_BICHROMATIC = 3  /* BichromaticLaser.jl:7 */
} etraj_laser_kind;

typedef struct etraj_mono_laser {
    int32_t kind;      /* ETRAJ_LASER_COS4, _COS2 or _GAUSSIAN */
    int32_t reserved;
    double peak_int;   /* W/cm^2 */
    double wave_len;   /* nm */
    double cyc_num;    /* Cos4/Cos2: number of cycles N; Gaussian: spread_cyc_num (sigma in cycles) */
    double ellip;      /* -1 <= ellip <= 1 */
    double azi;        /* azimuth of the principal axis, rad */
    double cep;        /* carrier-envelope phase, rad */
    double t_shift;    /* a.u. */
} etraj_mono_laser;

typedef struct etraj_laser {
    int32_t kind;               /* monochromatic: mono[0]; BICHROMATIC: mono[0] + mono[1] */
    int32_t reserved;
    etraj_mono_laser mono[2];
    double delay;               /* BICHROMATIC: delay of mono[1] (BichromaticLaser.jl:73-85) */
} etraj_laser;

/* ---- targets: src/Targets/{HydrogenLikeAtom,SAEAtom,GenericMolecule}.jl ---------- */
typedef enum etraj_target_kind {
    ETRAJ_TARGET_HYDROGEN_LIKE = 0, /* HydrogenLikeAtom.jl:7 */
    ETRAJ_TARGET_SAE = 1,           /* SAEAtom.jl:7 */
    ETRAJ_TARGET_MOLECULE = 2       /* GenericMolecule.jl:7 */
} etraj_target_kind;

/* Largest l of a molecule's asymptotic coefficients and WFAT integrals, and
 * the largest WFAT channel indices n_xi and |m| (the database files hold 6). */
#define ETRAJ_MOL_MAX_L 6

typedef struct etraj_target {
    int32_t kind;
    int32_t Z;              /* asymptotic nuclear charge (nucl_charge; molecule: charge + 1) */
    int32_t l, m;           /* atoms only */
    double Ip;              /* a.u.; molecule: IonPotential(mol, orbit_ridx), the ionizing orbital's */
    double asymp_coeff;     /* atoms: C_kl, already resolved (the :hartree default is SAEAtomBase_shared.jl:3-11) */
    double quan_ax_theta;   /* rad */
    double quan_ax_phi;     /* rad */
    double a1, b1, a2, b2, a3, b3; /* SAE potential parameters; ignored for other targets */
    double soft_core;       /* atoms; a molecule's trajectories use 1.0 (GenericMolecule.jl:444-445) */
    /* ETRAJ_TARGET_MOLECULE: the ionizing orbital's data as GenericMolecule
     * holds it (GenericMolecule.jl:7-41), read from the molecule's data file by
     * the caller.  The arrays are caller-owned and read only during the call
     * that takes the job (etraj_run, etraj_submit, ...). */
    double mol_rot[3];          /* MolRotation: Euler angles alpha, beta, gamma (z-y'-z''), rad */
    double mol_Ip_traj;         /* IonPotential(mol), the Ip of the trajectories' phase (:438-443) */
    int32_t asymp_lmax;         /* MolAsympCoeff: C_lm for l = 0..asymp_lmax (<= ETRAJ_MOL_MAX_L) */
    int32_t wfat_nxi_max;       /* MolWFATMaxChannels: n_xi = 0..wfat_nxi_max */
    int32_t wfat_m_max;         /* m = -wfat_m_max..wfat_m_max */
    int32_t wfat_lmax;          /* the integrals' l = 0..wfat_lmax */
    const double* asymp_coeff_lm;  /* (asymp_lmax+1) x (2 asymp_lmax+1) complex (re, im pairs),
                                      column-major: C[l+1, m+l+1] as in MolAsympCoeff; NULL: none */
    const double* wfat_intdata;    /* (nxi+1) x (2 m_max+1) x (lmax+1) x (2 lmax+1) complex, column-major,
                                      as MolWFATData's IntData; NULL: none */
    double wfat_mu[3];             /* MolWFATData's orbital dipole mu */
} etraj_target;

/* ---- job: the keyword arguments of perform_traj_simulation ---------------- */
typedef enum etraj_sampler_kind {
    ETRAJ_SAMPLER_ADK = 0,   /* :ADK   ADKSampler.jl */
    ETRAJ_SAMPLER_SPANE = 1, /* :SPANE SPANESampler.jl */
    ETRAJ_SAMPLER_SPA = 2,   /* :SPA   SPASampler.jl */
    ETRAJ_SAMPLER_WFAT = 3   /* :WFAT  WFATSampler.jl (molecular targets, CTMC) */
} etraj_sampler_kind;

/* rate_prefix bit mask (ADKSampler.jl:49-77): :Exp = 0, :Full = PRECC|JAC */
#define ETRAJ_PREFIX_PRE 1
#define ETRAJ_PREFIX_PRECC 2
#define ETRAJ_PREFIX_JAC 4

typedef enum etraj_phase_method {
    ETRAJ_PHASE_CTMC = 0,
    ETRAJ_PHASE_QTMC = 1,
    ETRAJ_PHASE_SCTS = 2
} etraj_phase_method;

typedef enum etraj_precision {
    ETRAJ_PRECISION_FP64 = 0,      /* one thread per trajectory, FP64, bit-compatible with the oracle */
    ETRAJ_PRECISION_FP32_BULK = 1, /* persistent work-stealing integrator, FP32 stages, compensated state */
    ETRAJ_PRECISION_FP32_DF = 2    /* persistent work-stealing integrator on the FP32 pipe, every stage value
                                      a double-float pair (~48-bit significand) formed as a difference from the
                                      accepted state: the FP64 path's step sequence, final states within ~1e-10
                                      of it; FP64 sampling, collection and deposit */
} etraj_precision;

typedef struct etraj_job {
    int32_t init_cond_method;    /* etraj_sampler_kind */
    int32_t dimension;           /* 2 or 3 */
    int32_t sample_monte_carlo;  /* 0: step sampling (ss_*), 1: Monte-Carlo (mc_*) */
    int32_t rate_prefix;         /* ETRAJ_PREFIX_* mask */
    int32_t traj_phase_method;   /* etraj_phase_method */
    int32_t precision;           /* etraj_precision */
    double sample_t_intv[2];     /* a.u. */
    int64_t sample_t_num;
    double traj_t_final;         /* a.u. */
    double traj_rtol;            /* reference default 1e-6 */
    double final_p_max[3];
    int64_t final_p_num[3];      /* 2D jobs ignore index 2 */
    double ss_kd_max;
    int64_t ss_kd_num;
    double ss_kz_max;
    int64_t ss_kz_num;
    int64_t mc_kt_num;
    double mc_kd_max;
    double mc_kz_max;
    double sample_cutoff_limit;  /* reference default 1e-16 */
    uint64_t seed;               /* Monte-Carlo stream; the reference draws from an unseeded global RNG */
    etraj_laser laser;
    etraj_target target;
    int32_t mc_kt_proposal;      /* Monte-Carlo ADK / SPANE: ETRAJ_PROPOSAL_* (0, the reference's, by default) */
    int32_t reserved2;
} etraj_job;

/* How Monte-Carlo ADK and SPANE candidates draw their transverse momenta.
 * UNIFORM is the reference's gen_rand_pt (shared_methods.jl:3-12): kd (and kz)
 * uniform in [-mc_kd_max, mc_kd_max] (and +-mc_kz_max), each candidate weighted
 * by dkdt = step_t * spans / mc_kt_num.  ADK_GAUSS is not in the reference: kd
 * (and, in 3D, kz) normal with the ADK width sigma^2 = F(t_r) / (2 kappa) of the
 * candidate's time sample (Box-Muller from the same two draws), a draw outside
 * +-mc_kd_max (+-mc_kz_max) dropped, and each candidate weighted by
 * step_t / (mc_kt_num pdf(kd) [pdf(kz)]) -- an importance-sampling estimate of
 * the same integral, with the candidates where the rate is. */
typedef enum { ETRAJ_PROPOSAL_UNIFORM = 0, ETRAJ_PROPOSAL_ADK_GAUSS = 1 } etraj_mc_proposal;

typedef struct etraj_result {
    /* caller-owned outputs; either pointer may be NULL to skip that copy */
    double* momentum_spec;   /* prod(final_p_num) doubles, column-major; |amplitude|^2 for QTMC/SCTS */
    double* amplitude;       /* QTMC/SCTS: 2*prod(final_p_num) doubles (re,im) before |.|^2 */
    /* scalars written by the library (write_output!, TrajectorySimulation.jl:541-543) */
    double ion_prob;
    double ion_prob_uncollected;
    int64_t num_effective_traj;  /* electrons that survived the cutoff, failed ODE solves included */
    int64_t num_failed_traj;     /* ODE retcode != Success: skipped, as at :347-355 */
    int64_t num_ionized_traj;    /* E_inf >= 0 */
    int64_t num_steps;           /* Tsit5 step attempts over all trajectories */
    int64_t num_kernel_launches; /* kernels this library launched for the job */
    double elapsed_ms;           /* device time from the first to the last launch */
} etraj_result;

typedef struct etraj_ctx etraj_ctx;

/* ---- library and context ---------------------------------------------------- */
const char* etraj_version(void);

/* Creates a context on `device`.  hbm_budget_bytes == 0 means "all free memory
 * minus 1 GiB".  A context owns its device buffers and one CUDA stream. */
int etraj_create(etraj_ctx** ctx, int device, size_t hbm_budget_bytes);
void etraj_destroy(etraj_ctx* ctx);
const char* etraj_last_error(const etraj_ctx* ctx);

/* Runs subsequent work on a caller-provided cudaStream_t (NULL restores the
 * context's own stream). */
int etraj_set_stream(etraj_ctx* ctx, void* cuda_stream);

/* Host-only validation with the reference's messages, e.g.
 * TrajectorySimulation.jl:178-186, ADKSampler.jl:44-47,79-105. */
int etraj_validate(const etraj_job* job, char* msg, size_t msg_len);

/* Replaces the `@threads for i in 1:batch_num` loop: samples, integrates,
 * collects and reduces the whole job on the device, then copies the spectrum
 * into out->momentum_spec / out->amplitude (skipped when NULL). */
int etraj_run(etraj_ctx* ctx, const etraj_job* job, etraj_result* out);

/* ---- component entry points (parity tests and the Julia shim's debug path) --- */

/* Number of batches (= time samples, ADKSampler.jl:153-155) and the largest
 * batch (:158-164). */
int etraj_batch_info(const etraj_job* job, int64_t* batch_num, int64_t* batch_max_size);

/* gen_electron_batch(sp, batch_id) for one 1-based batch id: writes the
 * surviving electrons' columns into `init` (capacity columns of `rows`
 * doubles) and their count into *count (0 where the reference returns
 * `nothing`).  rows = 6/7 (2D) or 8/9 (3D), CTMC/phase. */
int etraj_sample_batch(etraj_ctx* ctx, const etraj_job* job, int64_t batch_id,
                       double* init, int64_t capacity, int64_t* count);

/* The sampling stage of the whole job, batches concatenated in order.  Both
 * entry points sample as the job's precision does: FP64 for
 * ETRAJ_PRECISION_FP64, the bulk path's FP32 candidate kernels for
 * ETRAJ_PRECISION_FP32_BULK (atomic targets). */
int etraj_sample_all(etraj_ctx* ctx, const etraj_job* job,
                     double* init, int64_t capacity, int64_t* count);

/* The ensemble ODE solve for n electrons given in reference `init` layout.
 * final_state: n columns of the ODE state (x,y[,z],px,py[,pz][,phase]);
 * status: 0 Success, 1 MaxIters, 2 DtLessThanMin, 3 Unstable; steps: step
 * attempts.  Any output pointer may be NULL. */
int etraj_integrate(etraj_ctx* ctx, const etraj_job* job, int64_t n, const double* init,
                    double* final_state, int32_t* status, int32_t* steps);

/* ---- asynchronous jobs on one context -----------------------------------------
 * No counterpart in the reference.  etraj_submit enqueues a job on the
 * context's stream and returns; jobs run in submission order, and the host
 * set-up of one overlaps the device work of the one before.  `out` supplies the
 * caller-owned output pointers (momentum_spec, amplitude), which must stay
 * valid until etraj_poll or etraj_wait has returned for the ticket.
 * etraj_poll returns ETRAJ_ERR_NOT_READY while the job runs; poll and wait
 * fill the scalars of `out` (its pointers are left as they are), copy the
 * spectra out of the library's pinned staging and release the ticket.  A job
 * that fails its checks reports the error at poll/wait. */
int etraj_submit(etraj_ctx* ctx, const etraj_job* job, etraj_result* out, uint64_t* ticket);
int etraj_poll(etraj_ctx* ctx, uint64_t ticket, etraj_result* out);
int etraj_wait(etraj_ctx* ctx, uint64_t ticket, etraj_result* out);

/* ---- multi-instance batch ------------------------------------------------------
 * No counterpart in the reference, which runs one simulation per call.  Runs
 * n_jobs (1..64) FP32-bulk jobs as one batch: per-instance sampling, then one
 * compaction, ONE bulk-integrator launch whose work stealing spans the
 * electrons of every instance, one collection and one deposit into an
 * instance-major grid.  The jobs may differ in laser and sampler; they must
 * share precision (FP32_BULK), dimension, phase method, rtol, target and
 * momentum grid (else ETRAJ_ERR_INVALID_ARGUMENT).  results[i] receives job
 * i's scalars and, through its own pointers, its spectrum and amplitude;
 * each equals the result of running job i alone.  With weights (n_jobs
 * values), weighted_spec (one grid) receives sum_i weights[i] *
 * momentum_spec_i, summed in instance order (e.g. an intensity-weighted
 * focal-volume average); pass NULL for both to skip it.  Blocking. */
int etraj_run_batch(etraj_ctx* ctx, const etraj_job* jobs, int n_jobs, etraj_result* results,
                    const double* weights, double* weighted_spec);

/* ---- serving: continuous batching on one GPU ---------------------------------
 * No counterpart in the reference, which runs one job per call.  A server owns
 * `slots` (1..64) contexts, each with its own stream and device buffers, and
 * one HBM budget over all of them (0 = free memory less 1 GiB).  A submitted
 * job is checked (errors return at once), queued first-in first-out, and
 * enqueued as soon as a slot is free and the device bytes it would add fit in
 * the budget (idle slots give their buffers back when memory is short; a job
 * that cannot fit even on an empty server fails with ETRAJ_ERR_OUT_OF_MEMORY).
 * Jobs on different slots overlap on the device; nothing is shared between
 * slots, so a job's result is the same alone and in any mix.  Every call
 * retires finished jobs and admits queued ones.  etraj_server_poll returns
 * ETRAJ_ERR_NOT_READY while the job is queued or running; etraj_server_wait
 * blocks up to timeout_s seconds (negative: no limit), then returns
 * ETRAJ_ERR_TIMEOUT.  Output pointers follow the rules of etraj_submit. */
typedef struct etraj_server etraj_server;
int etraj_server_create(etraj_server** out, int device, int slots, size_t hbm_budget_bytes);
void etraj_server_destroy(etraj_server* srv);
int etraj_server_submit(etraj_server* srv, const etraj_job* job, etraj_result* out, uint64_t* ticket);
int etraj_server_poll(etraj_server* srv, uint64_t ticket, etraj_result* out);
int etraj_server_wait(etraj_server* srv, uint64_t ticket, etraj_result* out, double timeout_s);
int etraj_server_stats(etraj_server* srv, int64_t* running, int64_t* queued, size_t* hbm_in_use);
const char* etraj_server_last_error(const etraj_server* srv);

/* ---- CUDA graphs ------------------------------------------------------------------
 * No counterpart in the reference.  On by default: the kernel sequence of a job
 * (prologue to deposit), or of a multi-instance batch (etraj_run_batch: every
 * instance's sampling, one integrator launch, the deposit, the per-instance
 * reductions and the weighted sum), runs directly the first time; when the
 * same launch parameters come again (same jobs, same buffers, same launch
 * shape) it is captured into a CUDA graph and replayed from then on.  Jobs
 * that do not repeat never pay for a capture.  etraj_set_graphs(ctx, 0) turns
 * it off and frees the graphs. */
int etraj_set_graphs(etraj_ctx* ctx, int enable);

/* ---- autotuner --------------------------------------------------------------------
 * No counterpart in the reference.  The FP32-bulk integrator's launch shape
 * (threads per block, blocks per SM, free lanes a warp waits for before it
 * refills, and with it the register budget of the build: <= 128 registers per
 * thread up to 16 warps per SM, <= 85 up to 24) is tuned once per device,
 * process and kernel variant on the first 2^18 electrons of the first job with
 * enough work (each capped at 4096 steps), by timing 12 candidates; every
 * context of the process then uses that choice.  Results never depend on the
 * shape.  etraj_set_autotune(ctx, 0) switches tuning off for the context and
 * returns it to the fixed shape 256 x 2 x 4.  etraj_bulk_tile reports the
 * shape in use for a variant (ETRAJ_ERR_NOT_FOUND: not tuned yet, fixed shape
 * reported).  etraj_set_bulk_tile pins a variant's shape on one context
 * (threads 64, 128 or 256; at most 24 warps per SM; refill_min 1..32);
 * ETRAJ_ERR_INVALID_ARGUMENT for any other. */
int etraj_set_autotune(etraj_ctx* ctx, int enable);
int etraj_bulk_tile(etraj_ctx* ctx, int dimension, int phase, int target, int multi, int* threads,
                    int* blocks_per_sm, int* refill_min);
int etraj_set_bulk_tile(etraj_ctx* ctx, int dimension, int phase, int target, int multi, int threads,
                        int blocks_per_sm, int refill_min);
/* The step chunk of a variant: the step budget per electron of the bulk
 * integrator's first round (round r: chunk 16^r; see etraj_set_straggler_repack).
 * The autotuner picks it after the shape, from 256, 1024 (the default) and 4096
 * steps, on the same sample; etraj_set_bulk_step_chunk pins it (16 .. 65536). */
int etraj_bulk_step_chunk(etraj_ctx* ctx, int dimension, int phase, int target, int multi, int* steps);
int etraj_set_bulk_step_chunk(etraj_ctx* ctx, int dimension, int phase, int target, int multi, int steps);

/* ---- rounds of the bulk integrator ------------------------------------------------------
 * No counterpart in the reference.  A few electrons of a job can need up to
 * maxiters (10^6) steps while the rest finish in ~100.  Left in place, each
 * keeps its whole thread block -- and that block's share of an SM -- resident
 * for seconds, so concurrent jobs (the serving loop) cannot get onto the GPU.
 * With repacking on (the default) the bulk integrator of a job runs in
 * rounds: once the queue is empty, an electron that has taken the step chunk
 * in round 0 (1024 steps by default, tuned; then 16x, 256x that in the next
 * rounds) writes its integrator state
 * to a device buffer and frees its lane, and the next round resumes the parked
 * electrons in as few blocks as they fill.  Batches (etraj_run_batch) run as
 * one launch.  Each electron's arithmetic does not depend on where it runs, so
 * results are the same bits either way. */
int etraj_set_straggler_repack(etraj_ctx* ctx, int enable);

/* Static assignment (off by default): the bulk integrator of a job launches one
 * lane per electron and each lane integrates its electron and stops, as the
 * plain one-thread-per-trajectory kernel does -- no queue, no refill, no
 * rounds.  A warp then runs until its slowest electron is done.  It exists to
 * measure what work stealing gains at the same precision; results are the same
 * bits either way. */
int etraj_set_static_assignment(etraj_ctx* ctx, int enable);


/* ---- per-trajectory final states ---------------------------------------------------
 * For parity checks against the reference's per-trajectory results: with
 * etraj_set_keep_final_states(ctx, 1) on when a job is enqueued (etraj_run or
 * etraj_submit), the context keeps, per surviving electron in the order of the
 * reference's concatenated `init` columns, the asymptotic momentum p_inf
 * (p_inf_vec of TrajectorySimulation.jl:383-384 / :478-479; zeros when not
 * ionized), the final phase (after the SCTS correction of :362-369 / :457-464;
 * 0 for CTMC) and the status: the ODE retcode (0 Success, 1 MaxIters,
 * 2 DtLessThanMin, 3 Unstable, 4 DtNaN) with bit 0x100 set when E_inf >= 0.
 * etraj_dump_final_states copies them (n = num_effective_traj rows; any pointer
 * may be NULL) for `ticket` (0: the last job) once the job has finished; the
 * data is kept until the context's next job.  ETRAJ_ERR_NOT_FOUND otherwise.
 * etraj_dump_step_counts gives each survivor's Tsit5 step attempts, and
 * etraj_dump_min_radius, for a job of the FP64 path (ETRAJ_ERR_UNSUPPORTED for
 * the bulk path), each survivor's least distance |r| from the core over its
 * initial state and the end of every accepted step: how close a trajectory
 * returns to the core (rescattering), which sets how many steps it needs. */
int etraj_set_keep_final_states(etraj_ctx* ctx, int enable);
int etraj_dump_final_states(etraj_ctx* ctx, uint64_t ticket, double* p_inf, double* phase, int32_t* status);
int etraj_dump_step_counts(etraj_ctx* ctx, uint64_t ticket, int32_t* steps);
int etraj_dump_min_radius(etraj_ctx* ctx, uint64_t ticket, double* rmin);

/* ---- diagnostics ----------------------------------------------------------------
 * Device time (ms) of the stages of the last etraj_run on this context: sampling,
 * compaction, field table, integrator, collection, deposit.  Writes up to n
 * values and returns how many were written (0 before the first run).  No
 * counterpart in the reference, which has no stage timers. */
int etraj_stage_times(etraj_ctx* ctx, double* ms, int n);

/* ---- deposit without allocation ---------------------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory while they call this library (their own memory pool owns the device,
 * or they reserve everything before a run): the deterministic deposit of n
 * per-electron contributions into a momentum grid, with no cudaMalloc, no
 * cudaFree and no context.  All pointers are device pointers owned by the
 * caller:
 *   key[i]        bin of electron i in [0, grid), or grid for "not deposited";
 *                 a key above grid is taken as grid (not deposited)
 *   c_re, c_im    its contribution (c_im read only when coherent != 0)
 *   spec_re/im    outputs: per-bin sums in electron order (spec_im when coherent)
 *   momentum_spec output: spec_re (CTMC) or spec_re^2 + spec_im^2 (coherent)
 * Work is queued on cuda_stream (NULL = legacy default stream); the call
 * returns without synchronizing.  The sort scratch is one fixed device array
 * of the library, sized for at most 524288 (2^19) contributions per call
 * (about 10.5 MiB, held by every GPU that loads the library until the process
 * exits); larger n returns ETRAJ_ERR_INVALID_ARGUMENT.  That array comes into
 * being when the library's device code is loaded on a device, which with
 * CUDA's lazy module loading can be this entry point's first call: make that
 * first call (or any other call of this library on the device) before a memory
 * pool of the caller claims the device's free memory, or it can fail with
 * ETRAJ_ERR_CUDA.  The array is shared
 * by all calls: calls whose work overlaps on the GPU (different streams,
 * different host threads) race, so serialize them.  The first call on a
 * device looks up the array's device address; make that first call before
 * any stream capture on that device. */
int etraj_deposit_noalloc(int64_t n, const uint32_t* key, const double* c_re, const double* c_im,
                          int64_t grid, int coherent, double* spec_re, double* spec_im,
                          double* momentum_spec, void* cuda_stream);

#ifdef __cplusplus
}
#endif

#endif /* ETRAJ_H */
