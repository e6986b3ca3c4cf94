// integrate_df.cu -- the double-float integrator: persistent, warp-cooperative,
// work-stealing Tsit5 on the FP32 pipe with every stage value, sum, error
// estimate and controller power a double-float pair (dfloat.h).  Two passes: a
// start-up pass over an electron's first steps, whose stages are formed as
// differences from the accepted state (df_solve.cuh), and a main pass, every
// stage evaluated directly, over the electrons the start-up hands on.
//
// It restates the plain FP64 solve of integrate_fp64.cu step for step, so it
// takes the FP64 path's step sequence and its final states agree with the FP64
// path's to ~1e-11 (the spread a 1-ulp change of an FP64 input gives); the FP64
// collection (Kepler asymptote, SCTS phase) and deposit then run on them
// unchanged.  What FP32 stage values cannot do is resolve the error estimate,
// whose weighted sums cancel to ~1e-10 of the stage derivatives in an electron's
// first steps: with FP32 stages the controller sees another error and takes
// another step sequence.
//
// Schedule.  A warp advances its lanes stage by stage in lock-step: a counter
// st = 1..6 shared by the warp selects the Tsit5 stage every stepping lane
// evaluates, and each turn of the loop makes exactly one right-hand-side
// evaluation site, so the kernel holds one copy of that (long) double-float code
// and the instruction cache keeps it.  The stage differences of the attempt live in
// shared memory (6 slots per lane).  At each attempt boundary (st = 1) lanes that
// finished take new electrons from a global queue (warp-aggregated atomicAdd); a
// new electron spends the first two turns on its starting step and joins the
// stepping lanes at the next boundary.  The laser table at the end of the
// attempt (stage 5) serves stage 6 and the new accepted state too, whose target
// terms are stage 6's.  The start-up pass hands an electron on at the first
// boundary where it needs no differences (to a list, warp-aggregated atomicAdd);
// a main-pass lane that takes one spends one turn evaluating its state.  Since
// ~95% of the attempts run in the main pass, no warp there carries the longer
// difference code for one lane, and it is not compiled into that pass.
//
// Field table.  F(t) is one function of time for every electron, tabulated once
// per job in FP64: pieces of width h = T_min/1024 (T_min the shortest laser
// period), each the degree-7 polynomial through F at the piece's 8 Chebyshev
// nodes, stored as monomials in u in [-1, 1] (c0 exact as three floats, c1..c3 as
// double-float pairs, c4..c7 as floats), 112 B per piece read through the L1
// cache.  Time is a clock of an integer piece index and a double-float fraction.
//
// Roofline: FP32 issue bound (a double-float add is ~11 FP32 instructions, a
// product ~7); no tensor cores (not a contraction).  Compiled with
// --fmad=false: every fused multiply-add is an explicit fmaf(), as the
// error-free transformations need.

#include "df_solve.cuh"

namespace etraj {

__device__ const float g_df_exp2[2 * kExpTabN] = {ETRAJ_DF_EXP2_TABLE};
__device__ const float g_df_log2c[2 * kLogTabN] = {ETRAJ_DF_LOG2C_TABLE};
__device__ const float g_df_rcpc[2 * kLogTabN] = {ETRAJ_DF_RCPC_TABLE};

namespace {

// Threads per block and resident blocks per SM of the two passes: a register
// budget of 128 a thread, a few hundred bytes spilled.  With 128-thread blocks
// whose warps ran freely, the argon headline job (4.0e6 electrons) took 93.8,
// 93.5, 96.9 and 98.8 ms with (start-up, main) blocks per SM of (3, 4), (2, 4),
// (4, 4) and (3, 5), with identical results; without launch bounds (up to 251
// registers) it took 139 ms.  With the warps of a block in step (below), blocks
// of 256 threads were faster than 128 or 512 on a 2e6-candidate job: main pass
// 13.5 ms against 14.1 and 13.9; start-up pass in 2 x 256 threads (128
// registers) against 3 x 128 (168 registers), 13.2 against 13.5 ms for both.
constexpr int kDfThreadsStart = 256;
constexpr int kDfMinBlocksStart = 2;
constexpr int kDfThreadsMain = 256;
constexpr int kDfMinBlocksMain = 2;

template <int DIM, int PHASE>
constexpr int slot_floats() {
    return 6 * dfs::Lane<DIM, PHASE>::KW;
}

enum LaneMode { kFree = 0, kBase = 1, kInit1 = 2, kWait = 3, kStep = 4 };

// MAIN = false: the start-up pass, from the initial conditions (the starting
// step's two evaluations, then attempts whose stages are differences) to each
// electron's first attempt that needs no differences, where it is carried over;
// MAIN = true: the main pass over the carried electrons, every stage direct.
// work[0] and work[2] are the passes' queues, work[1] counts carried electrons.
template <int DIM, int PHASE, int TGT, bool MAIN>
__global__ void __launch_bounds__(MAIN ? kDfThreadsMain : kDfThreadsStart, MAIN ? kDfMinBlocksMain : kDfMinBlocksStart)
k_integrate_df(const __grid_constant__ DFParams P, InitSoA soa, const double* __restrict__ tsamp,
               const int64_t* __restrict__ idx, const unsigned long long* __restrict__ count,
               unsigned long long* __restrict__ work, TrajOut out) {
    using LaneT = dfs::Lane<DIM, PHASE>;
    constexpr int KW = LaneT::KW;
    constexpr int N = LaneT::N;
    extern __shared__ float s_slots[];
    __shared__ float s_exp2[2 * kExpTabN], s_log2c[2 * kLogTabN], s_rcpc[2 * kLogTabN];
    for (int i = threadIdx.x; i < 2 * kExpTabN; i += blockDim.x) s_exp2[i] = g_df_exp2[i];
    for (int i = threadIdx.x; i < 2 * kLogTabN; i += blockDim.x) {
        s_log2c[i] = g_df_log2c[i];
        s_rcpc[i] = g_df_rcpc[i];
    }
    __syncthreads();
    const dfs::Tabs T{s_exp2, s_log2c, s_rcpc};
    const dfs::Slots<KW> ks{s_slots + threadIdx.x, (int)blockDim.x};
    const dfs::Carry C{P.carry, P.max_n};
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned lt_mask = (1u << lane) - 1u;
    unsigned long long* queue = work + (MAIN ? 2 : 0);
    unsigned long long* n_carried = work + 1;
    const unsigned long long n_traj = MAIN ? *n_carried : *count;

    LaneT L = {};
    dfs::TAt B;  // the target's terms at the accepted state (start-up: for the differences)
    int mode = kFree;
    unsigned long long s = 0;
    bool drained = false;

    auto finish = [&](int status) {
        out.status[s] = status;
        out.steps[s] = L.attempts;
        double fs[N];
        dfs::final_state(L, fs);
#pragma unroll
        for (int j = 0; j < N; ++j) out.final_state[s * N + j] = fs[j];
        mode = kFree;
    };

    // The block's warps go through the evaluations in step (a barrier at each): the
    // loop's code is far larger than the instruction cache, and warps at the same
    // place share the lines they fetch.
    for (int st = 1;; st = (st == 6) ? 1 : st + 1) {
        if (st != 1) __syncthreads();
        if (st == 1) {
            // ---- attempt boundary: hand over, start the next attempts, refill ------------
            if (mode == kWait) mode = kStep;
            if (!MAIN) {
                const bool leave = (mode == kStep) && !dfs::precise(L);
                const unsigned lm = __ballot_sync(FULL, leave);
                if (lm) {
                    const int leader = __ffs(lm) - 1;
                    unsigned long long k0 = 0ull;
                    if (lane == leader) k0 = atomicAdd(n_carried, (unsigned long long)__popc(lm));
                    k0 = __shfl_sync(FULL, k0, leader);
                    if (leave) {
                        dfs::save_carry(L, C, (int64_t)(k0 + __popc(lm & lt_mask)), s);
                        mode = kFree;
                    }
                }
            }
            if (mode == kStep) {
                const int status = dfs::prologue(L, P);
                if (status) finish(status);
            }
            const unsigned freem = __ballot_sync(FULL, mode == kFree);
            if (freem && !drained) {
                const int leader = __ffs(freem) - 1;
                unsigned long long base = 0ull;
                if (lane == leader) base = atomicAdd(queue, (unsigned long long)__popc(freem));
                base = __shfl_sync(FULL, base, leader);
                drained = base + (unsigned long long)__popc(freem) >= n_traj;
                if (mode == kFree) {
                    const unsigned long long k = base + __popc(freem & lt_mask);
                    if (k < n_traj) {
                        if (MAIN) {
                            s = dfs::restore_carry(L, C, (int64_t)k);
                        } else {
                            s = k;
                            const int64_t g = idx ? idx[s] : (int64_t)s;
                            double x0[DIM], p0[DIM];
                            x0[0] = soa.x[g];
                            x0[1] = soa.y[g];
                            p0[0] = soa.kx[g];
                            p0[1] = soa.ky[g];
                            if (DIM == 3) {
                                x0[2] = 0.0;
                                p0[2] = soa.kz[g];
                            }
                            dfs::load(L, P, x0, p0, LaneT::HASPH ? soa.phase[g] : 0.0, tsamp[soa.batch[g]]);
                        }
                        mode = kBase;
                    }
                }
            }
            if (!__syncthreads_or(mode != kFree)) break;  // the block leaves together
        }
        // ---- the inputs of this turn's evaluation ------------------------------------------
        if (mode == kStep) dfs::stage_in<MAIN>(L, ks, st);
        // ---- one evaluation: the laser table, and the target's terms at the new point
        //      directly (an accepted state: a new electron's, stage 6's; every stage of
        //      the main pass) and/or as the change from the accepted state (start-up) ------
        if (mode == kStep || mode == kInit1 || mode == kBase) {
            const bool step6 = (mode == kStep && st == 6);
            dfs::FieldAt F;
            if (step6) F = L.F5;  // stage 6 is at stage 5's time
            else dfs::field_at(P, L.ni, L.fi, F);
            const bool diff = !MAIN && mode != kBase;
            dfs::TAt Tl;
            df KT[DIM], dKT[DIM], dkph, kph;
            dfs::target_eval<DIM, PHASE, TGT, !MAIN>(P, T.exp2, L, B, diff, !diff || step6, Tl, KT, dKT, dkph, kph);
            if (mode == kBase) {
                if (!MAIN) B = Tl;
                dfs::set_base(L, F, KT, kph);
                mode = (!MAIN && dfs::init_first(L, P)) ? kInit1 : kWait;
            } else {
                if (MAIN) dfs::set_full(L, ks, st, F, KT, kph);
                else dfs::set_diff(L, ks, (mode == kInit1) ? 1 : st, F, dKT, dkph);
                if (mode == kInit1) {
                    dfs::init_second(L, P, ks, T);
                    mode = kWait;
                } else if (st == 5) {
                    L.F5 = F;
                } else if (step6) {
                    const int status = dfs::epilogue<MAIN>(L, P, ks, T);
                    if (status) {
                        finish(status < 0 ? 0 : status);
                    } else if (L.accept) {
                        if (!MAIN) B = Tl;
                        dfs::set_base(L, L.F5, KT, kph);
                    }
                }
            }
        }
    }
}

__global__ void k_field_table_df(const __grid_constant__ DJob J, double T0, double h, int n_int,
                                 const __grid_constant__ DfTableNodes nodes, float4* __restrict__ tab) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_int) return;
    dfs::table_piece(J.laser, T0, h, k, nodes, tab + kDfTableF4 * (size_t)k);
}

// Both passes may take the stage slots of their whole block in dynamic shared
// memory (up to kDfThreads x slot_floats floats, above the default 48 KB).
template <int DIM, int PHASE, int TGT>
void allow_smem() {
    static bool done[64] = {};  // per device
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        dev = 0;
    }
    if (done[dev]) return;
    const int most = (int)((size_t)slot_floats<DIM, PHASE>() * sizeof(float) *
                           (size_t)(kDfThreadsMain > kDfThreadsStart ? kDfThreadsMain : kDfThreadsStart));
    cudaFuncSetAttribute(k_integrate_df<DIM, PHASE, TGT, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, most);
    cudaFuncSetAttribute(k_integrate_df<DIM, PHASE, TGT, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, most);
    done[dev] = true;
}

template <int DIM, int PHASE, int TGT>
int launch_df_t(const DFParams& P, InitSoA soa, const double* t, const int64_t* idx, const unsigned long long* count,
                unsigned long long* work, TrajOut out, cudaStream_t s) {
    const size_t smem = (size_t)slot_floats<DIM, PHASE>() * sizeof(float) * (size_t)P.threads;
    const size_t smem_main = (size_t)slot_floats<DIM, PHASE>() * sizeof(float) * (size_t)P.threads_main;
    allow_smem<DIM, PHASE, TGT>();
    cudaMemsetAsync(work, 0, 3 * sizeof(unsigned long long), s);
    k_integrate_df<DIM, PHASE, TGT, false><<<P.blocks, P.threads, smem, s>>>(P, soa, t, idx, count, work, out);
    k_integrate_df<DIM, PHASE, TGT, true><<<P.blocks_main, P.threads_main, smem_main, s>>>(P, soa, t, idx, count,
                                                                                         work, out);
    return 2;
}

template <int DIM, int PHASE, int TGT>
int blocks_t(bool main, int threads) {
    allow_smem<DIM, PHASE, TGT>();
    const size_t smem = (size_t)slot_floats<DIM, PHASE>() * sizeof(float) * (size_t)threads;
    int nb = 0;
    const cudaError_t e =
        main ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_integrate_df<DIM, PHASE, TGT, true>, threads, smem)
             : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_integrate_df<DIM, PHASE, TGT, false>, threads, smem);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    return nb > 0 ? nb : 1;
}

}  // namespace

int launch_field_table_df(const DJob& J, double T0, double h, int n_int, const DfTableNodes& nodes, float4* tab,
                          cudaStream_t s) {
    k_field_table_df<<<(n_int + 127) / 128, 128, 0, s>>>(J, T0, h, n_int, nodes, tab);
    return 1;
}

#define ETRAJ_DF_DISPATCH(FN, ARGS)                                                                  \
    if (dim == 2) {                                                                                  \
        if (phase == ETRAJ_PHASE_CTMC)                                                               \
            return tgt == ETRAJ_TARGET_HYDROGEN_LIKE ? FN<2, ETRAJ_PHASE_CTMC, ETRAJ_TARGET_HYDROGEN_LIKE> ARGS \
                                                     : FN<2, ETRAJ_PHASE_CTMC, ETRAJ_TARGET_SAE> ARGS;         \
        if (phase == ETRAJ_PHASE_QTMC)                                                               \
            return tgt == ETRAJ_TARGET_HYDROGEN_LIKE ? FN<2, ETRAJ_PHASE_QTMC, ETRAJ_TARGET_HYDROGEN_LIKE> ARGS \
                                                     : FN<2, ETRAJ_PHASE_QTMC, ETRAJ_TARGET_SAE> ARGS;         \
        return tgt == ETRAJ_TARGET_HYDROGEN_LIKE ? FN<2, ETRAJ_PHASE_SCTS, ETRAJ_TARGET_HYDROGEN_LIKE> ARGS     \
                                                 : FN<2, ETRAJ_PHASE_SCTS, ETRAJ_TARGET_SAE> ARGS;             \
    }                                                                                                \
    if (phase == ETRAJ_PHASE_CTMC)                                                                   \
        return tgt == ETRAJ_TARGET_HYDROGEN_LIKE ? FN<3, ETRAJ_PHASE_CTMC, ETRAJ_TARGET_HYDROGEN_LIKE> ARGS     \
                                                 : FN<3, ETRAJ_PHASE_CTMC, ETRAJ_TARGET_SAE> ARGS;             \
    if (phase == ETRAJ_PHASE_QTMC)                                                                   \
        return tgt == ETRAJ_TARGET_HYDROGEN_LIKE ? FN<3, ETRAJ_PHASE_QTMC, ETRAJ_TARGET_HYDROGEN_LIKE> ARGS     \
                                                 : FN<3, ETRAJ_PHASE_QTMC, ETRAJ_TARGET_SAE> ARGS;             \
    return tgt == ETRAJ_TARGET_HYDROGEN_LIKE ? FN<3, ETRAJ_PHASE_SCTS, ETRAJ_TARGET_HYDROGEN_LIKE> ARGS         \
                                             : FN<3, ETRAJ_PHASE_SCTS, ETRAJ_TARGET_SAE> ARGS;

int df_threads(bool main) { return main ? kDfThreadsMain : kDfThreadsStart; }

int launch_integrate_df(const DFParams& P, InitSoA soa, const double* t, const int64_t* idx,
                        const unsigned long long* count, unsigned long long* work, TrajOut out, cudaStream_t s) {
    const int dim = P.dim, phase = P.phase, tgt = P.tgt;
    ETRAJ_DF_DISPATCH(launch_df_t, (P, soa, t, idx, count, work, out, s))
}

int df_blocks_per_sm(int dim, int phase, int tgt, bool main, int threads) {
    ETRAJ_DF_DISPATCH(blocks_t, (main, threads))
}

#undef ETRAJ_DF_DISPATCH

}  // namespace etraj
