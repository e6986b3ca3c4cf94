// Host build of the double-float integrator's per-electron solve
// (etraj.jl_gb300/csrc/df_solve.cuh, the code the device kernel runs) for
// tests/test_df_host.py, which checks it against the FP64 oracle on the CPU.
// One electron after another: load, the starting step's two evaluations, then
// prologue, six stages and epilogue per attempt, as a lane of the kernel does
// (stage 6's direct target terms become the next accepted state's), with the
// hand-over from the start-up pass to the main pass at the same boundary.
#include <vector>

#include "df_solve.cuh"
#include "integrate_setup.h"

using namespace etraj;

namespace {

template <int DIM, int PHASE, int TGT>
void solve_all(const DFParams& P, int64_t n, const double* init, double* final_state, int32_t* status,
               int32_t* steps) {
    using LaneT = dfs::Lane<DIM, PHASE>;
    constexpr int N = LaneT::N;
    constexpr int KW = LaneT::KW;
    const int rows = (DIM == 3 ? 8 : 6) + (LaneT::HASPH ? 1 : 0);
    const dfs::Tabs T{kExp2Tab, kLog2cTab, kRcpcTab};
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < n; ++i) {
        const double* r = init + i * rows;
        double x0[3] = {r[0], r[1], 0.0}, p0[3] = {0.0, 0.0, 0.0};
        for (int d = 0; d < DIM; ++d) p0[d] = r[DIM + d];
        const double t0 = r[2 * DIM], ph0 = LaneT::HASPH ? r[rows - 1] : 0.0;
        float slots[6 * KW], carry[kDfCarryWords];
        const dfs::Slots<KW> ks{slots, 1};
        const dfs::Carry Cw{carry, 1};
        LaneT L = {};
        dfs::TAt B, Tl;
        dfs::FieldAt F;
        df KT[DIM], dKT[DIM], dkph, kph;
        // start-up pass: the starting step, then attempts with stage differences
        dfs::load(L, P, x0, p0, ph0, t0);
        dfs::field_at(P, L.ni, L.fi, F);
        dfs::target_eval<DIM, PHASE, TGT, true>(P, T.exp2, L, B, false, true, Tl, KT, dKT, dkph, kph);
        B = Tl;
        dfs::set_base(L, F, KT, kph);
        if (dfs::init_first(L, P)) {
            dfs::field_at(P, L.ni, L.fi, F);
            dfs::target_eval<DIM, PHASE, TGT, true>(P, T.exp2, L, B, true, false, Tl, KT, dKT, dkph, kph);
            dfs::set_diff(L, ks, 1, F, dKT, dkph);
            dfs::init_second(L, P, ks, T);
        }
        int st = 0;
        bool main = false;
        while (true) {
            if (!main && !dfs::precise(L)) {
                // hand-over to the main pass, through the carry words as on the device
                dfs::save_carry(L, Cw, 0, (uint64_t)i);
                L = LaneT{};
                dfs::restore_carry(L, Cw, 0);
                dfs::field_at(P, L.ni, L.fi, F);
                dfs::target_eval<DIM, PHASE, TGT, false>(P, T.exp2, L, B, false, true, Tl, KT, dKT, dkph, kph);
                dfs::set_base(L, F, KT, kph);
                main = true;
            }
            st = dfs::prologue(L, P);
            if (st) break;
            for (int s = 1; s <= 6; ++s) {
                if (main) dfs::stage_in<true>(L, ks, s);
                else dfs::stage_in<false>(L, ks, s);
                if (s == 6) F = L.F5;  // stage 6 is at stage 5's time
                else dfs::field_at(P, L.ni, L.fi, F);
                dfs::target_eval<DIM, PHASE, TGT, true>(P, T.exp2, L, B, !main, main || s == 6, Tl, KT, dKT, dkph,
                                                        kph);
                if (main) dfs::set_full(L, ks, s, F, KT, kph);
                else dfs::set_diff(L, ks, s, F, dKT, dkph);
                if (s == 5) L.F5 = F;
            }
            st = main ? dfs::epilogue<true>(L, P, ks, T) : dfs::epilogue<false>(L, P, ks, T);
            if (st) break;
            if (L.accept) {
                B = Tl;
                dfs::set_base(L, L.F5, KT, kph);
            }
        }
        status[i] = st < 0 ? 0 : st;
        steps[i] = L.attempts;
        double fs[N];
        dfs::final_state(L, fs);
        for (int j = 0; j < N; ++j) final_state[i * N + j] = fs[j];
    }
}

}  // namespace

// init: n electrons in the reference's init layout; tmin: the job's first time sample
extern "C" int dfhost_integrate(const etraj_job* job, int64_t n, const double* init, double tmin,
                                double* final_state, int32_t* status, int32_t* steps) {
    DJob J;
    std::memset(&J, 0, sizeof J);
    prepare_integration(job, J);
    DFParams P;
    prepare_df_params(J, tmin, n, P);
    DfTableNodes nodes;
    df_table_nodes(nodes);
    std::vector<float4> tab((size_t)P.n_int * kDfTableF4);
#pragma omp parallel for
    for (int k = 0; k < P.n_int; ++k) dfs::table_piece(J.laser, P.T0, P.h_d, k, nodes, tab.data() + kDfTableF4 * (size_t)k);
    P.table = tab.data();
    const bool h = J.target.kind == ETRAJ_TARGET_HYDROGEN_LIKE;
#define DFH_CALL(D, PH)                                                                     \
    (h ? solve_all<D, PH, ETRAJ_TARGET_HYDROGEN_LIKE>(P, n, init, final_state, status, steps) \
       : solve_all<D, PH, ETRAJ_TARGET_SAE>(P, n, init, final_state, status, steps))
    if (J.dim == 2) {
        if (J.phase == ETRAJ_PHASE_CTMC) DFH_CALL(2, ETRAJ_PHASE_CTMC);
        else if (J.phase == ETRAJ_PHASE_QTMC) DFH_CALL(2, ETRAJ_PHASE_QTMC);
        else DFH_CALL(2, ETRAJ_PHASE_SCTS);
    } else {
        if (J.phase == ETRAJ_PHASE_CTMC) DFH_CALL(3, ETRAJ_PHASE_CTMC);
        else if (J.phase == ETRAJ_PHASE_QTMC) DFH_CALL(3, ETRAJ_PHASE_QTMC);
        else DFH_CALL(3, ETRAJ_PHASE_SCTS);
    }
#undef DFH_CALL
    return 0;
}
