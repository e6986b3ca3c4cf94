// integrate_setup.h -- host-side set-up of what the integrators read: the
// device laser and target of a job (the reference's getters) and the
// parameters of the double-float integrator.  Shared by the library and by
// the host build of the double-float solve that the CPU tests run.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstring>

#include "engine.h"

namespace etraj {

// Laser constants with the reference's expressions (Cos4Laser.jl:81-87,
// Cos2Laser.jl:81-87, GaussianLaser.jl:85-87).
inline void mono_prepare(const etraj_mono_laser& in, DMono& L) {
    std::memset(&L, 0, sizeof L);
    L.kind = in.kind;
    L.omega = 45.563352525 / in.wave_len;        // AngFreq, Cos4Laser.jl:81
    L.period = 6.283185307179586 / L.omega;      // Period = 2pi/omega
    L.F0 = std::sqrt((in.peak_int / (1.0 + in.ellip * in.ellip)) / 3.50944521e16);  // :85
    L.A0 = L.F0 / L.omega;
    L.N = in.cyc_num;
    L.cep = in.cep;
    L.t_shift = in.t_shift;
    L.ellip = in.ellip;
    L.azi_zero = (in.azi == 0.0);
    dm_sincos(in.azi, &L.sphi, &L.cphi);
    if (L.kind == ETRAJ_LASER_GAUSSIAN) {
        L.sigma = in.cyc_num * L.period;          // SpreadDuration, GaussianLaser.jl:85
        L.inv_s2 = 1.0 / (L.sigma * L.sigma);
        L.inv_2s2 = 1.0 / (2.0 * (L.sigma * L.sigma));
    } else {
        L.w2n = L.omega / (2.0 * L.N);
        L.cN = (L.kind == ETRAJ_LASER_COS4) ? 2.0 / L.N : 1.0 / L.N;
        L.k = 200.0 / L.period;
        L.Npiw = (L.N * 3.141592653589793) / L.omega;
    }
}

// The fields of a device job that the integrators and the collection read:
// dimension, phase method, state size, laser, target, rtol and t_final.  A
// molecule's trajectories are the hydrogen-like equations with Z = charge + 1,
// soft core 1.0 and the phase's Ip = IonPotential(mol) (GenericMolecule.jl:438-445).
inline void prepare_integration(const etraj_job* job, DJob& J) {
    J.dim = job->dimension;
    J.phase = job->traj_phase_method;
    J.n_state = (J.dim == 3 ? 6 : 4) + (J.phase != ETRAJ_PHASE_CTMC ? 1 : 0);
    J.laser.kind = job->laser.kind;
    mono_prepare(job->laser.mono[0], J.laser.m[0]);
    if (job->laser.kind == ETRAJ_LASER_BICHROMATIC) {
        mono_prepare(job->laser.mono[1], J.laser.m[1]);
        J.laser.delay = job->laser.delay;
        J.laser.nmono = 2;
    } else {
        J.laser.nmono = 1;
    }
    const etraj_target& T = job->target;
    J.target.kind = T.kind;
    J.target.Z = (double)T.Z;
    J.target.Ip = T.Ip;
    J.target.sc = T.soft_core;
    J.target.a1 = T.a1; J.target.b1 = T.b1;
    J.target.a2 = T.a2; J.target.b2 = T.b2;
    J.target.a3 = T.a3; J.target.b3 = T.b3;
    {
        const double a[3] = {T.a1, T.a2, T.a3}, b[3] = {T.b1, T.b2, T.b3};
        J.target.skip_ok = etraj_sae_skip_exact((double)T.Z, a, b, T.soft_core);
    }
    if (T.kind == ETRAJ_TARGET_MOLECULE) {
        J.target.kind = ETRAJ_TARGET_HYDROGEN_LIKE;
        J.target.Ip = T.mol_Ip_traj;
        J.target.sc = 1.0;
        J.target.skip_ok = 0;
    }
    J.rtol = job->traj_rtol;
    J.t_final = job->traj_t_final;
}

inline float2 df_split2(double v) {
    const float h = (float)v;
    return make_float2(h, (float)(v - (double)h));
}

// Double-float integrator parameters (launch shape aside): a field table of
// degree-7 pieces spanning [tmin, t_final] with spacing T_min/kDfTablePerPeriod
// (T_min the shortest laser period), its clock, tolerances and the target.
inline void prepare_df_params(const DJob& J, double tmin, int64_t max_n, DFParams& D) {
    std::memset(&D, 0, sizeof D);
    D.dim = J.dim;
    D.phase = J.phase;
    D.tgt = J.target.kind;
    double T = J.laser.m[0].period;
    if (J.laser.nmono == 2) T = std::min(T, J.laser.m[1].period);
    const double h = T / (double)kDfTablePerPeriod;
    D.T0 = tmin - h;
    D.n_int = (int)std::ceil((J.t_final - D.T0) / h) + 2;
    D.h_d = h;
    D.inv_h_d = 1.0 / h;
    D.h = df_split2(h);
    D.inv_h = df_split2(1.0 / h);
    D.t_final = J.t_final;
    const double q = (J.t_final - D.T0) / h;
    const double fl = std::floor(q);
    D.nf = (int)fl;
    D.ff = df_split2(q - fl);
    D.rtol = df_split2(J.rtol);
    // t_final is reached once within 100 ulp of it (the FP64 solve's snap)
    D.t_snap = (float)(100.0 * (std::nextafter(std::fabs(J.t_final), INFINITY) - std::fabs(J.t_final)));
    const DTarget& T_ = J.target;
    D.Z = df_split2(T_.Z);
    D.Ip = df_split2(T_.Ip);
    D.sc = df_split2(T_.sc);
    D.a1 = df_split2(T_.a1); D.b1 = df_split2(T_.b1);
    D.a2 = df_split2(T_.a2); D.b2 = df_split2(T_.b2);
    D.a3 = df_split2(T_.a3); D.b3 = df_split2(T_.b3);
    D.a2b2 = df_split2(T_.a2 * T_.b2);
    // beyond r^2 = r2_far every b_i r exceeds the exponentials' skip bound (50) by a
    // margin that rounding cannot close, so each exp(-b_i r) is taken as 0 there
    {
        const double bmin = std::min(T_.b1, std::min(T_.b2, T_.b3));
        const double rf = 50.0 / bmin;
        D.r2_far = (bmin > 0.0) ? (float)(rf * rf * (1.0 + 1.0 / 1024.0)) : INFINITY;
    }
    D.max_iters = kBulkMaxIters;
    D.max_n = max_n;
}

// The 8 Chebyshev nodes u_j = cos((2j+1) pi/16) of a table piece and the values
// T_m(u_j) = cos(m (2j+1) pi/16), computed once on the host so that every build
// of the table does the same FP64 arithmetic.
inline void df_table_nodes(DfTableNodes& N) {
    for (int j = 0; j < 8; ++j) {
        N.u[j] = std::cos((2.0 * j + 1.0) * 3.141592653589793 / 16.0);
        for (int m = 0; m < 8; ++m) N.Tm[m][j] = std::cos((double)m * (2.0 * j + 1.0) * 3.141592653589793 / 16.0);
    }
}

}  // namespace etraj
