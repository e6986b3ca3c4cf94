/* oracle_mol_ref.c -- an independent restatement of the molecular rate pieces
 * the device sampler and the oracle's twin share (csrc/mol.h): the MO-ADK /
 * MO-SPANE / MO-SPA prefactor numerator and the WFAT rate.  TEST
 * INFRASTRUCTURE ONLY: nothing in the product includes or calls this file.
 *
 * Written from the reference with C99 complex arithmetic and the C library's
 * functions:
 *   - the field-frame -> molecular-frame Euler angles (obtain_FF_MF_Euler,
 *     shared_methods.jl:29-37): R = RotZYZ(mol_rot)^T FF, then the z-y-z angles
 *     of R (Rotations.jl's `params(RotZYZ(R))`);
 *   - Wigner's D^l_{m'm}(a, b, g) = exp(-i m' a) d^l_{m'm}(b) exp(-i m g) with
 *     d from Wigner's explicit sum (the convention of WignerD.jl's wignerdjmn
 *     and wignerDjmn, which the reference calls);
 *   - the solid harmonics of gen_sph_harm_funcs (shared_methods.jl:15-25) at
 *     complex k;
 *   - the prefactor numerator sum_{l, m, m'} C_lm D^l_{m'm} Y_{l m'}(k) in
 *     lmm_list order (ADKSampler.jl:188-265);
 *   - the structure factor G_{n_xi m}(beta, gamma) (GenericMolecule.jl:236-259)
 *     and the WFAT rate sum |G|^2 W dkdt (WFATSampler.jl:129-170).
 * Agreement with the twin is to rounding; the tests state the tolerance. */
#include <math.h>
#include <stdlib.h>

#include "oracle_sampler.h"

#include <complex.h>
#undef I /* the imaginary unit is IU here: I names arrays in the headers above */
#define IU _Complex_I

typedef double complex zc;

static double ref_fact(int n) { return tgamma((double)n + 1.0); }

/* R = Rz(a) Ry(b) Rz(g), row-major */
static void ref_rotzyz(double a, double b, double g, double R[9]) {
    const double ca = cos(a), sa = sin(a), cb = cos(b), sb = sin(b), cg = cos(g), sg = sin(g);
    R[0] = ca * cb * cg - sa * sg;
    R[1] = -ca * cb * sg - sa * cg;
    R[2] = ca * sb;
    R[3] = sa * cb * cg + ca * sg;
    R[4] = -sa * cb * sg + ca * cg;
    R[5] = sa * sb;
    R[6] = -sb * cg;
    R[7] = sb * sg;
    R[8] = cb;
}

/* obtain_FF_MF_Euler (shared_methods.jl:29-37) */
static void ref_euler(const double rot[3], double Fx, double Fy, double* a, double* b, double* g) {
    const double F = hypot(Fx, Fy);
    const double FF[9] = {0.0, Fy / F, Fx / F, 0.0, -Fx / F, Fy / F, 1.0, 0.0, 0.0};
    double M[9], R[9];
    ref_rotzyz(rot[0], rot[1], rot[2], M);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double s = 0.0;
            for (int k = 0; k < 3; ++k) s += M[3 * k + i] * FF[3 * k + j]; /* M^T FF */
            R[3 * i + j] = s;
        }
    *a = atan2(R[5], R[2]);
    *b = atan2(hypot(R[2], R[5]), R[8]);
    *g = atan2(R[7], -R[6]);
}

/* Wigner's small d^j_{m'm}(b) by his explicit sum */
static double ref_wigner_d(int j, int mp, int m, double b) {
    const double c = cos(b / 2.0), s = sin(b / 2.0);
    const double pre = sqrt(ref_fact(j + mp) * ref_fact(j - mp) * ref_fact(j + m) * ref_fact(j - m));
    double sum = 0.0;
    for (int k = 0; k <= 2 * j; ++k) {
        if (j + m - k < 0 || mp - m + k < 0 || j - mp - k < 0) continue;
        const double den = ref_fact(j + m - k) * ref_fact(k) * ref_fact(mp - m + k) * ref_fact(j - mp - k);
        const double sign = ((mp - m + k) & 1) ? -1.0 : 1.0;
        sum += sign * pow(c, 2 * j + m - mp - 2 * k) * pow(s, mp - m + 2 * k) / den;
    }
    return pre * sum;
}

static zc ref_wigner_D(int j, int mp, int m, double a, double b, double g) {
    return cexp(-IU * (double)mp * a) * ref_wigner_d(j, mp, m, b) * cexp(-IU * (double)m * g);
}

static zc ref_cpowi(zc z, int n) {
    zc r = 1.0;
    for (int i = 0; i < n; ++i) r *= z;
    return r;
}

/* Y_{lm}(x, y, z) of gen_sph_harm_funcs (shared_methods.jl:15-25) for k^2 = -kappa^2 */
static zc ref_sph(int l, int m, zc x, zc y, zc z, double kappa) {
    zc acc = 0.0;
    const int k0 = m < 0 ? -m : 0, k1 = (l - m) / 2; /* floor for l - m >= 0 */
    for (int k = k0; k <= k1; ++k) {
        const double c = ((k & 1) ? -1.0 : 1.0) /
                         (ldexp(1.0, 2 * k + m) * ref_fact(k + m) * ref_fact(k) * ref_fact(l - m - 2 * k));
        acc += c * ref_cpowi(x + IU * y, k + m) * ref_cpowi(x - IU * y, k) * ref_cpowi(z, l - m - 2 * k);
    }
    const double norm = ((m & 1) ? -1.0 : 1.0) * sqrt((2 * l + 1) / (4.0 * M_PI) * ref_fact(l - m) / ref_fact(l + m));
    return norm / ref_cpowi(-IU * kappa, l) * ref_fact(l + m) * acc;
}

static zc ref_clm(const o_sampler* S, int l, int m) {
    const int lmax = S->T.lmax, e = l + (m + l) * (lmax + 1);
    return S->clm[2 * e] + IU * S->clm[2 * e + 1];
}

/* the molecular prefactor numerator at the field-frame momentum (nkx, nky, nkz) */
dm_cplx o_mol_numerator_ref(const o_sampler* S, const o_batch* B, dm_cplx nkx, dm_cplx nky, dm_cplx nkz) {
    double a, b, g;
    ref_euler(S->mol_rot, B->Fx, B->Fy, &a, &b, &g);
    const zc x = nkx.re + IU * nkx.im, y = nky.re + IU * nky.im, z = nkz.re + IU * nkz.im;
    zc acc = 0.0;
    for (int l = 0; l <= S->T.lmax; ++l)
        for (int m = -l; m <= l; ++m) {
            const zc C = ref_clm(S, l, m);
            if (C == 0.0) continue;
            for (int mp = -l; mp <= l; ++mp)
                acc += C * ref_wigner_D(l, mp, m, a, b, g) * ref_sph(l, mp, x, y, z, S->kappa);
        }
    return dm_c(creal(acc), cimag(acc));
}

/* G_{n_xi m}(theta, chi) (GenericMolecule.jl:236-259) */
static zc ref_wfat_G(int nxi, int m, int nxi_max, int m_max, int lmax, const double* Idat, const double mu[3],
                     double kappa, double theta, double chi) {
    zc s = 0.0;
    const int am = m < 0 ? -m : m;
    for (int l = am; l <= lmax; ++l)
        for (int mp = -l; mp <= l; ++mp) {
            const int e = nxi + (nxi_max + 1) * (m + m_max + (2 * m_max + 1) * (l + (lmax + 1) * (mp + l)));
            const zc Iv = Idat[2 * e] + IU * Idat[2 * e + 1];
            s += Iv * ref_wigner_d(l, m, mp, theta) * cexp(-IU * (double)mp * chi);
        }
    /* mu_z of RotZYZ(chi, theta, 0) mu: the third row of Ry(theta) */
    const double muz = -sin(theta) * mu[0] + cos(theta) * mu[2];
    return s * exp(-kappa * muz);
}

void oracle_mol_wfat_G_ref(const etraj_target* T, int nxi, int m, double theta, double chi, double* out) {
    const zc G = ref_wfat_G(nxi, m, T->wfat_nxi_max, T->wfat_m_max, T->wfat_lmax, T->wfat_intdata, T->wfat_mu,
                            sqrt(2.0 * T->Ip), theta, chi);
    out[0] = creal(G);
    out[1] = cimag(G);
}

/* the WFAT rate of one candidate (WFATSampler.jl:150-170) */
double o_wfat_rate_ref(const o_sampler* S, const o_batch* B, double kd, double kz) {
    double a, b, g;
    ref_euler(S->mol_rot, B->Fx, B->Fy, &a, &b, &g);
    const double k = S->kappa, n = S->n, F = B->F, k2 = kd * kd + kz * kz;
    double rate = 0.0;
    for (int m = -S->mmax; m <= S->mmax; ++m)
        for (int nxi = 0; nxi <= S->nxi; ++nxi) {
            const zc G = ref_wfat_G(nxi, m, S->nxi, S->mmax, S->wl, S->wint, S->mu, k, b, g);
            const int am = m < 0 ? -m : m;
            const double W = pow(k, am + 2) / 2.0 / pow(F, am + 1) / ref_fact(am) *
                             pow(4.0 * k * k / F, 2.0 * n - 2.0 * nxi - am - 1.0) * pow(k2, am) *
                             exp(-2.0 * pow(k * k + k2, 1.5) / (3.0 * F));
            rate += (creal(G) * creal(G) + cimag(G) * cimag(G)) * W;
        }
    return rate * S->dkdt;
}
