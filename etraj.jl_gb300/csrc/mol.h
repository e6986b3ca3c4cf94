// mol.h -- molecular targets: the MO-ADK rate prefactor and the WFAT rate.
//
// Plain functions over plain arrays, compiled both into the device sampler
// and into the CPU oracle, so the two evaluate the same operations in the
// same order.  Needs detmath.h (dm_*) included first.
//
// Reference:
//   src/ElectronSamplers/ADKSampler.jl:188-265, SPANESampler.jl:187-262,
//     SPASampler.jl:183-268: the molecular branch of the rate prefactor,
//     sum over (l, m, m') of C_lm D^l_{m' m}(alpha, beta, gamma) Y_{l m'}(k),
//     with (l, m, m') in the order of `lmm_list` (l outermost, m' innermost).
//   src/ElectronSamplers/WFATSampler.jl:129-249: the WFAT rate
//     sum_{n_xi, m} |G_{n_xi m}|^2 W_{n_xi |m|}(kd, kz) dkdt.
//   src/Targets/GenericMolecule.jl:236-259: the structure factor G.
//   src/ElectronSamplers/shared_methods.jl:15-38: solid harmonics and the
//     field-frame -> molecular-frame Euler angles.
//
// Layouts (all complex values as (re, im) pairs, Julia column-major arrays):
//   C_lm:     C[l + (m + l) (lmax + 1)]                      (MolAsympCoeff)
//   IntData:  I[nxi + (nxi_max+1) (m + m_max + (2 m_max+1) (l + (lmax+1) (m' + l)))]
//   Y prefactors:  P[l^2 + l + m']
//   per time sample, MO-ADK:  cd[e] = C_lm D^l_{m' m} for the e-th (l, m, m')
//                             with C_lm != 0, in lmm_list order
//   per time sample, WFAT:    g2[nxi + (m + m_max)(nxi_max+1)] = |G_{nxi m}|^2,
//                             A[nxi + |m| (nxi_max+1)] = the factors of W that
//                             depend on the time sample only
#ifndef ETRAJ_MOL_H
#define ETRAJ_MOL_H

#ifdef __CUDACC__
#define MOL_FN static __host__ __device__ __noinline__
#define MOL_INL static __host__ __device__ __forceinline__
#else
#define MOL_FN static
#define MOL_INL static inline
#endif

#define MOL_MAX_L 6
#define MOL_NLM ((MOL_MAX_L + 1) * (MOL_MAX_L + 1))        /* (l, m) pairs: 49 */
#define MOL_NCD 455                                         /* sum over l of (2l+1)^2 */
#define MOL_NCH ((MOL_MAX_L + 1) * (2 * MOL_MAX_L + 1))    /* WFAT channels: 91 */
#define MOL_NA ((MOL_MAX_L + 1) * (MOL_MAX_L + 1))          /* WFAT (n_xi, |m|) factors: 49 */

// The (l, m) pairs with C_lm != 0, in lmm_list order.  z[k] marks a run of
// pairs with C_lm == 0 just before pair k (tail: after the last one); those
// contribute the real 0.0 of `(C_lm == 0) && return 0.0` to the sum.
typedef struct {
    int n, ncd, tail, lmax;
    signed char l[MOL_NLM], m[MOL_NLM], z[MOL_NLM];
} mol_terms;

MOL_INL double mol_fact(int n) {
    double f = 1.0;
    for (int i = 2; i <= n; ++i) f *= (double)i;
    return f;
}

// x^n for n >= 0 as Julia's Float64^Integer evaluates it: power by squaring
// carried in double-double (Julia Base, math.jl `pow_body`), which keeps the
// result within about one rounding of the exact power.
MOL_INL double mol_powi(double x, int n) {
    if (n == 0) return 1.0;
    if (n == 3) return (x * x) * x;
    double y = 1.0, xnlo = 0.0, ynlo = 0.0;
    while (n > 1) {
        if (n & 1) {
            const double err = fma(y, xnlo, x * ynlo);
            const double hi = x * y, lo = fma(x, y, -hi);
            y = hi;
            ynlo = lo + err;
        }
        const double err = (x * 2.0) * xnlo;
        const double hi = x * x, lo = fma(x, x, -hi);
        x = hi;
        xnlo = lo + err;
        n >>= 1;
    }
    const double err = fma(y, xnlo, x * ynlo);
    return (!dm_isinf(x) && !dm_isnan(x) && !dm_isinf(err) && !dm_isnan(err)) ? fma(x, y, err) : x * y;
}

// n! for n <= 2 MOL_MAX_L, exact in double (the products mol_fact forms)
#define MOL_FACT_TABLE {1.0, 1.0, 2.0, 6.0, 24.0, 120.0, 720.0, 5040.0, 40320.0, 362880.0, 3628800.0, \
                        39916800.0, 479001600.0}

// d^j_{m'm}(beta) from (sin, cos) of beta/2, Wigner's explicit sum (standard
// convention); the powers are the running products cos^k = cos^(k-1) cos.
MOL_FN double mol_wigner_d_sc(int j, int mp, int m, double sh, double ch) {
    const double F[2 * MOL_MAX_L + 1] = MOL_FACT_TABLE;
    double cp[2 * MOL_MAX_L + 1], sp[2 * MOL_MAX_L + 1];
    cp[0] = 1.0;
    sp[0] = 1.0;
    for (int i = 1; i <= 2 * j; ++i) {
        cp[i] = cp[i - 1] * ch;
        sp[i] = sp[i - 1] * sh;
    }
    const double pref = sqrt(F[j + mp] * F[j - mp] * F[j + m] * F[j - m]);
    double sum = 0.0;
    for (int s = 0; s <= 2 * j; ++s) {
        const int a1 = j + m - s, a3 = mp - m + s, a4 = j - mp - s;
        if (a1 < 0 || a3 < 0 || a4 < 0) continue;
        const double den = F[a1] * F[s] * F[a3] * F[a4];
        const double sign = ((mp - m + s) & 1) ? -1.0 : 1.0;
        sum = sum + ((sign * pref / den) * cp[2 * j + m - mp - 2 * s]) * sp[mp - m + 2 * s];
    }
    return sum;
}

MOL_FN double mol_wigner_d(int j, int mp, int m, double beta) {
    double sh, ch;
    dm_sincos(0.5 * beta, &sh, &ch);
    return mol_wigner_d_sc(j, mp, m, sh, ch);
}

// D^l_{m' m}(a, b, g) = e^{-i m' a} d^l_{m' m}(b) e^{-i m g}
MOL_INL dm_cplx mol_wigner_D(int l, int mp, int m, double a, double b, double g) {
    double s1, c1, s3, c3;
    dm_sincos(-((double)mp * a), &s1, &c1);
    dm_sincos(-((double)m * g), &s3, &c3);
    const double d = mol_wigner_d(l, mp, m, b);
    return dm_cmul(dm_cscale(dm_c(c1, s1), d), dm_c(c3, s3));
}

MOL_INL void mol_rotzyz(double a, double b, double g, double R[3][3]) {
    double sa, ca, sb, cb, sg, cg;
    dm_sincos(a, &sa, &ca);
    dm_sincos(b, &sb, &cb);
    dm_sincos(g, &sg, &cg);
    R[0][0] = ca * cb * cg - sa * sg; R[0][1] = -(ca * cb * sg) - sa * cg; R[0][2] = ca * sb;
    R[1][0] = sa * cb * cg + ca * sg; R[1][1] = -(sa * cb * sg) + ca * cg; R[1][2] = sa * sb;
    R[2][0] = -(sb * cg);             R[2][1] = sb * sg;                   R[2][2] = cb;
}

// Euler angles (z-y'-z'') of the rotation from the field frame (F along z)
// to the molecular frame RotZYZ(rot) (obtain_FF_MF_Euler, shared_methods.jl:31-38).
MOL_FN void mol_euler(const double rot[3], double Fx, double Fy, double F, double* a, double* b, double* g) {
    const double FF[3][3] = {{0.0, Fy / F, Fx / F}, {0.0, -Fx / F, Fy / F}, {1.0, 0.0, 0.0}};
    double MF[3][3], M[3][3];
    mol_rotzyz(rot[0], rot[1], rot[2], MF);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) M[i][j] = (MF[0][i] * FF[0][j] + MF[1][i] * FF[1][j]) + MF[2][i] * FF[2][j];
    const double t1 = dm_atan2(M[1][2], M[0][2]);
    double st1, ct1;
    dm_sincos(t1, &st1, &ct1);
    *a = t1;
    *b = dm_atan2(M[0][2] * ct1 + M[1][2] * st1, M[2][2]);
    *g = dm_atan2(M[1][0] * ct1 - M[0][0] * st1, M[1][1] * ct1 - M[0][1] * st1);
}

// Prefactor of the solid harmonic Y_{l m} (shared_methods.jl:21):
// (-1)^m sqrt((2l+1)/4pi (l-m)!/(l+m)!) / (-i kappa)^l * (l+m)!.
MOL_INL dm_cplx mol_sph_prefactor(int l, int m, double kappa) {
    const double A = (m & 1) ? -1.0 : 1.0;
    const double B = sqrt((((2.0 * l + 1.0) / 12.566370614359172) * mol_fact(l - m)) / mol_fact(l + m));
    const dm_cplx C = dm_cpowi(dm_c(0.0, -kappa), l);
    const dm_cplx P = dm_cdiv(dm_c(A * B, 0.0), C);
    return dm_cscale(P, mol_fact(l + m));
}

// The k-sum of the solid harmonic (shared_methods.jl:21) at complex (x, y, z).
MOL_FN dm_cplx mol_sph_sum(int l, int m, dm_cplx x, dm_cplx y, dm_cplx z) {
    const dm_cplx xp = dm_c(x.re - y.im, x.im + y.re);  // x + i y
    const dm_cplx xm = dm_c(x.re + y.im, x.im - y.re);  // x - i y
    const int kmin = (m < 0) ? -m : 0, kmax = (l - m) / 2;
    dm_cplx acc = dm_c(0.0, 0.0);
    for (int k = kmin; k <= kmax; ++k) {
        const double den = mol_fact(k + m) * mol_fact(k) * mol_fact(l - m - 2 * k);
        double p2 = 1.0;
        for (int i = 0; i < 2 * k + m; ++i) p2 *= 2.0;
        const double coef = ((k & 1) ? -1.0 : 1.0) / (p2 * den);
        dm_cplx t = dm_cscale(dm_cpowi(xp, k + m), coef);
        t = dm_cmul(t, dm_cpowi(xm, k));
        t = dm_cmul(t, dm_cpowi(z, l - m - 2 * k));
        acc = (k == kmin) ? t : dm_cadd(acc, t);
    }
    return acc;
}

// ---- MO-ADK -----------------------------------------------------------------------
// Term list of a C_lm matrix (host side, once per job).
MOL_INL void mol_terms_build(int lmax, const double* clm, mol_terms* T) {
    T->n = 0;
    T->ncd = 0;
    T->tail = 0;
    T->lmax = lmax;
    int zero_run = 0;
    for (int l = 0; l <= lmax; ++l) {
        for (int m = -l; m <= l; ++m) {
            const int i = l + (m + l) * (lmax + 1);
            if (clm[2 * i] == 0.0 && clm[2 * i + 1] == 0.0) {
                zero_run = 1;
                continue;
            }
            T->l[T->n] = (signed char)l;
            T->m[T->n] = (signed char)m;
            T->z[T->n] = (signed char)zero_run;
            zero_run = 0;
            T->n += 1;
            T->ncd += 2 * l + 1;
        }
    }
    T->tail = zero_run;
}

// Entry e (0 <= e < ncd) of the per-time-sample table: C_lm D^l_{m' m}.
MOL_FN dm_cplx mol_cd_entry(const mol_terms* T, const double* clm, int e, double a, double b, double g) {
    int k = 0;
    while (e >= 2 * T->l[k] + 1) {
        e -= 2 * T->l[k] + 1;
        ++k;
    }
    const int l = T->l[k], m = T->m[k], mp = e - l;
    const int i = l + (m + l) * (T->lmax + 1);
    const dm_cplx C = dm_c(clm[2 * i], clm[2 * i + 1]);
    return dm_cmul(C, mol_wigner_D(l, mp, m, a, b, g));
}

// sum over (l, m, m') of C_lm D^l_{m' m} Y_{l m'}(nk) (the molecular
// pre_numerator, ADKSampler.jl:243-253), summed left to right as Julia's
// mapreduce does: pairs with C_lm == 0 add a real 0.0, which touches only
// the real part of the running sum.
MOL_FN dm_cplx mol_numerator(const mol_terms* T, const double* cd, const double* P, dm_cplx nkx, dm_cplx nky,
                             dm_cplx nkz) {
    double are = 0.0, aim = 0.0;
    int first = 1, first_im = 1, e = 0;
    dm_cplx Y[2 * MOL_MAX_L + 1];
    int ycur = -1;
    for (int k = 0; k < T->n; ++k) {
        const int l = T->l[k];
        if (T->z[k]) {
            are = first ? 0.0 : are + 0.0;
            first = 0;
        }
        if (l != ycur) {
            for (int mp = -l; mp <= l; ++mp) {
                const int pi = l * l + l + mp;
                Y[mp + l] = dm_cmul(dm_c(P[2 * pi], P[2 * pi + 1]), mol_sph_sum(l, mp, nkx, nky, nkz));
            }
            ycur = l;
        }
        for (int mp = -l; mp <= l; ++mp, ++e) {
            const dm_cplx t = dm_cmul(dm_c(cd[2 * e], cd[2 * e + 1]), Y[mp + l]);
            are = first ? t.re : are + t.re;
            aim = first_im ? t.im : aim + t.im;
            first = 0;
            first_im = 0;
        }
    }
    if (T->tail) are = first ? 0.0 : are + 0.0;
    return dm_c(are, aim);
}

// ---- WFAT ---------------------------------------------------------------------------
// G_{nxi m}(theta, chi) of MolWFATStructureFactor_G (GenericMolecule.jl:236-259):
// sum_{l=|m|..lmax} sum_{m'=-l..l} I[nxi, m, l, m'] d^l_{m m'}(theta) e^{-i m' chi},
// times exp(-kappa mu_z), mu_z = (RotZYZ(chi, theta, 0) mu)_z.
MOL_FN dm_cplx mol_wfat_G(int nxi, int m, int nxi_max, int m_max, int lmax, const double* I, const double mu[3],
                          double kappa, double theta, double chi) {
    dm_cplx sum = dm_c(0.0, 0.0);
    const int am = m < 0 ? -m : m;
    for (int l = am; l <= lmax; ++l) {
        for (int mp = -l; mp <= l; ++mp) {
            const long i = (long)nxi + (long)(nxi_max + 1) *
                                           ((long)(m + m_max) + (long)(2 * m_max + 1) *
                                                                    ((long)l + (long)(lmax + 1) * (long)(mp + l)));
            const dm_cplx v = dm_c(I[2 * i], I[2 * i + 1]);
            double s, c;
            dm_sincos(-((double)mp) * chi, &s, &c);
            const dm_cplx t = dm_cmul(dm_cscale(v, mol_wigner_d(l, m, mp, theta)), dm_c(c, s));
            sum = dm_cadd(sum, t);
        }
    }
    double R[3][3];
    mol_rotzyz(chi, theta, 0.0, R);
    const double muz = (R[2][0] * mu[0] + R[2][1] * mu[1]) + R[2][2] * mu[2];
    return dm_cscale(sum, dm_exp(-kappa * muz));
}

// mol_wfat_G with its Wigner d values and phase factors taken from tables:
// d[(l (2L+1) + m + L)(2L+1) + m' + L] = d^l_{m m'}(theta) and
// cs[2 (m' + L)] = (cos, sin) of -m' chi, L = MOL_MAX_L; the same values and
// the same sum as mol_wfat_G (the tables are filled by mol_wigner_d and
// dm_sincos with the same arguments).
MOL_FN dm_cplx mol_wfat_G_tab(int nxi, int m, int nxi_max, int m_max, int lmax, const double* I, const double mu[3],
                              double kappa, double theta, double chi, const double* d, const double* cs) {
    const int L = MOL_MAX_L, W = 2 * MOL_MAX_L + 1;
    dm_cplx sum = dm_c(0.0, 0.0);
    const int am = m < 0 ? -m : m;
    for (int l = am; l <= lmax; ++l) {
        for (int mp = -l; mp <= l; ++mp) {
            const long i = (long)nxi + (long)(nxi_max + 1) *
                                           ((long)(m + m_max) + (long)(2 * m_max + 1) *
                                                                    ((long)l + (long)(lmax + 1) * (long)(mp + l)));
            const dm_cplx v = dm_c(I[2 * i], I[2 * i + 1]);
            const double dv = d[(l * W + m + L) * W + mp + L];
            const dm_cplx t = dm_cmul(dm_cscale(v, dv), dm_c(cs[2 * (mp + L)], cs[2 * (mp + L) + 1]));
            sum = dm_cadd(sum, t);
        }
    }
    double R[3][3];
    mol_rotzyz(chi, theta, 0.0, R);
    const double muz = (R[2][0] * mu[0] + R[2][1] * mu[1]) + R[2][2] * mu[2];
    return dm_cscale(sum, dm_exp(-kappa * muz));
}

// |G|^2 of channel ch (= nxi + (m + m_max)(nxi_max+1)) at the time sample's
// Euler angles (beta, gamma).
MOL_FN double mol_wfat_g2(int ch, int nxi_max, int m_max, int lmax, const double* I, const double mu[3],
                          double kappa, double beta, double gamma) {
    const int nxi = ch % (nxi_max + 1), m = ch / (nxi_max + 1) - m_max;
    const dm_cplx G = mol_wfat_G(nxi, m, nxi_max, m_max, lmax, I, mu, kappa, beta, gamma);
    return G.re * G.re + G.im * G.im;
}

// The factors of W_{nxi |m|} (WFATSampler.jl:157) that depend on the time
// sample only: (kappa^(|m|+2)/2/F^(|m|+1)/|m|!) (4 kappa^2/F)^(2n - 2nxi - |m| - 1).
MOL_FN double mol_wfat_A(int e, int nxi_max, double kappa, double nstar, double F) {
    const int nxi = e % (nxi_max + 1), am = e / (nxi_max + 1);
    const double x1 = ((mol_powi(kappa, am + 2) / 2.0) / mol_powi(F, am + 1)) / mol_fact(am);
    const double ex = ((2.0 * nstar - (double)(2 * nxi)) - (double)am) - 1.0;
    const double x2 = dm_pow_pos((4.0 * (kappa * kappa)) / F, ex);
    return x1 * x2;
}

// The WFAT rate of one candidate (WFATSampler.jl:169): the channels in the
// order of [(nxi, m) for nxi in 0:nxi_max, m in -m_max:m_max] (nxi fastest),
// summed left to right, times dkdt.
MOL_FN double mol_wfat_rate(int nxi_max, int m_max, const double* g2, const double* A, double kappa, double F,
                            double kd, double kz, double dkdt) {
    const double k2 = kd * kd + kz * kz;
    const double X = (kappa * kappa + kd * kd) + kz * kz;
    const double E = dm_exp(((-2.0) * (X * sqrt(X))) / (3.0 * F));
    double K[MOL_MAX_L + 1];
    for (int a = 0; a <= m_max; ++a) K[a] = mol_powi(k2, a);
    double sum = 0.0;
    int first = 1;
    for (int m = -m_max; m <= m_max; ++m) {
        const int am = m < 0 ? -m : m;
        for (int nxi = 0; nxi <= nxi_max; ++nxi) {
            const double W = (A[nxi + am * (nxi_max + 1)] * K[am]) * E;
            const double t = g2[nxi + (m + m_max) * (nxi_max + 1)] * W;
            sum = first ? t : sum + t;
            first = 0;
        }
    }
    return sum * dkdt;
}

#endif
