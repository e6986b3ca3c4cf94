/* mol_check.h -- the target checks of the samplers' constructors for
 * molecular targets and for WFAT, shared by the library's host validation and
 * the CPU oracle.  Needs etraj.h.
 *
 * Reference: src/ElectronSamplers/ADKSampler.jl:107-114, SPANESampler.jl:79-86,
 * SPASampler.jl:107-114 (molecules: asymptotic coefficients present, Ip > 0),
 * WFATSampler.jl:36-41,76-81 (CTMC only, molecular targets only, WFAT data
 * present, Ip > 0).  Where the reference would run its molecular calculator
 * (MolCalcAsympCoeff!, MolCalcWFATData!) to fill missing data, this engine
 * has none and reports ETRAJ_ERR_UNSUPPORTED.
 *
 * Returns ETRAJ_OK, or a status with *msg set; -1 means "not a molecular or
 * WFAT job, apply the atom checks". */
#ifndef ETRAJ_MOL_CHECK_H
#define ETRAJ_MOL_CHECK_H

static inline int etraj_mol_check(const etraj_job* job, const char** msg) {
    const etraj_target* T = &job->target;
    const int wfat = (job->init_cond_method == ETRAJ_SAMPLER_WFAT);
    if (T->kind != ETRAJ_TARGET_MOLECULE) {
        if (wfat) {
            *msg = "[WFATSampler] The WFAT sampler supports molecular targets only.";
            return ETRAJ_ERR_INVALID_ARGUMENT;
        }
        return -1;
    }
    if (wfat && job->traj_phase_method != ETRAJ_PHASE_CTMC) {
        *msg = "[WFATSampler] Unsupported phase method.";
        return ETRAJ_ERR_INVALID_ARGUMENT;
    }
    if (!(T->Ip > 0)) {
        *msg = wfat ? "[WFATSampler] The energy of the ionizing orbit is non-negative."
                    : "[ADKSampler] The energy of the ionizing orbital of the molecule target is non-negative.";
        return ETRAJ_ERR_INVALID_ARGUMENT;
    }
    if (!(T->mol_Ip_traj > 0)) {
        *msg = "[GenericMolecule] The molecule's ionization potential must be positive.";
        return ETRAJ_ERR_INVALID_ARGUMENT;
    }
    if (T->Z < 1) {
        *msg = "[GenericMolecule] The asymptotic charge (charge + 1) must be positive.";
        return ETRAJ_ERR_INVALID_ARGUMENT;
    }
    if (wfat) {
        if (!T->wfat_intdata) {
            *msg = "[GenericMolecule] The WFAT data of the ionizing orbital is not available; computing it needs "
                   "a molecular calculator, which this engine does not have.";
            return ETRAJ_ERR_UNSUPPORTED;
        }
        if (T->wfat_nxi_max < 0 || T->wfat_m_max < 0 || T->wfat_lmax < 0 || T->wfat_nxi_max > ETRAJ_MOL_MAX_L ||
            T->wfat_m_max > ETRAJ_MOL_MAX_L || T->wfat_lmax > ETRAJ_MOL_MAX_L) {
            *msg = "WFAT channels and integrals beyond n_xi, |m|, l = 6 are not supported.";
            return ETRAJ_ERR_UNSUPPORTED;
        }
    } else {
        if (!T->asymp_coeff_lm) {
            *msg = "[GenericMolecule] The asymptotic coefficient of the ionizing orbital is not available; "
                   "computing it needs a molecular calculator, which this engine does not have.";
            return ETRAJ_ERR_UNSUPPORTED;
        }
        if (T->asymp_lmax < 0 || T->asymp_lmax > ETRAJ_MOL_MAX_L) {
            *msg = "asymptotic coefficients beyond l = 6 are not supported.";
            return ETRAJ_ERR_UNSUPPORTED;
        }
    }
    return ETRAJ_OK;
}

#endif
