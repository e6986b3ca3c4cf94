"""ctypes mirror of include/etraj.h and the loader of the CUDA library.

The structures below must match include/etraj.h field for field; the test
suite checks their sizes against the library's own sizeof values.
"""
import ctypes as C
import os

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(PKG_DIR, "lib")
LIB_PATH = os.path.join(LIB_DIR, "libetraj_gb300.so")

# status codes (etraj_status)
OK = 0
ERR_INVALID_ARGUMENT = 1
ERR_UNSUPPORTED = 2
ERR_CUDA = 3
ERR_OUT_OF_MEMORY = 4
ERR_TIMEOUT = 5
ERR_NOT_READY = 6
ERR_NOT_FOUND = 7

LASER_COS4, LASER_COS2, LASER_GAUSSIAN, LASER_BICHROMATIC = 0, 1, 2, 3
TARGET_HYDROGEN_LIKE, TARGET_SAE, TARGET_MOLECULE = 0, 1, 2
MOL_MAX_L = 6
SAMPLER_ADK, SAMPLER_SPANE, SAMPLER_SPA, SAMPLER_WFAT = 0, 1, 2, 3
PREFIX_PRE, PREFIX_PRECC, PREFIX_JAC = 1, 2, 4
PHASE_CTMC, PHASE_QTMC, PHASE_SCTS = 0, 1, 2
PRECISION_FP64, PRECISION_FP32_BULK, PRECISION_FP32_DF = 0, 1, 2
PROPOSAL_UNIFORM, PROPOSAL_ADK_GAUSS = 0, 1


class MonoLaser(C.Structure):
    _fields_ = [("kind", C.c_int32), ("reserved", C.c_int32),
                ("peak_int", C.c_double), ("wave_len", C.c_double), ("cyc_num", C.c_double),
                ("ellip", C.c_double), ("azi", C.c_double), ("cep", C.c_double),
                ("t_shift", C.c_double)]


class Laser(C.Structure):
    _fields_ = [("kind", C.c_int32), ("reserved", C.c_int32),
                ("mono", MonoLaser * 2), ("delay", C.c_double)]


class Target(C.Structure):
    _fields_ = [("kind", C.c_int32), ("Z", C.c_int32), ("l", C.c_int32), ("m", C.c_int32),
                ("Ip", C.c_double), ("asymp_coeff", C.c_double),
                ("quan_ax_theta", C.c_double), ("quan_ax_phi", C.c_double),
                ("a1", C.c_double), ("b1", C.c_double), ("a2", C.c_double),
                ("b2", C.c_double), ("a3", C.c_double), ("b3", C.c_double),
                ("soft_core", C.c_double),
                ("mol_rot", C.c_double * 3), ("mol_Ip_traj", C.c_double),
                ("asymp_lmax", C.c_int32), ("wfat_nxi_max", C.c_int32), ("wfat_m_max", C.c_int32),
                ("wfat_lmax", C.c_int32),
                ("asymp_coeff_lm", C.POINTER(C.c_double)), ("wfat_intdata", C.POINTER(C.c_double)),
                ("wfat_mu", C.c_double * 3)]


class Job(C.Structure):
    _fields_ = [("init_cond_method", C.c_int32), ("dimension", C.c_int32),
                ("sample_monte_carlo", C.c_int32), ("rate_prefix", C.c_int32),
                ("traj_phase_method", C.c_int32), ("precision", C.c_int32),
                ("sample_t_intv", C.c_double * 2), ("sample_t_num", C.c_int64),
                ("traj_t_final", C.c_double), ("traj_rtol", C.c_double),
                ("final_p_max", C.c_double * 3), ("final_p_num", C.c_int64 * 3),
                ("ss_kd_max", C.c_double), ("ss_kd_num", C.c_int64),
                ("ss_kz_max", C.c_double), ("ss_kz_num", C.c_int64),
                ("mc_kt_num", C.c_int64), ("mc_kd_max", C.c_double), ("mc_kz_max", C.c_double),
                ("sample_cutoff_limit", C.c_double), ("seed", C.c_uint64),
                ("laser", Laser), ("target", Target), ("mc_kt_proposal", C.c_int32), ("reserved2", C.c_int32)]

    @property
    def rows(self):
        """Rows of the reference's `init` matrix (ADKSampler.jl:299-303)."""
        base = 8 if self.dimension == 3 else 6
        return base + (0 if self.traj_phase_method == PHASE_CTMC else 1)

    @property
    def state_size(self):
        """Size of the ODE state (TrajectorySimulation.jl:324 / :419)."""
        base = 6 if self.dimension == 3 else 4
        return base + (0 if self.traj_phase_method == PHASE_CTMC else 1)

    @property
    def grid_size(self):
        g = 1
        for d in range(self.dimension):
            g *= self.final_p_num[d]
        return g

    def copy(self):
        j = Job()
        C.pointer(j)[0] = self
        keep = getattr(self, "_keep", None)
        if keep is not None:
            j._keep = keep  # arrays the target's pointers refer to
        return j


class Result(C.Structure):
    _fields_ = [("momentum_spec", C.POINTER(C.c_double)), ("amplitude", C.POINTER(C.c_double)),
                ("ion_prob", C.c_double), ("ion_prob_uncollected", C.c_double),
                ("num_effective_traj", C.c_int64), ("num_failed_traj", C.c_int64),
                ("num_ionized_traj", C.c_int64), ("num_steps", C.c_int64),
                ("num_kernel_launches", C.c_int64), ("elapsed_ms", C.c_double)]


# (name, restype, argtypes) of every entry point declared in include/etraj.h
_DP = C.POINTER(C.c_double)
_I32P = C.POINTER(C.c_int32)
_I64P = C.POINTER(C.c_int64)
SIGNATURES = [
    ("etraj_version", C.c_char_p, []),
    ("etraj_create", C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.c_size_t]),
    ("etraj_destroy", None, [C.c_void_p]),
    ("etraj_last_error", C.c_char_p, [C.c_void_p]),
    ("etraj_set_stream", C.c_int, [C.c_void_p, C.c_void_p]),
    ("etraj_validate", C.c_int, [C.POINTER(Job), C.c_char_p, C.c_size_t]),
    ("etraj_run", C.c_int, [C.c_void_p, C.POINTER(Job), C.POINTER(Result)]),
    ("etraj_batch_info", C.c_int, [C.POINTER(Job), _I64P, _I64P]),
    ("etraj_sample_batch", C.c_int, [C.c_void_p, C.POINTER(Job), C.c_int64, _DP, C.c_int64, _I64P]),
    ("etraj_sample_all", C.c_int, [C.c_void_p, C.POINTER(Job), _DP, C.c_int64, _I64P]),
    ("etraj_integrate", C.c_int, [C.c_void_p, C.POINTER(Job), C.c_int64, _DP, _DP, _I32P, _I32P]),
    ("etraj_submit", C.c_int, [C.c_void_p, C.POINTER(Job), C.POINTER(Result), C.POINTER(C.c_uint64)]),
    ("etraj_poll", C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(Result)]),
    ("etraj_wait", C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(Result)]),
    ("etraj_run_batch", C.c_int, [C.c_void_p, C.POINTER(Job), C.c_int, C.POINTER(Result), _DP, _DP]),
    ("etraj_server_create", C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.c_int, C.c_size_t]),
    ("etraj_server_destroy", None, [C.c_void_p]),
    ("etraj_server_submit", C.c_int, [C.c_void_p, C.POINTER(Job), C.POINTER(Result), C.POINTER(C.c_uint64)]),
    ("etraj_server_poll", C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(Result)]),
    ("etraj_server_wait", C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(Result), C.c_double]),
    ("etraj_server_stats", C.c_int, [C.c_void_p, _I64P, _I64P, C.POINTER(C.c_size_t)]),
    ("etraj_server_last_error", C.c_char_p, [C.c_void_p]),
    ("etraj_set_graphs", C.c_int, [C.c_void_p, C.c_int]),
    ("etraj_set_autotune", C.c_int, [C.c_void_p, C.c_int]),
    ("etraj_bulk_tile", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, _I32P, _I32P, _I32P]),
    ("etraj_set_bulk_tile", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                      C.c_int]),
    ("etraj_bulk_step_chunk", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int)]),
    ("etraj_set_bulk_step_chunk", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]),
    ("etraj_set_straggler_repack", C.c_int, [C.c_void_p, C.c_int]),
    ("etraj_set_static_assignment", C.c_int, [C.c_void_p, C.c_int]),
    ("etraj_set_keep_final_states", C.c_int, [C.c_void_p, C.c_int]),
    ("etraj_dump_final_states", C.c_int, [C.c_void_p, C.c_uint64, _DP, _DP, _I32P]),
    ("etraj_dump_step_counts", C.c_int, [C.c_void_p, C.c_uint64, _I32P]),
    ("etraj_dump_min_radius", C.c_int, [C.c_void_p, C.c_uint64, _DP]),
    ("etraj_stage_times", C.c_int, [C.c_void_p, _DP, C.c_int]),
    ("etraj_deposit_noalloc", C.c_int, [C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64,
                                        C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
]

_lib = None


def load_library(path=None):
    """Load libetraj_gb300.so.  Raises if it has not been built: there is no
    CPU fallback for the trajectory path."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(
            "libetraj_gb300.so is not built (%s); run __graft_entry__.build() first" % p)
    lib = C.CDLL(p)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def dptr(a):
    """double* of a contiguous float64 numpy array (or NULL for None)."""
    if a is None:
        return None
    return a.ctypes.data_as(_DP)


def i32ptr(a):
    if a is None:
        return None
    return a.ctypes.data_as(_I32P)
