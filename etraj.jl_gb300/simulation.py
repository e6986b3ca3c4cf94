"""perform_traj_simulation: the reference's keyword API over the C ABI.

Mirrors src/TrajectorySimulation.jl:103-161 (keywords, defaults and
checks).  The batch loop at :154-157 becomes one etraj_run call on the GPU;
there is no CPU path.  Output: the result is returned as a dict with the keys
of the reference's output file (px, py[, pz], momentum_spec, ion_prob,
ion_prob_uncollected, num_effective_traj, params_text) and, when output_path
is given, written as that JLD2 or HDF5 file (h5write.py) or a NumPy .npz.
"""
import ctypes as C
import math
import warnings

import numpy as np

from . import abi
from .lasers import Laser, MonochromaticLaser, BichromaticLaser
from .targets import Target, SAEAtomBase, MoleculeBase

# init_sampler's method names and aliases (ElectronSamplers.jl:11-24)
_METHODS = {"ADK": abi.SAMPLER_ADK, "MOADK": abi.SAMPLER_ADK,
            "SPANE": abi.SAMPLER_SPANE, "SFAAE": abi.SAMPLER_SPANE, "MOSPANE": abi.SAMPLER_SPANE,
            "MOSFAAE": abi.SAMPLER_SPANE,
            "SPA": abi.SAMPLER_SPA, "SFA": abi.SAMPLER_SPA, "MOSPA": abi.SAMPLER_SPA, "MOSFA": abi.SAMPLER_SPA,
            "WFAT": abi.SAMPLER_WFAT}
_PHASES = {"CTMC": abi.PHASE_CTMC, "QTMC": abi.PHASE_QTMC, "SCTS": abi.PHASE_SCTS}
_PREFIX_BITS = {"Pre": abi.PREFIX_PRE, "PreCC": abi.PREFIX_PRECC, "Jac": abi.PREFIX_JAC}
_PRECISIONS = {"fp64": abi.PRECISION_FP64, "fp32_bulk": abi.PRECISION_FP32_BULK, "fp32_df": abi.PRECISION_FP32_DF}


def _sym(x):
    return x[1:] if isinstance(x, str) and x.startswith(":") else x


def rate_prefix_bits(rate_prefix):
    """:Exp, :Full, :Pre, :PreCC, :Jac or a collection of them -> ETRAJ_PREFIX_* mask
    (ADKSampler.jl:49-77)."""
    if isinstance(rate_prefix, str):
        p = _sym(rate_prefix)
        if p == "Exp":
            return 0
        if p == "Full":
            return abi.PREFIX_PRECC | abi.PREFIX_JAC
        if p in _PREFIX_BITS:
            return _PREFIX_BITS[p]
        raise ValueError("[ADKSampler] Undefined tunneling rate prefix [%s]." % p)
    items = [_sym(p) for p in rate_prefix]
    if not all(p in _PREFIX_BITS for p in items):
        raise ValueError("[ADKSampler] Undefined tunneling rate prefix [%s]." % (items,))
    if "Pre" in items and "PreCC" in items:
        raise ValueError("[ADKSampler] Rate prefixes [Pre] & [PreCC] conflict.")
    bits = 0
    for p in items:
        bits |= _PREFIX_BITS[p]
    return bits


def make_job(*, init_cond_method, laser, target, dimension, sample_t_intv, sample_t_num,
             traj_t_final, final_p_max, final_p_num, ss_kd_max=0.0, ss_kd_num=0, ss_kz_max=0.0,
             ss_kz_num=0, mc_kt_num=0, mc_kd_max=0.0, mc_kz_max=0.0, traj_phase_method="CTMC",
             traj_rtol=1e-6, sample_monte_carlo=False, sample_cutoff_limit=1e-16,
             rate_prefix="Full", mol_orbit_ridx=0, precision="fp64", seed=0, mc_kt_proposal="uniform"):
    """Checks the keywords as TrajectorySimulationJob (TrajectorySimulation.jl:164-298) and
    the sampler constructors do, and packs them into an etraj_job.  mc_kt_proposal
    ("uniform", the reference's, or "adk_gauss": normal transverse momenta of the
    ADK width with importance weights) applies to Monte-Carlo ADK and SPANE."""
    method = _sym(init_cond_method)
    if method not in _METHODS:
        raise ValueError("[ElectronSamplers] Undefined initial condition method [%s]." % method)
    if not isinstance(laser, Laser):
        raise TypeError("`laser` must be a Laser.")
    if not isinstance(target, (SAEAtomBase, MoleculeBase)):
        raise TypeError("`target` must be an atom (HydrogenLikeAtom, SAEAtom) or a molecule (GenericMolecule).")
    if method == "WFAT" and not isinstance(target, MoleculeBase):
        raise TypeError("[WFATSampler] The WFAT sampler supports molecular targets only.")
    phase = _sym(traj_phase_method)
    if phase not in _PHASES:
        raise ValueError("[ADKSampler] Undefined phase method [%s]." % phase)
    if method == "WFAT" and phase != "CTMC":
        raise ValueError("[WFATSampler] Unsupported phase method [%s]." % phase)
    assert sample_t_intv[0] < sample_t_intv[1], \
        "[TrajectorySimulationJob] `sample_t_intv` must be a valid interval."
    assert traj_t_final > sample_t_intv[1], \
        "[TrajectorySimulationJob] `traj_t_final` must be greater than the last time point of `sample_t_intv`."
    assert dimension in (2, 3), "[TrajectorySimulationJob] `dimension` must be either 2 or 3."
    assert len(final_p_max) == len(final_p_num) == dimension, \
        "[TrajectorySimulationJob] `length(final_p_max)` and `length(final_p_num)` should match `dimension`."
    bits = rate_prefix_bits(rate_prefix)
    if (bits & abi.PREFIX_PRECC) and isinstance(laser, BichromaticLaser):
        warnings.warn("[ADKSampler] Laser is not monochromatic, Coulomb correction in rate prefix is unavailable.")
    j = abi.Job()
    j.init_cond_method = _METHODS[method]
    j.dimension = dimension
    j.sample_monte_carlo = 1 if sample_monte_carlo else 0
    j.rate_prefix = bits
    j.traj_phase_method = _PHASES[phase]
    j.precision = _PRECISIONS[precision]
    j.sample_t_intv[0], j.sample_t_intv[1] = float(sample_t_intv[0]), float(sample_t_intv[1])
    j.sample_t_num = int(sample_t_num)
    j.traj_t_final = float(traj_t_final)
    j.traj_rtol = float(traj_rtol)
    for d in range(3):
        j.final_p_max[d] = float(final_p_max[d]) if d < dimension else 0.0
        j.final_p_num[d] = int(final_p_num[d]) if d < dimension else 1
    j.ss_kd_max, j.ss_kd_num = float(ss_kd_max), int(ss_kd_num)
    j.ss_kz_max, j.ss_kz_num = float(ss_kz_max), int(ss_kz_num)
    j.mc_kt_num, j.mc_kd_max, j.mc_kz_max = int(mc_kt_num), float(mc_kd_max), float(mc_kz_max)
    j.sample_cutoff_limit = float(sample_cutoff_limit)
    j.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
    proposals = {"uniform": abi.PROPOSAL_UNIFORM, "adk_gauss": abi.PROPOSAL_ADK_GAUSS}
    if _sym(mc_kt_proposal) not in proposals:
        raise ValueError("`mc_kt_proposal` must be \"uniform\" or \"adk_gauss\".")
    j.mc_kt_proposal = proposals[_sym(mc_kt_proposal)]
    j.laser = laser.to_c()
    if isinstance(target, MoleculeBase):
        j.target, keep = target.to_c(orbit_ridx=mol_orbit_ridx, wfat=(method == "WFAT"))
        j._keep = keep  # the arrays behind the target's pointers
    else:
        j.target = target.to_c()
    return j


class EtrajError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("etraj status %d: %s" % (status, message))
        self.status = status


class Engine:
    """One etraj_ctx: a device, its buffers and its stream."""

    def __init__(self, device=0, hbm_budget_bytes=0):
        self.lib = abi.load_library()
        self.ctx = C.c_void_p()
        st = self.lib.etraj_create(C.byref(self.ctx), device, hbm_budget_bytes)
        if st != abi.OK:
            raise EtrajError(st, "etraj_create failed on device %d" % device)

    def close(self):
        if self.ctx:
            self.lib.etraj_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st):
        if st != abi.OK:
            msg = self.lib.etraj_last_error(self.ctx)
            raise EtrajError(st, msg.decode() if msg else "")

    def set_stream(self, stream_handle):
        self._check(self.lib.etraj_set_stream(self.ctx, C.c_void_p(stream_handle or 0)))

    def run(self, job, want_spectrum=True, want_amplitude=False):
        res = abi.Result()
        spec = amp = None
        if want_spectrum:
            spec = np.zeros(job.grid_size, dtype=np.float64)
            res.momentum_spec = abi.dptr(spec)
        if want_amplitude and job.traj_phase_method != abi.PHASE_CTMC:
            amp = np.zeros(2 * job.grid_size, dtype=np.float64)
            res.amplitude = abi.dptr(amp)
        self._check(self.lib.etraj_run(self.ctx, C.byref(job), C.byref(res)))
        return res, spec, amp

    def batch_info(self, job):
        nb, mx = C.c_int64(), C.c_int64()
        self._check(self.lib.etraj_batch_info(C.byref(job), C.byref(nb), C.byref(mx)))
        return nb.value, mx.value

    def sample_batch(self, job, batch_id):
        """gen_electron_batch(sp, batch_id): (rows, count) matrix, or None when empty."""
        _, mx = self.batch_info(job)
        buf = np.zeros(job.rows * max(mx, 1), dtype=np.float64)
        n = C.c_int64()
        self._check(self.lib.etraj_sample_batch(self.ctx, C.byref(job), batch_id, abi.dptr(buf), mx,
                                                C.byref(n)))
        if n.value == 0:
            return None
        return buf[: job.rows * n.value].reshape(n.value, job.rows).T

    def sample_all(self, job):
        nb, mx = self.batch_info(job)
        cap = nb * mx
        buf = np.zeros(job.rows * max(cap, 1), dtype=np.float64)
        n = C.c_int64()
        self._check(self.lib.etraj_sample_all(self.ctx, C.byref(job), abi.dptr(buf), cap, C.byref(n)))
        return buf[: job.rows * n.value].reshape(n.value, job.rows)

    def integrate(self, job, init):
        """init: (n, rows) float64 -> (final (n, state), status (n,), steps (n,))."""
        init = np.ascontiguousarray(init, dtype=np.float64)
        n = init.shape[0]
        fin = np.zeros((n, job.state_size), dtype=np.float64)
        status = np.zeros(n, dtype=np.int32)
        steps = np.zeros(n, dtype=np.int32)
        self._check(self.lib.etraj_integrate(self.ctx, C.byref(job), n, abi.dptr(init), abi.dptr(fin),
                                             abi.i32ptr(status), abi.i32ptr(steps)))
        return fin, status, steps

    def set_graphs(self, enable):
        self._check(self.lib.etraj_set_graphs(self.ctx, 1 if enable else 0))

    def set_autotune(self, enable):
        self._check(self.lib.etraj_set_autotune(self.ctx, 1 if enable else 0))

    def bulk_tile(self, dimension, phase, target, multi=False):
        """(threads, blocks_per_sm, refill_min, tuned) of a bulk-integrator variant."""
        t, b, r = C.c_int32(), C.c_int32(), C.c_int32()
        st = self.lib.etraj_bulk_tile(self.ctx, dimension, phase, target, 1 if multi else 0, C.byref(t),
                                      C.byref(b), C.byref(r))
        if st not in (abi.OK, abi.ERR_NOT_FOUND):
            self._check(st)
        return t.value, b.value, r.value, st == abi.OK

    def set_static_assignment(self, enable):
        """Bulk path: one electron per lane and no work stealing (for comparison)."""
        self._check(self.lib.etraj_set_static_assignment(self.ctx, 1 if enable else 0))

    def set_straggler_repack(self, enable):
        """Bulk path: run the integrator in rounds that repack long-running electrons."""
        self._check(self.lib.etraj_set_straggler_repack(self.ctx, 1 if enable else 0))

    def keep_final_states(self, enable=True):
        """Keep per-survivor final states of the following jobs (dump_final_states)."""
        self._check(self.lib.etraj_set_keep_final_states(self.ctx, 1 if enable else 0))

    def dump_final_states(self, n, ticket=0):
        """(p_inf (n, 3), phase (n,), status (n,)) of the last job's n survivors;
        status = retcode | 0x100 when ionized."""
        p = np.zeros((n, 3))
        ph = np.zeros(n)
        st = np.zeros(n, dtype=np.int32)
        self._check(self.lib.etraj_dump_final_states(self.ctx, ticket, abi.dptr(p), abi.dptr(ph),
                                                     st.ctypes.data_as(C.POINTER(C.c_int32))))
        return p, ph, st

    def dump_step_counts(self, n, ticket=0):
        steps = np.zeros(n, dtype=np.int32)
        self._check(self.lib.etraj_dump_step_counts(self.ctx, ticket, steps.ctypes.data_as(C.POINTER(C.c_int32))))
        return steps

    def dump_min_radius(self, n, ticket=0):
        """Least |r| of each of the last FP64-path job's n survivors (initial state
        and the end of every accepted step)."""
        r = np.zeros(n)
        self._check(self.lib.etraj_dump_min_radius(self.ctx, ticket, abi.dptr(r)))
        return r

    def set_bulk_tile(self, dimension, phase, target, threads, blocks_per_sm, refill_min, multi=False):
        """Pin a bulk-integrator variant's launch shape on this engine."""
        self._check(self.lib.etraj_set_bulk_tile(self.ctx, dimension, phase, target, 1 if multi else 0,
                                                 threads, blocks_per_sm, refill_min))

    def bulk_step_chunk(self, dimension, phase, target, multi=False):
        """(steps, tuned): the step budget of the bulk integrator's first round."""
        v = C.c_int32()
        st = self.lib.etraj_bulk_step_chunk(self.ctx, dimension, phase, target, 1 if multi else 0, C.byref(v))
        if st not in (abi.OK, abi.ERR_NOT_FOUND):
            self._check(st)
        return v.value, st == abi.OK

    def set_bulk_step_chunk(self, dimension, phase, target, steps, multi=False):
        """Pin the step budget of the bulk integrator's first round on this engine."""
        self._check(self.lib.etraj_set_bulk_step_chunk(self.ctx, dimension, phase, target, 1 if multi else 0,
                                                       steps))

    def run_batch(self, jobs, want_spectrum=True, want_amplitude=False, weights=None):
        """Run up to 64 FP32-bulk jobs (same dimension, phase, rtol, target and grid)
        as one batch; returns [(result, spectrum, amplitude)] and, with `weights`,
        the weighted sum of the spectra."""
        n = len(jobs)
        arr = (abi.Job * n)(*jobs)
        res = (abi.Result * n)()
        outs = []
        for i, job in enumerate(jobs):
            spec = amp = None
            if want_spectrum:
                spec = np.zeros(job.grid_size, dtype=np.float64)
                res[i].momentum_spec = abi.dptr(spec)
            if want_amplitude and job.traj_phase_method != abi.PHASE_CTMC:
                amp = np.zeros(2 * job.grid_size, dtype=np.float64)
                res[i].amplitude = abi.dptr(amp)
            outs.append((spec, amp))
        w = wout = None
        if weights is not None:
            w = np.ascontiguousarray(weights, dtype=np.float64)
            assert w.size == n
            wout = np.zeros(jobs[0].grid_size, dtype=np.float64)
        self._check(self.lib.etraj_run_batch(self.ctx, arr, n, res, abi.dptr(w), abi.dptr(wout)))
        return [(res[i], outs[i][0], outs[i][1]) for i in range(n)], wout

    def submit(self, job, res):
        """Queue `job`; `res` (an abi.Result) carries the output pointers, which must stay
        valid until poll/wait reports the ticket done."""
        t = C.c_uint64()
        self._check(self.lib.etraj_submit(self.ctx, C.byref(job), C.byref(res), C.byref(t)))
        return t.value

    def poll(self, ticket, res):
        st = self.lib.etraj_poll(self.ctx, ticket, C.byref(res))
        if st == abi.ERR_NOT_READY:
            return False
        self._check(st)
        return True

    def wait(self, ticket, res):
        self._check(self.lib.etraj_wait(self.ctx, ticket, C.byref(res)))


class Server:
    """An etraj_server: continuous batching of many jobs on one GPU.  Jobs are
    queued first-in first-out and admitted to `slots` contexts (own stream, own
    buffers) as slots and HBM free up; their work overlaps on the device."""

    def __init__(self, device=0, slots=4, hbm_budget_bytes=0):
        self.lib = abi.load_library()
        self.srv = C.c_void_p()
        st = self.lib.etraj_server_create(C.byref(self.srv), device, slots, hbm_budget_bytes)
        if st != abi.OK:
            raise EtrajError(st, "etraj_server_create failed on device %d" % device)
        self._pending = {}

    def close(self):
        if self.srv:
            self.lib.etraj_server_destroy(self.srv)
            self.srv = C.c_void_p()
            self._pending.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st):
        if st != abi.OK:
            msg = self.lib.etraj_server_last_error(self.srv)
            raise EtrajError(st, msg.decode() if msg else "")

    def submit(self, job, want_spectrum=True, want_amplitude=False):
        """Queue a copy of `job`; returns its ticket.  The output arrays are held
        here until the ticket is retired by poll or wait."""
        res = abi.Result()
        spec = amp = None
        if want_spectrum:
            spec = np.zeros(job.grid_size, dtype=np.float64)
            res.momentum_spec = abi.dptr(spec)
        if want_amplitude and job.traj_phase_method != abi.PHASE_CTMC:
            amp = np.zeros(2 * job.grid_size, dtype=np.float64)
            res.amplitude = abi.dptr(amp)
        t = C.c_uint64()
        self._check(self.lib.etraj_server_submit(self.srv, C.byref(job), C.byref(res), C.byref(t)))
        self._pending[t.value] = (res, spec, amp)
        return t.value

    def _finish(self, ticket, st):
        res, spec, amp = self._pending.pop(ticket)
        self._check(st)
        return res, spec, amp

    def poll(self, ticket):
        """(result, spectrum, amplitude) when the job is done, else None."""
        res = self._pending[ticket][0]
        st = self.lib.etraj_server_poll(self.srv, ticket, C.byref(res))
        if st == abi.ERR_NOT_READY:
            return None
        return self._finish(ticket, st)

    def wait(self, ticket, timeout=-1.0):
        res = self._pending[ticket][0]
        st = self.lib.etraj_server_wait(self.srv, ticket, C.byref(res), float(timeout))
        if st == abi.ERR_TIMEOUT:
            raise EtrajError(st, "timed out")
        return self._finish(ticket, st)

    def stats(self):
        """(running, queued, device bytes held by the slots)."""
        r, q, m = C.c_int64(), C.c_int64(), C.c_size_t()
        self._check(self.lib.etraj_server_stats(self.srv, C.byref(r), C.byref(q), C.byref(m)))
        return r.value, q.value, m.value


_default_engine = None


def default_engine():
    global _default_engine
    if _default_engine is None:
        _default_engine = Engine()
    return _default_engine


def _axis(pmax, num):
    return np.linspace(-pmax, pmax, num) if num > 1 else np.array([0.0])


def perform_traj_simulation(*, init_cond_method, laser, target, dimension, sample_t_intv,
                            sample_t_num, traj_t_final, final_p_max, final_p_num,
                            ss_kd_max=0.0, ss_kd_num=0, ss_kz_max=0.0, ss_kz_num=0,
                            mc_kt_num=0, mc_kd_max=0.0, mc_kz_max=0.0,
                            traj_phase_method="CTMC", traj_rtol=1e-6, output_fmt="jld2",
                            output_compress=True, output_path=None, sample_monte_carlo=False,
                            sample_cutoff_limit=1e-16, rate_prefix="Full", mol_orbit_ridx=0,
                            show_progress=False, precision="fp64", seed=0, engine=None, mc_kt_proposal="uniform"):
    """Performs a semiclassical trajectory simulation (TrajectorySimulation.jl:103-161) on the GPU.

    Returns a dict with the keys of the reference's output file, and writes
    that file when `output_path` is given: `output_fmt` :jld2 (the default) or
    :h5 as write_output! does (h5write.py; momentum_spec deflated when output_compress), or "npz".  As in the
    reference (:199-215) an existing file is not overwritten (a time-stamped
    name is used instead) and the extension is appended when missing.  Extra
    keywords: `precision` ("fp64", "fp32_df" or "fp32_bulk"), `seed` (Monte-Carlo
    stream), `engine`."""
    job = make_job(init_cond_method=init_cond_method, laser=laser, target=target,
                   dimension=dimension, sample_t_intv=sample_t_intv, sample_t_num=sample_t_num,
                   traj_t_final=traj_t_final, final_p_max=final_p_max, final_p_num=final_p_num,
                   ss_kd_max=ss_kd_max, ss_kd_num=ss_kd_num, ss_kz_max=ss_kz_max,
                   ss_kz_num=ss_kz_num, mc_kt_num=mc_kt_num, mc_kd_max=mc_kd_max,
                   mc_kz_max=mc_kz_max, traj_phase_method=traj_phase_method, traj_rtol=traj_rtol,
                   sample_monte_carlo=sample_monte_carlo, sample_cutoff_limit=sample_cutoff_limit,
                   rate_prefix=rate_prefix, mol_orbit_ridx=mol_orbit_ridx, precision=precision, seed=seed,
                   mc_kt_proposal=mc_kt_proposal)
    fmt = _sym(output_fmt)
    if fmt == "hdf5":
        fmt = "h5"
    if fmt not in ("jld2", "h5", "npz"):
        raise ValueError("[TrajectorySimulationJob] Unsupported output format `%s`." % output_fmt)
    eng = engine or default_engine()
    res, spec, amp = eng.run(job, want_spectrum=True,
                             want_amplitude=(_sym(traj_phase_method) != "CTMC"))
    shape = tuple(int(x) for x in final_p_num)
    out = {
        "px": _axis(final_p_max[0], final_p_num[0]),
        "py": _axis(final_p_max[1], final_p_num[1]),
        "momentum_spec": spec.reshape(shape, order="F"),
        "ion_prob": res.ion_prob,
        "ion_prob_uncollected": res.ion_prob_uncollected,
        "num_effective_traj": res.num_effective_traj,
        "num_failed_traj": res.num_failed_traj,
    }
    if dimension == 3:
        out["pz"] = _axis(final_p_max[2], final_p_num[2])
    if amp is not None:
        out["amplitude"] = (amp[0::2] + 1j * amp[1::2]).reshape(shape, order="F")
    path = None
    if output_path:
        import os
        import time
        path = output_path
        if os.path.isfile(path) or os.path.isfile(path + "!"):
            warnings.warn("[TrajectorySimulationJob] File `%s` already exists, saving under a time-stamped name." % path)
            path = time.strftime("TrajectorySimulation-%Y%m%d.%H%M%S")
        ext = "." + fmt
        if not path.endswith(ext):
            path += ext
    params = _params(locals())
    out["params"] = params
    out["params_text"] = _yaml(params)
    if path:
        if fmt == "npz":
            flat = {k: v for k, v in out.items() if k != "params"}
            (np.savez_compressed if output_compress else np.savez)(path, **flat)
        else:
            # the names and order of write_output! (TrajectorySimulation.jl:237, 508-543)
            from . import h5write
            items = [("info", "Trajectory simulation output generated by etraj-gb300"),
                     ("params_text", out["params_text"])]
            if fmt == "jld2":
                items.append(("params", params))
            items += [("px", out["px"]), ("py", out["py"])]
            if dimension == 3:
                items.append(("pz", out["pz"]))
            items += [("momentum_spec", out["momentum_spec"]), ("ion_prob", float(out["ion_prob"])),
                      ("ion_prob_uncollected", float(out["ion_prob_uncollected"])),
                      ("num_effective_traj", int(out["num_effective_traj"]))]
            h5write.write(path + "!", items, jld2=(fmt == "jld2"),
                          compress=("momentum_spec",) if output_compress else ())
            os.replace(path + "!", path)
        out["output_path"] = path
    return out


def _params(kw):
    """The effective parameters that TrajectorySimulation.jl:275-296 packs into
    `params`, in its order: symbols as strings, the laser and target as their
    Serialize dicts; the method's sample ranges, rate_prefix for the ADK / SPA /
    SPANE family and mol_orbit_ridx for molecules."""
    method = _sym(kw["init_cond_method"])
    p = {"init_cond_method": method, "laser": kw["laser"].Serialize(), "target": kw["target"].Serialize(),
         "sample_t_intv": tuple(float(x) for x in kw["sample_t_intv"]), "sample_t_num": int(kw["sample_t_num"]),
         "sample_monte_carlo": bool(kw["sample_monte_carlo"]),
         "sample_cutoff_limit": float(kw["sample_cutoff_limit"]),
         "traj_phase_method": _sym(kw["traj_phase_method"]), "traj_rtol": float(kw["traj_rtol"]),
         "traj_t_final": float(kw["traj_t_final"]), "output_fmt": kw["fmt"], "output_path": kw["path"] or "",
         "final_p_max": tuple(float(x) for x in kw["final_p_max"]),
         "final_p_num": tuple(int(x) for x in kw["final_p_num"])}
    three = int(kw["dimension"]) == 3
    if not kw["sample_monte_carlo"]:
        p["ss_kd_max"], p["ss_kd_num"] = float(kw["ss_kd_max"]), int(kw["ss_kd_num"])
        if three:
            p["ss_kz_max"], p["ss_kz_num"] = float(kw["ss_kz_max"]), int(kw["ss_kz_num"])
    else:
        p["mc_kd_max"], p["mc_kt_num"] = float(kw["mc_kd_max"]), int(kw["mc_kt_num"])
        if three:
            p["mc_kz_max"] = float(kw["mc_kz_max"])
    if method.endswith(("ADK", "SPA", "SPANE", "SFA", "SFAAE")):
        rp = kw["rate_prefix"]
        p["rate_prefix"] = _sym(rp) if isinstance(rp, str) else [_sym(x) for x in rp]
    if getattr(kw["target"], "MolEnergyLevels", None) is not None:
        p["mol_orbit_ridx"] = int(kw["mol_orbit_ridx"])
    return p


def _jl_float(x):
    """A float as Julia prints it: the shortest digits that round-trip, in
    scientific notation (mantissa with a decimal point, bare exponent) outside
    [1e-4, 1e6)."""
    x = float(x)
    if x != x:
        return "NaN"
    if x in (float("inf"), float("-inf")):
        return "Inf" if x > 0 else "-Inf"
    if x == 0.0 or 1e-4 <= abs(x) < 1e6:
        r = repr(x)
        return r if "." in r else r + ".0"
    m, e = np.format_float_scientific(x, unique=True, trim="0").split("e")
    return "%se%d" % (m, int(e))


def _yaml_scalar(v):
    if isinstance(v, (bool, np.bool_)):
        return "true" if v else "false"
    if isinstance(v, (int, np.integer)):
        return str(int(v))
    if isinstance(v, (float, np.floating)):
        return _jl_float(v)
    return str(v)


def _yaml(d, indent=0):
    """Block-style YAML of the params dict (the params_text entry, YAML.write at
    TrajectorySimulation.jl:507)."""
    pad = "  " * indent
    lines = []
    for k, v in d.items():
        if isinstance(v, dict):
            lines.append("%s%s:" % (pad, k))
            lines.append(_yaml(v, indent + 1))
        elif isinstance(v, (list, tuple, np.ndarray)):
            lines.append("%s%s:" % (pad, k))
            for x in np.asarray(v, dtype=object).ravel(order="F"):
                lines.append("%s  - %s" % (pad, _yaml_scalar(x)))
        else:
            lines.append("%s%s: %s" % (pad, k, _yaml_scalar(v)))
    return "\n".join(lines)
