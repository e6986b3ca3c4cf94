"""etraj_deposit_noalloc: the deposit for callers that cannot allocate device
memory during the call (their own pool owns the device, or they reserve all
memory before a run).  Its sort scratch is a fixed array inside the library.

The test feeds it the per-electron bins and contributions of a job and checks
that it reproduces the momentum distribution that etraj_run computes for the
same job, on two calls in a row (the scratch keeps the first call's contents).
Between them runs a call with fewer electrons, another grid and some keys above
that grid (taken as "not deposited"), checked against a deposit done on the
host: left-over pairs, histograms or counts of a larger call must not leak into
a smaller one, nor the smaller one's into the next.
Tolerance: the same 1e-10 relative L2 as the other parity tests (the deposit
order is fixed, so the results are in fact bit-identical).  Inputs and outputs
are device buffers the test allocates with torch, as such a caller would.

Kept in a file that pytest collects last.
"""
import ctypes as C

import numpy as np
import pytest

import _oracle as O
import etraj_gb300 as et
from etraj_gb300 import abi

pytestmark = pytest.mark.gpu


def _job(phase, **kw):
    T = 2 * np.pi / (45.563352525 / 800.0)
    laser = et.Cos2Laser(peak_int=1.2e14, wave_len=800.0, cyc_num=2, ellip=1.0)
    args = dict(init_cond_method="SPANE", laser=laser, target=et.get_atom("Ar"), dimension=2,
                sample_t_intv=(-T, T), sample_t_num=300, traj_t_final=3 * T, final_p_max=(2.0, 2.0),
                final_p_num=(300, 300), sample_monte_carlo=True, mc_kt_num=400, mc_kd_max=1.0,
                traj_phase_method=phase, seed=5)
    args.update(kw)
    return et.make_job(**args)


def _rel_l2(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("phase", ["SCTS", "CTMC"])
def test_noalloc_deposit_matches_run(phase):
    import torch

    lib = abi.load_library()
    job = _job(phase)
    eng = et.Engine(device=0)
    res, spec_ref, amp_ref = eng.run(job, want_spectrum=True, want_amplitude=True)
    eng.close()
    # the same job's electrons, final states and deposit inputs
    init = O.sample_all(job)
    fin, st, _ = O.integrate(job, init)
    key, cre, cim = O.contributions(job, init, fin, st)
    n = key.size
    assert n == res.num_effective_traj and 0 < n <= (1 << 19)
    coherent = 0 if phase == "CTMC" else 1
    grid = job.grid_size
    dev = torch.device("cuda", 0)
    d_key = torch.from_numpy(key.view(np.int32)).to(dev)
    d_re = torch.from_numpy(cre).to(dev)
    d_im = torch.from_numpy(cim).to(dev)
    stream = torch.cuda.Stream(device=dev)

    def deposit(d_key, d_re, d_im, n, grid):
        s_re = torch.full((grid,), 7.0, dtype=torch.float64, device=dev)  # outputs start dirty
        s_im = torch.full((grid,), 7.0, dtype=torch.float64, device=dev)
        mspec = torch.empty(grid, dtype=torch.float64, device=dev)
        torch.cuda.synchronize(dev)
        stc = lib.etraj_deposit_noalloc(n, C.c_void_p(d_key.data_ptr()), C.c_void_p(d_re.data_ptr()),
                                        C.c_void_p(d_im.data_ptr()), grid, coherent,
                                        C.c_void_p(s_re.data_ptr()), C.c_void_p(s_im.data_ptr()),
                                        C.c_void_p(mspec.data_ptr()), C.c_void_p(stream.cuda_stream))
        assert stc == abi.OK
        stream.synchronize()
        return mspec.cpu().numpy(), s_re.cpu().numpy(), s_im.cpu().numpy()

    def check_full(out):
        mspec, s_re, s_im = out
        assert _rel_l2(mspec, spec_ref) <= 1e-10
        assert np.array_equal(mspec, spec_ref)
        if coherent:
            assert _rel_l2(s_re + 1j * s_im, amp_ref[0::2] + 1j * amp_ref[1::2]) <= 1e-10

    check_full(deposit(d_key, d_re, d_im, n, grid))
    # a smaller call on another grid: a prefix of the electrons, their bins folded
    # onto grid2, every 97th key replaced by one far above grid2
    n2 = n // 3
    grid2 = grid // 2 + 7
    k2 = key[:n2].astype(np.int64)
    k2 = np.where(k2 == grid, grid2, k2 % grid2)
    k2[::97] = 0xFFFFFFF0
    k2 = k2.astype(np.uint32)
    want_re, want_im = np.zeros(grid2), np.zeros(grid2)
    for i in range(n2):  # bins summed in electron order, from 0.0, as the device does
        if k2[i] < grid2:
            want_re[k2[i]] += cre[i]
            want_im[k2[i]] += cim[i]
    want = want_re * want_re + want_im * want_im if coherent else want_re
    m2, r2, i2 = deposit(torch.from_numpy(k2.view(np.int32)).to(dev), d_re, d_im, n2, grid2)
    assert _rel_l2(m2, want) <= 1e-10 and np.array_equal(m2, want)
    assert np.array_equal(r2, want_re) and (not coherent or np.array_equal(i2, want_im))
    # and the first call again, after the smaller one
    check_full(deposit(d_key, d_re, d_im, n, grid))


def test_noalloc_deposit_rejects_oversize_and_empty_is_zero():
    import torch

    lib = abi.load_library()
    dev = torch.device("cuda", 0)
    grid = 64
    s_re = torch.full((grid,), 3.0, dtype=torch.float64, device=dev)
    mspec = torch.full((grid,), 3.0, dtype=torch.float64, device=dev)
    dummy = torch.zeros(1, dtype=torch.float64, device=dev)
    big = (1 << 19) + 1
    st = lib.etraj_deposit_noalloc(big, C.c_void_p(dummy.data_ptr()), C.c_void_p(dummy.data_ptr()),
                                   None, grid, 0, C.c_void_p(s_re.data_ptr()), None,
                                   C.c_void_p(mspec.data_ptr()), None)
    assert st == abi.ERR_INVALID_ARGUMENT
    st = lib.etraj_deposit_noalloc(0, None, None, None, grid, 0, C.c_void_p(s_re.data_ptr()), None,
                                   C.c_void_p(mspec.data_ptr()), None)
    assert st == abi.OK
    torch.cuda.synchronize(dev)
    assert not mspec.any() and not s_re.any()
