"""gtk_reconstruction_error_noalloc: the reconstruction error without any device allocation.

For callers that cannot allocate device memory where they run (latency-critical
loops that must not touch the allocator, device memory owned or capped by
another runtime's pool).  The entry point reads the caller's device arrays and
keeps its scratch in a fixed device array of the library.  Checked on two calls
in a row against the existing entry point (gtk_reconstruction on a handle) and
against the FP64 oracle's error of the same factors and core; the FP32 fits
agree to the tolerance the FP32 tests use (1e-5).

The device buffers here come from torch (any allocator works: the entry point
only needs device pointers).  This file sorts last so that a run stopping at the
first failure has run every other test first.
"""

import ctypes as C

import numpy as np
import pytest

import gputucker_gb300 as gtk
from gputucker_gb300 import _native as nat
from oracle_util import Oracle, random_coo

pytestmark = pytest.mark.gpu

FIT_TOL = 1e-5


def _dev(torch, a):
    a = np.ascontiguousarray(a)
    if a.dtype == np.uint32:
        a = a.view(np.int32)  # same bits; the kernel reads them as uint32
    return torch.from_numpy(a).cuda()


@pytest.mark.parametrize("case", [([25, 30, 20, 22], [2, 1, 2, 1], 10, 20000), ([40, 35, 30], [1, 2, 1], 8, 12000)])
def test_noalloc_error_matches_reconstruction(case):
    torch = pytest.importorskip("torch")
    dims, P, J, nnz = case
    rng = np.random.default_rng(31)
    idx = random_coo(rng, dims, nnz)
    vals = rng.random(len(idx[0])).astype(np.float32)
    coo = gtk.coo_from_arrays(idx, vals, dims=dims)
    lib = nat.load()
    with gtk.create_tensor_blocks(coo, P, J) as t:
        t.init_random(1, 0)
        t.update_factor_matrices()  # real (post-update) factors
        N = len(dims)
        facs = [t.get_factor(n)[:dims[n]] for n in range(N)]
        core = t.get_core()
        fit_ref = t.reconstruction()
        # the oracle's error of the same factors and core (FP64 arithmetic on the FP32 values)
        ora = Oracle(1, idx, vals.astype(np.float64), dims, P, J)
        for n in range(N):
            ora.set_factor(n, t.get_factor(n).astype(np.float64))
        ora.set_core(core.astype(np.float64))
        fit_ora = ora.fit()["fit64"]
        d_idx = [_dev(torch, i) for i in idx]
        d_val = _dev(torch, vals)
        d_fac = [_dev(torch, f) for f in facs]
        d_core = _dev(torch, core.reshape(-1))
        d_err = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
        idx_tab = (C.c_void_p * N)(*[x.data_ptr() for x in d_idx])
        fac_tab = (C.c_void_p * N)(*[x.data_ptr() for x in d_fac])
        stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        for call in range(2):  # the shared scratch keeps the last call's contents
            d_err.fill_(-1.0)
            rc = lib.gtk_reconstruction_error_noalloc(N, J, len(vals), idx_tab, C.c_void_p(d_val.data_ptr()), fac_tab,
                                                      C.c_void_p(d_core.data_ptr()), C.c_void_p(d_err.data_ptr()),
                                                      stream)
            assert rc == 0, lib.gtk_last_error()
            torch.cuda.synchronize()
            err = float(d_err.item())
            fit = 1.0 - np.sqrt(err) / t.info.norm
            assert abs(fit - fit_ref) <= FIT_TOL, (call, fit, fit_ref)
            assert abs(fit - fit_ora) <= FIT_TOL, (call, fit, fit_ora)


def test_noalloc_rejects_core_beyond_scratch():
    torch = pytest.importorskip("torch")
    lib = nat.load()
    d = torch.zeros(4, dtype=torch.float32, device="cuda")
    e = torch.zeros(1, dtype=torch.float64, device="cuda")
    # order 5, rank 20: 20^4 * 20 floats > 2^20
    rc = lib.gtk_reconstruction_error_noalloc(5, 20, 0, None, None, None, C.c_void_p(d.data_ptr()),
                                              C.c_void_p(e.data_ptr()), None)
    assert rc == nat.GTK_ERR_UNSUPPORTED
    assert b"no-allocation scratch" in lib.gtk_last_error()
