"""The tensor-core precision form (tcgen05, BF16 / TF32 inputs, FP32 accumulation).

Bounds, stated here and in the kernel's docs:
  * delta from identical inputs, relative Frobenius against the FP32 oracle:
        BF16 <= 1e-2, TF32 <= 2e-3   (inputs rounded to 8 / 11 significant bits)
  * the fit after 3 sweeps within 1e-3 (BF16) / 2e-4 (TF32) of the FP64 oracle's,
    on the well-posed cases.
"""

import numpy as np
import pytest

import gputucker_gb300 as gtk
from oracle_util import Oracle, rel_fro
from test_gpu_parity import CASES, data

pytestmark = pytest.mark.gpu

TC_CASES = [c for c in CASES if (len(c[1]), c[4]) in
            {(3, 4), (3, 8), (3, 10), (3, 12), (3, 16), (4, 4), (4, 8), (4, 10), (4, 12)}]
BOUND = {"bf16": dict(delta=1e-2, fit=1e-3), "tf32": dict(delta=2e-3, fit=2e-4)}


@pytest.mark.parametrize("prec", ["bf16", "tf32"])
@pytest.mark.parametrize("case", TC_CASES, ids=[c[0] for c in TC_CASES])
def test_tensor_core_delta(case, prec):
    name, dims, nnz, P, J, _ = case
    idx, vals = data(case, 0)
    with gtk.create_tensor_blocks(gtk.coo_from_arrays(idx, vals, dims=dims), P, J) as t:
        ora = Oracle(0, idx, vals, dims, P, J)
        t.init_random(1, 0)
        ora.init_random(1, 0)
        t.set_precision(prec)
        for n in range(len(dims)):
            err = rel_fro(t.compute_delta(n), ora.delta(n))
            print(f"{name} {prec} delta mode {n}: {err:.3e}")
            assert err <= BOUND[prec]["delta"], (n, err)


@pytest.mark.parametrize("prec", ["bf16", "tf32"])
@pytest.mark.parametrize("case", TC_CASES, ids=[c[0] for c in TC_CASES])
def test_tensor_core_sweeps_fit(case, prec):
    name, dims, nnz, P, J, _ = case
    idx, vals = data(case, 0)
    with gtk.create_tensor_blocks(gtk.coo_from_arrays(idx, vals, dims=dims), P, J) as t:
        o64 = Oracle(1, idx, vals.astype(np.float64), dims, P, J)
        t.init_random(1, 0)
        o64.init_random(1, 0)
        t.set_precision(prec)
        for s in range(3):
            t.update_factor_matrices()
            fit = t.reconstruction()
            f64 = o64.sweep()["fit64"]
            print(f"{name} {prec} sweep {s}: fit {fit:.8f} fp64 oracle {f64:.8f} diff {abs(fit - f64):.2e}")
        assert abs(fit - f64) <= BOUND[prec]["fit"]


def test_precision_rejects_unsupported_shape():
    idx, vals = data(CASES[7], 0)  # N = 5
    name, dims, nnz, P, J, _ = CASES[7]
    with gtk.create_tensor_blocks(gtk.coo_from_arrays(idx, vals, dims=dims), P, J) as t:
        with pytest.raises(gtk.GTKError) as e:
            t.set_precision("bf16")
        assert e.value.code == gtk._native.GTK_ERR_UNSUPPORTED
        t.set_precision("plain")
