"""The reference-order variant against the reference's own fixtures.

GTK_VARIANT_REFERENCE_ORDER computes delta exactly as computing_delta_kernel
does (delta.cuh:62-90): core entries in linear order, the product of the core
value and the other modes' factor entries left to right with every product
rounded, accumulated per output column in that order.  So delta is
bit-identical to the reference's, in FP32 as in FP64, and the FP32 sweep follows
the reference's FP32 path exactly: B and C are summed in double in the
reference's order (ComputingBC, update.cuh:52-100), the row solve inverts B by LU
with row pivoting and accumulates a = C^T B^-1 in value_t (update.cuh:163-194),
the fit reconstructs x_hat in core order and sums the errors serially in value_t
against the reference's value_t norm (reconstruction.cuh:58-81, 259-276;
tensor_manager.tpp:263-293).  Against the fixtures the reference's own code
produced (tests/golden/make_golden.py): FP32 factors, fit and core bit-exact
through 3 sweeps; FP64 within 1e-12 (the restated LU and Eigen's blocked LU
round differently in double).
"""

import glob
import os

import numpy as np
import pytest

import gputucker_gb300 as gtk
from oracle_util import ROOT, rel_fro

pytestmark = pytest.mark.gpu

GOLDEN = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "*.npz")))


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_reference_order_matches_reference(path):
    g = np.load(path)
    dtype = int(g["dtype"])
    N = len(g["dims"])
    P = [int(x) for x in g["P"]]
    J = int(g["J"])
    coo = gtk.parse_from_file(path[:-4] + ".tns", N, dtype, rand_seed=1)
    with gtk.create_tensor_blocks(coo, P, J) as t:
        t.init_random(1, coo.rand_draws)
        t.set_kernel_variant("reference_order")
        for n in range(N):
            d = t.compute_delta(n)
            ref = g[f"delta0_{n}"].reshape(d.shape)
            assert np.array_equal(d, ref), (n, np.abs(d - ref).max())
        for s in range(3):
            t.update_factor_matrices()
            fit = t.reconstruction()
            for n in range(N):
                f = t.get_factor(n)
                ref = g[f"fac{s + 1}_{n}"]
                print(f"{os.path.basename(path)} sweep {s} mode {n}: {rel_fro(f, ref):.2e}")
                if dtype == 0:
                    assert np.array_equal(f, ref), (s, n, rel_fro(f, ref))
                else:
                    assert rel_fro(f, ref) <= 1e-12, (s, n)
            print(f"fit {fit!r} reference {float(g[f'fit{s + 1}'])!r}")
            if dtype == 0:
                assert fit == float(g[f"fit{s + 1}"]), (s, fit)
            else:
                assert abs(fit - float(g[f"fit{s + 1}"])) <= 1e-12
        assert np.array_equal(t.get_core(), g["core"])


from test_gpu_parity import CASES, ILL, data  # noqa: E402


@pytest.mark.parametrize("case", CASES + ILL, ids=[c[0] for c in CASES + ILL])
def test_reference_order_bit_exact_vs_oracle(case):
    """The oracle restates the reference's path bit for bit in FP32 (pinned against
    the fixtures in test_oracle.py); the reference-order variant matches it bit for
    bit too -- on every shape, including the Zipf-skewed cases where FP32 ALS is
    chaotic and any other order of operations drifts by O(1)."""
    from oracle_util import Oracle
    name, dims, nnz, P, J, _ = case
    idx, vals = data(case, 0)
    with gtk.create_tensor_blocks(gtk.coo_from_arrays(idx, vals, dims=dims), P, J) as t:
        ora = Oracle(0, idx, vals, dims, P, J)
        t.init_random(1, 0)
        ora.init_random(1, 0)
        t.set_kernel_variant("reference_order")
        for s in range(3):
            fit = t.sweep()
            of = ora.sweep()["fit_ref"]
            for n in range(len(dims)):
                assert np.array_equal(t.get_factor(n), ora.get_factor(n)), (name, s, n)
            assert fit == of, (name, s, fit, of)
