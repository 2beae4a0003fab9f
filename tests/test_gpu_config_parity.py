"""Parity at the sizes and shapes of the workload table, not only on small cases.

* The 4-order 100M-nonzero Zipf(1.1) tensor with P_n = 4 on every mode (256
  blocks), at full size: every block's coordinates and values, every
  count_nnz and where_nnz, bit-exact against the oracle's restatement of
  CreateTensorBlocks / AssignIndicesToEachMode (tensor_manager.tpp:201-302,
  block.tpp:115-186).  GTK_CONFIG_PARITY_NNZ lowers the size.
* A 1M-nonzero sample of the same configuration (dims 100,000^4, P = 4^4,
  rank 10): one plain FP32 sweep held to the accuracy-parity rule of
  test_gpu_parity.py, and the reference-order variant held bit-exact to the
  oracle's FP32 path (factors, fit, core) with its time per sweep printed.
* The precision forms' FP64 branch: rows whose FP32 Cholesky shows a condition
  estimate above 1e5 are re-solved in FP64.  On data whose BF16 contraction is
  exact (factor entries small integers, core entries in halves, values in
  eighths), the Gram and right-hand side equal the FP64 oracle's, so
  the rows that took the FP64 branch must match the FP64 oracle's solution to
  FP64 accuracy; the branch is counted by gtk_solve_counters.
"""

import os
import time

import numpy as np
import pytest

import gputucker_gb300 as gtk
from oracle_util import Oracle, random_coo, rel_fro
from test_gpu_parity import check_partition, fp32_sweeps

pytestmark = pytest.mark.gpu

ZIPF4D = dict(order=4, dims=[100_000] * 4, zipf_s=1.1, rank=10, P=[4, 4, 4, 4])


def test_zipf4d_partition_bit_exact_full_size():
    nnz = int(os.environ.get("GTK_CONFIG_PARITY_NNZ", 100_000_000))
    c = ZIPF4D
    coo = gtk.generate(c["order"], c["dims"], nnz, "zipf", c["zipf_s"], "uniform", "f32", seed=0)
    idx, vals = coo.arrays()
    with gtk.create_tensor_blocks(coo, c["P"], c["rank"]) as t:
        coo.free()
        ora = Oracle(0, idx, vals, t.info.dims, c["P"], c["rank"])
        assert ora.status == 0
        del idx, vals
        assert t.info.block_count == 256
        # ||X|| over 1e8 terms: FP64 sums in two orders differ by ~sqrt(nnz) * 2^-53 (measured 1.9e-12)
        check_partition(t, ora, norm_rtol=1e-10)


def _zipf4d_sample(nnz=1_000_000):
    c = ZIPF4D
    coo = gtk.generate(c["order"], c["dims"], nnz, "zipf", c["zipf_s"], "uniform", "f32", seed=0)
    idx, vals = coo.arrays()
    return coo, idx, vals


def test_zipf4d_sample_fp32_accuracy_parity():
    c = ZIPF4D
    coo, idx, vals = _zipf4d_sample()
    with gtk.create_tensor_blocks(coo, c["P"], c["rank"]) as t:
        o32 = Oracle(0, idx, vals, coo.dims, c["P"], c["rank"])
        o64 = Oracle(1, idx, vals.astype(np.float64), coo.dims, c["P"], c["rank"])
        rep = fp32_sweeps(t, o32, o64, sweeps=1)
    worst = max(rep, key=lambda r: r[3])
    print(f"zipf4d 1M sample, FP32 sweep: worst factor {worst[1]} {worst[3]:.2e} from FP64 "
          f"(reference FP32 {worst[4]:.2e} from FP64)")


def test_zipf4d_sample_reference_order_bit_exact():
    c = ZIPF4D
    coo, idx, vals = _zipf4d_sample()
    with gtk.create_tensor_blocks(coo, c["P"], c["rank"]) as t:
        ora = Oracle(0, idx, vals, coo.dims, c["P"], c["rank"])
        t.init_random(1, 0)
        ora.init_random(1, 0)
        t.set_kernel_variant("reference_order")
        t.sweep()  # first sweep: kernels prepared, the reference's value_t norm summed
        ora.sweep()
        t.synchronize()
        t0 = time.perf_counter()
        fit = t.sweep()
        dt = time.perf_counter() - t0
        of = ora.sweep()["fit_ref"]
        for n in range(c["order"]):
            assert np.array_equal(t.get_factor(n), ora.get_factor(n)), n
        assert fit == of, (fit, of)
        assert np.array_equal(t.get_core(), ora.get_core())
        t.set_kernel_variant("auto")
        t.synchronize()
        t0 = time.perf_counter()
        t.sweep()
        dt_fast = time.perf_counter() - t0
    print(f"zipf4d 1M sample: reference-order sweep {dt * 1e3:.1f} ms, default plain FP32 sweep "
          f"{dt_fast * 1e3:.1f} ms")


def _exact_case(seed=5):
    """3-order data whose BF16 products and FP32 MMA sums are exact: factor entries
    in {1, 2, 3, 4}, core entries in {-1, -1/2, 0, 1/2, 1}, values in eighths.
    Zipf(1.2) rows: the light ones (fewer nonzeros than the rank) have Gram
    matrices of condition ~1e5..1e7, the heavy ones are well conditioned."""
    rng = np.random.default_rng(seed)
    dims, J = [300, 48, 40], 4
    idx = random_coo(rng, dims, 3000, distinct=True, zipf=1.2)
    vals = (rng.integers(0, 8, len(idx[0])) / 8.0).astype(np.float32)
    facs = [rng.integers(1, 5, (d, J)).astype(np.float32) for d in dims]
    core = (rng.integers(-2, 3, (J,) * 3) / 2.0).astype(np.float32)
    return dims, J, idx, vals, facs, core


def test_precision_form_fp64_branch_rows():
    dims, J, idx, vals, facs, core = _exact_case()
    P = [1, 1, 1]
    ora = Oracle(1, idx, vals.astype(np.float64), dims, P, J)
    for n in range(3):
        ora.set_factor(n, facs[n].astype(np.float64))
    ora.set_core(core.astype(np.float64))
    # the exact Gram of mode 0 and the host's condition estimate of every row
    d = ora.delta(0)
    rows = idx[0].astype(np.int64)
    lam = float(np.float32(1e-4))
    cond = np.ones(dims[0])
    for r in range(dims[0]):
        D = d[rows == r]
        cond[r] = np.linalg.cond(D.T @ D + lam * np.eye(J))
    # the kernel's 1-norm estimate kappa_1 lies within a small factor of the
    # 2-norm condition (kappa_2 <= kappa_1 <= J kappa_2; Hager's estimate of
    # ||B^-1||_1 is a lower bound, in practice within ~3): clear of its 1e5 threshold
    sure64 = cond > 1e6
    sure32 = cond < 1e4
    est = cond
    assert sure64.sum() >= 5 and sure32.sum() >= 5, (sure64.sum(), sure32.sum())
    ora.update_mode(0)
    want = ora.get_factor(0)
    coo = gtk.coo_from_arrays(idx, vals, dims=dims)
    with gtk.create_tensor_blocks(coo, P, J) as t:
        for n in range(3):
            t.set_factor(n, facs[n])
        t.set_core(core)
        t.set_precision("bf16")
        t.solve_counters(reset=True)
        t.update_mode(0)
        n64, _ = t.solve_counters()
        got = t.get_factor(0).astype(np.float64)
    print(f"rows {dims[0]}: condition number > 1e6 on {int(sure64.sum())}, < 1e4 on {int(sure32.sum())}; "
          f"FP64 branch taken by {n64}")
    assert sure64.sum() <= n64 <= dims[0] - sure32.sum()
    # FP64 Cholesky against the oracle's FP64 LU inverse on the same system: both
    # backward stable, so within a modest multiple of cond(B) * 2^-53 of each other
    # (measured up to ~80x; an FP32 solve of these rows is off by ~cond(B) * 2^-24,
    # checked below)
    for r in np.flatnonzero(sure64):
        e = np.linalg.norm(got[r] - want[r]) / max(np.linalg.norm(want[r]), 1e-300)
        assert e <= 512 * cond[r] * 2.0 ** -53, (r, est[r], cond[r], e)
    for r in np.flatnonzero(sure32):
        e = np.linalg.norm(got[r] - want[r]) / max(np.linalg.norm(want[r]), 1e-300)
        assert e <= 1e-4, (r, est[r], e)
    # the FP64 branch matters: an FP32 solve of those rows lands far from FP64
    worst32 = 0.0
    for r in np.flatnonzero(sure64):
        D = d[rows == r]
        B = (D.T @ D + lam * np.eye(J)).astype(np.float32)
        C = (vals[idx[0] == r].astype(np.float64) @ D).astype(np.float32)
        a32 = np.linalg.solve(B, C).astype(np.float64)
        worst32 = max(worst32, np.linalg.norm(a32 - want[r]) / np.linalg.norm(want[r]))
    assert worst32 > 1e-6, worst32
    assert rel_fro(got, want) <= 1e-4
