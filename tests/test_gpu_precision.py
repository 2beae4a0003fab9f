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
# BF16 only: the core streams through shared memory (N = 5, and N = 4 at J = 16)
TS_CASES = [c for c in CASES if (len(c[1]), c[4]) in {(5, 4), (5, 8)}]
BOUND = {"bf16": dict(delta=1e-2, fit=1e-3), "tf32": dict(delta=2e-3, fit=2e-4)}


@pytest.mark.parametrize("prec,case", [(p, c) for p in ("bf16", "tf32") for c in TC_CASES] +
                         [("bf16", c) for c in TS_CASES],
                         ids=[f"{p}-{c[0]}" for p in ("bf16", "tf32") for c in TC_CASES] +
                         [f"bf16-{c[0]}" for c in TS_CASES])
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


@pytest.mark.parametrize("prec,case", [(p, c) for p in ("bf16", "tf32") for c in TC_CASES] +
                         [("bf16", c) for c in TS_CASES],
                         ids=[f"{p}-{c[0]}" for p in ("bf16", "tf32") for c in TC_CASES] +
                         [f"bf16-{c[0]}" for c in TS_CASES])
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


@pytest.mark.parametrize("prec,case", [(p, c) for p in ("bf16", "tf32") for c in TC_CASES] +
                         [("bf16", c) for c in TS_CASES],
                         ids=[f"{p}-{c[0]}" for p in ("bf16", "tf32") for c in TC_CASES] +
                         [f"bf16-{c[0]}" for c in TS_CASES])
def test_fit_from_gram_matches_direct_fit(case, prec):
    """In the tensor-core forms a sweep's fit comes from the last mode's Gram/RHS
    (err = ||X||^2 - sum_i (2 a_i.c_i - a_i^T G_i a_i)); after the factors are set
    again the fit kernel recomputes delta and sums (x - x_hat)^2 directly.  Both
    within 1e-5 (the expansion loses ~||X||^2/err of the Gram sums' ~1e-7)."""
    name, dims, nnz, P, J, _ = case
    idx, vals = data(case, 0)
    with gtk.create_tensor_blocks(gtk.coo_from_arrays(idx, vals, dims=dims), P, J) as t:
        t.init_random(1, 0)
        t.set_precision(prec)
        for s in range(2):
            t.update_factor_matrices()
            f_gram = t.reconstruction()
            t.set_factor(len(dims) - 1, t.get_factor(len(dims) - 1))  # the Gram no longer describes the factors
            f_direct = t.reconstruction()
            print(f"{name} {prec} sweep {s}: from Gram {f_gram:.9f} direct {f_direct:.9f}")
            assert abs(f_gram - f_direct) <= 1e-5 * max(1.0, abs(f_direct)), (s, f_gram, f_direct)
        # the graph-replayed sweep's fit is the Gram one too
        t.set_graph(True)
        f_graph = t.sweep()
        t.set_factor(0, t.get_factor(0))
        assert abs(f_graph - t.reconstruction()) <= 1e-5 * max(1.0, abs(f_graph))


def test_precision_rejects_unsupported_shape():
    for ci, prec in ((9, "bf16"), (7, "tf32")):  # N = 2; N = 5 has a BF16 form only
        idx, vals = data(CASES[ci], 0)
        name, dims, nnz, P, J, _ = CASES[ci]
        with gtk.create_tensor_blocks(gtk.coo_from_arrays(idx, vals, dims=dims), P, J) as t:
            with pytest.raises(gtk.GTKError) as e:
                t.set_precision(prec)
            assert e.value.code == gtk._native.GTK_ERR_UNSUPPORTED
            t.set_precision("plain")


# larger cores (the whole core streams per tile in many chunks): checked against the
# plain FP32 delta and the FP64 sweep of the same tensor on the GPU (the FP64
# sweep itself matches the oracle: test_gpu_parity, test_gpu_batch)
BIG_TS = [("n4_j16", [14, 15, 16, 17], 20000, 16), ("n5_j12", [9, 10, 11, 12, 13], 8000, 12),
          ("n5_j16", [9, 10, 11, 12, 13], 8000, 16)]


@pytest.mark.parametrize("case", BIG_TS, ids=[c[0] for c in BIG_TS])
def test_streamed_tensor_core_form(case):
    from oracle_util import random_coo
    name, dims, nnz, J = case
    rng = np.random.default_rng(J * 7 + len(dims))
    idx = random_coo(rng, dims, nnz)
    vals = rng.random(len(idx[0]))
    P = [1] * len(dims)
    c32 = gtk.coo_from_arrays(idx, vals.astype(np.float32), dims=dims)
    c64 = gtk.coo_from_arrays(idx, vals, dims=dims)
    with gtk.create_tensor_blocks(c32, P, J) as tb, gtk.create_tensor_blocks(c32, P, J) as tp, \
            gtk.create_tensor_blocks(c64, P, J) as t64:
        for t in (tb, tp, t64):
            t.init_random(1, 0)
        tb.set_precision("bf16")
        for n in range(len(dims)):
            err = rel_fro(tb.compute_delta(n), tp.compute_delta(n))
            print(f"{name} delta mode {n}: {err:.3e}")
            assert err <= BOUND["bf16"]["delta"], (n, err)
        for s in range(3):
            fb, f64 = tb.sweep(), t64.sweep()
            print(f"{name} sweep {s}: bf16 {fb:.8f} fp64 {f64:.8f} diff {abs(fb - f64):.2e}")
        assert abs(fb - f64) <= BOUND["bf16"]["fit"]
        # the direct fit kernel of the streamed form agrees with the stored-delta fit
        tb.set_core(tb.get_core())
        assert abs(tb.reconstruction() - fb) <= 1e-4
        # and a graph-replayed sweep equals an eager one
        tg_fit = []
        tb.set_graph(True)
        tg_fit = [tb.sweep() for _ in range(2)]
        assert all(np.isfinite(tg_fit))


def test_cli_precision_form(tmp_path):
    """--precision bf16 on the CLI runs the tensor-core form: the fits equal the
    same sweeps through the Python mirror (up to the order of FP64 atomic adds)."""
    import re
    import subprocess

    from gputucker_gb300 import build
    from oracle_util import random_coo, write_tns
    rng = np.random.default_rng(21)
    dims = [30, 35, 40, 45]
    idx = random_coo(rng, dims, 20000)
    vals = rng.random(len(idx[0]))
    f = tmp_path / "t.tns"
    write_tns(f, idx, vals, dtype=0)
    r = subprocess.run([build.CLI, "-i", str(f), "-o", "4", "-r", "10", "-p", "2,1,1,2", "--dtype", "f32",
                        "--precision", "bf16", "--iters", "3", "--tol", "0"], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    fits = [float(x) for x in re.findall(r"^iter \d+\t Fit: (\S+)$", r.stdout, flags=re.M)]
    coo = gtk.parse_from_file(str(f), 4, "f32", rand_seed=1)
    with gtk.create_tensor_blocks(coo, [2, 1, 1, 2], 10) as t:
        t.init_random(1, coo.rand_draws)
        t.set_precision("bf16")
        ref = []
        for _ in range(3):
            t.update_factor_matrices()
            ref.append(t.reconstruction())
    print(fits, ref)
    np.testing.assert_allclose(fits, ref, rtol=0, atol=1e-6)
