"""The optional core update (no reference counterpart: GPUTucker keeps G fixed).

gtk_update_core solves (Phi^T Phi + lambda I) vec(G) = Phi^T x by conjugate
gradients, Phi's rows being the Kronecker products a_0[i_0] (x) ... (x) a_{N-1}[i_{N-1}]
of each nonzero's factor rows (mode N-1 fastest, the core's linear order).  Checked
against the same normal equations formed explicitly and solved by numpy in FP64.
"""

import numpy as np
import pytest

import gputucker_gb300 as gtk
from oracle_util import random_coo

pytestmark = pytest.mark.gpu

LAMBDA = float(np.float32(1e-4))  # (double)0.0001f


def explicit_system(idx, vals, facs, J):
    """Phi (nnz x J^N) and the exact regularised least-squares core."""
    rows = []
    for t in range(len(vals)):
        r = np.ones(1)
        for n, f in enumerate(facs):
            r = np.kron(r, f[idx[n][t]].astype(np.float64))
        rows.append(r)
    phi = np.array(rows)
    x = np.asarray(vals, np.float64)
    H = phi.T @ phi + LAMBDA * np.eye(phi.shape[1])
    return phi, x, np.linalg.solve(H, phi.T @ x)


def objective(phi, x, g):
    r = x - phi @ g
    return float(r @ r + LAMBDA * g @ g)


CASES = [("n3_j3", [12, 13, 14], 1500, [1, 2, 1], 3), ("n4_j3", [9, 10, 11, 12], 3000, [2, 1, 1, 2], 3),
         ("n2_j5", [30, 40], 900, [2, 2], 5), ("n5_j2", [6, 7, 8, 9, 10], 2500, [1, 1, 2, 1, 1], 2)]


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_core_update_fp64_matches_exact_least_squares(case):
    name, dims, nnz, P, J = case
    rng = np.random.default_rng(len(dims) * 100 + J)
    idx = random_coo(rng, dims, nnz)
    vals = rng.random(len(idx[0]))
    with gtk.create_tensor_blocks(gtk.coo_from_arrays(idx, vals, dims=dims), P, J) as t:
        t.init_random(1, 0)
        t.sweep()  # factors of one sweep, so that the system is not the initial one
        facs = [t.get_factor(n) for n in range(len(dims))]
        phi, x, g_star = explicit_system(idx, vals, facs, J)
        f0 = objective(phi, x, t.get_core().ravel().astype(np.float64))
        steps, res = t.update_core(cg_iters=4 * J ** len(dims))
        g = t.get_core().ravel()
        rel = np.linalg.norm(g - g_star) / np.linalg.norm(g_star)
        print(f"{name}: {steps} CG steps, residual {res:.2e}, |g - g*| / |g*| = {rel:.2e}, "
              f"objective {f0:.6e} -> {objective(phi, x, g):.6e} (exact {objective(phi, x, g_star):.6e})")
        # the objective to 1e-10 of the exact optimum; the core itself to 1e-5 (the
        # five-factor case is the worst conditioned)
        assert objective(phi, x, g) <= objective(phi, x, g_star) * (1 + 1e-10)
        assert rel <= 1e-5, rel
        # the factors are untouched and the next sweep runs on the new core
        for n in range(len(dims)):
            assert np.array_equal(t.get_factor(n), facs[n])
        assert np.isfinite(t.sweep())


@pytest.mark.parametrize("prec", ["plain", "bf16"])
def test_core_update_fp32_tracks_fp64(prec):
    """FP32 tensors: the same system (factors and starting core copied into an FP64
    handle) after the same number of CG steps.  With positive factors the normal
    equations are ill-conditioned and 30 steps close only part of the gap in FP64
    too (measured: 984.8 -> 965.0 against the optimum 954.4; FP32 965.9); the FP32
    products with Phi^T Phi (FP32 delta, products of five factors, partial sums
    over 1024 nonzeros) keep the FP32 objective within 5 % of the initial gap of
    the FP64 one, and both improve on the starting core."""
    dims, nnz, P, J = [20, 21, 22, 23], 12000, [2, 1, 1, 2], 4
    rng = np.random.default_rng(7)
    idx = random_coo(rng, dims, nnz)
    vals = rng.random(len(idx[0])).astype(np.float32)
    with gtk.create_tensor_blocks(gtk.coo_from_arrays(idx, vals, dims=dims), P, J) as t, \
            gtk.create_tensor_blocks(gtk.coo_from_arrays(idx, vals.astype(np.float64), dims=dims), P, J) as t64:
        t.init_random(1, 0)
        t.set_precision(prec)
        t.sweep()
        facs = [t.get_factor(n) for n in range(len(dims))]
        core0 = t.get_core()
        t64.init_random(1, 0)
        for n in range(len(dims)):
            t64.set_factor(n, facs[n].astype(np.float64))
        t64.set_core(core0.astype(np.float64))
        phi, x, g_star = explicit_system(idx, vals, facs, J)
        f0 = objective(phi, x, core0.ravel().astype(np.float64))
        f_star = objective(phi, x, g_star)
        fit0 = t.reconstruction()
        steps, res = t.update_core(cg_iters=30)
        s64, res64 = t64.update_core(cg_iters=30)
        f32 = objective(phi, x, t.get_core().ravel().astype(np.float64))
        f64 = objective(phi, x, t64.get_core().ravel())
        fit1 = t.reconstruction()
        print(f"{prec}: objective {f0:.6e} -> FP32 {f32:.6e} ({steps} steps, residual {res:.1e}), "
              f"FP64 {f64:.6e} ({s64} steps, residual {res64:.1e}), exact {f_star:.6e}; fit {fit0:.6f} -> {fit1:.6f}")
        assert f32 < f0 and f64 < f0
        assert f32 - f64 <= 0.05 * (f0 - f_star), (f0, f32, f64, f_star)
        assert fit1 >= fit0 - 1e-6
        assert np.isfinite(t.sweep())  # sweeps go on in the handle's own form


def test_core_update_rejects_large_cores():
    dims, J = [30, 31, 32, 33], 20  # 20^4 = 160,000 core entries
    rng = np.random.default_rng(3)
    idx = random_coo(rng, dims, 2000)
    vals = rng.random(len(idx[0])).astype(np.float32)
    with gtk.create_tensor_blocks(gtk.coo_from_arrays(idx, vals, dims=dims), [1] * 4, J) as t:
        t.init_random(1, 0)
        core = t.get_core()
        with pytest.raises(gtk.GTKError) as e:
            t.update_core(3)
        assert e.value.code == gtk._native.GTK_ERR_UNSUPPORTED
        assert np.array_equal(t.get_core(), core)


def test_cli_core_update(tmp_path):
    """--core-update K: the CLI's sweeps with K CG steps of the core after each
    sweep's factor updates equal the same steps through the Python mirror."""
    import re
    import subprocess

    from gputucker_gb300 import build
    from oracle_util import write_tns
    rng = np.random.default_rng(11)
    dims = [25, 30, 35]
    idx = random_coo(rng, dims, 5000)
    vals = rng.random(len(idx[0]))
    f = tmp_path / "t.tns"
    write_tns(f, idx, vals, dtype=1)
    r = subprocess.run([build.CLI, "-i", str(f), "-o", "3", "-r", "4", "-p", "1,1,1", "--iters", "3", "--tol", "0",
                        "--core-update", "8"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert len(re.findall(r"^Core Time", r.stdout, flags=re.M)) == 3
    fits = [float(x) for x in re.findall(r"^iter \d+\t Fit: (\S+)$", r.stdout, flags=re.M)]
    coo = gtk.parse_from_file(str(f), 3, "f64", rand_seed=1)
    with gtk.create_tensor_blocks(coo, [1, 1, 1], 4) as t:
        t.init_random(1, coo.rand_draws)
        ref = []
        for _ in range(3):
            t.update_factor_matrices()
            t.update_core(8)
            ref.append(t.reconstruction())
    print(fits, ref)
    np.testing.assert_allclose(fits, ref, rtol=0, atol=1e-9)
