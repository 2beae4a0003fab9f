"""Learned warm start: features, the MLP's forward/backward kernels against the
CPU oracle (oracle/warmstart_oracle.py, float64 numpy), training, and what the
trained network gains over uniform [0,1) initialisation.

Tolerances (FP32 outputs vs float64 oracle): features 1e-5 relative to the
feature's scale (FP64 row sums, FP32 result); loss
1e-5 relative; gradient 1e-4 relative Frobenius and per entry 1e-3 relative
(+1e-6 of the largest entry).
"""

import numpy as np
import pytest

import gputucker_gb300 as gtk
from oracle_util import random_coo, ws_oracle

pytestmark = pytest.mark.gpu


def test_features_match_oracle():
    orc = ws_oracle()
    for dims, P, nnz, zipf in (([60, 45, 50], [2, 1, 2], 20000, None), ([30, 25, 20, 28], [1, 2, 1, 2], 15000, 1.2)):
        rng = np.random.default_rng(len(dims))
        idx = random_coo(rng, dims, nnz, zipf=zipf)
        vals = rng.random(len(idx[0])).astype(np.float32)
        coo = gtk.coo_from_arrays(idx, vals, dims=dims)
        with gtk.create_tensor_blocks(coo, P, 4) as t:
            rows = [t.factor_rows(n) for n in range(len(dims))]
            for n in range(len(dims)):
                got = gtk.ws_features(t, n)
                want = orc.row_features(idx, vals, rows, n)
                assert got.shape == want.shape
                scale = np.maximum(np.abs(want).max(axis=0), 1e-6)
                err = np.abs(got - want).max(axis=0) / scale
                assert err.max() <= 1e-5, (n, err)


@pytest.mark.parametrize("order,rank,hidden,B", [(3, 8, 64, 300), (4, 10, 32, 1000), (2, 5, 17, 33)])
def test_gradients_match_oracle(order, rank, hidden, B):
    orc = ws_oracle()
    rng = np.random.default_rng(order * 100 + rank)
    with gtk.WarmStart(order, rank, hidden=hidden, seed=3) as ws:
        F = ws.features
        p = (rng.standard_normal(ws.n_params) * 0.3).astype(np.float32)
        ws.set_params(p)
        x = rng.standard_normal((B, F)).astype(np.float32)
        t = rng.standard_normal((B, rank)).astype(np.float32)
        loss, g = ws.loss_grad(x, t)
        lo, go = orc.loss_grad(p, x, t, F, hidden, rank)
        assert abs(loss - lo) <= 1e-5 * abs(lo)
        assert np.linalg.norm(g - go) <= 1e-4 * np.linalg.norm(go)
        assert np.all(np.abs(g - go) <= 1e-3 * np.abs(go) + 1e-6 * np.abs(go).max())
        y = ws.predict(x)
        yo, _ = orc.forward(p, x, F, hidden, rank)
        assert np.abs(y - yo).max() <= 1e-4 * np.abs(yo).max()


def test_training_fits_a_known_mapping():
    """The forward/backward kernels drive gradient descent on a synthetic
    regression: the loss falls by more than 10x."""
    rng = np.random.default_rng(9)
    with gtk.WarmStart(3, 8, hidden=32, seed=4) as ws:
        F = ws.features
        x = rng.standard_normal((4096, F)).astype(np.float32)
        A = rng.standard_normal((F, 8)).astype(np.float32) / np.sqrt(F)
        t = np.tanh(x @ A).astype(np.float32)
        l0, _ = ws.loss_grad(x, t)
        # train through the public path: examples come from tensors, so drive the
        # optimiser with the host-batch API instead (plain gradient descent here)
        p, _, _ = ws.get_params()
        for _ in range(300):
            _, g = ws.loss_grad(x, t)
            p = p - 0.2 * g
            ws.set_params(p)
        l1, _ = ws.loss_grad(x, t)
        assert l1 <= 0.1 * l0, (l0, l1)


def _planted(dim, nnz, seed):
    return gtk.generate_planted(3, [dim] * 3, nnz, 8, 0.01, "f32", seed=seed)


def test_warm_start_gains_over_random_init():
    """Planted 3-order family (50,000^3, 2M observed entries, rank-8 planted model,
    noise 0.01): train on the factors the plain method converges to (30 sweeps) on
    8 seeds; on 3 held-out seeds the warm start reaches the plain method's fit
    after K = 10 sweeps in at most half the sweeps, and its first sweep is better
    than the plain method's."""
    J, K, dim, nnz = 8, 10, 50_000, 2_000_000
    with gtk.WarmStart(3, J, hidden=64, seed=1) as ws:
        for s in range(8):
            with gtk.create_tensor_blocks(_planted(dim, nnz, 100 + s), [1, 1, 1], J) as t:
                t.init_random(1, 0)
                for _ in range(30):
                    t.sweep()
                ws.add_example(t)
        assert ws.examples() > 0
        loss = ws.train(3000, 4096, 1e-3)
        assert np.isfinite(loss)
        gains = []
        for s in range(3):
            with gtk.create_tensor_blocks(_planted(dim, nnz, 900 + s), [1, 1, 1], J) as t:
                t.init_random(1, 0)
                plain = [t.sweep() for _ in range(K)]
                t.init_random(1, 0)
                ws.apply(t)
                warm = [t.sweep() for _ in range(K)]
            target = plain[-1]
            n_warm = next((i + 1 for i, f in enumerate(warm) if f >= target), K + 1)
            gains.append((K, n_warm, plain[0], warm[0]))
            assert warm[0] > plain[0], (plain, warm)
        assert sum(g[1] for g in gains) <= sum(g[0] for g in gains) / 2, gains


def test_model_save_load_and_cli_init(tmp_path):
    """A trained model saved and loaded predicts the same rows; the CLI's
    --init-model starts from the same factors as WarmStart.apply (its fits equal
    the Python path's)."""
    import re
    import subprocess

    from gputucker_gb300 import build
    coo = gtk.generate_planted(3, [2000, 2100, 2200], 200_000, 4, 0.01, "f64", seed=5)
    with gtk.create_tensor_blocks(coo, [1, 1, 1], 4) as t:
        t.init_random(1, 0)
        for _ in range(5):
            t.sweep()
        ws = gtk.WarmStart(3, 4, hidden=16, seed=2)
        ws.add_example(t)
        ws.train(200, 512, 1e-3)
        path = tmp_path / "model.ws"
        ws.save(path)
        m = gtk.WarmStart.load(path)
        assert (m.order, m.rank, m.hidden) == (3, 4, 16)
        for a, b in zip(ws.get_params(), m.get_params()):
            assert np.array_equal(a, b)
        x = np.random.default_rng(0).random((64, ws.features)).astype(np.float32)
        assert np.array_equal(ws.predict(x), m.predict(x))
        f = tmp_path / "t.tns"
        coo.write_text(f)
        ws.close()
        m.close()
    m = gtk.WarmStart.load(path)
    c2 = gtk.parse_from_file(str(f), 3, "f64", rand_seed=1)
    with gtk.create_tensor_blocks(c2, [1, 1, 1], 4) as t:
        t.init_random(1, c2.rand_draws)
        m.apply(t)
        ref = []
        for _ in range(3):
            t.update_factor_matrices()
            ref.append(t.reconstruction())
    m.close()
    r = subprocess.run([build.CLI, "-i", str(f), "-o", "3", "-r", "4", "-p", "1,1,1", "--iters", "3", "--tol", "0",
                        "--init-model", str(path)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    fits = [float(x) for x in re.findall(r"^iter \d+\t Fit: (\S+)$", r.stdout, flags=re.M)]
    print(fits, ref)
    np.testing.assert_allclose(fits, ref, rtol=0, atol=1e-9)
