"""The public API end to end on the GPU: files -> decomposition, the CLI, errors."""

import glob
import os
import re
import subprocess

import numpy as np
import pytest

import gputucker_gb300 as gtk
from gputucker_gb300 import _native as nat
from oracle_util import ROOT, Oracle, random_coo, rel_fro, write_tns

pytestmark = pytest.mark.gpu

GOLDEN = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "*.npz")))


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_golden_through_public_api(path):
    """Reference-produced fixtures: parse -> blocks -> init (continuing the parser's
    rand() stream) -> 3 sweeps, through the C ABI."""
    g = np.load(path)
    dtype = int(g["dtype"])
    N = len(g["dims"])
    P = [int(x) for x in g["P"]]
    J = int(g["J"])
    coo = gtk.parse_from_file(path[:-4] + ".tns", N, dtype, rand_seed=1)
    assert coo.rand_draws == int(g["skip"])
    with gtk.create_tensor_blocks(coo, P, J) as t:
        for b in range(t.info.block_count):
            coord, idx, vals = t.block(b)
            s, e = int(g["blk_ptr"][b]), int(g["blk_ptr"][b + 1])
            assert coord == [int(x) for x in g["blk_coord"][b]]
            for n in range(N):
                np.testing.assert_array_equal(idx[n], g[f"idx{n}"][s:e])
                cnt, where = t.segments(b, n)
                rows = t.info.block_dims[n] + 1
                np.testing.assert_array_equal(cnt, g[f"count{n}"][b * rows:(b + 1) * rows])
                np.testing.assert_array_equal(where, g[f"where{n}"][s:e])
            np.testing.assert_array_equal(vals, g["vals"][s:e])
        t.init_random(1, coo.rand_draws)
        for n in range(N):
            np.testing.assert_array_equal(t.get_factor(n), g[f"fac0_{n}"])
        np.testing.assert_array_equal(t.get_core(), g["core"])
        for s in range(3):
            t.update_factor_matrices()
            fit = t.reconstruction()
            if dtype == 1:
                for n in range(N):
                    assert rel_fro(t.get_factor(n), g[f"fac{s + 1}_{n}"]) <= 1e-9
                # the reference sums the error in value_t serially; the fixtures are FP64 here
                assert abs(fit - float(g[f"fit{s + 1}"])) <= 1e-9
            else:
                # FP32: the reference's fit sums the error in float; within its rounding
                assert abs(fit - float(g[f"fit{s + 1}"])) <= 1e-4


def test_cli_end_to_end(tmp_path):
    from gputucker_gb300 import build
    rng = np.random.default_rng(5)
    dims = [30, 40, 35]
    idx = random_coo(rng, dims, 6000)
    vals = rng.random(len(idx[0]))
    f = tmp_path / "t.tns"
    write_tns(f, idx, vals, dtype=1)
    r = subprocess.run([build.CLI, "-i", str(f), "-o", "3", "-r", "6", "-p", "2,2,1", "--iters", "3",
                        "--write-factors", str(tmp_path / "A")], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    fits = [float(x) for x in re.findall(r"^iter \d+\t Fit: (\S+)$", r.stdout, flags=re.M)]
    ora = Oracle(1, idx, vals, dims, [2, 2, 1], 6)
    ora.init_random(1, 0)
    ofits = []
    for it in range(3):
        ofits.append(ora.sweep()["fit64"])
        if it > 0 and abs(ofits[-1] - ofits[-2]) <= 1e-4:
            break
    assert len(fits) == len(ofits)
    np.testing.assert_allclose(fits, ofits, atol=1e-9)
    a0 = np.loadtxt(tmp_path / "A0.txt")
    assert rel_fro(a0, ora.get_factor(0)[:dims[0]]) <= 1e-9


def test_state_error_before_init():
    coo = gtk.coo_from_arrays([np.arange(10, dtype=np.uint32)] * 3, np.ones(10))
    with gtk.create_tensor_blocks(coo, [1, 1, 1], 4) as t:
        with pytest.raises(gtk.GTKError) as e:
            t.update_factor_matrices()
        assert e.value.code == nat.GTK_ERR_STATE
        with pytest.raises(gtk.GTKError) as e:
            t.update_mode(3)
        assert e.value.code in (nat.GTK_ERR_STATE, nat.GTK_ERR_ARG)


def test_memory_cap_reports_oom(monkeypatch):
    """An allocation cap (GTK_DEVICE_MEMORY_CAP) stands in for an exhausted HBM: a cap
    below the resident layout gives the streamed layout, a cap below even the
    factors and Gram/RHS that the streamed layout keeps resident is GTK_ERR_OOM."""
    coo = gtk.generate(3, [1000] * 3, 100_000, "uniform", 0, "uniform", "f32", seed=1)
    monkeypatch.setenv("GTK_DEVICE_MEMORY_CAP", str(1 << 16))
    with pytest.raises(gtk.GTKError) as e:
        gtk.create_tensor_blocks(coo, [1, 1, 1], 8)
    assert e.value.code == nat.GTK_ERR_OOM
    monkeypatch.setenv("GTK_DEVICE_MEMORY_CAP", str(1 << 20))
    with gtk.create_tensor_blocks(coo, [1, 1, 1], 8) as t:
        assert t.info.streamed and t.info.device_bytes <= (1 << 20)
    monkeypatch.delenv("GTK_DEVICE_MEMORY_CAP")
    with gtk.create_tensor_blocks(coo, [1, 1, 1], 8) as t:
        assert not t.info.streamed and t.info.device_bytes > (1 << 20)


def test_direct_fit_after_set_factor_matches_stored_delta_fit():
    """The fit from the last mode's stored delta equals the direct reconstruction."""
    rng = np.random.default_rng(2)
    dims = [25, 30, 20, 22]
    idx = random_coo(rng, dims, 8000)
    vals = rng.random(len(idx[0]))
    coo = gtk.coo_from_arrays(idx, vals, dims=dims)
    with gtk.create_tensor_blocks(coo, [2, 1, 2, 1], 6) as t:
        t.init_random(1, 0)
        t.update_factor_matrices()
        f_stored = t.reconstruction()
        t.set_factor(0, t.get_factor(0))  # invalidates the stored delta
        f_direct = t.reconstruction()
        assert abs(f_stored - f_direct) <= 1e-10


def test_profile_and_timer():
    coo = gtk.generate(3, [500] * 3, 50_000, "zipf", 1.1, "uniform", "f32", seed=4)
    with gtk.create_tensor_blocks(coo, [1, 1, 1], 8) as t:
        t.init_random(1, 0)
        t.profile(True)
        t.timer_begin()
        t.update_factor_matrices()
        t.reconstruction()
        ms = t.timer_end()
        k_ms, k_n = t.profile_read(0)
        s_ms, s_n = t.profile_read(1)
        assert k_n == 3 and s_n == 3 and 0 < k_ms <= ms * 1.5 and ms > 0
        t.profile_reset()
        assert t.profile_read(3) == (0.0, 0)


def test_compute_delta_block_major_order():
    """gtk_compute_delta returns delta in the reference's block-major order."""
    rng = np.random.default_rng(9)
    dims = [20, 21, 22]
    idx = random_coo(rng, dims, 3000)
    vals = rng.random(len(idx[0]))
    coo = gtk.coo_from_arrays(idx, vals, dims=dims)
    P = [2, 3, 2]
    with gtk.create_tensor_blocks(coo, P, 5) as t:
        ora = Oracle(1, idx, vals, dims, P, 5)
        t.init_random(1, 0)
        ora.init_random(1, 0)
        for n in range(3):
            assert rel_fro(t.compute_delta(n), ora.delta(n)) <= 1e-13


@pytest.mark.parametrize("prec", ["plain", "bf16"])
def test_graph_replay_matches_eager(prec):
    """gtk_set_graph: the captured sweep replays the same kernels as the eager one."""
    rng = np.random.default_rng(12)
    dims = [30, 25, 28, 20]
    idx = random_coo(rng, dims, 20000)
    vals = rng.random(len(idx[0])).astype(np.float32)
    coo = gtk.coo_from_arrays(idx, vals, dims=dims)
    with gtk.create_tensor_blocks(coo, [2, 1, 2, 1], 10) as te, gtk.create_tensor_blocks(coo, [2, 1, 2, 1], 10) as tg:
        for t in (te, tg):
            t.init_random(1, 0)
            t.set_precision(prec)
        tg.set_graph(True)
        for _ in range(3):
            fe = te.sweep()
            fg = tg.sweep()
            # same kernels; only the order of FP64 atomic adds in the Gram may differ
            assert abs(fe - fg) <= 1e-6
        for n in range(4):
            assert rel_fro(tg.get_factor(n), te.get_factor(n)) <= 1e-4
        tg.profile_reset()
        tg.sweep()
        assert tg.profile_read(4)[1] >= 2 * 4 + 2
        # contents may change between replays: a new core is picked up
        g = tg.get_core() * 0.5
        tg.set_core(g)
        te.set_core(g)
        for n in range(4):
            te.set_factor(n, tg.get_factor(n))
        assert abs(te.sweep() - tg.sweep()) <= 1e-6


def test_cached_device_blocks_are_reused_cleanly():
    """A handle created after another of the same shape was destroyed gets the
    cached blocks back (stale contents): its sweeps equal the first handle's; the
    cached bytes count as free, and releasing them returns them to the driver."""
    coo = gtk.generate(4, [3000] * 4, 400_000, "zipf", 1.1, "uniform", "f32", seed=3)
    fits = []
    for _ in range(2):
        with gtk.create_tensor_blocks(coo, [2, 2, 2, 2], 8) as t:
            t.init_random(1, 0)
            t.set_precision("bf16")
            fits.append([t.sweep() for _ in range(2)])
    np.testing.assert_allclose(fits[0], fits[1], rtol=0, atol=1e-6)  # up to the order of FP64 atomic adds
    free_cached, total = gtk.device_memory()
    gtk.release_cached_memory()
    free_after, _ = gtk.device_memory()
    assert abs(free_after - free_cached) <= total // 100, (free_cached, free_after)


def test_host_direct_read_matches_upload(monkeypatch):
    """The partition reading the host COO in place (where the device reaches pageable
    host memory) and the one reading an uploaded copy give identical handles."""
    from oracle_util import random_coo
    rng = np.random.default_rng(9)
    dims, P = [60, 50, 40, 30], [2, 2, 1, 3]
    idx = random_coo(rng, dims, 20_000, distinct=True, zipf=1.1)
    vals = rng.random(len(idx[0])).astype(np.float32)
    coo = gtk.coo_from_arrays(idx, vals, dims=dims)
    monkeypatch.setenv("GTK_HOST_DIRECT", "0")
    with gtk.create_tensor_blocks(coo, P, 8) as up:
        assert not up.info.host_direct
        monkeypatch.delenv("GTK_HOST_DIRECT")
        with gtk.create_tensor_blocks(coo, P, 8) as dr:
            print("host_direct", dr.info.host_direct)
            assert dr.info.norm == up.info.norm
            for b in range(dr.info.block_count):
                c1, i1, v1 = dr.block(b)
                c2, i2, v2 = up.block(b)
                assert c1 == c2 and np.array_equal(v1, v2)
                assert all(np.array_equal(x, y) for x, y in zip(i1, i2))
                for n in range(4):
                    s1, s2 = dr.segments(b, n), up.segments(b, n)
                    assert np.array_equal(s1[0], s2[0]) and np.array_equal(s1[1], s2[1])
            for t in (dr, up):
                t.init_random(1, 0)
            assert abs(dr.sweep() - up.sweep()) <= 1e-6  # FP64 atomic adds in either order
