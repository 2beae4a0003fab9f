"""Checkpoint dump + resume, and the partition planner on a device.

No reference counterpart for the checkpoint (the reference keeps nothing
between runs): the oracle is an uninterrupted run.  A run saved after s sweeps
and resumed in a fresh handle must give the uninterrupted run's factors and
fits (FP64: 1e-12 fits, 1e-10 factors -- same kernels, only the order of FP64
atomic adds may differ).  The planner's arithmetic is pinned on the CPU against
the reference's optimizer (test_native_cpu.py); here it plans with the
device's real free memory.
"""

import re
import subprocess

import numpy as np
import pytest

import gputucker_gb300 as gtk
from gputucker_gb300 import _native as nat
from oracle_util import random_coo, rel_fro, write_tns

pytestmark = pytest.mark.gpu


def _coo(seed=3, dims=(30, 26, 22, 18), nnz=15000, dtype=np.float64):
    rng = np.random.default_rng(seed)
    idx = random_coo(rng, list(dims), nnz)
    vals = rng.random(len(idx[0])).astype(dtype)
    return gtk.coo_from_arrays(idx, vals, dims=list(dims)), idx, vals


def test_save_resume_matches_uninterrupted(tmp_path):
    coo, _, _ = _coo()
    P, J = [2, 1, 2, 1], 6
    ck = tmp_path / "run.ckpt"
    with gtk.create_tensor_blocks(coo, P, J) as a, gtk.create_tensor_blocks(coo, P, J) as b:
        a.init_random(1, 0)
        fits = [a.sweep(), a.sweep()]
        a.checkpoint_save(ck, fits)
        info = gtk.checkpoint_info(ck)
        assert info == dict(order=4, rank=J, dtype="f64", dims=coo.dims, partition_dims=P, nfits=2)
        saved = b.checkpoint_load(ck)
        assert saved == fits
        for n in range(4):
            assert np.array_equal(b.get_factor(n), a.get_factor(n))
        assert np.array_equal(b.get_core(), a.get_core())
        # the stored-delta fit is not carried over: reconstruction recomputes it
        assert abs(b.reconstruction() - fits[-1]) <= 1e-12
        for _ in range(2):
            fa, fb = a.sweep(), b.sweep()
            assert abs(fa - fb) <= 1e-12
        for n in range(4):
            assert rel_fro(b.get_factor(n), a.get_factor(n)) <= 1e-10
        # fit history capped by the caller: the most recent ones
        assert b.checkpoint_load(ck, fits_cap=1) == fits[-1:]


def test_load_rejects_other_shapes_and_damage(tmp_path):
    coo, _, _ = _coo()
    ck = tmp_path / "x.ckpt"
    with gtk.create_tensor_blocks(coo, [2, 1, 2, 1], 6) as a:
        a.init_random(1, 0)
        a.sweep()
        a.checkpoint_save(ck, [0.5])
        with pytest.raises(gtk.GTKError) as e:  # uninitialised handles cannot be saved
            with gtk.create_tensor_blocks(coo, [1, 1, 1, 1], 6) as u:
                u.checkpoint_save(tmp_path / "y.ckpt")
        assert e.value.code == nat.GTK_ERR_STATE
    for P, J in (([1, 1, 1, 1], 6), ([2, 1, 2, 1], 5)):
        with gtk.create_tensor_blocks(coo, P, J) as b:
            with pytest.raises(gtk.GTKError) as e:
                b.checkpoint_load(ck)
            assert e.value.code == nat.GTK_ERR_ARG
    raw = bytearray(ck.read_bytes())
    with gtk.create_tensor_blocks(coo, [2, 1, 2, 1], 6) as b:
        for damage in ("flip", "truncate", "append"):
            bad = bytearray(raw)
            if damage == "flip":
                bad[len(bad) // 2] ^= 0x40
            elif damage == "truncate":
                bad = bad[:-9]
            else:
                bad += b"\0"
            p = tmp_path / f"{damage}.ckpt"
            p.write_bytes(bytes(bad))
            with pytest.raises(gtk.GTKError) as e:
                b.checkpoint_load(p)
            assert e.value.code == nat.GTK_ERR_PARSE, damage


def test_cli_checkpoint_resume(tmp_path):
    from gputucker_gb300 import build
    rng = np.random.default_rng(8)
    dims = [30, 40, 35]
    idx = random_coo(rng, dims, 6000)
    vals = rng.random(len(idx[0]))
    f = tmp_path / "t.tns"
    write_tns(f, idx, vals, dtype=1)
    base = [build.CLI, "-i", str(f), "-o", "3", "-r", "6", "-p", "2,2,1", "--tol", "0"]

    def fits_of(r):
        assert r.returncode == 0, r.stdout + r.stderr
        return [float(x) for x in re.findall(r"^iter \d+\t Fit: (\S+)$", r.stdout, flags=re.M)]

    full = fits_of(subprocess.run(base + ["--iters", "4"], capture_output=True, text=True, timeout=300))
    first = fits_of(subprocess.run(base + ["--iters", "2", "--checkpoint", str(tmp_path / "c.ckpt")],
                                   capture_output=True, text=True, timeout=300))
    rest = subprocess.run(base + ["--iters", "4", "--resume", str(tmp_path / "c.ckpt")], capture_output=True,
                          text=True, timeout=300)
    assert "Resumed from" in rest.stdout
    rest = fits_of(rest)
    assert len(full) == 4 and len(first) == 2 and len(rest) == 2
    np.testing.assert_allclose(first + rest, full, atol=1e-9)


def test_planner_with_device_memory():
    free, total = gtk.device_memory(0)
    assert 0 < free <= total
    # the 100M-nonzero 4-order tensor fits one GB300: nonzero-based, P_n = 1
    plan = gtk.plan_partition([100_000] * 4, 100_000_000, 10, "f32")
    assert plan["partition_dims"] == [1, 1, 1, 1] and not plan["dimension_based"]
    assert plan["required_bytes"] <= free
    # tucker_decomposition without P_n plans them, as TuckerDecomposition does
    coo, _, _ = _coo(dims=(20, 18, 16), nnz=3000)
    t, fits = gtk.tucker_decomposition(coo, 4, max_iters=2)
    with t:
        assert t.info.partition_dims[:3] == [1, 1, 1]
        assert len(fits) == 2
