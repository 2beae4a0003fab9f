"""Batches of handles swept as one CUDA graph, kernel variants, and the autotuner.

No reference counterpart: the reference decomposes one tensor per process.  The
oracle for a batch is the same handles swept one by one (gtk_sweep on twins made
from the same data and initialisation); for the variants, the default kernel.
Same kernels, so results agree up to the order of FP64 atomic adds in the Gram
rows cut by tile edges: fits within 1e-6 (FP32 data) / 1e-10 (FP64 data),
factors within 1e-4 / 1e-9 relative Frobenius.
"""

import ctypes as C

import numpy as np
import pytest

import gputucker_gb300 as gtk
from gputucker_gb300 import _native as nat
from oracle_util import random_coo, rel_fro

pytestmark = pytest.mark.gpu

# (dims, P, J, nnz, dtype, precision)
CASES = [
    ([30, 25, 28, 20], [2, 1, 2, 1], 10, 20000, np.float32, "plain"),
    ([40, 35, 30], [1, 2, 1], 8, 12000, np.float32, "bf16"),
    ([22, 18, 26], [2, 2, 1], 4, 6000, np.float64, "plain"),
    ([50, 40, 45, 30], [1, 1, 1, 2], 8, 30000, np.float32, "tf32"),
    ([16, 12, 14, 10, 9], [1, 1, 1, 1, 1], 4, 5000, np.float32, "plain"),
]


def _tol(dtype):
    return (1e-6, 1e-4) if dtype == np.float32 else (1e-10, 1e-9)


def _make(case, seed):
    dims, P, J, nnz, dtype, prec = case
    rng = np.random.default_rng(seed)
    idx = random_coo(rng, dims, nnz)
    vals = rng.random(len(idx[0])).astype(dtype)
    coo = gtk.coo_from_arrays(idx, vals, dims=dims)
    pair = []
    for _ in range(2):
        t = gtk.create_tensor_blocks(coo, P, J)
        t.init_random(1, 0)
        if prec != "plain":
            t.set_precision(prec)
        pair.append(t)
    return pair


def test_batch_matches_one_by_one():
    pairs = [_make(c, 40 + i) for i, c in enumerate(CASES)]
    batch_ts = [p[0] for p in pairs]
    solo_ts = [p[1] for p in pairs]
    try:
        with gtk.Batch(batch_ts) as b:
            assert b.kernels() == 0
            for sweep in range(4):  # eager, capture + replay, replays
                fb = b.sweep()
                fs = [t.sweep() for t in solo_ts]
                for i, c in enumerate(CASES):
                    ftol, _ = _tol(c[4])
                    assert abs(fb[i] - fs[i]) <= ftol, (sweep, i, fb[i], fs[i])
                if sweep >= 1:
                    # every mode's fused kernel and solve kernel(s), the fit kernels, the gather
                    assert b.kernels() >= sum(2 * len(c[0]) + 2 for c in CASES) + 1
            for i, c in enumerate(CASES):
                _, rtol = _tol(c[4])
                for n in range(len(c[0])):
                    assert rel_fro(batch_ts[i].get_factor(n), solo_ts[i].get_factor(n)) <= rtol, (i, n)
                # the stored-delta fit of the batch sweep is the handle's reconstruction
                assert abs(batch_ts[i].reconstruction() - fb[i]) <= _tol(c[4])[0]
    finally:
        for p in pairs:
            for t in p:
                t.close()


def test_batch_sees_changes_between_sweeps():
    """Factor/core contents and a precision change between replays are picked up."""
    pairs = [_make(c, 60 + i) for i, c in enumerate(CASES[:2])]
    try:
        with gtk.Batch([p[0] for p in pairs]) as b:
            b.sweep()
            b.sweep()
            for tb, ts in pairs:
                ts.sweep()
                ts.sweep()
            k0 = b.kernels()
            # halve the core of tensor 0, switch tensor 1 to TF32, mirror on the twins
            tb, ts = pairs[0]
            g = tb.get_core() * 0.5
            tb.set_core(g)
            ts.set_core(g)
            for n in range(len(CASES[0][0])):
                ts.set_factor(n, tb.get_factor(n))
            tb1, ts1 = pairs[1]
            for t in (tb1, ts1):
                t.set_precision("tf32")
            for n in range(len(CASES[1][0])):
                ts1.set_factor(n, tb1.get_factor(n))
            ts1.set_core(tb1.get_core())
            fb = b.sweep()
            fs = [ts.sweep(), ts1.sweep()]
            assert np.all(np.abs(fb - np.array(fs)) <= 1e-6), (fb, fs)
            assert b.kernels() >= k0 - 2  # recaptured (TF32 and BF16 launch the same kernel count)
    finally:
        for p in pairs:
            for t in p:
                t.close()


def test_batch_rejects_duplicates_and_empty():
    t, u = _make(CASES[2], 5)
    try:
        lib = nat.load()
        tab = (C.c_void_p * 2)(t.handle, t.handle)
        h = C.c_void_p()
        assert lib.gtk_batch_create(tab, 2, C.byref(h)) == nat.GTK_ERR_ARG
        assert lib.gtk_batch_create(tab, 0, C.byref(h)) == nat.GTK_ERR_ARG
    finally:
        t.close()
        u.close()


@pytest.mark.parametrize("ci", [0, 2, 4])
def test_variants_agree(ci):
    """Every SIMT variant gives the default kernel's sweep."""
    case = CASES[ci]
    ftol, rtol = _tol(case[4])
    ref, _ = _make(case, 80)
    f_ref = [ref.sweep() for _ in range(2)]
    try:
        for v in ("simt2", "simt1", "generic"):
            t, u = _make(case, 80)
            u.close()
            t.set_kernel_variant(v)
            assert t.kernel_variant() == v
            f = [t.sweep() for _ in range(2)]
            assert np.all(np.abs(np.array(f) - f_ref) <= ftol), (v, f, f_ref)
            for n in range(len(case[0])):
                assert rel_fro(t.get_factor(n), ref.get_factor(n)) <= rtol, (v, n)
            t.close()
    finally:
        ref.close()


def test_tensor_core_variant_needs_precision_form():
    t, u = _make(CASES[0], 90)
    try:
        with pytest.raises(gtk.GTKError):
            t.set_kernel_variant("tensor_core")
        t.set_precision("bf16")
        t.set_kernel_variant("tensor_core")
        t.set_precision("plain")  # drops the tensor-core variant
        assert t.kernel_variant() == "auto"
        assert abs(t.sweep() - u.sweep()) <= 1e-6
    finally:
        t.close()
        u.close()


@pytest.mark.parametrize("ci", [0, 1, 2])
def test_autotune_keeps_factors_and_caches(ci):
    case = CASES[ci]
    ftol, _ = _tol(case[4])
    t, u = _make(case, 100 + ci)
    try:
        before = [t.get_factor(n) for n in range(len(case[0]))]
        v = t.autotune()
        assert v in ("simt2", "simt1", "tensor_core")
        if case[5] == "plain":
            assert v != "tensor_core"
        for n in range(len(case[0])):
            assert np.array_equal(t.get_factor(n), before[n])
        # the tuned handle sweeps like a handle with the same variant forced
        u.set_kernel_variant(v)
        assert abs(t.sweep() - u.sweep()) <= ftol
        # a second handle of the same shape class takes the cached choice
        w, x = _make(case, 100 + ci)
        x.close()
        assert w.autotune() == v
        w.close()
    finally:
        t.close()
        u.close()


@pytest.mark.parametrize("prec", ["plain", "bf16"])
def test_tile_shape_ctas_per_sm(prec):
    """The tile-shape axis: one CTA per SM (each CTA sweeps ~20 tiles of the
    3,125 here) gives the default grid's results up to the order of the Gram
    rows' FP64 atomic adds; a batch re-captures its graph when a member's shape
    changes; the autotuner's choice is one of the shapes it times."""
    case = ([200, 150, 180, 120], [2, 1, 2, 1], 10, 400000, np.float32, prec)
    ftol, rtol = _tol(np.float32)
    if prec == "bf16":  # FP32 row solves of weakly determined rank-10 factors (uniform data)
        rtol = 1e-3
    t, u = _make(case, 77)
    try:
        assert t.ctas_per_sm() == 0
        with pytest.raises(nat.GTKError):
            t.set_ctas_per_sm(-1)
        t.set_ctas_per_sm(1)
        assert t.ctas_per_sm() == 1
        ft, fu = t.sweep(), u.sweep()
        assert abs(ft - fu) <= ftol, (ft, fu)
        for n in range(4):
            assert rel_fro(t.get_factor(n), u.get_factor(n)) <= rtol, n
        ft, fu = t.sweep(), u.sweep()
        assert abs(ft - fu) <= ftol, (ft, fu)
        t.set_ctas_per_sm(0)
        u.init_random(1, 0)
        with gtk.Batch([t]) as b:
            t.init_random(1, 0)
            f0 = [b.sweep()[0] for _ in range(3)]
            t.set_ctas_per_sm(2)  # the next batch sweep captures a new graph
            t.init_random(1, 0)
            f2 = [b.sweep()[0] for _ in range(3)]
        fu = [u.sweep() for _ in range(3)]
        assert np.allclose(f0, fu, rtol=0, atol=ftol) and np.allclose(f2, fu, rtol=0, atol=ftol), (f0, f2, fu)
        u.autotune()
        assert u.ctas_per_sm() in (0, 1, 2)
    finally:
        t.close()
        u.close()


@pytest.mark.parametrize("N,J", [(4, 16), (5, 12), (5, 16)])
def test_streamed_core_kernels(N, J):
    """Cores too large for shared memory (J^(N-1) * J values) stream through it in
    chunks: the FP32 sweep of each variant agrees with the FP64 sweep (generic kernel)
    of the same well-determined tensor (every factor row sees hundreds of nonzeros)."""
    dims = [14] * N
    rng = np.random.default_rng(7 + N * J)
    idx = random_coo(rng, dims, 30000)
    vals = rng.random(len(idx[0]))
    ts = {}
    try:
        for dt in (np.float64, np.float32):
            coo = gtk.coo_from_arrays(idx, vals.astype(dt), dims=dims)
            for v in (["generic"] if dt == np.float64 else ["simt2", "simt1", "generic"]):
                t = gtk.create_tensor_blocks(coo, [1] * N, J)
                t.init_random(1, 0)
                t.set_kernel_variant(v)
                ts[(dt, v)] = t
        fits = {k: [t.sweep() for _ in range(2)] for k, t in ts.items()}
        ref = fits[(np.float64, "generic")]
        for v in ("simt2", "simt1", "generic"):
            f = fits[(np.float32, v)]
            assert np.all(np.abs(np.array(f) - ref) <= 2e-5), (v, f, ref)
            for n in range(N):
                assert rel_fro(ts[(np.float32, v)].get_factor(n), ts[(np.float64, "generic")].get_factor(n)) <= 1e-3
        # the direct fit kernel (no stored delta) of the streamed form
        t = ts[(np.float32, "simt2")]
        g = t.get_core()
        t.set_core(g)  # a new core invalidates the stored delta: the fit is recomputed
        assert abs(t.reconstruction() - fits[(np.float32, "simt2")][-1]) <= 2e-5
    finally:
        for t in ts.values():
            t.close()


# FP32 handles of every kernel family: SIMT (orders 3-5), tcgen05 BF16/TF32, the
# streamed-core tcgen05 form (order 5; order 4 at rank 16)
FUSED = [
    ([30, 25, 28, 20], [2, 1, 2, 1], 10, 20000, np.float32, "plain"),
    ([40, 35, 30], [1, 2, 1], 8, 12000, np.float32, "bf16"),
    ([50, 40, 45, 30], [1, 1, 1, 2], 8, 30000, np.float32, "tf32"),
    ([16, 12, 14, 10, 9], [1, 1, 1, 1, 1], 4, 5000, np.float32, "plain"),
    ([14, 12, 13, 11, 10], [1, 1, 1, 1, 1], 8, 8000, np.float32, "bf16"),
    ([30, 28, 26, 24], [1, 1, 1, 1], 16, 20000, np.float32, "bf16"),
    ([60, 50, 40], [2, 1, 1], 12, 15000, np.float32, "plain"),
    ([45, 40, 35], [1, 1, 1], 4, 9000, np.float32, "plain"),
    # rank 10 on the tensor cores: rows of 12 floats, read from the gather copies
    # that the fused form refreshes in its per-level zeroing kernel
    ([40, 36, 30, 28], [1, 1, 2, 1], 10, 20000, np.float32, "bf16"),
]


def test_fused_batch_few_launches_match_one_by_one_and_oracle(monkeypatch):
    """The fused sweep (GTK_BATCH_FUSED=1; per mode index: one zeroing kernel, one
    launch per update kernel class, the batched row solves; one fit and one
    reduction) against the same handles swept one by one, against the default
    per-handle graph, and three members against the FP64 oracle."""
    from oracle_util import Oracle
    monkeypatch.setenv("GTK_BATCH_FUSED", "1")
    pairs = [_make(c, 200 + i) for i, c in enumerate(FUSED)]
    batch_ts = [p[0] for p in pairs]
    solo_ts = [p[1] for p in pairs]
    try:
        with gtk.Batch(batch_ts) as b:
            for sweep in range(3):
                fb = b.sweep()
                fs = [t.sweep() for t in solo_ts]
                assert np.all(np.abs(fb - np.array(fs)) <= 1e-6), (sweep, fb, fs)
            k_fused = b.kernels()
            maxN = max(len(c[0]) for c in FUSED)
            classes = len({(len(c[0]), c[2], c[5]) for c in FUSED})
            solve_groups = len({(c[2], c[5] != "plain") for c in FUSED})
            # per mode index: zeroing + at most one launch per class + one row solve per (rank,
            # path) + the FP64 and LU list passes; then fit + reduction
            assert 0 < k_fused <= maxN * (1 + classes + solve_groups + 2) + 2, k_fused
            for i, c in enumerate(FUSED):
                for n in range(len(c[0])):
                    assert rel_fro(batch_ts[i].get_factor(n), solo_ts[i].get_factor(n)) <= 1e-4, (i, n)
        # the per-handle graph gives the same sweep with one launch chain per handle
        monkeypatch.setenv("GTK_BATCH_FUSED", "0")
        for t in batch_ts:
            t.init_random(1, 0)
        with gtk.Batch(batch_ts) as b2:
            f2 = [b2.sweep() for _ in range(2)][-1]
            # 2N + 2 or more per handle, against per-class launches (the gap grows with the handle count)
            assert b2.kernels() > k_fused
        for t in batch_ts:
            t.init_random(1, 0)
        monkeypatch.setenv("GTK_BATCH_FUSED", "1")
        with gtk.Batch(batch_ts) as b3:
            f3 = [b3.sweep() for _ in range(2)][-1]
        assert np.all(np.abs(f3 - f2) <= 1e-6), (f3, f2)
        # three members against the FP64 oracle after 3 fused sweeps of the same data
        # and initialisation: plain FP32 within the FP32 bound, BF16 / TF32 within theirs
        for t in batch_ts:
            t.init_random(1, 0)
        with gtk.Batch(batch_ts) as b4:
            f4 = [b4.sweep() for _ in range(3)][-1]
        for i, tol in ((0, 1e-4), (1, 1e-3), (2, 2e-4)):
            dims, P, J, nnz, dtype, prec = FUSED[i]
            rng = np.random.default_rng(200 + i)
            idx = random_coo(rng, dims, nnz)
            vals = rng.random(len(idx[0])).astype(dtype)
            ora = Oracle(1, idx, vals.astype(np.float64), dims, P, J)
            ora.init_random(1, 0)
            fo = [ora.sweep()["fit64"] for _ in range(3)][-1]
            assert abs(f4[i] - fo) <= tol, (i, prec, f4[i], fo)
    finally:
        for p in pairs:
            for t in p:
                t.close()
