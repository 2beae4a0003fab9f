"""The oracle itself, pinned before it is trusted (CPU only).

1. glibc rand() replay against the C library's own rand().
2. The oracle against the committed golden fixtures, which were produced by the
   reference's own host code (tests/golden/make_golden.py).
3. Where the reference-compiled checker exists (oracle/_ref, built from the
   reference sources in this container), the oracle against it on more cases.
"""

import ctypes as C
import glob
import os

import numpy as np
import pytest

from oracle_util import NPDT, Oracle, Ref, glibc_rand, ora_parse, random_coo, ref_available, rel_fro, write_tns

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


@pytest.mark.parametrize("seed", [0, 1, 2, 42, 123456789, 2**31 + 5, 2**32 - 1])
def test_glibc_rand_replay(seed):
    libc = C.CDLL("libc.so.6")
    libc.srand.argtypes = [C.c_uint]
    libc.srand(seed)
    want = np.array([libc.rand() for _ in range(2000)], np.int32)
    np.testing.assert_array_equal(glibc_rand(seed, 2000), want)
    np.testing.assert_array_equal(glibc_rand(seed, 500, skip=1500), want[1500:])


def test_unseeded_stream_first_draw():
    # the reference never seeds rand(); srand(1) and srand(0) give that stream
    assert glibc_rand(1, 1)[0] == 1804289383
    assert glibc_rand(0, 1)[0] == 1804289383


def _golden(path):
    g = np.load(path)
    name = os.path.basename(path)[:-4]
    return name, g, path[:-4] + ".tns"


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_oracle_against_golden(path):
    name, g, tns = _golden(path)
    dtype = int(g["dtype"])
    dims = [int(x) for x in g["dims"]]
    N = len(dims)
    P = [int(x) for x in g["P"]]
    J = int(g["J"])
    data = open(tns, "rb").read()
    rc, idx, vals, pdims, draws = ora_parse(data, N, dtype, seed=1)
    assert rc == 0
    assert pdims == dims
    assert draws == int(g["skip"])
    for n in range(N):
        np.testing.assert_array_equal(idx[n], g[f"parsed_idx{n}"])
    np.testing.assert_array_equal(vals, g["parsed_vals"])
    o = Oracle(dtype, idx, vals, dims, P, J)
    part = o.partition()
    np.testing.assert_array_equal(part["blk_ptr"], g["blk_ptr"])
    np.testing.assert_array_equal(part["blk_coord"], g["blk_coord"])
    np.testing.assert_array_equal(part["vals"], g["vals"])
    for n in range(N):
        np.testing.assert_array_equal(part["idx"][n], g[f"idx{n}"])
        np.testing.assert_array_equal(part["count"][n], g[f"count{n}"])
        np.testing.assert_array_equal(part["where"][n], g[f"where{n}"])
    assert o.norm_ref == pytest.approx(float(g["norm"]), rel=0, abs=0)
    o.init_random(1, int(g["skip"]))
    for n in range(N):
        np.testing.assert_array_equal(o.get_factor(n), g[f"fac0_{n}"])
        np.testing.assert_array_equal(o.delta(n), g[f"delta0_{n}"])  # same loop order: bit-exact
    np.testing.assert_array_equal(o.get_core(), g["core"])
    for s in range(3):
        f = o.sweep()
        for n in range(N):
            # float: bit-exact (same order, same LU); double: Eigen's blocked LU rounds differently
            tol = 0.0 if dtype == 0 else 1e-11
            assert rel_fro(o.get_factor(n), g[f"fac{s + 1}_{n}"]) <= tol
        assert abs(f["fit_ref"] - float(g[f"fit{s + 1}"])) <= (0.0 if dtype == 0 else 1e-12)


needs_ref = pytest.mark.skipif(not ref_available(), reason="reference-compiled checker not built here")

PIN_CASES = [
    ("pin_n3_zipf_f32", [50, 60, 40], 5000, [2, 2, 2], 8, 0, 1.4),
    ("pin_n4_f64", [20, 18, 16, 22], 3000, [2, 1, 2, 1], 6, 1, None),
    ("pin_n5_f32", [8, 9, 10, 11, 12], 2000, [1, 1, 1, 2, 1], 4, 0, None),
    ("pin_n2_f64", [60, 70], 900, [3, 2], 9, 1, None),
]


@needs_ref
@pytest.mark.parametrize("case", PIN_CASES, ids=[c[0] for c in PIN_CASES])
def test_oracle_pinned_to_reference(case, tmp_path):
    name, dims, nnz, P, J, dtype, zipf = case
    rng = np.random.default_rng(sum(map(ord, name)))
    idx = random_coo(rng, dims, nnz, distinct=True, zipf=zipf)
    vals = rng.random(len(idx[0]))
    path = tmp_path / (name + ".tns")
    write_tns(path, idx, vals, dtype=1)
    r = Ref(str(path), len(dims), dtype, seed=1)
    assert r.status == 0
    assert r.blocks(P, J) == 0
    ridx, rvals = r.parsed()
    o = Oracle(dtype, ridx, rvals, r.dims, P, J)
    a, b = o.partition(), r.partition()
    for k in ("blk_ptr", "blk_coord", "vals"):
        np.testing.assert_array_equal(a[k], b[k])
    for n in range(len(dims)):
        for k in ("idx", "count", "where"):
            np.testing.assert_array_equal(a[k][n], b[k][n])
    o.init_random(1, 0)
    r.init_random(1, 0)
    for s in range(3):
        for n in range(len(dims)):
            o.update_mode(n)
            r.update_mode(n)
        fr, _ = r.fit()
        fo = o.fit()["fit_ref"]
        for n in range(len(dims)):
            assert rel_fro(o.get_factor(n), r.get_factor(n)) <= (0.0 if dtype == 0 else 1e-9)
        assert abs(fo - fr) <= (0.0 if dtype == 0 else 1e-10)


@needs_ref
def test_reference_rejects_infeasible_partition(tmp_path):
    # dims 10, P = 4: block dim 3, ceil(10/3) = 4 -- feasible; dims 10, P = 6: block dim 2, ceil(10/2) = 5 != 6
    rng = np.random.default_rng(0)
    idx = random_coo(rng, [10, 10, 10], 100)
    write_tns(tmp_path / "t.tns", idx, rng.random(100))
    r = Ref(str(tmp_path / "t.tns"), 3, 1)
    assert r.blocks([6, 1, 1], 3) != 0
    o = Oracle(1, idx, rng.random(100), [10, 10, 10], [6, 1, 1], 3)
    assert o.status == 4


@needs_ref
@pytest.mark.parametrize("text", [
    b"1\t2\t3\t0.5\n2 3 4 0.25\n",                      # tabs and spaces
    b"1\t2\t3\t0.5\n4\t4\t4\t1.5\ntrailing text without newline",  # dropped tail
    b"1\t1\t1\n2\t2\t2\t0.75\n3\t3\t3\n",                # value-less lines draw frand
    b"1\t2\t3\t0.5\r\n2\t3\t4\t0.25\r\n",                  # CRLF
    b"  1 \t 2\t3   7e-1\n",                             # repeated delimiters
])
def test_parser_matches_reference(text, tmp_path):
    # One OpenMP thread: with several, the reference's parser races on files whose
    # per-thread byte ranges hold no newline (tensor_manager.tpp:96-99 reads the
    # previous thread's last position while that thread rewrites it) and draws
    # rand() for value-less lines in thread order.
    gomp = C.CDLL("libgomp.so.1")
    gomp.omp_get_max_threads.restype = C.c_int
    before = gomp.omp_get_max_threads()
    gomp.omp_set_num_threads(1)
    try:
        _compare_parsers(text, tmp_path)
    finally:
        gomp.omp_set_num_threads(before)


def _compare_parsers(text, tmp_path):
    p = tmp_path / "x.tns"
    p.write_bytes(text)
    for dtype in (0, 1):
        r = Ref(str(p), 3, dtype, seed=1)
        assert r.status == 0
        ridx, rvals = r.parsed()
        rc, idx, vals, dims, _ = ora_parse(text, 3, dtype, seed=1)
        assert rc == 0
        assert dims == r.dims
        for n in range(3):
            np.testing.assert_array_equal(idx[n], ridx[n])
        np.testing.assert_array_equal(vals, rvals)


def test_parser_rejects_zero_index():
    rc, *_ = ora_parse(b"1\t0\t3\t0.5\n", 3, 1)
    assert rc == 3


def test_oracle_fp32_vs_fp64_gap():
    """How far the reference's FP32 instantiation drifts from FP64 in 3 sweeps: the scale
    against which the CUDA path's FP32 tolerance is set."""
    rng = np.random.default_rng(11)
    dims = [40, 50, 30, 20]
    idx = random_coo(rng, dims, 4000, zipf=1.3)
    vals = rng.random(len(idx[0]))
    o32 = Oracle(0, idx, vals.astype(np.float32), dims, [2, 2, 2, 2], 10)
    o64 = Oracle(1, idx, vals.astype(np.float32).astype(np.float64), dims, [2, 2, 2, 2], 10)
    o32.init_random(1, 0)
    o64.init_random(1, 0)
    for _ in range(3):
        f32 = o32.sweep()["fit64"]
        f64 = o64.sweep()["fit64"]
    assert abs(f32 - f64) < 1e-4
    # Small tensors with few nonzeros per row leave B_r = lambda*I + sum delta delta^T
    # nearly singular, so FP32 rounding moves the factors by ~1e-2 relative while the
    # fit agrees to 1e-4: factor parity in FP32 is only meaningful on well-posed rows.
    gaps = [rel_fro(o32.get_factor(n), o64.get_factor(n)) for n in range(4)]
    assert max(gaps) < 5e-2


def test_warmstart_oracle_gradient_finite_differences():
    """The warm-start oracle's backward pass against central differences (float64)."""
    from oracle_util import ws_oracle
    orc = ws_oracle()
    rng = np.random.default_rng(2)
    F, H, J, B = 12, 7, 4, 9
    n = H * F + H + H * H + H + J * H + J
    p = rng.standard_normal(n) * 0.5
    x = rng.standard_normal((B, F))
    t = rng.standard_normal((B, J))
    _, g = orc.loss_grad(p, x, t, F, H, J)
    eps = 1e-6
    num = np.empty(n)
    for k in range(n):
        e = np.zeros(n)
        e[k] = eps
        num[k] = (orc.loss_grad(p + e, x, t, F, H, J)[0] - orc.loss_grad(p - e, x, t, F, H, J)[0]) / (2 * eps)
    assert np.abs(num - g).max() <= 1e-7 * max(1.0, np.abs(g).max())


def test_warmstart_oracle_features_by_hand():
    """3 nonzeros of a 2-order tensor, features written out by hand."""
    from oracle_util import ws_oracle
    orc = ws_oracle()
    idx = [np.array([0, 0, 1]), np.array([1, 2, 2])]
    vals = np.array([1.0, 3.0, 5.0])
    f = orc.row_features(idx, vals, [2, 3], 0)
    # row 0 of mode 0: c = 2, values 1, 3 -> mean 2, std 1; co-indexed mode-1 rows 1 (mean 1, c 1)
    # and 2 (mean 4, c 2): mean 2.5, std 1.5, mean log1p(c) = (log 2 + log 3) / 2;
    # E[x mu] = (1*1 + 3*4)/2, E[x mu^2] = (1*1 + 3*16)/2, E[x lc] = (log 2 + 3 log 3)/2;
    # E[x prod mu] = E[x mu]; one-hot [1, 0]
    l2, l3 = np.log(2), np.log(3)
    np.testing.assert_allclose(f[0], [l3, 2, 1, 2.5, 1.5, (l2 + l3) / 2, 6.5, 24.5, (l2 + 3 * l3) / 2, 6.5, 1, 0])
    np.testing.assert_allclose(f[1], [l2, 5, 0, 4, 0, l3, 20, 80, 5 * l3, 20, 1, 0])
