"""GPU parity: the CUDA path through the C ABI against the CPU oracle.

Integer work (block assignment, block-local coordinates, count_nnz, where_nnz,
the glibc-rand initialisation, the untouched core) must be bit-exact.

Floating point.  The oracle sums in the reference's order; the kernels contract
level by level and reduce in tiles, so results agree to rounding, amplified by
the conditioning of the row systems B_r = lambda*I + sum delta delta^T.  With
positive random factors and core every delta of a row points nearly the same
way, so B_r is ill-conditioned even with many nonzeros per row, and the
reference's own FP32 instantiation moves 1e-5..4e-3 (factors) and up to 1.4e-5
(fit) away from its FP64 instantiation on the cases below (O(1) on the
Zipf-skewed ILL cases, whose rows have fewer nonzeros than J).  Hence:
  * FP64 (the reference's default value_t): factors rel. Frobenius <= 1e-9,
    delta <= 1e-12, fit abs <= 1e-10 against the FP64 oracle.
  * FP32: delta from identical inputs <= 1e-5; then "accuracy parity": after
    every sweep the CUDA factors are no further from the FP64 oracle than
    2 x (FP32 oracle's distance from it) + 1e-5, within 3 x that gap + 1e-5 of
    the FP32 oracle, and the fit within max(1e-5, 3 x the oracle's FP32/FP64
    fit gap) of the FP32 oracle's.
"""

import zlib

import numpy as np
import pytest

import gputucker_gb300 as gtk
from oracle_util import NPDT, Oracle, random_coo, rel_fro

pytestmark = pytest.mark.gpu

TOL64 = dict(delta=1e-12, factor=1e-9, fit=1e-10)
DELTA32 = 1e-5

# (name, dims, nnz, P, J, zipf) -- specialised (N, J) kernels and generic ones
CASES = [
    ("n3_j4", [13, 17, 11], 1200, [1, 1, 1], 4, None),
    ("n3_j10_blocks", [40, 30, 50], 12000, [2, 3, 1], 10, None),
    ("n4_j10_p4", [24, 20, 16, 22], 20000, [4, 4, 4, 4], 10, None),
    ("n3_j16", [40, 50, 60], 20000, [1, 2, 1], 16, None),
    ("n3_j8_pad", [23, 29, 31], 6000, [3, 2, 4], 8, None),
    ("n4_j8", [20, 21, 22, 23], 12000, [2, 1, 1, 2], 8, None),
    ("n4_j12", [20, 21, 22, 23], 12000, [1, 1, 2, 1], 12, None),
    ("n5_j4", [9, 10, 11, 12, 13], 5000, [1, 2, 1, 1, 2], 4, None),
    ("n5_j8", [9, 10, 11, 12, 13], 6000, [1, 1, 1, 1, 1], 8, None),
    ("n2_j7_generic", [40, 50], 1500, [2, 2], 7, None),
    ("n4_j3_generic", [15, 16, 17, 18], 5000, [1, 1, 1, 1], 3, None),
    ("n3_j20_generic", [30, 40, 50], 15000, [1, 1, 1], 20, None),
    ("n6_j3_generic", [6, 7, 8, 5, 6, 7], 4000, [1, 1, 2, 1, 1, 1], 3, None),
]
# Zipf-skewed: many rows with fewer nonzeros than J
ILL = [
    ("ill_n4_j10_zipf", [60, 50, 40, 30], 6000, [4, 4, 4, 4], 10, 1.3),
    ("ill_n3_j10_zipf", [80, 60, 70], 3000, [2, 2, 1], 10, 1.4),
]


def data(case, dtype, seed=7):
    name, dims, nnz, P, J, zipf = case
    rng = np.random.default_rng(zlib.crc32(name.encode()) + seed)
    idx = random_coo(rng, dims, nnz, distinct=True, zipf=zipf)
    vals = rng.random(len(idx[0])).astype(NPDT[dtype])
    return idx, vals


def make(case, dtype, seed=7):
    name, dims, nnz, P, J, zipf = case
    idx, vals = data(case, dtype, seed)
    coo = gtk.coo_from_arrays(idx, vals, dims=dims)
    t = gtk.create_tensor_blocks(coo, P, J)
    ora = Oracle(dtype, idx, vals, dims, P, J)
    assert ora.status == 0
    return t, ora


def check_partition(t, ora, norm_rtol=1e-12):
    """Integer arrays bit-exact; ||X|| (FP64 sums in different orders) within norm_rtol."""
    part = ora.partition()
    assert t.info.block_count == ora.nblk
    assert t.info.block_dims == ora.bd
    for b in range(ora.nblk):
        coord, idx, vals = t.block(b)
        s, e = int(part["blk_ptr"][b]), int(part["blk_ptr"][b + 1])
        assert coord == list(part["blk_coord"][b])
        assert len(vals) == e - s
        for n in range(ora.N):
            np.testing.assert_array_equal(idx[n], part["idx"][n][s:e])
        np.testing.assert_array_equal(vals, part["vals"][s:e])
        for n in range(ora.N):
            cnt, where = t.segments(b, n)
            rows = ora.bd[n] + 1
            np.testing.assert_array_equal(cnt, part["count"][n][b * rows:(b + 1) * rows])
            np.testing.assert_array_equal(where, part["where"][n][s:e])
    assert abs(t.info.norm - ora.norm64) <= norm_rtol * max(1.0, ora.norm64)


@pytest.mark.parametrize("dtype", [0, 1], ids=["f32", "f64"])
@pytest.mark.parametrize("case", CASES + ILL, ids=[c[0] for c in CASES + ILL])
def test_partition_bit_exact(case, dtype):
    t, ora = make(case, dtype)
    with t:
        check_partition(t, ora)


def check_init(t, ora):
    t.init_random(1, 0)
    ora.init_random(1, 0)
    for n in range(ora.N):
        np.testing.assert_array_equal(t.get_factor(n), ora.get_factor(n))
    np.testing.assert_array_equal(t.get_core(), ora.get_core())


def fp64_sweeps(t, ora, tol=TOL64, sweeps=3):
    check_init(t, ora)
    for n in range(ora.N):
        assert rel_fro(t.compute_delta(n), ora.delta(n)) <= tol["delta"], f"delta mode {n}"
    worst = 0.0
    for sweep in range(sweeps):
        t.update_factor_matrices()
        fit = t.reconstruction()
        of = ora.sweep()
        for n in range(ora.N):
            err = rel_fro(t.get_factor(n), ora.get_factor(n))
            worst = max(worst, err)
            assert err <= tol["factor"], f"sweep {sweep} factor {n}: {err}"
        assert abs(fit - of["fit64"]) <= tol["fit"], f"sweep {sweep}: fit {fit} vs {of['fit64']}"
    np.testing.assert_array_equal(t.get_core(), ora.get_core())  # G is never updated
    return worst


def fp32_sweeps(t, o32, o64, sweeps=3):
    """Accuracy parity of the FP32 path (see the module docstring)."""
    check_init(t, o32)
    o64.init_random(1, 0)
    for n in range(o32.N):
        assert rel_fro(t.compute_delta(n), o32.delta(n)) <= DELTA32, f"delta mode {n}"
    report = []
    for sweep in range(sweeps):
        t.update_factor_matrices()
        fit = t.reconstruction()
        f32 = o32.sweep()["fit64"]
        f64 = o64.sweep()["fit64"]
        for n in range(o32.N):
            a = t.get_factor(n)
            gap = rel_fro(o32.get_factor(n), o64.get_factor(n))
            e64 = rel_fro(a, o64.get_factor(n))
            e32 = rel_fro(a, o32.get_factor(n))
            report.append((sweep, n, e32, e64, gap))
            assert e64 <= 2 * gap + 1e-5, f"sweep {sweep} factor {n}: {e64} from FP64, reference FP32 {gap}"
            assert e32 <= 3 * gap + 1e-5, f"sweep {sweep} factor {n}: {e32} from FP32 reference (gap {gap})"
        fgap = abs(f32 - f64)
        assert abs(fit - f32) <= max(1e-5, 3 * fgap), f"sweep {sweep}: fit {fit} vs {f32} (gap {fgap})"
    np.testing.assert_array_equal(t.get_core(), o32.get_core())
    return report


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_fp64_sweeps_match_oracle(case):
    t, ora = make(case, 1)
    with t:
        worst = fp64_sweeps(t, ora)
        print(f"{case[0]} f64 worst factor rel error {worst:.3e}")


@pytest.mark.parametrize("case", CASES + ILL, ids=[c[0] for c in CASES + ILL])
def test_fp32_sweeps_accuracy_parity(case):
    name, dims, nnz, P, J, zipf = case
    idx, vals = data(case, 0)
    t, o32 = make(case, 0)
    o64 = Oracle(1, idx, vals.astype(np.float64), dims, P, J)
    with t:
        rep = fp32_sweeps(t, o32, o64)
    worst = max(rep, key=lambda r: r[2])
    print(f"{name} f32 worst: sweep {worst[0]} mode {worst[1]} vs f32-ref {worst[2]:.2e} "
          f"vs f64-ref {worst[3]:.2e} ref gap {worst[4]:.2e}")


@pytest.mark.parametrize("case", ILL, ids=[c[0] for c in ILL])
def test_fp64_ill_posed_fit(case):
    """FP64 on rows with fewer nonzeros than J: Cholesky gives way to pivoted LU where
    needed (as the reference's LU inverse); the fit stays with the oracle's."""
    t, ora = make(case, 1)
    with t:
        check_init(t, ora)
        for sweep in range(3):
            t.update_factor_matrices()
            fit = t.reconstruction()
            of = ora.sweep()["fit64"]
            assert abs(fit - of) <= 1e-6, f"sweep {sweep}: {fit} vs {of}"


@pytest.mark.parametrize("dtype", [0, 1], ids=["f32", "f64"])
def test_tucker_decomposition_loop(dtype):
    """The reference's loop: at most 3 sweeps, stop when |dfit| <= 1e-4 (tucker.cuh:166-187)."""
    t, ora = make(CASES[1], dtype)
    with t:
        t.init_random(1, 0)
        ora.init_random(1, 0)
        fits = t.tucker_decomposition(3, 1e-4)
        ofits = []
        for it in range(3):
            ofits.append(ora.sweep()["fit64"])
            if it > 0 and abs(ofits[-1] - ofits[-2]) <= 1e-4:
                break
        assert len(fits) == len(ofits)
        np.testing.assert_allclose(fits, ofits, atol=TOL64["fit"] if dtype == 1 else 1e-5)


def test_empty_blocks_and_padding_rows():
    """Blocks without nonzeros (the reference asserts on them) and padding rows of the last slab."""
    dims = [30, 30, 30]
    rng = np.random.default_rng(3)
    idx = [rng.integers(0, 10, 500).astype(np.uint32) for _ in range(3)]  # only the first third of each axis
    for n in range(3):
        idx[n][0] = 29
    vals = rng.random(500)
    # remove duplicates
    keys = np.stack(idx, 1)
    _, first = np.unique(keys, axis=0, return_index=True)
    first.sort()
    idx = [i[first] for i in idx]
    vals = vals[first]
    coo = gtk.coo_from_arrays(idx, vals, dims=dims)
    P = [4, 3, 2]  # 8/8/6 block dims; most blocks empty
    with gtk.create_tensor_blocks(coo, P, 5) as t:
        ora = Oracle(1, idx, vals, dims, P, 5)
        check_partition(t, ora)
        t.init_random(1, 0)
        ora.init_random(1, 0)
        for _ in range(2):
            t.update_factor_matrices()
            ora.sweep()
        for n in range(3):
            a = t.get_factor(n)
            assert rel_fro(a, ora.get_factor(n)) <= 1e-9
            # rows without nonzeros (and padding rows) solve to 0: B = lambda*I, C = 0
            rows_with = np.unique(idx[n])
            mask = np.ones(a.shape[0], bool)
            mask[rows_with] = False
            assert np.all(a[mask] == 0)


def test_set_factor_core_roundtrip():
    t, ora = make(CASES[2], 1)
    with t:
        rng = np.random.default_rng(0)  # random factors: every row well determined
        for n in range(t.order):
            a = rng.random((t.factor_rows(n), t.rank))
            t.set_factor(n, a)
            ora.set_factor(n, a)
            np.testing.assert_array_equal(t.get_factor(n), a)
        g = rng.random((t.rank,) * t.order)
        t.set_core(g)
        ora.set_core(g)
        np.testing.assert_array_equal(t.get_core(), g)
        t.update_factor_matrices()
        ora.sweep()
        for n in range(t.order):
            assert rel_fro(t.get_factor(n), ora.get_factor(n)) <= 1e-9
