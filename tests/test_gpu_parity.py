"""GPU parity: the CUDA path through the C ABI against the CPU oracle.

Integer work (block assignment, block-local coordinates, count_nnz, where_nnz,
the glibc-rand initialisation) must be bit-exact.  Floating point: the oracle
sums in the reference's order, the kernels contract level by level and reduce
in tiles, so results agree to rounding:
    FP64: factors rel. Frobenius <= 1e-9, delta <= 1e-12, fit abs <= 1e-10
    FP32: factors rel. Frobenius <= FP32_FACTOR_TOL, delta <= 1e-5, fit abs <= 1e-5
"""

import zlib

import numpy as np
import pytest

import gputucker_gb300 as gtk
from oracle_util import NPDT, Oracle, random_coo, rel_fro

pytestmark = pytest.mark.gpu

FP32_FACTOR_TOL = 1e-4  # after 3 ALS sweeps; delta and fit are held to 1e-5
TOL = {
    0: dict(delta=1e-5, factor=FP32_FACTOR_TOL, fit=1e-5),
    1: dict(delta=1e-12, factor=1e-9, fit=1e-10),
}

# (name, dims, nnz, P, J, zipf)  -- specialised (N, J) kernels and generic ones
CASES = [
    ("n3_j4", [13, 17, 11], 400, [1, 1, 1], 4, None),
    ("n3_j10_blocks", [40, 30, 50], 3000, [2, 3, 1], 10, None),
    ("n4_j10_p4_zipf", [60, 50, 40, 30], 6000, [4, 4, 4, 4], 10, 1.3),
    ("n3_j16_zipf", [50, 60, 70], 4000, [1, 2, 1], 16, 1.5),
    ("n3_j8_pad", [23, 29, 31], 2500, [3, 2, 4], 8, None),
    ("n4_j8", [20, 21, 22, 23], 3000, [2, 1, 1, 2], 8, None),
    ("n4_j12", [20, 21, 22, 23], 2000, [1, 1, 2, 1], 12, None),
    ("n5_j4", [9, 10, 11, 12, 13], 2000, [1, 2, 1, 1, 2], 4, None),
    ("n5_j8", [9, 10, 11, 12, 13], 1500, [1, 1, 1, 1, 1], 8, None),
    ("n2_j7_generic", [40, 50], 800, [2, 2], 7, None),
    ("n4_j3_generic", [15, 16, 17, 18], 1500, [1, 1, 1, 1], 3, None),
    ("n3_j20_generic", [30, 40, 50], 1500, [1, 1, 1], 20, None),
    ("n6_j3_generic", [6, 7, 8, 5, 6, 7], 1500, [1, 1, 2, 1, 1, 1], 3, None),
]


def make(case, dtype, seed=7):
    name, dims, nnz, P, J, zipf = case
    rng = np.random.default_rng(zlib.crc32(name.encode()) + seed)
    idx = random_coo(rng, dims, nnz, distinct=True, zipf=zipf)
    vals = rng.random(len(idx[0])).astype(NPDT[dtype])
    coo = gtk.coo_from_arrays(idx, vals, dims=dims)
    t = gtk.create_tensor_blocks(coo, P, J)
    ora = Oracle(dtype, idx, vals, dims, P, J)
    assert ora.status == 0
    return t, ora


def check_partition(t, ora):
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
    assert abs(t.info.norm - ora.norm64) <= 1e-12 * max(1.0, ora.norm64)


@pytest.mark.parametrize("dtype", [0, 1], ids=["f32", "f64"])
@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_partition_bit_exact(case, dtype):
    t, ora = make(case, dtype)
    with t:
        check_partition(t, ora)


@pytest.mark.parametrize("dtype", [0, 1], ids=["f32", "f64"])
@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_sweeps_match_oracle(case, dtype):
    tol = TOL[dtype]
    t, ora = make(case, dtype)
    with t:
        t.init_random(1, 0)
        ora.init_random(1, 0)
        for n in range(ora.N):
            np.testing.assert_array_equal(t.get_factor(n), ora.get_factor(n))
        np.testing.assert_array_equal(t.get_core(), ora.get_core())
        for n in range(ora.N):
            assert rel_fro(t.compute_delta(n), ora.delta(n)) <= tol["delta"], f"delta mode {n}"
        for sweep in range(3):
            t.update_factor_matrices()
            fit = t.reconstruction()
            of = ora.sweep()
            for n in range(ora.N):
                err = rel_fro(t.get_factor(n), ora.get_factor(n))
                assert err <= tol["factor"], f"sweep {sweep} factor {n}: {err}"
            assert abs(fit - of["fit64"]) <= tol["fit"], f"sweep {sweep}: fit {fit} vs {of['fit64']}"
        # the core is never updated (the reference keeps G fixed)
        np.testing.assert_array_equal(t.get_core(), ora.get_core())


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
        np.testing.assert_allclose(fits, ofits, atol=TOL[dtype]["fit"])


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
    t, ora = make(CASES[2], 0)
    with t:
        rng = np.random.default_rng(0)
        for n in range(t.order):
            a = rng.random((t.factor_rows(n), t.rank)).astype(np.float32)
            t.set_factor(n, a)
            ora.set_factor(n, a)
            np.testing.assert_array_equal(t.get_factor(n), a)
        g = rng.random((t.rank,) * t.order).astype(np.float32)
        t.set_core(g)
        ora.set_core(g)
        np.testing.assert_array_equal(t.get_core(), g)
        t.update_factor_matrices()
        ora.sweep()
        for n in range(t.order):
            assert rel_fro(t.get_factor(n), ora.get_factor(n)) <= FP32_FACTOR_TOL
