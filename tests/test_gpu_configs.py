"""The configurations of the workload table at (or near) their real sizes.

* 3-order 10,000^3, 1M distinct uniform nonzeros, FP64, rank 10, P = 1: the
  configuration the reference runs end to end; held against the FP64 oracle
  (the reference's CPU path) for 3 sweeps at full size.
* 3-order Zipf(1.05) lognormal precision configuration (rank 16): BF16 and TF32
  tensor-core forms against plain FP32 on a 20M-nonzero instance whose dims are
  scaled with the nonzeros (40,000^3: ~500 nonzeros per row, as 500M over
  1,000,000^3 has; at 20M over 10^6 rows most rows are under-determined and every
  form, plain FP32 included, oscillates).
* size-independent properties of the 4-order 100M configuration's partition on
  a 10M instance: every block's where_nnz is a permutation sorted by its row
  pointer, count_nnz sums to the block size.
"""

import numpy as np
import pytest

import gputucker_gb300 as gtk
from oracle_util import Oracle, rel_fro

pytestmark = pytest.mark.gpu


def test_config_uniform3d_1m_fp64_full_size():
    coo = gtk.generate(3, [10000] * 3, 1_000_000, "uniform", 0.0, "uniform", "f64", seed=0)
    idx, vals = coo.arrays()
    assert coo.dims == [10000] * 3
    with gtk.create_tensor_blocks(coo, [1, 1, 1], 10) as t:
        ora = Oracle(1, idx, vals, coo.dims, [1, 1, 1], 10)
        t.init_random(1, 0)
        ora.init_random(1, 0)
        for s in range(3):
            t.update_factor_matrices()
            fit = t.reconstruction()
            of = ora.sweep()["fit64"]
            assert abs(fit - of) <= 1e-10, (s, fit, of)
            for n in range(3):
                assert rel_fro(t.get_factor(n), ora.get_factor(n)) <= 1e-9


def test_config_precision3d_forms_agree():
    coo = gtk.generate(3, [40_000] * 3, 20_000_000, "zipf", 1.05, "lognormal", "f32", seed=0)
    fits = {}
    with gtk.create_tensor_blocks(coo, [1, 1, 1], 16) as t:
        for prec in ("plain", "bf16", "tf32"):
            t.init_random(1, 0)
            t.set_precision(prec)
            fits[prec] = [t.sweep() for _ in range(3)]
    print(fits)
    for prec in ("bf16", "tf32"):
        assert abs(fits[prec][-1] - fits["plain"][-1]) <= 1e-3, (prec, fits)


def test_config_zipf4d_partition_properties():
    coo = gtk.generate(4, [100_000] * 4, 10_000_000, "zipf", 1.1, "uniform", "f32", seed=0)
    idx, vals = coo.arrays()
    with gtk.create_tensor_blocks(coo, [4, 4, 4, 4], 10) as t:
        nb = t.info.block_count
        assert nb == 256
        total = 0
        rng = np.random.default_rng(0)
        for b in sorted(rng.choice(nb, 12, replace=False)):
            coord, bidx, bvals = t.block(int(b))
            total += len(bvals)
            for n in range(4):
                cnt, where = t.segments(int(b), n)
                assert cnt[0] == 0 and cnt[-1] == len(bvals) and np.all(np.diff(cnt.astype(np.int64)) >= 0)
                assert np.array_equal(np.sort(where), np.arange(len(bvals), dtype=np.uint32))
                rows = bidx[n][where]
                assert np.all(np.diff(rows.astype(np.int64)) >= 0)  # sorted by local row
                # stable: equal rows keep block order
                same = np.diff(rows.astype(np.int64)) == 0
                assert np.all(np.diff(where.astype(np.int64))[same] > 0)
                assert np.all(bidx[n] < t.info.block_dims[n])
        sizes = [t.block_nnz(b)[1] for b in range(nb)]
        assert sum(sizes) == coo.nnz
        assert abs(t.info.norm - float(np.sqrt(np.sum(vals.astype(np.float64) ** 2)))) <= 1e-9 * t.info.norm
