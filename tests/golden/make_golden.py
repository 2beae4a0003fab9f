"""Regenerates the golden fixtures of tests/golden/ from the reference itself.

Runs the GPUTucker reference's own host code, compiled in place from its
sources into oracle/_ref/libgtk_ref.so (`make -C oracle ref`):
ParseFromFile, CreateTensorBlocks, AssignIndicesToEachMode, ComputingBC and the
Eigen row solve, with the delta/reconstruction kernel bodies restated on the CPU
(the reference ships them only as CUDA kernels).  For every case it writes the
input text file (<case>.tns) and <case>.npz holding:

  dims, blk_ptr, blk_coord, idx<n>, vals, count<n>, where<n>   partition (bit-exact)
  fac0_<n>, core                                               initial factors / core
  delta0_<n>                                                   delta of mode n, initial factors
  fac<s+1>_<n>, fit<s+1>                                       factors and fit after sweep s

It also writes planner_cases.json: Optimizer::FindPartitionParms of the
reference (optimizer.tpp:71-89) on the shapes and memory sizes of PLANNER_CASES.

Usage (needs the reference sources): python tests/golden/make_golden.py [--planner-only]
"""

from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
# The reference's parser draws rand() for value-less lines inside an OpenMP
# region (tensor_manager.tpp:152-155), so its draw order is the thread
# schedule; with one thread it is file order, the order this library uses.
os.environ["OMP_NUM_THREADS"] = "1"
from oracle_util import Ref, random_coo, ref_available, write_tns  # noqa: E402

# name, dims, nnz, P, J, dtype (0 float / 1 double), zipf, missing-value lines
CASES = [
    ("g3_small_f64", [12, 9, 14], 300, [2, 3, 1], 4, 1, None, 0),
    ("g3_blocks_f32", [40, 30, 50], 2000, [2, 3, 2], 10, 0, None, 0),
    ("g4_p_f32", [30, 25, 20, 28], 3000, [3, 2, 4, 2], 10, 0, None, 0),
    ("g3_missing_values_f64", [10, 11, 12], 200, [1, 1, 1], 5, 1, None, 17),
]
SWEEPS = 3


def make(case):
    name, dims, nnz, P, J, dtype, zipf, missing = case
    rng = np.random.default_rng(abs(sum(map(ord, name))))
    idx = random_coo(rng, dims, nnz, distinct=True, zipf=zipf)
    vals = rng.random(len(idx[0]))
    path = os.path.join(HERE, name + ".tns")
    write_tns(path, idx, vals, dtype=1)
    if missing:
        # drop the value of some lines: the reference draws frand for them
        lines = open(path).read().splitlines(keepends=True)
        for k in rng.choice(len(lines), missing, replace=False):
            lines[k] = "\t".join(lines[k].split("\t")[:-1]) + "\n"
        open(path, "w").write("".join(lines))
    r = Ref(path, len(dims), dtype, seed=1)
    assert r.status == 0, r.status
    assert r.blocks(P, J) == 0
    part = r.partition()
    out = dict(dims=np.array(r.dims, np.uint32), P=np.array(P, np.uint32), J=np.array(J), dtype=np.array(dtype),
               blk_ptr=part["blk_ptr"], blk_coord=part["blk_coord"], vals=part["vals"],
               norm=np.array(r.norm))
    for n in range(len(dims)):
        out[f"idx{n}"] = part["idx"][n]
        out[f"count{n}"] = part["count"][n]
        out[f"where{n}"] = part["where"][n]
    pidx, pvals = r.parsed()
    for n in range(len(dims)):
        out[f"parsed_idx{n}"] = pidx[n]
    out["parsed_vals"] = pvals
    # the parse consumed `missing` rand() draws; the init continues the stream
    r.init_random(1, missing)
    out["skip"] = np.array(missing)
    for n in range(len(dims)):
        out[f"fac0_{n}"] = r.get_factor(n)
        out[f"delta0_{n}"] = r.delta(n)
    out["core"] = r.get_core()
    for s in range(SWEEPS):
        for n in range(len(dims)):
            r.update_mode(n)
        fit, err = r.fit()
        for n in range(len(dims)):
            out[f"fac{s + 1}_{n}"] = r.get_factor(n)
        out[f"fit{s + 1}"] = np.array(fit)
        out[f"err{s + 1}"] = np.array(err)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(name, "nnz", r.nnz, "blocks", r.nblk, "fits", [float(out[f"fit{s + 1}"]) for s in range(SWEEPS)])


# partition planner cases: dims, nnz, rank, dtype, gpus, GPU memory bytes
GB = 1 << 30
PLANNER_CASES = [
    ([10_000] * 3, 1_000_000, 10, 1, 1, 280 * GB),             # uniform 3-order, 1M nonzeros (fits)
    ([100_000] * 4, 100_000_000, 10, 0, 1, 280 * GB),          # 4-order Zipf, 100M nonzeros (fits)
    ([1_000_000] * 3, 500_000_000, 16, 0, 1, 280 * GB),        # 3-order, 500M nonzeros (fits)
    ([50_000] * 3, 20_000_000, 8, 0, 1, 280 * GB),             # planted 3-order, 20M observed
    ([100_000] * 4, 100_000_000, 10, 0, 1, 4 * GB),            # does not fit: dimension-based
    ([100_000] * 4, 100_000_000, 10, 0, 4, 4 * GB),
    ([1_000_000] * 3, 500_000_000, 16, 0, 1, 16 * GB),
    ([1_000_000] * 3, 500_000_000, 16, 1, 2, 24 * GB),
    ([37, 12_345, 999_999], 3_000_000, 8, 1, 1, 256 << 20),
    ([5, 7, 3, 11], 300, 4, 1, 1, 1 << 16),                   # tiny memory: P grows until a slab is empty
    ([1000, 2000, 3000, 4000, 5000], 10_000_000, 4, 0, 3, 1 * GB),
    ([123_456, 654_321], 50_000_000, 32, 1, 1, 2 * GB),
    ([2**20, 3, 2**20], 80_000_000, 12, 0, 1, 3 * GB),
    ([10] * 8, 90_000, 2, 1, 1, 1 << 20),
    ([3, 3, 3], 27, 4, 1, 1, 1000),                            # never fits: the reference throws
    ([10, 10], 100, 2, 0, 1, 600),                             # P = 6 of dim 10 leaves an empty slab
]


def make_planner():
    import json
    from oracle_util import ref_plan
    out = []
    for dims, nnz, J, dt, gpus, mem in PLANNER_CASES:
        st, P, bd, nblk, dim_based, streams, avail = ref_plan(dims, nnz, J, dt, gpus, mem)
        out.append(dict(dims=dims, nnz=nnz, rank=J, dtype=dt, gpus=gpus, mem=mem, status=st, P=P, block_dims=bd,
                        block_count=nblk, dimension_based=dim_based, streams=streams, avail_nnz_per_task=avail))
        print("planner", dims, nnz, J, dt, gpus, mem, "->", st, P, nblk, dim_based)
    with open(os.path.join(HERE, "planner_cases.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    if not ref_available():
        sys.exit("oracle/_ref/libgtk_ref.so is missing: build it with `make -C oracle ref`")
    if "--planner-only" not in sys.argv:
        for c in CASES:
            make(c)
    make_planner()
