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

Usage (needs the reference sources): python tests/golden/make_golden.py
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


if __name__ == "__main__":
    if not ref_available():
        sys.exit("oracle/_ref/libgtk_ref.so is missing: build it with `make -C oracle ref`")
    for c in CASES:
        make(c)
