"""gtk_validate: the device arrays of a handle built by gtk_create_blocks pass every
consistency check on every parity shape (orders 2..6, partitioned and not), before
and after sweeps; a non-finite factor entry planted through the ABI is counted."""

import numpy as np
import pytest

import gputucker_gb300 as gtk
from test_gpu_parity import CASES, data

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_validate_clean_handles(case):
    name, dims, nnz, P, J, _ = case
    idx, vals = data(case, 0)
    with gtk.create_tensor_blocks(gtk.coo_from_arrays(idx, vals, dims=dims), P, J) as t:
        assert t.validate() == [0] * 8
        t.init_random(1, 0)
        t.sweep()
        assert t.validate() == [0] * 8


def test_validate_counts_non_finite_factor_entries():
    name, dims, nnz, P, J, _ = CASES[2]
    idx, vals = data(CASES[2], 0)
    with gtk.create_tensor_blocks(gtk.coo_from_arrays(idx, vals, dims=dims), P, J) as t:
        t.init_random(1, 0)
        a = t.get_factor(1)
        a[3, 1] = np.nan
        a[5, 0] = np.inf
        t.set_factor(1, a)
        v = t.validate()
        assert v[6] == 2 and sum(v) == 2, v
