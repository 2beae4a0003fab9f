"""ctypes wrappers of the parity checkers (test infrastructure only).

Oracle -> oracle/bin/libgtk_oracle.so, the CPU restatement of the reference
          (oracle/gtk_oracle.cpp), built by `make -C oracle`.
Ref    -> oracle/_ref/libgtk_ref.so, the reference's own host code compiled in
          place from its sources (`make -C oracle ref`); only exists where the
          reference sources were present at build time.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_LIB = os.path.join(ROOT, "oracle", "bin", "libgtk_oracle.so")
REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libgtk_ref.so")

_ora = None
_ref = None


def build_oracle() -> None:
    src = os.path.join(ROOT, "oracle", "gtk_oracle.cpp")
    if not os.path.exists(ORACLE_LIB) or os.path.getmtime(ORACLE_LIB) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)


def ora_lib():
    global _ora
    if _ora is None:
        build_oracle()
        lib = C.CDLL(ORACLE_LIB)
        lib.ora_create.restype = C.c_void_p
        lib.ora_create.argtypes = [C.c_int, C.c_int, C.c_uint64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                   C.c_int, C.POINTER(C.c_int)]
        for name in ["ora_destroy", "ora_info", "ora_partition", "ora_init_random", "ora_get_factor",
                     "ora_set_factor", "ora_get_core", "ora_set_core", "ora_delta", "ora_update_mode", "ora_sweep",
                     "ora_fit"]:
            getattr(lib, name).restype = None
        lib.ora_destroy.argtypes = [C.c_void_p]
        lib.ora_info.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        lib.ora_partition.argtypes = [C.c_void_p] * 7
        lib.ora_init_random.argtypes = [C.c_void_p, C.c_uint32, C.c_uint64]
        lib.ora_get_factor.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        lib.ora_set_factor.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        lib.ora_get_core.argtypes = [C.c_void_p, C.c_void_p]
        lib.ora_set_core.argtypes = [C.c_void_p, C.c_void_p]
        lib.ora_delta.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        lib.ora_update_mode.argtypes = [C.c_void_p, C.c_int]
        lib.ora_sweep.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        lib.ora_fit.argtypes = [C.c_void_p] * 5
        lib.ora_rand.argtypes = [C.c_uint32, C.c_uint64, C.c_uint64, C.c_void_p]
        lib.ora_rand.restype = None
        lib.ora_parse.argtypes = [C.c_char_p, C.c_uint64, C.c_int, C.c_int, C.c_uint32, C.c_void_p, C.c_void_p,
                                  C.c_void_p, C.c_void_p, C.c_void_p]
        lib.ora_parse.restype = C.c_int
        lib.ora_last_error.restype = C.c_char_p
        lib.ora_num_threads.restype = C.c_int
        lib.ora_set_num_threads.argtypes = [C.c_int]
        lib.ora_set_num_threads.restype = None
        _ora = lib
    return _ora


def ref_available() -> bool:
    return os.path.exists(REF_LIB)


def ref_lib():
    global _ref
    if _ref is None:
        lib = C.CDLL(REF_LIB)
        lib.ref_parse_file.restype = C.c_void_p
        lib.ref_parse_file.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_uint, C.POINTER(C.c_int)]
        lib.ref_parsed.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        lib.ref_blocks.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
        lib.ref_info.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        lib.ref_partition.argtypes = [C.c_void_p] * 7
        lib.ref_init_random.argtypes = [C.c_void_p, C.c_uint, C.c_uint64]
        lib.ref_get_factor.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        lib.ref_get_core.argtypes = [C.c_void_p, C.c_void_p]
        lib.ref_delta.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        lib.ref_update_mode.argtypes = [C.c_void_p, C.c_int]
        lib.ref_fit.argtypes = [C.c_void_p, C.c_void_p]
        lib.ref_fit.restype = C.c_double
        lib.ref_last_error.restype = C.c_char_p
        lib.ref_plan.argtypes = [C.c_int, C.c_void_p, C.c_uint64, C.c_int, C.c_int, C.c_int, C.c_uint64, C.c_void_p,
                                 C.c_void_p, C.c_void_p]
        _ref = lib
    return _ref


NPDT = {0: np.float32, 1: np.float64}


def glibc_rand(seed: int, n: int, skip: int = 0) -> np.ndarray:
    out = np.empty(n, np.int32)
    ora_lib().ora_rand(seed, skip, n, out.ctypes.data)
    return out


def ora_parse(data: bytes, order: int, dtype: int, seed: int = 1):
    """(rc, idx list, values, dims, draws) of the oracle's restated parser."""
    lib = ora_lib()
    nnz = C.c_uint64()
    dims = (C.c_uint32 * order)()
    rc = lib.ora_parse(data, len(data), order, dtype, seed, C.byref(nnz), dims, None, None, None)
    if rc:
        return rc, None, None, None, None
    n = nnz.value
    idx = [np.empty(n, np.uint32) for _ in range(order)]
    vals = np.empty(n, NPDT[dtype])
    ptrs = (C.c_void_p * order)(*[a.ctypes.data for a in idx])
    draws = C.c_uint64()
    rc = lib.ora_parse(data, len(data), order, dtype, seed, C.byref(nnz), dims, ptrs, vals.ctypes.data,
                       C.byref(draws))
    return rc, idx, vals, list(dims), draws.value


class _Common:
    dtype: int
    N: int
    J: int
    bd: list
    P: list
    nblk: int
    nnz: int

    def _alloc_partition(self):
        N, nnz, nblk = self.N, self.nnz, self.nblk
        blk_ptr = np.empty(nblk + 1, np.uint64)
        blk_coord = np.empty(nblk * N, np.uint32)
        idx = [np.empty(nnz, np.uint32) for _ in range(N)]
        vals = np.empty(nnz, NPDT[self.dtype])
        count = [np.empty(nblk * (self.bd[n] + 1), np.uint64) for n in range(N)]
        where = [np.empty(nnz, np.uint32) for _ in range(N)]
        args = [blk_ptr.ctypes.data, blk_coord.ctypes.data,
                (C.c_void_p * N)(*[a.ctypes.data for a in idx]), vals.ctypes.data,
                (C.c_void_p * N)(*[a.ctypes.data for a in count]),
                (C.c_void_p * N)(*[a.ctypes.data for a in where])]
        out = dict(blk_ptr=blk_ptr, blk_coord=blk_coord.reshape(nblk, N), idx=idx, vals=vals, count=count,
                   where=where)
        return args, out

    def factor_shape(self, n):
        return (self.P[n] * self.bd[n], self.J)


class Oracle(_Common):
    """The CPU restatement on a COO given as arrays."""

    def __init__(self, dtype: int, idx, vals, dims, P, J: int):
        lib = ora_lib()
        self.dtype, self.N, self.J, self.P = dtype, len(idx), J, list(P)
        self.nnz = len(vals)
        gi = [np.ascontiguousarray(i, dtype=np.uint32) for i in idx]
        self._keep = gi
        v = np.ascontiguousarray(vals, dtype=NPDT[dtype])
        self._v = v
        d = np.ascontiguousarray(dims, dtype=np.uint32)
        p = np.ascontiguousarray(P, dtype=np.uint32)
        st = C.c_int()
        self.h = lib.ora_create(dtype, self.N, self.nnz, (C.c_void_p * self.N)(*[a.ctypes.data for a in gi]),
                                v.ctypes.data, d.ctypes.data, p.ctypes.data, J, C.byref(st))
        self.status = st.value
        if not self.h:
            return
        bd = np.empty(self.N, np.uint32)
        nb, nr, n64 = C.c_uint64(), C.c_double(), C.c_double()
        lib.ora_info(self.h, bd.ctypes.data, C.byref(nb), C.byref(nr), C.byref(n64))
        self.bd, self.nblk, self.norm_ref, self.norm64 = [int(x) for x in bd], nb.value, nr.value, n64.value

    def partition(self):
        args, out = self._alloc_partition()
        ora_lib().ora_partition(self.h, *args)
        return out

    def init_random(self, seed=1, skip=0):
        ora_lib().ora_init_random(self.h, seed, skip)

    def get_factor(self, n):
        a = np.empty(self.factor_shape(n), NPDT[self.dtype])
        ora_lib().ora_get_factor(self.h, n, a.ctypes.data)
        return a

    def set_factor(self, n, a):
        a = np.ascontiguousarray(a, dtype=NPDT[self.dtype])
        ora_lib().ora_set_factor(self.h, n, a.ctypes.data)

    def get_core(self):
        g = np.empty((self.J,) * self.N, NPDT[self.dtype])
        ora_lib().ora_get_core(self.h, g.ctypes.data)
        return g

    def set_core(self, g):
        g = np.ascontiguousarray(g, dtype=NPDT[self.dtype])
        ora_lib().ora_set_core(self.h, g.ctypes.data)

    def delta(self, mode):
        d = np.empty((self.nnz, self.J), NPDT[self.dtype])
        ora_lib().ora_delta(self.h, mode, d.ctypes.data)
        return d

    def update_mode(self, mode):
        ora_lib().ora_update_mode(self.h, mode)

    def fit(self):
        fr, f64, er, e64 = C.c_double(), C.c_double(), C.c_double(), C.c_double()
        ora_lib().ora_fit(self.h, C.byref(fr), C.byref(f64), C.byref(er), C.byref(e64))
        return dict(fit_ref=fr.value, fit64=f64.value, err_ref=er.value, err64=e64.value)

    def sweep(self):
        for n in range(self.N):
            self.update_mode(n)
        return self.fit()

    def __del__(self):
        if getattr(self, "h", None):
            ora_lib().ora_destroy(self.h)
            self.h = None


class Ref(_Common):
    """The reference's own host code (parse from file, CreateTensorBlocks, ComputingBC, Eigen)."""

    def __init__(self, path: str, order: int, dtype: int, seed: int = 1):
        lib = ref_lib()
        st = C.c_int()
        self.h = lib.ref_parse_file(str(path).encode(), order, dtype, seed, C.byref(st))
        self.status = st.value
        self.dtype, self.N = dtype, order
        if not self.h:
            return
        nnz = C.c_uint64()
        dims = np.empty(order, np.uint32)
        lib.ref_parsed(self.h, C.byref(nnz), dims.ctypes.data, None, None)
        self.nnz, self.dims = nnz.value, [int(x) for x in dims]

    def parsed(self):
        idx = [np.empty(self.nnz, np.uint32) for _ in range(self.N)]
        vals = np.empty(self.nnz, NPDT[self.dtype])
        nnz = C.c_uint64()
        dims = np.empty(self.N, np.uint32)
        ref_lib().ref_parsed(self.h, C.byref(nnz), dims.ctypes.data,
                             (C.c_void_p * self.N)(*[a.ctypes.data for a in idx]), vals.ctypes.data)
        return idx, vals

    def blocks(self, P, J):
        self.P, self.J = list(P), J
        p = np.ascontiguousarray(P, dtype=np.uint32)
        rc = ref_lib().ref_blocks(self.h, p.ctypes.data, J)
        if rc:
            return rc
        bd = np.empty(self.N, np.uint32)
        nb, norm = C.c_uint64(), C.c_double()
        ref_lib().ref_info(self.h, bd.ctypes.data, C.byref(nb), C.byref(norm))
        self.bd, self.nblk, self.norm = [int(x) for x in bd], nb.value, norm.value
        return 0

    def partition(self):
        args, out = self._alloc_partition()
        ref_lib().ref_partition(self.h, *args)
        return out

    def init_random(self, seed=1, skip=0):
        ref_lib().ref_init_random(self.h, seed, skip)

    def get_factor(self, n):
        a = np.empty(self.factor_shape(n), NPDT[self.dtype])
        ref_lib().ref_get_factor(self.h, n, a.ctypes.data)
        return a

    def get_core(self):
        g = np.empty((self.J,) * self.N, NPDT[self.dtype])
        ref_lib().ref_get_core(self.h, g.ctypes.data)
        return g

    def delta(self, mode):
        d = np.empty((self.nnz, self.J), NPDT[self.dtype])
        ref_lib().ref_delta(self.h, mode, d.ctypes.data)
        return d

    def update_mode(self, mode):
        ref_lib().ref_update_mode(self.h, mode)

    def fit(self):
        e = C.c_double()
        f = ref_lib().ref_fit(self.h, C.byref(e))
        return f, e.value


def write_tns(path, idx, vals, dtype=1):
    """The reference's text format: 1-based indices and a value, tab-separated."""
    fmt = "%.17g" if dtype == 1 else "%.9g"
    with open(path, "w") as f:
        for t in range(len(vals)):
            f.write("\t".join(str(int(i[t]) + 1) for i in idx) + "\t" + (fmt % float(vals[t])) + "\n")


def random_coo(rng, dims, nnz, distinct=True, zipf=None):
    """Seeded small COO (0-based) with optional distinct coordinates and Zipf skew."""
    N = len(dims)
    out = []
    seen = set()
    tries = 0
    while len(out) < nnz and tries < nnz * 50:
        tries += 1
        if zipf:
            c = tuple(int(min(d - 1, rng.zipf(zipf) - 1)) for d in dims)
        else:
            c = tuple(int(rng.integers(0, d)) for d in dims)
        if distinct and c in seen:
            continue
        seen.add(c)
        out.append(c)
    idx = [np.array([c[n] for c in out], np.uint32) for n in range(N)]
    # make the max index of every mode appear, so dims are as given
    for n in range(N):
        if len(out):
            idx[n][n % len(out)] = dims[n] - 1
    return idx


def rel_fro(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


def ref_plan(dims, nnz, rank, dtype, gpus, mem):
    """Optimizer::FindPartitionParms of the reference (optimizer.tpp:71-89), compiled in
    place: (status, P, block_dims, block_count, dimension_based, streams, avail_nnz_per_task)."""
    N = len(dims)
    d = np.ascontiguousarray(dims, dtype=np.uint32)
    P = np.zeros(N, np.uint32)
    bd = np.zeros(N, np.uint32)
    info = np.zeros(4, np.uint64)
    st = ref_lib().ref_plan(N, d.ctypes.data, nnz, rank, dtype, gpus, mem, P.ctypes.data, bd.ctypes.data,
                            info.ctypes.data)
    return st, P.tolist(), bd.tolist(), int(info[0]), int(info[1]), int(info[2]), int(info[3])


def ws_oracle():
    """oracle/warmstart_oracle.py (the warm start's CPU restatement)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("warmstart_oracle", os.path.join(ROOT, "oracle",
                                                                                   "warmstart_oracle.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod
