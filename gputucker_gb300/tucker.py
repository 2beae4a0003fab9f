"""Host-side API mirroring GPUTucker's interface for the factor-update path.

Reference interface (paths inside the GPUTucker project) -> this module:

    ParseFromFile(path, &tensor)            tensor_manager.tpp:19   -> parse_from_file
    CreateTensorBlocks(&src, &dst, opt)     tensor_manager.tpp:201  -> create_tensor_blocks
    init of factors/core in TuckerDecomposition  tucker.cuh:71-134  -> BlockedTensor.init_random
    UpdateFactorMatrices(...)               update.cuh:128          -> BlockedTensor.update_factor_matrices
    Reconstruction(..., &fit, ...)          reconstruction.cuh:228  -> BlockedTensor.reconstruction
    TuckerDecomposition(tensor, rank, gpus) tucker.cuh:30           -> tucker_decomposition

Every call goes through the C ABI of libgputucker_gb300.so (include/gputucker_gb300.h);
the arithmetic runs in that library's CUDA kernels.  Arrays cross as numpy
arrays in the reference's layouts (factor n = its slabs stacked, [P_n*block_dims[n], J]).
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _native as nat
from ._native import call

_DT = {"f32": nat.GTK_F32, "f64": nat.GTK_F64, np.float32: nat.GTK_F32, np.float64: nat.GTK_F64}
_NP = {nat.GTK_F32: np.float32, nat.GTK_F64: np.float64}


def _dtype_code(dtype) -> int:
    if isinstance(dtype, int):
        return dtype
    if isinstance(dtype, np.dtype):
        dtype = dtype.type
    return _DT[dtype]


def _ptr(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


class Coo:
    """A parsed tensor held on the host (one block, global 0-based coordinates)."""

    def __init__(self, handle: C.c_void_p):
        self._h = handle
        lib = nat.load()
        order, dtype, nnz, draws = C.c_int(), C.c_int(), C.c_uint64(), C.c_uint64()
        dims = (C.c_uint32 * nat.GTK_MAX_ORDER)()
        nat.check(lib.gtk_coo_info(handle, C.byref(order), C.byref(dtype), C.byref(nnz), dims, C.byref(draws)))
        self.order = order.value
        self.dtype = dtype.value
        self.nnz = nnz.value
        self.dims = [dims[i] for i in range(self.order)]
        self.rand_draws = draws.value

    @property
    def handle(self) -> C.c_void_p:
        if self._h is None:
            raise ValueError("Coo already freed")
        return self._h

    def arrays(self) -> tuple[list[np.ndarray], np.ndarray]:
        idx = [np.empty(self.nnz, np.uint32) for _ in range(self.order)]
        vals = np.empty(self.nnz, _NP[self.dtype])
        ptrs = (C.c_void_p * self.order)(*[a.ctypes.data for a in idx])
        call("gtk_coo_export", self.handle, ptrs, _ptr(vals))
        return idx, vals

    def pin(self) -> None:
        """Page-lock the host arrays (cudaHostRegister) for full-speed uploads."""
        call("gtk_coo_pin", self.handle)

    def write_text(self, path: str) -> None:
        call("gtk_write_text", self.handle, str(path).encode())

    def free(self) -> None:
        if self._h is not None:
            nat.load().gtk_coo_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def parse_from_file(path: str, order: int, dtype="f64", rand_seed: int = 1) -> Coo:
    """The reference's text format (tensor_manager.tpp:19-191); see gtk_parse_file."""
    h = C.c_void_p()
    call("gtk_parse_file", str(path).encode(), order, _dtype_code(dtype), rand_seed, C.byref(h))
    return Coo(h)


def parse_buffer(data: bytes, order: int, dtype="f64", rand_seed: int = 1) -> Coo:
    h = C.c_void_p()
    call("gtk_parse_buffer", data, len(data), order, _dtype_code(dtype), rand_seed, C.byref(h))
    return Coo(h)


def coo_from_arrays(indices, values: np.ndarray, dims=None) -> Coo:
    """COO from 0-based coordinate arrays (one per mode) and values (float32/float64)."""
    values = np.ascontiguousarray(values)
    code = _dtype_code(values.dtype)
    idx = [np.ascontiguousarray(i, dtype=np.uint32) for i in indices]
    order = len(idx)
    ptrs = (C.c_void_p * order)(*[a.ctypes.data for a in idx])
    d = None
    if dims is not None:
        d = np.ascontiguousarray(dims, dtype=np.uint32)
    h = C.c_void_p()
    call("gtk_coo_from_arrays", order, len(values), ptrs, _ptr(values), code,
         _ptr(d) if d is not None else None, C.byref(h))
    return Coo(h)


def generate(order: int, dims, nnz: int, index_dist: str = "zipf", zipf_s: float = 1.1,
             value_dist: str = "uniform", dtype="f32", seed: int = 0) -> Coo:
    """Seeded synthetic tensor with distinct coordinates (gtk_generate)."""
    d = np.ascontiguousarray(dims, dtype=np.uint32)
    idist = {"uniform": nat.GTK_GEN_UNIFORM, "zipf": nat.GTK_GEN_ZIPF}[index_dist]
    vdist = {"uniform": nat.GTK_VAL_UNIFORM, "lognormal": nat.GTK_VAL_LOGNORMAL}[value_dist]
    h = C.c_void_p()
    call("gtk_generate", order, d.ctypes.data_as(nat.U32P), nnz, idist, zipf_s, vdist, _dtype_code(dtype), seed,
         C.byref(h))
    return Coo(h)


def generate_planted(order: int, dims, nnz: int, planted_rank: int, noise_sigma: float, dtype="f32",
                     seed: int = 0) -> Coo:
    d = np.ascontiguousarray(dims, dtype=np.uint32)
    h = C.c_void_p()
    call("gtk_generate_planted", order, d.ctypes.data_as(nat.U32P), nnz, planted_rank, noise_sigma,
         _dtype_code(dtype), seed, C.byref(h))
    return Coo(h)


@dataclass
class Info:
    order: int
    rank: int
    dtype: int
    device: int
    nnz: int
    block_count: int
    dims: list
    partition_dims: list
    block_dims: list
    norm: float
    device_bytes: int
    streamed: bool = False
    stream_chunk: int = 0
    host_direct: bool = False


class BlockedTensor:
    """A blocked sparse tensor with its factor matrices and core, resident on one GPU."""

    def __init__(self, handle: C.c_void_p):
        self._h = handle
        self.info = self._info()
        self.order = self.info.order
        self.rank = self.info.rank
        self.np_dtype = _NP[self.info.dtype]

    @property
    def handle(self) -> C.c_void_p:
        if self._h is None:
            raise ValueError("tensor already destroyed")
        return self._h

    def _info(self) -> Info:
        ti = nat.TensorInfo()
        call("gtk_tensor_info_get", self._h, C.byref(ti))
        n = ti.order
        return Info(ti.order, ti.rank, ti.dtype, ti.device, ti.nnz, ti.block_count, list(ti.dims[:n]),
                    list(ti.partition_dims[:n]), list(ti.block_dims[:n]), ti.norm, ti.device_bytes,
                    bool(ti.streamed), ti.stream_chunk, bool(ti.host_direct))

    # ---- partition readback (bit-exact with the reference's blocks)
    def block(self, b: int):
        """(block coordinate, block-local coords per mode, values) of block b."""
        coord = (C.c_uint32 * self.order)()
        nnz = C.c_uint64()
        call("gtk_block_info", self.handle, b, coord, C.byref(nnz))
        n = nnz.value
        idx = [np.empty(n, np.uint32) for _ in range(self.order)]
        vals = np.empty(n, self.np_dtype)
        ptrs = (C.c_void_p * self.order)(*[a.ctypes.data for a in idx])
        call("gtk_block_data", self.handle, b, ptrs, _ptr(vals))
        return list(coord), idx, vals

    def segments(self, b: int, mode: int):
        """(count_nnz, where_nnz) of block b for `mode` (block.tpp:115-186)."""
        _, nnz = self.block_nnz(b)
        cnt = np.empty(self.info.block_dims[mode] + 1, np.uint64)
        where = np.empty(nnz, np.uint32)
        call("gtk_block_segments", self.handle, b, mode, _ptr(cnt), _ptr(where))
        return cnt, where

    def block_nnz(self, b: int):
        coord = (C.c_uint32 * self.order)()
        nnz = C.c_uint64()
        call("gtk_block_info", self.handle, b, coord, C.byref(nnz))
        return list(coord), nnz.value

    # ---- factors and core
    def init_random(self, rand_seed: int = 1, skip_draws: int = 0) -> None:
        call("gtk_init_random", self.handle, rand_seed, skip_draws)

    def factor_rows(self, mode: int) -> int:
        return self.info.partition_dims[mode] * self.info.block_dims[mode]

    def get_factor(self, mode: int) -> np.ndarray:
        a = np.empty((self.factor_rows(mode), self.rank), self.np_dtype)
        call("gtk_get_factor", self.handle, mode, _ptr(a))
        return a

    def set_factor(self, mode: int, a: np.ndarray) -> None:
        a = np.ascontiguousarray(a, dtype=self.np_dtype)
        if a.shape != (self.factor_rows(mode), self.rank):
            raise ValueError(f"factor {mode} must have shape {(self.factor_rows(mode), self.rank)}")
        call("gtk_set_factor", self.handle, mode, _ptr(a))

    def get_core(self) -> np.ndarray:
        g = np.empty((self.rank,) * self.order, self.np_dtype)
        call("gtk_get_core", self.handle, _ptr(g))
        return g

    def set_core(self, g: np.ndarray) -> None:
        g = np.ascontiguousarray(g, dtype=self.np_dtype)
        if g.size != self.rank ** self.order:
            raise ValueError("core must have J^N entries")
        call("gtk_set_core", self.handle, _ptr(g))

    # ---- the sweep
    def set_precision(self, precision: str) -> None:
        code = {"plain": nat.GTK_PREC_PLAIN, "bf16": nat.GTK_PREC_BF16, "tf32": nat.GTK_PREC_TF32}[precision]
        call("gtk_set_precision", self.handle, code)

    def update_mode(self, mode: int) -> None:
        call("gtk_update_mode", self.handle, mode)

    def update_factor_matrices(self) -> None:
        call("gtk_update_factor_matrices", self.handle)

    def validate(self) -> list[int]:
        """gtk_validate: violation counts of the device arrays' consistency checks
        (all zero for a handle built by create_tensor_blocks)."""
        out = np.zeros(nat.GTK_VALIDATE_CHECKS, np.uint64)
        call("gtk_validate", self.handle, out.ctypes.data_as(nat.U64P))
        return [int(x) for x in out]

    def update_core(self, cg_iters: int = 10) -> tuple[int, float]:
        """Least-squares core with the factors fixed (no reference counterpart:
        GPUTucker never updates G).  Returns (CG steps taken, relative residual
        of the normal equations)."""
        k = C.c_int()
        res = C.c_double()
        call("gtk_update_core", self.handle, cg_iters, C.byref(k), C.byref(res))
        return k.value, res.value

    def reconstruction(self) -> float:
        f = C.c_double()
        call("gtk_reconstruction", self.handle, C.byref(f))
        return f.value

    def sweep(self) -> float:
        """One ALS sweep (all modes) and its fit; replays a CUDA graph when set_graph(True)."""
        f = C.c_double()
        call("gtk_sweep", self.handle, C.byref(f))
        return f.value

    def set_graph(self, on: bool = True) -> None:
        call("gtk_set_graph", self.handle, 1 if on else 0)

    # ---- checkpoint
    def checkpoint_save(self, path: str, fits=()) -> None:
        """Factors, core and fit history to `path` (gtk_checkpoint_save)."""
        f = (C.c_double * max(1, len(fits)))(*fits)
        call("gtk_checkpoint_save", self.handle, str(path).encode(), f, len(fits))

    def checkpoint_load(self, path: str, fits_cap: int = 1024) -> list:
        """Restore factors and core from `path`; returns the saved fit history."""
        f = (C.c_double * max(1, fits_cap))()
        n = C.c_int()
        call("gtk_checkpoint_load", self.handle, str(path).encode(), f, fits_cap, C.byref(n))
        k = min(n.value, fits_cap)
        return [f[i] for i in range(k)]

    VARIANTS = {"auto": -1, "simt2": 0, "simt1": 1, "generic": 2, "tensor_core": 3, "reference_order": 4}

    def set_kernel_variant(self, variant: str) -> None:
        """Force the update kernel ('auto', 'simt2', 'simt1', 'generic', 'tensor_core', 'reference_order')."""
        call("gtk_set_kernel_variant", self.handle, self.VARIANTS[variant])

    def kernel_variant(self) -> str:
        v = C.c_int()
        call("gtk_get_kernel_variant", self.handle, C.byref(v))
        return {c: n for n, c in self.VARIANTS.items()}[v.value]

    def autotune(self) -> str:
        """Time the applicable update kernels on mode 0, each at the tile shapes of
        ctas_per_sm() in (as many as fit, 2, 1), and keep the fastest pair
        (factors unchanged); returns the variant."""
        v = C.c_int()
        call("gtk_autotune", self.handle, C.byref(v))
        return {c: n for n, c in self.VARIANTS.items()}[v.value]

    def set_ctas_per_sm(self, ctas: int) -> None:
        """Size the update kernels' grids for `ctas` CTAs per SM (0: as many as fit)."""
        call("gtk_set_ctas_per_sm", self.handle, ctas)

    def ctas_per_sm(self) -> int:
        c = C.c_int()
        call("gtk_get_ctas_per_sm", self.handle, C.byref(c))
        return c.value

    def tucker_decomposition(self, max_iters: int = 3, tol: float = 1e-4) -> list:
        fits = (C.c_double * max_iters)()
        it = C.c_int()
        call("gtk_tucker_decomposition", self.handle, max_iters, tol, fits, C.byref(it))
        return [fits[i] for i in range(it.value)]

    def compute_delta(self, mode: int) -> np.ndarray:
        d = np.empty((self.info.nnz, self.rank), self.np_dtype)
        call("gtk_compute_delta", self.handle, mode, _ptr(d))
        return d

    # ---- timing
    def profile(self, on: bool = True) -> None:
        call("gtk_profile_enable", self.handle, 1 if on else 0)

    def profile_read(self, kind: int) -> tuple[float, int]:
        ms, n = C.c_double(), C.c_uint64()
        call("gtk_profile_read", self.handle, kind, C.byref(ms), C.byref(n))
        return ms.value, n.value

    def solve_counters(self, reset: bool = False) -> tuple[int, int]:
        """(rows re-solved in FP64 by the precision forms, rows solved by pivoted LU)
        since creation or the last reset (gtk_solve_counters)."""
        f, l = C.c_uint64(), C.c_uint64()
        call("gtk_solve_counters", self.handle, C.byref(f), C.byref(l), 1 if reset else 0)
        return f.value, l.value

    def profile_reset(self) -> None:
        call("gtk_profile_reset", self.handle)

    def timer_begin(self) -> None:
        call("gtk_timer_begin", self.handle)

    def timer_end(self) -> float:
        ms = C.c_double()
        call("gtk_timer_end", self.handle, C.byref(ms))
        return ms.value

    def synchronize(self) -> None:
        call("gtk_synchronize", self.handle)

    def close(self) -> None:
        if self._h is not None:
            nat.load().gtk_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Several BlockedTensors on one device swept together (gtk_batch_*): the first
    sweep runs eagerly, later ones replay one CUDA graph in which every tensor's
    sweep is an independent branch.  Close the batch before its tensors."""

    def __init__(self, tensors):
        self.tensors = list(tensors)
        tab = (C.c_void_p * len(self.tensors))(*[t.handle for t in self.tensors])
        h = C.c_void_p()
        call("gtk_batch_create", tab, len(self.tensors), C.byref(h))
        self._h = h

    def sweep(self) -> np.ndarray:
        fits = (C.c_double * len(self.tensors))()
        call("gtk_batch_sweep", self._h, fits)
        return np.array(fits[:], dtype=np.float64)

    def kernels(self) -> int:
        n = C.c_uint64()
        call("gtk_batch_kernels", self._h, C.byref(n))
        return n.value

    def close(self) -> None:
        if self._h is not None:
            nat.load().gtk_batch_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def plan_partition(dims, nnz: int, rank: int, dtype="f32", gpu_count: int = 1, gpu_mem_bytes: int | None = None,
                   device: int = 0) -> dict:
    """Optimizer::FindPartitionParms (optimizer.tpp:71-89): P_n for a tensor of this size on
    gpu_count GPUs of gpu_mem_bytes each (default: the free memory of `device`)."""
    if gpu_mem_bytes is None:
        gpu_mem_bytes = device_memory(device)[0]
    d = np.ascontiguousarray(dims, dtype=np.uint32)
    plan = nat.Plan()
    call("gtk_plan_partition", len(d), d.ctypes.data_as(nat.U32P), nnz, rank, _dtype_code(dtype), gpu_count,
         gpu_mem_bytes, C.byref(plan))
    N = len(d)
    return dict(partition_dims=list(plan.partition_dims[:N]), block_dims=list(plan.block_dims[:N]),
                block_count=plan.block_count, dimension_based=bool(plan.dimension_based), streams=plan.streams,
                avail_nnz_per_task=plan.avail_nnz_per_task, required_bytes=plan.required_bytes,
                block_bytes=plan.block_bytes)


def device_memory(device: int = 0) -> tuple[int, int]:
    """(free, total) bytes of a device (cudaMemGetInfo)."""
    f, t = C.c_uint64(), C.c_uint64()
    call("gtk_device_memory", device, C.byref(f), C.byref(t))
    return f.value, t.value


def checkpoint_info(path: str) -> dict:
    """Header of a checkpoint file (no device needed)."""
    o, r, d, nf = C.c_int(), C.c_int(), C.c_int(), C.c_int()
    dims = (C.c_uint32 * nat.GTK_MAX_ORDER)()
    P = (C.c_uint32 * nat.GTK_MAX_ORDER)()
    call("gtk_checkpoint_info", str(path).encode(), C.byref(o), C.byref(r), C.byref(d), dims, P, C.byref(nf))
    return dict(order=o.value, rank=r.value, dtype="f64" if d.value == nat.GTK_F64 else "f32",
                dims=list(dims[:o.value]), partition_dims=list(P[:o.value]), nfits=nf.value)


class WarmStart:
    """Learned warm start (gtk_ws_*): an MLP from per-row statistics to initial factor rows,
    trained and run by the library's CUDA kernels.  Uniform [0,1) init stays the fallback."""

    def __init__(self, order: int, rank: int, hidden: int = 64, seed: int = 0, device: int = 0):
        h = C.c_void_p()
        call("gtk_ws_create", order, rank, hidden, seed, device, C.byref(h))
        self._h = h
        self.order, self.rank, self.hidden = order, rank, hidden
        f, n = C.c_int(), C.c_uint64()
        call("gtk_ws_info", h, C.byref(f), C.byref(n), None)
        self.features, self.n_params = f.value, n.value

    @property
    def handle(self):
        if self._h is None:
            raise ValueError("warm-start model is closed")
        return self._h

    def examples(self) -> int:
        n = C.c_uint64()
        call("gtk_ws_info", self.handle, None, None, C.byref(n))
        return n.value

    def add_example(self, t: BlockedTensor) -> None:
        call("gtk_ws_add_example", self.handle, t.handle)

    def train(self, steps: int, batch: int = 1024, lr: float = 1e-3) -> float:
        loss = C.c_double()
        call("gtk_ws_train", self.handle, steps, batch, lr, C.byref(loss))
        return loss.value

    def apply(self, t: BlockedTensor) -> None:
        call("gtk_ws_apply", self.handle, t.handle)

    def save(self, path: str) -> None:
        """The trained model to a file (gtk_ws_save)."""
        call("gtk_ws_save", self.handle, str(path).encode())

    @classmethod
    def load(cls, path: str, device: int = 0) -> "WarmStart":
        """A model saved by save() (gtk_ws_load)."""
        h = C.c_void_p()
        call("gtk_ws_load", str(path).encode(), device, C.byref(h))
        m = cls.__new__(cls)
        m._h = h
        f, n = C.c_int(), C.c_uint64()
        call("gtk_ws_info", h, C.byref(f), C.byref(n), None)
        m.features, m.n_params = f.value, n.value
        with open(path, "rb") as fh:  # order, rank, width from the header (checked by gtk_ws_load)
            m.order, m.rank, m.hidden, _ = np.frombuffer(fh.read(24)[8:], np.uint32).tolist()
        return m

    def get_params(self):
        p = np.empty(self.n_params, np.float32)
        mu = np.empty(self.features, np.float32)
        sd = np.empty(self.features, np.float32)
        call("gtk_ws_get_params", self.handle, _ptr(p), _ptr(mu), _ptr(sd))
        return p, mu, sd

    def set_params(self, params=None, feat_mean=None, feat_std=None) -> None:
        arrs = [None if a is None else np.ascontiguousarray(a, np.float32) for a in (params, feat_mean, feat_std)]
        call("gtk_ws_set_params", self.handle, *[None if a is None else _ptr(a) for a in arrs])

    def loss_grad(self, x, t):
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        g = np.empty(self.n_params, np.float32)
        loss = C.c_double()
        call("gtk_ws_loss_grad", self.handle, _ptr(x), _ptr(t), x.shape[0], C.byref(loss), _ptr(g))
        return loss.value, g

    def predict(self, x):
        x = np.ascontiguousarray(x, np.float32)
        y = np.empty((x.shape[0], self.rank), np.float32)
        call("gtk_ws_predict", self.handle, _ptr(x), x.shape[0], _ptr(y))
        return y

    def close(self) -> None:
        if self._h is not None:
            nat.load().gtk_ws_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def ws_features(t: BlockedTensor, mode: int) -> np.ndarray:
    """Raw warm-start features of every row of `mode` (rows x F)."""
    F = 4 + 6 * (t.order - 1) + t.order
    out = np.empty((t.factor_rows(mode), F), np.float32)
    call("gtk_ws_features", t.handle, mode, _ptr(out))
    return out


def release_cached_memory() -> None:
    """Return the device blocks the library keeps cached to the driver
    (gtk_release_cached_memory)."""
    nat.load().gtk_release_cached_memory()


def create_tensor_blocks(coo: Coo, partition_dims, rank: int, device: int = 0) -> BlockedTensor:
    """CreateTensorBlocks + AssignIndicesOfEachBlock on the GPU (gtk_create_blocks)."""
    P = np.ascontiguousarray(partition_dims, dtype=np.uint32)
    if len(P) != coo.order:
        raise ValueError("one partition parameter per mode")
    h = C.c_void_p()
    call("gtk_create_blocks", coo.handle, P.ctypes.data_as(nat.U32P), rank, device, C.byref(h))
    return BlockedTensor(h)


def tucker_decomposition(coo: Coo, rank: int, partition_dims=None, max_iters: int = 3, tol: float = 1e-4,
                         rand_seed: int = 1, device: int = 0):
    """TuckerDecomposition (tucker.cuh:30-190): blocks, init from the glibc stream that
    continues after the parser's draws, then sweeps until max_iters or |dfit| <= tol.
    Returns (tensor, fits)."""
    if partition_dims is None:  # the reference plans P_n from the GPU memory (tucker.cuh:49-55)
        partition_dims = plan_partition(coo.dims, coo.nnz, rank, coo.dtype, 1, None, device)["partition_dims"]
    t = create_tensor_blocks(coo, partition_dims, rank, device)
    t.init_random(rand_seed, coo.rand_draws)
    return t, t.tucker_decomposition(max_iters, tol)
