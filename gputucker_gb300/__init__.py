"""gputucker_gb300 -- GB300-native sparse Tucker ALS (the GPUTucker factor-update path).

The compute path is the native library libgputucker_gb300.so (hand-written
sm_103a CUDA kernels behind a C ABI, include/gputucker_gb300.h); this package
is a thin host binding over it.
"""

from ._native import GTKError, LIB_PATH  # noqa: F401
from .tucker import (  # noqa: F401
    Batch,
    BlockedTensor,
    Coo,
    checkpoint_info,
    device_memory,
    plan_partition,
    coo_from_arrays,
    create_tensor_blocks,
    release_cached_memory,
    generate,
    generate_planted,
    parse_buffer,
    parse_from_file,
    tucker_decomposition,
    WarmStart,
    ws_features,
)

__all__ = [
    "GTKError", "LIB_PATH", "Batch", "BlockedTensor", "Coo", "checkpoint_info", "coo_from_arrays",
    "create_tensor_blocks", "release_cached_memory", "device_memory", "generate", "generate_planted", "parse_buffer", "parse_from_file",
    "plan_partition", "tucker_decomposition", "WarmStart", "ws_features",
]
