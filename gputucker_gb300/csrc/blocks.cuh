// blocks.cuh -- device helpers over the block-major arrays of a handle.
#pragma once

#include <cstdint>

namespace gtk {

// block of block-major position t: the last b with blk_ptr[b] <= t (empty blocks
// share their start with the next block and are skipped)
__device__ __forceinline__ uint32_t block_of(const uint64_t *__restrict__ blk_ptr, uint32_t nblk, uint64_t t) {
  uint32_t lo = 0, hi = nblk;  // blk_ptr[lo] <= t < blk_ptr[hi]
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) / 2;
    if (blk_ptr[mid] <= t)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

}  // namespace gtk
