// 32-bit packing of a pattern column's (row << 32 | slot) keys: (row - rmin)
// << sb | (slot - smin), valid when the row span and the slot span need at
// most 31 bits together.  The packing keeps the order of the keys and leaves
// ~0u above every packed key (the sorts' padding).
#pragma once
#include <stdint.h>

#include <cuda_runtime.h>

namespace elfel {

struct Pack32 {
  uint32_t rmin, smin;
  int sb;  // bits of the slot span
};

__host__ __device__ __forceinline__ uint32_t pack32(uint64_t v, const Pack32& p) {
  return (((uint32_t)(v >> 32) - p.rmin) << p.sb) | ((uint32_t)v - p.smin);
}

__host__ __device__ __forceinline__ uint64_t unpack32(uint32_t k, const Pack32& p) {
  return ((uint64_t)(p.rmin + (k >> p.sb)) << 32) | (uint64_t)(p.smin + (k & ((1u << p.sb) - 1u)));
}

}  // namespace elfel
