// Device sorting and scan primitives.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"

namespace plan {

// Stable LSD radix sort of (w2:w1:w0) 96-bit keys carrying `payload`, in place.
// pass_mask selects which of the 12 byte-digits may be sorted (bit p = byte p, byte 0 is
// the least significant byte of w0); constant digits are skipped automatically.
size_t radix_sort96_scratch_bytes(size_t n);
int radix_sort96(uint32_t *w0, uint32_t *w1, uint32_t *w2, uint32_t *payload, size_t n, void *scratch, size_t scratch_bytes,
                 cudaStream_t stream, unsigned pass_mask = 0xfffu);

// Exclusive scan of n u32 values (out may alias in); *total receives the sum when non-null
// (device pointer).
size_t scan_u32_scratch_bytes(size_t n);
int scan_u32(const uint32_t *in, uint32_t *out, size_t n, uint32_t *d_total, void *scratch, size_t scratch_bytes, cudaStream_t stream);

// The exact arrangement std::sort (libstdc++ introsort) gives 96-bit keys in input order
// (w0..w2 low word first, ix the payload), in place; used when keys repeat, where the
// order of equal keys is the library's and not a stable one. Scratch: see below.
struct Context;
size_t morton_sort_scratch_bytes(size_t n);
int morton_sort_std(Context &c, uint32_t *w0, uint32_t *w1, uint32_t *w2, uint32_t *ix, uint32_t n, void *scratch, size_t bytes,
                    cudaStream_t stream);

}  // namespace plan
