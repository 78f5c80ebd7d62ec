// sv_noalloc_grid.h -- launch-size rule of the collapse entry point that allocates
// nothing (sv_collapse_state_noalloc), kept free of CUDA types so host code and CPU
// tests can evaluate it.
//
// The norm reduction runs one block of `block` threads per `block` kept amplitudes,
// capped at 8 blocks per SM; every block writes one FP64 partial and the finish kernel
// writes two more values (norm^2, 1/norm), all into a static device array of
// kNoAllocScratchDoubles doubles.
#pragma once

#include <stdint.h>

namespace sv {

constexpr int kNoAllocScratchDoubles = 4096;  // 32 KiB

inline unsigned noalloc_grid(int64_t work, int num_sms, int block) {
  const int64_t cap = (int64_t)num_sms * 8;
  int64_t g = (work + block - 1) / block;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (unsigned)g;
}

// true when the partials of a reduction over `grid` blocks fit the static array
inline bool noalloc_norm_fits(unsigned grid) { return (int64_t)grid + 2 <= kNoAllocScratchDoubles; }

}  // namespace sv
