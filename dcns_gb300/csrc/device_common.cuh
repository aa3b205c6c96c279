// Device helpers shared by the kernels: packed-sequence decode and score lookup.
#pragma once

#include "common.h"

namespace dcns {

// dCNS code (A0 C1 N2 G3 T4) of base k of the arena.
__device__ __forceinline__ int base_code(const Arena &ar, int64_t k) {
  const uint32_t w = __ldg(ar.pk + (k >> 4));
  const uint32_t two = (w >> ((uint32_t)(k & 15) * 2u)) & 3u;
  const uint32_t n = (__ldg(ar.nm + (k >> 5)) >> (uint32_t)(k & 31)) & 1u;
  return n ? 2 : (int)(two + (two >> 1));
}

// Scorei (model/Score.cpp:105-135): N (code 2) scores 0 against anything.
__device__ __forceinline__ int score_of(int a, int b, int match, int mismatch) {
  return (a == 2 || b == 2) ? 0 : (a == b ? match : mismatch);
}

// Sequence view for the DP kernels: forward (s[i] = seq[a + i]) or reverse-complement ending at a
// (s[i] = 4 - seq[a - i]).
struct SeqView {
  int64_t base;
  int32_t a, dir;
  __device__ __forceinline__ int at(const Arena &ar, int32_t i) const {
    return dir == 0 ? base_code(ar, base + a + i) : 4 - base_code(ar, base + a - i);
  }
};

}  // namespace dcns
