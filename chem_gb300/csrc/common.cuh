// Shared device-side helpers and the engine context of libgbjk.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "gbjk.h"

namespace gbjk {

// One GEMM of a grouped launch: C = alpha * A * op(B) (+ C if kAccum).
// A is M x K row-major (lda); B is K x N row-major (ldb) or, with kTransB,
// N x K row-major so that op(B)(k, n) = B[n * ldb + k].
struct GemmGroup {
  const double* A;
  const double* B;
  double* C;
  int M, N, K;
  int lda, ldb, ldc;
  int flags;
};
enum : int { kTransB = 1, kLowerA = 2, kAccum = 4 };

// One output tile of a group (64 rows x 64 or 16 columns), over the k range
// [k0, k1); the tile is written at C + coff (split-K partial buffers).
struct GemmTile {
  int group, mt, nt, k0, k1;
  long long coff;
};

struct Profile {
  const char* name;
  double ms = 0.0;
  int64_t launches = 0;
};

}  // namespace gbjk
