// Split-precision (BF16 slices on tcgen05 tensor cores) path of the K build.
#pragma once
#include <string>
#include <vector>

#include "common.cuh"

namespace gbjk {

constexpr int kMaxSlices = 8;

struct SplitState {
  size_t bytes = 0;
  void init(int, int, int, const std::vector<int>&, const std::vector<int>&,
            const std::vector<int>&, const std::vector<int>&, const std::vector<long long>&) {}
  void release() {}
  void invalidate_b() {}
  void reset_profile() {}
  int profile_read(int, const char**, double*, int64_t*) const { return 0; }
  gbjk_status prepare(cudaStream_t, const double*, const double*, const double*, const double*,
                      int, int, int64_t*, size_t*, std::string* err) {
    *err = "split-precision path not available in this build";
    return GBJK_NOT_READY;
  }
};

inline gbjk_status split_run_k(SplitState&, cudaStream_t, int, int, double*, int64_t*,
                               std::string* err) {
  *err = "split-precision path not available in this build";
  return GBJK_NOT_READY;
}

}  // namespace gbjk
