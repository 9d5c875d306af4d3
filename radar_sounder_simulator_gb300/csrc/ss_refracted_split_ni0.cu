// Split refracted kernels (fast pass and fix-up) for the sequential path.
#include "ss_refracted_split.cuh"

namespace ss {

int split_launch_ni0(RefArgs &a, const RefSplitConsts &k, const Plan &p,
                     size_t smem, cudaStream_t st) {
  return launch_split_r<0>(a, k, p, smem, st);
}

}  // namespace ss
