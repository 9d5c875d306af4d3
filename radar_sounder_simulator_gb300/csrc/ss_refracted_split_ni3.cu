// Split refracted kernels (fast pass and fix-up) for the joint solve through 3 interfaces.
#include "ss_refracted_split.cuh"

namespace ss {

int split_launch_ni3(RefArgs &a, const RefSplitConsts &k, const Plan &p,
                     size_t smem, cudaStream_t st) {
  return launch_split_r<3>(a, k, p, smem, st);
}

}  // namespace ss
