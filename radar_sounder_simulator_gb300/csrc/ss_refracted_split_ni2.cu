// Split refracted kernels (fast pass and fix-up) for the joint solve through 2 interfaces.
#include "ss_refracted_split.cuh"

namespace ss {

int split_launch_ni2(RefArgs &a, const RefSplitConsts &k, const Plan &p,
                     size_t smem, cudaStream_t st) {
  return launch_split_r<2>(a, k, p, smem, st);
}

}  // namespace ss
