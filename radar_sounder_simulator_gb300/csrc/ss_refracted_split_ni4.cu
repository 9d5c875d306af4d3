// Split refracted kernels (fast pass and fix-up) for the joint solve through 4 interfaces.
#include "ss_refracted_split.cuh"

namespace ss {

int split_launch_ni4(RefArgs &a, const RefSplitConsts &k, const Plan &p,
                     size_t smem, cudaStream_t st) {
  return launch_split_r<4>(a, k, p, smem, st);
}

}  // namespace ss
