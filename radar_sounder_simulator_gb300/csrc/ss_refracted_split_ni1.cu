// Split refracted kernels (fast pass and fix-up) for the joint solve through 1 interface.
#include "ss_refracted_split.cuh"

namespace ss {

int split_launch_ni1(RefArgs &a, const RefSplitConsts &k, const Plan &p,
                     size_t smem, cudaStream_t st) {
  return launch_split_r<1>(a, k, p, smem, st);
}

}  // namespace ss
