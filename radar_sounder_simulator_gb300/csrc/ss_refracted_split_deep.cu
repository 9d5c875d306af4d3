// Split refracted kernels (fast pass and fix-up) for the joint solve through
// 5 to SS_MAX_IFACE interfaces (deep stacks such as firn layering): the
// solve's per-interface arrays hold SS_MAX_IFACE entries and live in local
// memory; the count crossed is the call's.
#include "ss_refracted_split.cuh"

namespace ss {

int split_launch_deep(RefArgs &a, const RefSplitConsts &k, const Plan &p,
                      size_t smem, cudaStream_t st) {
  return launch_split_r<kDeepNI>(a, k, p, smem, st);
}

}  // namespace ss
