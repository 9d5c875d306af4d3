// Split refracted kernels (fast pass and fix-up) for the joint solve through 3 interfaces.
#include "ss_refracted_split.cuh"

namespace ss {

int split_launch_ni3(RefArgs &a, const RefSplitConsts &k, const Plan &p,
                     size_t smem, cudaStream_t st) {
  return launch_split_r<3>(a, k, p, smem, st);
}

int refracted_batch_launch_ni3(const RefBatchJob *jobs, int n_jobs,
                               long long n_items, long long n_words,
                               unsigned long long *counter, int rough_kind,
                               bool plain, int ctas, size_t smem,
                               size_t fix_smem, cudaStream_t st) {
  return ref_batch_launch_r<3>(jobs, n_jobs, n_items, n_words, counter,
                               rough_kind, plain, ctas, smem, fix_smem, st);
}

int refracted_batch_occupancy_ni3(int rough_kind, bool plain, size_t smem) {
  return ref_batch_occupancy<3>(rough_kind, plain, smem);
}

}  // namespace ss
