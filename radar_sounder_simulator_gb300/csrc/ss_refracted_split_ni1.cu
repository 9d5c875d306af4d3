// Split refracted kernels (fast pass and fix-up) for the joint solve through 1 interface.
#include "ss_refracted_split.cuh"

namespace ss {

int split_launch_ni1(RefArgs &a, const RefSplitConsts &k, const Plan &p,
                     size_t smem, cudaStream_t st) {
  return launch_split_r<1>(a, k, p, smem, st);
}

int refracted_batch_launch_ni1(const RefBatchJob *jobs, int n_jobs,
                               long long n_items, long long n_words,
                               unsigned long long *counter, int rough_kind,
                               bool plain, int ctas, size_t smem,
                               size_t fix_smem, cudaStream_t st) {
  return ref_batch_launch_r<1>(jobs, n_jobs, n_items, n_words, counter,
                               rough_kind, plain, ctas, smem, fix_smem, st);
}

int refracted_batch_occupancy_ni1(int rough_kind, bool plain, size_t smem) {
  return ref_batch_occupancy<1>(rough_kind, plain, smem);
}

}  // namespace ss
