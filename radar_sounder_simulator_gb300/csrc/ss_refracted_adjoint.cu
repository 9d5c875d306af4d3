// Adjoint of the split refracted kernel: host dispatch and the sequential
// chain's instantiations (device code in ss_refracted_adjoint.cuh).
#include "ss_refracted_adjoint.cuh"

namespace ss {

int refracted_adjoint_blocks(int N) {
  return (N + kAdjThreads - 1) / kAdjThreads;
}

size_t refracted_adjoint_mask_bytes(int T, int N) {
  return (size_t)(((unsigned long long)T * N + 31) / 32) * sizeof(uint32_t);
}

int refracted_adjoint_launch(RefArgs &a, const AdjArgs &j,
                             const double *alpha_mask, cudaStream_t st) {
  int pa_len, pb_len;
  pattern_lengths(a.pat_kind, a.pat_n, pa_len, pb_len);
  if (pa_len + pb_len > SS_PAT_MAX) {
    set_error("antenna table too large for the split kernel");
    return SS_ERR_UNSUPPORTED;
  }
  if (a.joint && a.ni > 4) {
    set_error("the joint-path adjoint supports up to 4 interfaces");
    return SS_ERR_UNSUPPORTED;
  }
  if (!a.coherent || a.split) {
    set_error("the adjoint needs coherent mode without split sides");
    return SS_ERR_UNSUPPORTED;
  }
  RefSplitConsts k = split_consts(a);
  for (int m = 0; m <= a.leg_last; ++m)
    k.att_mask[m] = alpha_mask ? (float)alpha_mask[m] : 0.0f;
  const size_t smem =
      a.rough_kind ? (size_t)(a.n_terms + 1) * sizeof(float) : 0;
  cudaError_t e = cudaMemsetAsync(
      j.defer_mask, 0, refracted_adjoint_mask_bytes(a.T, a.N), st);
  if (e != cudaSuccess) return cuda_status(e, "adjoint mask clear");
  if (a.joint)
    return a.ni <= 2 ? adjoint_launch_joint12(a, k, j, smem, st)
                     : adjoint_launch_joint34(a, k, j, smem, st);
  return adjoint_launch_ni<0>(a, k, j, smem, st);
}

}  // namespace ss
