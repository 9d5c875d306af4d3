// Adjoint of the split refracted kernel: the joint solve's instantiations
// through 1 and 2 interfaces (device code in ss_refracted_adjoint.cuh;
// split across translation units so the build compiles them in parallel).
#include "ss_refracted_adjoint.cuh"

namespace ss {

int adjoint_launch_joint12(RefArgs &a, const RefSplitConsts &k,
                           const AdjArgs &j, size_t smem, cudaStream_t st) {
  switch (a.ni) {
    case 1: return adjoint_launch_ni<1>(a, k, j, smem, st);
    case 2: return adjoint_launch_ni<2>(a, k, j, smem, st);
    default:
      set_error("joint adjoint: unsupported interface count");
      return SS_ERR_UNSUPPORTED;
  }
}

}  // namespace ss
