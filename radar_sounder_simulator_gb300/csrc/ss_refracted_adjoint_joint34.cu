// Adjoint of the split refracted kernel: the joint solve's instantiations
// through 3 and 4 interfaces (device code in ss_refracted_adjoint.cuh;
// split across translation units so the build compiles them in parallel).
#include "ss_refracted_adjoint.cuh"

namespace ss {

int adjoint_launch_joint34(RefArgs &a, const RefSplitConsts &k,
                           const AdjArgs &j, size_t smem, cudaStream_t st) {
  switch (a.ni) {
    case 3: return adjoint_launch_ni<3>(a, k, j, smem, st);
    case 4: return adjoint_launch_ni<4>(a, k, j, smem, st);
    default:
      set_error("joint adjoint: unsupported interface count");
      return SS_ERR_UNSUPPORTED;
  }
}

}  // namespace ss
