// Split-precision refracted kernel (placeholder until the float32 solve
// lands): reports the option as unsupported.
#include "ss_refracted.cuh"

namespace ss {

int refracted_split_launch(RefArgs &a, const Plan &p, cudaStream_t st) {
  (void)a; (void)p; (void)st;
  set_error("split precision not yet available for the refracted kernel");
  return SS_ERR_UNSUPPORTED;
}

}  // namespace ss
