// Host utilities and shared float64 device functions.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <mutex>

#include "ss_internal.cuh"

namespace ss {

static thread_local char g_last_error[256] = "";

void set_error(const char *msg) {
  strncpy(g_last_error, msg, sizeof(g_last_error) - 1);
  g_last_error[sizeof(g_last_error) - 1] = 0;
}

int cuda_status(cudaError_t e, const char *where) {
  if (e == cudaSuccess) return SS_OK;
  char buf[256];
  snprintf(buf, sizeof(buf), "%s: %s", where, cudaGetErrorString(e));
  set_error(buf);
  return SS_ERR_CUDA;
}

// Weideman (1994): with M = 2N, L = sqrt(N / sqrt 2), t_k = L tan(pi k / 2M),
// a_j = (1/2M) sum_{|k|<M} exp(-t_k^2) (L^2 + t_k^2) cos(pi j k / M); the
// rational approximation uses a_1..a_N (roughness.py:56-64 computes the same
// numbers by an FFT of the shifted samples).
const FadCoeffs &faddeeva_coeffs() {
  static FadCoeffs c;
  static std::once_flag once;
  std::call_once(once, [] {
    const int n = SS_FAD_N, m = 2 * n;
    const double L = sqrt(n / sqrt(2.0));
    double a[SS_FAD_N + 1];
    for (int j = 0; j <= n; ++j) {
      double s = 0.0;
      for (int k = -m + 1; k < m; ++k) {
        double t = L * tan(kPi * k / (2.0 * m));
        double f = exp(-t * t) * (L * L + t * t);
        s += f * cos(kPi * (double)j * (double)k / (double)m);
      }
      a[j] = s / (2.0 * m);
    }
    c.L = L;
    for (int j = 0; j < n; ++j) c.a[j] = a[n - j];  // highest power first
  });
  return c;
}

}  // namespace ss

extern "C" const char *ss_last_error(void) { return ss::g_last_error; }

extern "C" const char *ss_version(void) {
  return "soundersim_gb300 kernels 2026-12 sm_103a";
}
