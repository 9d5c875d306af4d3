// Refracted multilayer kernel: argument block (internal).
#pragma once

#include "ss_internal.cuh"

namespace ss {

struct RefArgs {
  ss_facets F;
  const double *pos, *uct, *pv;
  const int32_t *off;
  int T, N, pv_len;
  // crossed stack (top-down, joint pads first)
  int ni, k_pad, leg_last;  // final leg uses leg index leg_last
  ss_interface ifc[SS_MAX_IFACE];
  double n_leg[SS_MAX_IFACE + 1], eps_leg[SS_MAX_IFACE + 1],
      att_leg[SS_MAX_IFACE + 1], sig_c[SS_MAX_IFACE];
  int rough_cross;
  double k0, gamma, t0, dt, c, taper_s, n_exp;
  int n_samples, n_seg, bs, n_win, split, coherent, joint, n_newton,
      n_backtrack, taper, precision;
  int pat_kind, pat_n;
  const double *pa, *pb;
  int rough_kind, n_terms;
  double sigma, corr;
  FadCoeffs fad;
  int tb, n_chunks;
  void *part;
  double *part_drop;
  // split form: one bit per (trace, window slot) for pairs deferred to the
  // fix-up kernel; defer_w = window slots per trace
  uint32_t *defer_mask;
  long long defer_w;
};

// Threads per CTA of the split fast kernel (its __launch_bounds__).
constexpr int kSplitThreads = 512;

int refracted_split_launch(RefArgs &a, const Plan &p, cudaStream_t st);

// Validate one refracted call and fill its argument block (everything but
// the scratch layout); shared by the forward and adjoint entry points.
int build_ref_args(const ss_refracted_opts *opts, const ss_facets *target,
                   const ss_traces *traces, const ss_pattern *pattern,
                   const ss_roughness *rough, bool need_output,
                   const ss_output *out, Plan &p, RefArgs &a);

// Adjoint inputs and outputs (see ss_refracted_adjoint).
struct AdjArgs {
  const double *field;       // (T, n_seg, 2) forward field
  const double *grad_power;  // (T,) dL/dP_t
  int bin_lo, bin_hi;        // power window [bin_lo, bin_hi)
  double *grad_gamma_db;     // (N,)
  double *grad_sigma;        // (N,) or null
  double *grad_alpha;        // (refracted_adjoint_blocks(N),) partials
  uint32_t *defer_mask;      // T x N bits: pairs for the fix-up pass
};

int refracted_adjoint_blocks(int N);
size_t refracted_adjoint_mask_bytes(int T, int N);
int refracted_adjoint_launch(RefArgs &a, const AdjArgs &j,
                             const double *alpha_mask, cudaStream_t st);

}  // namespace ss
