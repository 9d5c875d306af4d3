// Split-precision refracted multilayer kernel: host-side constants and the
// dispatch over the crossed-interface count. The device code and its
// precision design are described in ss_refracted_split.cuh; each
// interface count is compiled in its own translation unit
// (ss_refracted_split_ni*.cu) so the build runs them in parallel.
#include "ss_refracted_split.cuh"

namespace ss {

// float32 / double-float constants of the split kernels.
RefSplitConsts split_consts(const RefArgs &a) {
  RefSplitConsts k{};
  k.k0 = (float)a.k0;
  const double kj = a.k0 * a.n_leg[a.leg_last];
  k.kj = (float)kj;
  k.amp_pref_j = (float)(kj / kTwoPi);
  k.taper_inv = a.taper ? (float)(1.0 / (2.0 * a.taper_s * a.taper_s)) : 0.f;
  k.sigma = (float)a.sigma;
  k.corr = (float)a.corr;
  k.fadL = (float)a.fad.L;
  k.n_exp = (float)a.n_exp;
  const df k2 = df_from_double(2.0 * a.k0);
  k.K2h = k2.hi;
  k.K2l = k2.lo;
  const df A = df_from_double(2.0 / (a.c * a.dt));
  const df B = df_from_double(a.t0 / a.dt);
  k.Ah = A.hi;
  k.Al = A.lo;
  k.Bh = B.hi;
  k.Bl = B.lo;
  // a sequential chain through two or more interfaces is not stationary
  // in its upper crossings, whose float32 in-plane error then reaches the
  // optical path at first order: a wider band there. Joint paths and
  // single crossings agree with the float64 path to ~1e-9 m.
  const double og = (!a.joint && a.ni > 1) ? kOplGuardChain : 0.0;
  k.bin_guard = (float)std::max((double)kBinGuard, og * 2.0 / (a.c * a.dt));
  for (int i = 0; i <= a.leg_last; ++i) {
    const df n = df_from_double(a.n_leg[i]);
    k.n_leg[i] = n.hi;
    k.n_leg_lo[i] = n.lo;
    k.eps_leg[i] = (float)a.eps_leg[i];
    k.att_leg[i] = (float)a.att_leg[i];
  }
  for (int i = 0; i < a.ni; ++i) {
    const ss_interface &I = a.ifc[i];
    MeanPlane32 &M = k.mean[i];
    k.sig_c[i] = (float)a.sig_c[i];
    for (int j = 0; j < 3; ++j) {
      M.mp[j] = (float)I.mean_point[j];
      M.mn[j] = (float)I.mean_normal[j];
      M.dmp[j] = i == 0 ? 0.0f
                        : (float)(a.ifc[i - 1].mean_point[j] - I.mean_point[j]);
    }
    for (int c = 0; c < 4; ++c) {
      const df cd = df_from_double(I.coef[c]);
      M.coef[c] = cd.hi;
      M.coefl[c] = cd.lo;
    }
    for (int c = 0; c < 2; ++c) {
      const double rbv = (double)M.mp[0] * I.coef[c] +
                         (double)M.mp[1] * I.coef[2 + c] + I.coef[4 + c];
      const df r = df_from_double(rbv);
      M.rb[c] = r.hi;
      M.rbl[c] = r.lo;
    }
  }
  return k;
}

// Dynamic shared memory of the fast kernel: the trace block's histograms
// and the series table.
size_t split_smem_bytes(const RefArgs &a, int tb) {
  return (size_t)tb * a.n_seg * sizeof(float2) +
         (a.rough_kind ? (a.n_terms + 1) * sizeof(float) : 0);
}

int refracted_split_launch(RefArgs &a, const Plan &p, cudaStream_t st) {
  int pa_len, pb_len;
  pattern_lengths(a.pat_kind, a.pat_n, pa_len, pb_len);
  if (pa_len + pb_len > SS_PAT_MAX) {
    set_error("antenna table too large for the split kernel");
    return SS_ERR_UNSUPPORTED;
  }
  const RefSplitConsts k = split_consts(a);
  const size_t smem = split_smem_bytes(a, p.tb);
  if (!a.joint) return split_launch_ni0(a, k, p, smem, st);
  switch (a.ni) {
    case 1: return split_launch_ni1(a, k, p, smem, st);
    case 2: return split_launch_ni2(a, k, p, smem, st);
    case 3: return split_launch_ni3(a, k, p, smem, st);
    case 4: return split_launch_ni4(a, k, p, smem, st);
    default: return split_launch_deep(a, k, p, smem, st);
  }
}

}  // namespace ss
