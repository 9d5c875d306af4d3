// Adjoint of the split refracted kernel (sequential path).
#include "ss_refracted_split.cuh"

namespace ss {

// ---------------------------------------------------------------------
// adjoint: gradients of windowed trace power
// ---------------------------------------------------------------------
// For P_t = sum_{b in [bin_lo, bin_hi)} |F_t[b]|^2 of one target's field F
// and an upstream gradient g_t = dL/dP_t, a parameter theta of facet i gets
//   dL/dtheta = sum_t g_t 2 Re(conj(F_t[b_ti]) dc_ti/dtheta)
// over the pairs whose bin lies in the window (bins and paths do not depend
// on reflectivity, roughness or attenuation). Each pair's contribution c_ti
// is recomputed from the geometry -- no per-pair state is stored -- with the
// float64 lookup and bin decisions (EXACT), so the adjoint sees exactly the
// forward's pairs. Thread <-> facet, loop over all traces (staged in shared
// memory in blocks), so each facet's gradient is summed by one thread in
// trace order; the attenuation-rate gradient is reduced per CTA.
constexpr int kAdjThreads = 128, kAdjTB = 32;


template <int ROUGH>
__global__ void __launch_bounds__(kAdjThreads)
refracted_adjoint_kernel(RefArgs a, RefSplitConsts k, AdjArgs j) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float *lg = reinterpret_cast<float *>(smem_raw);
  __shared__ double s_p64[kAdjTB][3];
  __shared__ TraceS s_tr[kAdjTB];
  __shared__ float s_u[kAdjTB][3], s_pv[kAdjTB][6];
  __shared__ int s_lo[kAdjTB], s_hi[kAdjTB];
  __shared__ double s_g[kAdjTB];
  __shared__ float s_pat[SS_PAT_MAX];
  __shared__ float s_fad[SS_FAD_N];
  __shared__ double s_red[kAdjThreads / 32];
  const int tid = threadIdx.x;
  const int i = blockIdx.x * kAdjThreads + tid;
  const int i_first = blockIdx.x * kAdjThreads;
  const int i_last = min(i_first + kAdjThreads, a.N) - 1;
  int pa_len, pb_len;
  pattern_lengths(a.pat_kind, a.pat_n, pa_len, pb_len);
  for (int m = tid; m < pa_len; m += blockDim.x) s_pat[m] = (float)a.pa[m];
  for (int m = tid; m < pb_len; m += blockDim.x)
    s_pat[pa_len + m] = (float)a.pb[m];
  if (ROUGH == SS_ROUGH_GAUSS_FULL && tid < SS_FAD_N)
    s_fad[tid] = (float)a.fad.a[tid];
  if (ROUGH != SS_ROUGH_NONE)
    for (int m = tid; m <= a.n_terms; m += blockDim.x)
      lg[m] = (float)lgamma((double)m + 1.0);
  float q[3] = {0.0f, 0.0f, 0.0f};
  if (i < a.N) {
    q[0] = a.F.cx[i];
    q[1] = a.F.cy[i];
    q[2] = a.F.cz[i];
  }
  double gR = 0.0, gS = 0.0, gA = 0.0;
  const double2 *F = reinterpret_cast<const double2 *>(j.field);
  for (int t0 = 0; t0 < a.T; t0 += kAdjTB) {
    const int nt = min(kAdjTB, a.T - t0);
    __syncthreads();
    if (tid < nt) {
      const int t = t0 + tid;
      load_trace(a, t, s_tr[tid], s_p64[tid], s_u[tid], s_pv[tid]);
      const long lo = (long)a.off[t] * a.bs;
      const long hi = min((long)(a.off[t] + a.n_win) * a.bs, (long)a.N);
      s_lo[tid] = (int)min(lo, (long)a.N);
      s_hi[tid] = (int)hi;
      s_g[tid] = 2.0 * j.grad_power[t];
    }
    __syncthreads();
    for (int tt = 0; tt < nt; ++tt) {
      // CTA-uniform skip of traces whose window misses the CTA's facets
      if (s_hi[tt] <= i_first || s_lo[tt] > i_last || s_g[tt] == 0.0)
        continue;
      if (i >= a.N || i < s_lo[tt] || i >= s_hi[tt]) continue;
      PairOut o;
      PairGrad pg;
      pair_eval<0, ROUGH, true, true>(a, k, s_tr[tt], s_p64[tt], s_u[tt],
                                      s_pv[tt], s_pat, pa_len, lg, s_fad, i,
                                      q, o, &pg);
      if (o.bin < j.bin_lo || o.bin >= j.bin_hi) continue;
      const double2 f = F[(size_t)(t0 + tt) * a.n_seg + o.bin];
      const double g = s_g[tt];
      gR += g * (f.x * pg.gre + f.y * pg.gim);
      gS += g * (f.x * pg.sre + f.y * pg.sim);
      gA += g * (f.x * o.re + f.y * o.im) * (double)pg.dloss;
    }
  }
  // d c / d gamma_dB = c ln(10) / 20; d c / d alpha = -c ln(10) / 10 dloss
  const double ln10 = 2.302585092994045684;
  if (i < a.N) {
    j.grad_gamma_db[i] = gR * (ln10 / 20.0);
    if (j.grad_sigma) j.grad_sigma[i] = gS;
  }
  gA *= -ln10 / 10.0;
  for (int d = 16; d > 0; d >>= 1) gA += __shfl_down_sync(0xffffffffu, gA, d);
  if ((tid & 31) == 0) s_red[tid >> 5] = gA;
  __syncthreads();
  if (tid == 0) {
    double s = 0.0;
    for (int w = 0; w < kAdjThreads / 32; ++w) s += s_red[w];
    j.grad_alpha[blockIdx.x] = s;
  }
}

int refracted_adjoint_blocks(int N) {
  return (N + kAdjThreads - 1) / kAdjThreads;
}

int refracted_adjoint_launch(RefArgs &a, const AdjArgs &j,
                             const double *alpha_mask, cudaStream_t st) {
  int pa_len, pb_len;
  pattern_lengths(a.pat_kind, a.pat_n, pa_len, pb_len);
  if (pa_len + pb_len > SS_PAT_MAX) {
    set_error("antenna table too large for the split kernel");
    return SS_ERR_UNSUPPORTED;
  }
  if (a.joint) {
    set_error("the adjoint follows the sequential path only");
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
  const int blocks = refracted_adjoint_blocks(a.N);
  switch (a.rough_kind) {
    case SS_ROUGH_NONE:
      refracted_adjoint_kernel<SS_ROUGH_NONE>
          <<<blocks, kAdjThreads, smem, st>>>(a, k, j);
      break;
    case SS_ROUGH_GAUSS_FULL:
      refracted_adjoint_kernel<SS_ROUGH_GAUSS_FULL>
          <<<blocks, kAdjThreads, smem, st>>>(a, k, j);
      break;
    case SS_ROUGH_GAUSS_AREA:
      refracted_adjoint_kernel<SS_ROUGH_GAUSS_AREA>
          <<<blocks, kAdjThreads, smem, st>>>(a, k, j);
      break;
    default:
      refracted_adjoint_kernel<SS_ROUGH_EXP_AREA>
          <<<blocks, kAdjThreads, smem, st>>>(a, k, j);
      break;
  }
  return cuda_status(cudaGetLastError(), "refracted adjoint launch");
}

}  // namespace ss
