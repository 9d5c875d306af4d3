// Adjoint of the split refracted kernel: device code and launch templates,
// instantiated for the sequential chain in ss_refracted_adjoint.cu and for
// the joint solve in ss_refracted_adjoint_joint12.cu / _joint34.cu.
#pragma once

#include <algorithm>

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
// forward's lookup and bin decisions: the fast pass holds no float64 code
// and marks the pairs that need a float64 decision (bit t * N + i of the
// caller's scratch); the fix-up pass evaluates those with EXACT and adds
// their terms. Thread <-> facet, loop over all traces (staged in shared
// memory in blocks), so each facet's gradient is summed by one thread in
// trace order; the attenuation-rate gradient is reduced per CTA.
constexpr int kAdjThreads = 128, kAdjTB = 32;
constexpr double kLn10 = 2.302585092994045684;

int refracted_adjoint_blocks(int N);

// One pair's terms of the three gradients (before the ln10 factors).
template <int NI, int ROUGH, bool EXACT>
__device__ __forceinline__ bool adjoint_pair(
    const RefArgs &a, const RefSplitConsts &k, const AdjArgs &j,
    const TraceS &T, const double *p64, const float *u, const float *pv,
    const float *pat, int pa_len, const float *lg, const float *fad, int t,
    int i, const float *q, double g, double &gR, double &gS, double &gA) {
  PairOut o;
  PairGrad pg;
  if (!pair_eval<NI, ROUGH, EXACT, true>(a, k, T, p64, u, pv, pat, pa_len, lg,
                                        fad, i, q, o, &pg))
    return false;
  if (o.bin < j.bin_lo || o.bin >= j.bin_hi) return true;
  const double2 f =
      reinterpret_cast<const double2 *>(j.field)[(size_t)t * a.n_seg + o.bin];
  gR += g * (f.x * pg.gre + f.y * pg.gim);
  gS += g * (f.x * pg.sre + f.y * pg.sim);
  gA += g * (f.x * o.re + f.y * o.im) * (double)pg.dloss;
  return true;
}

template <int ROUGH>
__device__ __forceinline__ void adjoint_stage_tables(const RefArgs &a,
                                                     float *s_pat,
                                                     float *s_fad, float *lg,
                                                     int &pa_len) {
  const int tid = threadIdx.x;
  int pb_len;
  pattern_lengths(a.pat_kind, a.pat_n, pa_len, pb_len);
  for (int m = tid; m < pa_len; m += blockDim.x) s_pat[m] = (float)a.pa[m];
  for (int m = tid; m < pb_len; m += blockDim.x)
    s_pat[pa_len + m] = (float)a.pb[m];
  if (ROUGH == SS_ROUGH_GAUSS_FULL && tid < SS_FAD_N)
    s_fad[tid] = (float)a.fad.a[tid];
  if (ROUGH != SS_ROUGH_NONE) fill_inv_table(lg, a.n_terms, tid, blockDim.x);
}

// The sequential chain fits 80 registers without spills: six 128-thread
// CTAs per SM (24 warps) hide this latency-bound kernel's dependent chains
// better than the 152 registers the compiler takes unasked. The joint
// solves keep their registers (they spill heavily at 80).
//
// Grid: x = facet blocks (thread <-> facet), y = parts of the trace range.
// With one part a CTA writes its facets' sums and its alpha partial; with
// several (chosen so the grid fills whole waves) each part adds them to
// outputs the launch has zeroed.
template <int NI, int ROUGH>
__global__ void __launch_bounds__(kAdjThreads, NI == 0 ? 6 : 1)
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
  int pa_len;
  adjoint_stage_tables<ROUGH>(a, s_pat, s_fad, lg, pa_len);
  float q[3] = {0.0f, 0.0f, 0.0f};
  if (i < a.N) {
    q[0] = a.F.cx[i];
    q[1] = a.F.cy[i];
    q[2] = a.F.cz[i];
  }
  const int parts = gridDim.y;
  const int t_begin = (int)((long)a.T * blockIdx.y / parts);
  const int t_end = (int)((long)a.T * (blockIdx.y + 1) / parts);
  double gR = 0.0, gS = 0.0, gA = 0.0;
  for (int t0 = t_begin; t0 < t_end; t0 += kAdjTB) {
    const int nt = min(kAdjTB, t_end - t0);
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
      if (!adjoint_pair<NI, ROUGH, false>(a, k, j, s_tr[tt], s_p64[tt], s_u[tt],
                                      s_pv[tt], s_pat, pa_len, lg, s_fad,
                                      t0 + tt, i, q, s_g[tt], gR, gS, gA)) {
        const unsigned long long bit =
            (unsigned long long)(t0 + tt) * a.N + i;
        atomicOr(&j.defer_mask[bit >> 5], 1u << (bit & 31));
      }
    }
  }
  // d c / d gamma_dB = c ln(10) / 20; d c / d alpha = -c ln(10) / 10 dloss
  if (i < a.N) {
    if (parts == 1) {
      j.grad_gamma_db[i] = gR * (kLn10 / 20.0);
      if (j.grad_sigma) j.grad_sigma[i] = gS;
    } else {
      atomicAdd(&j.grad_gamma_db[i], gR * (kLn10 / 20.0));
      if (j.grad_sigma) atomicAdd(&j.grad_sigma[i], gS);
    }
  }
  gA *= -kLn10 / 10.0;
  for (int d = 16; d > 0; d >>= 1) gA += __shfl_down_sync(0xffffffffu, gA, d);
  if ((tid & 31) == 0) s_red[tid >> 5] = gA;
  __syncthreads();
  if (tid == 0) {
    double s = 0.0;
    for (int w = 0; w < kAdjThreads / 32; ++w) s += s_red[w];
    if (parts == 1)
      j.grad_alpha[blockIdx.x] = s;
    else
      atomicAdd(&j.grad_alpha[blockIdx.x], s);
  }
}

// Fix-up: the deferred pairs with the float64 decisions, added atomically
// (the fast pass has written every facet's sum). Warp-queued over the
// bitmask like the forward fix-up.
template <int NI, int ROUGH>
__global__ void __launch_bounds__(32 * kFixWarps)
refracted_adjoint_fixup(RefArgs a, RefSplitConsts k, AdjArgs j) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float *lg = reinterpret_cast<float *>(smem_raw);
  __shared__ float s_pat[SS_PAT_MAX];
  __shared__ float s_fad[SS_FAD_N];
  __shared__ unsigned long long s_q[kFixWarps][kFixQueue];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int pa_len;
  adjoint_stage_tables<ROUGH>(a, s_pat, s_fad, lg, pa_len);
  __syncthreads();
  const unsigned long long n_words =
      ((unsigned long long)a.T * a.N + 31) >> 5;
  const unsigned long long n_warps =
      (unsigned long long)gridDim.x * kFixWarps;
  unsigned long long *qv = s_q[warp];
  auto eval = [&](unsigned long long bit) {
    const int t = (int)(bit / a.N), i = (int)(bit % a.N);
    TraceS T;
    double p64[3];
    float u[3], pv[6];
    load_trace(a, t, T, p64, u, pv);
    const float q[3] = {a.F.cx[i], a.F.cy[i], a.F.cz[i]};
    double gR = 0.0, gS = 0.0, gA = 0.0;
    adjoint_pair<NI, ROUGH, true>(a, k, j, T, p64, u, pv, s_pat, pa_len, lg,
                              s_fad, t, i, q, 2.0 * j.grad_power[t], gR, gS,
                              gA);
    if (gR != 0.0) atomicAdd(&j.grad_gamma_db[i], gR * (kLn10 / 20.0));
    if (gS != 0.0 && j.grad_sigma) atomicAdd(&j.grad_sigma[i], gS);
    if (gA != 0.0) atomicAdd(&j.grad_alpha[0], gA * (-kLn10 / 10.0));
  };
  int qn = 0;
  for (unsigned long long base =
           ((unsigned long long)blockIdx.x * kFixWarps + warp) * 32;
       base < n_words; base += n_warps * 32) {
    const unsigned long long w = base + lane;
    unsigned int m = w < n_words ? j.defer_mask[w] : 0u;
    const int c = __popc(m);
    int incl = c;
    for (int d = 1; d < 32; d <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= d) incl += v;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    int pos = qn + incl - c;
    while (m) {
      const int b = __ffs(m) - 1;
      m &= m - 1;
      qv[pos++] = (w << 5) + b;
    }
    __syncwarp();
    qn += total;
    while (qn >= 32) {
      const unsigned long long bit = qv[qn - 32 + lane];
      __syncwarp();
      eval(bit);
      qn -= 32;
    }
    __syncwarp();
  }
  if (lane < qn) eval(qv[lane]);
}

template <int NI, int ROUGH>
inline int adjoint_launch_r(RefArgs &a, const RefSplitConsts &k,
                            const AdjArgs &j, size_t smem, cudaStream_t st) {
  const int blocks = refracted_adjoint_blocks(a.N);
  // trace parts: the count (up to 8) whose grid fills whole waves of the
  // resident CTAs best, for grids under eight waves (a last wave a quarter
  // full costs a full one); the fewest parts on a tie
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(
          &per_sm, refracted_adjoint_kernel<NI, ROUGH>, kAdjThreads, smem) !=
          cudaSuccess ||
      per_sm < 1)
    per_sm = 1;
  const long slots = (long)per_sm * sm_count();
  int parts = 1;
  if ((long)blocks < 8 * slots) {
    double best = -1.0;
    for (int pp = 1; pp <= 8 && pp <= a.T; ++pp) {
      const long items = (long)blocks * pp;
      const long waves = (items + slots - 1) / slots;
      const double eff = (double)items / (double)(waves * slots);
      if (eff > best + 1e-9) {
        best = eff;
        parts = pp;
      }
    }
  }
  cudaError_t e;
  if (parts > 1) {
    e = cudaMemsetAsync(j.grad_gamma_db, 0, (size_t)a.N * sizeof(double), st);
    if (e == cudaSuccess && j.grad_sigma)
      e = cudaMemsetAsync(j.grad_sigma, 0, (size_t)a.N * sizeof(double), st);
    if (e == cudaSuccess)
      e = cudaMemsetAsync(j.grad_alpha, 0, (size_t)blocks * sizeof(double),
                          st);
    if (e != cudaSuccess) return cuda_status(e, "adjoint output clear");
  }
  refracted_adjoint_kernel<NI, ROUGH>
      <<<dim3(blocks, parts), kAdjThreads, smem, st>>>(a, k, j);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_status(e, "refracted adjoint launch");
  const unsigned long long n_words =
      ((unsigned long long)a.T * a.N + 31) >> 5;
  const unsigned long long want =
      (n_words + 32 * kFixWarps - 1) / (32 * kFixWarps);
  const int fb = (int)std::max<unsigned long long>(
      1, std::min<unsigned long long>(want, 8ull * sm_count()));
  refracted_adjoint_fixup<NI, ROUGH><<<fb, 32 * kFixWarps, smem, st>>>(a, k, j);
  return cuda_status(cudaGetLastError(), "refracted adjoint fix-up launch");
}

// The four roughness kinds of one path (NI = 0: the sequential chain; NI =
// 1..4: the joint solve through that many interfaces).
template <int NI>
inline int adjoint_launch_ni(RefArgs &a, const RefSplitConsts &k,
                             const AdjArgs &j, size_t smem, cudaStream_t st) {
  switch (a.rough_kind) {
    case SS_ROUGH_NONE:
      return adjoint_launch_r<NI, SS_ROUGH_NONE>(a, k, j, smem, st);
    case SS_ROUGH_GAUSS_FULL:
      return adjoint_launch_r<NI, SS_ROUGH_GAUSS_FULL>(a, k, j, smem, st);
    case SS_ROUGH_GAUSS_AREA:
      return adjoint_launch_r<NI, SS_ROUGH_GAUSS_AREA>(a, k, j, smem, st);
    default:
      return adjoint_launch_r<NI, SS_ROUGH_EXP_AREA>(a, k, j, smem, st);
  }
}

// Joint-path adjoint launches through 1-2 and 3-4 interfaces
// (ss_refracted_adjoint_joint12.cu, ss_refracted_adjoint_joint34.cu).
int adjoint_launch_joint12(RefArgs &a, const RefSplitConsts &k,
                           const AdjArgs &j, size_t smem, cudaStream_t st);
int adjoint_launch_joint34(RefArgs &a, const RefSplitConsts &k,
                           const AdjArgs &j, size_t smem, cudaStream_t st);

}  // namespace ss
