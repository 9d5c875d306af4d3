// Split-precision surface coherent kernel.
//
// Same decomposition as the FP64 form (ss_coherent.cu). Per pair, only three
// quantities need more than float32:
//   * the slant range r (20 km at 1 mm f32 ulp; 1e-3 rad at 450 MHz needs
//     ~50 um): carried as double-float from a double-float platform position
//     and the float32 facet centroid (exact), one rsqrt + Newton correction;
//   * the carrier phase 2 k r: a double-float product reduced modulo 2 pi
//     with a two-constant Cody-Waite step (exact first step by construction),
//     then MUFU sin/cos on an argument in [-pi, pi];
//   * the fast-time bin floor((2r/c - t0)/dt): evaluated from the
//     double-float range; a pair whose fractional bin position lies within
//     1e-6 of an edge is re-binned with the float64 round-to-nearest chain of
//     the oracle, so bins are bit-identical to the float64 form.
// Everything else (incidence, sincs, taper, antenna gain, roughness series)
// runs in float32; histograms accumulate float32 per CTA chunk and chunks are
// summed in float64 by the reduce kernel.
#include <algorithm>

#include "ss_coherent.cuh"
#include "ss_df.cuh"
#include "ss_f32.cuh"

namespace ss {

// (dh + dl) . e for a double-float vector d and float e: exact products
// (two_prod), compensated sum, rounded once to float.
__device__ __forceinline__ float dot_df(float xh, float xl, float yh, float yl,
                                        float zh, float zl, float ex, float ey,
                                        float ez) {
  float px, qx, py, qy, pz, qz, s, e1, e2;
  two_prod(xh, ex, px, qx);
  two_prod(yh, ey, py, qy);
  two_prod(zh, ez, pz, qz);
  two_sum(px, py, s, e1);
  two_sum(s, pz, s, e2);
  const float lo = (e1 + e2) + (qx + qy + qz) +
                   __fmaf_rn(xl, ex, __fmaf_rn(yl, ey, zl * ez));
  return s + lo;
}


// One CTA's work item: facet chunk `chunk` of trace block `group`. Shared
// by the one-call kernel (item = block index) and the batched persistent
// kernel (item pulled from a work queue).
template <int ROUGH>
__device__ __forceinline__ void coherent_split_cta(const CoArgs &a,
                                                   const SplitConsts &k,
                                                   int chunk, int group,
                                                   unsigned char *smem_raw) {
  float2 *hist = reinterpret_cast<float2 *>(smem_raw);
  float *lg = reinterpret_cast<float *>(hist + (size_t)a.tb * a.n_seg);
  __shared__ float s_ph[SS_MAX_TB][3], s_pl[SS_MAX_TB][3];
  __shared__ double s_p64[SS_MAX_TB][3];
  __shared__ float s_u[SS_MAX_TB][3];
  __shared__ float s_pv[SS_MAX_TB][6];
  __shared__ int s_lo[SS_MAX_TB], s_hi[SS_MAX_TB];
  __shared__ float s_drop[SS_MAX_TB];
  __shared__ float s_pat[SS_PAT_MAX];
  __shared__ float s_fad[SS_FAD_N];
  __shared__ int s_rng[2];
  __shared__ int s_next;

  const int t_base = group * a.tb;
  const int nt = min(a.tb, a.T - t_base);
  const int tid = threadIdx.x;
  int pa_len, pb_len;
  pattern_lengths(a.pat_kind, a.pat_n, pa_len, pb_len);

  if (tid < nt) {
    const int t = t_base + tid;
    for (int j = 0; j < 3; ++j) {
      const double pj = a.pos[3 * t + j];
      const df v = df_from_double(pj);
      s_ph[tid][j] = v.hi;
      s_pl[tid][j] = v.lo;
      s_p64[tid][j] = pj;
      s_u[tid][j] = a.uct ? (float)a.uct[3 * t + j] : 0.0f;
    }
    for (int j = 0; j < 6; ++j)
      s_pv[tid][j] =
          (a.pv && j < a.pv_len) ? (float)a.pv[a.pv_len * t + j] : 0.0f;
    long lo = (long)a.off[t] * a.bs;
    long hi = min((long)(a.off[t] + a.n_win) * a.bs, (long)a.N);
    s_lo[tid] = (int)min(lo, (long)a.N);
    s_hi[tid] = (int)hi;
    s_drop[tid] = 0.0f;
  }
  for (int j = tid; j < pa_len; j += blockDim.x) s_pat[j] = (float)a.pa[j];
  for (int j = tid; j < pb_len; j += blockDim.x)
    s_pat[pa_len + j] = (float)a.pb[j];
  if (ROUGH == SS_ROUGH_GAUSS_FULL && tid < SS_FAD_N)
    s_fad[tid] = (float)a.fad.a[tid];
  for (int j = tid; j < a.tb * a.n_seg; j += blockDim.x)
    hist[j] = make_float2(0.0f, 0.0f);
  if (ROUGH != SS_ROUGH_NONE)
    for (int m = tid; m <= a.n_terms; m += blockDim.x)
      lg[m] = (float)lgamma((double)m + 1.0);
  __syncthreads();
  if (tid == 0) {
    int lo = s_lo[0], hi = s_hi[0];
    for (int j = 1; j < nt; ++j) {
      lo = min(lo, s_lo[j]);
      hi = max(hi, s_hi[j]);
    }
    long len = max(hi - lo, 0);
    s_rng[0] = lo + (int)(len * chunk / a.n_chunks);
    s_rng[1] = lo + (int)(len * (chunk + 1) / a.n_chunks);
    s_next = s_rng[0];
  }
  __syncthreads();

  const float nsf = (float)a.n_samples;
  // lane l meets the block's traces starting at trace l mod nt, so the 32
  // neighbouring facets of a warp -- often in one bin -- spread their
  // histogram atomics over the block's traces; dropped power collects per
  // thread and trace and reaches shared memory once per trace at the end
  const int rot = (tid & 31) % max(nt, 1);
  float dropl[SS_MAX_TB];
#pragma unroll
  for (int j = 0; j < SS_MAX_TB; ++j) dropl[j] = 0.0f;
  // warps take 32 consecutive facets at a time from a shared counter (the
  // roughness series makes pair costs uneven)
  const int lane = tid & 31;
  const int i_end = s_rng[1];
  for (;;) {
    int base = 0;
    if (lane == 0) base = atomicAdd(&s_next, 32);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= i_end) break;
    const int i = base + lane;
    if (i >= i_end) continue;
    const float cx = a.F.cx[i], cy = a.F.cy[i], cz = a.F.cz[i];
    const float nx = a.F.nx[i], ny = a.F.ny[i], nz = a.F.nz[i];
    const float e1x = a.F.e1x[i], e1y = a.F.e1y[i], e1z = a.F.e1z[i];
    const float e2x = a.F.e2x[i], e2y = a.F.e2y[i], e2z = a.F.e2z[i];
    const float area = a.F.area[i];
    const float gam = a.F.gamma_f32 ? a.F.gamma_f32[i] : k.gamma;
    float sg = 0.f, lc = 0.f, phr = 0.f, phi = 0.f, l1 = 0.f, l2 = 0.f;
    if (ROUGH != SS_ROUGH_NONE) {
      sg = a.F.sigma ? a.F.sigma[i] : k.sigma;
      lc = a.F.corr ? a.F.corr[i] : k.corr;
      phr = a.F.phasor[2 * i];
      phi = a.F.phasor[2 * i + 1];
      l1 = sqrtf(dot3f(e1x, e1y, e1z, e1x, e1y, e1z));
      l2 = sqrtf(dot3f(e2x, e2y, e2z, e2x, e2y, e2z));
    }
    for (int st = 0; st < nt; ++st) {
      const int tt = rot + st < nt ? rot + st : rot + st - nt;
      if (i < s_lo[tt] || i >= s_hi[tt]) continue;
      // --- d = p - c as double-float per component ---
      float dxh, dxl, dyh, dyl, dzh, dzl, e;
      two_sum(s_ph[tt][0], -cx, dxh, e);
      fast_two_sum(dxh, e + s_pl[tt][0], dxh, dxl);
      two_sum(s_ph[tt][1], -cy, dyh, e);
      fast_two_sum(dyh, e + s_pl[tt][1], dyh, dyl);
      two_sum(s_ph[tt][2], -cz, dzh, e);
      fast_two_sum(dzh, e + s_pl[tt][2], dzh, dzl);
      // --- S = |d|^2 (double-float) ---
      float qx, ex, qy, ey, qz, ez;
      two_prod(dxh, dxh, qx, ex);
      two_prod(dyh, dyh, qy, ey);
      two_prod(dzh, dzh, qz, ez);
      float s1_, e1_, Sh, e2_;
      two_sum(qx, qy, s1_, e1_);
      two_sum(s1_, qz, Sh, e2_);
      float Sl = (e1_ + e2_) + (ex + ey + ez) +
                 2.0f * (dxh * dxl + dyh * dyl + dzh * dzl);
      fast_two_sum(Sh, Sl, Sh, Sl);
      // --- r = sqrt(S): rsqrt + one Newton correction ---
      const float y = rsqrtf(Sh);
      const float r0 = Sh * y;
      const float res = __fmaf_rn(-r0, r0, Sh) + Sl;
      float rh, rl;
      fast_two_sum(r0, res * (0.5f * y), rh, rl);
      const float inv_r = y;
      // --- amplitude (float32) ---
      const float rx = dxh * inv_r, ry = dyh * inv_r, rz = dzh * inv_r;
      const float cosv = dot3f(rx, ry, rz, nx, ny, nz);
      // r_hat . e: the sinc argument k (r_hat . e) reaches tens of radians,
      // and its products cancel to ~1e-2 of their size near nadir, so the
      // dot product is formed error-free (two_prod) from the double-float d
      const float d1 = dot_df(dxh, dxl, dyh, dyl, dzh, dzl, e1x, e1y, e1z) *
                       inv_r;
      const float d2 = dot_df(dxh, dxl, dyh, dyl, dzh, dzl, e2x, e2y, e2z) *
                       inv_r;
      const float inv_r2 = inv_r * inv_r;
      float amp = k.amp_pref * gam * cosv * area * sinc32(k.k * d1) *
                  sinc32(k.k * d2) * inv_r2;
      if (a.taper) {
        float cc = fminf(fmaxf(cosv, 1e-9f), 1.0f);
        float c2 = cc * cc;
        amp *= __expf(-__fdividef(1.0f - c2, c2) * k.taper_inv);
      }
      float cr = amp, ci = 0.0f;
      if (ROUGH != SS_ROUGH_NONE) {
        const float kk = 2.0f * k.k * cosv;
        const float dp = d_phi32<ROUGH>(a.n_terms, lg, s_fad, k.fadL, sg, lc,
                                        kk, 2.0f * k.k * d1 / l1,
                                        2.0f * k.k * d2 / l2, l1, l2);
        const float amp_i =
            area > 0.0f ? k.amp_pref * gam * cosv * inv_r2 * sqrtf(dp) : 0.0f;
        const float sk = sg * kk;
        const float att = __expf(-0.5f * sk * sk);
        cr = amp * att + amp_i * phr;
        ci = amp_i * phi;
      }
      // --- carrier phase 2 k r mod 2 pi (double-float) ---
      float ph, pe;
      two_prod(k.K2h, rh, ph, pe);
      const float pl = pe + __fmaf_rn(k.K2h, rl, k.K2l * rh);
      const float n2 = rintf(ph * 0.159154943091895336f);
      float red = __fmaf_rn(-n2, 6.28318548202514648f, ph);  // exact
      red = __fmaf_rn(-n2, -1.74845553146951e-07f, red) + pl;
      float sn, cs;
      __sincosf(red, &sn, &cs);
      float re = cr * sn - ci * cs;
      float im = cr * cs + ci * sn;
      if (a.pat_kind != SS_PAT_ISOTROPIC) {
        const float g = gain32(a.pat_kind, a.pat_n, pa_len, s_pat, s_pv[tt],
                               -rx, -ry, -rz);
        re *= g * g;
        im *= g * g;
      }
      // --- bin: u = r A - B (double-float), exact re-bin near edges ---
      float up, ue, us, ue2;
      two_prod(rh, k.Ah, up, ue);
      two_sum(up, -k.Bh, us, ue2);
      const float ul = (ue2 + ue) + __fmaf_rn(rh, k.Al, rl * k.Ah) - k.Bl;
      float fb = floorf(us);
      float frac = (us - fb) + ul;
      if (frac < 0.0f) { fb -= 1.0f; frac += 1.0f; }
      else if (frac >= 1.0f) { fb += 1.0f; frac -= 1.0f; }
      if ((frac < 1e-6f || frac > 0.999999f) && us > -4.0f &&
          us < nsf + 4.0f) {
        // float64 round-to-nearest chain, identical to the oracle
        const double ddx = __dsub_rn(s_p64[tt][0], (double)cx);
        const double ddy = __dsub_rn(s_p64[tt][1], (double)cy);
        const double ddz = __dsub_rn(s_p64[tt][2], (double)cz);
        const double rr = __dsqrt_rn(__dadd_rn(
            __dadd_rn(__dmul_rn(ddx, ddx), __dmul_rn(ddy, ddy)),
            __dmul_rn(ddz, ddz)));
        const double u64 = __ddiv_rn(
            __dsub_rn(__ddiv_rn(__dmul_rn(2.0, rr), a.c), a.t0), a.dt);
        const double f64b = floor(u64);
        fb = (float)f64b;
        frac = (float)(u64 - f64b);
      }
      int side_off = 0;
      if (a.split &&
          dot3f(-dxh, -dyh, -dzh, s_u[tt][0], s_u[tt][1], s_u[tt][2]) > 0.0f)
        side_off = a.n_samples;
      float2 *h = hist + (size_t)tt * a.n_seg + side_off;
      if (a.interp) {
        const float wq[2] = {1.0f - frac, frac};
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          const float bq = fb + (float)q;
          const float pr = re * wq[q], pim = im * wq[q];
          if (bq >= 0.0f && bq < nsf) {
            atomicAdd(&h[(int)bq].x, pr);
            atomicAdd(&h[(int)bq].y, pim);
          } else {
            dropl[tt] += pr * pr + pim * pim;
          }
        }
      } else if (fb >= 0.0f && fb < nsf) {
        atomicAdd(&h[(int)fb].x, re);
        atomicAdd(&h[(int)fb].y, im);
      } else {
        dropl[tt] += re * re + im * im;
      }
    }
  }
  for (int tt = 0; tt < nt; ++tt)
    if (dropl[tt] != 0.0f) atomicAdd(&s_drop[tt], dropl[tt]);
  __syncthreads();
  float2 *part = reinterpret_cast<float2 *>(a.part);
  for (int tt = 0; tt < nt; ++tt) {
    const size_t base = ((size_t)chunk * a.T + t_base + tt) * a.n_seg;
    for (int j = tid; j < a.n_seg; j += blockDim.x)
      part[base + j] = hist[(size_t)tt * a.n_seg + j];
  }
  if (tid < nt)
    a.part_drop[(size_t)chunk * a.T + t_base + tid] = (double)s_drop[tid];
}

template <int ROUGH>
__global__ void __launch_bounds__(256)
coherent_split_kernel(CoArgs a, SplitConsts k) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  coherent_split_cta<ROUGH>(a, k, blockIdx.x, blockIdx.y, smem_raw);
}

// Batched persistent kernel: CTAs pull (job, trace block, facet chunk)
// items from a global counter until the queue is empty, so jobs of very
// different sizes share one launch without tail effects.
template <int ROUGH>
__global__ void __launch_bounds__(256)
coherent_batch_split_kernel(const BatchJob *jobs, int n_jobs,
                            long long n_items, unsigned long long *counter) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ long long s_item;
  __shared__ int s_job;
  for (;;) {
    __syncthreads();  // the previous item's shared memory is free
    if (threadIdx.x == 0) {
      const long long it = (long long)atomicAdd(counter, 1ull);
      s_item = it;
      s_job = it < n_items ? batch_find_job(jobs, n_jobs, it, true) : 0;
    }
    __syncthreads();
    const long long it = s_item;
    if (it >= n_items) break;
    const BatchJob &J = jobs[s_job];
    const long long local = it - J.item0;
    coherent_split_cta<ROUGH>(J.a, J.k, (int)(local % J.n_chunks),
                              (int)(local / J.n_chunks), smem_raw);
  }
}

template <int ROUGH>
static int batch_split_launch_r(const BatchJob *jobs, int n_jobs,
                                long long n_items,
                                unsigned long long *counter, int threads,
                                int ctas, size_t smem, cudaStream_t st) {
  // the dynamic shared-memory limit was raised at prepare time, so this
  // path holds only stream operations (it may run under graph capture)
  coherent_batch_split_kernel<ROUGH><<<ctas, threads, smem, st>>>(
      jobs, n_jobs, n_items, counter);
  return cuda_status(cudaGetLastError(), "batch split launch");
}

int coherent_batch_split_launch(const BatchJob *jobs, int n_jobs,
                                long long n_items,
                                unsigned long long *counter, int rough_kind,
                                int threads, int ctas, size_t smem,
                                cudaStream_t st) {
  switch (rough_kind) {
    case SS_ROUGH_NONE:
      return batch_split_launch_r<SS_ROUGH_NONE>(jobs, n_jobs, n_items,
                                                 counter, threads, ctas, smem,
                                                 st);
    case SS_ROUGH_GAUSS_FULL:
      return batch_split_launch_r<SS_ROUGH_GAUSS_FULL>(
          jobs, n_jobs, n_items, counter, threads, ctas, smem, st);
    case SS_ROUGH_GAUSS_AREA:
      return batch_split_launch_r<SS_ROUGH_GAUSS_AREA>(
          jobs, n_jobs, n_items, counter, threads, ctas, smem, st);
    default:
      return batch_split_launch_r<SS_ROUGH_EXP_AREA>(
          jobs, n_jobs, n_items, counter, threads, ctas, smem, st);
  }
}

int batch_split_blocks_per_sm(int rough_kind, int threads, size_t smem) {
  // raise the kernel's dynamic shared-memory limit to the largest size any
  // prepared batch uses (never lowered: earlier batches stay launchable)
  static size_t limit[4] = {0, 0, 0, 0};
  const int r = rough_kind & 3;
  limit[r] = std::max(limit[r], smem);
  const int lim = (int)limit[r];
  int n = 0;
  cudaError_t e = cudaSuccess;
  switch (rough_kind) {
#define SS_OCC(R)                                                            \
  case R:                                                                    \
    e = cudaFuncSetAttribute(coherent_batch_split_kernel<R>,                 \
                             cudaFuncAttributeMaxDynamicSharedMemorySize,    \
                             lim);                                           \
    if (e == cudaSuccess)                                                    \
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(                     \
          &n, coherent_batch_split_kernel<R>, threads, smem);                \
    break;
    SS_OCC(SS_ROUGH_NONE)
    SS_OCC(SS_ROUGH_GAUSS_FULL)
    SS_OCC(SS_ROUGH_GAUSS_AREA)
    default:
      SS_OCC(SS_ROUGH_EXP_AREA)
#undef SS_OCC
  }
  return e == cudaSuccess ? n : 0;
}

SplitConsts coherent_split_consts(const CoArgs &a) {
  SplitConsts k{};
  k.k = (float)a.k;
  k.amp_pref = (float)(a.k / kTwoPi);
  k.gamma = (float)a.gamma;
  k.taper_inv = a.taper ? (float)(1.0 / (2.0 * a.taper_s * a.taper_s)) : 0.f;
  const df k2 = df_from_double(2.0 * a.k);
  k.K2h = k2.hi;
  k.K2l = k2.lo;
  const df A = df_from_double(2.0 / (a.c * a.dt));
  const df B = df_from_double(a.t0 / a.dt);
  k.Ah = A.hi;
  k.Al = A.lo;
  k.Bh = B.hi;
  k.Bl = B.lo;
  k.fadL = (float)a.fad.L;
  k.sigma = (float)a.sigma;
  k.corr = (float)a.corr;
  return k;
}

int coherent_split_launch(CoArgs &a, const Plan &p, cudaStream_t st) {
  int pa_len, pb_len;
  pattern_lengths(a.pat_kind, a.pat_n, pa_len, pb_len);
  if (pa_len + pb_len > SS_PAT_MAX) {
    set_error("antenna table too large for the split kernel");
    return SS_ERR_UNSUPPORTED;
  }
  const SplitConsts k = coherent_split_consts(a);
  dim3 grid(p.n_chunks, p.n_groups);
  size_t smem = (size_t)p.tb * a.n_seg * sizeof(float2) +
                (a.rough_kind ? (a.n_terms + 1) * sizeof(float) : 0);
  cudaError_t e = cudaSuccess;
  switch (a.rough_kind) {
#define SS_LAUNCH(R)                                                         \
  case R:                                                                    \
    e = cudaFuncSetAttribute(coherent_split_kernel<R>,                       \
                             cudaFuncAttributeMaxDynamicSharedMemorySize,    \
                             (int)smem);                                     \
    if (e != cudaSuccess) return cuda_status(e, "coherent_split smem");      \
    coherent_split_kernel<R><<<grid, p.threads, smem, st>>>(a, k);           \
    break;
    SS_LAUNCH(SS_ROUGH_NONE)
    SS_LAUNCH(SS_ROUGH_GAUSS_FULL)
    SS_LAUNCH(SS_ROUGH_GAUSS_AREA)
    SS_LAUNCH(SS_ROUGH_EXP_AREA)
#undef SS_LAUNCH
    default:
      return SS_ERR_ARG;
  }
  return cuda_status(cudaGetLastError(), "coherent_split launch");
}

}  // namespace ss
