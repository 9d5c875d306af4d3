// Surface coherent facet sum (Mode D, delta-binned) on GB300.
//
// Work decomposition: the grid is (facet chunks) x (trace blocks). A CTA owns
// `tb` consecutive traces and one contiguous chunk of the union of their
// along-track facet windows; each thread takes one facet at a time and
// evaluates it against every trace of the block (the facet record is loaded
// once per `tb` pairs). Contributions accumulate into per-trace shared-memory
// histograms; each CTA writes its partial histogram to scratch and a second
// kernel sums the chunks in a fixed order (no global atomics, deterministic
// chunk reduction).
//
// Two precisions share that skeleton:
//   FP64  -- every operation in float64, the binning chain written with
//            round-to-nearest intrinsics so bins are bit-identical to the
//            NumPy float64 oracle; histograms in float64.
//   SPLIT -- see ss_coherent_split.cu.
#include <algorithm>

#include "ss_internal.cuh"
#include "ss_coherent.cuh"
#include "ss_f32.cuh"

namespace ss {

// ---------------------------------------------------------------------
// float64 pair evaluation (coherent.py:107-168 + :216-236)
// ---------------------------------------------------------------------
// One CTA's work item (facet chunk `chunk` of trace block `group`); shared
// by the one-call kernel and the batched persistent kernel.
__device__ __forceinline__ void coherent_fp64_cta(const CoArgs &a, int chunk,
                                                  int group,
                                  unsigned char *smem_raw) {
  double2 *hist = reinterpret_cast<double2 *>(smem_raw);
  double *lgam = reinterpret_cast<double *>(hist + (size_t)a.tb * a.n_seg);
  __shared__ double s_p[SS_MAX_TB][3];
  __shared__ double s_u[SS_MAX_TB][3];
  __shared__ double s_pv[SS_MAX_TB][6];
  __shared__ int s_lo[SS_MAX_TB], s_hi[SS_MAX_TB];
  __shared__ double s_drop[SS_MAX_TB];
  __shared__ int s_rng[2];

  const int t_base = group * a.tb;
  const int nt = min(a.tb, a.T - t_base);
  const int tid = threadIdx.x;

  if (tid < nt) {
    const int t = t_base + tid;
    for (int j = 0; j < 3; ++j) s_p[tid][j] = a.pos[3 * t + j];
    for (int j = 0; j < 3; ++j) s_u[tid][j] = a.uct ? a.uct[3 * t + j] : 0.0;
    for (int j = 0; j < 6; ++j)
      s_pv[tid][j] = (a.pv && j < a.pv_len) ? a.pv[a.pv_len * t + j] : 0.0;
    long lo = (long)a.off[t] * a.bs;
    long hi = min((long)(a.off[t] + a.n_win) * a.bs, (long)a.N);
    s_lo[tid] = (int)min(lo, (long)a.N);
    s_hi[tid] = (int)hi;
    s_drop[tid] = 0.0;
  }
  for (int j = tid; j < a.tb * a.n_seg; j += blockDim.x)
    hist[j] = make_double2(0.0, 0.0);
  if (a.rough_kind != SS_ROUGH_NONE)
    for (int m = tid; m <= a.n_terms; m += blockDim.x)
      lgam[m] = lgamma((double)m + 1.0);
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
  }
  __syncthreads();

  const double k = a.k;
  const double amp_pref = k / kTwoPi;
  // traces rotated across lanes and dropped power kept per thread, as in
  // the split form (ss_coherent_split.cu)
  const int rot = (tid & 31) % max(nt, 1);
  double dropl[SS_MAX_TB];
#pragma unroll
  for (int j = 0; j < SS_MAX_TB; ++j) dropl[j] = 0.0;
  for (int i = s_rng[0] + tid; i < s_rng[1]; i += blockDim.x) {
    const double cx = a.F.cx[i], cy = a.F.cy[i], cz = a.F.cz[i];
    const double nx = a.F.nx[i], ny = a.F.ny[i], nz = a.F.nz[i];
    const double e1x = a.F.e1x[i], e1y = a.F.e1y[i], e1z = a.F.e1z[i];
    const double e2x = a.F.e2x[i], e2y = a.F.e2y[i], e2z = a.F.e2z[i];
    const double area = a.F.area[i];
    const double gam = a.F.gamma_f32 ? (double)a.F.gamma_f32[i] : a.gamma;
    for (int st = 0; st < nt; ++st) {
      const int tt = rot + st < nt ? rot + st : rot + st - nt;
      if (i < s_lo[tt] || i >= s_hi[tt]) continue;
      // range chain in round-to-nearest (bins bit-identical to NumPy)
      const double dx = __dsub_rn(s_p[tt][0], cx);
      const double dy = __dsub_rn(s_p[tt][1], cy);
      const double dz = __dsub_rn(s_p[tt][2], cz);
      const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx),
                                            __dmul_rn(dy, dy)),
                                  __dmul_rn(dz, dz));
      const double r = __dsqrt_rn(r2);
      const double cosv = dot3(dx, dy, dz, nx, ny, nz) / r;
      const double rx = dx / r, ry = dy / r, rz = dz / r;
      const double d1 = dot3(rx, ry, rz, e1x, e1y, e1z);
      const double d2 = dot3(rx, ry, rz, e2x, e2y, e2z);
      const double s1 = sinc_np(d1 * (k / kPi));
      const double s2 = sinc_np(d2 * (k / kPi));
      double amp = amp_pref * gam * cosv * area * s1 * s2 / (r * r);
      if (a.taper) {
        double cc = fmin(fmax(cosv, 1e-9), 1.0);
        double c2 = cc * cc;
        amp *= exp(-(1.0 - c2) / (c2 * (2.0 * a.taper_s * a.taper_s)));
      }
      double cr = amp, ci = 0.0;
      if (a.rough_kind != SS_ROUGH_NONE) {
        const double sg = a.F.sigma ? (double)a.F.sigma[i] : a.sigma;
        const double lc = a.F.corr ? (double)a.F.corr[i] : a.corr;
        const double l1 = sqrt(dot3(e1x, e1y, e1z, e1x, e1y, e1z));
        const double l2 = sqrt(dot3(e2x, e2y, e2z, e2x, e2y, e2z));
        const double kk = 2.0 * k * cosv;
        const double dp = d_phi64(a.rough_kind, a.n_terms, lgam, a.fad.a,
                                  a.fad.L, sg, lc, kk, 2.0 * k * d1 / l1,
                                  2.0 * k * d2 / l2, l1, l2);
        const double amp_i =
            area > 0.0 ? amp_pref * gam * cosv / (r * r) * sqrt(dp) : 0.0;
        const double sk = sg * kk;
        const double att = exp(-0.5 * (sk * sk));
        const double phr = a.F.phasor[2 * i], phi = a.F.phasor[2 * i + 1];
        cr = amp * att + amp_i * phr;
        ci = amp_i * phi;
      }
      // 1j * (cr + j ci) * exp(-2j k r)
      double sn, cs;
      sincos(2.0 * k * r, &sn, &cs);
      double re = cr * sn - ci * cs;
      double im = cr * cs + ci * sn;
      if (a.pat_kind != SS_PAT_ISOTROPIC) {
        const double g = gain64(a.pat_kind, a.pat_n, a.pa, a.pb, s_pv[tt],
                                -rx, -ry, -rz);
        re *= g * g;
        im *= g * g;
      }
      // fast-time bin (geometry.py:18-24), round-to-nearest like NumPy
      const double twtt = __ddiv_rn(__dmul_rn(2.0, r), a.c);
      const double u = __ddiv_rn(__dsub_rn(twtt, a.t0), a.dt);
      int side_off = 0;
      if (a.split) {
        const double ax = -dx, ay = -dy, az = -dz;  // c - p
        if (dot3(ax, ay, az, s_u[tt][0], s_u[tt][1], s_u[tt][2]) > 0.0)
          side_off = a.n_samples;
      }
      double2 *h = hist + (size_t)tt * a.n_seg + side_off;
      const double fb = floor(u);
      if (a.interp) {
        const double w = __dsub_rn(u, fb);
        const double parts[2] = {1.0 - w, w};
        for (int q = 0; q < 2; ++q) {
          const double bq = fb + q;
          const double pr = re * parts[q], pim = im * parts[q];
          if (bq >= 0.0 && bq < (double)a.n_samples) {
            atomicAdd(&h[(int)bq].x, pr);
            atomicAdd(&h[(int)bq].y, pim);
          } else {
            dropl[tt] += pr * pr + pim * pim;
          }
        }
      } else if (fb >= 0.0 && fb < (double)a.n_samples) {
        atomicAdd(&h[(int)fb].x, re);
        atomicAdd(&h[(int)fb].y, im);
      } else {
        dropl[tt] += re * re + im * im;
      }
    }
  }
  for (int tt = 0; tt < nt; ++tt)
    if (dropl[tt] != 0.0) atomicAdd(&s_drop[tt], dropl[tt]);
  __syncthreads();
  double2 *part = reinterpret_cast<double2 *>(a.part);
  for (int tt = 0; tt < nt; ++tt) {
    const size_t base = ((size_t)chunk * a.T + t_base + tt) * a.n_seg;
    for (int j = tid; j < a.n_seg; j += blockDim.x)
      part[base + j] = hist[(size_t)tt * a.n_seg + j];
  }
  if (tid < nt) a.part_drop[(size_t)chunk * a.T + t_base + tid] = s_drop[tid];
}

__global__ void __launch_bounds__(256)
coherent_fp64_kernel(CoArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  coherent_fp64_cta(a, blockIdx.x, blockIdx.y, smem_raw);
}

// Batched persistent form (see coherent_batch_split_kernel).
__global__ void __launch_bounds__(256)
coherent_batch_fp64_kernel(const BatchJob *jobs, int n_jobs,
                           long long n_items, unsigned long long *counter) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ long long s_item;
  __shared__ int s_job;
  for (;;) {
    __syncthreads();
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
    coherent_fp64_cta(J.a, (int)(local % J.n_chunks),
                      (int)(local / J.n_chunks), smem_raw);
  }
}

int coherent_batch_fp64_launch(const BatchJob *jobs, int n_jobs,
                               long long n_items, unsigned long long *counter,
                               int threads, int ctas, size_t smem,
                               cudaStream_t st) {
  coherent_batch_fp64_kernel<<<ctas, threads, smem, st>>>(jobs, n_jobs,
                                                           n_items, counter);
  return cuda_status(cudaGetLastError(), "batch fp64 launch");
}

int batch_fp64_blocks_per_sm(int threads, size_t smem) {
  static size_t limit = 0;
  limit = std::max(limit, smem);
  int n = 0;
  if (cudaFuncSetAttribute(coherent_batch_fp64_kernel,
                           cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)limit) != cudaSuccess)
    return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(
          &n, coherent_batch_fp64_kernel, threads, smem) != cudaSuccess)
    return 0;
  return n;
}

// ---------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------
int coherent_plan(const ss_coherent_opts *o, int T, int N, Plan *p,
                  bool rough) {
  if (o->n_samples <= 0 || T <= 0 || N <= 0 || o->block_size <= 0 ||
      o->n_win <= 0)
    return SS_ERR_ARG;
  const int n_seg = o->n_samples * (o->split_sides ? 2 : 1);
  const bool fp64 = o->precision == SS_PREC_FP64;
  const size_t elt = fp64 ? 16 : 8;
  // split form: 32 resident warps per SM at 64 registers hide the
  // shared-memory atomic latency of this short per-pair computation. Smooth
  // facets run two 512-thread CTAs of 96 KB of histograms (six traces of
  // 2048 bins share each facet's double-float reference); the roughness
  // series needs 80 registers, so three 256-thread CTAs of 48 KB.
  const size_t budget = fp64 ? 96 * 1024 : (rough ? 48 * 1024 : 96 * 1024);
  const size_t per_trace = (size_t)n_seg * elt;
  if (per_trace > 200 * 1024) return SS_ERR_UNSUPPORTED;
  int tb = (int)std::max<size_t>(1, std::min<size_t>(budget / per_trace,
                                                     SS_MAX_TB));
  tb = std::min(tb, T);
  p->tb = tb;
  p->n_groups = (T + tb - 1) / tb;
  p->threads = fp64 || rough ? 256 : 512;
  const long window = std::min<long>((long)o->n_win * o->block_size, N);
  const int max_chunks = (int)std::max<long>(1, window / 512);
  // resident CTAs per SM: 2 (512-thread smooth split, 96 KB FP64), 3
  // (rough split at 80 registers); the chunk count whose item total fills
  // 1-4 whole waves best (a last wave a tenth full costs a full wave); on
  // a tie the fewest waves, whose CTAs zero, fill and write their
  // histograms fewer times per pair
  const long slots = (long)sm_count() * (fp64 ? 2 : (rough ? 3 : 2));
  int best = 1;
  double best_eff = -1.0;
  for (int k = 1; k <= 4; ++k) {
    const int nc = (int)std::max<long>(
        1, std::min<long>(max_chunks, k * slots / p->n_groups));
    const long items = (long)nc * p->n_groups;
    const long waves = (items + slots - 1) / slots;
    const double eff = (double)items / (double)(waves * slots);
    if (eff > best_eff + 1e-9) {
      best_eff = eff;
      best = nc;
    }
  }
  p->n_chunks = best;
  p->smem = (size_t)tb * per_trace + (SS_MAX_TERMS + 1) * sizeof(double);
  return SS_OK;
}

size_t coherent_scratch(const ss_coherent_opts *o, int T, int N) {
  // the options do not say whether the facets are rough: size for the
  // larger chunk count of the two plans
  Plan p, pr;
  if (coherent_plan(o, T, N, &p, false) != SS_OK ||
      coherent_plan(o, T, N, &pr, true) != SS_OK)
    return 0;
  p.n_chunks = std::max(p.n_chunks, pr.n_chunks);
  const int n_seg = o->n_samples * (o->split_sides ? 2 : 1);
  const size_t elt = o->precision == SS_PREC_FP64 ? 16 : 8;
  size_t hist = (size_t)p.n_chunks * T * n_seg * elt;
  hist = (hist + 255) & ~(size_t)255;
  return hist + (size_t)p.n_chunks * T * sizeof(double);
}

int coherent_launch(CoArgs &a, const Plan &p, const ss_output *out,
                    cudaStream_t st) {
  a.tb = p.tb;
  a.n_chunks = p.n_chunks;
  dim3 grid(p.n_chunks, p.n_groups);
  if (a.precision == SS_PREC_FP64) {
    size_t smem = (size_t)p.tb * a.n_seg * 16 +
                  (a.rough_kind ? (a.n_terms + 1) * sizeof(double) : 0);
    cudaError_t e = cudaFuncSetAttribute(
        coherent_fp64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
        (int)smem);
    if (e != cudaSuccess) return cuda_status(e, "coherent_fp64 smem");
    coherent_fp64_kernel<<<grid, p.threads, smem, st>>>(a);
    int s = cuda_status(cudaGetLastError(), "coherent_fp64 launch");
    if (s) return s;  } else {
    int s = coherent_split_launch(a, p, st);
    if (s) return s;
  }
  ReduceArgs r{a.T, a.n_seg, a.n_samples, a.split, a.n_chunks, a.part,
               a.part_drop};
  return launch_reduce(r, a.precision == SS_PREC_FP64, out, st);
}

}  // namespace ss

// ---------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------
extern "C" size_t ss_coherent_scratch_bytes(const ss_coherent_opts *opts,
                                            int32_t n_traces,
                                            int32_t n_facets) {
  if (!opts) return 0;
  return ss::coherent_scratch(opts, n_traces, n_facets);
}

namespace ss {

// Validate one coherent call and fill its argument block (everything but
// the scratch layout); shared by the one-call and the batched entry points.
int build_co_args(const ss_coherent_opts *opts, const ss_facets *facets,
                  const ss_traces *traces, const ss_pattern *pattern,
                  const ss_roughness *rough, const ss_output *out, Plan &p,
                  CoArgs &a) {
  if (!opts || !facets || !traces || !out) {
    set_error("null argument");
    return SS_ERR_ARG;
  }
  const int T = traces->n_traces, N = facets->n_facets;
  if (!traces->pos || !traces->off || !facets->cx || !facets->area ||
      !out->dropped || (!out->field_c128 && !out->field_c64)) {
    set_error("missing required device pointer");
    return SS_ERR_ARG;
  }
  if (opts->split_sides && !traces->uct) {
    set_error("split_sides needs u_ct");
    return SS_ERR_ARG;
  }
  if (opts->precision != SS_PREC_FP64 && opts->precision != SS_PREC_SPLIT) {
    set_error("unknown precision");
    return SS_ERR_ARG;
  }
  int s = coherent_plan(opts, T, N, &p,
                        rough && rough->kind != SS_ROUGH_NONE);
  if (s) {
    set_error(s == SS_ERR_UNSUPPORTED ? "n_samples too large for the "
                                        "shared-memory histogram"
                                      : "bad sizes");
    return s;
  }
  a = CoArgs{};
  a.F = *facets;
  a.pos = traces->pos;
  a.uct = traces->uct;
  a.pv = traces->pv;
  a.off = traces->off;
  a.T = T;
  a.N = N;
  a.pv_len = traces->pv_len;
  a.k = opts->k;
  a.gamma = opts->gamma;
  a.t0 = opts->t0;
  a.dt = opts->dt;
  a.c = opts->c;
  a.taper_s = opts->taper_s;
  a.n_samples = opts->n_samples;
  a.n_seg = opts->n_samples * (opts->split_sides ? 2 : 1);
  a.bs = opts->block_size;
  a.n_win = opts->n_win;
  a.split = opts->split_sides;
  a.interp = opts->interp_bins;
  a.taper = opts->taper;
  a.precision = opts->precision;
  a.pat_kind = pattern ? pattern->kind : SS_PAT_ISOTROPIC;
  a.pat_n = pattern ? pattern->n : 0;
  a.pa = pattern ? pattern->pa : nullptr;
  a.pb = pattern ? pattern->pb : nullptr;
  if (a.precision == SS_PREC_SPLIT) {
    // the split kernels stage the antenna table in shared memory
    int pa_len, pb_len;
    pattern_lengths(a.pat_kind, a.pat_n, pa_len, pb_len);
    if (pa_len + pb_len > SS_PAT_MAX) {
      set_error("antenna table too large for the split kernel");
      return SS_ERR_UNSUPPORTED;
    }
  }
  if (a.pat_kind != SS_PAT_ISOTROPIC && (!traces->pv || traces->pv_len < 3)) {
    set_error("antenna pattern needs per-trace pattern vectors");
    return SS_ERR_ARG;
  }
  if ((a.pat_kind == SS_PAT_ARRAY || a.pat_kind == SS_PAT_ARRAY_TAPERED) &&
      traces->pv_len < 6) {
    set_error("array patterns need (T, 2, 3) pattern vectors");
    return SS_ERR_ARG;
  }
  a.rough_kind = rough ? rough->kind : SS_ROUGH_NONE;
  if (a.rough_kind != SS_ROUGH_NONE) {
    if (!facets->phasor || rough->n_terms < 0 ||
        rough->n_terms > SS_MAX_TERMS) {
      set_error("roughness needs phasors and 0 <= n_terms <= 4096");
      return SS_ERR_ARG;
    }
    a.n_terms = rough->n_terms;
    a.sigma = rough->sigma;
    a.corr = rough->corr;
    a.fad = faddeeva_coeffs();
  }
  a.tb = p.tb;
  a.n_chunks = p.n_chunks;
  return SS_OK;
}

}  // namespace ss

extern "C" int ss_coherent_fwd(const ss_coherent_opts *opts,
                               const ss_facets *facets,
                               const ss_traces *traces,
                               const ss_pattern *pattern,
                               const ss_roughness *rough,
                               const ss_output *out, void *scratch,
                               size_t scratch_bytes, void *stream) {
  using namespace ss;
  Plan p;
  CoArgs a;
  int s = build_co_args(opts, facets, traces, pattern, rough, out, p, a);
  if (s) return s;
  const int T = traces->n_traces, N = facets->n_facets;
  const size_t need = coherent_scratch(opts, T, N);
  if (!scratch || scratch_bytes < need) {
    set_error("scratch buffer too small");
    return SS_ERR_SCRATCH;
  }
  a.part = scratch;
  size_t hist = (size_t)p.n_chunks * T * a.n_seg *
                (opts->precision == SS_PREC_FP64 ? 16 : 8);
  hist = (hist + 255) & ~(size_t)255;
  a.part_drop = reinterpret_cast<double *>(static_cast<char *>(scratch) +
                                           hist);
  return coherent_launch(a, p, out, static_cast<cudaStream_t>(stream));
}
