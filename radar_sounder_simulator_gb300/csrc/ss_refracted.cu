// Refracted multilayer facet sum (FP64 form) on GB300.
//
// Same trace-block x facet-chunk decomposition and shared-memory histograms
// as the surface kernel (ss_coherent.cu). Per (trace, target facet) pair the
// refracted path is solved in float64 exactly as the reference program does:
//   sequential: per crossed interface a 10-iteration two-point Snell solve
//     on the mean plane anchors an affine facet lookup, then a 25-iteration
//     solve on that facet's tangent plane (multilayer.py:352-406);
//   joint: the mean-plane chain anchors every lookup, then a damped Newton on
//     2-D in-plane offsets with block-tridiagonal (Thomas) steps and step
//     halving solves all crossings at once (multilayer.py:408-457,
//     refraction_joint.py:249-322);
// followed by Fresnel transmission, ray-tube spreading, two-way attenuation,
// antenna gain, the facet's sinc response at the local wavenumber,
// roughness, diffuse channel and binning (multilayer.py:500-583).
#include <algorithm>

#include "ss_refracted_fp64.cuh"

namespace ss {

template <int NI>
__global__ void __launch_bounds__(128)
refracted_fp64_kernel(RefArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2 *hist = reinterpret_cast<double2 *>(smem_raw);
  double *lgam = reinterpret_cast<double *>(hist + (size_t)a.tb * a.n_seg);
  __shared__ double s_p[SS_MAX_TB][3], s_u[SS_MAX_TB][3], s_pv[SS_MAX_TB][6];
  __shared__ int s_lo[SS_MAX_TB], s_hi[SS_MAX_TB];
  __shared__ double s_drop[SS_MAX_TB];
  __shared__ int s_rng[2];
  const int chunk = blockIdx.x;
  const int t_base = blockIdx.y * a.tb;
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

  const int nj = a.leg_last;  // final medium (multilayer.py:506)
  const double n0 = a.n_leg[0], njn = a.n_leg[nj];
  for (int i = s_rng[0] + tid; i < s_rng[1]; i += blockDim.x) {
    const double q[3] = {(double)a.F.cx[i], (double)a.F.cy[i],
                         (double)a.F.cz[i]};
    const double fn[3] = {(double)a.F.nx[i], (double)a.F.ny[i],
                          (double)a.F.nz[i]};
    const double fa = a.F.area[i];
    for (int tt = 0; tt < nt; ++tt) {
      if (i < s_lo[tt] || i >= s_hi[tt]) continue;
      Path64 P;
      if (NI == 0)
        path_sequential64(a, s_p[tt], q, P);
      else
        path_joint64<NI == 0 ? 1 : NI>(a, s_p[tt], q, P);
      // final leg (medium j): crossing -> facet
      double d[3] = {P.cur[0] - q[0], P.cur[1] - q[1], P.cur[2] - q[2]};
      const double s_j = sqrt(dot3v(d, d));
      const double inv = 1.0 / fmax(s_j, 1e-30);
      const double rh[3] = {d[0] * inv, d[1] * inv, d[2] * inv};
      const double opl = P.opl + njn * s_j;
      const double loss = P.loss_db + s_j * (a.att_leg[nj] / 1000.0);
      const double sperp = P.sum_perp + s_j / njn;
      const double spar = P.sum_par + s_j / (njn * P.c_last * P.c_last);
      const double l_perp = n0 * sperp;
      const double l_par = n0 * P.c0 * P.c0 * spar;
      const double flux = (n0 * P.c0) / (njn * P.c_last);
      const double att_f = pow(10.0, -loss / 10.0);
      const double cos_t = dot3v(rh, fn);
      double spread = P.tau2 * flux / (l_par * l_perp);
      if (a.pat_kind != SS_PAT_ISOTROPIC) {
        double d0[3] = {P.xf[0] - s_p[tt][0], P.xf[1] - s_p[tt][1],
                        P.xf[2] - s_p[tt][2]};
        const double dm = fmax(sqrt(dot3v(d0, d0)), 1e-30);
        const double g = gain64(a.pat_kind, a.pat_n, a.pa, a.pb, s_pv[tt],
                                d0[0] / dm, d0[1] / dm, d0[2] / dm);
        spread = spread * (g * g);
      }
      double re, im, pwr;
      if (a.coherent) {
        const double gam = a.F.gamma_f64 ? a.F.gamma_f64[i] : a.gamma;
        const double kj = a.k0 * njn;
        const double f1[3] = {(double)a.F.e1x[i], (double)a.F.e1y[i],
                              (double)a.F.e1z[i]};
        const double f2[3] = {(double)a.F.e2x[i], (double)a.F.e2y[i],
                              (double)a.F.e2z[i]};
        const double d1 = dot3v(rh, f1), d2 = dot3v(rh, f2);
        const double s1 = sinc_np(d1 * (kj / kPi));
        const double s2 = sinc_np(d2 * (kj / kPi));
        double amp = (kj / kTwoPi) * gam * cos_t * fa * s1 * s2 * spread * att_f;
        if (a.taper) {
          double ct = fmin(fmax(cos_t, kCMin), 1.0);
          const double ct2 = ct * ct;
          amp = amp * exp(-(1.0 - ct2) / (ct2 * (2.0 * a.taper_s * a.taper_s)));
        }
        double cr = amp, ci = 0.0;
        if (a.rough_kind != SS_ROUGH_NONE) {
          const double sg = a.F.sigma ? (double)a.F.sigma[i] : a.sigma;
          const double lc = a.F.corr ? (double)a.F.corr[i] : a.corr;
          const double l1 = sqrt(dot3v(f1, f1)), l2 = sqrt(dot3v(f2, f2));
          const double kk = 2.0 * kj * cos_t;
          const double dp = d_phi64(a.rough_kind, a.n_terms, lgam, a.fad.a,
                                    a.fad.L, sg, lc, kk, 2.0 * kj * d1 / l1,
                                    2.0 * kj * d2 / l2, l1, l2);
          const double sk = sg * kk;
          cr = amp * exp(-0.5 * (sk * sk));
          if (fa > 0.0) {
            const double ai = (kj / kTwoPi) * gam * cos_t * spread * att_f *
                              sqrt(dp);
            cr += ai * (double)a.F.phasor[2 * i];
            ci += ai * (double)a.F.phasor[2 * i + 1];
          }
        }
        if (a.F.diffuse_amp && fa > 0.0) {
          const double ct = fmax(cos_t, 0.0);
          const double ad = sqrt(fmax(fa, 0.0) / kTwoPi) * a.F.diffuse_amp[i] *
                            ct * pow(ct, 0.5 * a.n_exp) * spread * att_f;
          cr += ad * (double)a.F.diffuse_phasor[2 * i];
          ci += ad * (double)a.F.diffuse_phasor[2 * i + 1];
        }
        double sn, cs;
        sincos(2.0 * a.k0 * opl, &sn, &cs);
        re = cr * sn - ci * cs;
        im = cr * cs + ci * sn;
        pwr = re * re + im * im;
      } else {
        const double aa = fa * cos_t * spread;
        re = aa * aa * att_f * att_f;
        im = 0.0;
        pwr = re;
      }
      const double twtt = __ddiv_rn(__dmul_rn(2.0, opl), a.c);
      const double fb = floor(__ddiv_rn(__dsub_rn(twtt, a.t0), a.dt));
      const bool ok = P.valid && fb >= 0.0 && fb < (double)a.n_samples;
      if (ok) {
        int b = (int)fb;
        if (a.split) {
          double v[3] = {q[0] - s_p[tt][0], q[1] - s_p[tt][1],
                         q[2] - s_p[tt][2]};
          if (dot3v(v, s_u[tt]) > 0.0) b += a.n_samples;
        }
        double2 *h = hist + (size_t)tt * a.n_seg + b;
        atomicAdd(&h->x, re);
        if (a.coherent) atomicAdd(&h->y, im);
      } else {
        atomicAdd(&s_drop[tt], pwr);
      }
    }
  }
  __syncthreads();
  double2 *part = reinterpret_cast<double2 *>(a.part);
  for (int tt = 0; tt < nt; ++tt) {
    const size_t base = ((size_t)chunk * a.T + t_base + tt) * a.n_seg;
    for (int j = tid; j < a.n_seg; j += blockDim.x)
      part[base + j] = hist[(size_t)tt * a.n_seg + j];
  }
  if (tid < nt) a.part_drop[(size_t)chunk * a.T + t_base + tid] = s_drop[tid];
}

// ---------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------
static int refracted_plan(const ss_refracted_opts *o, int T, int N, Plan *p) {
  if (o->n_samples <= 0 || T <= 0 || N <= 0 || o->block_size <= 0 ||
      o->n_win <= 0 || o->n_crossed < 1 || o->n_crossed > SS_MAX_IFACE)
    return SS_ERR_ARG;
  const int n_seg = o->n_samples * (o->split_sides ? 2 : 1);
  const size_t elt = o->precision == SS_PREC_FP64 ? 16 : 8;
  const size_t per_trace = (size_t)n_seg * elt;
  if (per_trace > 200 * 1024) return SS_ERR_UNSUPPORTED;
  const size_t budget = 96 * 1024;
  int tb = (int)std::max<size_t>(1, std::min<size_t>(budget / per_trace,
                                                     SS_MAX_TB));
  tb = std::min(tb, T);
  p->tb = tb;
  p->n_groups = (T + tb - 1) / tb;
  p->threads = o->precision == SS_PREC_FP64 ? 128 : kSplitThreads;
  const long window = std::min<long>((long)o->n_win * o->block_size, N);
  const int max_chunks = (int)std::max<long>(1, window / 256);
  if (o->precision == SS_PREC_FP64) {
    const int target = 8 * sm_count();
    p->n_chunks = std::max(
        1, std::min(max_chunks, (target + p->n_groups - 1) / p->n_groups));
  } else {
    // resident CTAs per SM of the split kernel that runs: two 512-thread
    // CTAs (64 registers) for the sequential chain and joint solves through
    // up to two interfaces, one (~128 registers) through three or more; the
    // chunk count whose item total fills 4-12 whole waves best (a last
    // wave half full costs a full one), the fewest waves on a tie
    const long slots = (long)sm_count() *
                       (!o->joint || o->n_crossed <= 2 ? 2 : 1);
    int best = 1;
    double best_eff = -1.0;
    for (int k = 4; k <= 12; ++k) {
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
  }
  p->smem = (size_t)tb * per_trace;
  return SS_OK;
}

// Deferral bitmask of the split form: one bit per (trace, window slot).
static long long defer_slots(const ss_refracted_opts *o, int N) {
  return std::min<long long>((long long)o->n_win * o->block_size, N);
}

static size_t defer_mask_bytes(const ss_refracted_opts *o, int T, int N) {
  const unsigned long long bits = (unsigned long long)T * defer_slots(o, N);
  return (size_t)((bits + 31) / 32) * sizeof(uint32_t);
}

static size_t refracted_scratch(const ss_refracted_opts *o, int T, int N) {
  Plan p;
  if (refracted_plan(o, T, N, &p) != SS_OK) return 0;
  const int n_seg = o->n_samples * (o->split_sides ? 2 : 1);
  const size_t elt = o->precision == SS_PREC_FP64 ? 16 : 8;
  size_t hist = (size_t)p.n_chunks * T * n_seg * elt;
  hist = (hist + 255) & ~(size_t)255;
  size_t drop = (size_t)p.n_chunks * T * sizeof(double);
  if (o->precision == SS_PREC_FP64) return hist + drop;
  drop = (drop + 255) & ~(size_t)255;
  return hist + drop + defer_mask_bytes(o, T, N);
}

template <int NI>
static int launch_fp64(RefArgs &a, const Plan &p, size_t smem,
                       cudaStream_t st) {
  cudaError_t e = cudaFuncSetAttribute(
      refracted_fp64_kernel<NI>, cudaFuncAttributeMaxDynamicSharedMemorySize,
      (int)smem);
  if (e != cudaSuccess) return cuda_status(e, "refracted_fp64 smem");
  dim3 grid(p.n_chunks, p.n_groups);
  refracted_fp64_kernel<NI><<<grid, p.threads, smem, st>>>(a);
  return cuda_status(cudaGetLastError(), "refracted_fp64 launch");
}

}  // namespace ss

extern "C" size_t ss_refracted_scratch_bytes(const ss_refracted_opts *opts,
                                             int32_t n_traces,
                                             int32_t n_facets) {
  if (!opts) return 0;
  return ss::refracted_scratch(opts, n_traces, n_facets);
}

namespace ss {

// Validate the call and fill the argument block shared by the forward and
// adjoint entry points (everything but the scratch layout).
int build_ref_args(const ss_refracted_opts *opts,
                          const ss_facets *target, const ss_traces *traces,
                          const ss_pattern *pattern, const ss_roughness *rough,
                          bool need_output, const ss_output *out, Plan &p,
                          RefArgs &a) {
  if (!opts || !target || !traces || (need_output && !out) || !opts->crossed ||
      !opts->n_leg || !opts->eps_leg || !opts->att_leg) {
    set_error("null argument");
    return SS_ERR_ARG;
  }
  const int T = traces->n_traces, N = target->n_facets;
  if (!traces->pos || !traces->off || !target->cx || !target->area ||
      (need_output &&
       (!out->dropped || (!out->field_c128 && !out->field_c64)))) {
    set_error("missing required device pointer");
    return SS_ERR_ARG;
  }
  if (opts->split_sides && !traces->uct) {
    set_error("split_sides needs u_ct");
    return SS_ERR_ARG;
  }
  int s = refracted_plan(opts, T, N, &p);
  if (s) {
    set_error(s == SS_ERR_UNSUPPORTED ? "n_samples too large" :
              "bad sizes or crossed-interface count (1..40)");
    return s;
  }
  if (opts->joint && (opts->k_pad < 0 || opts->k_pad >= opts->n_crossed)) {
    set_error("k_pad out of range");
    return SS_ERR_ARG;
  }
  a = RefArgs{};
  a.F = *target;
  a.pos = traces->pos;
  a.uct = traces->uct;
  a.pv = traces->pv;
  a.off = traces->off;
  a.T = T;
  a.N = N;
  a.pv_len = traces->pv_len;
  a.ni = opts->n_crossed;
  a.k_pad = opts->joint ? opts->k_pad : 0;
  for (int i = 0; i < a.ni; ++i) {
    a.ifc[i] = opts->crossed[i];
    if (!a.ifc[i].table || a.ifc[i].ny < 1 || a.ifc[i].nx < 1) {
      set_error("crossed interface without a lookup table");
      return SS_ERR_ARG;
    }
    a.sig_c[i] = opts->sigma_crossed ? opts->sigma_crossed[i] : 0.0;
  }
  const int n_legs = opts->n_legs > 0 ? opts->n_legs : a.ni + 1;
  if (n_legs < a.ni + 1 || n_legs > SS_MAX_IFACE + 1 ||
      (opts->joint && n_legs != a.ni + 1)) {
    set_error("leg arrays need n_crossed + 1 entries");
    return SS_ERR_ARG;
  }
  a.leg_last = n_legs - 1;
  for (int i = 0; i < n_legs; ++i) {
    a.n_leg[i] = opts->n_leg[i];
    a.eps_leg[i] = opts->eps_leg[i];
    a.att_leg[i] = opts->att_leg[i];
  }
  a.rough_cross = opts->sigma_crossed != nullptr;
  a.k0 = opts->k0;
  a.gamma = opts->gamma;
  a.t0 = opts->t0;
  a.dt = opts->dt;
  a.c = opts->c;
  a.taper_s = opts->taper_s;
  a.n_exp = opts->diffuse_exp;
  a.n_samples = opts->n_samples;
  a.n_seg = opts->n_samples * (opts->split_sides ? 2 : 1);
  a.bs = opts->block_size;
  a.n_win = opts->n_win;
  a.split = opts->split_sides;
  a.coherent = opts->coherent;
  a.joint = opts->joint;
  a.n_newton = opts->joint_newton;
  a.n_backtrack = opts->joint_backtrack;
  a.taper = opts->taper;
  a.precision = opts->precision;
  a.pat_kind = pattern ? pattern->kind : SS_PAT_ISOTROPIC;
  a.pat_n = pattern ? pattern->n : 0;
  a.pa = pattern ? pattern->pa : nullptr;
  a.pb = pattern ? pattern->pb : nullptr;
  if (a.pat_kind != SS_PAT_ISOTROPIC && (!traces->pv || traces->pv_len < 3)) {
    set_error("antenna pattern needs per-trace pattern vectors");
    return SS_ERR_ARG;
  }
  a.rough_kind = rough ? rough->kind : SS_ROUGH_NONE;
  if (a.rough_kind != SS_ROUGH_NONE) {
    if (!target->phasor || rough->n_terms < 0 ||
        rough->n_terms > SS_MAX_TERMS) {
      set_error("roughness needs phasors and 0 <= n_terms <= 4096");
      return SS_ERR_ARG;
    }
    a.n_terms = rough->n_terms;
    a.sigma = rough->sigma;
    a.corr = rough->corr;
    a.fad = faddeeva_coeffs();
  }
  if (!a.coherent && (a.rough_kind || a.rough_cross || target->diffuse_amp ||
                      a.taper || target->gamma_f64)) {
    set_error("roughness, taper, diffuse and per-facet gamma require "
              "coherent mode");
    return SS_ERR_ARG;
  }
  a.tb = p.tb;
  a.n_chunks = p.n_chunks;
  return SS_OK;
}

}  // namespace ss

extern "C" int ss_refracted_fwd(const ss_refracted_opts *opts,
                                const ss_facets *target,
                                const ss_traces *traces,
                                const ss_pattern *pattern,
                                const ss_roughness *rough,
                                const ss_output *out, void *scratch,
                                size_t scratch_bytes, void *stream) {
  using namespace ss;
  Plan p;
  RefArgs a;
  int s = build_ref_args(opts, target, traces, pattern, rough, true, out, p,
                         a);
  if (s) return s;
  const int T = traces->n_traces, N = target->n_facets;
  const size_t need = refracted_scratch(opts, T, N);
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
  if (opts->precision != SS_PREC_FP64) {
    const size_t drop =
        ((size_t)p.n_chunks * T * sizeof(double) + 255) & ~(size_t)255;
    a.defer_mask = reinterpret_cast<uint32_t *>(static_cast<char *>(scratch) +
                                                hist + drop);
    a.defer_w = defer_slots(opts, N);
  }
  a.tb = p.tb;
  a.n_chunks = p.n_chunks;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (opts->precision == SS_PREC_FP64) {
    const size_t smem = (size_t)p.tb * a.n_seg * 16 +
                        (a.rough_kind ? (a.n_terms + 1) * sizeof(double) : 0);
    if (!a.joint) s = launch_fp64<0>(a, p, smem, st);
    else switch (a.ni) {
      case 1: s = launch_fp64<1>(a, p, smem, st); break;
      case 2: s = launch_fp64<2>(a, p, smem, st); break;
      case 3: s = launch_fp64<3>(a, p, smem, st); break;
      case 4: s = launch_fp64<4>(a, p, smem, st); break;
      case 5: s = launch_fp64<5>(a, p, smem, st); break;
      case 6: s = launch_fp64<6>(a, p, smem, st); break;
      case 7: s = launch_fp64<7>(a, p, smem, st); break;
      case 8: s = launch_fp64<8>(a, p, smem, st); break;
      // deeper stacks (firn runs cross tens of layers): one instantiation
      // whose joint-solve arrays hold SS_MAX_IFACE interfaces
      default: s = launch_fp64<kDeepNI>(a, p, smem, st); break;
    }
  } else {
    s = refracted_split_launch(a, p, st);
  }
  if (s) return s;
  ReduceArgs r{a.T, a.n_seg, a.n_samples, a.split, a.n_chunks, a.part,
               a.part_drop};
  return launch_reduce(r, opts->precision == SS_PREC_FP64, out, st);
}

extern "C" int32_t ss_refracted_adjoint_blocks(int32_t n_facets) {
  return n_facets > 0 ? ss::refracted_adjoint_blocks(n_facets) : 0;
}

extern "C" size_t ss_refracted_adjoint_scratch_bytes(int32_t n_traces,
                                                     int32_t n_facets) {
  if (n_traces <= 0 || n_facets <= 0) return 0;
  return ss::refracted_adjoint_mask_bytes(n_traces, n_facets);
}

extern "C" int ss_refracted_adjoint(const ss_refracted_opts *opts,
                                    const ss_facets *target,
                                    const ss_traces *traces,
                                    const ss_pattern *pattern,
                                    const ss_roughness *rough,
                                    const ss_adjoint_io *io, void *stream) {
  using namespace ss;
  if (!io || !io->field || !io->grad_power || !io->grad_gamma_db ||
      !io->grad_alpha) {
    set_error("null adjoint argument");
    return SS_ERR_ARG;
  }
  Plan p;
  RefArgs a;
  int s = build_ref_args(opts, target, traces, pattern, rough, false, nullptr,
                         p, a);
  if (s) return s;
  if (io->bin_lo < 0 || io->bin_hi > a.n_seg || io->bin_lo >= io->bin_hi) {
    set_error("power window outside [0, n_samples)");
    return SS_ERR_ARG;
  }
  if (io->grad_sigma && !target->sigma) {
    set_error("sigma gradients need per-facet rms heights (facets->sigma)");
    return SS_ERR_ARG;
  }
  if (!io->scratch ||
      io->scratch_bytes < refracted_adjoint_mask_bytes(a.T, a.N)) {
    set_error("adjoint scratch buffer too small");
    return SS_ERR_SCRATCH;
  }
  AdjArgs j{io->field, io->grad_power, io->bin_lo, io->bin_hi,
            io->grad_gamma_db, io->grad_sigma, io->grad_alpha,
            static_cast<uint32_t *>(io->scratch)};
  return refracted_adjoint_launch(a, j, io->alpha_mask,
                                  static_cast<cudaStream_t>(stream));
}
