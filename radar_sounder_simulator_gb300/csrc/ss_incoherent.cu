// Incoherent (power-summing) facet kernel on GB300.
//
// Replaces the jitted program of soundersim kernels/incoherent.py:32-61:
// per facet and trace the power (A cos)^2 / r^4 (weighted g^4 by the antenna
// pattern), binned at floor((2r/c - t0)/dt), out-of-window power dropped into
// a per-trace scalar, optionally split into left/right halves by the sign of
// (c - p) . u_ct. Every facet is summed for every trace (the reference has no
// culling here).
//
// Everything is float32 like the reference. The bin is an integer decision
// that must match the reference's float32 chain
//   r = sqrt((dx^2 + dy^2) + dz^2), tw = (2 r) / c, u = (tw - t0) / dt
// bit for bit, with each operation rounded to nearest. The kernel evaluates
// it first as r A - B from a MUFU reciprocal square root, with an error
// bound; only pairs whose fast value lies within that bound of an integer
// re-run the exactly rounded chain (__fsqrt_rn / __fdiv_rn), so the bins
// equal the reference's while the common case costs a few instructions.
//
// Work decomposition: the grid is (facet chunks) x (trace blocks of TB
// traces). Each thread takes one facet at a time and evaluates it against
// the TB traces of its block, lane l starting at trace (l + s) mod TB on step
// s, so the 32 lanes of a warp -- 32 neighbouring facets, often in the same
// bin -- spread their shared-memory atomics over TB histograms instead of
// piling onto one address. Dropped power stays in registers (each step s
// maps a thread to one fixed trace). Per-CTA histograms go to scratch and a
// second kernel sums the chunks in a fixed order in float64.
#include <algorithm>

#include "ss_chunksum.cuh"
#include "ss_f32.cuh"
#include "ss_internal.cuh"

namespace ss {

struct IncArgs {
  const float *cx, *cy, *cz, *nx, *ny, *nz, *area;
  const double *pos, *uct, *pv;
  int pv_len, T, N, n_samples, n_seg, stride, split;
  float t0, dt, c;  // window scalars rounded to float32
  float A, B, bandA;  // 2/(c dt), t0/dt, 1e-6 A of those float32 scalars
  int pat_kind, pat_n;
  const double *pa, *pb;
  int n_chunks;
  float *part;        // (n_chunks, T, n_seg) partial histograms
  double *part_drop;  // (n_chunks, T) partial dropped power
};

// Exactly rounded float32 bin chain of the reference (geometry.py:6-24).
__device__ __forceinline__ float bin_exact(float S, const IncArgs &a) {
  const float r = __fsqrt_rn(S);
  const float tw = __fdiv_rn(__fmul_rn(2.0f, r), a.c);
  return floorf(__fdiv_rn(__fsub_rn(tw, a.t0), a.dt));
}

template <int TB, bool PAT>
__global__ void __launch_bounds__(256)
incoherent_kernel(IncArgs a) {
  extern __shared__ __align__(16) float hist[];  // (TB, stride)
  __shared__ float4 s_p[TB], s_u[TB];
  __shared__ float s_pv[TB][6];
  __shared__ float s_pat[SS_PAT_MAX];
  __shared__ float s_drop[TB];

  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int t_base = blockIdx.y * TB;
  const int nt = min(TB, a.T - t_base);
  int pa_len = 0, pb_len = 0;
  if (PAT) pattern_lengths(a.pat_kind, a.pat_n, pa_len, pb_len);

  if (tid < TB) {
    // missing traces of a short last block get NaN positions: their pairs
    // fail every comparison, bin nowhere and their dropped sums are unused
    float4 p = make_float4(__int_as_float(0x7fc00000), 0.f, 0.f, 0.f);
    float4 u = make_float4(0.f, 0.f, 0.f, 0.f);
    if (tid < nt) {
      const int t = t_base + tid;
      // positions and u_ct rounded to float32 (incoherent.py:86-87)
      p = make_float4((float)a.pos[3 * t], (float)a.pos[3 * t + 1],
                      (float)a.pos[3 * t + 2], 0.f);
      if (a.uct)
        u = make_float4((float)a.uct[3 * t], (float)a.uct[3 * t + 1],
                        (float)a.uct[3 * t + 2], 0.f);
      for (int j = 0; j < 6; ++j)
        s_pv[tid][j] =
            (PAT && a.pv && j < a.pv_len) ? (float)a.pv[a.pv_len * t + j]
                                          : 0.f;
    }
    s_p[tid] = p;
    s_u[tid] = u;
    s_drop[tid] = 0.f;
  }
  if (PAT) {
    for (int j = tid; j < pa_len; j += blockDim.x) s_pat[j] = (float)a.pa[j];
    for (int j = tid; j < pb_len; j += blockDim.x)
      s_pat[pa_len + j] = (float)a.pb[j];
  }
  for (int j = tid; j < TB * a.stride; j += blockDim.x) hist[j] = 0.f;
  __syncthreads();

  // step s always pairs this thread with trace (lane + s) mod TB: its
  // position, histogram row and dropped sum live in registers
  float px[TB], py[TB], pz[TB], drop[TB];
  int hoff[TB];
#pragma unroll
  for (int s = 0; s < TB; ++s) {
    const int tt = (lane + s) & (TB - 1);
    const float4 P = s_p[tt];
    px[s] = P.x;
    py[s] = P.y;
    pz[s] = P.z;
    hoff[s] = tt * a.stride;
    drop[s] = 0.f;
  }

  const long len = a.N;
  const int i0 = (int)(len * blockIdx.x / a.n_chunks);
  const int i1 = (int)(len * (blockIdx.x + 1) / a.n_chunks);
  const float nsf = (float)a.n_samples;

  for (int i = i0 + tid; i < i1; i += blockDim.x) {
    const float cx = a.cx[i], cy = a.cy[i], cz = a.cz[i];
    const float nx = a.nx[i], ny = a.ny[i], nz = a.nz[i];
    const float ar = a.area[i];
#pragma unroll
    for (int s = 0; s < TB; ++s) {
      const float dx = __fsub_rn(px[s], cx);
      const float dy = __fsub_rn(py[s], cy);
      const float dz = __fsub_rn(pz[s], cz);
      const float S = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx),
                                          __fmul_rn(dy, dy)),
                                __fmul_rn(dz, dz));
      const float y = rsqrtf(S);  // 1/r
      // power (A cos)^2 / r^4 = (A (d . n))^2 / r^6
      const float q = ar * dot3f(dx, dy, dz, nx, ny, nz);
      const float y2 = y * y;
      float pw = (q * q) * (y2 * y2 * y2);
      if (PAT) {
        // departure direction antenna -> facet (incoherent.py:45)
        const int tt = (lane + s) & (TB - 1);
        const float g = gain32(a.pat_kind, a.pat_n, pa_len, s_pat, s_pv[tt],
                               -dx * y, -dy * y, -dz * y);
        const float g2 = g * g;
        pw *= g2 * g2;
      }
      // fast bin u ~ r A - B (A = 2/(c dt), B = t0/dt) and its error bound
      // |uf - u| <= 4.8e-7 r A + 2.4e-7 |u| (rsqrt 2 ulp, A, B and the
      // roundings of both chains); the band doubles that. A pair the bound
      // cannot settle takes the exact chain; a band of half a bin or more
      // sends every pair there.
      const float rf = S * y;
      const float uf = __fmaf_rn(rf, a.A, -a.B);
      float fb = floorf(uf);
      const float fr = uf - fb;
      const float band =
          __fmaf_rn(a.bandA, rf, __fmaf_rn(7e-7f, fabsf(uf), 1e-6f));
      if (fminf(fr, 1.0f - fr) < band) fb = bin_exact(S, a);
      if (fb >= 0.0f && fb < nsf) {
        int seg = (int)fb;
        if (a.split) {
          const float4 U = s_u[(lane + s) & (TB - 1)];
          // (c - p) . u_ct, rounded like the reference's sum
          const float sd = __fadd_rn(__fadd_rn(__fmul_rn(-dx, U.x),
                                               __fmul_rn(-dy, U.y)),
                                     __fmul_rn(-dz, U.z));
          if (sd > 0.0f) seg += a.n_samples;
        }
        atomicAdd(&hist[hoff[s] + seg], pw);
      } else {
        drop[s] += pw;
      }
    }
  }
#pragma unroll
  for (int s = 0; s < TB; ++s) {
    const int tt = (lane + s) & (TB - 1);
    if (tt < nt) atomicAdd(&s_drop[tt], drop[s]);
  }
  __syncthreads();
  for (int tt = 0; tt < nt; ++tt) {
    float *dst = a.part + ((size_t)blockIdx.x * a.T + t_base + tt) * a.n_seg;
    for (int j = tid; j < a.n_seg; j += blockDim.x)
      dst[j] = hist[tt * a.stride + j];
  }
  if (tid < nt)
    a.part_drop[(size_t)blockIdx.x * a.T + t_base + tid] = (double)s_drop[tid];
}

// Chunk sums (compensated float32, ~2^-48 relative), in chunk order, into
// the (T, n[, 2]) float32 layout.
__global__ void incoherent_reduce_kernel(const float *part,
                                         const double *part_drop, int T,
                                         int n_seg, int n_samples, int split,
                                         int n_chunks,
                                         ss_incoherent_output out) {
  const long total = (long)T * n_seg;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total;
       e += (long)gridDim.x * blockDim.x) {
    const int t = (int)(e / n_seg);
    const int b = (int)(e % n_seg);
    ChunkSum<float> cs;
    for (int c = 0; c < n_chunks; ++c)
      cs.add(part[((size_t)c * T + t) * n_seg + b]);
    const double s = cs.value();
    long o = e;
    if (split) {  // (T, 2, n) -> (T, n, 2) [left, right]
      const int side = b / n_samples, bl = b % n_samples;
      o = ((long)t * n_samples + bl) * 2 + side;
    }
    out.power[o] = (float)s;
    if (b == 0) {
      double d = 0.0;
      for (int c = 0; c < n_chunks; ++c) d += part_drop[(size_t)c * T + t];
      out.dropped[t] = (float)d;
    }
  }
}

namespace {

struct IncPlan {
  int tb, n_groups, n_chunks, stride;
  size_t smem;
};

constexpr size_t kIncSmemBudget = 100 * 1024;  // two CTAs per SM
constexpr size_t kIncSmemMax = 200 * 1024;

int inc_plan(const ss_incoherent_opts *o, int T, int N, IncPlan *p) {
  if (!o || T <= 0 || N <= 0 || o->n_samples <= 0) return SS_ERR_ARG;
  const int n_seg = o->n_samples * (o->split_sides ? 2 : 1);
  p->stride = n_seg | 1;  // odd: traces' equal bins fall in distinct banks
  const size_t row = (size_t)p->stride * sizeof(float);
  int tb = 8;
  while (tb > 1 && tb * row > kIncSmemBudget) tb >>= 1;
  if (tb * row > kIncSmemMax) return SS_ERR_UNSUPPORTED;
  p->tb = tb;
  p->smem = tb * row;
  p->n_groups = (T + tb - 1) / tb;
  // about eight CTAs per SM in total, each chunk at least 2048 facets and
  // enough pairs to amortise zeroing and writing its histograms
  const int sms = sm_count();
  const long target = 8L * sms;
  long nc = (target + p->n_groups - 1) / p->n_groups;
  nc = std::min(nc, std::max(1L, (long)N / 2048));
  nc = std::min(nc, std::max(1L, (long)N * tb / (4L * n_seg)));
  p->n_chunks = (int)std::max(1L, nc);
  return SS_OK;
}

template <int TB, bool PAT>
int inc_launch_t(const IncArgs &a, const IncPlan &p, cudaStream_t st) {
  cudaError_t e = cudaFuncSetAttribute(
      incoherent_kernel<TB, PAT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
      (int)p.smem);
  if (e != cudaSuccess) return cuda_status(e, "incoherent smem");
  dim3 grid(p.n_chunks, p.n_groups);
  incoherent_kernel<TB, PAT><<<grid, 256, p.smem, st>>>(a);
  return cuda_status(cudaGetLastError(), "incoherent launch");
}

template <bool PAT>
int inc_launch_p(const IncArgs &a, const IncPlan &p, cudaStream_t st) {
  switch (p.tb) {
    case 8: return inc_launch_t<8, PAT>(a, p, st);
    case 4: return inc_launch_t<4, PAT>(a, p, st);
    case 2: return inc_launch_t<2, PAT>(a, p, st);
    default: return inc_launch_t<1, PAT>(a, p, st);
  }
}

}  // namespace
}  // namespace ss

using namespace ss;

extern "C" size_t ss_incoherent_scratch_bytes(const ss_incoherent_opts *opts,
                                              int32_t n_traces,
                                              int32_t n_facets) {
  IncPlan p;
  if (inc_plan(opts, n_traces, n_facets, &p) != SS_OK) return 0;
  const size_t n_seg = (size_t)opts->n_samples * (opts->split_sides ? 2 : 1);
  const size_t part = (size_t)p.n_chunks * n_traces * n_seg * sizeof(float);
  const size_t drop = (size_t)p.n_chunks * n_traces * sizeof(double);
  return ((part + 255) & ~(size_t)255) + drop;
}

extern "C" int ss_incoherent_fwd(const ss_incoherent_opts *opts,
                                 const ss_facets *facets,
                                 const ss_traces *traces,
                                 const ss_pattern *pattern,
                                 const ss_incoherent_output *out,
                                 void *scratch, size_t scratch_bytes,
                                 void *stream) {
  if (!opts || !facets || !traces || !out || !out->power || !out->dropped) {
    set_error("ss_incoherent_fwd: null argument");
    return SS_ERR_ARG;
  }
  const int T = traces->n_traces, N = facets->n_facets;
  if (!traces->pos || !facets->cx || !facets->cy || !facets->cz ||
      !facets->nx || !facets->ny || !facets->nz || !facets->area ||
      (opts->split_sides && !traces->uct) || !(opts->dt > 0.0) ||
      !(opts->c > 0.0)) {
    set_error("ss_incoherent_fwd: missing input array or bad window");
    return SS_ERR_ARG;
  }
  IncPlan p;
  int st = inc_plan(opts, T, N, &p);
  if (st != SS_OK) {
    set_error(st == SS_ERR_UNSUPPORTED
                  ? "ss_incoherent_fwd: n_samples beyond shared memory"
                  : "ss_incoherent_fwd: bad sizes");
    return st;
  }
  const size_t need = ss_incoherent_scratch_bytes(opts, T, N);
  if (!scratch || scratch_bytes < need) {
    set_error("ss_incoherent_fwd: scratch too small");
    return SS_ERR_SCRATCH;
  }
  const int kind = pattern ? pattern->kind : SS_PAT_ISOTROPIC;
  if (kind != SS_PAT_ISOTROPIC) {
    int pa_len, pb_len;
    pattern_lengths(kind, pattern->n, pa_len, pb_len);
    if (pa_len + pb_len > SS_PAT_MAX) {
      set_error("ss_incoherent_fwd: antenna table too large");
      return SS_ERR_UNSUPPORTED;
    }
    if (!traces->pv || ((pa_len && !pattern->pa) || (pb_len && !pattern->pb))) {
      set_error("ss_incoherent_fwd: pattern arrays missing");
      return SS_ERR_ARG;
    }
  }
  IncArgs a{};
  a.cx = facets->cx; a.cy = facets->cy; a.cz = facets->cz;
  a.nx = facets->nx; a.ny = facets->ny; a.nz = facets->nz;
  a.area = facets->area;
  a.pos = traces->pos;
  a.uct = traces->uct;
  a.pv = traces->pv;
  a.pv_len = traces->pv_len;
  a.T = T;
  a.N = N;
  a.n_samples = opts->n_samples;
  a.n_seg = opts->n_samples * (opts->split_sides ? 2 : 1);
  a.stride = p.stride;
  a.split = opts->split_sides ? 1 : 0;
  // window scalars rounded to float32 (incoherent.py:101-102)
  a.t0 = (float)opts->t0;
  a.dt = (float)opts->dt;
  a.c = (float)opts->c;
  a.A = (float)(2.0 / ((double)a.c * (double)a.dt));
  a.B = (float)((double)a.t0 / (double)a.dt);
  a.bandA = 1e-6f * a.A;
  a.pat_kind = kind;
  a.pat_n = pattern ? pattern->n : 0;
  a.pa = pattern ? pattern->pa : nullptr;
  a.pb = pattern ? pattern->pb : nullptr;
  a.n_chunks = p.n_chunks;
  const size_t n_seg = (size_t)a.n_seg;
  const size_t part_bytes = (size_t)p.n_chunks * T * n_seg * sizeof(float);
  a.part = reinterpret_cast<float *>(scratch);
  a.part_drop = reinterpret_cast<double *>(
      reinterpret_cast<char *>(scratch) + ((part_bytes + 255) & ~(size_t)255));
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  st = kind != SS_PAT_ISOTROPIC ? inc_launch_p<true>(a, p, s)
                                : inc_launch_p<false>(a, p, s);
  if (st != SS_OK) return st;
  incoherent_reduce_kernel<<<4 * sm_count(), 256, 0, s>>>(
      a.part, a.part_drop, T, a.n_seg, a.n_samples, a.split, p.n_chunks,
      *out);
  return cuda_status(cudaGetLastError(), "incoherent reduce launch");
}
