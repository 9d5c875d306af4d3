// Per-trace output products over every facet (soundersim output.py:47-82):
// the nadir facet (horizontally nearest centre), nadir twtt, and the first
// return (earliest exact float64 twtt 2r/c inside the fast-time window).
//
// The reference forms a (T, N, 3) float64 array for each; here one pass
// streams the facets once per block of traces. GB300's float64 rate is
// 1/64 of its float32 rate, so every pair is first screened in float32
// (coordinates relative to a scene reference point; distances are then
// accurate to a few millimetres): a first pass finds each chunk's float32
// minima, and only pairs within 1e-3 relative plus 1 m^2 of them are
// evaluated in float64, in the reference's operation order. The
// minima are lexicographic in (value, facet index), so ties go to the
// first facet exactly as NumPy's argmin does, and a facet the screen lets
// through never changes a result it should not.
#include <algorithm>

#include "ss_internal.cuh"

namespace ss {

constexpr int kOutTB = 4;  // traces per CTA

struct Best {
  double v;
  long long i;
};

__device__ __forceinline__ bool better(double v, long long i, const Best &b) {
  return v < b.v || (v == b.v && i < b.i);
}

__device__ __forceinline__ void take(Best &a, const Best &b) {
  if (better(b.v, b.i, a)) a = b;
}

struct OutArgs {
  const double *cen;   // (N, 3) float64
  const float *rel;    // (N, 3) float32 centres minus the first centre
  const double *pos;   // (T, 3)
  int T, N, n_chunks;
  double t0, t_end, c;
  double A, B;         // squared ranges of the window's edges
  const unsigned *max_abs;  // largest |relative coordinate| (float bits)
  Best *part;          // (n_chunks, T, 2): nadir, first
};

// float32 centres relative to the first facet's centre (the screen's
// frame), and the largest |coordinate| there (bounds the screen's error)
__global__ void rel_centers_kernel(const double *cen, long n, float *rel,
                                   unsigned *max_abs) {
  float m = 0.f;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
       i += (long)gridDim.x * blockDim.x)
    for (int k = 0; k < 3; ++k) {
      const float v = (float)(cen[3 * i + k] - cen[k]);
      rel[3 * i + k] = v;
      m = fmaxf(m, fabsf(v));
    }
  for (int o = 16; o > 0; o >>= 1)
    m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(max_abs, __float_as_uint(m));
}

// Margin on a squared range x that covers the float32 screen's error on
// two values (a pair and the minimum it is compared with): a distance is
// off by at most e (below), so x by at most 2 e sqrt(x) + e^2, plus the
// float32 rounding of the sums (< 2e-7 x); twice that, plus 1e-3 m^2.
__device__ __forceinline__ float screen_margin(float x, float e) {
  return x * 1e-6f + 4.0f * e * sqrtf(x) + 4.0f * e * e + 1e-3f;
}

__global__ void __launch_bounds__(256) trace_scan_kernel(OutArgs a) {
  __shared__ Best s_red[kOutTB][2][8];
  const int tid = threadIdx.x;
  const int t0i = blockIdx.y * kOutTB;
  const int nt = min(kOutTB, a.T - t0i);
  double px[kOutTB], py[kOutTB], pz[kOutTB];
  float qx[kOutTB], qy[kOutTB], qz[kOutTB];
  Best nad[kOutTB], fst[kOutTB];
  float nad_f[kOutTB], fst_f[kOutTB];
  float Rmax = __uint_as_float(*a.max_abs);
#pragma unroll
  for (int t = 0; t < kOutTB; ++t) {
    const int ti = min(t0i + t, a.T - 1);
    px[t] = a.pos[3 * ti];
    py[t] = a.pos[3 * ti + 1];
    pz[t] = a.pos[3 * ti + 2];
    qx[t] = (float)(px[t] - a.cen[0]);
    qy[t] = (float)(py[t] - a.cen[1]);
    qz[t] = (float)(pz[t] - a.cen[2]);
    nad[t] = Best{INFINITY, (long long)1 << 62};
    fst[t] = Best{INFINITY, (long long)1 << 62};
    nad_f[t] = INFINITY;
    fst_f[t] = INFINITY;
    Rmax = fmaxf(Rmax, fmaxf(fabsf(qx[t]), fmaxf(fabsf(qy[t]), fabsf(qz[t]))));
  }
  // per component: rounding c and p to float32 (|v| 2^-24 each) and the
  // float32 difference (|d| <= 2R: 2R 2^-24) -> R 2^-22; times sqrt(3)
  const float e_r = 1.75f * Rmax * 2.3841858e-7f;
  // uncertain bands around the window's edges; inside [a_hi, b_lo] a pair
  // is surely in the window, outside [a_lo, b_hi] surely not
  const float Af = (float)a.A, Bf = (float)a.B;
  const float a_lo = Af - screen_margin(Af, e_r);
  const float a_hi = Af + screen_margin(Af, e_r);
  const float b_lo = Bf - screen_margin(Bf, e_r);
  const float b_hi = Bf + screen_margin(Bf, e_r);
  const long i0 = (long)a.N * blockIdx.x / a.n_chunks;
  const long i1 = (long)a.N * (blockIdx.x + 1) / a.n_chunks;
  // pass 1, float32 only: the chunk's approximate minima per trace
  for (long i = i0 + tid; i < i1; i += blockDim.x) {
    const float cx = a.rel[3 * i], cy = a.rel[3 * i + 1],
                cz = a.rel[3 * i + 2];
#pragma unroll
    for (int t = 0; t < kOutTB; ++t) {
      const float dx = cx - qx[t], dy = cy - qy[t], dz = cz - qz[t];
      const float h2 = dx * dx + dy * dy;
      const float r2 = h2 + dz * dz;
      nad_f[t] = fminf(nad_f[t], h2);
      if (r2 >= a_hi && r2 <= b_lo) fst_f[t] = fminf(fst_f[t], r2);
    }
  }
  __shared__ float s_thr[kOutTB][2];
  if (tid < kOutTB * 2) s_thr[tid >> 1][tid & 1] = INFINITY;
  __syncthreads();
#pragma unroll
  for (int t = 0; t < kOutTB; ++t) {
    float n = nad_f[t], f = fst_f[t];
    for (int o = 16; o > 0; o >>= 1) {
      n = fminf(n, __shfl_xor_sync(0xffffffffu, n, o));
      f = fminf(f, __shfl_xor_sync(0xffffffffu, f, o));
    }
    // non-negative floats order like their bit patterns
    if ((tid & 31) == 0) {
      atomicMin(reinterpret_cast<int *>(&s_thr[t][0]), __float_as_int(n));
      atomicMin(reinterpret_cast<int *>(&s_thr[t][1]), __float_as_int(f));
    }
  }
  __syncthreads();
  // thresholds: every pair whose float64 value can equal or beat the
  // chunk's minimum lies within twice the screen's error of the float32
  // minimum (for the first return: of the minimum over pairs surely in the
  // window; pairs in the uncertain bands are always evaluated)
#pragma unroll
  for (int t = 0; t < kOutTB; ++t) {
    const float n = s_thr[t][0], f = s_thr[t][1];
    nad_f[t] = n + screen_margin(n, e_r);
    fst_f[t] = f + screen_margin(f, e_r);
  }
  // pass 2: float64 for the few pairs at the minima
  for (long i = i0 + tid; i < i1; i += blockDim.x) {
    const float cx = a.rel[3 * i], cy = a.rel[3 * i + 1],
                cz = a.rel[3 * i + 2];
#pragma unroll
    for (int t = 0; t < kOutTB; ++t) {
      const float dx = cx - qx[t], dy = cy - qy[t], dz = cz - qz[t];
      const float h2 = dx * dx + dy * dy;
      const float r2 = h2 + dz * dz;
      const bool cand_n = h2 <= nad_f[t];
      const bool cand_f =
          r2 >= a_lo && r2 <= b_hi && (r2 <= fst_f[t] || r2 < a_hi);
      if (!(cand_n || cand_f)) continue;
      // float64 in the reference's order: d = c - p, squares, sums
      const double ex = __dsub_rn(a.cen[3 * i], px[t]);
      const double ey = __dsub_rn(a.cen[3 * i + 1], py[t]);
      const double ez = __dsub_rn(a.cen[3 * i + 2], pz[t]);
      const double hh = __dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey));
      if (cand_n && better(hh, i, nad[t])) nad[t] = Best{hh, i};
      if (cand_f) {
        const double r = __dsqrt_rn(__dadd_rn(hh, __dmul_rn(ez, ez)));
        const double ft = __ddiv_rn(__dmul_rn(2.0, r), a.c);
        if (ft >= a.t0 && ft < a.t_end && better(ft, i, fst[t]))
          fst[t] = Best{ft, i};
      }
    }
  }
  // warp then block reduction, lexicographic in (value, index)
  const int lane = tid & 31, warp = tid >> 5;
#pragma unroll
  for (int t = 0; t < kOutTB; ++t) {
    for (int k = 0; k < 2; ++k) {
      Best b = k == 0 ? nad[t] : fst[t];
      for (int o = 16; o > 0; o >>= 1) {
        Best q;
        q.v = __shfl_down_sync(0xffffffffu, b.v, o);
        q.i = __shfl_down_sync(0xffffffffu, b.i, o);
        take(b, q);
      }
      if (lane == 0) s_red[t][k][warp] = b;
    }
  }
  __syncthreads();
  if (tid < nt * 2) {
    const int t = tid >> 1, k = tid & 1;
    Best b = s_red[t][k][0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) take(b, s_red[t][k][w]);
    a.part[((size_t)blockIdx.x * a.T + t0i + t) * 2 + k] = b;
  }
}

__global__ void trace_finish_kernel(OutArgs a, ss_trace_products_out o) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= a.T) return;
  Best n = a.part[(size_t)t * 2], f = a.part[(size_t)t * 2 + 1];
  for (int ch = 1; ch < a.n_chunks; ++ch) {
    take(n, a.part[((size_t)ch * a.T + t) * 2]);
    take(f, a.part[((size_t)ch * a.T + t) * 2 + 1]);
  }
  const long long ni = n.i < a.N ? n.i : 0;
  if (o.nadir_index) o.nadir_index[t] = ni;
  if (o.nadir_twtt)  // 2 (z_platform - z_facet) / c (output.py:71-72)
    o.nadir_twtt[t] = __ddiv_rn(
        __dmul_rn(2.0, __dsub_rn(a.pos[3 * t + 2], a.cen[3 * ni + 2])), a.c);
  const bool any = f.i < a.N;
  if (o.first_index) o.first_index[t] = any ? f.i : 0;
  if (o.first_twtt) o.first_twtt[t] = any ? f.v : INFINITY;
}

}  // namespace ss

using namespace ss;

static int out_chunks(int T, int N) {
  const int groups = (T + kOutTB - 1) / kOutTB;
  const long target = 8L * sm_count();
  long nc = (target + groups - 1) / groups;
  nc = std::min(nc, std::max(1L, (long)N / 4096));
  return (int)std::max(1L, nc);
}

extern "C" size_t ss_trace_products_scratch_bytes(int32_t n_traces,
                                                  int32_t n_facets) {
  if (n_traces <= 0 || n_facets <= 0) return 0;
  const size_t rel = ((size_t)n_facets * 3 * sizeof(float) + 255) & ~255ul;
  return rel + 256 + (size_t)out_chunks(n_traces, n_facets) * n_traces * 2 *
                         sizeof(Best);
}

extern "C" int ss_trace_products(const ss_trace_products_opts *opts,
                                 const double *centers, int32_t n_facets,
                                 const double *positions, int32_t n_traces,
                                 const ss_trace_products_out *out,
                                 void *scratch, size_t scratch_bytes,
                                 void *stream) {
  if (!opts || !centers || !positions || !out || n_traces <= 0 ||
      n_facets <= 0 || !(opts->c > 0.0) || !(opts->dt > 0.0)) {
    set_error("ss_trace_products: bad argument");
    return SS_ERR_ARG;
  }
  const size_t need = ss_trace_products_scratch_bytes(n_traces, n_facets);
  if (!scratch || scratch_bytes < need) {
    set_error("ss_trace_products: scratch too small");
    return SS_ERR_SCRATCH;
  }
  OutArgs a{};
  a.cen = centers;
  a.rel = reinterpret_cast<const float *>(scratch);
  a.pos = positions;
  a.T = n_traces;
  a.N = n_facets;
  a.n_chunks = out_chunks(n_traces, n_facets);
  a.t0 = opts->t0;
  a.t_end = opts->t0 + opts->n_samples * opts->dt;  // output.py:79
  a.c = opts->c;
  const double ra = 0.5 * opts->c * opts->t0, rb = 0.5 * opts->c * a.t_end;
  a.A = ra > 0 ? ra * ra : 0.0;
  a.B = rb > 0 ? rb * rb : 0.0;
  const size_t rel = ((size_t)n_facets * 3 * sizeof(float) + 255) & ~255ul;
  unsigned *max_abs = reinterpret_cast<unsigned *>(
      reinterpret_cast<char *>(scratch) + rel);
  a.max_abs = max_abs;
  a.part = reinterpret_cast<Best *>(reinterpret_cast<char *>(scratch) + rel +
                                    256);
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  int e0 = cuda_status(cudaMemsetAsync(max_abs, 0, sizeof(unsigned), st),
                       "trace products memset");
  if (e0 != SS_OK) return e0;
  rel_centers_kernel<<<(int)std::min<long>((n_facets + 255) / 256,
                                           16L * sm_count()),
                       256, 0, st>>>(centers, n_facets,
                                     reinterpret_cast<float *>(scratch),
                                     max_abs);
  e0 = cuda_status(cudaGetLastError(), "relative centres launch");
  if (e0 != SS_OK) return e0;
  dim3 grid(a.n_chunks, (n_traces + kOutTB - 1) / kOutTB);
  trace_scan_kernel<<<grid, 256, 0, st>>>(a);
  int e = cuda_status(cudaGetLastError(), "trace scan launch");
  if (e != SS_OK) return e;
  trace_finish_kernel<<<(n_traces + 255) / 256, 256, 0, st>>>(a, *out);
  return cuda_status(cudaGetLastError(), "trace finish launch");
}
