// Surface coherent facet sum for callers that cannot allocate device memory.
//
// ss_coherent_fwd takes its scratch (the per-chunk partial histograms) from
// the caller. Some callers cannot provide it: a host application whose
// device memory is owned entirely by another allocator (a framework pool or
// a budget reserved at start-up), or a processing loop that must not
// allocate once it is running. ss_coherent_fwd_noalloc serves them from a
// fixed scratch array that lives in this library's device image instead.
//
// The array (SS_NOALLOC_SCRATCH_BYTES) is reserved on every GPU that loads
// the library and stays reserved until the process exits. Host code cannot
// use the array's name as a device address (on the host it only names a
// stand-in symbol), so the device address is looked up once per device with
// cudaGetSymbolAddress, with that device current, the first time the entry
// point is called on it; make that first call before any stream capture.
// Every call shares the one array and leaves its contents behind: calls that
// overlap on the GPU (other streams, other host threads) race on it. The
// main kernel overwrites every partial that the reduction later reads, so no
// part of the array has to be cleared between calls.
#include <mutex>

#include "ss_coherent.cuh"

namespace ss {

int coherent_launch(CoArgs &a, const Plan &p, const ss_output *out,
                    cudaStream_t st);

static __device__ __align__(256) unsigned char
    g_noalloc_scratch[SS_NOALLOC_SCRATCH_BYTES];

#define SS_NOALLOC_MAX_DEVICES 64
static void *g_noalloc_ptr[SS_NOALLOC_MAX_DEVICES];
static std::mutex g_noalloc_mu;

// Device address of the scratch array on the current device (looked up
// once per device).
static int noalloc_scratch(void **ptr) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_status(e, "cudaGetDevice");
  if (dev < 0 || dev >= SS_NOALLOC_MAX_DEVICES) {
    set_error("device ordinal beyond the no-alloc table");
    return SS_ERR_UNSUPPORTED;
  }
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress");
    g_noalloc_ptr[dev] = p;
  }
  *ptr = g_noalloc_ptr[dev];
  return SS_OK;
}

}  // namespace ss

extern "C" int ss_coherent_fwd_noalloc(const ss_coherent_opts *opts,
                                       const ss_facets *facets,
                                       const ss_traces *traces,
                                       const ss_pattern *pattern,
                                       const ss_roughness *rough,
                                       const ss_output *out, void *stream) {
  using namespace ss;
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
  Plan p;
  int s = coherent_plan(opts, T, N, &p);
  if (s) {
    set_error(s == SS_ERR_UNSUPPORTED ? "n_samples too large for the "
                                        "shared-memory histogram"
                                      : "bad sizes");
    return s;
  }
  // As many facet chunks as the fixed array holds (at most what
  // ss_coherent_fwd would use); one chunk must fit.
  const int n_seg = opts->n_samples * (opts->split_sides ? 2 : 1);
  const size_t elt = opts->precision == SS_PREC_FP64 ? 16 : 8;
  const size_t hist1 = (size_t)T * n_seg * elt;
  auto need = [&](int nc) {
    size_t h = ((size_t)nc * hist1 + 255) & ~(size_t)255;
    return h + (size_t)nc * T * sizeof(double);
  };
  if (need(1) > (size_t)SS_NOALLOC_SCRATCH_BYTES) {
    set_error("n_traces x n_samples too large for the fixed no-alloc "
              "scratch (SS_NOALLOC_SCRATCH_BYTES); use ss_coherent_fwd");
    return SS_ERR_SCRATCH;
  }
  while (p.n_chunks > 1 && need(p.n_chunks) > (size_t)SS_NOALLOC_SCRATCH_BYTES)
    --p.n_chunks;
  void *scratch = nullptr;
  s = noalloc_scratch(&scratch);
  if (s) return s;

  CoArgs a{};
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
  a.n_seg = n_seg;
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
  a.part = scratch;
  const size_t hist = ((size_t)p.n_chunks * hist1 + 255) & ~(size_t)255;
  a.part_drop = reinterpret_cast<double *>(static_cast<char *>(scratch) +
                                           hist);
  return coherent_launch(a, p, out, static_cast<cudaStream_t>(stream));
}
