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
  // the same validation and argument block as ss_coherent_fwd
  Plan p;
  CoArgs a;
  int s = build_co_args(opts, facets, traces, pattern, rough, out, p, a);
  if (s) return s;
  const int T = traces->n_traces;
  // As many facet chunks as the fixed array holds (at most what
  // ss_coherent_fwd would use); one chunk must fit. coherent_launch takes
  // the chunk count from the plan, and every partial the reduction reads
  // is written by the main kernel first.
  const size_t elt = opts->precision == SS_PREC_FP64 ? 16 : 8;
  const size_t hist1 = (size_t)T * a.n_seg * elt;
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
  a.part = scratch;
  const size_t hist = ((size_t)p.n_chunks * hist1 + 255) & ~(size_t)255;
  a.part_drop = reinterpret_cast<double *>(static_cast<char *>(scratch) +
                                           hist);
  return coherent_launch(a, p, out, static_cast<cudaStream_t>(stream));
}
