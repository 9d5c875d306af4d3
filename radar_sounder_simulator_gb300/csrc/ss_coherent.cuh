// Surface coherent kernel: argument block and launch helpers (internal).
#pragma once

#include "ss_internal.cuh"

namespace ss {

struct CoArgs {
  ss_facets F;
  const double *pos, *uct, *pv;
  const int32_t *off;
  int T, N, pv_len;
  double k, gamma, t0, dt, c, taper_s;
  int n_samples, n_seg, bs, n_win, split, interp, taper, precision;
  int pat_kind, pat_n;
  const double *pa, *pb;
  int rough_kind, n_terms;
  double sigma, corr;
  FadCoeffs fad;
  int tb, n_chunks;
  void *part;          // (n_chunks, T, n_seg) complex partial histograms
  double *part_drop;   // (n_chunks, T) partial dropped power
};

int coherent_plan(const ss_coherent_opts *o, int T, int N, Plan *p,
                  bool rough);
size_t coherent_scratch(const ss_coherent_opts *o, int T, int N);
int coherent_split_launch(CoArgs &a, const Plan &p, cudaStream_t st);
int build_co_args(const ss_coherent_opts *opts, const ss_facets *facets,
                  const ss_traces *traces, const ss_pattern *pattern,
                  const ss_roughness *rough, const ss_output *out, Plan &p,
                  CoArgs &a);

// Shared-memory histograms of the split coherent kernel: planar real and
// imaginary planes of `tb` traces each, a trace's row padded to n_seg + 11
// floats so the block's traces start 11 banks apart (neighbouring facets
// of a warp, spread over the traces, then rarely meet in one bank).
__host__ __device__ __forceinline__ int split_hist_stride(int n_seg) {
  return n_seg + 11;
}
__host__ __device__ __forceinline__ size_t split_hist_bytes(int n_seg,
                                                            int tb) {
  return (size_t)2 * tb * split_hist_stride(n_seg) * sizeof(float);
}

// float32 / double-float constants of the split coherent kernel.
struct SplitConsts {
  float k, amp_pref, gamma, taper_inv;  // taper_inv = 1 / (2 s^2)
  float K2h, K2l;                       // 2k as double-float
  float Ah, Al, Bh, Bl;                 // u = r A - B, A = 2/(c dt), B = t0/dt
  float fadL;
  float sigma, corr;
};
SplitConsts coherent_split_consts(const CoArgs &a);

// One job of a batched launch: its arguments, split constants, the range of
// work items and reduce elements it owns, and its output.
struct BatchJob {
  CoArgs a;
  SplitConsts k;
  long long item0;  // first work item (trace block x facet chunk)
  long long out0;   // first reduce element (trace x segment)
  int n_chunks, n_groups;
  ss_output out;
};

// Persistent work-queue kernels over a device job table: `ctas` CTAs pull
// items from `counter` (zeroed by the caller) until n_items are done.
int coherent_batch_split_launch(const BatchJob *jobs, int n_jobs,
                                long long n_items,
                                unsigned long long *counter, int rough_kind,
                                int threads, int ctas, size_t smem,
                                cudaStream_t st);
int coherent_batch_fp64_launch(const BatchJob *jobs, int n_jobs,
                               long long n_items, unsigned long long *counter,
                               int threads, int ctas, size_t smem,
                               cudaStream_t st);
int batch_split_blocks_per_sm(int rough_kind, int threads, size_t smem);
int batch_fp64_blocks_per_sm(int threads, size_t smem);
// Ordered chunk reduction of every job's partials into its output.
int batch_reduce_launch(const BatchJob *jobs, int n_jobs, long long n_out,
                        bool f64_parts, cudaStream_t st);

// Index of the job owning position `x` of a prefix array (first[j] <= x).
__device__ __forceinline__ int batch_find_job(const BatchJob *jobs,
                                              int n_jobs, long long x,
                                              bool by_item) {
  int lo = 0, hi = n_jobs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    const long long f = by_item ? jobs[mid].item0 : jobs[mid].out0;
    if (f <= x) lo = mid; else hi = mid - 1;
  }
  return lo;
}

}  // namespace ss
