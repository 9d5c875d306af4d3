// Batched surface coherent facet sums in one persistent launch.
//
// Many independent jobs -- instances of a design sweep with their own
// scene, track, frequency and antenna, whose culled facet counts per trace
// differ by an order of magnitude or more -- are cut into work items of
// about equal size (trace block x facet chunk, the one-call kernel's CTA
// unit, with each job's chunk count scaled to its window length) and served
// from one global queue by a persistent grid, so no job's tail idles the
// GPU. A batched reduce then writes every job's output.
//
// prepare: validates every job, lays out the caller's scratch (queue
//   counter, job table, per-job partials), uploads the job table (the one
//   host-to-device copy, synchronous) and raises the kernels' shared-memory
//   limit;
// run: zero the counter, persistent kernel, batched reduce -- stream
//   operations only, so a caller can capture run() in a CUDA graph and
//   replay it.
#include <algorithm>
#include <cstring>
#include <vector>

#include "ss_coherent.cuh"

namespace ss {

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

struct BatchLayout {
  std::vector<BatchJob> jobs;
  size_t table_off = 256, bytes = 0, smem = 0;
  long long n_items = 0, n_out = 0;
  int precision = 0, rough_kind = 0, threads = 256;
};

static int batch_layout(const ss_coherent_job *jobs, int n_jobs,
                        const ss_batch_tuning *tune, BatchLayout &L) {
  if (!jobs || n_jobs <= 0) {
    set_error("empty batch");
    return SS_ERR_ARG;
  }
  const int threads = tune && tune->threads ? tune->threads : 256;
  if (threads != 128 && threads != 256 && threads != 512) {
    set_error("batch threads must be 128, 256 or 512");
    return SS_ERR_ARG;
  }
  const int max_tb = tune && tune->max_tb ? tune->max_tb : SS_MAX_TB;
  if (max_tb < 1 || max_tb > SS_MAX_TB) {
    set_error("batch max_tb must be in 1..8");
    return SS_ERR_ARG;
  }
  const int ips = tune && tune->items_per_sm ? tune->items_per_sm : 16;
  if (ips < 1) {
    set_error("batch items_per_sm must be positive");
    return SS_ERR_ARG;
  }
  L.jobs.assign(n_jobs, BatchJob{});
  L.threads = threads;
  double total_pairs = 0.0;
  std::vector<long> window(n_jobs);
  for (int j = 0; j < n_jobs; ++j) {
    const ss_coherent_job &q = jobs[j];
    Plan p;
    int s = build_co_args(&q.opts, &q.facets, &q.traces, &q.pattern,
                          &q.rough, &q.out, p, L.jobs[j].a);
    if (s) return s;
    CoArgs &a = L.jobs[j].a;
    if (j == 0) {
      L.precision = a.precision;
      L.rough_kind = a.rough_kind;
    } else if (a.precision != L.precision || a.rough_kind != L.rough_kind) {
      set_error("all jobs of a batch need the same precision and roughness "
                "kind");
      return SS_ERR_ARG;
    }
    if (threads == 512 &&
        (a.precision == SS_PREC_FP64 || a.rough_kind != SS_ROUGH_NONE)) {
      set_error("512-thread batches take smooth split-precision jobs only");
      return SS_ERR_ARG;
    }
    // histogram budget as the one-call plan: rough split jobs (80
    // registers, three 256-thread CTAs per SM) 48 KB, so three CTAs fit
    const size_t elt = a.precision == SS_PREC_FP64 ? 16 : 8;
    const size_t budget =
        a.precision == SS_PREC_FP64
            ? 96 * 1024
            : (a.rough_kind != SS_ROUGH_NONE ? 48 * 1024 : 100 * 1024);
    const size_t per_trace = (size_t)a.n_seg * elt;
    a.tb = (int)std::min<size_t>(
        std::max<size_t>(1, std::min<size_t>(budget / per_trace, max_tb)),
        (size_t)a.T);
    L.jobs[j].n_groups = (a.T + a.tb - 1) / a.tb;
    window[j] = std::min<long>((long)a.n_win * a.bs, a.N);
    total_pairs += (double)a.T * window[j];
  }
  // equal-work items: pairs per item ~ total / (items_per_sm x SMs)
  const double per_item =
      std::max(1.0, total_pairs / ((double)ips * sm_count()));
  // the costliest jobs' items first (longest-processing-time order): a
  // pair's cost grows with the job's series length, and a queue that ends
  // on the cheapest items leaves the persistent grid a short tail; each
  // job keeps its own outputs, so the table order is free
  std::vector<int> order(n_jobs);
  for (int j = 0; j < n_jobs; ++j) order[j] = j;
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
    return L.jobs[x].a.n_terms > L.jobs[y].a.n_terms;
  });
  {
    std::vector<BatchJob> sorted(n_jobs);
    std::vector<long> win(n_jobs);
    for (int r = 0; r < n_jobs; ++r) {
      sorted[r] = L.jobs[order[r]];
      win[r] = window[order[r]];
    }
    L.jobs.swap(sorted);
    window.swap(win);
  }
  size_t off = L.table_off + align256(sizeof(BatchJob) * n_jobs);
  long long item = 0, out = 0;
  for (int j = 0; j < n_jobs; ++j) {
    BatchJob &J = L.jobs[j];
    CoArgs &a = J.a;
    const double item_pairs = (double)window[j] * a.tb;
    const long max_chunks = std::max<long>(1, window[j] / 64);
    J.n_chunks = (int)std::min<long>(
        max_chunks, std::max<long>(1, (long)(item_pairs / per_item + 0.5)));
    a.n_chunks = J.n_chunks;
    J.item0 = item;
    J.out0 = out;
    item += (long long)J.n_chunks * J.n_groups;
    out += (long long)a.T * a.n_seg;
    J.k = coherent_split_consts(a);
    J.out = jobs[order[j]].out;
    const size_t elt = a.precision == SS_PREC_FP64 ? 16 : 8;
    a.part = reinterpret_cast<void *>(off);  // offset until prepare
    off += align256((size_t)J.n_chunks * a.T * a.n_seg * elt);
    a.part_drop = reinterpret_cast<double *>(off);
    off += align256((size_t)J.n_chunks * a.T * sizeof(double));
    // the series table: log-factorials (FP64 kernel, doubles) or 1/m
    // (split kernel, floats)
    const size_t lg = a.rough_kind ? (size_t)(a.n_terms + 1) *
                                         (a.precision == SS_PREC_FP64 ? 8 : 4)
                                   : 0;
    const size_t hist = a.precision == SS_PREC_FP64
                            ? (size_t)a.tb * a.n_seg * elt
                            : split_hist_bytes(a.n_seg, a.tb);
    L.smem = std::max(L.smem, hist + lg);
  }
  L.n_items = item;
  L.n_out = out;
  L.bytes = off;
  if (L.smem > 200 * 1024) {
    set_error("a job's shared-memory histogram exceeds 200 KB");
    return SS_ERR_UNSUPPORTED;
  }
  return SS_OK;
}

}  // namespace ss

extern "C" size_t ss_coherent_batch_scratch_bytes(
    const ss_coherent_job *jobs, int32_t n_jobs,
    const ss_batch_tuning *tune) {
  ss::BatchLayout L;
  if (ss::batch_layout(jobs, n_jobs, tune, L) != SS_OK) return 0;
  return L.bytes;
}

extern "C" int ss_coherent_batch_prepare(const ss_coherent_job *jobs,
                                         int32_t n_jobs,
                                         const ss_batch_tuning *tune,
                                         void *scratch, size_t scratch_bytes,
                                         ss_batch_info *info) {
  using namespace ss;
  if (!info) {
    set_error("null info");
    return SS_ERR_ARG;
  }
  BatchLayout L;
  int s = batch_layout(jobs, n_jobs, tune, L);
  if (s) return s;
  if (!scratch || scratch_bytes < L.bytes) {
    set_error("scratch buffer too small");
    return SS_ERR_SCRATCH;
  }
  char *base = static_cast<char *>(scratch);
  for (BatchJob &J : L.jobs) {
    J.a.part = base + reinterpret_cast<size_t>(J.a.part);
    J.a.part_drop = reinterpret_cast<double *>(
        base + reinterpret_cast<size_t>(J.a.part_drop));
  }
  int per_sm = L.precision == SS_PREC_FP64
                   ? batch_fp64_blocks_per_sm(L.threads, L.smem)
                   : batch_split_blocks_per_sm(L.rough_kind, L.threads,
                                               L.smem);
  if (per_sm <= 0) {
    set_error("batched kernel does not fit on an SM with this shared memory");
    return SS_ERR_UNSUPPORTED;
  }
  if (tune && tune->ctas_per_sm > 0) per_sm = std::min(per_sm, tune->ctas_per_sm);
  cudaError_t e = cudaMemcpy(base + L.table_off, L.jobs.data(),
                             sizeof(BatchJob) * L.jobs.size(),
                             cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_status(e, "batch job table upload");
  std::memset(info, 0, sizeof(*info));
  info->n_jobs = n_jobs;
  info->precision = L.precision;
  info->rough_kind = L.rough_kind;
  info->threads = L.threads;
  info->ctas = per_sm * sm_count();
  info->n_items = L.n_items;
  info->n_out = L.n_out;
  info->smem = L.smem;
  info->table_offset = L.table_off;
  return SS_OK;
}

extern "C" int ss_coherent_batch_run(const ss_batch_info *info,
                                     void *scratch, void *stream) {
  using namespace ss;
  if (!info || !scratch || info->n_jobs <= 0) {
    set_error("null or empty batch");
    return SS_ERR_ARG;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  char *base = static_cast<char *>(scratch);
  auto *counter = reinterpret_cast<unsigned long long *>(base);
  const BatchJob *jobs =
      reinterpret_cast<const BatchJob *>(base + info->table_offset);
  cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(unsigned long long), st);
  if (e != cudaSuccess) return cuda_status(e, "batch counter clear");
  const bool f64 = info->precision == SS_PREC_FP64;
  int s = f64 ? coherent_batch_fp64_launch(jobs, info->n_jobs, info->n_items,
                                           counter, info->threads, info->ctas,
                                           info->smem, st)
              : coherent_batch_split_launch(jobs, info->n_jobs,
                                            info->n_items, counter,
                                            info->rough_kind, info->threads,
                                            info->ctas, info->smem, st);
  if (s) return s;
  return batch_reduce_launch(jobs, info->n_jobs, info->n_out, f64, st);
}
