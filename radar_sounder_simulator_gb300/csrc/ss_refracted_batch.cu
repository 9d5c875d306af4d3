// Batched refracted targets in one persistent launch.
//
// The reference's simulate() calls refracted_cluttergram once per target
// layer and frequency band (simulate.py:338-381); a multi-band or
// multi-layer run is then a series of launches whose per-trace costs differ
// by the band's series length and the target's depth. Here the jobs of one
// path class (sequential chain, or the joint solve through a given number
// of interfaces), roughness kind and form are cut into work items of about
// equal pair counts (trace block x facet chunk, the one-call kernel's CTA
// unit) and served from one queue by a persistent grid; one batched fix-up
// evaluates every job's deferred pairs and one batched reduce writes every
// job's output.
//
// prepare: validates every job, lays out the caller's scratch (queue
//   counter, job table, per-job partials, the jobs' deferral masks end to
//   end in 32-word groups) and uploads the job table (synchronous);
// run: clear the counter and the masks, persistent kernel, batched fix-up,
//   batched reduce -- stream operations only (graph-capturable).
#include <algorithm>
#include <cstring>
#include <vector>

#include "ss_chunksum.cuh"
#include "ss_refracted_split.cuh"

namespace ss {

static size_t rb_align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Batched reduce: every job's partial histograms, chunk by chunk in a fixed
// order, into its output (the one-call chunk reduce, per job).
__global__ void refracted_batch_reduce(const RefBatchJob *jobs, int n_jobs,
                                       long long n_out) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
       e < n_out; e += (long long)gridDim.x * blockDim.x) {
    const RefBatchJob &J = jobs[ref_batch_find<1>(jobs, n_jobs, e)];
    const RefArgs &a = J.a;
    const long long local = e - J.out0;
    const int t = (int)(local / a.n_seg);
    const int b = (int)(local % a.n_seg);
    const float2 *part = reinterpret_cast<const float2 *>(a.part);
    ChunkSum<float2> s;
    for (int c = 0; c < J.n_chunks; ++c)
      s.add(part[((size_t)c * a.T + t) * a.n_seg + b]);
    const double sr = s.re(), si = s.im();
    long o = (long)local;
    if (a.split) {  // (T, 2, n) -> (T, n, 2) [left, right]
      const int side = b / a.n_samples, bl = b % a.n_samples;
      o = ((long)t * a.n_samples + bl) * 2 + side;
    }
    if (J.out.field_c128) {
      J.out.field_c128[2 * o] = sr;
      J.out.field_c128[2 * o + 1] = si;
    } else {
      J.out.field_c64[2 * o] = (float)sr;
      J.out.field_c64[2 * o + 1] = (float)si;
    }
    if (b == 0) {
      double d = 0.0;
      for (int c = 0; c < J.n_chunks; ++c)
        d += a.part_drop[(size_t)c * a.T + t];
      J.out.dropped[t] = d;
    }
  }
}

struct RefBatchLayout {
  std::vector<RefBatchJob> jobs;
  size_t table_off = 256, mask_off = 0, bytes = 0, smem = 0;
  long long n_items = 0, n_out = 0, n_words = 0;
  int path_class = 0, rough_kind = 0, plain = 1;
};

static bool job_plain(const RefArgs &a) {
  return a.rough_kind == SS_ROUGH_NONE && a.pat_kind == SS_PAT_ISOTROPIC &&
         !a.taper && !a.F.diffuse_amp && !a.split;
}

static int ref_batch_layout(const ss_refracted_job *jobs, int n_jobs,
                            const ss_batch_tuning *tune, RefBatchLayout &L) {
  if (!jobs || n_jobs <= 0) {
    set_error("empty batch");
    return SS_ERR_ARG;
  }
  if (tune && tune->threads && tune->threads != kSplitThreads) {
    set_error("refracted batch threads must be 512");
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
  L.jobs.assign(n_jobs, RefBatchJob{});
  double total_pairs = 0.0;
  std::vector<long long> window(n_jobs);
  for (int j = 0; j < n_jobs; ++j) {
    const ss_refracted_job &q = jobs[j];
    if (q.opts.precision != SS_PREC_SPLIT) {
      set_error("refracted batches run the split form");
      return SS_ERR_ARG;
    }
    Plan p;
    int s = build_ref_args(&q.opts, &q.target, &q.traces, &q.pattern,
                           &q.rough, true, &q.out, p, L.jobs[j].a);
    if (s) return s;
    RefArgs &a = L.jobs[j].a;
    const int cls = a.joint ? a.ni : 0;
    if (a.joint && a.ni > 4) {
      set_error("batched joint solve supports up to 4 interfaces");
      return SS_ERR_UNSUPPORTED;
    }
    if (j == 0) {
      L.path_class = cls;
      L.rough_kind = a.rough_kind;
    } else if (cls != L.path_class || a.rough_kind != L.rough_kind) {
      set_error("all jobs of a refracted batch need the same path class "
                "(sequential, or joint through the same interface count) "
                "and roughness kind");
      return SS_ERR_ARG;
    }
    const RefArgs &a0 = L.jobs[0].a;
    if (a.pat_kind != a0.pat_kind || a.pat_n != a0.pat_n || a.pa != a0.pa ||
        a.pb != a0.pb) {
      set_error("all jobs of a refracted batch need one antenna table");
      return SS_ERR_ARG;
    }
    L.plain = L.plain && job_plain(a);
    const size_t per_trace = (size_t)a.n_seg * sizeof(float2);
    a.tb = (int)std::min<size_t>(
        std::max<size_t>(1, std::min<size_t>(96 * 1024 / per_trace, max_tb)),
        (size_t)a.T);
    L.jobs[j].n_groups = (a.T + a.tb - 1) / a.tb;
    window[j] = std::min<long long>((long long)a.n_win * a.bs, a.N);
    total_pairs += (double)a.T * window[j];
  }
  const double per_item =
      std::max(1.0, total_pairs / ((double)ips * sm_count()));
  // The queue serves the costliest jobs first (longest-processing-time
  // order): items hold about equal pair counts, a pair's cost grows with
  // the job's series length, and a queue that ends on the cheapest items
  // leaves the persistent grid a short tail. Each job keeps its own
  // outputs, so the table order is free.
  std::vector<int> order(n_jobs);
  for (int j = 0; j < n_jobs; ++j) order[j] = j;
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
    return L.jobs[x].a.n_terms > L.jobs[y].a.n_terms;
  });
  {
    std::vector<RefBatchJob> sorted(n_jobs);
    std::vector<long long> win(n_jobs);
    for (int r = 0; r < n_jobs; ++r) {
      sorted[r] = L.jobs[order[r]];
      win[r] = window[order[r]];
    }
    L.jobs.swap(sorted);
    window.swap(win);
  }
  size_t off = L.table_off + rb_align256(sizeof(RefBatchJob) * n_jobs);
  long long item = 0, out = 0, word = 0;
  for (int j = 0; j < n_jobs; ++j) {
    RefBatchJob &J = L.jobs[j];
    RefArgs &a = J.a;
    const double item_pairs = (double)window[j] * a.tb;
    const long long max_chunks = std::max<long long>(1, window[j] / 256);
    J.n_chunks = (int)std::min<long long>(
        max_chunks, std::max<long long>(1, (long long)(item_pairs / per_item +
                                                       0.5)));
    a.n_chunks = J.n_chunks;
    J.item0 = item;
    J.out0 = out;
    item += (long long)J.n_chunks * J.n_groups;
    out += (long long)a.T * a.n_seg;
    a.defer_w = window[j];
    J.words = (long long)(((unsigned long long)a.T * a.defer_w + 31) / 32);
    J.word0 = word;
    word += (J.words + 31) / 32 * 32;  // 32-word groups never straddle jobs
    J.out = jobs[order[j]].out;
    a.part = reinterpret_cast<void *>(off);  // offsets until prepare
    off += rb_align256((size_t)J.n_chunks * a.T * a.n_seg * sizeof(float2));
    a.part_drop = reinterpret_cast<double *>(off);
    off += rb_align256((size_t)J.n_chunks * a.T * sizeof(double));
    L.smem = std::max(L.smem, split_smem_bytes(a, a.tb));
  }
  L.mask_off = off;
  off += rb_align256((size_t)word * sizeof(uint32_t));
  for (RefBatchJob &J : L.jobs) {
    J.a.defer_mask = reinterpret_cast<uint32_t *>(
        L.mask_off + (size_t)J.word0 * sizeof(uint32_t));
    J.k = split_consts(J.a);
  }
  L.n_items = item;
  L.n_out = out;
  L.n_words = word;
  L.bytes = off;
  if (L.smem > 200 * 1024) {
    set_error("a job's shared-memory histogram exceeds 200 KB");
    return SS_ERR_UNSUPPORTED;
  }
  return SS_OK;
}

static int ref_batch_occupancy_class(int cls, int rough, bool plain,
                                     size_t smem) {
  switch (cls) {
    case 0: return refracted_batch_occupancy_ni0(rough, plain, smem);
    case 1: return refracted_batch_occupancy_ni1(rough, plain, smem);
    case 2: return refracted_batch_occupancy_ni2(rough, plain, smem);
    case 3: return refracted_batch_occupancy_ni3(rough, plain, smem);
    default: return refracted_batch_occupancy_ni4(rough, plain, smem);
  }
}

}  // namespace ss

extern "C" size_t ss_refracted_batch_scratch_bytes(
    const ss_refracted_job *jobs, int32_t n_jobs,
    const ss_batch_tuning *tune) {
  ss::RefBatchLayout L;
  if (ss::ref_batch_layout(jobs, n_jobs, tune, L) != SS_OK) return 0;
  return L.bytes;
}

extern "C" int ss_refracted_batch_prepare(const ss_refracted_job *jobs,
                                          int32_t n_jobs,
                                          const ss_batch_tuning *tune,
                                          void *scratch, size_t scratch_bytes,
                                          ss_refracted_batch_info *info) {
  using namespace ss;
  if (!info) {
    set_error("null info");
    return SS_ERR_ARG;
  }
  RefBatchLayout L;
  int s = ref_batch_layout(jobs, n_jobs, tune, L);
  if (s) return s;
  if (!scratch || scratch_bytes < L.bytes) {
    set_error("scratch buffer too small");
    return SS_ERR_SCRATCH;
  }
  char *base = static_cast<char *>(scratch);
  for (RefBatchJob &J : L.jobs) {
    J.a.part = base + reinterpret_cast<size_t>(J.a.part);
    J.a.part_drop = reinterpret_cast<double *>(
        base + reinterpret_cast<size_t>(J.a.part_drop));
    J.a.defer_mask = reinterpret_cast<uint32_t *>(
        base + reinterpret_cast<size_t>(J.a.defer_mask));
  }
  int per_sm = ref_batch_occupancy_class(L.path_class, L.rough_kind,
                                         L.plain != 0, L.smem);
  if (per_sm <= 0) {
    set_error("batched refracted kernel does not fit on an SM with this "
              "shared memory");
    return SS_ERR_UNSUPPORTED;
  }
  if (tune && tune->ctas_per_sm > 0)
    per_sm = std::min(per_sm, tune->ctas_per_sm);
  cudaError_t e = cudaMemcpy(base + L.table_off, L.jobs.data(),
                             sizeof(RefBatchJob) * L.jobs.size(),
                             cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_status(e, "refracted batch table upload");
  std::memset(info, 0, sizeof(*info));
  info->n_jobs = n_jobs;
  info->path_class = L.path_class;
  info->rough_kind = L.rough_kind;
  info->plain = L.plain;
  info->ctas = per_sm * sm_count();
  info->n_items = L.n_items;
  info->n_out = L.n_out;
  info->n_words = L.n_words;
  info->smem = L.smem;
  info->fix_smem = 0;
  info->table_offset = L.table_off;
  info->mask_offset = L.mask_off;
  return SS_OK;
}

extern "C" int ss_refracted_batch_run(const ss_refracted_batch_info *info,
                                      void *scratch, void *stream) {
  using namespace ss;
  if (!info || !scratch || info->n_jobs <= 0) {
    set_error("null or empty batch");
    return SS_ERR_ARG;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  char *base = static_cast<char *>(scratch);
  auto *counter = reinterpret_cast<unsigned long long *>(base);
  const RefBatchJob *jobs =
      reinterpret_cast<const RefBatchJob *>(base + info->table_offset);
  cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(unsigned long long), st);
  if (e != cudaSuccess) return cuda_status(e, "batch counter clear");
  e = cudaMemsetAsync(base + info->mask_offset, 0,
                      (size_t)info->n_words * sizeof(uint32_t), st);
  if (e != cudaSuccess) return cuda_status(e, "batch mask clear");
  int s;
  const bool plain = info->plain != 0;
#define SS_RB(N)                                                              \
  refracted_batch_launch_ni##N(jobs, info->n_jobs, info->n_items,           \
                               info->n_words, counter, info->rough_kind,     \
                               plain, info->ctas, info->smem,                \
                               info->fix_smem, st)
  switch (info->path_class) {
    case 0: s = SS_RB(0); break;
    case 1: s = SS_RB(1); break;
    case 2: s = SS_RB(2); break;
    case 3: s = SS_RB(3); break;
    default: s = SS_RB(4); break;
  }
#undef SS_RB
  if (s) return s;
  refracted_batch_reduce<<<4 * sm_count(), 256, 0, st>>>(jobs, info->n_jobs,
                                                         info->n_out);
  return cuda_status(cudaGetLastError(), "refracted batch reduce launch");
}
