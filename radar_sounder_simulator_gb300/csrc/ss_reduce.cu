// Ordered reduction of per-CTA partial histograms into the output layout.
#include <algorithm>

#include "ss_chunksum.cuh"
#include "ss_coherent.cuh"

namespace ss {

// grid: x over segments of a trace, y over traces (one element a thread,
// the chunk loads of an element independent of one another)
template <typename P>
__global__ void chunk_reduce_kernel(ReduceArgs r, ss_output out) {
  const P *part = reinterpret_cast<const P *>(r.part);
  for (int t = blockIdx.y; t < r.T; t += gridDim.y) {
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < r.n_seg;
         b += gridDim.x * blockDim.x) {
      ChunkSum<P> s;
      for (int c = 0; c < r.n_chunks; ++c)
        s.add(part[((size_t)c * r.T + t) * r.n_seg + b]);
      long o = (long)t * r.n_seg + b;
      if (r.split) {  // (T, 2, n) -> (T, n, 2) [left, right]
        const int side = b / r.n_samples, bl = b % r.n_samples;
        o = ((long)t * r.n_samples + bl) * 2 + side;
      }
      const double sr = s.re(), si = s.im();
      if (out.field_c128) {
        out.field_c128[2 * o] = sr;
        out.field_c128[2 * o + 1] = si;
      } else {
        out.field_c64[2 * o] = (float)sr;
        out.field_c64[2 * o + 1] = (float)si;
      }
      if (b == 0) {
        double d = 0.0;
        for (int c = 0; c < r.n_chunks; ++c)
          d += r.part_drop[(size_t)c * r.T + t];
        out.dropped[t] = d;
      }
    }
  }
}

// Batched form: one grid-stride pass over every job's (trace, segment)
// elements; each element sums its job's chunk partials in chunk order.
template <typename P>
__global__ void batch_reduce_kernel(const BatchJob *jobs, int n_jobs,
                                    long long n_out) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
       e < n_out; e += (long long)gridDim.x * blockDim.x) {
    const BatchJob &J = jobs[batch_find_job(jobs, n_jobs, e, false)];
    const CoArgs &a = J.a;
    const long long local = e - J.out0;
    const int t = (int)(local / a.n_seg);
    const int b = (int)(local % a.n_seg);
    const P *part = reinterpret_cast<const P *>(a.part);
    ChunkSum<P> s;
    for (int c = 0; c < J.n_chunks; ++c)
      s.add(part[((size_t)c * a.T + t) * a.n_seg + b]);
    const double sr = s.re(), si = s.im();
    long o = (long)local;
    if (a.split) {
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

int batch_reduce_launch(const BatchJob *jobs, int n_jobs, long long n_out,
                        bool f64_parts, cudaStream_t st) {
  const int grid = 4 * sm_count();
  if (f64_parts)
    batch_reduce_kernel<double2><<<grid, 256, 0, st>>>(jobs, n_jobs, n_out);
  else
    batch_reduce_kernel<float2><<<grid, 256, 0, st>>>(jobs, n_jobs, n_out);
  return cuda_status(cudaGetLastError(), "batch reduce launch");
}

int sm_count() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 152;
  }
  return n;
}

int launch_reduce(const ReduceArgs &r, bool f64_parts, const ss_output *out,
                  cudaStream_t st) {
  const dim3 grid((unsigned)std::min((r.n_seg + 255) / 256, 65535),
                  (unsigned)std::min(r.T, 65535));
  if (f64_parts)
    chunk_reduce_kernel<double2><<<grid, 256, 0, st>>>(r, *out);
  else
    chunk_reduce_kernel<float2><<<grid, 256, 0, st>>>(r, *out);
  return cuda_status(cudaGetLastError(), "chunk_reduce launch");
}

}  // namespace ss
