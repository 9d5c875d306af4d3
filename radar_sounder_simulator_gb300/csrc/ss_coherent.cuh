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

int coherent_plan(const ss_coherent_opts *o, int T, int N, Plan *p);
size_t coherent_scratch(const ss_coherent_opts *o, int T, int N);
int coherent_split_launch(CoArgs &a, const Plan &p, cudaStream_t st);

}  // namespace ss
