/*
 * soundersim_gb300.h -- C ABI of the GB300 (sm_103a) coherent facet kernels.
 *
 * Plain C: device pointers, sizes, status codes; no exceptions and no
 * framework types cross this boundary. Every pointer marked (device) must
 * be a CUDA device pointer owned by the caller; nothing here retains a
 * pointer after the call returns. Work is enqueued on `stream` (a
 * cudaStream_t passed as void*, NULL = legacy default stream) and the
 * functions return without synchronising, except where noted.
 *
 * The reference (soundersim, paths relative to src/soundersim/) exposes this
 * path as two Python functions, kernels/coherent.py:247-362
 * (coherent_cluttergram) and kernels/multilayer.py:594-770
 * (refracted_cluttergram). Their host preparation (along-track sort, block
 * windows, lookup tables) stays on the host in the Python mirror
 * (radar_sounder_simulator_gb300.kernels); the jitted device programs they
 * launch (coherent.py:172-244 `_coherent_fn`, multilayer.py:333-591
 * `_refracted_fn`) are what the entry points below replace.
 */
#ifndef SOUNDERSIM_GB300_H
#define SOUNDERSIM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ----------------------------------------------------- */
#define SS_OK 0
#define SS_ERR_ARG 1         /* invalid argument (null pointer, bad size)  */
#define SS_ERR_CUDA 2        /* a CUDA runtime call failed                  */
#define SS_ERR_UNSUPPORTED 3 /* option combination not implemented          */
#define SS_ERR_SCRATCH 4     /* scratch buffer smaller than required        */

/* ---- enumerations ------------------------------------------------------ */
#define SS_PREC_FP64 0   /* plain float64 form (the drop-in)               */
#define SS_PREC_SPLIT 1  /* float32 bulk, double-float range/phase/bins    */

/* antenna.py:204-258 gain_fn kinds */
#define SS_PAT_ISOTROPIC 0
#define SS_PAT_DIPOLE 1
#define SS_PAT_ARRAY 2
#define SS_PAT_ARRAY_TAPERED 3
#define SS_PAT_FINITE_DIPOLE 4
#define SS_PAT_TABULATED 5

/* roughness.py:217-276 d_phi variants */
#define SS_ROUGH_NONE 0
#define SS_ROUGH_GAUSS_FULL 1  /* Eqs 22-24 through the Faddeeva function  */
#define SS_ROUGH_GAUSS_AREA 2  /* area-only, Gaussian ACF                  */
#define SS_ROUGH_EXP_AREA 3    /* area-only, exponential ACF               */

/* ---- inputs ------------------------------------------------------------ */

/* Target facets in along-track sorted order, structure of arrays, float32
 * (the reference quantises facet geometry to float32: coherent.py:298-301,
 * multilayer.py:699-702). Optional arrays may be NULL. */
typedef struct {
  const float *cx, *cy, *cz;       /* (device) centroid                     */
  const float *nx, *ny, *nz;       /* (device) unit normal                  */
  const float *e1x, *e1y, *e1z;    /* (device) mean edge along +column      */
  const float *e2x, *e2y, *e2z;    /* (device) mean edge along +row         */
  const float *area;               /* (device) |e1 x e2|                    */
  const float *gamma_f32;          /* (device) per-facet field gamma or NULL
                                      (surface path, float32 like
                                      coherent.py:338-345)                  */
  const double *gamma_f64;         /* (device) per-facet field gamma or NULL
                                      (refracted path, float64 like
                                      multilayer.py:728-735)                */
  const float *sigma;              /* (device) per-facet rms height or NULL */
  const float *corr;               /* (device) per-facet corr length or NULL*/
  const float *phasor;             /* (device) complex64 speckle phasors
                                      interleaved (re, im), or NULL        */
  const double *diffuse_amp;       /* (device) diffuse field amp or NULL    */
  const float *diffuse_phasor;     /* (device) complex64 diffuse phasors    */
  int32_t n_facets;
} ss_facets;

/* Per-trace inputs. */
typedef struct {
  const double *pos;  /* (device) (T, 3) platform positions, local frame    */
  const double *uct;  /* (device) (T, 3) cross-track unit vectors; used with
                         split_sides only (else may be NULL)                 */
  const double *pv;   /* (device) (T, pv_len) antenna pattern vectors, or
                         NULL when isotropic                                 */
  const int32_t *off; /* (device) (T,) first facet block of each trace's
                         along-track window (geometry.py:63-78)              */
  int32_t n_traces;
  int32_t pv_len;     /* 3, or 6 for the array kinds ((2,3) frame)          */
} ss_traces;

/* Antenna pattern (antenna.py:76-118 pattern_args). pa/pb are device
 * arrays: array -> pa[0] = n_elements, pb[0..3]; array_tapered -> pa (2, n)
 * tx/rx weights, pb[0..3]; finite_dipole -> pa[0] = length_lam; tabulated
 * -> pa theta samples (rad, ascending), pb gains (n each). */
typedef struct {
  int32_t kind;
  int32_t n;          /* array_tapered: elements; tabulated: samples        */
  const double *pa;   /* (device) or NULL                                    */
  const double *pb;   /* (device) or NULL                                    */
} ss_pattern;

/* Sub-facet roughness of the target interface (roughness.py). */
typedef struct {
  int32_t kind;       /* SS_ROUGH_*                                          */
  int32_t n_terms;    /* static series length (roughness.py:189-196)         */
  double sigma;       /* scalar rms height (used when facets.sigma == NULL)  */
  double corr;        /* scalar corr length (used when facets.corr == NULL)  */
} ss_roughness;

/* Surface coherent kernel options (coherent.py:247-362 keywords). */
typedef struct {
  double k;           /* wavenumber (rad/m)                                  */
  double gamma;       /* scalar field reflection coefficient                 */
  double t0, dt, c;   /* fast-time window start, bin width, speed of light  */
  double taper_s;     /* off-specular taper s_eff (used when taper != 0)     */
  int32_t n_samples;
  int32_t block_size; /* culling block size (facets)                         */
  int32_t n_win;      /* blocks per trace window                             */
  int32_t split_sides;
  int32_t interp_bins;
  int32_t taper;
  int32_t precision;  /* SS_PREC_*                                           */
} ss_coherent_opts;

/* Outputs. Exactly one of field_c128 / field_c64 is non-NULL. Layout
 * (T, n_samples) or, with split_sides, (T, n_samples, 2) [left, right]
 * (coherent.py:360-361). */
typedef struct {
  double *field_c128;  /* (device) complex128 interleaved, or NULL          */
  float *field_c64;    /* (device) complex64 interleaved, or NULL           */
  double *dropped;     /* (device) (T,) out-of-window power                 */
} ss_output;

/* ---- surface coherent facet sum ------------------------------------- */

/* Bytes of device scratch that ss_coherent_fwd needs for these shapes
 * (per-CTA partial histograms, reduced deterministically afterwards).
 * Replaces nothing in the reference (XLA allocates internally). */
size_t ss_coherent_scratch_bytes(const ss_coherent_opts *opts,
                                 int32_t n_traces, int32_t n_facets);

/* Binned coherent field of every trace over the culled target facets.
 * Replaces the jitted vmap(one_trace) program of
 * kernels/coherent.py:172-244 (`_coherent_fn`), called at
 * kernels/coherent.py:350-358; the returned field already carries the
 * absolute carrier phase (the reference's phase_ref fold-back at
 * coherent.py:359 is folded in). `scratch` (device) must hold
 * ss_coherent_scratch_bytes(...) bytes. */
int ss_coherent_fwd(const ss_coherent_opts *opts, const ss_facets *facets,
                    const ss_traces *traces, const ss_pattern *pattern,
                    const ss_roughness *rough, const ss_output *out,
                    void *scratch, size_t scratch_bytes, void *stream);

/* ---- surface facet sum without caller scratch ------------------------ */

/* Size of the fixed device scratch array behind ss_coherent_fwd_noalloc. */
#define SS_NOALLOC_SCRATCH_BYTES (64u << 20)

/* ss_coherent_fwd for callers that cannot allocate device memory: the same
 * inputs, outputs and results (within float rounding: it may sum the facet
 * chunks in fewer groups), with the scratch taken from a fixed array of
 * SS_NOALLOC_SCRATCH_BYTES compiled into this library instead of a caller
 * buffer. It has no counterpart in the reference, which only runs inside
 * its own Python process and leaves device memory to XLA.
 *
 * Who needs it: programs whose device memory belongs to another allocator
 * (a framework's pool, or a budget fixed at start-up) and processing loops
 * that must not allocate once running, so they cannot hand ss_coherent_fwd
 * a scratch buffer.
 *
 * Limits and sharing: one facet chunk of partial histograms for all traces,
 * n_traces * n_samples * (2 with split_sides) * (16 bytes FP64, 8 bytes
 * split) + 8 bytes per trace, must fit in the array, else SS_ERR_SCRATCH
 * is returned before any work is queued. The array is reserved on every GPU
 * that loads the library until the process exits. The first call on each
 * device looks up the array's device address (cudaGetSymbolAddress) with
 * that device current; make that call before any stream capture. All calls
 * share the array and leave their partials in it: calls that overlap on the
 * GPU (different streams or host threads) race. Nothing in it needs
 * clearing, since every partial read is first written by the same call.
 * No device memory is allocated or freed. */
int ss_coherent_fwd_noalloc(const ss_coherent_opts *opts,
                            const ss_facets *facets, const ss_traces *traces,
                            const ss_pattern *pattern,
                            const ss_roughness *rough, const ss_output *out,
                            void *stream);

/* ---- refracted multilayer facet sum ---------------------------------- */

/* Crossed interfaces per call after padding: the reference's deepest firn
 * runs cross 40 layers. Above 4 (split form) or 8 (FP64 form) interfaces the
 * joint solve keeps its per-interface arrays in local memory, which the
 * driver reserves for every resident thread while such a call runs. */
#define SS_MAX_IFACE 40

/* One crossed interface: its facet lookup table and mean plane
 * (multilayer.py:269-283 `_grid_consts`; joint no-op pads per :286-330 are
 * 1x1 tables with a zero affine fit). */
typedef struct {
  const float *table;     /* (device) (ny, nx, 6) float32 [centre, normal]  */
  int32_t ny, nx;
  double coef[6];         /* (3, 2) row-major fit (x, y, 1) -> (row, col)  */
  double mean_point[3];   /* area-weighted mean point                       */
  double mean_normal[3];  /* unit area-weighted mean normal                 */
} ss_interface;

/* Refracted kernel options (multilayer.py:594-770 keywords). The small
 * per-leg arrays are HOST pointers, copied at the call. */
typedef struct {
  int32_t n_crossed;             /* crossed interfaces incl. joint pads     */
  int32_t k_pad;                 /* leading no-op pads (joint only)         */
  int32_t n_legs;                /* entries in the leg arrays: crossing i
                                    uses [i] and [i + 1], the final leg the
                                    last entry (multilayer.py:506-508 reads
                                    n_leg[-1] / att[-1]); >= n_crossed + 1,
                                    == n_crossed + 1 for the joint solve    */
  const ss_interface *crossed;   /* (host) n_crossed descriptors, top-down  */
  const double *n_leg;           /* (host) n_legs refractive indices        */
  const double *eps_leg;         /* (host) n_legs permittivities            */
  const double *att_leg;         /* (host) n_legs one-way dB/km             */
  const double *sigma_crossed;   /* (host) n_crossed rms heights, or NULL   */
  double k0, gamma, t0, dt, c;
  double taper_s;                /* used when taper != 0                    */
  double diffuse_exp;            /* cos^n law of the diffuse channel        */
  int32_t n_samples, block_size, n_win;
  int32_t split_sides;
  int32_t coherent;              /* 1 coherent field, 0 incoherent power    */
  int32_t joint;                 /* 0 sequential chain, 1 joint solve       */
  int32_t joint_newton, joint_backtrack;
  int32_t taper;
  int32_t precision;             /* SS_PREC_*                               */
} ss_refracted_opts;

/* Scratch bytes ss_refracted_fwd needs for these shapes. */
size_t ss_refracted_scratch_bytes(const ss_refracted_opts *opts,
                                  int32_t n_traces, int32_t n_facets);

/* Binned refracted-path contributions of one target interface under the
 * crossed stack. Replaces the jitted vmap(one_trace) program of
 * kernels/multilayer.py:333-591 (`_refracted_fn`: `path` :352-406,
 * `path_joint` :408-457, `step` :464-583), called at
 * kernels/multilayer.py:758-767. Coherent mode writes the complex field,
 * incoherent mode the power in the real part (imaginary part zero). */
int ss_refracted_fwd(const ss_refracted_opts *opts, const ss_facets *target,
                     const ss_traces *traces, const ss_pattern *pattern,
                     const ss_roughness *rough, const ss_output *out,
                     void *scratch, size_t scratch_bytes, void *stream);

/* ---- incoherent (power) facet sum ------------------------------------ */

/* Incoherent kernel options (kernels/incoherent.py:64-66 keywords). The
 * window scalars are rounded to float32 inside, as the reference does
 * (incoherent.py:101-102). block_size has no counterpart: it only groups the
 * reference's float32 sums. */
typedef struct {
  double t0, dt, c;
  int32_t n_samples;
  int32_t split_sides;
} ss_incoherent_opts;

/* float32 outputs, the reference's return types (incoherent.py:96-103). */
typedef struct {
  float *power;    /* (device) (T, n_samples) or (T, n_samples, 2)
                      [left, right]                                        */
  float *dropped;  /* (device) (T,) out-of-window power                    */
} ss_incoherent_output;

size_t ss_incoherent_scratch_bytes(const ss_incoherent_opts *opts,
                                   int32_t n_traces, int32_t n_facets);

/* Binned incoherent power (A cos)^2 / r^4, times g^4 with a pattern, of
 * every facet for every trace (no culling, like the reference). Replaces the
 * jitted vmap(one_trace) program of kernels/incoherent.py:32-61
 * (`_incoherent_fn`), called at kernels/incoherent.py:100-103. Uses
 * facets->cx..nz and area only (float32), traces->pos, ->uct (split_sides)
 * and ->pv (pattern); traces->off is ignored. Bins equal the reference's
 * float32 bins bit for bit; powers are float32 sums (chunk partials added
 * in float64). */
int ss_incoherent_fwd(const ss_incoherent_opts *opts, const ss_facets *facets,
                      const ss_traces *traces, const ss_pattern *pattern,
                      const ss_incoherent_output *out, void *scratch,
                      size_t scratch_bytes, void *stream);

/* ---- focused SAR (time-domain backprojection) ------------------------ */

#define SS_WIN_HANN 0  /* 0.5 (1 + cos(pi d / (L/2))) */
#define SS_WIN_RECT 1  /* rectangular ("none")        */

/* processing.py:262-348 focused_sar arguments, on plain arrays. */
typedef struct {
  double wavelength;   /* carrier wavelength (m): k = 2 pi / wavelength     */
  double aperture_m;   /* full aperture L; traces with |s_j - s_i| <= L/2   */
  double c;            /* wave speed of the twtt -> range map (air)         */
  int32_t n_traces;    /* T */
  int32_t n_bins;      /* nb >= 2: t0 = twtt[0], dt = twtt[1] - twtt[0]     */
  int32_t window;      /* SS_WIN_*                                          */
  int32_t precision;   /* SS_PREC_FP64 (the reference's float64 chain) or
                          SS_PREC_SPLIT (float32 arithmetic)                */
  int32_t in_f64;      /* field elements: 1 complex128, 0 complex64         */
} ss_focus_opts;

/* Any subset may be NULL (at least one set); layout (T, nb). */
typedef struct {
  double *field_c128;  /* (device) complex128 interleaved                   */
  float *field_c64;    /* (device) complex64 interleaved                    */
  float *power;        /* (device) float32 |out|^2 (processing.py:345)      */
} ss_focus_output;

/* Scratch for the per-trace aperture bounds (8 bytes per trace). */
size_t ss_focused_sar_scratch_bytes(const ss_focus_opts *opts);

/* Focused field of every trace: replaces the loop of processing.py:317-329.
 * field (device) (T, nb) complex, twtt (device) (nb,) float64 fast-time
 * axis, s (device) (T,) float64 along-track arc length, non-decreasing
 * (processing.py:65-69 computes it from the positions). */
int ss_focused_sar(const ss_focus_opts *opts, const void *field,
                   const double *twtt, const double *s,
                   const ss_focus_output *out, void *scratch,
                   size_t scratch_bytes, void *stream);

/* ---- scene assembly ---------------------------------------------------- */

/* Projected CRS of a DEM window (the reference takes any CRS from pyproj;
 * these are the ones its synthetic scenes and ice-sheet DEMs use). */
#define SS_PROJ_IDENTITY 0     /* projected (E, N, h) already are ECEF      */
#define SS_PROJ_POLAR_NORTH 1  /* EPSG:3413, WGS84 polar stereographic N    */
#define SS_PROJ_POLAR_SOUTH 2  /* EPSG:3031, WGS84 polar stereographic S    */

/* ENU frame (scene.py:24-82 LocalFrame): local = R (ecef - origin), R's
 * rows the E, N, U unit vectors in ECEF, row-major. */
typedef struct {
  double origin[3];
  double R[9];
} ss_frame;

/* A DEM window sampled on its facet lattice (scene.py:126-156). */
typedef struct {
  const double *dem;       /* (device) (ny, nx) heights above WGS84 (m)   */
  int32_t ny, nx;
  const double *rows;      /* (device) (n_rows,) fractional pixel rows    */
  const double *cols;      /* (device) (n_cols,) fractional pixel columns */
  int32_t n_rows, n_cols;
  double transform[6];     /* pixel (x, y) -> (x a + y b + c, x d + y e + f),
                              (a, b, c, d, e, f)                          */
  int32_t projection;      /* SS_PROJ_*                                    */
  ss_frame frame;
} ss_dem_grid;

/* Vertices (n_rows, n_cols, 3) float64 in the local frame: bilinear DEM
 * sample at each lattice point (scene.py:104-112), pixel centre through the
 * affine transform, projected -> geodetic -> ECEF (WGS84) -> local. */
int ss_scene_vertices(const ss_dem_grid *grid, double *vertices,
                      void *stream);

/* Mean-plane facets of a vertex grid (scene.py:158-176). Any output may be
 * NULL. centers/normals/e1/e2 (N, 3), areas (N,), cell and phase_keys
 * (N, 2) int64 (phase_keys from row_keys[i], col_keys[j]); N = (H-1)(W-1),
 * facet (i, j) at i (W-1) + j. */
typedef struct {
  double *centers, *normals, *areas, *e1, *e2;
  int64_t *cell, *phase_keys;
} ss_facet_out;

int ss_facets_from_vertices(const double *vertices, int32_t H, int32_t W,
                            const int64_t *row_keys, const int64_t *col_keys,
                            const ss_facet_out *out, void *stream);

/* Stateless Gaussian speckle phasors of (n, 2) int64 parent-grid keys
 * (roughness.py:207-233); base = the seed's SeedSequence state word.
 * out: (n,) complex64 interleaved (device). */
int ss_speckle_phasors_keyed(const int64_t *keys, int64_t n, uint64_t base,
                             float *out, void *stream);

/* Facet centres moved `offset` metres along local ellipsoidal up
 * (layered.py:38-53 offset_facets; normals, areas and edges unchanged). */
int ss_offset_centers(const double *centers, int64_t n, const ss_frame *frame,
                      double offset, double *out, void *stream);

/* ---- per-trace output products ---------------------------------------- */

/* output.py:47-82 build_dataset window (twtt axis t0 + k dt, k < n_samples)
 * and wave speed. */
typedef struct {
  double t0, dt, c;
  int32_t n_samples;
} ss_trace_products_opts;

/* Any output may be NULL. nadir: the horizontally nearest facet centre
 * (first index on ties) and 2 (z_platform - z_facet) / c; first return:
 * the facet with the earliest float64 twtt 2r/c inside [t0, t0 +
 * n_samples dt) (first index on ties), or index 0 and +inf if none. */
typedef struct {
  int64_t *nadir_index;
  double *nadir_twtt;
  int64_t *first_index;
  double *first_twtt;
} ss_trace_products_out;

size_t ss_trace_products_scratch_bytes(int32_t n_traces, int32_t n_facets);

/* Every facet for every trace: centers (device) (N, 3) float64, positions
 * (device) (T, 3) float64. Replaces the (T, N, 3) NumPy scans of
 * output.py:64-82 (same results: float64 values in the reference's
 * operation order, NumPy's first-index tie rule). */
int ss_trace_products(const ss_trace_products_opts *opts,
                      const double *centers, int32_t n_facets,
                      const double *positions, int32_t n_traces,
                      const ss_trace_products_out *out, void *scratch,
                      size_t scratch_bytes, void *stream);

/* Batched surface coherent sums (no counterpart in the reference, which
 * calls coherent_cluttergram once per scene): one job per call of
 * ss_coherent_fwd, all jobs of a batch with the same precision and
 * roughness kind. */
typedef struct {
  ss_coherent_opts opts;
  ss_facets facets;
  ss_traces traces;
  ss_pattern pattern;   /* kind SS_PAT_ISOTROPIC for none */
  ss_roughness rough;   /* kind SS_ROUGH_NONE for none */
  ss_output out;
} ss_coherent_job;

/* Work decomposition of a batch (0 = default). */
typedef struct {
  int32_t threads;       /* CTA size: 128 or 256 (default 256), or 512 for
                            smooth split-precision coherent batches;
                            refracted batches take 512 only */
  int32_t max_tb;        /* traces per work item, 1..8 (default 8) */
  int32_t items_per_sm;  /* work items per SM; sets facet-chunk sizes
                            (default 16) */
  int32_t ctas_per_sm;   /* persistent CTAs per SM (default: as many as fit) */
} ss_batch_tuning;

/* Filled by ss_coherent_batch_prepare; passed back to ss_coherent_batch_run. */
typedef struct {
  int32_t n_jobs, precision, rough_kind, threads, ctas, reserved;
  int64_t n_items, n_out;
  uint64_t smem, table_offset;
} ss_batch_info;

size_t ss_coherent_batch_scratch_bytes(const ss_coherent_job *jobs,
                                       int32_t n_jobs,
                                       const ss_batch_tuning *tune);

/* Validates every job, lays out `scratch` (work-queue counter, job table,
 * per-job partials) and uploads the job table (synchronous). The jobs'
 * device pointers must stay valid while the batch is run. */
int ss_coherent_batch_prepare(const ss_coherent_job *jobs, int32_t n_jobs,
                              const ss_batch_tuning *tune, void *scratch,
                              size_t scratch_bytes, ss_batch_info *info);

/* Runs a prepared batch on `stream`: one persistent work-queue kernel over
 * every job's (trace block x facet chunk) items, then one batched reduce
 * into every job's output. Stream operations only (graph-capturable). */
int ss_coherent_batch_run(const ss_batch_info *info, void *scratch,
                          void *stream);

/* Batched refracted targets (no counterpart in the reference, whose
 * simulate() calls refracted_cluttergram once per target layer and
 * frequency band: simulate.py:338-381, the call at :373-379): one job per
 * call of ss_refracted_fwd in split precision, all jobs of a batch on the
 * same path class (the sequential chain, or the joint solve through the
 * same number of interfaces after padding, at most 4), the same roughness
 * kind and one antenna table. */
typedef struct {
  ss_refracted_opts opts;  /* host arrays (crossed, legs) read at prepare */
  ss_facets target;
  ss_traces traces;
  ss_pattern pattern;      /* kind SS_PAT_ISOTROPIC for none */
  ss_roughness rough;      /* kind SS_ROUGH_NONE for none */
  ss_output out;
} ss_refracted_job;

/* Filled by ss_refracted_batch_prepare; passed back to
 * ss_refracted_batch_run. */
typedef struct {
  int32_t n_jobs, path_class, rough_kind, plain, ctas, reserved;
  int64_t n_items, n_out, n_words;
  uint64_t smem, fix_smem, table_offset, mask_offset;
} ss_refracted_batch_info;

size_t ss_refracted_batch_scratch_bytes(const ss_refracted_job *jobs,
                                        int32_t n_jobs,
                                        const ss_batch_tuning *tune);

/* Validates every job, lays out `scratch` (work-queue counter, job table,
 * per-job partials and deferral masks) and uploads the job table
 * (synchronous). The jobs' device pointers must stay valid while the batch
 * is run. */
int ss_refracted_batch_prepare(const ss_refracted_job *jobs, int32_t n_jobs,
                               const ss_batch_tuning *tune, void *scratch,
                               size_t scratch_bytes,
                               ss_refracted_batch_info *info);

/* Runs a prepared batch on `stream`: clears the masks, one persistent
 * work-queue kernel over every job's (trace block x facet chunk) items, one
 * batched fix-up of the deferred pairs, one batched reduce into every
 * job's output. Stream operations only (graph-capturable). */
int ss_refracted_batch_run(const ss_refracted_batch_info *info,
                           void *scratch, void *stream);

/* Pulse compression of kernel output along fast time. */
typedef struct {
  int32_t n_traces;  /* T */
  int32_t n_samples; /* B: fast-time samples per trace */
  int32_t n_lanes;   /* L: trailing lanes, e.g. 2 for split sides (T, B, 2) */
  int32_t n_taps;    /* pulse length 2M + 1 */
  int32_t center;    /* index of the pulse's zero lag (M) */
  int32_t power;     /* 0: complex field with complex taps;
                        1: real power with real taps (|p|^2), output >= 0 */
  int32_t in_f64;    /* input elements: 1 = float64, 0 = float32
                        (complex: interleaved re, im) */
} ss_waveform_opts;

/* 'same'-mode convolution y[t, i, l] = sum_j taps[j] x[t, i + center - j, l]
 * of a (T, B, L) array with the compressed pulse; replaces
 * convolve_fast_time (waveform.py:126-138) as used by apply_waveform
 * (waveform.py:141-160). taps: device float64, (n_taps, 2) re/im pairs
 * (power = 0) or (n_taps,) (power = 1). Input is rounded to float32 first
 * (the reference convolves the kernel's complex64 output); out: float32
 * (re, im) pairs (power = 0) or float32 clipped at 0 (power = 1). */
int ss_range_compress(const ss_waveform_opts *opts, const double *taps,
                      const void *in, void *out, void *stream);

/* The same convolution by FFT in float64 (the reference's method,
 * waveform.py:126-138), for n_samples + n_taps - 1 <= 8192; 0 bytes of
 * scratch means the size is beyond that (use ss_range_compress). */
size_t ss_range_compress_fft_scratch_bytes(const ss_waveform_opts *opts);
int ss_range_compress_fft(const ss_waveform_opts *opts, const double *taps,
                          const void *in, void *out, void *scratch,
                          size_t scratch_bytes, void *stream);

/* The FFT convolution in two steps, so that a pulse used for many arrays
 * is transformed once (apply_waveform, waveform.py:141-160, compresses
 * every kernel output with the same pulse): ss_range_compress_plan writes
 * the twiddles and the pulse spectrum into `plan`; ss_range_compress_apply
 * convolves one (T, B, L) array with them. Both take the same n_samples,
 * n_taps, center and power (n_traces, n_lanes and in_f64 may differ
 * between applies). precision: SS_PREC_FP64 (float64 transforms, as
 * ss_range_compress_fft) or SS_PREC_SPLIT (double-float transforms on the
 * FP32 pipe, ~1e-14 of the row's magnitude from the float64 ones, below
 * the float32 rounding of the output). Plan size 0: n_samples + n_taps - 1
 * is above 8192 (use ss_range_compress). Stream operations only. */
size_t ss_range_compress_plan_bytes(const ss_waveform_opts *opts,
                                    int precision);
int ss_range_compress_plan(const ss_waveform_opts *opts, int precision,
                           const double *taps, void *plan, size_t plan_bytes,
                           void *stream);
int ss_range_compress_apply(const ss_waveform_opts *opts, int precision,
                            const void *plan, size_t plan_bytes,
                            const void *in, void *out, void *stream);

/* Frequency-sampled synthesis (Mode F). */
typedef struct {
  double f0;          /* band centre (Hz) */
  double bandwidth;   /* band width B (Hz) */
  double c;           /* wave speed (m/s) */
  double gamma;       /* reflection coefficient (facets->gamma_f32 overrides) */
  double taper_s;     /* off-specular taper slope (used when taper != 0) */
  int32_t n_freq;     /* K midpoint samples f_k = f0 - B/2 + (k + 1/2) B/K */
  int32_t freeze_amplitudes; /* 1: amplitudes at f0, exact phase per f_k */
  int32_t taper;
  int32_t block_size; /* per-trace facet windows, as ss_coherent_opts */
  int32_t n_win;
  int32_t precision;  /* SS_PREC_FP64 or SS_PREC_SPLIT */
} ss_multifreq_opts;

size_t ss_multifreq_scratch_bytes(const ss_multifreq_opts *opts,
                                  int32_t n_traces, int32_t n_facets);

/* Band response H[t, k] = sum over the trace's facet window of the LPA
 * contribution at f_k (compare/multifreq.py:78-96, lpa_contributions of
 * kernels/coherent.py:107-128), for every trace. H: device float64
 * (T, K, 2) re/im. Roughness (frozen amplitudes, split form) uses
 * facets->sigma/corr/phasor as ss_coherent_fwd does. */
int ss_multifreq_response(const ss_multifreq_opts *opts,
                          const ss_facets *facets, const ss_traces *traces,
                          const ss_roughness *rough, double *H,
                          void *scratch, size_t scratch_bytes, void *stream);

/* Synthesis y[t, b] = sum_k wbar[k] H[t, k] exp(2j pi (f_k - f0) twtt[b])
 * (compare/multifreq.py:98). wbar (K,), twtt (B,), y (T, B, 2) float64
 * device arrays. */
int ss_multifreq_synth(const ss_multifreq_opts *opts, int32_t n_traces,
                       const double *H, const double *wbar,
                       const double *twtt, int32_t n_twtt, double *y,
                       void *stream);

/* FP32 FMA throughput probe (no counterpart in the reference; measurement
 * helper). Launches `blocks` CTAs of 256 threads, each thread running eight
 * independent FMA chains of `iters` steps, and writes blocks * 256 floats to
 * `out`. FLOP per launch = blocks * 256 * 8 * iters * 2; the caller times
 * the launch on `stream`. */
int ss_fp32_fma_probe(int32_t blocks, int32_t iters, float *out,
                      void *stream);

/* FP64 twin of ss_fp32_fma_probe (double chains, `out` blocks * 256
 * doubles); the roofline denominator of float64-bound kernels. */
int ss_fp64_fma_probe(int32_t blocks, int32_t iters, double *out,
                      void *stream);

/* MUFU (SFU) throughput probe: blocks CTAs of 256 threads, eight chains of
 * iters base-2 exponentials each; operations per launch = blocks * 256 * 8
 * * iters. The roofline denominator of the transcendental-heavy work (the
 * roughness series). */
int ss_mufu_probe(int32_t blocks, int32_t iters, float *out, void *stream);

/* Adjoint of windowed trace power (no counterpart in the reference). */
typedef struct {
  const double *field;       /* (T, n_samples, 2) forward field of the target
                                (device, the ss_refracted_fwd output) */
  const double *grad_power;  /* (T,) dL/dP_t, P_t = sum over the window of
                                |field[t, b]|^2 (device) */
  int32_t bin_lo, bin_hi;    /* power window [bin_lo, bin_hi) */
  const double *alpha_mask;  /* host (n_legs,): d att_leg[l] / d alpha */
  double *grad_gamma_db;     /* (N,) dL/d reflectivity in dB (device) */
  double *grad_sigma;        /* (N,) dL/d rms height, or NULL (device) */
  double *grad_alpha;        /* (ss_refracted_adjoint_blocks(N),) partial
                                sums of dL/d alpha (device; caller adds) */
  void *scratch;             /* device, ss_refracted_adjoint_scratch_bytes */
  size_t scratch_bytes;
} ss_adjoint_io;

int32_t ss_refracted_adjoint_blocks(int32_t n_facets);
size_t ss_refracted_adjoint_scratch_bytes(int32_t n_traces,
                                          int32_t n_facets);

/* Gradients of a loss of windowed trace power with respect to per-facet
 * reflectivity (dB; facets->gamma_f64 holds 10^(R/20)), per-facet
 * rms height (facets->sigma) and an attenuation rate alpha scaling the legs
 * of alpha_mask, for the sequential refracted path in coherent mode.
 * Recomputes every pair in the split form -- nothing per pair is stored by
 * the forward -- and re-evaluates the few pairs that need a float64 lookup
 * or bin decision in a fix-up pass (marked in `scratch`). Outputs are in
 * the facet order of the call. */
int ss_refracted_adjoint(const ss_refracted_opts *opts,
                         const ss_facets *target, const ss_traces *traces,
                         const ss_pattern *pattern, const ss_roughness *rough,
                         const ss_adjoint_io *io, void *stream);

/* Library build string (kernel version, arch) for result provenance. */
const char *ss_version(void);

/* Last CUDA error string seen by the library (thread-local), or "". */
const char *ss_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* SOUNDERSIM_GB300_H */
