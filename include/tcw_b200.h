/*
 * tcw_b200.h -- C ABI of the GB300 (sm_103a) transient-CW F-statistic map.
 *
 * This library is the compute behind a 'b200' version of PyFstat's
 * transient F-stat map, a drop-in beside the 'lal' and 'pycuda' versions of
 * pyfstat/tcw_fstat_map_funcs.py (version table at :320-327, dispatcher
 * call_compute_transient_fstat_map at :495-544).  Its entry points replace
 * what the pycuda version does per call:
 *   - the H2D copy of the (numAtoms, 7) atoms matrix        (tcw:864, :945)
 *   - the rect / exp kernel launch                          (tcw:896-909, :977-991)
 *   - the D2H copy of the full FP32 map                     (tcw:912, :994)
 *   - max, argmax, lnBtSG and the t0/tau posteriors on host (tcw:810-828, :196-287)
 * and add a batched form for many templates in one launch.
 *
 * Conventions
 *   - Every function returns an int status: TCW_OK (0) or a negative
 *     TCW_ERR_* code; nothing throws or aborts.  tcw_strerror() names a code,
 *     tcw_last_error() gives the handle's last detailed message.
 *   - Atoms are row-major (numAtoms, 7) float32 matrices with columns
 *     [a2, b2, ab, Fa_re, Fa_im, Fb_re, Fb_im] -- the matrix PyFstat builds at
 *     tcw:711-721 -- on the binned grid t_i = t0_data + i*TAtom.
 *   - Grids are explicit u32 arrays t0s[N_t0] and taus[N_tau] (seconds); a
 *     lalpulsar transientWindowRange_t expands to t0 + m*dt0, tau + n*dtau.
 *     Rectangular maps need a non-decreasing tau grid.
 *   - The F map is row-major float32 [m][n] (m over t0, n over tau) and
 *     holds F, not 2F, exactly like pyTransientFstatMap.F_mn.
 *   - One handle per host thread; calls on a handle are asynchronous on its
 *     stream unless named *_host (those synchronise before returning).
 */
#ifndef TCW_B200_H
#define TCW_B200_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TCW_ABI_VERSION 1

/* status codes */
#define TCW_OK 0
#define TCW_ERR_INVALID_ARG (-1)
#define TCW_ERR_CUDA (-2)
#define TCW_ERR_NO_DEVICE (-3)
#define TCW_ERR_ALLOC (-4)
#define TCW_ERR_TIMEOUT (-5)
#define TCW_ERR_UNSUPPORTED (-6)
#define TCW_ERR_OVERFLOW (-7)
#define TCW_ERR_IO (-8)      /* file could not be opened, read or written */
#define TCW_ERR_FORMAT (-9)  /* malformed line in a text file */

/* window types: lalpulsar's transientWindowType_t values */
#define TCW_WINDOW_NONE 0
#define TCW_WINDOW_RECT 1
#define TCW_WINDOW_EXP 2

/* flags for map calls */
#define TCW_FLAG_LNBTSG 0x1       /* compute lnBtSG (tcw:196-217) */
#define TCW_FLAG_POSTERIORS 0x2   /* t0/tau max-posterior indices (tcw:219-287); needs a map */
#define TCW_FLAG_FP64_DET 0x4     /* determinant D in native FP64 instead of FP32 double-word */
#define TCW_FLAG_UNCOMPENSATED 0x8 /* plain FP32 sums and D (precision studies only) */

/* Per-map / per-template result. */
typedef struct {
  double lnBtSG;      /* ln(70/(N_t0 N_tau)) + ln sum_mn exp(F_mn), FP64 */
  int64_t argmax;     /* flat index m*N_tau + n of maxF, first occurrence */
  int64_t t0_mp_idx;  /* argmax_m sum_n exp(F_mn - maxF) (TCW_FLAG_POSTERIORS) */
  int64_t tau_mp_idx; /* argmax_n sum_m exp(F_mn - maxF) (TCW_FLAG_POSTERIORS) */
  float maxF;         /* max F (not 2F) */
  int32_t status;     /* 0 */
} tcw_result;

/* One template of a batched call. */
typedef struct {
  uint64_t atom_offset; /* first row of this template in the concatenated atoms */
  uint64_t t0_offset;   /* first entry in the concatenated t0 grid */
  uint64_t tau_offset;  /* first entry in the concatenated tau grid */
  uint32_t numAtoms;
  uint32_t TAtom;
  uint32_t t0_data;
  int32_t window;       /* TCW_WINDOW_RECT or TCW_WINDOW_EXP */
  uint32_t N_t0;
  uint32_t N_tau;
} tcw_template_desc;

/* Tile shapes of a batched plan (0 = library default / autotuned). */
typedef struct {
  uint32_t rect_tn;       /* columns per rect tile (any >= 1) */
  uint32_t rect_tm;       /* rows per rect tile: 32, 64 or 128 (one thread per row) */
  uint32_t exp_tn;        /* columns per exp block: 32, 64 or 128 (single-template
                             calls; batched plans run 32-column warp tiles) */
  uint32_t exp_rows;      /* rows per exp thread chunk (0 = whole column) */
  uint32_t blocks_per_sm; /* cap on persistent blocks per SM (occupancy limits it too) */
} tcw_tile_config;

typedef struct tcw_handle tcw_handle;
typedef struct tcw_plan tcw_plan;

int tcw_abi_version(void);
const char *tcw_strerror(int status);
const char *tcw_last_error(const tcw_handle *h);

/* Device discovery (replaces the pycuda device probing of tcw:419-470). */
int tcw_device_count(int *count);
int tcw_device_info(int device, char *name, size_t name_len, int *cc_major, int *cc_minor,
                    size_t *total_mem);
/* Free and total device memory of `device` (cudaMemGetInfo; replaces the
 * pycuda mem_get_info of _print_GPU_memory_MB, tcw:648-653).  The calling
 * thread's current device is restored. */
int tcw_device_memory(int device, size_t *free_bytes, size_t *total_bytes);

/* Handle: owns a CUDA stream and a grow-only device workspace on `device`
 * (the pycuda context of tcw:419-470 and its per-call allocations,
 * tcw:861-912).  tcw_set_stream takes a caller's cudaStream_t, NULL for the
 * handle's own stream, or cudaStreamLegacy for the legacy default stream.
 * tcw_create returns TCW_ERR_NO_DEVICE unless `device` has compute
 * capability 10.3: the kernels are built for sm_103a only. */
int tcw_create(tcw_handle **h, int device);
int tcw_destroy(tcw_handle *h);
int tcw_get_stream(tcw_handle *h, void **stream);
int tcw_set_stream(tcw_handle *h, void *stream);
int tcw_sync(tcw_handle *h, int timeout_ms);     /* TCW_ERR_TIMEOUT if not done in time */
/* Page-locked host memory (cudaHostAlloc / cudaFreeHost) for the asynchronous
 * host-buffer entry points: copies from or into pageable memory make the
 * calling thread wait for the copy.  A helper with no reference counterpart. */
int tcw_pinned_alloc(void **ptr, size_t bytes);
int tcw_pinned_free(void *ptr);

/* Plain per-template map on device buffers.  d_Fmn may be NULL (no map is
 * written; TCW_FLAG_POSTERIORS then needs a map and is rejected).  d_result
 * is one device tcw_result.  Replaces pycuda_compute_transient_fstat_map
 * (tcw:656-834) with its rect / exp launches (tcw:837-916, :919-998). */
int tcw_map_plain(tcw_handle *h, const float *d_atoms, uint32_t numAtoms, uint32_t TAtom,
                  uint32_t t0_data, int window, const uint32_t *d_t0s, uint32_t N_t0,
                  const uint32_t *d_taus, uint32_t N_tau, float *d_Fmn, tcw_result *d_result,
                  int flags);

/* The same with host buffers: copies in, computes, copies out, synchronises
 * -- one call of pycuda_compute_transient_fstat_map's kernel part
 * (tcw:837-916, :919-998) with its host reductions (tcw:810-828); window
 * TCW_WINDOW_NONE is one rectangular cell over all data (tcw:742-749). */
int tcw_map_plain_host(tcw_handle *h, const float *atoms, uint32_t numAtoms, uint32_t TAtom,
                       uint32_t t0_data, int window, const uint32_t *t0s, uint32_t N_t0,
                       const uint32_t *taus, uint32_t N_tau, float *Fmn, tcw_result *result,
                       int flags);

/* Batched form (no per-template map): a plan fixes the templates' geometry
 * and grids and the tile schedule; runs take atoms and give one result per
 * template.  Replaces the per-template loop of a transient grid search
 * (grid_based_searches.py:1186-1189) over call_compute_transient_fstat_map. */
int tcw_plan_create(tcw_handle *h, const tcw_template_desc *desc, uint32_t n_templates,
                    const uint32_t *t0s, uint64_t n_t0s, const uint32_t *taus, uint64_t n_taus,
                    const tcw_tile_config *cfg, int flags, tcw_plan **plan);
int tcw_plan_destroy(tcw_plan *plan);
int tcw_plan_info(const tcw_plan *plan, uint64_t *n_cells, uint32_t *n_items,
                  uint64_t *n_atom_rows, tcw_tile_config *cfg);
/* use_graph != 0: the first run captures the launch sequence into a CUDA
 * graph owned by the plan; later runs replay it (same d_atoms/d_results
 * pointers required; different pointers re-capture).  On the legacy default
 * stream (cudaStreamLegacy) runs are launched without a graph. */
int tcw_plan_run(tcw_handle *h, tcw_plan *plan, const float *d_atoms, tcw_result *d_results,
                 int use_graph);
int tcw_plan_run_host(tcw_handle *h, tcw_plan *plan, const float *atoms, tcw_result *results);
/* As tcw_plan_run_host without waiting: the upload of `atoms` runs on the
 * handle's copy stream and starts once the previous pipelined run on this
 * handle has read its atoms (after its prefix and repack kernels), so it
 * overlaps that run's map kernels; the results are copied back on the
 * handle's stream.  `atoms` must stay unchanged and `results` unread until
 * tcw_sync(h, ...) returns.  Both should be page-locked (tcw_pinned_alloc):
 * with pageable `results` the download makes the caller wait for the run,
 * and nothing overlaps.  Not for plans created with TCW_FLAG_POSTERIORS.  A
 * pipelining addition for streams of batches (no reference counterpart). */
int tcw_plan_run_host_async(tcw_handle *h, tcw_plan *plan, const float *atoms,
                            tcw_result *results);
/* As tcw_plan_run, and also writes every template's FP32 map: template k's
 * (N_t0, N_tau) row-major map starts at d_maps + sum_{j<k} N_t0(j) N_tau(j)
 * (descriptor order; tcw_plan_info's n_cells floats in all).  Replaces the
 * per-template map downloads of the reference's callers (tcw:810-815 and
 * core.py:1534-1540 read cells of full maps). */
int tcw_plan_run_maps(tcw_handle *h, tcw_plan *plan, const float *d_atoms, tcw_result *d_results,
                      float *d_maps, int use_graph);
/* Host-buffer form of tcw_plan_run_maps: host atoms in, results and all maps
 * (tcw_plan_info's n_cells floats) out; synchronises.  A plan created with
 * TCW_FLAG_POSTERIORS fills t0_mp_idx / tau_mp_idx of every result from the
 * maps (tcw:219-287); such a plan only runs through the _maps entry points. */
int tcw_plan_run_maps_host(tcw_handle *h, tcw_plan *plan, const float *atoms, tcw_result *results,
                           float *maps);
/* One-shot batched call on host buffers (plan, run, results, release):
 * per template max2F (2 maxF), the flat argmax and lnBtSG -- the batched
 * entry a transient grid search calls once instead of one map per Doppler
 * point (grid_based_searches.py:1186-1189).  Output arrays hold n_templates
 * values; cfg may be NULL (library tiles). */
int tcw_map_batched(tcw_handle *h, const tcw_template_desc *desc, uint32_t n_templates,
                    const uint32_t *t0s, uint64_t n_t0s, const uint32_t *taus, uint64_t n_taus,
                    const float *atoms_concat, const tcw_tile_config *cfg, float *max2F,
                    int64_t *argmax, double *lnBtSG);
/* One run without a graph and with the two map kernels one after the other,
 * CUDA events between the kernels on the handle's stream; synchronises and
 * writes the durations (ms) of the prefix, rectangular-map, exponential-map
 * and finalize kernels to ms[0..3].  For measurement. */
int tcw_plan_run_timed(tcw_handle *h, tcw_plan *plan, const float *d_atoms, tcw_result *d_results,
                       float *ms);

/* Differentiable maps, exponential or rectangular windows (desc.window) --
 * no counterpart in the reference: an
 * addition for gradient-based searches.  Per template the tau grid is
 * continuous, tau_n = tau_min + n (tau_max - tau_min) / (N_tau - 1); the
 * t0 grid (host array, seconds) must be non-decreasing and start no earlier
 * than t0_data - TAtom/2.  Outputs per template: lnBtSG (ln(70/(N_t0 N_tau))
 * + logsumexp F) and softmax2F = T logsumexp(2F/T).  F is evaluated in FP64
 * here (gradients of the T = 0.1 soft-max need F to ~1e-9). */
typedef struct {
  uint64_t atom_offset; /* first row of this template in the concatenated atoms */
  uint64_t t0_offset;   /* first entry in the concatenated t0 grid */
  uint32_t numAtoms;
  uint32_t TAtom;
  uint32_t t0_data;
  uint32_t N_t0;
  uint32_t N_tau;
  uint32_t window;      /* TCW_WINDOW_EXP (or 0) or TCW_WINDOW_RECT */
  double tau_min;
  double tau_max;
} tcw_diff_desc;

int tcw_map_forward(tcw_handle *h, const tcw_diff_desc *desc, uint32_t n_templates,
                    const float *d_atoms, const uint32_t *t0s, uint64_t n_t0s,
                    double temperature, double *d_lnBtSG, double *d_softmax2F);
/* Gradients of L(lnBtSG, softmax2F) given dL/dlnBtSG and dL/dsoftmax2F per
 * template (device arrays) and the forward's outputs: d_grad_atoms
 * (n_atom_rows x 7, FP64, overwritten) and d_grad_tau (n_templates x 2:
 * dL/dtau_min, dL/dtau_max, overwritten).  Recomputes the window sums. */
int tcw_map_backward(tcw_handle *h, const tcw_diff_desc *desc, uint32_t n_templates,
                     const float *d_atoms, const uint32_t *t0s, uint64_t n_t0s,
                     double temperature, const double *d_lnBtSG, const double *d_softmax2F,
                     const double *d_grad_lnBtSG, const double *d_grad_softmax2F,
                     double *d_grad_atoms, uint64_t n_atom_rows, double *d_grad_tau);

/* Device-side index checks of a debug build (compiled with -DTCW_DEBUG_CHECKS:
 * every index of a map / adjoint / reference kernel load or store is checked
 * and a failure is counted, never trapped).  Writes the number of failed checks
 * since the library was loaded; returns TCW_ERR_UNSUPPORTED (count 0) in
 * builds without the checks.  A debugging utility; no reference counterpart. */
int tcw_debug_check_failures(uint32_t *count);

/* Full-FP64 map by direct summation over each cell's window (FP64 weights
 * and sums, FP64 F with the reference's conditioning test, no recurrence and
 * no compensation): the GPU reference for precision reports.  Device
 * atoms/grids as in tcw_map_plain; `rows` is a HOST list of n_rows t0 indices
 * (each < N_t0; NULL = all rows, then n_rows == N_t0).  Writes
 * d_F[r * N_tau + n] for the r-th listed row, and the condition number to
 * d_cond (nullable).  Cost: one FP64 FMA per channel per atom of each window.
 * A precision utility; it has no counterpart in the reference, whose own
 * FP64 path is the 'lal' version (tcw:547-587). */
int tcw_map_f64(tcw_handle *h, const float *d_atoms, uint32_t numAtoms, uint32_t TAtom,
                uint32_t t0_data, int window, const uint32_t *d_t0s, uint32_t N_t0,
                const uint32_t *d_taus, uint32_t N_tau, const uint32_t *rows, uint32_t n_rows,
                double *d_F, double *d_cond);

/* ---- file formats (host only, no device or handle) ---- */

/* Text map body in the lalpulsar write_transientFstatMap_to_fp layout, one
 * line "  %10d %10d %- 11.8g\n" of (t0s[m], taus[n], 2 F[m, n]) per cell in
 * row-major order; header lines are the caller's (append != 0 appends).
 * Replaces the Python line loop of write_F_mn_to_file (tcw:289-317). */
int tcw_write_map_text(const char *path, const float *F, uint32_t N_t0, uint32_t N_tau,
                       const uint32_t *t0s, const uint32_t *taus, int append);
/* Columns (t0, tau, 2F) of a text map ('#' comment lines skipped), as read by
 * read_from_file (tcw:159-184).  With NULL outputs only counts the lines into
 * *n_lines; otherwise fills up to `capacity` lines (TCW_ERR_OVERFLOW beyond). */
int tcw_read_map_text(const char *path, uint64_t *n_lines, double *t0, double *tau, double *twoF,
                      uint64_t capacity);
/* F-statistic atoms text ('%' comment lines skipped; columns tGPS a2 b2 ab
 * Fa_re Fa_im Fb_re Fb_im, the file of core.py:1879-1910 as checked by
 * tests/test_core.py:811-826): timestamps and (n, 7) float32 rows, two-call
 * pattern as tcw_read_map_text. */
int tcw_read_atoms_text(const char *path, uint64_t *n_rows, uint32_t *timestamps, float *atoms7,
                        uint64_t capacity);
/* Writes atoms in the same column layout (header line "%% tGPS a2 b2 ab
 * Fa_re Fa_im Fb_re Fb_im", values with 9 significant digits). */
int tcw_write_atoms_text(const char *path, const uint32_t *timestamps, const float *atoms7,
                         uint64_t n_rows, int append);

/* Measured throughput of `device` for roofline denominators: FP32 and FP64
 * FMA in TFLOP/s (an FMA counts 2), MUFU ex2 in Tops/s, FP32 through packed
 * f32x2 FMAs in TFLOP/s.  A measurement utility; it has no counterpart in the
 * reference. */
int tcw_probe_peaks(int device, double *fp32_tflops, double *fp64_tflops, double *mufu_tops,
                    double *fp32x2_tflops);

/* Scratch size of tcw_map_plain_noalloc (bytes). */
#define TCW_NOALLOC_SCRATCH_BYTES (16u << 20)

/* The plain per-template map for callers that may not allocate device
 * memory (no cudaMalloc / cudaFree and no allocating library routine is
 * called).  It has no counterpart in the reference.  Same arguments, results
 * and flags as tcw_map_plain, with a stream (cudaStream_t, NULL for the
 * legacy default stream) instead of a handle; runs on the current device.
 * Its scratch is one static device array of TCW_NOALLOC_SCRATCH_BYTES that
 * every GPU loading this library holds until the process exits.  A problem
 * needing more -- 256-byte-aligned sections of 64 B x (numAtoms+1) prefix
 * rows (rect) or 32 B x numAtoms atom rows (exp), 56 B per tile, and with
 * TCW_FLAG_POSTERIORS 8 B x (N_t0 + ceil(N_t0/64) x N_tau) -- is rejected
 * with TCW_ERR_OVERFLOW.  The first call on a device looks the array's
 * address up and caches it per device: make it before any stream capture.
 * The cached address is that of the device's primary context (the one the
 * CUDA runtime uses); it is not valid after cudaDeviceReset of the device or
 * under another context made current through the driver API.  Calls share
 * the array: calls whose work overlaps on the GPU race and must be
 * serialised. */
int tcw_map_plain_noalloc(void *stream, const float *d_atoms, uint32_t numAtoms, uint32_t TAtom,
                          uint32_t t0_data, int window, const uint32_t *d_t0s, uint32_t N_t0,
                          const uint32_t *d_taus, uint32_t N_tau, float *d_Fmn,
                          tcw_result *d_result, int flags);

/* Test hook: make the n-th following workspace allocation on this handle
 * fail (n = 0 disables).  Host-side only; used to test error paths. */
int tcw_debug_fail_alloc(tcw_handle *h, int n);

#ifdef __cplusplus
}
#endif

#endif /* TCW_B200_H */
