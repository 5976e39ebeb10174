// Internal device-side data structures shared by the kernels and the C-ABI
// layer.  Not part of the public interface (include/tcw_b200.h).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "tcw_cell.h"

namespace tcw {

constexpr int kBlock = 128;  // threads per map block

enum PrecisionMode : int {
  kPrecFF = 0,        // double-word window sums, FP32 error-free D (default)
  kPrecFF_F64Det = 1, // double-word window sums, native FP64 D
  kPrecPlain32 = 2,   // uncompensated FP32 (precision report only)
};

// One template as the kernels see it.  Offsets index the concatenated
// arrays of a call: atoms in rows of 7 floats, grids in u32 entries, prefix
// rows of 16 floats, the output map in floats, per-item partials.
struct TemplateDev {
  uint64_t atom_off;
  uint64_t t0_off;
  uint64_t tau_off;
  uint64_t p_off;
  uint64_t a8_off;  // exp templates: first row in the 8-float atom rows
  uint64_t map_off;
  Geom g;
  uint32_t window;  // 1 rect, 2 exp
  uint32_t N_t0, N_tau;
  uint32_t part_off, n_parts;
  uint32_t pad;
  uint64_t row_off, col_off;  // posterior row partials / column sums (plans with posteriors)
};

// A tile of one template: rows [m0, m1) x columns [n0, n1).  For a
// rectangular tile the block's threads are (tn columns) x (128/tn row lanes);
// for an exponential tile each thread runs one column over a row chunk of
// `rows_per_lane` rows.
struct WorkItem {
  uint32_t tmpl;
  uint32_t part;
  uint32_t m0, m1;
  uint32_t n0, n1;
  uint16_t tn;            // columns per block (32, 64 or 128)
  uint16_t rows_per_lane; // exp only: rows per thread chunk
  uint32_t pad;
};

// Per-item reduction result.  s = sum over the item's cells of exp(F - maxF).
struct Partial {
  float maxF;
  uint32_t pad;
  int64_t argmax;  // flat m*N_tau + n, smallest index among ties
  double s;
};

#if defined(__CUDACC__)
// One template's atoms (rows of 7 floats, x) into 32-byte rows
// [a2 b2 ab nz Fa_re Fa_im Fb_re Fb_im] (o), by one block of 256 threads;
// nz (as u32 bits) is the lowest atom index >= i with a2 or b2 non-zero
// (0xFFFFFFFF: none).  Each thread owns a contiguous chunk of atoms and walks
// it backwards, starting from the first non-zero atom of the chunks above it.
__device__ __forceinline__ void repack_rows256(const float *__restrict__ x,
                                               float4 *__restrict__ o, uint32_t N,
                                               uint32_t *s_first) {
  const uint32_t tid = threadIdx.x;
  const uint32_t chunk = (N + 255u) / 256u;
  const uint32_t i0 = min(N, tid * chunk), i1 = min(N, i0 + chunk);
  uint32_t first = 0xFFFFFFFFu;
  for (uint32_t i = i0; i < i1; i++) {
    const float *r = x + (size_t)i * 7u;
    if (__ldg(r) != 0.0f || __ldg(r + 1) != 0.0f) {
      first = i;
      break;
    }
  }
  s_first[tid] = first;
  __syncthreads();
  uint32_t nz = 0xFFFFFFFFu;
  for (uint32_t k = tid + 1u; k < 256u; k++) {
    if (s_first[k] != 0xFFFFFFFFu) {
      nz = s_first[k];
      break;
    }
  }
  for (uint32_t i = i1; i > i0;) {
    i--;
    const float *r = x + (size_t)i * 7u;
    const float a2 = __ldg(r), b2 = __ldg(r + 1);
    if (a2 != 0.0f || b2 != 0.0f) nz = i;
    o[2u * i] = make_float4(a2, b2, __ldg(r + 2), __uint_as_float(nz));
    o[2u * i + 1u] = make_float4(__ldg(r + 3), __ldg(r + 4), __ldg(r + 5), __ldg(r + 6));
  }
}
#endif

// Launchers (tcw_kernels.cu).  All asynchronous on `stream`.
cudaError_t launch_prefix(const TemplateDev *d_T, const uint32_t *d_rect_list, uint32_t n_rect,
                          const float *d_atoms, float *d_P, int prec, cudaStream_t stream);
// Exp templates' atoms (rows of 7 floats) into rows of 8 (zero-padded).
cudaError_t launch_repack(const TemplateDev *d_T, const uint32_t *d_exp_list, uint32_t n_exp,
                          const float *d_atoms, float *d_atoms8, cudaStream_t stream);
struct MapLaunch {
  const TemplateDev *T;
  const WorkItem *items;  // this window's tiles
  uint32_t n_items;
  uint32_t *counter;      // persistent launches: tile counter, zeroed before
  uint32_t n_blocks;      // persistent grid size
  bool persistent, write_map;
  int prec;
  int priority;           // stream-priority value of the launch
  const float *atoms;
  const float *atoms8;    // exp tiles: atoms in 32-byte rows
  const uint32_t *t0s, *taus;
  const float *P;
  float *Fmn;
  Partial *parts;
};
cudaError_t launch_map(int window, const MapLaunch &L, cudaStream_t stream);
// Resident blocks per SM of the persistent (map-less) kernel of a window.
int map_blocks_per_sm(int window, int prec);

cudaError_t launch_finalize(const TemplateDev *d_T, uint32_t n_templates, const Partial *d_parts,
                            void *d_results, cudaStream_t stream);
cudaError_t launch_posteriors(const TemplateDev *d_T, const float *d_Fmn, void *d_result,
                              double *d_rowsum, double *d_colsum, uint32_t N_t0,
                              uint32_t N_tau, cudaStream_t stream);

// ---------------------------------------------------------------- differentiable path
// One template with a continuous tau grid (tcw_diff.cu); rectangular
// templates own, in the backward pass, the difference rows of their atom
// gradient at p_off: (numAtoms + 1) rows of 8 doubles.
struct DiffTemplate {
  uint64_t atom_off, t0_off;
  Geom g;
  uint32_t N_t0, N_tau;
  double tau_min, tau_max;
  uint32_t part_off, n_parts;
  uint32_t window, pad;
  uint64_t p_off;
};
// A tile: columns [n0, n1) (at most 128) of one template, all rows.
struct DiffItem {
  uint32_t tmpl, part, n0, n1;
};
// Per-tile online log-sum-exp pairs of F and of 2F/T.
// floats per column and t0 row in the backward pass's per-block scratch
#define TCW_DIFF_SLOTS 9u

struct DiffPartial {
  double m1, s1, m2, s2;
};
struct DiffLaunch {
  const DiffTemplate *T;
  const DiffItem *items;
  uint32_t n_items, n_blocks;
  uint32_t *counter;
  const float *atoms;
  float *atoms8;                     // exponential templates' atoms in 32-byte rows
                                     // (same row index as `atoms`), written by the launch
  const uint32_t *exp_list;          // the exponential templates' indices
  uint32_t n_exp;
  const uint32_t *t0s;
  double temp;
  DiffPartial *parts;                // pass A output
  const double *lnZ1, *lnZ2, *gB, *gS;  // pass B inputs per template: lnBtSG, softmax2F,
                                        // dL/dlnBtSG, dL/dsoftmax2F
  float *scratch;                    // pass B/C: n_blocks x scratch_rows x TCW_DIFF_SLOTS x 128 floats
  uint32_t scratch_rows;
  double *grad_atoms, *grad_tau;     // pass B/C outputs (accumulated; zero them first)
  // rectangular templates: their tiles (rows [n0, n1) of one template),
  // counter and persistent blocks, the list of their template indices and
  // (backward) the difference rows of the atom gradient (zeroed by the caller)
  const DiffItem *rect_items;
  uint32_t n_rect_items, n_rect_blocks;
  uint32_t *rect_counter;
  const uint32_t *rect_list;
  uint32_t n_rect;
  double *D64;
};
int rect_diff_blocks_per_sm(int pass);
int diff_blocks_per_sm(int pass);
cudaError_t launch_diff(int pass, const DiffLaunch &L, cudaStream_t stream);
// Failed device-side debug checks per translation unit (TCW_DEBUG_CHECKS).
unsigned int dcheck_failures_kernels();
unsigned int dcheck_failures_diff();
unsigned int dcheck_failures_f64();
unsigned int dcheck_failures_noalloc();
// Posterior indices of every template of a plan from its written maps:
// per column chunk (template, first column; kPostCols columns) one block
// reads its part of the map once and stores its row partials
// (d_rowpart + row_off + chunk * N_t0), then one warp per template takes
// the argmaxes.
constexpr uint32_t kPostCols = 1024;
cudaError_t launch_plan_posteriors(const TemplateDev *d_T, uint32_t n_templates,
                                   const uint2 *d_chunks, uint32_t n_chunks, const float *d_maps,
                                   tcw_result *d_results, float *d_rowpart, double *d_colsum,
                                   cudaStream_t stream);
// Full-FP64 direct-summation map of rows rows[0..n_rows) (all rows when rows
// is NULL) into F[r * N_tau + n]; cond optional.
cudaError_t launch_map_f64(int window, const float *atoms, const Geom &g, const uint32_t *t0s,
                           const uint32_t *taus, uint32_t N_tau, const uint32_t *rows,
                           uint32_t n_rows, double *F, double *cond, cudaStream_t stream);
cudaError_t launch_diff_finalize(const DiffTemplate *T, uint32_t n_templates,
                                 const DiffPartial *parts, double temp, double *lnB, double *soft,
                                 cudaStream_t stream);

}  // namespace tcw
