// Full-FP64 transient map by direct summation: the GPU reference for
// precision reports at sizes the CPU cannot evaluate.
//
// Each cell's window sums are accumulated atom by atom in FP64 over the
// reference's window (pyfstat/pyCUDAkernels/cudaTransientFstatExpWindow.cu:
// 27-100 for exponential windows, cudaTransientFstatRectWindow.cu:21-91 for
// rectangular ones, index rules as in the map kernels), then F is formed in
// FP64 with the reference's conditioning test (Exp.cu:109-129).  No
// recurrence across cells, no compensation, no FP32 arithmetic: the
// exponential weight of a window's first atom is an FP64 exp and later
// weights are multiplied by r = exp(-TAtom / tau) (relative error below
// L * 2^-53 after L atoms).
//
// Layout: one thread per tau column, blocks of 128 columns of one t0 row;
// the block stages 128-atom tiles of the shared window in shared memory as
// FP64 and every thread consumes the part of the tile inside its window.

#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/tcw_b200.h"
#include "tcw_cell.h"
#include "tcw_internal.h"

namespace tcw {
namespace {

constexpr int kF64Block = 128;
constexpr int kF64Tile = 128;
constexpr uint32_t kF64RowsPerLaunch = 256;  // bounds one launch to well under a second

__device__ __forceinline__ double fstat_direct64(const double s[7], double &cond) {
  const double A = s[0], B = s[1], C = s[2];
  const double sumAB = A + B, diffAB = A - B;
  const double disc = sqrt(diffAB * diffAB + 4.0 * C * C);
  const double denom = sumAB - disc;
  cond = denom > 0.0 ? (sumAB + disc) / denom : INFINITY;
  const double DdInv = cond < 1e4 ? 1.0 / (A * B - C * C) : 0.0;
  if (!(DdInv > 0.0)) return 2.0;
  return DdInv * (B * (s[3] * s[3] + s[4] * s[4]) + A * (s[5] * s[5] + s[6] * s[6]) -
                  2.0 * C * (s[3] * s[5] + s[4] * s[6]));
}

template <int kWin>
__global__ void __launch_bounds__(kF64Block)
    map_f64_kernel(const float *__restrict__ atoms, Geom g, const uint32_t *__restrict__ t0s,
                   const uint32_t *__restrict__ taus, uint32_t N_tau,
                   const uint32_t *__restrict__ rows, uint32_t row0, uint32_t n_rows,
                   double *__restrict__ F, double *__restrict__ cond) {
  __shared__ double xs[7][kF64Tile];
  __shared__ uint32_t s_hi;
  const uint32_t r = row0 + blockIdx.y;
  if (r >= n_rows) return;
  const uint32_t m = rows ? rows[r] : r;
  const uint32_t t0 = t0s[m];
  const uint32_t n = blockIdx.x * kF64Block + threadIdx.x;
  const bool active = n < N_tau;
  const uint32_t tau = taus[active ? n : N_tau - 1u];

  // this column's atom range [lo, hi] (empty when hi < lo or !has)
  uint32_t lo, hi;
  bool has;
  if (kWin == TCW_WINDOW_EXP) {
    lo = exp_lo(t0, g);
    has = exp_hi(t0, tau, g, hi) && lo <= hi;
  } else {
    lo = idx_start(t0, g);
    const bool wrapped = rect_row_wrapped(t0, taus[0], g);
    const uint32_t end_first = idx_end(t0 + taus[0], g);
    hi = rect_end(t0, tau, end_first, wrapped, g);
    has = lo <= hi;
  }
  has = has && active;
  TCW_DCHECK(!has || hi < g.numAtoms);
  if (threadIdx.x == 0) s_hi = 0;
  __syncthreads();
  if (has) atomicMax(&s_hi, hi + 1u);
  __syncthreads();
  const uint32_t end = s_hi;  // block's last atom + 1 (0: no atoms)

  double s[7] = {0, 0, 0, 0, 0, 0, 0};
  double w = 0.0, rr = 0.0;
  if (kWin == TCW_WINDOW_EXP && has) {
    const double dtau = (double)tau;
    rr = exp(-(double)g.TAtom / dtau);
    const uint32_t t_lo = g.t0_data + lo * g.TAtom;
    w = exp(-(double)(t_lo - t0) / dtau);
  }
  for (uint32_t i0 = lo; i0 < end; i0 += kF64Tile) {
    __syncthreads();
    for (uint32_t k = threadIdx.x; k < 7u * kF64Tile; k += kF64Block) {
      const uint32_t a = i0 + k / 7u, c = k % 7u;
      xs[c][k / 7u] = a < g.numAtoms ? (double)atoms[(size_t)a * 7u + c] : 0.0;
    }
    __syncthreads();
    if (!has || i0 > hi) continue;
    const uint32_t kend = min((uint32_t)kF64Tile, hi + 1u - i0);
    if (kWin == TCW_WINDOW_EXP) {
      for (uint32_t k = 0; k < kend; k++) {
        const double w2 = w * w;
        s[0] = fma(xs[0][k], w2, s[0]);
        s[1] = fma(xs[1][k], w2, s[1]);
        s[2] = fma(xs[2][k], w2, s[2]);
        s[3] = fma(xs[3][k], w, s[3]);
        s[4] = fma(xs[4][k], w, s[4]);
        s[5] = fma(xs[5][k], w, s[5]);
        s[6] = fma(xs[6][k], w, s[6]);
        w *= rr;
      }
    } else {
      for (uint32_t k = 0; k < kend; k++) {
#pragma unroll
        for (int c = 0; c < 7; c++) s[c] += xs[c][k];
      }
    }
  }
  if (!active) return;
  double cd;
  const double f = fstat_direct64(s, cd);
  F[(size_t)r * N_tau + n] = f;
  if (cond) cond[(size_t)r * N_tau + n] = cd;
}

}  // namespace

cudaError_t launch_map_f64(int window, const float *atoms, const Geom &g, const uint32_t *t0s,
                           const uint32_t *taus, uint32_t N_tau, const uint32_t *rows,
                           uint32_t n_rows, double *F, double *cond, cudaStream_t stream) {
  const uint32_t gx = (N_tau + kF64Block - 1) / kF64Block;
  for (uint32_t row0 = 0; row0 < n_rows; row0 += kF64RowsPerLaunch) {
    const dim3 grid(gx, min(kF64RowsPerLaunch, n_rows - row0));
    if (window == TCW_WINDOW_EXP)
      map_f64_kernel<TCW_WINDOW_EXP><<<grid, kF64Block, 0, stream>>>(atoms, g, t0s, taus, N_tau,
                                                                      rows, row0, n_rows, F, cond);
    else
      map_f64_kernel<TCW_WINDOW_RECT><<<grid, kF64Block, 0, stream>>>(
          atoms, g, t0s, taus, N_tau, rows, row0, n_rows, F, cond);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace tcw

namespace tcw {
// Failed debug checks of this file's kernels (0 unless built with TCW_DEBUG_CHECKS).
unsigned int dcheck_failures_f64() {
#if defined(TCW_DEBUG_CHECKS)
  return tcw_dcheck_read();
#else
  return 0;
#endif
}
}  // namespace tcw
