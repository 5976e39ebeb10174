// Host harness for the reference's own pycuda kernels.  TEST INFRASTRUCTURE
// ONLY (builds oracle/_ref/libtcw_ref.so, which pins the FP32 port and is the
// "reference" CPU baseline where it can be built).
//
// The two kernel sources are NOT copied: they are #included from the read-only
// reference checkout whose path the Makefile passes in (REF_RECT / REF_EXP).
// The shim only supplies what nvcc would: __global__, and the blockDim /
// blockIdx / threadIdx built-ins (thread_local so OpenMP threads can each
// "launch" their own block).  Overloads are arranged like CUDA device code:
// exp(float) resolves to the float overload, sqrt(double) to the double one.
#include <cmath>
#include <cstdint>
#include <cstddef>
#ifdef _OPENMP
#include <omp.h>
#endif

using std::exp;
using std::sqrt;

namespace {
struct shim_dim3 {
  unsigned int x, y, z;
};
thread_local shim_dim3 blockDim = {1, 1, 1};
thread_local shim_dim3 blockIdx = {0, 0, 0};
thread_local shim_dim3 threadIdx = {0, 0, 0};
}  // namespace

#define __global__ static
#include REF_RECT
#include REF_EXP
#undef __global__

extern "C" {

// Rectangular window on a uniform windowRange grid.  The reference kernel
// guards rows with `m < N_tauRange` (Rect.cu:48), so a grid with more t0 rows
// than tau columns would leave rows unwritten; the harness therefore runs one
// row per call with win_t0 shifted to that row and the output pointer offset
// by m * N_tau, which is the map the kernel would give without the guard.
int ref_rect_uniform(float *atoms7, unsigned numAtoms, unsigned TAtom,
                     unsigned t0_data, unsigned win_t0, unsigned win_dt0,
                     unsigned win_tau, unsigned win_dtau, unsigned N_t0,
                     unsigned N_tau, float *Fmn, int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
#pragma omp parallel for schedule(dynamic, 4)
  for (long m = 0; m < (long)N_t0; m++) {
    blockDim = {1, 1, 1};
    blockIdx = {0, 0, 0};
    threadIdx = {0, 0, 0};
    cudaTransientFstatRectWindow(atoms7, numAtoms, TAtom, t0_data,
                                 win_t0 + (unsigned)m * win_dt0, win_dt0,
                                 win_tau, win_dtau, N_tau,
                                 Fmn + (size_t)m * N_tau);
  }
  return 0;
}

// Exponential window on a uniform windowRange grid: one "thread" per cell.
int ref_exp_uniform(float *atoms7, unsigned numAtoms, unsigned TAtom,
                    unsigned t0_data, unsigned win_t0, unsigned win_dt0,
                    unsigned win_tau, unsigned win_dtau, unsigned N_t0,
                    unsigned N_tau, float *Fmn, int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
#pragma omp parallel for collapse(2) schedule(dynamic, 16)
  for (long m = 0; m < (long)N_t0; m++) {
    for (long n = 0; n < (long)N_tau; n++) {
      blockDim = {1, 1, 1};
      blockIdx = {(unsigned)m, (unsigned)n, 0};
      threadIdx = {0, 0, 0};
      cudaTransientFstatExpWindow(atoms7, numAtoms, TAtom, t0_data, win_t0,
                                  win_dt0, win_tau, win_dtau, N_t0, N_tau, Fmn);
    }
  }
  return 0;
}

// Either window on an explicit list of cells (t0s[k], taus[k]): one
// single-cell launch per entry (window 1 = rect, 2 = exp).  A fresh
// single-cell rect launch sums atoms i_t0..i_t1 in the same order as the
// running sum of a full row, so results equal the uniform-grid launches.
int ref_cells(float *atoms7, unsigned numAtoms, unsigned TAtom,
              unsigned t0_data, int window, const unsigned *t0s,
              const unsigned *taus, long ncells, float *F, int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
#pragma omp parallel for schedule(dynamic, 64)
  for (long k = 0; k < ncells; k++) {
    blockDim = {1, 1, 1};
    blockIdx = {0, 0, 0};
    threadIdx = {0, 0, 0};
    if (window == 1)
      cudaTransientFstatRectWindow(atoms7, numAtoms, TAtom, t0_data, t0s[k], 0,
                                   taus[k], 0, 1, F + k);
    else
      cudaTransientFstatExpWindow(atoms7, numAtoms, TAtom, t0_data, t0s[k], 0,
                                  taus[k], 0, 1, 1, F + k);
  }
  return 0;
}

}  // extern "C"
