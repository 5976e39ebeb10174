/*
 * CPU oracle for the transient-CW F-statistic map.  TEST INFRASTRUCTURE ONLY:
 * tests, the smoke check and the CPU-baseline leg of the benchmark use it as
 * the checker; the product path never links or calls it.
 *
 * Two restatements of the per-cell algorithm of PyFstat's pycuda kernels
 * (pyfstat/pyCUDAkernels/cudaTransientFstatRectWindow.cu and
 *  pyfstat/pyCUDAkernels/cudaTransientFstatExpWindow.cu):
 *
 *   *_f32 : the reference arithmetic, operation for operation, in FP32 with
 *           the same implicit FP64 promotions (double literals 4.0, 1.0, 2.0)
 *           and the same sequential accumulation order.  Built with
 *           -ffp-contract=off it reproduces the kernels compiled for the
 *           host bit for bit (pinned by tests against oracle/_ref).
 *           This is the "port" CPU baseline.
 *   *_f64 : the same per-cell math with every quantity in FP64 (window sums,
 *           weights, conditioning test, determinant, F).  This is the parity
 *           arbiter for the GPU path.
 *
 * Index arithmetic follows the reference exactly, including its unsigned
 * 32-bit wrap-around (Rect.cu:21-31, :54-69; Exp.cu:27-66).
 *
 * Grids are explicit arrays t0s[N_t0], taus[N_tau] (seconds, u32), which
 * generalise lalpulsar's uniform transientWindowRange_t
 * (t0 + m*dt0, tau + n*dtau; tcw_fstat_map_funcs.py:775-780).
 */
#include <math.h>
#include <stdint.h>
#include <stddef.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define TCWO_WIN_RECT 1
#define TCWO_WIN_EXP 2
#define TCWO_EXP_EFOLDING 3u /* Exp.cu:22, copied from lalpulsar */

/* Rect.cu:21-31: i_t0 = clamp(floor((t0 - t0_data + TAtom/2)/TAtom), 0, numAtoms-1)
 * with u32 arithmetic and the quotient assigned to a signed int. */
static inline uint32_t idx_start(uint32_t t0, uint32_t t0_data, uint32_t TAtom,
                                 uint32_t numAtoms) {
  uint32_t half = TAtom / 2u;
  uint32_t q = (t0 - t0_data + half) / TAtom;
  int32_t i = (int32_t)q;
  if (i < 0) i = 0;
  uint32_t u = (uint32_t)i;
  if (u >= numAtoms) u = numAtoms - 1u;
  return u;
}

/* Rect.cu:54-69: i_t1 = clamp(floor((t1 - t0_data + TAtom/2)/TAtom) - 1, 0, numAtoms-1);
 * the "- 1" is applied to the unsigned quotient (wraps to 0xFFFFFFFF -> -1). */
static inline uint32_t idx_end(uint32_t t1, uint32_t t0_data, uint32_t TAtom,
                               uint32_t numAtoms) {
  uint32_t half = TAtom / 2u;
  uint32_t q = (t1 - t0_data + half) / TAtom - 1u;
  int32_t i = (int32_t)q;
  if (i < 0) i = 0;
  uint32_t u = (uint32_t)i;
  if (u >= numAtoms) u = numAtoms - 1u;
  return u;
}

/* Rect.cu:93-118 / Exp.cu:104-129 in the reference's mixed FP32/FP64 arithmetic. */
static inline float fstat_ref_f32(float Ad, float Bd, float Cd, float Fa_re,
                                  float Fa_im, float Fb_re, float Fb_im) {
  float sumAB = Ad + Bd;
  float diffAB = Ad - Bd;
  double discArg = (double)(diffAB * diffAB) + (4.0 * (double)Cd) * (double)Cd;
  float disc = (float)sqrt(discArg);
  float denom = sumAB - disc;
  float cond = (denom > 0) ? ((sumAB + disc) / denom) : INFINITY;
  float DdInv = 0.0f;
  if ((double)cond < 1e4) {
    float det = Ad * Bd - Cd * Cd;
    DdInv = (float)(1.0 / (double)det);
  }
  float F = 2.0f;
  if (DdInv > 0) {
    float t1 = Bd * (Fa_re * Fa_re + Fa_im * Fa_im);
    float t2 = Ad * (Fb_re * Fb_re + Fb_im * Fb_im);
    float t12 = t1 + t2;
    float re = Fa_re * Fb_re + Fa_im * Fb_im;
    double inner = (double)t12 - (2.0 * (double)Cd) * (double)re;
    F = (float)((double)DdInv * inner);
  }
  return F;
}

/* The same conditioning test and F in FP64 throughout. */
static inline double fstat_f64(double A, double B, double C, double Fa_re,
                               double Fa_im, double Fb_re, double Fb_im,
                               double *cond_out) {
  double sumAB = A + B;
  double diffAB = A - B;
  double disc = sqrt(diffAB * diffAB + 4.0 * C * C);
  double denom = sumAB - disc;
  double cond = (denom > 0) ? ((sumAB + disc) / denom) : INFINITY;
  if (cond_out) *cond_out = cond;
  double DdInv = 0.0;
  if (cond < 1e4) DdInv = 1.0 / (A * B - C * C);
  double F = 2.0;
  if (DdInv > 0) {
    F = DdInv * (B * (Fa_re * Fa_re + Fa_im * Fa_im) +
                 A * (Fb_re * Fb_re + Fb_im * Fb_im) -
                 2.0 * C * (Fa_re * Fb_re + Fa_im * Fb_im));
  }
  return F;
}

static int check_args(const float *atoms, uint32_t numAtoms, uint32_t TAtom,
                      const uint32_t *t0s, uint32_t N_t0, const uint32_t *taus,
                      uint32_t N_tau) {
  if (!atoms || !t0s || !taus) return -1;
  if (numAtoms == 0 || TAtom == 0 || N_t0 == 0 || N_tau == 0) return -2;
  return 0;
}

static void set_threads(int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
}

/* ---------------------------------------------------------------- FP32 port */

/* Rectangular window, reference semantics (Rect.cu:16-128): per row a running
 * FP32 sum that is extended from i_t1_last to i_t1 as tau grows. */
int tcwo_rect_map_f32(const float *atoms, uint32_t numAtoms, uint32_t TAtom,
                      uint32_t t0_data, const uint32_t *t0s, uint32_t N_t0,
                      const uint32_t *taus, uint32_t N_tau, float *Fmn,
                      int nthreads) {
  int rc = check_args(atoms, numAtoms, TAtom, t0s, N_t0, taus, N_tau);
  if (rc) return rc;
  set_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 4)
  for (int64_t m = 0; m < (int64_t)N_t0; m++) {
    uint32_t t0 = t0s[m];
    uint32_t i_t0 = idx_start(t0, t0_data, TAtom, numAtoms);
    float Ad = 0, Bd = 0, Cd = 0, Far = 0, Fai = 0, Fbr = 0, Fbi = 0;
    uint32_t last = i_t0;
    for (uint32_t n = 0; n < N_tau; n++) {
      uint32_t t1 = t0 + taus[n];
      uint32_t i_t1 = idx_end(t1, t0_data, TAtom, numAtoms);
      for (uint32_t i = last; i <= i_t1; i++) {
        const float *x = atoms + (size_t)i * 7u;
        Ad += x[0];
        Bd += x[1];
        Cd += x[2];
        Far += x[3];
        Fai += x[4];
        Fbr += x[5];
        Fbi += x[6];
        last = i_t1 + 1u;
      }
      Fmn[(size_t)m * N_tau + n] = fstat_ref_f32(Ad, Bd, Cd, Far, Fai, Fbr, Fbi);
    }
  }
  return 0;
}

/* Exponential window, reference semantics (Exp.cu:16-134): a direct sum over
 * [i_t0, i_t1] with FP32 weights expf(-x), x = (float)((double)(t_i-t0)/tau). */
int tcwo_exp_map_f32(const float *atoms, uint32_t numAtoms, uint32_t TAtom,
                     uint32_t t0_data, const uint32_t *t0s, uint32_t N_t0,
                     const uint32_t *taus, uint32_t N_tau, float *Fmn,
                     int nthreads) {
  int rc = check_args(atoms, numAtoms, TAtom, t0s, N_t0, taus, N_tau);
  if (rc) return rc;
  set_threads(nthreads);
#pragma omp parallel for collapse(2) schedule(dynamic, 16)
  for (int64_t m = 0; m < (int64_t)N_t0; m++) {
    for (int64_t n = 0; n < (int64_t)N_tau; n++) {
      uint32_t t0 = t0s[m];
      uint32_t i_t0 = idx_start(t0, t0_data, TAtom, numAtoms);
      uint32_t tau = taus[n];
      uint32_t t1 = t0 + TCWO_EXP_EFOLDING * tau;
      uint32_t i_t1 = idx_end(t1, t0_data, TAtom, numAtoms);
      float Ad = 0, Bd = 0, Cd = 0, Far = 0, Fai = 0, Fbr = 0, Fbi = 0;
      for (uint32_t i = i_t0; i <= i_t1; i++) {
        uint32_t t_i = t0_data + i * TAtom;
        float w = 0.0f;
        if (t_i >= t0 && t_i <= t1) {
          float x = (float)((1.0 * (double)(t_i - t0)) / (double)tau);
          w = expf(-x);
        }
        float w2 = w * w;
        const float *x = atoms + (size_t)i * 7u;
        Ad += x[0] * w2;
        Bd += x[1] * w2;
        Cd += x[2] * w2;
        Far += x[3] * w;
        Fai += x[4] * w;
        Fbr += x[5] * w;
        Fbi += x[6] * w;
      }
      Fmn[(size_t)m * N_tau + n] = fstat_ref_f32(Ad, Bd, Cd, Far, Fai, Fbr, Fbi);
    }
  }
  return 0;
}

/* ---------------------------------------------------------------- FP64 arbiter */

/* Window sums in FP64 for one cell; weights in FP64.  Returns F, writes cond. */
static double cell_f64(const float *atoms, uint32_t numAtoms, uint32_t TAtom,
                       uint32_t t0_data, int window, uint32_t t0, uint32_t tau,
                       double *cond) {
  uint32_t i_t0 = idx_start(t0, t0_data, TAtom, numAtoms);
  double s[7] = {0, 0, 0, 0, 0, 0, 0};
  if (window == TCWO_WIN_RECT) {
    uint32_t i_t1 = idx_end(t0 + tau, t0_data, TAtom, numAtoms);
    for (uint32_t i = i_t0; i <= i_t1; i++) {
      const float *x = atoms + (size_t)i * 7u;
      for (int c = 0; c < 7; c++) s[c] += (double)x[c];
    }
  } else {
    uint32_t t1 = t0 + TCWO_EXP_EFOLDING * tau;
    uint32_t i_t1 = idx_end(t1, t0_data, TAtom, numAtoms);
    for (uint32_t i = i_t0; i <= i_t1; i++) {
      uint32_t t_i = t0_data + i * TAtom;
      if (!(t_i >= t0 && t_i <= t1)) continue;
      double w = exp(-(double)(t_i - t0) / (double)tau);
      double w2 = w * w;
      const float *x = atoms + (size_t)i * 7u;
      for (int c = 0; c < 3; c++) s[c] += (double)x[c] * w2;
      for (int c = 3; c < 7; c++) s[c] += (double)x[c] * w;
    }
  }
  return fstat_f64(s[0], s[1], s[2], s[3], s[4], s[5], s[6], cond);
}

/* Full FP64 map.  cond may be NULL. */
int tcwo_map_f64(const float *atoms, uint32_t numAtoms, uint32_t TAtom,
                 uint32_t t0_data, int window, const uint32_t *t0s,
                 uint32_t N_t0, const uint32_t *taus, uint32_t N_tau,
                 double *Fmn, double *cond, int nthreads) {
  int rc = check_args(atoms, numAtoms, TAtom, t0s, N_t0, taus, N_tau);
  if (rc) return rc;
  if (window != TCWO_WIN_RECT && window != TCWO_WIN_EXP) return -3;
  set_threads(nthreads);
  if (window == TCWO_WIN_RECT) {
    /* running FP64 sums per row when the tau grid is non-decreasing */
    int mono = 1;
    for (uint32_t n = 1; n < N_tau; n++)
      if (taus[n] < taus[n - 1]) mono = 0;
    if (mono) {
#pragma omp parallel for schedule(dynamic, 4)
      for (int64_t m = 0; m < (int64_t)N_t0; m++) {
        uint32_t t0 = t0s[m];
        uint32_t i_t0 = idx_start(t0, t0_data, TAtom, numAtoms);
        double s[7] = {0, 0, 0, 0, 0, 0, 0};
        uint32_t last = i_t0;
        for (uint32_t n = 0; n < N_tau; n++) {
          uint32_t i_t1 = idx_end(t0 + taus[n], t0_data, TAtom, numAtoms);
          for (uint32_t i = last; i <= i_t1; i++) {
            const float *x = atoms + (size_t)i * 7u;
            for (int c = 0; c < 7; c++) s[c] += (double)x[c];
            last = i_t1 + 1u;
          }
          double cd;
          Fmn[(size_t)m * N_tau + n] =
              fstat_f64(s[0], s[1], s[2], s[3], s[4], s[5], s[6], &cd);
          if (cond) cond[(size_t)m * N_tau + n] = cd;
        }
      }
      return 0;
    }
  }
#pragma omp parallel for collapse(2) schedule(dynamic, 16)
  for (int64_t m = 0; m < (int64_t)N_t0; m++) {
    for (int64_t n = 0; n < (int64_t)N_tau; n++) {
      double cd;
      Fmn[(size_t)m * N_tau + n] =
          cell_f64(atoms, numAtoms, TAtom, t0_data, window, t0s[m], taus[n], &cd);
      if (cond) cond[(size_t)m * N_tau + n] = cd;
    }
  }
  return 0;
}

/* FP64 F for an arbitrary list of cells (t0s[k], taus[k]) -- spot checks of
 * maps too large for the full CPU oracle. */
int tcwo_cells_f64(const float *atoms, uint32_t numAtoms, uint32_t TAtom,
                   uint32_t t0_data, int window, const uint32_t *t0s,
                   const uint32_t *taus, uint64_t ncells, double *F,
                   double *cond, int nthreads) {
  if (!atoms || !t0s || !taus || !F) return -1;
  if (numAtoms == 0 || TAtom == 0) return -2;
  if (window != TCWO_WIN_RECT && window != TCWO_WIN_EXP) return -3;
  set_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t k = 0; k < (int64_t)ncells; k++) {
    double cd;
    F[k] = cell_f64(atoms, numAtoms, TAtom, t0_data, window, t0s[k], taus[k], &cd);
    if (cond) cond[k] = cd;
  }
  return 0;
}

/* FP64 window sums for a list of cells: out[k*7 + c] (A, B, C, Fa_re, Fa_im,
 * Fb_re, Fb_im).  Used by the gradient tests as the linear part of the map. */
int tcwo_cell_sums_f64(const float *atoms, uint32_t numAtoms, uint32_t TAtom,
                       uint32_t t0_data, int window, const uint32_t *t0s,
                       const uint32_t *taus, uint64_t ncells, double *out) {
  if (!atoms || !t0s || !taus || !out) return -1;
  if (numAtoms == 0 || TAtom == 0) return -2;
  for (uint64_t k = 0; k < ncells; k++) {
    uint32_t t0 = t0s[k], tau = taus[k];
    uint32_t i_t0 = idx_start(t0, t0_data, TAtom, numAtoms);
    double *s = out + k * 7u;
    for (int c = 0; c < 7; c++) s[c] = 0.0;
    uint32_t t1 = (window == TCWO_WIN_RECT) ? t0 + tau : t0 + TCWO_EXP_EFOLDING * tau;
    uint32_t i_t1 = idx_end(t1, t0_data, TAtom, numAtoms);
    for (uint32_t i = i_t0; i <= i_t1; i++) {
      const float *x = atoms + (size_t)i * 7u;
      double w = 1.0, w2 = 1.0;
      if (window == TCWO_WIN_EXP) {
        uint32_t t_i = t0_data + i * TAtom;
        if (!(t_i >= t0 && t_i <= t1)) continue;
        w = exp(-(double)(t_i - t0) / (double)tau);
        w2 = w * w;
      }
      for (int c = 0; c < 3; c++) s[c] += (double)x[c] * w2;
      for (int c = 3; c < 7; c++) s[c] += (double)x[c] * w;
    }
  }
  return 0;
}

/* Exponential window with a real-valued tau (the differentiable variant):
 * t1 = t0 + 3 tau in FP64; the end index is the reference's formula with t1
 * real, i_t1 = clamp(floor((t1 - t0_data + TAtom/2) / TAtom) - 1), and atoms
 * count while t0 <= t_i <= t1.  For integral tau (no u32 wrap) this is the
 * reference's window.  Returns F in FP64. */
static double cell_f64_realtau(const float *atoms, uint32_t numAtoms, uint32_t TAtom,
                               uint32_t t0_data, uint32_t t0, double tau, double *cond) {
  uint32_t i_t0 = idx_start(t0, t0_data, TAtom, numAtoms);
  double t1 = (double)t0 + 3.0 * tau;
  double s[7] = {0, 0, 0, 0, 0, 0, 0};
  if (t1 >= (double)t0_data) {
    double q = floor((t1 - (double)t0_data + (double)(TAtom / 2u)) / (double)TAtom) - 1.0;
    uint32_t i_t1 = q < 0.0 ? 0u : (q >= (double)(numAtoms - 1u) ? numAtoms - 1u : (uint32_t)q);
    for (uint32_t i = i_t0; i <= i_t1; i++) {
      double t_i = (double)t0_data + (double)i * (double)TAtom;
      if (!(t_i >= (double)t0 && t_i <= t1)) continue;
      double w = exp(-(t_i - (double)t0) / tau);
      double w2 = w * w;
      const float *x = atoms + (size_t)i * 7u;
      for (int c = 0; c < 3; c++) s[c] += (double)x[c] * w2;
      for (int c = 3; c < 7; c++) s[c] += (double)x[c] * w;
    }
  }
  return fstat_f64(s[0], s[1], s[2], s[3], s[4], s[5], s[6], cond);
}

int tcwo_exp_map_f64_realtau(const float *atoms, uint32_t numAtoms, uint32_t TAtom,
                             uint32_t t0_data, const uint32_t *t0s, uint32_t N_t0,
                             const double *taus, uint32_t N_tau, double *Fmn, int nthreads) {
  if (!atoms || !t0s || !taus || !Fmn) return -1;
  if (numAtoms == 0 || TAtom == 0 || N_t0 == 0 || N_tau == 0) return -2;
  set_threads(nthreads);
#pragma omp parallel for collapse(2) schedule(dynamic, 16)
  for (int64_t m = 0; m < (int64_t)N_t0; m++)
    for (int64_t n = 0; n < (int64_t)N_tau; n++)
      Fmn[(size_t)m * N_tau + n] =
          cell_f64_realtau(atoms, numAtoms, TAtom, t0_data, t0s[m], taus[n], NULL);
  return 0;
}

/* Index helpers exported so tests can pin the u32 wrap-around semantics. */
uint32_t tcwo_idx_start(uint32_t t0, uint32_t t0_data, uint32_t TAtom,
                        uint32_t numAtoms) {
  return idx_start(t0, t0_data, TAtom, numAtoms);
}
uint32_t tcwo_idx_end(uint32_t t1, uint32_t t0_data, uint32_t TAtom,
                      uint32_t numAtoms) {
  return idx_end(t1, t0_data, TAtom, numAtoms);
}
