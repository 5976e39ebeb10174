// Differentiable transient maps (exponential and rectangular windows):
// forward values and the adjoint.
//
// Per template the tau grid is continuous, tau_n = tau_min + n (tau_max -
// tau_min) / (N_tau - 1), and the outputs are
//   lnBtSG    = ln(70 / (N_t0 N_tau)) + logsumexp_mn F_mn            (tcw:196-217)
//   softmax2F = T logsumexp_mn (2 F_mn / T)        (a smooth max of 2F, T > 0)
// with gradients with respect to the atoms (a2, b2, ab, Fa, Fb) and to
// tau_min / tau_max.  Window boundaries move in steps with tau; only the
// weights are differentiated (the boundaries are piecewise constant).
//
// At T = 0.1 the soft-max weights are exp(20 F), so a gradient good to 1e-4
// needs F to ~1e-9 of its value.  The exponential windows' sums slide down
// each tau column in double-word FP32 (ExpColumn, the map kernels'
// arithmetic, ~1e-14 of the sums' magnitude) rather than in FP64, whose rate
// on GB300 is 1/70 of FP32; for the cells that carry weight (an FP32 tier-1
// F far enough below the maximum or the normaliser skips a cell, whose
// weight is then below e^-40) the forward forms F and the log-sum-exps in
// FP64, the backward F, dF/dW and the sources in double-word FP32:
//
//   diff_fwd_kernel  per tau column, rows descending: double-word window
//            sums, FP64 log-sum-exps of F and 2F/T -> per-tile partials ->
//            finalize per template.
//   diff_bwd_kernel  pass B: the same walk plus the tau-derivative sums
//            V = sum (i - lo) x r^(i - lo) (ExpColumnV); per cell the adjoint
//            sources G_c = g dF/dW_c (g = dL/dF) go to per-block scratch (no
//            map is kept) and g dF/dtau accumulates per column;
//            pass C (same kernel): per column, atoms ascending, the
//            transposed recurrence H(i) = r H(i-1) + sum_{lo(m)=i} G(m)
//            - sum_{hi(m)+1=i} G(m) r^(L(m)) in double-word FP32 gives
//            dL/dx(i) = H(i); each warp reduces its 32 columns per atom
//            (recursive halving over the 7 channels) and adds the sums to
//            the FP64 atom gradient.
// The window-sum factor e^(-k (t_lo - t0)/tau) is left out everywhere: F does
// not depend on it, so neither do g, dF/dW (in this frame) or dF/dtau.
//
// Rectangular windows (rect_diff_kernel): one thread per t0 row, the tau
// columns in ascending order with FP64 running sums (the window end only
// grows with tau, as in the reference's running sums, Rect.cu:75-91); the
// sums of a window do not depend on tau between boundaries, so dL/dtau = 0.
// The atom gradient is scattered as a difference array: +sum_n G(m, n) at
// the row's start index lo(m), -G(m, n) at end(m, n) + 1 (consecutive cells
// with the same end merged), then one prefix scan per template
// (rect_diff_scan_kernel) gives dL/dx(i) = sum_{j <= i} D(j).
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "../../include/tcw_b200.h"
#include "tcw_internal.h"

namespace tcw {

namespace {

constexpr float kLog2eF = 1.4426950408889634f;

__device__ __forceinline__ double tau_of(const DiffTemplate &t, uint32_t n) {
  if (t.N_tau <= 1) return t.tau_min;
  return t.tau_min + (double)n * ((t.tau_max - t.tau_min) / (double)(t.N_tau - 1u));
}

// Upper window end for a real tau (the reference's formula with t1 real).
__device__ __forceinline__ bool exp_hi_real(uint32_t t0, double tau, const Geom &g, uint32_t &hi) {
  const double t1 = (double)t0 + 3.0 * tau;
  if (t1 < (double)g.t0_data) return false;
  const double d = t1 - (double)g.t0_data;
  const double q = floor((d + (double)g.half) / (double)g.TAtom) - 1.0;
  const uint32_t b = q < 0.0 ? 0u
                             : (q >= (double)(g.numAtoms - 1u) ? g.numAtoms - 1u : (uint32_t)q);
  const double l = floor(d / (double)g.TAtom);
  const uint32_t last = l >= 4294967295.0 ? 0xFFFFFFFFu : (uint32_t)l;
  hi = b < last ? b : last;
  return true;
}

// F in FP64 with the reference's conditioning test (Rect.cu:93-118).
struct F64Cell {
  double F, iD;  // F and 1/D
  bool ok;
};

// The conditioning test (sumAB + disc) / (sumAB - disc) < 1e4 is taken as
// sumAB + disc < 1e4 (sumAB - disc) with sumAB - disc > 0 (no division), and
// F = N (1/D) with the one reciprocal the derivatives reuse: FP64 divisions
// are long sequences at GB300's FP64 rate.
__device__ __forceinline__ F64Cell fstat64(const double W[7]) {
  const double A = W[0], B = W[1], C = W[2];
  const double sumAB = A + B, diffAB = A - B;
  const double disc = sqrt(diffAB * diffAB + 4.0 * C * C);
  const double denom = sumAB - disc;
  F64Cell r{2.0, 0.0, false};
  if (denom > 0.0 && sumAB + disc < 1e4 * denom) {
    const double D = A * B - C * C;
    if (D > 0.0) {
      const double N = B * (W[3] * W[3] + W[4] * W[4]) + A * (W[5] * W[5] + W[6] * W[6]) -
                       2.0 * C * (W[3] * W[5] + W[4] * W[6]);
      r.iD = 1.0 / D;
      r.F = N * r.iD;
      r.ok = true;
    }
  }
  return r;
}

// Online log-sum-exp in FP64 (exp in FP64 too: the forward values feed
// finite-difference checks, where FP32 rounding of the terms would show).
// Terms below e^-60 of the running maximum are skipped: the sum is >= 1, so
// even 1e9 of them change it by < 1e-17.
__device__ __forceinline__ void lse_add(double &m, double &s, double v) {
  if (v > m) {
    s = s * exp(m - v) + 1.0;
    m = v;
  } else if (v - m > -60.0) {
    s += exp(v - m);
  }
}

__device__ __forceinline__ void lse_merge(double &m, double &s, double m2, double s2) {
  if (s2 == 0.0) return;
  if (s == 0.0) {
    m = m2;
    s = s2;
    return;
  }
  const double M = fmax(m, m2);
  s = s * exp(m - M) + s2 * exp(m2 - M);
  m = M;
}

// Blocks of 128 threads, one tau column each; rows of a template all in one tile.
constexpr int kDiffBlock = 128;
// Per-block scratch row of one column: G_c (c = 0..6) and r^L as a float
// hi/lo pair, so that the removal in the transposed recurrence cancels the
// injected term to FP64 accuracy.
constexpr uint32_t kDiffSlots = TCW_DIFF_SLOTS;

// Minimum resident blocks per SM asked of the register allocator, per pass
// (build-time tunables; 1 leaves the allocation to ptxas).
#ifndef TCW_DIFF_MIN_BLOCKS_FWD
#define TCW_DIFF_MIN_BLOCKS_FWD 5
#endif
#ifndef TCW_DIFF_MIN_BLOCKS_BWD
#define TCW_DIFF_MIN_BLOCKS_BWD 1
#endif
constexpr int diff_min_blocks(int pass) {
  return pass == 0 ? TCW_DIFF_MIN_BLOCKS_FWD : TCW_DIFF_MIN_BLOCKS_BWD;
}

// ------------------------------------------------------------ exponential forward (double-word)

// Forward pass of exponential windows (lnBtSG and the soft-max 2F): the
// window sums of each tau column slide down the rows in double-word FP32
// (ExpColumn, the map kernel's arithmetic; sums good to ~1e-14 of the
// window's magnitude, against FP64 recurrences at GB300's 1/70 FP64 rate),
// with the per-row quantities tabulated per warp and the real tau's window
// end split as in ExpColumn::init_real.  F goes into the FP64 log-sum-exps:
// a cell whose FP32 tier-1 F lies more than 62 below a lower bound of the
// template's maximum (the column's running maximum, or the tile's largest
// tier-1 F found by a first, FP32-only sweep) carries exp(F - max) < e^-60
// in both sums (the soft-max's 2F/T - max is 2/T times lower still) and is
// skipped -- the tier-1 F is good
// to ~1.5e-6 relative and passes only for cond < 32, where the FP64 test
// passes too; every other cell gets F in FP64 from the double-word sums
// (the reference's formula and conditioning test, fstat64).  Rows that are
// not regular for the tile's taus (t0 + 3 tau + TAtom/2 beyond u32, or
// TAtom < 2) take the window end from exp_hi_real instead.
constexpr uint32_t kDiffRowTab = 128;

__global__ void __launch_bounds__(256) diff_repack_kernel(const DiffTemplate *__restrict__ T,
                                                          const uint32_t *__restrict__ list,
                                                          const float *__restrict__ atoms,
                                                          float *__restrict__ atoms8) {
  __shared__ uint32_t s_first[256];
  const DiffTemplate t = T[list[blockIdx.x]];
  repack_rows256(atoms + t.atom_off * 7u, reinterpret_cast<float4 *>(atoms8 + t.atom_off * 8u),
                 t.g.numAtoms, s_first);
}

__device__ __forceinline__ void lse_pair_add(double &m1, double &s1, double &m2, double &s2,
                                             double F, double temp, float &skip) {
  lse_add(m1, s1, F);
  lse_add(m2, s2, 2.0 * F / temp);
  skip = (float)(m1 - 62.0);
}

__global__ void __launch_bounds__(kDiffBlock, diff_min_blocks(0))
    diff_fwd_kernel(const DiffTemplate *__restrict__ T, const DiffItem *__restrict__ items,
                    uint32_t n_items, uint32_t *__restrict__ counter,
                    const float *__restrict__ atoms8, const uint32_t *__restrict__ t0s_all,
                    double temp, DiffPartial *__restrict__ parts) {
  __shared__ uint32_t s_item;
  __shared__ double sh[kDiffBlock / 32][4];
  __shared__ __align__(16) ExpRow s_tab[kDiffBlock / 32][kDiffRowTab];
  const uint32_t lane = threadIdx.x & 31u;
  ExpRow *tab = s_tab[threadIdx.x >> 5];
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(counter, 1u);
    __syncthreads();
    const uint32_t it = s_item;
    __syncthreads();
    if (it >= n_items) break;
    const DiffItem w = items[it];
    const DiffTemplate t = T[w.tmpl];
    const uint32_t n = w.n0 + threadIdx.x;
    const bool active = n < w.n1;
    const uint32_t *t0s = t0s_all + t.t0_off;
    const double tau = tau_of(t, active ? n : w.n0);
    const float *a8 = atoms8 + t.atom_off * 8u;
    const uint32_t *a8u = reinterpret_cast<const uint32_t *>(a8);
    double m1 = -INFINITY, s1 = 0.0, m2 = -INFINITY, s2 = 0.0;
    float skip = -INFINITY;
    // the warp's largest tau, rounded up, for the regularity test
    const uint32_t tau_up = !active ? 0u
                            : (tau >= 4294967295.0 ? 0xFFFFFFFFu : (uint32_t)ceil(tau));
    const uint32_t taumax = __reduce_max_sync(0xffffffffu, tau_up);
    ExpColumn<false> C;
    C.init_real(t.g, tau);
    // Two sweeps down the columns: the first finds the tile's largest tier-1
    // F (FP32 only), a lower bound of the template's maximum to within its
    // ~1e-5 error, so that the second skips the cells 62 below it from the
    // start instead of only below the running maximum.
    float est = -INFINITY, skip0 = -INFINITY;
    for (int sweep = 0; sweep < 2; sweep++) {
      if (sweep == 1) {
        float v = est;
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, d));
        if (lane == 0) sh[threadIdx.x >> 5][0] = (double)v;
        __syncthreads();
        double tile = sh[0][0];
        for (int k = 1; k < kDiffBlock / 32; k++) tile = fmax(tile, sh[k][0]);
        __syncthreads();
        if (tile > -INFINITY) skip0 = (float)(tile - 1e-5 * fabs(tile) - 63.0);
        skip = skip0;
        C.reset();
      }
      for (uint32_t ce = t.N_t0; ce > 0;) {
        const uint32_t cb = ce > kDiffRowTab ? ce - kDiffRowTab : 0u;
        bool reg = true;
        for (uint32_t r = lane; r < ce - cb; r += 32u)
          reg = reg && exp_row_regular(__ldg(t0s + cb + r), taumax, t.g);
        reg = __all_sync(0xffffffffu, reg);
        __syncwarp();
        for (uint32_t r = lane; r < ce - cb; r += 32u) {
          const uint32_t t0 = __ldg(t0s + cb + r);
          ExpRow e;
          e.lo = exp_lo(t0, t.g);
          e.nz = e.lo < t.g.numAtoms ? __ldg(a8u + (size_t)e.lo * 8u + 3u) : 0xFFFFFFFFu;
          const uint32_t d = t0 - t.g.t0_data;
          e.a = reg ? fdiv(d, t.g.div) : t0;  // irregular chunks: the generic branch reads t0
          e.b = reg ? d - e.a * t.g.TAtom : 0u;
          tab[r] = e;
        }
        __syncwarp();
        if (active) {
          for (uint32_t m = ce; m > cb;) {
            m--;
            const ExpRow e = tab[m - cb];
            bool data;
            if (reg) {
              data = C.window(a8, t.g, e);
            } else {  // the window end from the real t1 (e.a holds t0 on these rows)
              uint32_t hi;
              data = exp_hi_real(e.a, tau, t.g, hi) && e.lo <= hi &&
                     C.slide(a8, t.g, e.lo, hi + 1u, e.nz);
            }
            double F = 2.0;
            if (data) {
              float F32;
              const F2 s0 = add2(C.W0.h, C.W0.l), s2v = add2(C.W2.h, C.W2.l),
                       s3 = add2(C.W3.h, C.W3.l);
              const float sc = fadd(C.Wc.h, C.Wc.l);
              const bool t1 = fstat_fast_sums(s0.x, s0.y, sc, s2v.x, s2v.y, s3.x, s3.y, F32);
              if (sweep == 0) {
                if (t1) est = fmaxf(est, F32);
                continue;
              }
              if (t1 && F32 < skip) continue;
              double W[7];
              W[0] = (double)C.W0.h.x + (double)C.W0.l.x;
              W[1] = (double)C.W0.h.y + (double)C.W0.l.y;
              W[2] = (double)C.Wc.h + (double)C.Wc.l;
              W[3] = (double)C.W2.h.x + (double)C.W2.l.x;
              W[4] = (double)C.W2.h.y + (double)C.W2.l.y;
              W[5] = (double)C.W3.h.x + (double)C.W3.l.x;
              W[6] = (double)C.W3.h.y + (double)C.W3.l.y;
              F = fstat64(W).F;
            } else if (sweep == 0 || 2.0f < skip) {
              continue;
            }
            lse_pair_add(m1, s1, m2, s2, F, temp, skip);
            skip = fmaxf(skip, skip0);
          }
        }
        ce = cb;
      }
    }
    // block merge of the two log-sum-exp pairs (warp shuffles, then smem)
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
      const double om1 = __shfl_down_sync(0xffffffffu, m1, d);
      const double os1 = __shfl_down_sync(0xffffffffu, s1, d);
      const double om2 = __shfl_down_sync(0xffffffffu, m2, d);
      const double os2 = __shfl_down_sync(0xffffffffu, s2, d);
      lse_merge(m1, s1, om1, os1);
      lse_merge(m2, s2, om2, os2);
    }
    if (lane == 0) {
      sh[threadIdx.x >> 5][0] = m1;
      sh[threadIdx.x >> 5][1] = s1;
      sh[threadIdx.x >> 5][2] = m2;
      sh[threadIdx.x >> 5][3] = s2;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int k = 1; k < kDiffBlock / 32; k++) {
        lse_merge(m1, s1, sh[k][0], sh[k][1]);
        lse_merge(m2, s2, sh[k][2], sh[k][3]);
      }
      parts[w.part] = DiffPartial{m1, s1, m2, s2};
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------ exponential backward (double-word)

// Packed double-word helpers of the backward pass.
__device__ __forceinline__ FF2 ff2_add_dw(FF2 a, FF2 b) {  // a + b, low words summed
  const F2 s = add2(a.h, b.h);
  const F2 bb = sub2(s, a.h);
  const F2 e = add2(sub2(a.h, sub2(s, bb)), sub2(b.h, bb));
  return FF2{s, add2(e, add2(a.l, b.l))};
}
__device__ __forceinline__ FF2 ff2_scale_dw(F2 rh, F2 nrh, F2 rl, FF2 S) {  // r S (r = rh + rl)
  const F2 q = mul2(nrh, S.h);  // -p
  F2 pe = fma2(rh, S.h, q);
  pe = fma2(rh, S.l, pe);
  pe = fma2(rl, S.h, pe);
  return FF2{sub2(F2{0.0f, 0.0f}, q), pe};
}
__device__ __forceinline__ FF ff_add_dw(FF a, FF b) {
  float s, e;
  two_sum(a.h, b.h, s, e);
  return FF{s, fadd(e, fadd(a.l, b.l))};
}
__device__ __forceinline__ FF ff_scale_dw(FF r, FF S) {
  const float p = fmul(r.h, S.h);
  float pe = ffma(r.h, S.h, -p);
  pe = ffma(r.h, S.l, pe);
  pe = ffma(r.l, S.h, pe);
  return FF{p, pe};
}
// Double-word arithmetic on FF (hi + lo FP32 pairs, ~2^-44 relative per
// operation) for the adjoint's per-cell values.
__device__ __forceinline__ FF dw_norm(float s, float e) {
  const float h = fadd(s, e);
  return FF{h, fsub(e, fsub(h, s))};
}
__device__ __forceinline__ FF dw_add(FF a, FF b) {
  float s, e;
  two_sum(a.h, b.h, s, e);
  return dw_norm(s, fadd(e, fadd(a.l, b.l)));
}
__device__ __forceinline__ FF dw_sub(FF a, FF b) { return dw_add(a, FF{-b.h, -b.l}); }
__device__ __forceinline__ FF dw_mulf(FF a, float b) {
  const float p = fmul(a.h, b);
  float e = ffma(a.h, b, -p);
  e = ffma(a.l, b, e);
  return dw_norm(p, e);
}
__device__ __forceinline__ FF dw_twice(FF a) { return FF{2.0f * a.h, 2.0f * a.l}; }
__device__ __forceinline__ FF dw_from(double x) {
  const float h = (float)x;
  return FF{h, (float)(x - (double)h)};
}

// F of a cell from its double-word window sums, in double-word arithmetic:
// D = AB - C^2 from exact products of the high words, the conditioning test
// cond < 1e4 as 1e4 S^2 < (1 + 1e4)^2 D (S = A + B), G = B Fa - C Fb and
// F = (|G|^2 + D |Fb|^2) / (B D).
struct DwCell {
  FF F, iD, Gre, Gim, Fb2;
  bool ok;
};
__device__ __forceinline__ DwCell dw_fstat(FF A, FF B, FF C, FF Far, FF Fai, FF Fbr, FF Fbi) {
  DwCell r;
  const float p = fmul(A.h, B.h), pe = ffma(A.h, B.h, -p);
  const float q = fmul(C.h, C.h), qe = ffma(C.h, C.h, -q);
  float s, se;
  two_sum(p, -q, s, se);
  float corr = fadd(se, fsub(pe, qe));
  corr = ffma(A.h, B.l, corr);
  corr = ffma(A.l, B.h, corr);
  corr = ffma(-2.0f * C.h, C.l, corr);
  corr = ffma(A.l, B.l, corr);
  corr = ffma(-C.l, C.l, corr);
  const FF D = dw_norm(s, corr);
  const FF S = dw_add(A, B);
  const FF lhs = dw_mulf(ff_mul(S, S), 1.0e4f);
  const FF rhs = ff_mul(D, FF{100020000.0f, 1.0f});  // (1 + 1e4)^2
  const FF dd = dw_sub(rhs, lhs);
  r.ok = D.h > 0.0f && S.h > 0.0f && dd.h > 0.0f;
  r.Gre = dw_sub(ff_mul(B, Far), ff_mul(C, Fbr));
  r.Gim = dw_sub(ff_mul(B, Fai), ff_mul(C, Fbi));
  r.Fb2 = dw_add(ff_mul(Fbr, Fbr), ff_mul(Fbi, Fbi));
  const FF G2 = dw_add(ff_mul(r.Gre, r.Gre), ff_mul(r.Gim, r.Gim));
  const FF num = dw_add(G2, ff_mul(D, r.Fb2));
  r.iD = r.ok ? ff_recip(D) : FF{0.0f, 0.0f};
  const FF iB = r.ok ? ff_recip(B) : FF{0.0f, 0.0f};
  r.F = ff_mul(ff_mul(num, r.iD), iB);
  return r;
}

// E + x per lane (TwoSum of the high words, x's rounding into the low word).
__device__ __forceinline__ FF2 ff2_add_x(FF2 E, F2 x) {
  const F2 s = add2(E.h, x);
  const F2 bb = sub2(s, E.h);
  const F2 e = add2(sub2(E.h, sub2(s, bb)), sub2(x, bb));
  return FF2{s, add2(E.l, e)};
}


// The backward pass's column: the window sums W of ExpColumn and their
// tau-derivative sums V_c = sum_i (i - lo) x_c(i) r_c^(i - lo) (r_c = r^2
// for A, B, C, r for Fa, Fb), both in double-word FP32 and moved together:
// an atom entering at the bottom gives V' = r_c (V + W) (the old W), one
// leaving at the top with weight exponent e gives V' = V - e x r_c^e.
// dW_c / dtau = k_c (TAtom / tau^2) V_c (k_c = 2 for A, B, C; 1 otherwise).
struct ExpColumnV {
  ExpColumn<false> C;
  FF2 V0, V2, V3;
  FF Vc;

  __device__ __forceinline__ void reset_v() {
    const F2 z{0.0f, 0.0f};
    V0 = V2 = V3 = FF2{z, z};
    Vc = FF{0.0f, 0.0f};
  }

  __device__ __forceinline__ bool slide(const float *__restrict__ atoms8, const Geom &g,
                                        uint32_t lo, uint32_t top, uint32_t nz) {
    if (top > C.wtop || lo > C.wlo || top <= C.wlo) {
      C.reset_window(top);
      reset_v();
    }
    while (C.wtop > top) {
      C.wtop--;
      const uint32_t ex = C.wtop - C.wlo;
      C.power(ex);
      F2 x[4];
      TCW_DCHECK(C.wtop < g.numAtoms);
      load_row8(atoms8 + (size_t)C.wtop * 8u, x);
      const F2 ph0{C.p2.h, C.p2.h}, pl0{C.p2.l, C.p2.l}, nph0{-C.p2.h, -C.p2.h};
      const F2 ph1{C.pw.h, C.pw.h}, pl1{C.pw.l, C.pw.l}, nph1{-C.pw.h, -C.pw.h};
      C.W0 = ff2_sub_scaled_x(C.W0, ph0, nph0, pl0, x[0]);
      C.Wc = ff_sub_scaled_x1(C.Wc, C.p2, x[1].x);
      C.W2 = ff2_sub_scaled_x(C.W2, ph1, nph1, pl1, x[2]);
      C.W3 = ff2_sub_scaled_x(C.W3, ph1, nph1, pl1, x[3]);
      // V: the leaving atom's weight times its exponent
      const FF e2 = ff_mul(C.p2, FF{(float)ex, 0.0f}), e1 = ff_mul(C.pw, FF{(float)ex, 0.0f});
      const F2 eh0{e2.h, e2.h}, el0{e2.l, e2.l}, neh0{-e2.h, -e2.h};
      const F2 eh1{e1.h, e1.h}, el1{e1.l, e1.l}, neh1{-e1.h, -e1.h};
      V0 = ff2_sub_scaled_x(V0, eh0, neh0, el0, x[0]);
      Vc = ff_sub_scaled_x1(Vc, e2, x[1].x);
      V2 = ff2_sub_scaled_x(V2, eh1, neh1, el1, x[2]);
      V3 = ff2_sub_scaled_x(V3, eh1, neh1, el1, x[3]);
    }
    while (C.wlo > lo) {
      C.wlo--;
      F2 x[4];
      TCW_DCHECK(C.wlo < g.numAtoms);
      load_row8(atoms8 + (size_t)C.wlo * 8u, x);
      V0 = ff2_scale_dw(C.k2.rh[0], C.k2.nrh[0], C.k2.rl[0], ff2_add_dw(V0, C.W0));
      Vc = ff_scale_dw(C.k.r2, ff_add_dw(Vc, C.Wc));
      V2 = ff2_scale_dw(C.k2.rh[1], C.k2.nrh[1], C.k2.rl[1], ff2_add_dw(V2, C.W2));
      V3 = ff2_scale_dw(C.k2.rh[1], C.k2.nrh[1], C.k2.rl[1], ff2_add_dw(V3, C.W3));
      C.W0 = ff2_axpy(x[0], C.k2.rh[0], C.k2.nrh[0], C.k2.rl[0], C.W0);
      C.Wc = ff_axpy(x[1].x, C.k.r2, C.Wc);
      C.W2 = ff2_axpy(x[2], C.k2.rh[1], C.k2.nrh[1], C.k2.rl[1], C.W2);
      C.W3 = ff2_axpy(x[3], C.k2.rh[1], C.k2.nrh[1], C.k2.rl[1], C.W3);
    }
    return nz < top;
  }
};

// Backward pass of exponential windows.  Pass B slides W and V down each
// tau column in double-word FP32 (ExpColumnV) with the per-row quantities
// tabulated per warp; a cell gets F, dF/dW and its adjoint sources (in
// double-word arithmetic, dw_fstat) only when it carries weight.  Its weight g = gB e^(F - Z1) + 2 gS e^(2F/T - Z2)
// (Z1 = logsumexp F, Z2 = logsumexp 2F/T, from the forward outputs) is below
// e^-40 when the FP32 tier-1 F (good to ~1e-5 of F) lies more than 42 below
// Z1 (the lnBtSG term, gB != 0) and more than 40 T + 1 below (T/2) Z2 (the
// soft-max term, gS != 0: its exponent is then below -80); such cells
// contribute no sources.  Pass C (the transposed recurrence) runs in
// double-word FP32 (FP64 recurrences: 95 ms on the differentiation workload,
// with a per-channel butterfly reduction 67.6 ms, double-word 45.7 ms), with
// the window ends of regular rows from the integer split.
__global__ void __launch_bounds__(kDiffBlock, diff_min_blocks(1))
    diff_bwd_kernel(const DiffTemplate *__restrict__ T, const DiffItem *__restrict__ items,
                    uint32_t n_items, uint32_t *__restrict__ counter,
                    const float *__restrict__ atoms8, const uint32_t *__restrict__ t0s_all,
                    double temp, const double *__restrict__ lnZ1, const double *__restrict__ lnZ2,
                    const double *__restrict__ gB, const double *__restrict__ gS,
                    float *__restrict__ scratch, uint32_t scratch_rows,
                    double *__restrict__ grad_atoms, double *__restrict__ grad_tau) {
  __shared__ uint32_t s_item;
  __shared__ double sh[kDiffBlock / 32][8];
  __shared__ uint32_t s_end;
  __shared__ __align__(16) ExpRow s_tab[kDiffBlock / 32][kDiffRowTab];
  const uint32_t lane = threadIdx.x & 31u;
  ExpRow *tab = s_tab[threadIdx.x >> 5];
  float *my_scratch = scratch + (size_t)blockIdx.x * scratch_rows * kDiffSlots * kDiffBlock;
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(counter, 1u);
    __syncthreads();
    const uint32_t it = s_item;
    __syncthreads();
    if (it >= n_items) break;
    const DiffItem w = items[it];
    const DiffTemplate t = T[w.tmpl];
    const uint32_t n = w.n0 + threadIdx.x;
    const bool active = n < w.n1;
    const uint32_t *t0s = t0s_all + t.t0_off;
    const float *a8 = atoms8 + t.atom_off * 8u;
    const uint32_t *a8u = reinterpret_cast<const uint32_t *>(a8);
    const double tau = tau_of(t, active ? n : w.n0);
    const double r1 = exp(-(double)t.g.TAtom / tau);
    const double inv_r1 = r1 > 1e-280 ? 1.0 / r1 : 0.0;
    // normalisers from the forward outputs: logsumexp F and logsumexp 2F/T
    const double z1 = lnZ1[w.tmpl] - log(70.0 / ((double)t.N_t0 * (double)t.N_tau));
    const double z2 = lnZ2[w.tmpl] / temp;
    const double gb = gB[w.tmpl], gs = gS[w.tmpl];
    const FF z1w = dw_from(z1), z2w = dw_from(z2), twoT = dw_from(2.0 / temp);
    const float gbf = (float)gb, gsf = (float)gs;
    FF dtw{0.0f, 0.0f};
    // a tier-1 F below `skip` carries no weight in either sum
    const double sk1 = gb != 0.0 ? z1 - 42.0 : INFINITY;
    const double sk2 = gs != 0.0 ? 0.5 * temp * (z2 - 80.0) - 1.0 : INFINITY;
    const float skip = (float)fmin(sk1, sk2);
    const uint32_t tau_up = !active ? 0u
                            : (tau >= 4294967295.0 ? 0xFFFFFFFFu : (uint32_t)ceil(tau));
    const uint32_t taumax = __reduce_max_sync(0xffffffffu, tau_up);
    ExpColumnV CV;
    CV.C.init_real(t.g, tau);
    CV.reset_v();
    double dtau = 0.0, pw64 = 1.0;
    uint32_t Lp64 = 0;
    for (uint32_t ce = t.N_t0; ce > 0;) {
      const uint32_t cb = ce > kDiffRowTab ? ce - kDiffRowTab : 0u;
      bool reg = true;
      for (uint32_t r = lane; r < ce - cb; r += 32u)
        reg = reg && exp_row_regular(__ldg(t0s + cb + r), taumax, t.g);
      reg = __all_sync(0xffffffffu, reg);
      __syncwarp();
      for (uint32_t r = lane; r < ce - cb; r += 32u) {
        const uint32_t t0 = __ldg(t0s + cb + r);
        ExpRow e;
        e.lo = exp_lo(t0, t.g);
        e.nz = e.lo < t.g.numAtoms ? __ldg(a8u + (size_t)e.lo * 8u + 3u) : 0xFFFFFFFFu;
        const uint32_t d = t0 - t.g.t0_data;
        e.a = reg ? fdiv(d, t.g.div) : t0;  // irregular chunks: the generic branch reads t0
        e.b = reg ? d - e.a * t.g.TAtom : 0u;
        tab[r] = e;
      }
      __syncwarp();
      if (active) {
        for (uint32_t m = ce; m > cb;) {
          m--;
          const ExpRow e = tab[m - cb];
          uint32_t top = 0;
          bool data = false;
          if (reg) {
            const uint32_t v = e.b + CV.C.RmT;
            top = e.a + CV.C.Qp1 - (v >> 31);
            top = top < 1u ? 1u : (top < t.g.numAtoms ? top : t.g.numAtoms);
            data = e.lo < top && CV.slide(a8, t.g, e.lo, top, e.nz);
          } else {
            uint32_t hi;
            if (exp_hi_real(e.a, tau, t.g, hi) && e.lo <= hi) {
              top = hi + 1u;
              data = CV.slide(a8, t.g, e.lo, top, e.nz);
            }
          }
          float Gf[7] = {0, 0, 0, 0, 0, 0, 0};
          float p1h = 0.0f, p1l = 0.0f;
          if (data) {
            // r^L, L = top - lo, for the removal in the transposed recurrence
            // (FP64, one multiplication when L moves by one)
            const uint32_t L = top - e.lo;
            if (L != Lp64) {
              if (L == Lp64 + 1u)
                pw64 *= r1;
              else if (L + 1u == Lp64 && inv_r1 > 0.0)
                pw64 *= inv_r1;
              else
                pw64 = pow(r1, (double)L);
              Lp64 = L;
            }
            const ExpColumn<false> &C = CV.C;
            float F32;
            const F2 s0 = add2(C.W0.h, C.W0.l), s2v = add2(C.W2.h, C.W2.l),
                     s3 = add2(C.W3.h, C.W3.l);
            const float sc = fadd(C.Wc.h, C.Wc.l);
            const bool t1 = fstat_fast_sums(s0.x, s0.y, sc, s2v.x, s2v.y, s3.x, s3.y, F32);
            if (!(t1 && F32 < skip)) {
              const FF A{C.W0.h.x, C.W0.l.x}, B{C.W0.h.y, C.W0.l.y}, Cc = C.Wc;
              const FF Far{C.W2.h.x, C.W2.l.x}, Fai{C.W2.h.y, C.W2.l.y};
              const FF Fbr{C.W3.h.x, C.W3.l.x}, Fbi{C.W3.h.y, C.W3.l.y};
              const DwCell fc = dw_fstat(A, B, Cc, Far, Fai, Fbr, Fbi);
              if (fc.ok) {
                const FF F = fc.F;
                // exponents of the weights from double-word differences
                const FF d1 = dw_sub(F, z1w);
                const FF d2 = dw_sub(ff_mul(F, twoT), z2w);
                const float g = gbf * exp2f(fadd(d1.h, d1.l) * kLog2eF) +
                                gsf * 2.0f * exp2f(fadd(d2.h, d2.l) * kLog2eF);
                const FF Fa2 = dw_add(ff_mul(Far, Far), ff_mul(Fai, Fai));
                const FF re = dw_add(ff_mul(Far, Fbr), ff_mul(Fai, Fbi));
                FF dF[7];
                dF[0] = ff_mul(dw_sub(fc.Fb2, ff_mul(F, B)), fc.iD);
                dF[1] = ff_mul(dw_sub(Fa2, ff_mul(F, A)), fc.iD);
                dF[2] = dw_twice(ff_mul(dw_sub(ff_mul(F, Cc), re), fc.iD));
                dF[3] = dw_twice(ff_mul(fc.Gre, fc.iD));
                dF[4] = dw_twice(ff_mul(fc.Gim, fc.iD));
                dF[5] = dw_twice(ff_mul(dw_sub(ff_mul(A, Fbr), ff_mul(Cc, Far)), fc.iD));
                dF[6] = dw_twice(ff_mul(dw_sub(ff_mul(A, Fbi), ff_mul(Cc, Fai)), fc.iD));
                const FF V[7] = {FF{CV.V0.h.x, CV.V0.l.x}, FF{CV.V0.h.y, CV.V0.l.y}, CV.Vc,
                                 FF{CV.V2.h.x, CV.V2.l.x}, FF{CV.V2.h.y, CV.V2.l.y},
                                 FF{CV.V3.h.x, CV.V3.l.x}, FF{CV.V3.h.y, CV.V3.l.y}};
#pragma unroll
                for (int c = 0; c < 7; c++) {
                  const FF Gc = dw_mulf(dF[c], g);
                  Gf[c] = fadd(Gc.h, Gc.l);
                  const FF tv = ff_mul(Gc, V[c]);
                  dtw = dw_add(dtw, c < 3 ? dw_twice(tv) : tv);
                }
                p1h = (float)pw64;
                p1l = (float)(pw64 - (double)p1h);
              }
            }
          }
          TCW_DCHECK(m < scratch_rows);
          float *scr = my_scratch + (size_t)m * kDiffSlots * kDiffBlock + threadIdx.x;
#pragma unroll
          for (int c = 0; c < 7; c++) scr[(size_t)c * kDiffBlock] = Gf[c];
          scr[(size_t)7 * kDiffBlock] = p1h;
          scr[(size_t)8 * kDiffBlock] = p1l;
        }
      }
      ce = cb;
    }

    // ---- pass B done for this tile: tau gradient, then pass C (ascending)
    __syncthreads();  // scratch of all columns written
    dtau = (double)dtw.h + (double)dtw.l;
    const double scale = active ? (double)t.g.TAtom / (tau * tau) * dtau : 0.0;
    const double fr = (active && t.N_tau > 1) ? (double)n / (double)(t.N_tau - 1u) : 0.0;
    double dmax = scale * fr,
           dmin = scale * (active && t.N_tau > 1 ? 1.0 - fr : (active ? 1.0 : 0.0));
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
      dmax += __shfl_down_sync(0xffffffffu, dmax, d);
      dmin += __shfl_down_sync(0xffffffffu, dmin, d);
    }
    if (lane == 0) {
      sh[threadIdx.x >> 5][0] = dmin;
      sh[threadIdx.x >> 5][1] = dmax;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double a = 0.0, b = 0.0;
      for (int k = 0; k < kDiffBlock / 32; k++) {
        a += sh[k][0];
        b += sh[k][1];
      }
      atomicAdd(grad_tau + 2u * w.tmpl, a);
      atomicAdd(grad_tau + 2u * w.tmpl + 1u, b);
      s_end = 0;
    }
    __syncthreads();
    // one past the window end of row m (the window start for empty windows:
    // removal right after injection), from the integer split on regular
    // rows, else from the real t1
    auto row_end = [&](uint32_t m) -> uint32_t {
      const uint32_t t0 = __ldg(t0s + m);
      const uint32_t lo = exp_lo(t0, t.g);
      if (exp_row_regular(t0, taumax, t.g)) {
        const uint32_t dd = t0 - t.g.t0_data;
        const uint32_t a = fdiv(dd, t.g.div), b = dd - a * t.g.TAtom;
        uint32_t top = a + CV.C.Qp1 - ((b + CV.C.RmT) >> 31);
        top = top < 1u ? 1u : (top < t.g.numAtoms ? top : t.g.numAtoms);
        return lo < top ? top : lo;
      }
      uint32_t hi;
      return (exp_hi_real(t0, tau, t.g, hi) && lo <= hi) ? hi + 1u : lo;
    };
    // atom range of the transposed recurrence: from the first row's window
    // start to the largest window end of the tile
    const uint32_t i_begin = exp_lo(__ldg(t0s), t.g);
    atomicMax(&s_end, active ? row_end(t.N_t0 - 1u) : i_begin);
    __syncthreads();
    const uint32_t i_end = s_end;
    // H in double-word FP32: (A,B) and C decay with r^2, (Fa) and (Fb) with r
    const F2 zp{0.0f, 0.0f};
    FF2 H01{zp, zp}, H34{zp, zp}, H56{zp, zp};
    FF H2{0.0f, 0.0f};
    const ExpConsts &kc = CV.C.k;
    const ExpConsts2 &kp = CV.C.k2;
    uint32_t mi = 0, mr = 0;
    uint32_t lo_next = i_begin;
    uint32_t end_r = active ? row_end(0) : 0u;
    const float *sc0 = my_scratch + threadIdx.x;
    for (uint32_t i = i_begin; i < i_end; i++) {
      if (active) {
        H01 = ff2_scale_dw(kp.rh[0], kp.nrh[0], kp.rl[0], H01);
        H2 = ff_scale_dw(kc.r2, H2);
        H34 = ff2_scale_dw(kp.rh[1], kp.nrh[1], kp.rl[1], H34);
        H56 = ff2_scale_dw(kp.rh[1], kp.nrh[1], kp.rl[1], H56);
        while (mi < t.N_t0 && lo_next <= i) {
          const float *scr = sc0 + (size_t)mi * kDiffSlots * kDiffBlock;
          H01 = ff2_add_x(H01, F2{scr[0], scr[(size_t)1 * kDiffBlock]});
          H2 = ff_add1(H2, scr[(size_t)2 * kDiffBlock]);
          H34 = ff2_add_x(H34, F2{scr[(size_t)3 * kDiffBlock], scr[(size_t)4 * kDiffBlock]});
          H56 = ff2_add_x(H56, F2{scr[(size_t)5 * kDiffBlock], scr[(size_t)6 * kDiffBlock]});
          mi++;
          if (mi < t.N_t0) lo_next = exp_lo(__ldg(t0s + mi), t.g);
        }
        while (mr < mi && end_r <= i) {
          const float *scr = sc0 + (size_t)mr * kDiffSlots * kDiffBlock;
          const FF p1{scr[(size_t)7 * kDiffBlock], scr[(size_t)8 * kDiffBlock]};
          const FF p2 = ff_mul(p1, p1);
          const F2 ph0{p2.h, p2.h}, pl0{p2.l, p2.l}, nph0{-p2.h, -p2.h};
          const F2 ph1{p1.h, p1.h}, pl1{p1.l, p1.l}, nph1{-p1.h, -p1.h};
          H01 = ff2_sub_scaled_x(H01, ph0, nph0, pl0, F2{scr[0], scr[(size_t)1 * kDiffBlock]});
          H2 = ff_sub_scaled_x1(H2, p2, scr[(size_t)2 * kDiffBlock]);
          H34 = ff2_sub_scaled_x(H34, ph1, nph1, pl1,
                                 F2{scr[(size_t)3 * kDiffBlock], scr[(size_t)4 * kDiffBlock]});
          H56 = ff2_sub_scaled_x(H56, ph1, nph1, pl1,
                                 F2{scr[(size_t)5 * kDiffBlock], scr[(size_t)6 * kDiffBlock]});
          mr++;
          if (mr < t.N_t0) end_r = row_end(mr);
        }
      }
      // reduce the warp's columns' contributions to atom i (each warp adds its
      // own: no block barrier per atom) by recursive halving over 8 channel
      // slots in double-word arithmetic: at each step a lane keeps half of its
      // slots, sends the other half to its partner and adds what it receives
      // (9 double-word additions per lane); lane L ends with channel
      // (L >> 2) & 7 summed over the warp
      const bool u16 = (lane & 16u) != 0u, u8 = (lane & 8u) != 0u, u4 = (lane & 4u) != 0u;
      const FF zf{0.0f, 0.0f};
      const FF slot[8] = {active ? FF{H01.h.x, H01.l.x} : zf, active ? FF{H01.h.y, H01.l.y} : zf,
                          active ? H2 : zf,                    active ? FF{H34.h.x, H34.l.x} : zf,
                          active ? FF{H34.h.y, H34.l.y} : zf, active ? FF{H56.h.x, H56.l.x} : zf,
                          active ? FF{H56.h.y, H56.l.y} : zf, zf};
      auto xch = [&](FF send, int d) {
        return FF{__shfl_xor_sync(0xffffffffu, send.h, d), __shfl_xor_sync(0xffffffffu, send.l, d)};
      };
      FF k4[4], k2[2];
#pragma unroll
      for (int j = 0; j < 4; j++)
        k4[j] = ff_add_dw(u16 ? slot[4 + j] : slot[j], xch(u16 ? slot[j] : slot[4 + j], 16));
#pragma unroll
      for (int j = 0; j < 2; j++)
        k2[j] = ff_add_dw(u8 ? k4[2 + j] : k4[j], xch(u8 ? k4[j] : k4[2 + j], 8));
      FF v = ff_add_dw(u4 ? k2[1] : k2[0], xch(u4 ? k2[0] : k2[1], 4));
      v = ff_add_dw(v, xch(v, 2));
      v = ff_add_dw(v, xch(v, 1));
      const uint32_t ch = (lane >> 2) & 7u;
      if ((lane & 3u) == 0u && ch < 7u && i < t.g.numAtoms) {
        const double a = (double)v.h + (double)v.l;
        if (a != 0.0) atomicAdd(grad_atoms + (t.atom_off + i) * 7u + ch, a);
      }
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------ rectangular windows

// Inclusive end index of a rectangular window for a real tau (the
// reference's i_t1, Rect.cu:54-69, with t1 = t0 + tau real); t0 >= t0_data -
// TAtom/2 (checked on the host), so the quotient is >= -1.
__device__ __forceinline__ uint32_t rect_end_real(uint32_t t0, double tau, const Geom &g) {
  const double d = (double)t0 + tau - (double)g.t0_data + (double)g.half;
  const double q = floor(d / (double)g.TAtom) - 1.0;
  return q < 0.0 ? 0u : (q >= (double)(g.numAtoms - 1u) ? g.numAtoms - 1u : (uint32_t)q);
}

__device__ __forceinline__ void flush_diff(double *D, uint32_t row, const double v[7], double sgn,
                                           uint32_t numAtoms) {
  TCW_DCHECK(row <= numAtoms);
#pragma unroll
  for (int c = 0; c < 7; c++)
    if (v[c] != 0.0) atomicAdd(D + (size_t)row * 8u + c, sgn * v[c]);
}

template <int kPass>
__global__ void __launch_bounds__(kDiffBlock, diff_min_blocks(kPass))
    rect_diff_kernel(const DiffTemplate *__restrict__ T, const DiffItem *__restrict__ items,
                     uint32_t n_items, uint32_t *__restrict__ counter,
                     const float *__restrict__ atoms, const uint32_t *__restrict__ t0s_all,
                     double temp, DiffPartial *__restrict__ parts,
                     const double *__restrict__ lnZ1, const double *__restrict__ lnZ2,
                     const double *__restrict__ gB, const double *__restrict__ gS,
                     double *__restrict__ D64) {
  __shared__ uint32_t s_item;
  __shared__ double sh[kDiffBlock / 32][4];
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(counter, 1u);
    __syncthreads();
    const uint32_t it = s_item;
    __syncthreads();
    if (it >= n_items) break;
    const DiffItem w = items[it];
    const DiffTemplate t = T[w.tmpl];
    const uint32_t m = w.n0 + threadIdx.x;  // this thread's t0 row
    const bool active = m < w.n1;
    double m1 = -INFINITY, s1 = 0.0, m2 = -INFINITY, s2 = 0.0;
    double z1 = 0.0, z2 = 0.0, gb = 0.0, gs = 0.0;
    if (kPass == 1) {
      z1 = lnZ1[w.tmpl] - log(70.0 / ((double)t.N_t0 * (double)t.N_tau));
      z2 = lnZ2[w.tmpl] / temp;
      gb = gB[w.tmpl];
      gs = gS[w.tmpl];
    }
    if (active) {
      const float *x = atoms + t.atom_off * 7u;
      double *D = kPass == 1 ? D64 + t.p_off * 8u : nullptr;
      const uint32_t t0 = __ldg(t0s_all + t.t0_off + m);
      const uint32_t lo = idx_start(t0, t.g);
      double S[7] = {0, 0, 0, 0, 0, 0, 0};
      double R[7] = {0, 0, 0, 0, 0, 0, 0}, acc[7] = {0, 0, 0, 0, 0, 0, 0};
      uint32_t next = lo, acc_end = 0xFFFFFFFFu;
      for (uint32_t n = 0; n < t.N_tau; n++) {
        const uint32_t end = rect_end_real(t0, tau_of(t, n), t.g);
        for (; next <= end; next++) {
          TCW_DCHECK(next < t.g.numAtoms);
#pragma unroll
          for (int c = 0; c < 7; c++) S[c] += (double)__ldg(x + (size_t)next * 7u + c);
        }
        F64Cell fc{2.0, 0.0, false};
        if (end >= lo) fc = fstat64(S);
        const double F = fc.F;
        if (kPass == 0) {
          lse_add(m1, s1, F);
          lse_add(m2, s2, 2.0 * F / temp);
        } else if (fc.ok) {
          // dL/dF of this cell (FP32 exponentials: relative 1e-7 on a gradient
          // term; cells far below the maxima get exactly 0 and are skipped)
          const double g = gb * (double)exp2f((float)(F - z1) * kLog2eF) +
                           gs * 2.0 * (double)exp2f((float)(2.0 * F / temp - z2) * kLog2eF);
          if (g == 0.0) continue;
          const double A = S[0], B = S[1], C = S[2], iD = fc.iD;
          const double Fa2 = S[3] * S[3] + S[4] * S[4], Fb2 = S[5] * S[5] + S[6] * S[6];
          const double re = S[3] * S[5] + S[4] * S[6];
          double G[7];
          G[0] = (Fb2 - F * B) * iD;
          G[1] = (Fa2 - F * A) * iD;
          G[2] = (2.0 * F * C - 2.0 * re) * iD;
          G[3] = 2.0 * (B * S[3] - C * S[5]) * iD;
          G[4] = 2.0 * (B * S[4] - C * S[6]) * iD;
          G[5] = 2.0 * (A * S[5] - C * S[3]) * iD;
          G[6] = 2.0 * (A * S[6] - C * S[4]) * iD;
          if (end != acc_end) {
            if (acc_end != 0xFFFFFFFFu) flush_diff(D, acc_end + 1u, acc, -1.0, t.g.numAtoms);
#pragma unroll
            for (int c = 0; c < 7; c++) acc[c] = 0.0;
            acc_end = end;
          }
#pragma unroll
          for (int c = 0; c < 7; c++) {
            acc[c] += g * G[c];
            R[c] += g * G[c];
          }
        }
      }
      if (kPass == 1) {
        if (acc_end != 0xFFFFFFFFu) flush_diff(D, acc_end + 1u, acc, -1.0, t.g.numAtoms);
        flush_diff(D, lo, R, 1.0, t.g.numAtoms);
      }
    }
    if (kPass == 0) {
#pragma unroll
      for (int d = 16; d > 0; d >>= 1) {
        const double om1 = __shfl_down_sync(0xffffffffu, m1, d);
        const double os1 = __shfl_down_sync(0xffffffffu, s1, d);
        const double om2 = __shfl_down_sync(0xffffffffu, m2, d);
        const double os2 = __shfl_down_sync(0xffffffffu, s2, d);
        lse_merge(m1, s1, om1, os1);
        lse_merge(m2, s2, om2, os2);
      }
      if ((threadIdx.x & 31u) == 0) {
        sh[threadIdx.x >> 5][0] = m1;
        sh[threadIdx.x >> 5][1] = s1;
        sh[threadIdx.x >> 5][2] = m2;
        sh[threadIdx.x >> 5][3] = s2;
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        for (int k = 1; k < kDiffBlock / 32; k++) {
          lse_merge(m1, s1, sh[k][0], sh[k][1]);
          lse_merge(m2, s2, sh[k][2], sh[k][3]);
        }
        parts[w.part] = DiffPartial{m1, s1, m2, s2};
      }
      __syncthreads();
    }
  }
}

// dL/dx(i) = sum_{j <= i} D(j) for i < numAtoms, one block per rectangular
// template: per-thread chunk sums, an exclusive scan of the chunk sums, then
// each chunk written in order.
constexpr int kScanBlock = 256;

__global__ void __launch_bounds__(kScanBlock)
    rect_diff_scan_kernel(const DiffTemplate *__restrict__ T, const uint32_t *__restrict__ list,
                          const double *__restrict__ D64, double *__restrict__ grad_atoms) {
  __shared__ double sh[kScanBlock][7];
  const DiffTemplate t = T[list[blockIdx.x]];
  const uint32_t n = t.g.numAtoms;
  const double *D = D64 + t.p_off * 8u;
  const uint32_t chunk = (n + kScanBlock - 1u) / kScanBlock;
  const uint32_t a0 = min(n, threadIdx.x * chunk), a1 = min(n, a0 + chunk);
  double s[7] = {0, 0, 0, 0, 0, 0, 0};
  for (uint32_t i = a0; i < a1; i++)
#pragma unroll
    for (int c = 0; c < 7; c++) s[c] += D[(size_t)i * 8u + c];
#pragma unroll
  for (int c = 0; c < 7; c++) sh[threadIdx.x][c] = s[c];
  __syncthreads();
  if (threadIdx.x < 7u) {
    double run = 0.0;
    for (int k = 0; k < kScanBlock; k++) {
      const double v = sh[k][threadIdx.x];
      sh[k][threadIdx.x] = run;
      run += v;
    }
  }
  __syncthreads();
  double run[7];
#pragma unroll
  for (int c = 0; c < 7; c++) run[c] = sh[threadIdx.x][c];
  for (uint32_t i = a0; i < a1; i++) {
#pragma unroll
    for (int c = 0; c < 7; c++) {
      run[c] += D[(size_t)i * 8u + c];
      grad_atoms[(t.atom_off + i) * 7u + c] = run[c];
    }
  }
}

__global__ void diff_finalize_kernel(const DiffTemplate *__restrict__ T, uint32_t n_templates,
                                     const DiffPartial *__restrict__ parts, double temp,
                                     double *__restrict__ lnB, double *__restrict__ soft) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n_templates) return;
  const DiffTemplate t = T[k];
  double m1 = -INFINITY, s1 = 0.0, m2 = -INFINITY, s2 = 0.0;
  for (uint32_t p = 0; p < t.n_parts; p++) {
    const DiffPartial q = parts[t.part_off + p];
    lse_merge(m1, s1, q.m1, q.s1);
    lse_merge(m2, s2, q.m2, q.s2);
  }
  lnB[k] = log(70.0 / ((double)t.N_t0 * (double)t.N_tau)) + m1 + log(s1);
  soft[k] = temp * (m2 + log(s2));
}

}  // namespace

int diff_blocks_per_sm(int pass) {
  int n = 0;
  cudaError_t e = pass == 0
                      ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, diff_fwd_kernel, kDiffBlock, 0)
                      : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, diff_bwd_kernel, kDiffBlock, 0);
  if (e != cudaSuccess) {
    cudaGetLastError();
    n = 1;
  }
  return n > 0 ? n : 1;
}

int rect_diff_blocks_per_sm(int pass) {
  int n = 0;
  cudaError_t e =
      pass == 0
          ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, rect_diff_kernel<0>, kDiffBlock, 0)
          : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, rect_diff_kernel<1>, kDiffBlock, 0);
  if (e != cudaSuccess) {
    cudaGetLastError();
    n = 1;
  }
  return n > 0 ? n : 1;
}

cudaError_t launch_diff(int pass, const DiffLaunch &L, cudaStream_t stream) {
  if (L.n_items) {
    if (pass == 0) {
      diff_repack_kernel<<<L.n_exp, 256, 0, stream>>>(L.T, L.exp_list, L.atoms, L.atoms8);
      diff_fwd_kernel<<<L.n_blocks, kDiffBlock, 0, stream>>>(L.T, L.items, L.n_items, L.counter,
                                                             L.atoms8, L.t0s, L.temp, L.parts);
    } else {
      diff_repack_kernel<<<L.n_exp, 256, 0, stream>>>(L.T, L.exp_list, L.atoms, L.atoms8);
      diff_bwd_kernel<<<L.n_blocks, kDiffBlock, 0, stream>>>(
          L.T, L.items, L.n_items, L.counter, L.atoms8, L.t0s, L.temp, L.lnZ1, L.lnZ2, L.gB,
          L.gS, L.scratch, L.scratch_rows, L.grad_atoms, L.grad_tau);
    }
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  if (L.n_rect_items) {
    if (pass == 0) {
      rect_diff_kernel<0><<<L.n_rect_blocks, kDiffBlock, 0, stream>>>(
          L.T, L.rect_items, L.n_rect_items, L.rect_counter, L.atoms, L.t0s, L.temp, L.parts,
          nullptr, nullptr, nullptr, nullptr, nullptr);
    } else {
      rect_diff_kernel<1><<<L.n_rect_blocks, kDiffBlock, 0, stream>>>(
          L.T, L.rect_items, L.n_rect_items, L.rect_counter, L.atoms, L.t0s, L.temp, nullptr,
          L.lnZ1, L.lnZ2, L.gB, L.gS, L.D64);
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) return e;
      rect_diff_scan_kernel<<<L.n_rect, kScanBlock, 0, stream>>>(L.T, L.rect_list, L.D64,
                                                                 L.grad_atoms);
    }
    return cudaGetLastError();
  }
  return cudaSuccess;
}

cudaError_t launch_diff_finalize(const DiffTemplate *T, uint32_t n_templates,
                                 const DiffPartial *parts, double temp, double *lnB, double *soft,
                                 cudaStream_t stream) {
  if (n_templates == 0) return cudaSuccess;
  diff_finalize_kernel<<<(n_templates + 127u) / 128u, 128, 0, stream>>>(T, n_templates, parts,
                                                                         temp, lnB, soft);
  return cudaGetLastError();
}

}  // namespace tcw

namespace tcw {
// Failed debug checks of this file's kernels (0 unless built with TCW_DEBUG_CHECKS).
unsigned int dcheck_failures_diff() {
#if defined(TCW_DEBUG_CHECKS)
  return tcw_dcheck_read();
#else
  return 0;
#endif
}
}  // namespace tcw
