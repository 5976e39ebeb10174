// Per-cell arithmetic of the transient F-statistic map, shared by the CUDA
// kernels and a host build used only by the test-suite to check the
// algorithm against the oracle on the CPU.
//
// Reference semantics followed (PyFstat pyfstat/pyCUDAkernels/):
//   * atom index of a window start, cudaTransientFstatRectWindow.cu:21-31
//   * atom index of a window end,   cudaTransientFstatRectWindow.cu:54-69
//   * exponential window weights and truncation at t0 + 3 tau,
//     cudaTransientFstatExpWindow.cu:22, :53, :80-101
//   * conditioning test and F,      cudaTransientFstatRectWindow.cu:93-118
// all in u32 time arithmetic, wrap-around included.
//
// Precision design (the reference sums in FP32 and loses up to ~4e-4 of 2F
// on short windows, where D = A B - C^2 cancels):
//   * window sums are carried as unevaluated FP32 pairs (hi + lo);
//   * D = A B - C^2 and G = B Fa - C Fb are formed with error-free FMA
//     products from those pairs, so cancellation in them costs nothing;
//   * F = (|G|^2 + D |Fb|^2) / (B D), which equals the reference's
//     (B|Fa|^2 + A|Fb|^2 - 2C Re(Fa Fb*)) / D but is a sum of two non-negative
//     terms (no cancellation);
//   * the test cond < 1e4, cond = (A+B+disc)/(A+B-disc), is evaluated as
//     (A+B+disc)^2 < 4e4 D, the same inequality without the cancelling
//     denominator ((A+B+disc)(A+B-disc) = 4D).
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define TCW_HD __host__ __device__ __forceinline__
#define TCW_HDM __host__ __device__ __forceinline__  // member functions
#else
#define TCW_HD static inline
#define TCW_HDM inline
#include <math.h>
#endif

// Debug builds (-DTCW_DEBUG_CHECKS): every index used for a load or store of
// the map kernels is checked against its array on the device; a failed check
// increments a per-file device counter (read back by tcw_debug_check_failures)
// instead of trapping, so a bad index shows up as a count, not a GPU fault.
#if defined(__CUDACC__) && defined(TCW_DEBUG_CHECKS)
static __device__ unsigned int tcw_dcheck_failures;
#if defined(__CUDA_ARCH__)
#define TCW_DCHECK(cond)                                  \
  do {                                                    \
    if (!(cond)) atomicAdd(&tcw_dcheck_failures, 1u);     \
  } while (0)
#else
#define TCW_DCHECK(cond) \
  do {                   \
  } while (0)
#endif
// Host side: this file's counter (each translation unit has its own).
static inline unsigned int tcw_dcheck_read() {
  unsigned int v = 0;
  if (cudaMemcpyFromSymbol(&v, tcw_dcheck_failures, sizeof(v)) != cudaSuccess) {
    cudaGetLastError();
    return 0xFFFFFFFFu;
  }
  return v;
}
#else
#define TCW_DCHECK(cond) \
  do {                   \
  } while (0)
#endif

namespace tcw {

// ------------------------------------------------------------ rounding-exact ops
// Error-free transformations need every operation rounded exactly once, in
// the written order: on the device the _rn intrinsics are never contracted
// into FMAs; the host build is compiled with -ffp-contract=off.
TCW_HD float fadd(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fadd_rn(a, b);
#else
  return a + b;
#endif
}
TCW_HD float fsub(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fsub_rn(a, b);
#else
  return a - b;
#endif
}
TCW_HD float fmul(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}
TCW_HD float ffma(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
  return __fmaf_rn(a, b, c);
#else
  return fmaf(a, b, c);
#endif
}
TCW_HD float fexp2(float x) {
#if defined(__CUDA_ARCH__)
  return exp2f(x);
#else
  return exp2f(x);
#endif
}

// sqrt to ~2 ulp (feeds only the conditioning test).
TCW_HD float sqrt_approx(float x) {
#if defined(__CUDA_ARCH__)
  float r;
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
#else
  return sqrtf(x);
#endif
}

// a / b to ~1 ulp: approximate reciprocal, then one residual correction of
// the quotient (q + r (a - b q)).
TCW_HD float div_approx(float a, float b) {
#if defined(__CUDA_ARCH__)
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(b));
  float q = __fmul_rn(a, r);
  float e = __fmaf_rn(-b, q, a);
  return __fmaf_rn(e, r, q);
#else
  return a / b;
#endif
}

// 2^x, ~2 ulp, flushes to 0 below the normal range (lnBtSG partial sums).
TCW_HD float ex2_approx(float x) {
#if defined(__CUDA_ARCH__)
  float r;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
#else
  return exp2f(x);
#endif
}

// ------------------------------------------------------------ packed pairs
// Two FP32 lanes operated on together.  On the device these are the packed
// add/sub/mul/fma.rn.f32x2 instructions (one issue slot for two results);
// the host build does the same two IEEE operations one after the other, so
// both give identical results.
struct F2 {
  float x, y;
};

#if defined(__CUDA_ARCH__)
__device__ __forceinline__ unsigned long long f2_pack(F2 a) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a.x), "f"(a.y));
  return r;
}
__device__ __forceinline__ F2 f2_unpack(unsigned long long v) {
  F2 r;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(v));
  return r;
}
#endif

TCW_HD F2 add2(F2 a, F2 b) {
#if defined(__CUDA_ARCH__)
  unsigned long long r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(f2_pack(a)), "l"(f2_pack(b)));
  return f2_unpack(r);
#else
  return F2{a.x + b.x, a.y + b.y};
#endif
}
TCW_HD F2 sub2(F2 a, F2 b) {
#if defined(__CUDA_ARCH__)
  unsigned long long r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(f2_pack(a)), "l"(f2_pack(b)));
  return f2_unpack(r);
#else
  return F2{a.x - b.x, a.y - b.y};
#endif
}
TCW_HD F2 mul2(F2 a, F2 b) {
#if defined(__CUDA_ARCH__)
  unsigned long long r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(f2_pack(a)), "l"(f2_pack(b)));
  return f2_unpack(r);
#else
  return F2{a.x * b.x, a.y * b.y};
#endif
}
TCW_HD F2 fma2(F2 a, F2 b, F2 c) {
#if defined(__CUDA_ARCH__)
  unsigned long long r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(f2_pack(a)), "l"(f2_pack(b)),
      "l"(f2_pack(c)));
  return f2_unpack(r);
#else
  return F2{fmaf(a.x, b.x, c.x), fmaf(a.y, b.y, c.y)};
#endif
}

// Double-word pair: hi and lo words of two channels.
struct FF2 {
  F2 h, l;
};

// x + r*E for two channels at once (ff_axpy per lane).  nrh = -r.h.
TCW_HD FF2 ff2_axpy(F2 x, F2 rh, F2 nrh, F2 rl, FF2 E) {
  const F2 q = mul2(nrh, E.h);        // -p, p = fl(r.h E.h)
  F2 pe = fma2(rh, E.h, q);           // exact product error
  pe = fma2(rh, E.l, pe);
  pe = fma2(rl, E.h, pe);
  const F2 s = sub2(x, q);            // x + p
  const F2 bb = sub2(s, x);
  const F2 e = sub2(sub2(x, sub2(s, bb)), add2(q, bb));  // TwoSum error of x + p
  return FF2{s, add2(e, pe)};
}

// Unevaluated sum hi + lo.
struct FF {
  float h, l;
};

TCW_HD FF ff_zero() { return FF{0.0f, 0.0f}; }

// Knuth TwoSum: s + e == a + b exactly.
TCW_HD void two_sum(float a, float b, float &s, float &e) {
  s = fadd(a, b);
  float bb = fsub(s, a);
  e = fadd(fsub(a, fsub(s, bb)), fsub(b, bb));
}

// x + r*E for a double-word E and a double-word constant r.
TCW_HD FF ff_axpy(float x, FF r, FF E) {
  float p = fmul(r.h, E.h);
  float pe = ffma(r.h, E.h, -p);
  pe = ffma(r.h, E.l, pe);
  pe = ffma(r.l, E.h, pe);
  float s, se;
  two_sum(x, p, s, se);
  return FF{s, fadd(se, pe)};
}

// Running sum: E + x.
TCW_HD FF ff_add1(FF E, float x) {
  float s, se;
  two_sum(E.h, x, s, se);
  return FF{s, fadd(E.l, se)};
}

// E1 - p*E2 (p a plain float, E2 a double-word).
TCW_HD FF ff_sub_scaled(FF E1, float p, FF E2) {
  float a = fmul(p, E2.h);
  float ae = ffma(p, E2.h, -a);
  ae = ffma(p, E2.l, ae);
  float s, se;
  two_sum(E1.h, -a, s, se);
  return FF{s, fsub(fadd(se, E1.l), ae)};
}

// ------------------------------------------------------------ u32 division
// Division of u32 by a per-template constant d >= 1 (Granlund & Montgomery,
// "Division by invariant integers using multiplication", PLDI 1994, the
// round-up variant with a 33-bit multiplier split as 2^32 + mul):
//   l = ceil(log2 d), mul = floor(2^32 (2^l - d) / d) + 1,
//   t = mulhi(x, mul), q = (t + ((x - t) >> 1)) >> (l - 1)  for d >= 2.
struct FastDiv {
  uint32_t d, mul, shift;  // shift = l; d == 1 handled separately
};

static inline FastDiv make_fastdiv(uint32_t d) {
  FastDiv f;
  f.d = d;
  uint32_t l = 0;
  while (l < 32 && ((uint64_t)1 << l) < d) l++;
  f.shift = l;
  if (d <= 1) {
    f.mul = 0;
  } else {
    uint64_t num = (((uint64_t)1 << l) - d) << 32;
    f.mul = (uint32_t)(num / d + 1);
  }
  return f;
}

TCW_HD uint32_t umulhi32(uint32_t a, uint32_t b) {
#if defined(__CUDA_ARCH__)
  return __umulhi(a, b);
#else
  return (uint32_t)(((uint64_t)a * (uint64_t)b) >> 32);
#endif
}

TCW_HD uint32_t fdiv(uint32_t x, const FastDiv &f) {
  if (f.d <= 1) return x;
  uint32_t t = umulhi32(x, f.mul);
  return (t + ((x - t) >> 1)) >> (f.shift - 1);
}

// ------------------------------------------------------------ template geometry
struct Geom {
  uint32_t numAtoms, TAtom, t0_data, half;
  FastDiv div;
};

static inline Geom make_geom(uint32_t numAtoms, uint32_t TAtom, uint32_t t0_data) {
  Geom g;
  g.numAtoms = numAtoms;
  g.TAtom = TAtom;
  g.t0_data = t0_data;
  g.half = TAtom / 2u;
  g.div = make_fastdiv(TAtom);
  return g;
}

// i_t0 (Rect.cu:21-31): u32 wrap, quotient assigned to int, clamped.
TCW_HD uint32_t idx_start(uint32_t t0, const Geom &g) {
  uint32_t q = fdiv(t0 - g.t0_data + g.half, g.div);
  int32_t i = (int32_t)q;
  if (i < 0) i = 0;
  uint32_t u = (uint32_t)i;
  return u < g.numAtoms ? u : g.numAtoms - 1u;
}

// i_t1 (Rect.cu:54-69): "- 1" applied to the unsigned quotient.
TCW_HD uint32_t idx_end(uint32_t t1, const Geom &g) {
  uint32_t q = fdiv(t1 - g.t0_data + g.half, g.div) - 1u;
  int32_t i = (int32_t)q;
  if (i < 0) i = 0;
  uint32_t u = (uint32_t)i;
  return u < g.numAtoms ? u : g.numAtoms - 1u;
}

// Atoms with non-zero exponential weight for a cell: indices in
// [i_t0, i_t1] with t0 <= t_i <= t1 (Exp.cu:80-90), t_i = t0_data + i*TAtom,
// t1 = t0 + 3 tau (u32).  The lower end depends on t0 only, the upper end on
// t0 + 3 tau.
TCW_HD uint32_t exp_lo(uint32_t t0, const Geom &g) {
  const uint32_t a = idx_start(t0, g);
  uint32_t first = 0;  // first i with t_i >= t0
  if (t0 > g.t0_data) {
    const uint32_t d = t0 - g.t0_data;
    const uint32_t q = fdiv(d, g.div);
    first = q + ((d - q * g.TAtom) != 0u ? 1u : 0u);
  }
  return a > first ? a : first;
}

// Upper end; false if no atom has t_i <= t1.  With d = t1 - t0_data >= 0,
// last = floor(d / TAtom) is the last i with t_i <= t1, and idx_end's
// unclamped quotient floor((d + TAtom/2) / TAtom) - 1 is last - 1 plus one
// when the remainder d - last*TAtom reaches TAtom - TAtom/2; the u32 sum
// d + TAtom/2 wraps only for d > 2^32 - 1 - TAtom/2, left to idx_end.
TCW_HD bool exp_hi(uint32_t t0, uint32_t tau, const Geom &g, uint32_t &hi) {
  const uint32_t t1 = t0 + 3u * tau;
  if (t1 < g.t0_data) return false;
  const uint32_t d = t1 - g.t0_data;
  const uint32_t last = fdiv(d, g.div);
  if (d > 0xFFFFFFFFu - g.half) {
    const uint32_t b = idx_end(t1, g);
    hi = b < last ? b : last;
    return true;
  }
  // floor((d + half) / TAtom) = last + (rem + half >= TAtom): idx_end's
  // quotient q = that - 1 (u32), cast to int and clamped as in idx_end; q
  // never exceeds last, so min(idx_end, last) is idx_end.
  const uint32_t rem = d - last * g.TAtom;
  const uint32_t q = last + (rem >= g.TAtom - g.half ? 1u : 0u) - 1u;
  const int32_t i = (int32_t)q;
  const uint32_t u = i < 0 ? 0u : (uint32_t)i;
  hi = u < g.numAtoms ? u : g.numAtoms - 1u;
  return true;
}

TCW_HD bool exp_window(uint32_t t0, uint32_t tau, const Geom &g, uint32_t &lo,
                       uint32_t &hi) {
  lo = exp_lo(t0, g);
  if (!exp_hi(t0, tau, g, hi)) return false;
  return lo <= hi;
}

// ------------------------------------------------------------ F from window sums
// Conditioning flag of a cell whose F fell back to 2 is reported by the
// return value of fstat_ff through the `ok` out-parameter.
template <bool kFp64Det>
TCW_HD float fstat_ff(FF A, FF B, FF C, FF Far, FF Fai, FF Fbr, FF Fbi, bool &ok) {
  // D = A B - C^2 with exact products of the high words
  float p = fmul(A.h, B.h);
  float pe = ffma(A.h, B.h, -p);
  float q = fmul(C.h, C.h);
  float qe = ffma(C.h, C.h, -q);
  float corr = fsub(pe, qe);
  corr = ffma(A.h, B.l, corr);
  corr = ffma(A.l, B.h, corr);
  corr = ffma(-2.0f * C.h, C.l, corr);
  // low x low products matter: quantised prefix differences leave |lo| up to
  // ~1e-4 |hi|, and cond/4 amplifies what is dropped from D
  corr = ffma(A.l, B.l, corr);
  corr = ffma(-C.l, C.l, corr);
  float D;
  if (kFp64Det) {
    double Dd = (double)A.h * (double)B.h - (double)C.h * (double)C.h;
    Dd += (double)(fadd(fadd(fmul(A.h, B.l), fmul(A.l, B.h)), fmul(-2.0f * C.h, C.l)));
    Dd += (double)A.l * (double)B.l - (double)C.l * (double)C.l;
    D = (float)Dd;
  } else {
    D = fadd(fsub(p, q), corr);
  }
  float sumAB = fadd(fadd(A.h, B.h), fadd(A.l, B.l));
  float dAB = fadd(fsub(A.h, B.h), fsub(A.l, B.l));
  float Cs = fadd(C.h, C.l);
  float disc = sqrt_approx(ffma(dAB, dAB, fmul(4.0f * Cs, Cs)));
  float t = fadd(sumAB, disc);
  ok = (D > 0.0f) && (fmul(t, t) < fmul(4.0e4f, D));
  if (!ok) return 2.0f;
  // G = B Fa - C Fb, real and imaginary parts
  float u, ue, v, ve;
  u = fmul(B.h, Far.h);
  ue = ffma(B.h, Far.h, -u);
  v = fmul(C.h, Fbr.h);
  ve = ffma(C.h, Fbr.h, -v);
  float gc = fsub(ue, ve);
  gc = ffma(B.h, Far.l, gc);
  gc = ffma(B.l, Far.h, gc);
  gc = ffma(-C.h, Fbr.l, gc);
  gc = ffma(-C.l, Fbr.h, gc);
  gc = ffma(B.l, Far.l, gc);
  gc = ffma(-C.l, Fbr.l, gc);
  float Gre = fadd(fsub(u, v), gc);
  u = fmul(B.h, Fai.h);
  ue = ffma(B.h, Fai.h, -u);
  v = fmul(C.h, Fbi.h);
  ve = ffma(C.h, Fbi.h, -v);
  gc = fsub(ue, ve);
  gc = ffma(B.h, Fai.l, gc);
  gc = ffma(B.l, Fai.h, gc);
  gc = ffma(-C.h, Fbi.l, gc);
  gc = ffma(-C.l, Fbi.h, gc);
  gc = ffma(B.l, Fai.l, gc);
  gc = ffma(-C.l, Fbi.l, gc);
  float Gim = fadd(fsub(u, v), gc);
  float fbr = fadd(Fbr.h, Fbr.l), fbi = fadd(Fbi.h, Fbi.l);
  float Fb2 = ffma(fbr, fbr, fmul(fbi, fbi));
  float G2 = ffma(Gre, Gre, fmul(Gim, Gim));
  float num = ffma(D, Fb2, G2);
  float den = fmul(fadd(B.h, B.l), D);
  return div_approx(num, den);
}

// Tier 1: cells with cond < kFastCond (the bulk) in FP32 from the rounded
// window sums.  Error bound there: D = fma(A, B, -C^2) has relative error
// <= eps (2 A B / D + 1/2) <= 17.5 eps at cond = 32 ((cond+1)^2 / (4 cond)
// bounds A B / D), and F = |G|^2/(B D) + |Fb|^2/B with G = B Fa - C Fb adds
// <= 2 eps (1 + sqrt(cond)/2): about 1.5e-6 in all.  Returns false (and no
// F) when the cell needs tier 2 (fstat_ff on the double-word sums).
//
// The selection needs no square root: with S = A + B > 0 and D > 0 the
// eigenvalues of [[A, C], [C, B]] are (S +- sqrt(S^2 - 4D))/2, and
// cond < K  <=>  sqrt(S^2 - 4D) (1 + K) < S (K - 1)  <=>  K S^2 < (1 + K)^2 D.
// A cell with D <= 0 (or a NaN) fails the test and goes to tier 2.  With
// K = 32 a power of two the test is evaluated as S^2 < ((1 + K)^2 / K) D
// (1089 / 32 = 34.03125 exactly): scaling by K commutes with the roundings
// (away from overflow and underflow), so it decides as
// fl(fl(K S) S) < fl((1 + K)^2 D) with one multiplication fewer.
constexpr float kFastCond = 32.0f;
constexpr float kFastCondRhs = (1.0f + kFastCond) * (1.0f + kFastCond) / kFastCond;

TCW_HD bool fstat_fast_sums(float A, float B, float C, float Far, float Fai, float Fbr,
                            float Fbi, float &F) {
  const float D = ffma(A, B, -fmul(C, C));
  const float S = fadd(A, B);
  if (!(fmul(S, S) < fmul(kFastCondRhs, D))) return false;
  const float Gre = ffma(B, Far, -fmul(C, Fbr));
  const float Gim = ffma(B, Fai, -fmul(C, Fbi));
  const float num = ffma(D, ffma(Fbr, Fbr, fmul(Fbi, Fbi)), ffma(Gre, Gre, fmul(Gim, Gim)));
  F = div_approx(num, fmul(B, D));
  return true;
}

TCW_HD bool fstat_fast(const FF W[7], float &F) {
  return fstat_fast_sums(fadd(W[0].h, W[0].l), fadd(W[1].h, W[1].l), fadd(W[2].h, W[2].l),
                         fadd(W[3].h, W[3].l), fadd(W[4].h, W[4].l), fadd(W[5].h, W[5].l),
                         fadd(W[6].h, W[6].l), F);
}

// Rectangular window sums held as four channel pairs (A,B) (C,Fa_re) (Fa_im,Fb_re)
// (Fb_im,-): unpack to seven double-words.
TCW_HD void ff2_unpack(const FF2 P[4], FF W[7]) {
  W[0] = FF{P[0].h.x, P[0].l.x};
  W[1] = FF{P[0].h.y, P[0].l.y};
  W[2] = FF{P[1].h.x, P[1].l.x};
  W[3] = FF{P[1].h.y, P[1].l.y};
  W[4] = FF{P[2].h.x, P[2].l.x};
  W[5] = FF{P[2].h.y, P[2].l.y};
  W[6] = FF{P[3].h.x, P[3].l.x};
}

// Tier 1 from paired sums (one packed add per pair), tier 2 otherwise.
template <bool kFp64Det>
TCW_HD float fstat_tiered2(const FF2 P[4], bool &ok) {
  const F2 s0 = add2(P[0].h, P[0].l), s1 = add2(P[1].h, P[1].l);
  const F2 s2 = add2(P[2].h, P[2].l), s3 = add2(P[3].h, P[3].l);
  float F;
  if (fstat_fast_sums(s0.x, s0.y, s1.x, s1.y, s2.x, s2.y, s3.x, F)) {
    ok = true;
    return F;
  }
  FF W[7];
  ff2_unpack(P, W);
  return fstat_ff<kFp64Det>(W[0], W[1], W[2], W[3], W[4], W[5], W[6], ok);
}

// Exponential columns hold the channels by decay ratio: (A,B) as a packed
// pair and C as a scalar double-word decay with r^2, (Fa_re,Fa_im) and
// (Fb_re,Fb_im) as packed pairs with r, so each packed pair has one ratio in
// both lanes.  Atom rows of 8 floats hold the channels in that order:
// [a2 b2 ab nz Fa_re Fa_im Fb_re Fb_im] (slot 3, nz, is an index, not a
// channel: see ExpRow); kRow8Slot[c] is the slot of channel c
// (a2 b2 ab Fa_re Fa_im Fb_re Fb_im).
constexpr int kRow8Slot[7] = {0, 1, 2, 4, 5, 6, 7};

// Both tiers for double-word window sums that are exact enough for tier 2.
template <bool kFp64Det>
TCW_HD float fstat_tiered(const FF W[7], bool &ok) {
  float F;
  if (fstat_fast(W, F)) {
    ok = true;
    return F;
  }
  return fstat_ff<kFp64Det>(W[0], W[1], W[2], W[3], W[4], W[5], W[6], ok);
}

// The uncompensated FP32 variant (plain sums, D = AB - C^2 in FP32, the
// reference's numerator and conditioning formula in FP32) -- kept for the
// precision report only.
TCW_HD float fstat_plain32(float A, float B, float C, float Far, float Fai, float Fbr,
                           float Fbi, bool &ok) {
  float sumAB = fadd(A, B);
  float diffAB = fsub(A, B);
  float disc = sqrtf(fadd(fmul(diffAB, diffAB), fmul(fmul(4.0f, C), C)));
  float denom = fsub(sumAB, disc);
  float cond = denom > 0.0f ? fadd(sumAB, disc) / denom : INFINITY;
  float D = fsub(fmul(A, B), fmul(C, C));
  ok = (cond < 1.0e4f) && (D > 0.0f);
  if (!ok) return 2.0f;
  float num = fsub(fadd(fmul(B, fadd(fmul(Far, Far), fmul(Fai, Fai))),
                        fmul(A, fadd(fmul(Fbr, Fbr), fmul(Fbi, Fbi)))),
                   fmul(fmul(2.0f, C), fadd(fmul(Far, Fbr), fmul(Fai, Fbi))));
  return num / D;
}

// ------------------------------------------------------------ prefix rows
// Rectangular windows read exclusive prefix sums P(j) = sum_{i<j} x_i of the
// seven channels, stored per atom index as 16 floats: hi[0..6], pad, lo[0..6],
// pad.  The high words are integer multiples of a per-channel quantum
// Q_c = 2^(e_c - 22) with sum_i |x_c(i)| < 2^e_c, so any difference of two of
// them is exact in FP32; the low words carry the rest of the double-word
// prefix.  A window sum is then (hi1 - hi0) + (lo1 - lo0) with one rounding
// of size ~eps*Q in the low part.
constexpr int kPrefixStride = 16;

TCW_HD void rect_window_sums(const float *P0, const float *P1, FF W[7]) {
#pragma unroll
  for (int c = 0; c < 7; c++) {
    W[c].h = fsub(P1[c], P0[c]);
    W[c].l = fsub(P1[8 + c], P0[8 + c]);
  }
}

// Quantum exponent for a channel with sum of |x| equal to sabs.
TCW_HD float prefix_quantum(float sabs) {
  // smallest power of two strictly above sabs (with margin), times 2^-22
  float s = sabs * 1.01f + 1e-30f;
  int e;
  frexpf(s, &e);  // s = m * 2^e, 0.5 <= m < 1  ->  s < 2^e
  return ldexpf(1.0f, e - 22);
}

// Quantise a double-word prefix value (h, l) into (hq, lo) with hq = k*Q.
TCW_HD void quantise_prefix(float h, float l, float Q, float invQ, float &hq, float &lo) {
  hq = fmul(rintf(fmul(h, invQ)), Q);
  lo = fadd(fsub(h, hq), l);
}


// ------------------------------------------------------------ rectangular cell
// End index of a rectangular window.  The reference extends a running sum
// along tau (Rect.cu:75-91), so the summed range is [i_t0, max_{n'<=n} i_t1].
// For a non-decreasing tau grid without u32 overflow of t0 + tau, i_t1 only
// decreases where t1 + TAtom/2 < t0_data makes the u32 difference wrap (the
// first taus of such a row); there i_t1 is the clamped last atom, so the
// running maximum is max(i_t1(n), i_t1(tau_first)).
TCW_HD uint32_t rect_end(uint32_t t0, uint32_t tau, uint32_t end_first, bool row_wrapped,
                         const Geom &g) {
  uint32_t e = idx_end(t0 + tau, g);
  if (row_wrapped && end_first > e) e = end_first;
  return e;
}

// Whether a row's first tau lies in the wrapped regime (t1 + TAtom/2 < t0_data).
TCW_HD bool rect_row_wrapped(uint32_t t0, uint32_t tau_first, const Geom &g) {
  return (uint64_t)t0 + (uint64_t)tau_first + (uint64_t)g.half < (uint64_t)g.t0_data;
}

template <bool kComp, bool kFp64Det>
TCW_HD float rect_cell(const float *P, const float *P0, uint32_t j0, uint32_t e, bool &ok) {
  if (e < j0) {  // empty window: zero sums, cond = inf
    ok = false;
    return 2.0f;
  }
  const float *P1 = P + (size_t)(e + 1u) * kPrefixStride;
  if (kComp) {
    FF2 W[4];
    for (int k = 0; k < 4; k++) {
      W[k].h = sub2(F2{P1[2 * k], P1[2 * k + 1]}, F2{P0[2 * k], P0[2 * k + 1]});
      W[k].l = sub2(F2{P1[8 + 2 * k], P1[9 + 2 * k]}, F2{P0[8 + 2 * k], P0[9 + 2 * k]});
    }
    return fstat_tiered2<kFp64Det>(W, ok);
  }
  FF W[7];
  rect_window_sums(P0, P1, W);
  return fstat_plain32(W[0].h, W[1].h, W[2].h, W[3].h, W[4].h, W[5].h, W[6].h, ok);
}

// ------------------------------------------------------------ exponential column
// One tau column over rows [m_begin, m_end), visited from the last row down.
// With E(j) = sum_{J > i >= j} x_i r^(i-j) (r = e^(-TAtom/tau) for the F
// channels, r^2 for A, B, C) the window sum of a cell is
//     W = e^(-k (t_lo - t0)/tau) [E(lo) - r^(k L) E(hi+1)],  L = hi + 1 - lo.
// The common factor e^(-k (t_lo - t0)/tau) scales A, B, C by s^2 and Fa, Fb by
// s and cancels in F and in the conditioning test, so it is not applied.
// Two backward recurrences (lower and upper window edge) walk down the atoms
// as the rows descend; if a row's window lies above a pointer (only with u32
// wrap-around in the grid) both restart from that row's window end.
//
// The subtraction is exact only if r^L matches the weights the recurrence
// applied, so r^L is a double-word too: updated by one multiplication when L
// moves by one, otherwise rebuilt by square-and-multiply.  A window whose
// atoms are all zero (data gaps) has exactly zero sums and F = 2 in the
// reference; it is detected exactly (first atom with a2 or b2 non-zero at or
// above the lower pointer) instead of trusting a difference to cancel.
struct ExpConsts {
  FF r1, r2;   // e^(-TAtom/tau), e^(-2 TAtom/tau)
  FF r1inv;    // e^(+TAtom/tau), valid when has_inv
  bool has_inv;
  float c1;    // TAtom / tau * log2(e) (uncompensated variant)
};

TCW_HD FF ff_from_double(double x) {
  FF r;
  r.h = (float)x;
  r.l = (float)(x - (double)r.h);
  return r;
}

// a*b for double-words, normalised.
TCW_HD FF ff_mul(FF a, FF b) {
  float p = fmul(a.h, b.h);
  float e = ffma(a.h, b.h, -p);
  e = ffma(a.h, b.l, e);
  e = ffma(a.l, b.h, e);
  float s = fadd(p, e);
  return FF{s, fsub(e, fsub(s, p))};
}

// 1/a for a double-word a > 0: FP32 reciprocal refined by one Newton step
// in double-word arithmetic (relative error ~eps^2).
TCW_HD FF ff_recip(FF a) {
  const float y = 1.0f / a.h;
  // e = 1 - a*y exactly enough: a.h*y via its exact product, then a.l*y
  const float p = fmul(a.h, y);
  const float pe = ffma(a.h, y, -p);
  const float e = fsub(fsub(1.0f, p), ffma(a.l, y, pe));
  const float yl = fmul(y, e);
  const float s = fadd(y, yl);
  return FF{s, fsub(yl, fsub(s, y))};
}

// Decay constants of a window with x = TAtom / tau (tau may be real).
TCW_HD ExpConsts exp_consts_x(double x) {
  ExpConsts k;
  k.r1 = ff_from_double(exp(-x));
  k.r2 = ff_mul(k.r1, k.r1);
  k.has_inv = x < 60.0;
  k.r1inv = k.has_inv ? ff_recip(k.r1) : FF{0.0f, 0.0f};
  k.c1 = (float)(x * 1.4426950408889634);
  return k;
}

TCW_HD ExpConsts exp_consts(uint32_t TAtom, uint32_t tau) {
  return exp_consts_x((double)TAtom / (double)tau);
}

TCW_HD FF ff_pow(FF r, uint32_t L) {
  FF res{1.0f, 0.0f};
  FF base = r;
  while (L) {
    if (L & 1u) res = ff_mul(res, base);
    L >>= 1;
    if (L) base = ff_mul(base, base);
  }
  return res;
}

// E1 - p*E2 with a double-word p.
TCW_HD FF ff_sub_scaled2(FF E1, FF p, FF E2) {
  float a = fmul(p.h, E2.h);
  float ae = ffma(p.h, E2.h, -a);
  ae = ffma(p.h, E2.l, ae);
  ae = ffma(p.l, E2.h, ae);
  float s, se;
  two_sum(E1.h, -a, s, se);
  return FF{s, fsub(fadd(se, E1.l), ae)};
}

template <bool kComp>
TCW_HD void exp_step(FF E[7], const float *x, const ExpConsts &k) {
  if (kComp) {
#pragma unroll
    for (int c = 0; c < 3; c++) E[c] = ff_axpy(x[c], k.r2, E[c]);
#pragma unroll
    for (int c = 3; c < 7; c++) E[c] = ff_axpy(x[c], k.r1, E[c]);
  } else {
#pragma unroll
    for (int c = 0; c < 3; c++) E[c].h = ffma(k.r2.h, E[c].h, x[c]);
#pragma unroll
    for (int c = 3; c < 7; c++) E[c].h = ffma(k.r1.h, E[c].h, x[c]);
  }
}

TCW_HD void load_atom(const float *__restrict__ p, float x[7]) {
#pragma unroll
  for (int c = 0; c < 7; c++) x[c] = p[c];
}

// E1 - p*E2 formed so that only the high-word subtraction rounds: when it
// cancels (operands within a factor 2) it is exact, otherwise its rounding
// is relative to the result.  Accurate to ~eps/2 of the window sum however
// much of E1 the tail p*E2 removes -- enough for tier 1; tier 2 re-forms
// the sum with ff_sub_scaled2.
TCW_HD FF ff_sub_scaled_fast(FF E1, FF p, FF E2) {
  const float a = fmul(p.h, E2.h);
  float ae = ffma(p.h, E2.h, -a);
  ae = ffma(p.h, E2.l, ae);
  ae = ffma(p.l, E2.h, ae);
  return FF{fsub(E1.h, a), fsub(E1.l, ae)};
}

// Sink interface: sink(m, F, ok) for every row of the column.  `lo_tab`, if
// not null, holds exp_lo(t0s[m]) at lo_tab[m - m_begin].
template <bool kComp, bool kFp64Det, class Sink>
TCW_HD void exp_column(const float *__restrict__ atoms, const Geom &g,
                       const uint32_t *__restrict__ t0s, uint32_t m_begin, uint32_t m_end,
                       uint32_t tau, Sink &sink, const uint32_t *lo_tab = nullptr) {
  const ExpConsts k = exp_consts(g.TAtom, tau);
  FF Elo[7], Ehi[7];
#pragma unroll
  for (int c = 0; c < 7; c++) Elo[c] = Ehi[c] = ff_zero();
  uint32_t J = 0, jL = 0, jH = 0;
  uint32_t nz = 0xFFFFFFFFu;  // first atom >= jL with a2 or b2 non-zero
  uint32_t Lp = 0;            // exponent of the cached power pw = r1^Lp
  FF pw{1.0f, 0.0f};
  bool init = false;
  for (uint32_t mm = m_end; mm > m_begin; mm--) {
    const uint32_t m = mm - 1u;
    const uint32_t t0 = t0s[m];
    const uint32_t lo = lo_tab ? lo_tab[m - m_begin] : exp_lo(t0, g);
    uint32_t hi;
    if (!exp_hi(t0, tau, g, hi) || lo > hi) {
      sink(m, 2.0f, false);
      continue;
    }
    const uint32_t top = hi + 1u;
    if (!init || top > J || lo > jL || top > jH) {
      J = jL = jH = top;
      nz = 0xFFFFFFFFu;
#pragma unroll
      for (int c = 0; c < 7; c++) Elo[c] = Ehi[c] = ff_zero();
      init = true;
    }
    while (jH > top) {
      jH--;
      float x[7];
      TCW_DCHECK(jH < g.numAtoms);
      load_atom(atoms + (size_t)jH * 7u, x);
      exp_step<kComp>(Ehi, x, k);
    }
    while (jL > lo) {
      jL--;
      float x[7];
      TCW_DCHECK(jL < g.numAtoms);
      load_atom(atoms + (size_t)jL * 7u, x);
      exp_step<kComp>(Elo, x, k);
      if (x[0] != 0.0f || x[1] != 0.0f) nz = jL;
    }
    if (nz > hi) {  // no data in the window: zero sums, cond = inf
      sink(m, 2.0f, false);
      continue;
    }
    bool ok;
    float F;
    if (!kComp) {
      FF W[7];
      if (top == J) {
#pragma unroll
        for (int c = 0; c < 7; c++) W[c] = Elo[c];
      } else {
        const float p1 = fexp2(-(float)(top - lo) * k.c1);
        const float p2 = fmul(p1, p1);
#pragma unroll
        for (int c = 0; c < 3; c++) W[c] = FF{ffma(-p2, Ehi[c].h, Elo[c].h), 0.0f};
#pragma unroll
        for (int c = 3; c < 7; c++) W[c] = FF{ffma(-p1, Ehi[c].h, Elo[c].h), 0.0f};
      }
      F = fstat_plain32(W[0].h, W[1].h, W[2].h, W[3].h, W[4].h, W[5].h, W[6].h, ok);
    } else if (top == J) {
      F = fstat_tiered<kFp64Det>(Elo, ok);
    } else {
      const uint32_t L = top - lo;
      if (L != Lp) {
        if (L == Lp + 1u)
          pw = ff_mul(pw, k.r1);
        else if (L + 1u == Lp && k.has_inv)
          pw = ff_mul(pw, k.r1inv);
        else
          pw = ff_pow(k.r1, L);
        Lp = L;
      }
      const FF p2 = ff_mul(pw, pw);
      FF W[7];
#pragma unroll
      for (int c = 0; c < 3; c++) W[c] = ff_sub_scaled_fast(Elo[c], p2, Ehi[c]);
#pragma unroll
      for (int c = 3; c < 7; c++) W[c] = ff_sub_scaled_fast(Elo[c], pw, Ehi[c]);
      if (fstat_fast(W, F)) {
        ok = true;
      } else {
#pragma unroll
        for (int c = 0; c < 3; c++) W[c] = ff_sub_scaled2(Elo[c], p2, Ehi[c]);
#pragma unroll
        for (int c = 3; c < 7; c++) W[c] = ff_sub_scaled2(Elo[c], pw, Ehi[c]);
        F = fstat_ff<kFp64Det>(W[0], W[1], W[2], W[3], W[4], W[5], W[6], ok);
      }
    }
    sink(m, F, ok);
  }
}

// ------------------------------------------------------------ packed exponential column
// The same windows as exp_column with the atoms in 32-byte rows
// [a2 b2 ab nz Fa_re Fa_im Fb_re Fb_im] (one 256-bit load per step on the
// device) and the channels as three packed pairs (A,B) with r^2, (Fa) and
// (Fb) with r, plus C as a scalar double-word with r^2: one ratio per pair,
// so the per-column constants are two packed ratios and two packed tail
// factors, and C does not spend a packed operation (two FMA-pipe cycles) on
// an idle lane.
TCW_HD void load_row8(const float *__restrict__ p, F2 x[4]) {
#if defined(__CUDA_ARCH__)
  asm volatile("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=f"(x[0].x), "=f"(x[0].y), "=f"(x[1].x), "=f"(x[1].y), "=f"(x[2].x),
                 "=f"(x[2].y), "=f"(x[3].x), "=f"(x[3].y)
               : "l"(p));
#else
  for (int k = 0; k < 4; k++) x[k] = F2{p[2 * k], p[2 * k + 1]};
#endif
}

// Index 0: r^2 (the (A,B) pair); index 1: r (the Fa and Fb pairs).
struct ExpConsts2 {
  F2 rh[2], nrh[2], rl[2];
};

TCW_HD ExpConsts2 exp_consts2(const ExpConsts &k) {
  ExpConsts2 c;
  const FF r[2] = {k.r2, k.r1};
  for (int i = 0; i < 2; i++) {
    c.rh[i] = F2{r[i].h, r[i].h};
    c.nrh[i] = F2{-r[i].h, -r[i].h};
    c.rl[i] = F2{r[i].l, r[i].l};
  }
  return c;
}

// W - p*x per lane for a double-word W, a packed double-word factor p
// (ph + pl, nph = -ph) and single-word x: the product's rounding error is
// formed exactly (FMA) and the high-word subtraction is a TwoSum, so the
// result is a double-word as accurate as an ff2_axpy step.
TCW_HD FF2 ff2_sub_scaled_x(FF2 W, F2 ph, F2 nph, F2 pl, F2 x) {
  const F2 na = mul2(nph, x);        // -a, a = fl(p.h x)
  F2 ae = fma2(ph, x, na);           // p.h x - a exactly
  ae = fma2(pl, x, ae);              // + p.l x
  const F2 s = add2(W.h, na);        // TwoSum(W.h, -a)
  const F2 bb = sub2(s, W.h);
  const F2 e = add2(sub2(W.h, sub2(s, bb)), sub2(na, bb));
  return FF2{s, sub2(add2(e, W.l), ae)};
}

// Fast2Sum forms of ff2_axpy and ff2_sub_scaled_x (Dekker 1971): the error
// of s = fl(a + b) is formed as b - (s - a) in three operations instead of
// TwoSum's six.  It is exact whenever the exponent of a is at least that of
// b; otherwise the double-word misses at most one rounding of size
// 2^-24 |b|.  The exponential map kernels use them where that is exact or
// harmless:
//   * removing an atom from the (A,B) pair: a2, b2 >= 0 with non-negative
//     weights, so the window sum W.h holds the leaving term a = p x as one
//     of its summands and is never smaller (exact);
//   * adding or removing an atom of the Fa and Fb pairs: a miss needs the
//     decayed window sum to be smaller than the entering (leaving) term and
//     costs at most 2^-24 of that one term; a relative error e of (Fa, Fb)
//     moves F by at most 2 e sqrt(cond).  A, B and C, whose errors reach F
//     through D = AB - C^2 up to cond-fold, keep TwoSum on entry (and C on
//     removal).
// Measured on one-year templates (8192 t0 x 4096 tau, 3.4e7 cells each):
// the cells that change move by <= 9.1e-7 relative and stay within 8.6e-7 of
// FP64; the worst error over the reference's exp cases and random gappy
// grids is unchanged (1.2e-6).
TCW_HD FF2 ff2_axpy_fast(F2 x, F2 rh, F2 nrh, F2 rl, FF2 E) {
  const F2 q = mul2(nrh, E.h);        // -p, p = fl(r.h E.h)
  F2 pe = fma2(rh, E.h, q);           // exact product error
  pe = fma2(rh, E.l, pe);
  pe = fma2(rl, E.h, pe);
  const F2 s = sub2(x, q);            // x + p
  const F2 e = sub2(x, add2(s, q));   // x - (s - p)
  return FF2{s, add2(e, pe)};
}

TCW_HD FF2 ff2_sub_scaled_x_fast(FF2 W, F2 ph, F2 nph, F2 pl, F2 x) {
  const F2 na = mul2(nph, x);        // -a, a = fl(p.h x)
  F2 ae = fma2(ph, x, na);           // p.h x - a exactly
  ae = fma2(pl, x, ae);              // + p.l x
  const F2 s = add2(W.h, na);
  const F2 e = sub2(na, sub2(s, W.h));  // -a - (s - W.h)
  return FF2{s, sub2(add2(e, W.l), ae)};
}

// Exact Fast2Sum entries for A, B and C: Fast2Sum is exact when its first
// operand is the larger in magnitude, so ordering the two operands first
// makes it an error-free sum with the same result as TwoSum (bit for bit),
// in three FMA-pipe operations plus min / max or compare / select on the
// ALU pipe instead of six FMA-pipe operations.  For the (A,B) pair both
// terms are non-negative (a2, b2 >= 0, and the decayed window sum of
// non-negative terms), so max / min order them by magnitude.
TCW_HD FF2 ff2_axpy_nonneg(F2 x, F2 rh, F2 nrh, F2 rl, FF2 E) {
  const F2 q = mul2(nrh, E.h);        // -p, p = fl(r.h E.h)
  F2 pe = fma2(rh, E.h, q);           // exact product error
  pe = fma2(rh, E.l, pe);
  pe = fma2(rl, E.h, pe);
  const F2 a{fmaxf(-q.x, x.x), fmaxf(-q.y, x.y)};
  const F2 b{fminf(-q.x, x.x), fminf(-q.y, x.y)};
  const F2 s = add2(a, b);
  const F2 e = sub2(b, sub2(s, a));   // exact: a is the larger
  return FF2{s, add2(e, pe)};
}

// ff_axpy with the operands of the sum ordered by magnitude (C is signed).
TCW_HD FF ff_axpy_ord(float x, FF r, FF E) {
  const float p = fmul(r.h, E.h);
  float pe = ffma(r.h, E.h, -p);
  pe = ffma(r.h, E.l, pe);
  pe = ffma(r.l, E.h, pe);
  const bool pbig = fabsf(p) >= fabsf(x);
  const float a = pbig ? p : x, b = pbig ? x : p;
  const float s = fadd(a, b);
  const float e = fsub(b, fsub(s, a));
  return FF{s, fadd(e, pe)};
}

// The scalar form of ff2_sub_scaled_x (W - p*x for the C channel).
TCW_HD FF ff_sub_scaled_x1(FF W, FF p, float x) {
  const float a = fmul(p.h, x);
  float ae = ffma(p.h, x, -a);
  ae = ffma(p.l, x, ae);
  float sh, se;
  two_sum(W.h, -a, sh, se);
  return FF{sh, fsub(fadd(se, W.l), ae)};
}

// One sliding window sum per column.  W holds, for the atom range
// [wlo, wtop), sum_i x_i r^(i - wlo) (r^2 for A, B, C): the common factor
// e^(-k (t_wlo - t0)/tau) of the exponential weights is dropped as in
// exp_column.  Moving to the next (lower) row's window [lo, top):
//   * an atom i leaving at the top is removed with its current weight
//     r^(i - wlo) (a cached double-word power, updated by one
//     multiplication when the exponent moves by one);
//   * an atom entering at the bottom is added by W = x + r W.
// Every step is a double-word operation with an exact product error and an
// error-free sum (Fast2Sum with the operands ordered by magnitude for A, B
// and C on entry, TwoSum for C on removal, plain Fast2Sum where
// ff2_axpy_fast says it is exact or harmless), so W stays within a few
// eps^2 of the exact window sum of the recurrence's weights.  If the next
// window is not reachable that way (it
// lies above wlo or wtop, only with u32 wrap-around in the grid, or it does
// not overlap the current one), W restarts empty at the new window's top.
template <bool kFp64Det, class Sink>
TCW_HD void exp_column2(const float *__restrict__ atoms8, const Geom &g,
                        const uint32_t *__restrict__ t0s, uint32_t m_begin, uint32_t m_end,
                        uint32_t tau, Sink &sink, const uint32_t *lo_tab = nullptr) {
  const ExpConsts k = exp_consts(g.TAtom, tau);
  const ExpConsts2 k2 = exp_consts2(k);
  const F2 z{0.0f, 0.0f};
  FF2 W0{z, z}, W2{z, z}, W3{z, z};  // (A,B), (Fa_re,Fa_im), (Fb_re,Fb_im)
  FF Wc{0.0f, 0.0f};                 // C
  uint32_t wlo = 0, wtop = 0;        // W holds the window [wlo, wtop)
  uint32_t nz = 0xFFFFFFFFu;         // lowest atom >= wlo with a2 or b2 non-zero
  uint32_t Lp = 0;                   // exponent of the cached powers pw = r^Lp, p2 = r^(2 Lp)
  FF pw{1.0f, 0.0f}, p2{1.0f, 0.0f};
  bool pinit = false;
  for (uint32_t mm = m_end; mm > m_begin; mm--) {
    const uint32_t m = mm - 1u;
    const uint32_t t0 = t0s[m];
    const uint32_t lo = lo_tab ? lo_tab[m - m_begin] : exp_lo(t0, g);
    uint32_t hi;
    if (!exp_hi(t0, tau, g, hi) || lo > hi) {
      sink(m, 2.0f, false);
      continue;
    }
    const uint32_t top = hi + 1u;
    // (the first row restarts too: top >= 1 > wtop = 0)
    if (top > wtop || lo > wlo || top <= wlo) {
      wlo = wtop = top;
      nz = 0xFFFFFFFFu;
      W0 = W2 = W3 = FF2{z, z};
      Wc = FF{0.0f, 0.0f};
    }
    // The atom at wtop - 1 leaves with weight r^(wtop - 1 - wlo), then the
    // atom at wlo - 1 enters (shifting every weight by one power of r); while
    // atoms both leave and enter, alternating the two keeps that exponent,
    // so the cached powers need no update.
    auto leave = [&]() {
      wtop--;
      const uint32_t e = wtop - wlo;  // weight exponent of the leaving atom
      if (e != Lp || !pinit) {
        if (pinit && e == Lp + 1u)
          pw = ff_mul(pw, k.r1);
        else if (pinit && e + 1u == Lp && k.has_inv)
          pw = ff_mul(pw, k.r1inv);
        else
          pw = ff_pow(k.r1, e);
        Lp = e;
        pinit = true;
        p2 = ff_mul(pw, pw);
      }
      F2 x[4];
      TCW_DCHECK(wtop < g.numAtoms);
      load_row8(atoms8 + (size_t)wtop * 8u, x);
      // packed copies of the powers, formed here rather than held across rows
      const F2 ph0{p2.h, p2.h}, pl0{p2.l, p2.l}, nph0{-p2.h, -p2.h};
      const F2 ph1{pw.h, pw.h}, pl1{pw.l, pw.l}, nph1{-pw.h, -pw.h};
      W0 = ff2_sub_scaled_x_fast(W0, ph0, nph0, pl0, x[0]);
      Wc = ff_sub_scaled_x1(Wc, p2, x[1].x);
      W2 = ff2_sub_scaled_x_fast(W2, ph1, nph1, pl1, x[2]);
      W3 = ff2_sub_scaled_x_fast(W3, ph1, nph1, pl1, x[3]);
    };
    auto enter = [&]() {
      wlo--;
      F2 x[4];
      TCW_DCHECK(wlo < g.numAtoms);
      load_row8(atoms8 + (size_t)wlo * 8u, x);
      W0 = ff2_axpy_nonneg(x[0], k2.rh[0], k2.nrh[0], k2.rl[0], W0);
      Wc = ff_axpy_ord(x[1].x, k.r2, Wc);
      W2 = ff2_axpy_fast(x[2], k2.rh[1], k2.nrh[1], k2.rl[1], W2);
      W3 = ff2_axpy_fast(x[3], k2.rh[1], k2.nrh[1], k2.rl[1], W3);
      if (x[0].x != 0.0f || x[0].y != 0.0f) nz = wlo;
    };
    while (wtop > top && wlo > lo) {
      leave();
      enter();
    }
    while (wtop > top) leave();
    while (wlo > lo) enter();
    if (nz > hi) {  // no data in the window: zero sums, cond = inf
      sink(m, 2.0f, false);
      continue;
    }
    // tier 1 from the rounded sums, tier 2 from the double-words
    bool ok = true;
    float F;
    const F2 s0 = add2(W0.h, W0.l), s2 = add2(W2.h, W2.l), s3 = add2(W3.h, W3.l);
    const float sc = fadd(Wc.h, Wc.l);
    if (!fstat_fast_sums(s0.x, s0.y, sc, s2.x, s2.y, s3.x, s3.y, F)) {
      F = fstat_ff<kFp64Det>(FF{W0.h.x, W0.l.x}, FF{W0.h.y, W0.l.y}, Wc, FF{W2.h.x, W2.l.x},
                             FF{W2.h.y, W2.l.y}, FF{W3.h.x, W3.l.x}, FF{W3.h.y, W3.l.y}, ok);
    }
    sink(m, F, ok);
  }
}


// ------------------------------------------------------------ exponential column, row table
// Per-row quantities of an exponential tile, tabulated once per 128 rows by
// the warp that walks them: they depend on t0 only, so every column (lane)
// reads the same entry (one shared-memory broadcast per cell).  The first
// non-zero atom comes from slot 3 of the 32-byte atom rows, where the repack
// kernel stores, for every atom i, the lowest index >= i with a2 or b2
// non-zero.
struct ExpRow {
  uint32_t lo;  // exp_lo(t0): lowest atom with t_i >= t0
  uint32_t nz;  // lowest atom >= lo with a2 or b2 non-zero (0xFFFFFFFF: none)
  uint32_t a;   // floor((t0 - t0_data) / TAtom)
  uint32_t b;   // (t0 - t0_data) mod TAtom
};

// Whether the window end of row t0 can use the tabulated split
// (t0 - t0_data = a TAtom + b): t0 >= t0_data, no u32 wrap of
// t0 + 3 tau + TAtom/2 for any tau up to taumax, and TAtom >= 2 (so the
// quotient stays below 2^31 and the reference's cast to int keeps it).
TCW_HD bool exp_row_regular(uint32_t t0, uint32_t taumax, const Geom &g) {
  return g.TAtom >= 2u && t0 >= g.t0_data &&
         (uint64_t)t0 + 3ull * (uint64_t)taumax + (uint64_t)g.half <= 0xFFFFFFFFull;
}

// One tau column: the sliding double-word window sums of exp_column2, as
// state carried across row-table chunks.  Every arithmetic step is the same
// as exp_column2's, in the same order, so the results are identical; only
// the index work differs: the upper window end of a regular row is
//     top = clamp(a + Q' + [b + R'' >= TAtom], 1, numAtoms)
// with 3 tau + TAtom/2 = Q' TAtom + R'' fixed per column (the same
// floor((t0 + 3 tau - t0_data + TAtom/2) / TAtom) as idx_end, without a
// division per cell), and an empty-data window is one comparison with the
// row's tabulated first non-zero atom.  kFastSums selects exp_column2's
// Fast2Sum steps (the map kernels); without it every step is a TwoSum, for
// the differentiable statistics, whose FP64 F and log-sum-exps want the
// window sums good to ~1e-14.
template <bool kFp64Det, bool kFastSums = false>
struct ExpColumn {
  ExpConsts k;
  ExpConsts2 k2;
  uint32_t Qp1, RmT;  // Q' + 1 and R'' - TAtom (u32 wrap)
  FF2 W0, W2, W3;     // (A,B), (Fa_re,Fa_im), (Fb_re,Fb_im)
  FF Wc;              // C
  uint32_t wlo, wtop, Lp;
  FF pw, p2;          // r^Lp and r^(2 Lp); their packed copies are formed per removal
  bool pinit;
  float Fl;           // the last row's F and flag (row_clamped, row_steady)
  bool okl;

  TCW_HDM void init(const Geom &g, uint32_t tau) {
    k = exp_consts(g.TAtom, tau);
    k2 = exp_consts2(k);
    const uint32_t s = 3u * tau + g.half;  // no wrap on regular rows (checked per chunk)
    const uint32_t Q = fdiv(s, g.div);
    Qp1 = Q + 1u;
    RmT = (s - Q * g.TAtom) - g.TAtom;
    reset();
  }

  // A real tau (the differentiable statistics' continuous grid): with
  // 3 tau + TAtom/2 = Q' TAtom + R'' (R'' real in [0, TAtom)), the carry
  // [b + R'' >= TAtom] of an integer b is [b >= ceil(TAtom - R'')], so RmT
  // holds -ceil(TAtom - R'') and the same top formula applies.
  TCW_HDM void init_real(const Geom &g, double tau) {
    k = exp_consts_x((double)g.TAtom / tau);
    k2 = exp_consts2(k);
    const double s = 3.0 * tau + (double)g.half;
    const double Q = floor(s / (double)g.TAtom);
    const double R = s - Q * (double)g.TAtom;
    double bc = ceil((double)g.TAtom - R);
    bc = bc < 1.0 ? 1.0 : (bc > (double)g.TAtom ? (double)g.TAtom : bc);
    Qp1 = (uint32_t)Q + 1u;
    RmT = 0u - (uint32_t)bc;
    reset();
  }

  TCW_HDM void reset() {
    const F2 z{0.0f, 0.0f};
    W0 = W2 = W3 = FF2{z, z};
    Wc = FF{0.0f, 0.0f};
    wlo = wtop = 0;
    Lp = 0;
    pw = p2 = FF{1.0f, 0.0f};
    pinit = false;
  }

  // floor((t0 + 3 tau + TAtom/2 - t0_data) / TAtom) of row e, the window end
  // before its clamps to [1, numAtoms]: non-decreasing in t0.
  TCW_HDM uint32_t top_raw(const ExpRow &e) const {
    const uint32_t v = e.b + RmT;  // as int: >= 0 iff b + R'' >= TAtom
    return e.a + Qp1 - (v >> 31);
  }

  // Moves the window to row e's: false when it holds no atom or no data
  // (F = 2), true when W0, Wc, W2, W3 hold its sums.
  TCW_HDM bool window(const float *__restrict__ atoms8, const Geom &g, const ExpRow &e) {
    uint32_t top = top_raw(e);
    top = top < 1u ? 1u : top;
    top = top < g.numAtoms ? top : g.numAtoms;
    if (e.lo >= top) return false;
    return slide(atoms8, g, e.lo, top, e.nz);
  }

  // An empty window whose next atoms enter below `top`.
  TCW_HDM void reset_window(uint32_t top) {
    const F2 z{0.0f, 0.0f};
    wlo = wtop = top;
    W0 = W2 = W3 = FF2{z, z};
    Wc = FF{0.0f, 0.0f};
  }

  // pw = r^ex and p2 = r^(2 ex): one multiplication when the exponent moves
  // by one, square-and-multiply otherwise.
  TCW_HDM void power(uint32_t ex) {
    if (ex != Lp || !pinit) {
      if (pinit && ex == Lp + 1u)
        pw = ff_mul(pw, k.r1);
      else if (pinit && ex + 1u == Lp && k.has_inv)
        pw = ff_mul(pw, k.r1inv);
      else
        pw = ff_pow(k.r1, ex);
      Lp = ex;
      pinit = true;
      p2 = ff_mul(pw, pw);
    }
  }

  // Removes the atom at wtop - 1 (weight r^(wtop - 1 - wlo)).
  TCW_HDM void leave(const float *__restrict__ atoms8, const Geom &g) {
    wtop--;
    power(wtop - wlo);  // weight exponent of the leaving atom
    F2 x[4];
    TCW_DCHECK(wtop < g.numAtoms);
    load_row8(atoms8 + (size_t)wtop * 8u, x);
    // packed copies of the powers, formed here rather than held across rows
    const F2 ph0{p2.h, p2.h}, pl0{p2.l, p2.l}, nph0{-p2.h, -p2.h};
    const F2 ph1{pw.h, pw.h}, pl1{pw.l, pw.l}, nph1{-pw.h, -pw.h};
    if (kFastSums) {
      W0 = ff2_sub_scaled_x_fast(W0, ph0, nph0, pl0, x[0]);
      Wc = ff_sub_scaled_x1(Wc, p2, x[1].x);
      W2 = ff2_sub_scaled_x_fast(W2, ph1, nph1, pl1, x[2]);
      W3 = ff2_sub_scaled_x_fast(W3, ph1, nph1, pl1, x[3]);
    } else {
      W0 = ff2_sub_scaled_x(W0, ph0, nph0, pl0, x[0]);
      Wc = ff_sub_scaled_x1(Wc, p2, x[1].x);
      W2 = ff2_sub_scaled_x(W2, ph1, nph1, pl1, x[2]);
      W3 = ff2_sub_scaled_x(W3, ph1, nph1, pl1, x[3]);
    }
  }

  // Moves the window to the atoms [lo, top) (lo < top): false when none of
  // them holds data (nz, the first non-zero atom >= lo, is >= top).  The
  // steps are exp_column2's in the same order (leaving atoms alternate with
  // entering ones while both remain, so the leaving weight's exponent stays
  // put), hence the same bits.
  TCW_HDM bool slide(const float *__restrict__ atoms8, const Geom &g, uint32_t lo, uint32_t top,
                     uint32_t nz) {
    if (top > wtop || lo > wlo || top <= wlo) reset_window(top);
    while (wtop > top && wlo > lo) {
      F2 x[4];  // the entering row, requested before the removal
      TCW_DCHECK(wlo - 1u < g.numAtoms);
      load_row8(atoms8 + (size_t)(wlo - 1u) * 8u, x);
      leave(atoms8, g);
      wlo--;
      enter(x);
    }
    while (wtop > top) leave(atoms8, g);
    enter_to(atoms8, g, lo);
    return nz < top;  // else no data in the window: zero sums, cond = inf
  }

  // slide() for a window whose end is clamped at numAtoms, where no atom
  // leaves (wtop <= numAtoms): the same steps.
  TCW_HDM bool slide_clamped(const float *__restrict__ atoms8, const Geom &g, uint32_t lo,
                             uint32_t nz) {
    const uint32_t top = g.numAtoms;
    if (top > wtop || lo > wlo || top <= wlo) reset_window(top);
    enter_to(atoms8, g, lo);
    return nz < top;
  }

  // The entering atoms down to lo, two at a time: both rows are requested
  // before the first step (the steps themselves are sequential).
  TCW_HDM void enter_to(const float *__restrict__ atoms8, const Geom &g, uint32_t lo) {
    while (wlo > lo + 1u) {
      F2 x[4], y[4];
      TCW_DCHECK(wlo - 1u < g.numAtoms);
      load_row8(atoms8 + (size_t)(wlo - 1u) * 8u, x);
      load_row8(atoms8 + (size_t)(wlo - 2u) * 8u, y);
      wlo -= 2u;
      enter(x);
      enter(y);
    }
    if (wlo > lo) {
      wlo--;
      F2 x[4];
      TCW_DCHECK(wlo < g.numAtoms);
      load_row8(atoms8 + (size_t)wlo * 8u, x);
      enter(x);
    }
  }

  // W = x + r W for one entering atom row (exp_column2's steps).
  TCW_HDM void enter(const F2 x[4]) {
    if (kFastSums) {
      W0 = ff2_axpy_nonneg(x[0], k2.rh[0], k2.nrh[0], k2.rl[0], W0);
      Wc = ff_axpy_ord(x[1].x, k.r2, Wc);
      W2 = ff2_axpy_fast(x[2], k2.rh[1], k2.nrh[1], k2.rl[1], W2);
      W3 = ff2_axpy_fast(x[3], k2.rh[1], k2.nrh[1], k2.rl[1], W3);
    } else {
      W0 = ff2_axpy(x[0], k2.rh[0], k2.nrh[0], k2.rl[0], W0);
      Wc = ff_axpy(x[1].x, k.r2, Wc);
      W2 = ff2_axpy(x[2], k2.rh[1], k2.nrh[1], k2.rl[1], W2);
      W3 = ff2_axpy(x[3], k2.rh[1], k2.nrh[1], k2.rl[1], W3);
    }
  }

  template <class Sink>
  TCW_HDM void row(const float *__restrict__ atoms8, const Geom &g, const ExpRow &e, uint32_t m,
                   Sink &sink) {
    if (!window(atoms8, g, e)) {
      sink(m, 2.0f, false);
      return;
    }
    emit(m, sink);
  }

  // row() where the caller knows that top_raw(e) >= numAtoms (the window
  // end is clamped at numAtoms): the same steps without the window end's
  // arithmetic and with no atom leaving.
  template <class Sink>
  TCW_HDM void row_clamped(const float *__restrict__ atoms8, const Geom &g, const ExpRow &e,
                           uint32_t m, Sink &sink) {
    if (e.lo >= g.numAtoms || !slide_clamped(atoms8, g, e.lo, e.nz)) {
      Fl = 2.0f;
      okl = false;
      sink(m, 2.0f, false);
      return;
    }
    emit(m, sink);
  }

  // row_clamped() for a row that follows, in the same walk, a clamped row
  // whose window held an atom, with e.lo no larger than that row's: the
  // window neither restarts nor loses atoms, and it holds an atom.  A row
  // whose window starts where the previous row's did (t0 closer than TAtom)
  // has that row's window, hence its F.
  template <class Sink>
  TCW_HDM void row_steady(const float *__restrict__ atoms8, const Geom &g, const ExpRow &e,
                          uint32_t m, Sink &sink) {
    if (e.lo == wlo) {
      sink(m, Fl, okl);
      return;
    }
    enter_to(atoms8, g, e.lo);
    if (e.nz >= g.numAtoms) {  // no data in the window: zero sums, cond = inf
      Fl = 2.0f;
      okl = false;
      sink(m, 2.0f, false);
      return;
    }
    emit(m, sink);
  }

  // row_steady() for a row that follows, in the same walk, a steady row whose
  // window held data: its window (starting no higher) holds data too.
  template <class Sink>
  TCW_HDM void row_steady_data(const float *__restrict__ atoms8, const Geom &g, const ExpRow &e,
                               uint32_t m, Sink &sink) {
    if (e.lo == wlo) {
      sink(m, Fl, okl);
      return;
    }
    enter_to(atoms8, g, e.lo);
    emit(m, sink);
  }

  // F of the current window sums (tier 1, else tier 2) to the sink.
  template <class Sink>
  TCW_HDM void emit(uint32_t m, Sink &sink) {
    bool ok = true;
    float F;
    const F2 s0 = add2(W0.h, W0.l), s2 = add2(W2.h, W2.l), s3 = add2(W3.h, W3.l);
    const float sc = fadd(Wc.h, Wc.l);
    if (!fstat_fast_sums(s0.x, s0.y, sc, s2.x, s2.y, s3.x, s3.y, F)) {
      F = fstat_ff<kFp64Det>(FF{W0.h.x, W0.l.x}, FF{W0.h.y, W0.l.y}, Wc, FF{W2.h.x, W2.l.x},
                             FF{W2.h.y, W2.l.y}, FF{W3.h.x, W3.l.x}, FF{W3.h.y, W3.l.y}, ok);
    }
    Fl = F;
    okl = ok;
    sink(m, F, ok);
  }
};

}  // namespace tcw
