// CUDA kernels of the transient-CW F-statistic map for GB300 (sm_103a).
//
//   prefix_kernel    compensated exclusive prefix sums of the 7 atom channels of
//                    each rectangular template (one block per template), stored
//                    as quantised double-word rows (see tcw_cell.h)
//   map_kernel       the (t0, tau) cells of a list of tiles; a block owns one tile
//                    (grid launch) or pulls tiles from an atomic counter
//                    (persistent launch).  Rectangular tiles difference two prefix
//                    rows per cell; exponential tiles slide one double-word window
//                    sum down each tau column (atoms enter at the lower window end
//                    and leave at the upper end).  Every block (rect: every warp
//                    of a persistent launch) reduces its cells to
//                    (max F, first argmax, sum exp(F - max F)).
//   repack_kernel    exponential templates' atoms into 32-byte rows (one 256-bit
//                    load per recurrence step)
//   finalize_kernel  per template, merges the tile partials in a fixed order:
//                    maxF, argmax, lnBtSG in FP64.
//   posterior kernels  row / column sums of exp(F - maxF) over a written map and
//                    their argmax (t0 / tau max-posterior bins): one template
//                    (plain path) or every template of a plan
//                    (post_sums_kernel, post_argmax_kernel).
// No tensor cores: nothing on this path is a dense contraction.
#include <math.h>
#include <stdint.h>

#include "../../include/tcw_b200.h"
#include "tcw_internal.h"

namespace tcw {

constexpr float kLog2e = 1.4426950408889634f;

// ------------------------------------------------------------------ helpers

__device__ __forceinline__ FF ff_add(FF a, FF b) {
  float s, e;
  two_sum(a.h, b.h, s, e);
  e = fadd(e, fadd(a.l, b.l));
  float s2 = fadd(s, e);
  return FF{s2, fsub(e, fsub(s2, s))};
}

__device__ __forceinline__ FF shfl_up_ff(FF v, int d) {
  return FF{__shfl_up_sync(0xffffffffu, v.h, d), __shfl_up_sync(0xffffffffu, v.l, d)};
}

// One 64-byte prefix row as two 256-bit loads (each lane's request covers
// whole 32-byte sectors).
__device__ __forceinline__ void ld_row16(const float *p, float r[16]) {
#pragma unroll
  for (int k = 0; k < 2; k++)
    asm volatile("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=f"(r[8 * k + 0]), "=f"(r[8 * k + 1]), "=f"(r[8 * k + 2]),
                   "=f"(r[8 * k + 3]), "=f"(r[8 * k + 4]), "=f"(r[8 * k + 5]),
                   "=f"(r[8 * k + 6]), "=f"(r[8 * k + 7])
                 : "l"(p + 8 * k));
}

// ------------------------------------------------------------------ repack

__global__ void __launch_bounds__(256) repack_kernel(const TemplateDev *__restrict__ T,
                                                     const uint32_t *__restrict__ exp_list,
                                                     const float *__restrict__ atoms,
                                                     float *__restrict__ A8) {
  __shared__ uint32_t s_first[256];
  const TemplateDev t = T[exp_list[blockIdx.x]];
  repack_rows256(atoms + t.atom_off * 7u, reinterpret_cast<float4 *>(A8 + t.a8_off * 8u),
                 t.g.numAtoms, s_first);
}

// ------------------------------------------------------------------ prefix

template <bool kComp>
__global__ void __launch_bounds__(256) prefix_kernel(const TemplateDev *__restrict__ T,
                                                     const uint32_t *__restrict__ rect_list,
                                                     const float *__restrict__ atoms,
                                                     float *__restrict__ P) {
  const TemplateDev t = T[rect_list[blockIdx.x]];
  const uint32_t N = t.g.numAtoms;
  const float *x = atoms + t.atom_off * 7u;
  float *out = P + t.p_off * kPrefixStride;
  const uint32_t tid = threadIdx.x, lane = tid & 31u, wid = tid >> 5;
  const uint32_t chunk = (N + 255u) / 256u;
  const uint32_t i0 = min(N, tid * chunk), i1 = min(N, i0 + chunk);

  FF loc[7];
  float sabs[7];
#pragma unroll
  for (int c = 0; c < 7; c++) {
    loc[c] = ff_zero();
    sabs[c] = 0.0f;
  }
#pragma unroll 4
  for (uint32_t i = i0; i < i1; i++) {
#pragma unroll
    for (int c = 0; c < 7; c++) {
      float v = __ldg(x + (size_t)i * 7u + c);
      loc[c] = kComp ? ff_add1(loc[c], v) : FF{fadd(loc[c].h, v), 0.0f};
      sabs[c] += fabsf(v);
    }
  }

  __shared__ FF warp_tot[8][7];
  __shared__ float warp_abs[8][7];
#pragma unroll
  for (int c = 0; c < 7; c++) {
    FF v = loc[c];
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      FF o = shfl_up_ff(v, d);
      if (lane >= (uint32_t)d) v = kComp ? ff_add(o, v) : FF{fadd(o.h, v.h), 0.0f};
    }
    FF ex = shfl_up_ff(v, 1);
    if (lane == 0) ex = ff_zero();
    if (lane == 31) warp_tot[wid][c] = v;
    loc[c] = ex;
    float a = sabs[c];
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) a += __shfl_xor_sync(0xffffffffu, a, d);
    if (lane == 0) warp_abs[wid][c] = a;
  }
  __syncthreads();

  float Q[7], invQ[7];
#pragma unroll
  for (int c = 0; c < 7; c++) {
    FF off = ff_zero();
    for (uint32_t w = 0; w < wid; w++)
      off = kComp ? ff_add(off, warp_tot[w][c]) : FF{fadd(off.h, warp_tot[w][c].h), 0.0f};
    loc[c] = kComp ? ff_add(off, loc[c]) : FF{fadd(off.h, loc[c].h), 0.0f};
    float S = 0.0f;
    for (int w = 0; w < 8; w++) S += warp_abs[w][c];
    Q[c] = prefix_quantum(S);
    invQ[c] = 1.0f / Q[c];
  }

  auto write_row = [&](uint32_t j) {
    float r[16];
#pragma unroll
    for (int c = 0; c < 7; c++) {
      if (kComp) {
        quantise_prefix(loc[c].h, loc[c].l, Q[c], invQ[c], r[c], r[8 + c]);
      } else {
        r[c] = loc[c].h;
        r[8 + c] = 0.0f;
      }
    }
    r[7] = 0.0f;
    r[15] = 0.0f;
    float4 *o = reinterpret_cast<float4 *>(out + (size_t)j * kPrefixStride);
#pragma unroll
    for (int k = 0; k < 4; k++) o[k] = make_float4(r[4 * k], r[4 * k + 1], r[4 * k + 2], r[4 * k + 3]);
  };

#pragma unroll 4
  for (uint32_t i = i0; i < i1; i++) {
    write_row(i);
#pragma unroll
    for (int c = 0; c < 7; c++) {
      float v = __ldg(x + (size_t)i * 7u + c);
      loc[c] = kComp ? ff_add1(loc[c], v) : FF{fadd(loc[c].h, v), 0.0f};
    }
  }
  if (i0 < N && i1 == N) write_row(N);
}

// ------------------------------------------------------------------ reductions

struct Red {
  float mx;        // running max F (= best)
  int64_t bidx;    // its first flat index
  float s, c;      // sum of exp(F - mx), Kahan-compensated
  float f;         // rectangular rows: plain partial sum of the current
                   // 32-column chunk, added to (s, c) by fold()

  __device__ __forceinline__ void init() {
    mx = -INFINITY;
    bidx = INT64_MAX;
    brow = 0;
    last = 0.0f;
    s = 0.0f;
    c = 0.0f;
    f = 0.0f;
  }
  // Adds 2^d (d <= 0, relative to the running max).  Terms below 2^-60 are
  // dropped: the sum is >= 1, so even 2^22 of them change it by < 2^-38.
  __device__ __forceinline__ void add_small(float d) {
    if (d > -60.0f) add_term(ex2_approx(d));
  }
  __device__ __forceinline__ void add_term(float e) {
    float y = fsub(e, c);
    float t = fadd(s, y);
    c = fsub(fsub(t, s), y);
    s = t;
  }
  // Exponential columns visit rows in descending order at a fixed column:
  // the first occurrence of the max in row-major order is the last row seen
  // with it, so only that row is kept per cell (row_to_index forms the flat
  // index once per column).
  uint32_t brow;  // row (exp columns) or column (rect rows) of the max
  // NaN cells are skipped: they fail both comparisons and the -60 test.
  __device__ __forceinline__ void add_row_desc(float F, uint32_t m) {
    if (F >= mx) {  // one test for the common F < mx
      brow = m;
      if (F > mx) {
        const float sc = ex2_approx((mx - F) * kLog2e);
        s *= sc;
        c *= sc;
        mx = F;
        add_term(1.0f);
        return;
      }
    }
    add_small((F - mx) * kLog2e);
  }
  __device__ __forceinline__ void row_to_index(uint32_t N_tau, uint32_t n) {
    if (mx != -INFINITY) bidx = (int64_t)brow * N_tau + n;
  }
  // Rectangular rows visit columns in ascending order at a fixed row: a tie
  // never replaces the earlier maximum, so only the column of a strictly
  // larger F is kept (brow holds the column here); col_to_index forms the
  // flat index once per row.  The terms go into the plain partial f (at
  // most 32 terms <= 1 between folds, and every term is added: 2^d flushes
  // to 0 below 2^-126, and what lies between adds nothing to a sum >= 1),
  // which the row's walk folds into the Kahan pair after each 32-column
  // chunk: one addition per cell instead of a compensated one and a branch
  // (-2.7 % rect kernel time).
  __device__ __forceinline__ void add_col_asc(float F, uint32_t n) {
    if (F != F) return;  // NaN cells are skipped
    if (F > mx) {
      const float sc = ex2_approx((mx - F) * kLog2e);
      s *= sc;
      c *= sc;
      f *= sc;
      mx = F;
      brow = n;
      f = fadd(f, 1.0f);
      last = ex2_approx(0.0f);  // what add_col_asc would add for F again
    } else {
      last = ex2_approx((F - mx) * kLog2e);
      f = fadd(f, last);
    }
  }
  // add_col_asc for the same F as the previous column's: the same term.
  float last;
  __device__ __forceinline__ void add_col_same(float F) {
    if (F != F) return;
    f = fadd(f, last);
  }
  __device__ __forceinline__ void fold() {
    add_term(f);
    f = 0.0f;
  }
  __device__ __forceinline__ void col_to_index(int64_t rowidx) {
    if (mx != -INFINITY) bidx = rowidx + brow;
  }
};

struct RedVal {
  float mx;
  int64_t bidx;
  float s;
};

__device__ __forceinline__ RedVal red_combine(RedVal a, RedVal b) {
  if (a.mx == -INFINITY) return b;
  if (b.mx == -INFINITY) return a;
  RedVal r;
  if (b.mx > a.mx || (b.mx == a.mx && b.bidx < a.bidx)) {
    r.mx = b.mx;
    r.bidx = b.bidx;
  } else {
    r.mx = a.mx;
    r.bidx = a.bidx;
  }
  r.s = a.s * ex2_approx((a.mx - r.mx) * kLog2e) + b.s * ex2_approx((b.mx - r.mx) * kLog2e);
  return r;
}

__device__ __forceinline__ RedVal shfl_down_red(RedVal v, int d) {
  RedVal o;
  o.mx = __shfl_down_sync(0xffffffffu, v.mx, d);
  o.bidx = __shfl_down_sync(0xffffffffu, v.bidx, d);
  o.s = __shfl_down_sync(0xffffffffu, v.s, d);
  return o;
}

// Reduce a block's per-thread reducers and write one Partial (thread 0).
__device__ void block_reduce_store(const Red &red, Partial *out) {
  __shared__ RedVal sh[kBlock / 32];
  RedVal v{red.mx, red.bidx, fsub(red.s, red.c)};
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) v = red_combine(v, shfl_down_red(v, d));
  const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    RedVal r = sh[0];
    for (int w = 1; w < kBlock / 32; w++) r = red_combine(r, sh[w]);
    Partial p;
    p.maxF = r.mx;
    p.pad = 0;
    p.argmax = r.bidx;
    p.s = (r.mx == -INFINITY) ? 0.0 : (double)r.s;
    *out = p;
  }
  __syncthreads();
}

// ------------------------------------------------------------------ tiles

// Rectangular tile: each thread owns one row (t0) and walks the tile's
// columns, so the row's start index, its prefix row and the u32-wrap state
// are set up once per row; per cell only the end index and one prefix row
// are needed, and the next cell's prefix row is loaded while the current
// cell is computed.  A call covers the 32 rows of row group my_rg and
// column range my_cg of cgs equal ranges: one-tile-per-block launches give
// the block's 4 warps (rg row groups) x (4/rg column ranges), persistent
// launches give one warp all row groups in turn with cgs = 1.  The columns'
// taus are staged 32 at a time in the warp's `stau` slots of shared memory
// (one coalesced load per 32 columns instead of a global load on every
// cell's end-index chain).  With a map to write, each warp transposes
// 32 x 32 blocks through shared memory so that global stores are
// row-contiguous.
template <bool kWrite, int kPrec>
__device__ void rect_tile(const TemplateDev &t, const WorkItem &w,
                          const uint32_t *__restrict__ t0s_all,
                          const uint32_t *__restrict__ taus_all, const float *__restrict__ P_all,
                          float *__restrict__ Fmn, Red &red, float *smw, uint32_t my_rg,
                          uint32_t cgs, uint32_t my_cg, uint32_t *stau) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t mbase = w.m0 + 32u * my_rg;
  const uint32_t m = mbase + lane;
  const bool row_ok = m < w.m1;
  const uint32_t ncols = w.n1 - w.n0;
  const uint32_t per = (ncols + cgs - 1u) / cgs;
  const uint32_t nb = min(w.n1, w.n0 + my_cg * per), ne = min(w.n1, nb + per);
  const uint32_t *t0s = t0s_all + t.t0_off;
  const uint32_t *taus = taus_all + t.tau_off;
  const float *P = P_all + t.p_off * kPrefixStride;
  const uint32_t tau_first = __ldg(taus);
  uint32_t t0 = 0, j0 = 0, ef = 0;
  bool wr = false;
  float row0[16];
  if (row_ok) {
    t0 = __ldg(t0s + m);
    j0 = idx_start(t0, t.g);
    wr = rect_row_wrapped(t0, tau_first, t.g);
    ef = wr ? idx_end(t0 + tau_first, t.g) : 0u;
    TCW_DCHECK(j0 <= t.g.numAtoms);
    ld_row16(P + (size_t)j0 * kPrefixStride, row0);
  }
  auto end_of = [&](uint32_t tau) {
    uint32_t e = idx_end(t0 + tau, t.g);
    return (wr && ef > e) ? ef : e;
  };
  const int64_t rowidx = (int64_t)m * t.N_tau;
  // e < numAtoms always, so prefix row e + 1 exists even for empty windows
  uint32_t e_cur = 0;
  float cur[16], nxt[16];
  if (row_ok && nb < ne) {
    e_cur = end_of(__ldg(taus + nb));
    TCW_DCHECK(e_cur + 1u <= t.g.numAtoms);
    ld_row16(P + (size_t)(e_cur + 1u) * kPrefixStride, cur);
  }
  // One cell: F of column n from prefix row `a` (end ea); the next column's
  // prefix row is loaded into `b` (end eb) while this one is computed.  A
  // column whose window end equals the previous column's has the same
  // window, hence the same F: it takes the previous F, and its prefix row is
  // not loaded (the window ends of a row are clamped at the last atom once
  // t0 + tau passes the data, and taus closer than TAtom share ends).
  uint32_t e_prev = 0xFFFFFFFFu;  // end of the previous column (none yet)
  float F_prev = 2.0f;
  auto cell = [&](uint32_t n, uint32_t cb, const float *a, uint32_t ea, float *b,
                  uint32_t &eb) {
    if (row_ok && n + 1u < ne) {
      eb = end_of(n + 1u < cb + 32u ? stau[n + 1u - cb] : __ldg(taus + n + 1u));
      TCW_DCHECK(eb + 1u <= t.g.numAtoms);
      if (eb != ea) ld_row16(P + (size_t)(eb + 1u) * kPrefixStride, b);
    }
    float F = F_prev;
    if (row_ok) {
      if (ea != e_prev) F = 2.0f;
      if (ea != e_prev && ea >= j0) {
        bool ok;
        if (kPrec == kPrecPlain32) {
          F = fstat_plain32(fsub(a[0], row0[0]), fsub(a[1], row0[1]), fsub(a[2], row0[2]),
                            fsub(a[3], row0[3]), fsub(a[4], row0[4]), fsub(a[5], row0[5]),
                            fsub(a[6], row0[6]), ok);
        } else {
          FF2 W[4];
#pragma unroll
          for (int k = 0; k < 4; k++) {
            W[k].h = sub2(F2{a[2 * k], a[2 * k + 1]}, F2{row0[2 * k], row0[2 * k + 1]});
            W[k].l = sub2(F2{a[8 + 2 * k], a[9 + 2 * k]}, F2{row0[8 + 2 * k], row0[9 + 2 * k]});
          }
          F = fstat_tiered2<kPrec == kPrecFF_F64Det>(W, ok);
        }
      }
      if (ea != e_prev)
        red.add_col_asc(F, n);
      else
        red.add_col_same(F);
    }
    e_prev = ea;
    F_prev = F;
    if (kWrite) smw[lane * 33u + (n - cb)] = F;
  };
  for (uint32_t cb = nb; cb < ne; cb += 32u) {
    const uint32_t ce = min(ne, cb + 32u);
    __syncwarp();
    if (cb + lane < ne) stau[lane] = __ldg(taus + cb + lane);
    __syncwarp();
    // A chunk inside every warp row's clamped run -- the window ends of the
    // previous column and of column cb at the last atom, the chunk's taus
    // (and the next chunk's first) non-decreasing, t0 + tau past the u32
    // wrap of the reference's end index and without overflow, TAtom >= 2 (so
    // the end index's quotient never reaches 2^31) -- has the last atom as
    // every window end, so every column repeats the previous F.
    const uint32_t nlast = ce - cb - 1u;
    const uint32_t tx = ce < ne ? __ldg(taus + ce) : 0u;
    bool mono = true;
    if (lane < nlast) mono = stau[lane] <= stau[lane + 1u];
    if (lane == nlast && ce < ne) mono = stau[lane] <= tx;
    const uint32_t tmax = ce < ne ? tx : stau[nlast];
    const bool clamped_run =
        !row_ok || (t.g.TAtom >= 2u && e_cur == t.g.numAtoms - 1u &&
                    e_prev == t.g.numAtoms - 1u &&
                    (uint64_t)t0 + stau[0] + t.g.half >= (uint64_t)t.g.t0_data &&
                    (uint64_t)t0 + tmax + t.g.half - t.g.t0_data <= 0xFFFFFFFFull &&
                    (uint64_t)t0 + tmax <= 0xFFFFFFFFull);
    uint32_t n = cb;
    if (__all_sync(0xffffffffu, mono && clamped_run)) {
      for (; n < ce; n++) {
        if (row_ok) red.add_col_same(F_prev);
        if (kWrite) smw[lane * 33u + (n - cb)] = F_prev;
      }
      e_cur = t.g.numAtoms - 1u;  // the end of column ce
    }
    // ping-pong between the two row buffers; `cur` holds column n on entry
    for (; n + 1u < ce; n += 2u) {
      uint32_t e_nxt = 0;
      cell(n, cb, cur, e_cur, nxt, e_nxt);
      cell(n + 1u, cb, nxt, e_nxt, cur, e_cur);
    }
    if (n < ce) {  // odd chunk length: one more cell, then its successor moves to `cur`
      uint32_t e_nxt = 0;
      cell(n, cb, cur, e_cur, nxt, e_nxt);
#pragma unroll
      for (int k = 0; k < 16; k++) cur[k] = nxt[k];
      e_cur = e_nxt;
    }
    if (kWrite) {
      __syncwarp();
      const uint32_t col = cb + lane;
      for (uint32_t r = 0; r < 32u; r++) {
        const uint32_t mr = mbase + r;
        if (mr < w.m1 && col < ce) Fmn[t.map_off + (size_t)mr * t.N_tau + col] = smw[r * 33u + lane];
      }
      __syncwarp();
    }
    red.fold();
  }
  if (row_ok) red.col_to_index(rowidx);
}

template <bool kWrite>
struct MapSink {
  float *Fmn;
  uint32_t N_tau, n;
  Red *red;
  __device__ __forceinline__ void operator()(uint32_t m, float F, bool) {
    TCW_DCHECK(n < N_tau);
    if (kWrite) Fmn[(size_t)m * N_tau + n] = F;
    red->add_row_desc(F, m);
  }
};

// Exponential tile: each thread runs one tau column over a chunk of rows
// (the chunk is the same for the 32 lanes of a warp: tn >= 32).  When every
// row of the warp's chunk satisfies exp_row_regular for its columns' largest
// tau, the per-row quantities (ExpRow: window start, first non-zero atom,
// t0 split by TAtom) are tabulated 128 rows at a time by the warp itself in
// its own shared-memory slots (no block barrier) and every cell takes the
// division-free window end of ExpColumn; otherwise the warp runs
// exp_column2's generic index arithmetic.  Both give identical results.
constexpr uint32_t kExpRowTab = 128;

// The row-table walk of one warp's column chunk [mb, me) (regular rows):
// row tables of kExpRowTab rows built by the warp, then each lane's column
// slides down them (ExpColumn).
template <int kPrec, class Sink>
__device__ __forceinline__ void exp_rows(const TemplateDev &t, const float *__restrict__ a8,
                                         const uint32_t *__restrict__ t0s, uint32_t mb,
                                         uint32_t me, uint32_t tau, bool active, Sink &sink,
                                         ExpRow *tab) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t *a8u = reinterpret_cast<const uint32_t *>(a8);
  ExpColumn<kPrec == kPrecFF_F64Det, true> C;
  C.init(t.g, tau);
  for (uint32_t ce = me; ce > mb;) {
    const uint32_t cb = ce - mb > kExpRowTab ? ce - kExpRowTab : mb;
    __syncwarp();
    uint32_t t0min = 0xFFFFFFFFu;
    for (uint32_t r = lane; r < ce - cb; r += 32u) {
      const uint32_t t0 = __ldg(t0s + cb + r);
      t0min = min(t0min, t0);
      ExpRow e;
      e.lo = exp_lo(t0, t.g);
      e.nz = e.lo < t.g.numAtoms ? __ldg(a8u + (size_t)e.lo * 8u + 3u) : 0xFFFFFFFFu;
      const uint32_t d = t0 - t.g.t0_data;
      e.a = fdiv(d, t.g.div);
      e.b = d - e.a * t.g.TAtom;
      tab[r] = e;
    }
    __syncwarp();
    // the window end grows with t0: if it is clamped at numAtoms for the
    // chunk's smallest t0, it is for every row of the chunk
    ExpRow e0;
    const uint32_t d0 = __reduce_min_sync(0xffffffffu, t0min) - t.g.t0_data;
    e0.a = fdiv(d0, t.g.div);
    e0.b = d0 - e0.a * t.g.TAtom;
    const bool clamped = __all_sync(0xffffffffu, !active || C.top_raw(e0) >= t.g.numAtoms);
    // window starts that never grow along the walk (t0 non-decreasing in m)
    bool mono = true;
    for (uint32_t r = lane; r + 1u < ce - cb; r += 32u) mono = mono && tab[r].lo <= tab[r + 1u].lo;
    mono = __all_sync(0xffffffffu, mono);
    if (active) {
      if (clamped && mono) {
        // the rows before the first window with an atom, that row, then the
        // steady rows (row_steady's conditions hold for all of them; after
        // the first window with data, row_steady_data's too)
        uint32_t m = ce;
        while (m > cb) {
          m--;
          const ExpRow &e = tab[m - cb];
          C.row_clamped(a8, t.g, e, m, sink);
          if (e.lo < t.g.numAtoms) break;
        }
        // once a window holds data, every later (lower-starting) one does
        while (m > cb) {
          m--;
          const ExpRow &e = tab[m - cb];
          C.row_steady(a8, t.g, e, m, sink);
          if (e.nz < t.g.numAtoms) break;
        }
        while (m > cb) {
          m--;
          C.row_steady_data(a8, t.g, tab[m - cb], m, sink);
        }
      } else if (clamped) {
        for (uint32_t m = ce; m > cb;) {
          m--;
          C.row_clamped(a8, t.g, tab[m - cb], m, sink);
        }
      } else {
        for (uint32_t m = ce; m > cb;) {
          m--;
          C.row(a8, t.g, tab[m - cb], m, sink);
        }
      }
    }
    ce = cb;
  }
}

template <bool kWrite, int kPrec>
__device__ void exp_tile(const TemplateDev &t, const WorkItem &w, const float *__restrict__ atoms,
                         const float *__restrict__ atoms8,
                         const uint32_t *__restrict__ t0s_all,
                         const uint32_t *__restrict__ taus_all, float *__restrict__ Fmn,
                         Red &red, ExpRow *tab, bool warp_tile = false) {
  const uint32_t *t0s = t0s_all + t.t0_off;
  const uint32_t tn = w.tn;
  const uint32_t lane = threadIdx.x & 31u;
  // a warp tile (persistent launches) is 32 columns over all the tile's rows
  const uint32_t col = warp_tile ? lane : threadIdx.x % tn;
  const uint32_t rl = warp_tile ? 0u : threadIdx.x / tn;
  const uint32_t n = w.n0 + col;
  const uint32_t R = w.rows_per_lane;
  const uint32_t mb = w.m0 + rl * R;
  if (mb >= w.m1) return;  // uniform per warp (tn >= 32)
  const uint32_t me = min(w.m1, mb + R);
  const bool active = n < w.n1;
  const uint32_t tau = active ? __ldg(taus_all + t.tau_off + n) : 0u;
  MapSink<kWrite> sink{kWrite ? Fmn + t.map_off : nullptr, t.N_tau, n, &red};
  if (kPrec == kPrecPlain32) {
    if (active) {
      exp_column<false, false>(atoms + t.atom_off * 7u, t.g, t0s, mb, me, tau, sink, nullptr);
      red.row_to_index(t.N_tau, n);
    }
    return;
  }
  const float *a8 = atoms8 + t.a8_off * 8u;
  const uint32_t taumax = __reduce_max_sync(0xffffffffu, tau);
  bool reg = true;
  for (uint32_t m = mb + lane; m < me; m += 32u)
    reg = reg && exp_row_regular(__ldg(t0s + m), taumax, t.g);
  if (!__all_sync(0xffffffffu, reg)) {
    if (active) {
      exp_column2<kPrec == kPrecFF_F64Det>(a8, t.g, t0s, mb, me, tau, sink, nullptr);
      red.row_to_index(t.N_tau, n);
    }
    return;
  }
  exp_rows<kPrec>(t, a8, t0s, mb, me, tau, active, sink, tab);
  if (active) red.row_to_index(t.N_tau, n);
}

// Minimum resident blocks per SM requested from the register allocator
// (build-time tunables; 1 leaves the allocation to ptxas).
#ifndef TCW_RECT_MIN_BLOCKS
#define TCW_RECT_MIN_BLOCKS 5
#endif
// The persistent exp kernels (the batched plans' hot kernels, with or
// without maps) run fastest at 8 blocks (64 registers, a few spilled); the
// one-tile-per-block exp kernels of single-template calls keep 96 registers
// without spills (their grids are small, so latency matters more than
// occupancy).
#ifndef TCW_EXP_MIN_BLOCKS
#define TCW_EXP_MIN_BLOCKS 8
#endif
#ifndef TCW_EXP_MIN_BLOCKS_OTHER
#define TCW_EXP_MIN_BLOCKS_OTHER 5
#endif

template <int kWin, bool kPersist, bool kWrite>
constexpr int map_min_blocks() {
  return kWin == TCW_WINDOW_RECT ? TCW_RECT_MIN_BLOCKS
         : kPersist ? TCW_EXP_MIN_BLOCKS
                                 : TCW_EXP_MIN_BLOCKS_OTHER;
}

template <int kWin, bool kPersist, bool kWrite, int kPrec>
__global__ void __launch_bounds__(kBlock, (map_min_blocks<kWin, kPersist, kWrite>()))
    map_kernel(const TemplateDev *__restrict__ T, const WorkItem *__restrict__ items,
               uint32_t n_items, uint32_t *__restrict__ counter, const float *__restrict__ atoms,
               const float *__restrict__ atoms8, const uint32_t *__restrict__ t0s,
               const uint32_t *__restrict__ taus,
               const float *__restrict__ P, float *__restrict__ Fmn,
               Partial *__restrict__ parts) {
  __shared__ uint32_t s_item;
  constexpr uint32_t kSmem = kWin == TCW_WINDOW_RECT ? (kWrite ? (kBlock / 32) * 32 * 33 : 1)
                                                     : (kBlock / 32) * kExpRowTab * 4;
  __shared__ __align__(16) uint32_t sm[kSmem];
  __shared__ uint32_t s_tau[kWin == TCW_WINDOW_RECT ? kBlock : 1];
  if (kWin == TCW_WINDOW_RECT && kPersist) {
    // Persistent rectangular launches schedule by warp: each warp fetches
    // whole tiles and walks their 32-row groups in turn, merging the groups'
    // reducers in row order, so no block barrier waits on the slowest warp
    // (rect warps share no shared memory).
    const uint32_t lane = threadIdx.x & 31u;
    float *smw = reinterpret_cast<float *>(sm) + (threadIdx.x >> 5) * (32 * 33);
    for (;;) {
      uint32_t it2 = 0;
      if (lane == 0) it2 = atomicAdd(counter, 1u);
      it2 = __shfl_sync(0xffffffffu, it2, 0);
      if (it2 >= n_items) break;
      const WorkItem w = items[it2];
      const TemplateDev t = T[w.tmpl];
      RedVal acc{-INFINITY, INT64_MAX, 0.0f};
      for (uint32_t g = 0; g < w.tn; g++) {
        Red red;
        red.init();
        rect_tile<kWrite, kPrec>(t, w, t0s, taus, P, Fmn, red, smw, g, 1u, 0u,
                                 s_tau + (threadIdx.x >> 5) * 32u);
        acc = red_combine(acc, RedVal{red.mx, red.bidx, fsub(red.s, red.c)});
      }
#pragma unroll
      for (int d = 16; d > 0; d >>= 1) acc = red_combine(acc, shfl_down_red(acc, d));
      if (lane == 0) {
        Partial pp;
        pp.maxF = acc.mx;
        pp.pad = 0;
        pp.argmax = acc.bidx;
        pp.s = (acc.mx == -INFINITY) ? 0.0 : (double)acc.s;
        parts[w.part] = pp;
      }
    }
    return;
  }
  if (kWin == TCW_WINDOW_EXP && kPersist) {
    // Persistent exponential launches schedule by warp as well: each warp
    // fetches 32-column tiles (all rows of a row chunk), keeps its row table
    // in its own shared-memory slots and reduces its tile itself, so no block
    // barrier waits for the warp with the most removals.
    const uint32_t lane = threadIdx.x & 31u;
    ExpRow *tab = reinterpret_cast<ExpRow *>(sm) + (threadIdx.x >> 5) * kExpRowTab;
    for (;;) {
      uint32_t it2 = 0;
      if (lane == 0) it2 = atomicAdd(counter, 1u);
      it2 = __shfl_sync(0xffffffffu, it2, 0);
      if (it2 >= n_items) break;
      const WorkItem w = items[it2];
      const TemplateDev t = T[w.tmpl];
      Red red;
      red.init();
      exp_tile<kWrite, kPrec>(t, w, atoms, atoms8, t0s, taus, Fmn, red, tab, true);
      RedVal acc{red.mx, red.bidx, fsub(red.s, red.c)};
#pragma unroll
      for (int d = 16; d > 0; d >>= 1) acc = red_combine(acc, shfl_down_red(acc, d));
      if (lane == 0) {
        Partial pp;
        pp.maxF = acc.mx;
        pp.pad = 0;
        pp.argmax = acc.bidx;
        pp.s = (acc.mx == -INFINITY) ? 0.0 : (double)acc.s;
        parts[w.part] = pp;
      }
      __syncwarp();
    }
    return;
  }
  uint32_t it = blockIdx.x;
  for (;;) {
    if (kPersist) {
      if (threadIdx.x == 0) s_item = atomicAdd(counter, 1u);
      __syncthreads();
      it = s_item;
      __syncthreads();
    }
    if (it >= n_items) break;
    const WorkItem w = items[it];
    const TemplateDev t = T[w.tmpl];
    Red red;
    red.init();
    if (kWin == TCW_WINDOW_RECT) {
      const uint32_t warp = threadIdx.x >> 5, rg = w.tn;
      rect_tile<kWrite, kPrec>(t, w, t0s, taus, P, Fmn, red,
                               reinterpret_cast<float *>(sm) + warp * (32 * 33), warp % rg,
                               4u / rg, warp / rg, s_tau + warp * 32u);
    } else
      exp_tile<kWrite, kPrec>(t, w, atoms, atoms8, t0s, taus, Fmn, red,
                              reinterpret_cast<ExpRow *>(sm) + (threadIdx.x >> 5) * kExpRowTab);
    block_reduce_store(red, parts + w.part);
    if (!kPersist) break;
  }
}

// ------------------------------------------------------------------ finalize

// One warp per template: merge its partials in index order.
__global__ void __launch_bounds__(128) finalize_kernel(const TemplateDev *__restrict__ T,
                                                       uint32_t n_templates,
                                                       const Partial *__restrict__ parts,
                                                       tcw_result *__restrict__ results) {
  const uint32_t tmpl = blockIdx.x * 4u + (threadIdx.x >> 5);
  const uint32_t lane = threadIdx.x & 31u;
  if (tmpl >= n_templates) return;
  const TemplateDev t = T[tmpl];
  float best = -INFINITY;
  int64_t bidx = INT64_MAX;
  for (uint32_t k = lane; k < t.n_parts; k += 32) {
    const Partial p = parts[t.part_off + k];
    if (p.maxF > best || (p.maxF == best && p.argmax < bidx)) {
      best = p.maxF;
      bidx = p.argmax;
    }
  }
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) {
    float ob = __shfl_xor_sync(0xffffffffu, best, d);
    int64_t oi = __shfl_xor_sync(0xffffffffu, bidx, d);
    if (ob > best || (ob == best && oi < bidx)) {
      best = ob;
      bidx = oi;
    }
  }
  double S = 0.0;
  for (uint32_t k = lane; k < t.n_parts; k += 32) {
    const Partial p = parts[t.part_off + k];
    if (p.s > 0.0) S += p.s * (double)exp2f((p.maxF - best) * kLog2e);
  }
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) S += __shfl_xor_sync(0xffffffffu, S, d);
  if (lane == 0) {
    tcw_result r;
    r.maxF = best;
    r.argmax = bidx;
    r.lnBtSG = log(70.0 / ((double)t.N_t0 * (double)t.N_tau)) + (double)best + log(S);
    r.t0_mp_idx = -1;
    r.tau_mp_idx = -1;
    r.status = 0;
    results[tmpl] = r;
  }
}

// ------------------------------------------------------------------ posteriors

constexpr uint32_t kColChunk = 64;

__global__ void __launch_bounds__(256) rowsum_kernel(const float *__restrict__ Fmn,
                                                     const tcw_result *__restrict__ res,
                                                     uint32_t N_tau, double *__restrict__ rowsum) {
  const float maxF = res->maxF;
  const float *row = Fmn + (size_t)blockIdx.x * N_tau;
  float s = 0.0f, c = 0.0f;
  for (uint32_t n = threadIdx.x; n < N_tau; n += blockDim.x) {
    float y = fsub(exp2f((row[n] - maxF) * kLog2e), c);
    float t = fadd(s, y);
    c = fsub(fsub(t, s), y);
    s = t;
  }
  double v = (double)s - (double)c;
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
  __shared__ double sh[8];
  if ((threadIdx.x & 31u) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double tot = 0.0;
    for (int w = 0; w < 8; w++) tot += sh[w];
    rowsum[blockIdx.x] = tot;
  }
}

__global__ void __launch_bounds__(128) colsum_kernel(const float *__restrict__ Fmn,
                                                     const tcw_result *__restrict__ res,
                                                     uint32_t N_t0, uint32_t N_tau,
                                                     double *__restrict__ colpart) {
  const uint32_t n = blockIdx.x * 128u + threadIdx.x;
  if (n >= N_tau) return;
  const float maxF = res->maxF;
  const uint32_t m0 = blockIdx.y * kColChunk, m1 = min(N_t0, m0 + kColChunk);
  float s = 0.0f, c = 0.0f;
  for (uint32_t m = m0; m < m1; m++) {
    float y = fsub(exp2f((Fmn[(size_t)m * N_tau + n] - maxF) * kLog2e), c);
    float t = fadd(s, y);
    c = fsub(fsub(t, s), y);
    s = t;
  }
  colpart[(size_t)blockIdx.y * N_tau + n] = (double)s - (double)c;
}

// First-occurrence argmax of the row sums and of the chunked column sums.
__global__ void __launch_bounds__(1024) posterior_argmax_kernel(const double *__restrict__ rowsum,
                                                                const double *__restrict__ colpart,
                                                                uint32_t N_t0, uint32_t N_tau,
                                                                uint32_t n_chunks,
                                                                tcw_result *__restrict__ res) {
  __shared__ double sv[32];
  __shared__ int64_t si[32];
  for (int pass = 0; pass < 2; pass++) {
    const uint32_t N = pass == 0 ? N_t0 : N_tau;
    double best = -1.0;
    int64_t bidx = INT64_MAX;
    for (uint32_t k = threadIdx.x; k < N; k += blockDim.x) {
      double v;
      if (pass == 0) {
        v = rowsum[k];
      } else {
        v = 0.0;
        for (uint32_t ch = 0; ch < n_chunks; ch++) v += colpart[(size_t)ch * N_tau + k];
      }
      if (v > best) {  // k increases within a thread: keeps the first
        best = v;
        bidx = k;
      }
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
      double ob = __shfl_xor_sync(0xffffffffu, best, d);
      int64_t oi = __shfl_xor_sync(0xffffffffu, bidx, d);
      if (ob > best || (ob == best && oi < bidx)) {
        best = ob;
        bidx = oi;
      }
    }
    if ((threadIdx.x & 31u) == 0) {
      sv[threadIdx.x >> 5] = best;
      si[threadIdx.x >> 5] = bidx;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      best = sv[0];
      bidx = si[0];
      for (uint32_t w = 1; w < blockDim.x / 32u; w++) {
        if (sv[w] > best || (sv[w] == best && si[w] < bidx)) {
          best = sv[w];
          bidx = si[w];
        }
      }
      if (pass == 0)
        res->t0_mp_idx = bidx;
      else
        res->tau_mp_idx = bidx;
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------------ launchers

cudaError_t launch_prefix(const TemplateDev *d_T, const uint32_t *d_rect_list, uint32_t n_rect,
                          const float *d_atoms, float *d_P, int prec, cudaStream_t stream) {
  if (n_rect == 0) return cudaSuccess;
  if (prec == kPrecPlain32)
    prefix_kernel<false><<<n_rect, 256, 0, stream>>>(d_T, d_rect_list, d_atoms, d_P);
  else
    prefix_kernel<true><<<n_rect, 256, 0, stream>>>(d_T, d_rect_list, d_atoms, d_P);
  return cudaGetLastError();
}

template <int kWin, bool kPersist, bool kWrite>
static cudaError_t launch_map_prec(int prec, uint32_t grid, cudaStream_t s, int priority,
                                   const TemplateDev *T, const WorkItem *items, uint32_t n_items,
                                   uint32_t *counter, const float *atoms, const float *atoms8,
                                   const uint32_t *t0s, const uint32_t *taus, const float *P,
                                   float *Fmn, Partial *parts) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(kBlock);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributePriority;
  attr[0].val.priority = priority;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (prec == kPrecPlain32)
    return cudaLaunchKernelEx(&cfg, map_kernel<kWin, kPersist, kWrite, kPrecPlain32>, T, items,
                              n_items, counter, atoms, atoms8, t0s, taus, P, Fmn, parts);
  if (prec == kPrecFF_F64Det)
    return cudaLaunchKernelEx(&cfg, map_kernel<kWin, kPersist, kWrite, kPrecFF_F64Det>, T, items,
                              n_items, counter, atoms, atoms8, t0s, taus, P, Fmn, parts);
  return cudaLaunchKernelEx(&cfg, map_kernel<kWin, kPersist, kWrite, kPrecFF>, T, items, n_items,
                            counter, atoms, atoms8, t0s, taus, P, Fmn, parts);
}

template <int kWin>
static cudaError_t launch_map_win(const MapLaunch &L, cudaStream_t stream) {
  if (L.n_items == 0) return cudaSuccess;
  const uint32_t grid = L.persistent ? L.n_blocks : L.n_items;
  if (L.persistent) {
    if (L.write_map)
      return launch_map_prec<kWin, true, true>(L.prec, grid, stream, L.priority, L.T, L.items,
                                               L.n_items, L.counter, L.atoms, L.atoms8, L.t0s, L.taus, L.P,
                                               L.Fmn, L.parts);
    return launch_map_prec<kWin, true, false>(L.prec, grid, stream, L.priority, L.T, L.items,
                                              L.n_items, L.counter, L.atoms, L.atoms8, L.t0s, L.taus, L.P,
                                              L.Fmn, L.parts);
  }
  if (L.write_map)
    return launch_map_prec<kWin, false, true>(L.prec, grid, stream, L.priority, L.T, L.items,
                                              L.n_items, L.counter, L.atoms, L.atoms8, L.t0s, L.taus, L.P,
                                              L.Fmn, L.parts);
  return launch_map_prec<kWin, false, false>(L.prec, grid, stream, L.priority, L.T, L.items,
                                             L.n_items, L.counter, L.atoms, L.atoms8, L.t0s, L.taus, L.P,
                                             L.Fmn, L.parts);
}

cudaError_t launch_repack(const TemplateDev *d_T, const uint32_t *d_exp_list, uint32_t n_exp,
                          const float *d_atoms, float *d_atoms8, cudaStream_t stream) {
  if (n_exp == 0) return cudaSuccess;
  repack_kernel<<<n_exp, 256, 0, stream>>>(d_T, d_exp_list, d_atoms, d_atoms8);
  return cudaGetLastError();
}

cudaError_t launch_map(int window, const MapLaunch &L, cudaStream_t stream) {
  cudaError_t e = window == TCW_WINDOW_RECT ? launch_map_win<TCW_WINDOW_RECT>(L, stream)
                                            : launch_map_win<TCW_WINDOW_EXP>(L, stream);
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

template <int kWin>
static int blocks_per_sm_win(int prec) {
  int n = 0;
  cudaError_t e;
  if (prec == kPrecPlain32)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &n, map_kernel<kWin, true, false, kPrecPlain32>, kBlock, 0);
  else if (prec == kPrecFF_F64Det)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &n, map_kernel<kWin, true, false, kPrecFF_F64Det>, kBlock, 0);
  else
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, map_kernel<kWin, true, false, kPrecFF>,
                                                      kBlock, 0);
  if (e != cudaSuccess) {
    cudaGetLastError();
    n = 1;
  }
  return n > 0 ? n : 1;
}

// Resident blocks per SM of the persistent (map-less) kernel of a window.
int map_blocks_per_sm(int window, int prec) {
  return window == TCW_WINDOW_RECT ? blocks_per_sm_win<TCW_WINDOW_RECT>(prec)
                                   : blocks_per_sm_win<TCW_WINDOW_EXP>(prec);
}

// One template, one block: the partials of a large single-template call (up
// to thousands of tiles) merged by 256 threads; warps' results combined in
// warp order.
__global__ void __launch_bounds__(256) finalize_one_kernel(const TemplateDev *__restrict__ T,
                                                           const Partial *__restrict__ parts,
                                                           tcw_result *__restrict__ results) {
  __shared__ float s_best[8];
  __shared__ int64_t s_bidx[8];
  __shared__ double s_sum[8];
  const TemplateDev t = T[0];
  const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
  float best = -INFINITY;
  int64_t bidx = INT64_MAX;
  for (uint32_t k = threadIdx.x; k < t.n_parts; k += blockDim.x) {
    const Partial p = parts[t.part_off + k];
    if (p.maxF > best || (p.maxF == best && p.argmax < bidx)) {
      best = p.maxF;
      bidx = p.argmax;
    }
  }
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) {
    float ob = __shfl_xor_sync(0xffffffffu, best, d);
    int64_t oi = __shfl_xor_sync(0xffffffffu, bidx, d);
    if (ob > best || (ob == best && oi < bidx)) {
      best = ob;
      bidx = oi;
    }
  }
  if (lane == 0) {
    s_best[wid] = best;
    s_bidx[wid] = bidx;
  }
  __syncthreads();
  best = s_best[0];
  bidx = s_bidx[0];
  for (uint32_t w = 1; w < blockDim.x / 32u; w++)
    if (s_best[w] > best || (s_best[w] == best && s_bidx[w] < bidx)) {
      best = s_best[w];
      bidx = s_bidx[w];
    }
  double S = 0.0;
  for (uint32_t k = threadIdx.x; k < t.n_parts; k += blockDim.x) {
    const Partial p = parts[t.part_off + k];
    if (p.s > 0.0) S += p.s * (double)exp2f((p.maxF - best) * kLog2e);
  }
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) S += __shfl_xor_sync(0xffffffffu, S, d);
  if (lane == 0) s_sum[wid] = S;
  __syncthreads();
  if (threadIdx.x == 0) {
    S = 0.0;
    for (uint32_t w = 0; w < blockDim.x / 32u; w++) S += s_sum[w];
    tcw_result r;
    r.maxF = best;
    r.argmax = bidx;
    r.lnBtSG = log(70.0 / ((double)t.N_t0 * (double)t.N_tau)) + (double)best + log(S);
    r.t0_mp_idx = -1;
    r.tau_mp_idx = -1;
    r.status = 0;
    results[0] = r;
  }
}

cudaError_t launch_finalize(const TemplateDev *d_T, uint32_t n_templates, const Partial *d_parts,
                            void *d_results, cudaStream_t stream) {
  if (n_templates == 0) return cudaSuccess;
  if (n_templates == 1)
    finalize_one_kernel<<<1, 256, 0, stream>>>(d_T, d_parts,
                                               reinterpret_cast<tcw_result *>(d_results));
  else
    finalize_kernel<<<(n_templates + 3u) / 4u, 128, 0, stream>>>(
        d_T, n_templates, d_parts, reinterpret_cast<tcw_result *>(d_results));
  return cudaGetLastError();
}

// Batched posteriors of a plan whose maps were written (tcw:219-287): the
// row and column sums of exp(F - maxF) in one read of the maps.  A block
// owns kPostCols columns of one template: each thread sums its four
// adjacent columns down the rows (FP32, Kahan); the block's row sums (the
// thread's four terms, warp shuffles, then shared memory) are stored per
// column chunk and summed in FP64 by the argmax kernel (no global atomics).
constexpr uint32_t kPostRowTile = 1024;
constexpr uint32_t kPostThreads = 256;  // kPostCols / 4: four adjacent columns per thread

__global__ void __launch_bounds__(kPostThreads) post_sums_kernel(
    const TemplateDev *__restrict__ T, const uint2 *__restrict__ chunks,
    const float *__restrict__ maps, const tcw_result *__restrict__ results,
    float *__restrict__ rowpart, double *__restrict__ colsum) {
  __shared__ float srow[kPostRowTile];
  const uint2 ch = chunks[blockIdx.x];
  const TemplateDev t = T[ch.x];
  const float maxF = results[ch.x].maxF;
  const float *F = maps + t.map_off;
  const uint32_t n0 = ch.y + 4u * threadIdx.x;  // this thread's first column
  const uint32_t lane = threadIdx.x & 31u;
  float *rp = rowpart + t.row_off + (size_t)(ch.y / kPostCols) * t.N_t0;  // this chunk's rows
  float cs[4] = {0, 0, 0, 0}, cc[4] = {0, 0, 0, 0};
  for (uint32_t m0 = 0; m0 < t.N_t0; m0 += kPostRowTile) {
    const uint32_t m1 = min(t.N_t0, m0 + kPostRowTile);
    for (uint32_t k = threadIdx.x; k < kPostRowTile; k += kPostThreads) srow[k] = 0.0f;
    __syncthreads();
    // four rows per step: independent loads and shuffle chains
    for (uint32_t m = m0; m < m1; m += 4u) {
      float w[4];
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const uint32_t mq = m + q;
        const float *row = F + (size_t)mq * t.N_tau;
        float e[4];
#pragma unroll
        for (int j = 0; j < 4; j++)
          e[j] = (mq < m1 && n0 + j < t.N_tau) ? ex2_approx((row[n0 + j] - maxF) * kLog2e) : 0.0f;
#pragma unroll
        for (int j = 0; j < 4; j++) {
          const float y = fsub(e[j], cc[j]);
          const float u = fadd(cs[j], y);
          cc[j] = fsub(fsub(u, cs[j]), y);
          cs[j] = u;
        }
        w[q] = fadd(fadd(e[0], e[1]), fadd(e[2], e[3]));
      }
#pragma unroll
      for (int d = 16; d > 0; d >>= 1) {
#pragma unroll
        for (int q = 0; q < 4; q++) w[q] += __shfl_xor_sync(0xffffffffu, w[q], d);
      }
      if (lane == 0) {
#pragma unroll
        for (int q = 0; q < 4; q++)
          if (m + q < m1 && w[q] != 0.0f) atomicAdd(&srow[m + q - m0], w[q]);
      }
    }
    __syncthreads();
    for (uint32_t k = threadIdx.x; k < m1 - m0; k += kPostThreads) rp[m0 + k] = srow[k];
    __syncthreads();
  }
#pragma unroll
  for (int j = 0; j < 4; j++)
    if (n0 + j < t.N_tau) colsum[t.col_off + n0 + j] = (double)cs[j] - (double)cc[j];
}

// One warp per template: first-occurrence argmax of its row sums (the
// column chunks' partials summed in FP64) and of its column sums.
__global__ void __launch_bounds__(128) post_argmax_kernel(const TemplateDev *__restrict__ T,
                                                          uint32_t n_templates,
                                                          const float *__restrict__ rowpart,
                                                          const double *__restrict__ colsum,
                                                          tcw_result *__restrict__ results) {
  const uint32_t tmpl = blockIdx.x * 4u + (threadIdx.x >> 5);
  const uint32_t lane = threadIdx.x & 31u;
  if (tmpl >= n_templates) return;
  const TemplateDev t = T[tmpl];
  int64_t out[2];
  for (int pass = 0; pass < 2; pass++) {
    const uint32_t N = pass == 0 ? t.N_t0 : t.N_tau;
    const uint32_t n_chunks = (t.N_tau + kPostCols - 1u) / kPostCols;
    double best = -1.0;
    int64_t bidx = INT64_MAX;
    for (uint32_t k = lane; k < N; k += 32u) {
      double x;
      if (pass == 0) {
        x = 0.0;
        for (uint32_t c = 0; c < n_chunks; c++) x += (double)rowpart[t.row_off + (size_t)c * N + k];
      } else {
        x = colsum[t.col_off + k];
      }
      if (x > best) {  // k increases within a lane: keeps the first
        best = x;
        bidx = k;
      }
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
      const double ob = __shfl_xor_sync(0xffffffffu, best, d);
      const int64_t oi = __shfl_xor_sync(0xffffffffu, bidx, d);
      if (ob > best || (ob == best && oi < bidx)) {
        best = ob;
        bidx = oi;
      }
    }
    out[pass] = bidx == INT64_MAX ? -1 : bidx;
  }
  if (lane == 0) {
    results[tmpl].t0_mp_idx = out[0];
    results[tmpl].tau_mp_idx = out[1];
  }
}

cudaError_t launch_plan_posteriors(const TemplateDev *d_T, uint32_t n_templates,
                                   const uint2 *d_chunks, uint32_t n_chunks, const float *d_maps,
                                   tcw_result *d_results, float *d_rowpart, double *d_colsum,
                                   cudaStream_t stream) {
  if (n_chunks) {
    post_sums_kernel<<<n_chunks, kPostThreads, 0, stream>>>(d_T, d_chunks, d_maps, d_results,
                                                            d_rowpart, d_colsum);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  post_argmax_kernel<<<(n_templates + 3u) / 4u, 128, 0, stream>>>(d_T, n_templates, d_rowpart,
                                                                  d_colsum, d_results);
  return cudaGetLastError();
}

cudaError_t launch_posteriors(const TemplateDev *d_T, const float *d_Fmn, void *d_result,
                              double *d_rowsum, double *d_colsum, uint32_t N_t0,
                              uint32_t N_tau, cudaStream_t stream) {
  (void)d_T;
  tcw_result *res = reinterpret_cast<tcw_result *>(d_result);
  rowsum_kernel<<<N_t0, 256, 0, stream>>>(d_Fmn, res, N_tau, d_rowsum);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const uint32_t n_chunks = (N_t0 + kColChunk - 1u) / kColChunk;
  dim3 grid((N_tau + 127u) / 128u, n_chunks);
  colsum_kernel<<<grid, 128, 0, stream>>>(d_Fmn, res, N_t0, N_tau, d_colsum);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  posterior_argmax_kernel<<<1, 1024, 0, stream>>>(d_rowsum, d_colsum, N_t0, N_tau, n_chunks,
                                                  res);
  return cudaGetLastError();
}

}  // namespace tcw

namespace tcw {
// Failed debug checks of this file's kernels (0 unless built with TCW_DEBUG_CHECKS).
unsigned int dcheck_failures_kernels() {
#if defined(TCW_DEBUG_CHECKS)
  return tcw_dcheck_read();
#else
  return 0;
#endif
}
}  // namespace tcw
