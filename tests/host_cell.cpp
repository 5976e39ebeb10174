// Host build of the device cell arithmetic (pyfstat_gb300/csrc/tcw_cell.h),
// used only by the CPU test-suite to check the GPU algorithm -- compensated
// prefix sums, quantised prefix rows, the two-pointer exponential recurrence,
// the u32 division -- against the FP64 oracle without a GPU.  Sequential scan
// order here; the CUDA prefix kernel scans in chunks, with the same error bound.
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../pyfstat_gb300/csrc/tcw_cell.h"

using namespace tcw;

extern "C" {

// Exclusive prefix rows (numAtoms + 1) x 16 floats.
void hc_prefix(const float *atoms, uint32_t n, int comp, float *P) {
  float Q[7], invQ[7];
  for (int c = 0; c < 7; c++) {
    float s = 0.0f;
    for (uint32_t i = 0; i < n; i++) s += fabsf(atoms[(size_t)i * 7 + c]);
    Q[c] = prefix_quantum(s);
    invQ[c] = 1.0f / Q[c];
  }
  FF acc[7];
  for (int c = 0; c < 7; c++) acc[c] = ff_zero();
  for (uint32_t j = 0; j <= n; j++) {
    float *row = P + (size_t)j * kPrefixStride;
    for (int c = 0; c < 7; c++) {
      if (comp) {
        quantise_prefix(acc[c].h, acc[c].l, Q[c], invQ[c], row[c], row[8 + c]);
      } else {
        row[c] = acc[c].h;
        row[8 + c] = 0.0f;
      }
    }
    row[7] = row[15] = 0.0f;
    if (j < n) {
      for (int c = 0; c < 7; c++) {
        float x = atoms[(size_t)j * 7 + c];
        if (comp)
          acc[c] = ff_add1(acc[c], x);
        else
          acc[c].h = acc[c].h + x;
      }
    }
  }
}

int hc_rect_map(const float *atoms, uint32_t n, uint32_t TAtom, uint32_t t0_data,
                const uint32_t *t0s, uint32_t N_t0, const uint32_t *taus, uint32_t N_tau,
                int comp, float *F, uint8_t *okmap) {
  Geom g = make_geom(n, TAtom, t0_data);
  float *P = (float *)malloc(sizeof(float) * (size_t)(n + 1) * kPrefixStride);
  if (!P) return -1;
  hc_prefix(atoms, n, comp, P);
  for (uint32_t m = 0; m < N_t0; m++) {
    uint32_t t0 = t0s[m];
    uint32_t j0 = idx_start(t0, g);
    bool wr = rect_row_wrapped(t0, taus[0], g);
    uint32_t end_first = idx_end(t0 + taus[0], g);
    const float *P0 = P + (size_t)j0 * kPrefixStride;
    for (uint32_t k = 0; k < N_tau; k++) {
      uint32_t e = rect_end(t0, taus[k], end_first, wr, g);
      bool ok;
      float v = comp ? rect_cell<true, false>(P, P0, j0, e, ok)
                     : rect_cell<false, false>(P, P0, j0, e, ok);
      F[(size_t)m * N_tau + k] = v;
      if (okmap) okmap[(size_t)m * N_tau + k] = ok;
    }
  }
  free(P);
  return 0;
}

struct HostSink {
  float *col;
  uint8_t *ok;
  uint32_t stride;
  void operator()(uint32_t m, float F, bool k) {
    col[(size_t)m * stride] = F;
    if (ok) ok[(size_t)m * stride] = k;
  }
};

}  // extern "C"

// The map kernels' row-table walk of one column chunk (exp_rows): row tables
// of 128 rows, each taking the clamped-window-end rows (row_clamped, and
// row_steady after the first window with an atom when the window starts never
// grow) when the window end is clamped at numAtoms for the table's smallest
// t0.
template <class Sink>
static void exp_rows_host(const float *a8, const Geom &g, const uint32_t *t0s, uint32_t mb,
                          uint32_t me, uint32_t tau, Sink &s) {
  ExpColumn<false, true> C;
  C.init(g, tau);
  auto row_of = [&](uint32_t t0) {
    ExpRow e;
    e.lo = exp_lo(t0, g);
    e.nz = 0xFFFFFFFFu;
    if (e.lo < g.numAtoms) memcpy(&e.nz, &a8[(size_t)e.lo * 8u + 3u], sizeof(e.nz));
    const uint32_t d = t0 - g.t0_data;
    e.a = fdiv(d, g.div);
    e.b = d - e.a * g.TAtom;
    return e;
  };
  for (uint32_t ce = me; ce > mb;) {
    const uint32_t cb = ce - mb > 128u ? ce - 128u : mb;
    uint32_t t0min = 0xFFFFFFFFu;
    for (uint32_t m = cb; m < ce; m++) t0min = t0s[m] < t0min ? t0s[m] : t0min;
    const bool clamped = C.top_raw(row_of(t0min)) >= g.numAtoms;
    bool mono = true;
    for (uint32_t m = cb; m + 1u < ce; m++) mono = mono && row_of(t0s[m]).lo <= row_of(t0s[m + 1u]).lo;
    if (clamped && mono) {
      uint32_t m = ce;
      while (m > cb) {
        m--;
        const ExpRow e = row_of(t0s[m]);
        C.row_clamped(a8, g, e, m, s);
        if (e.lo < g.numAtoms) break;
      }
      while (m > cb) {
        m--;
        const ExpRow e = row_of(t0s[m]);
        C.row_steady(a8, g, e, m, s);
        if (e.nz < g.numAtoms) break;
      }
      while (m > cb) {
        m--;
        C.row_steady_data(a8, g, row_of(t0s[m]), m, s);
      }
    } else {
      for (uint32_t m = ce; m-- > cb;) {
        if (clamped)
          C.row_clamped(a8, g, row_of(t0s[m]), m, s);
        else
          C.row(a8, g, row_of(t0s[m]), m, s);
      }
    }
    ce = cb;
  }
}

extern "C" {

// comp = 1: what the GPU runs -- atoms in rows of 8 with the first-non-zero
//           index in slot 3 (as the repack kernel writes them), each row
//           chunk through the row-table column (ExpColumn) when all its rows
//           are regular for the column's tau, else through exp_column2;
// comp = 2: exp_column2 only (the generic index arithmetic);
// comp = 0: the uncompensated FP32 variant.
int hc_exp_map(const float *atoms, uint32_t n, uint32_t TAtom, uint32_t t0_data,
               const uint32_t *t0s, uint32_t N_t0, const uint32_t *taus, uint32_t N_tau,
               int comp, uint32_t row_chunk, float *F, uint8_t *okmap) {
  Geom g = make_geom(n, TAtom, t0_data);
  if (row_chunk == 0) row_chunk = N_t0;
  float *a8 = (float *)calloc((size_t)n * 8u, sizeof(float));
  if (!a8) return -1;
  uint32_t nz = 0xFFFFFFFFu;
  for (uint32_t i = n; i-- > 0;) {
    for (int c = 0; c < 7; c++) a8[(size_t)i * 8u + kRow8Slot[c]] = atoms[(size_t)i * 7u + c];
    if (atoms[(size_t)i * 7u] != 0.0f || atoms[(size_t)i * 7u + 1u] != 0.0f) nz = i;
    memcpy(&a8[(size_t)i * 8u + 3u], &nz, sizeof(nz));
  }
  for (uint32_t k = 0; k < N_tau; k++) {
    for (uint32_t mb = 0; mb < N_t0; mb += row_chunk) {
      uint32_t me = mb + row_chunk < N_t0 ? mb + row_chunk : N_t0;
      HostSink s{F + k, okmap ? okmap + k : nullptr, N_tau};
      bool reg = comp == 1;
      for (uint32_t m = mb; reg && m < me; m++) reg = exp_row_regular(t0s[m], taus[k], g);
      if (reg) {
        exp_rows_host(a8, g, t0s, mb, me, taus[k], s);
      } else if (comp) {
        exp_column2<false>(a8, g, t0s, mb, me, taus[k], s);
      } else {
        exp_column<false, false>(atoms, g, t0s, mb, me, taus[k], s);
      }
    }
  }
  free(a8);
  return 0;
}

// Window sums of exponential windows on a real tau grid (the differentiable
// statistics' forward pass): the double-word sums of ExpColumn (init_real,
// row tables) as FP64 values, W[(m * N_tau + n) * 7 + c], and whether the
// window holds data.  Rows must be regular for every tau (t0 >= t0_data).
int hc_exp_real_sums(const float *atoms, uint32_t n, uint32_t TAtom, uint32_t t0_data,
                     const uint32_t *t0s, uint32_t N_t0, const double *taus, uint32_t N_tau,
                     double *W, uint8_t *valid) {
  Geom g = make_geom(n, TAtom, t0_data);
  float *a8 = (float *)calloc((size_t)n * 8u, sizeof(float));
  if (!a8) return -1;
  uint32_t nz = 0xFFFFFFFFu;
  for (uint32_t i = n; i-- > 0;) {
    for (int c = 0; c < 7; c++) a8[(size_t)i * 8u + kRow8Slot[c]] = atoms[(size_t)i * 7u + c];
    if (atoms[(size_t)i * 7u] != 0.0f || atoms[(size_t)i * 7u + 1u] != 0.0f) nz = i;
    memcpy(&a8[(size_t)i * 8u + 3u], &nz, sizeof(nz));
  }
  for (uint32_t k = 0; k < N_tau; k++) {
    ExpColumn<false> C;
    C.init_real(g, taus[k]);
    for (uint32_t m = N_t0; m-- > 0;) {
      ExpRow e;
      e.lo = exp_lo(t0s[m], g);
      e.nz = 0xFFFFFFFFu;
      if (e.lo < n) memcpy(&e.nz, &a8[(size_t)e.lo * 8u + 3u], sizeof(e.nz));
      const uint32_t d = t0s[m] - t0_data;
      e.a = fdiv(d, g.div);
      e.b = d - e.a * TAtom;
      const bool ok = C.window(a8, g, e);
      double *w = W + ((size_t)m * N_tau + k) * 7u;
      w[0] = (double)C.W0.h.x + (double)C.W0.l.x;
      w[1] = (double)C.W0.h.y + (double)C.W0.l.y;
      w[2] = (double)C.Wc.h + (double)C.Wc.l;
      w[3] = (double)C.W2.h.x + (double)C.W2.l.x;
      w[4] = (double)C.W2.h.y + (double)C.W2.l.y;
      w[5] = (double)C.W3.h.x + (double)C.W3.l.x;
      w[6] = (double)C.W3.h.y + (double)C.W3.l.y;
      valid[(size_t)m * N_tau + k] = ok;
    }
  }
  free(a8);
  return 0;
}

// The error-free sum forms of the exponential columns' entering step, for
// n cases (x, E = Eh + El, r = rh + rl): out[i * 8 + ...] =
//   0-1 ff_axpy (TwoSum), 2-3 ff_axpy_ord, 4-5 ff2_axpy_nonneg (lane 0),
//   6-7 ff2_axpy_fast (lane 0); each as (hi, lo).
void hc_sum_forms(const float *x, const float *Eh, const float *El, const float *rh,
                  const float *rl, uint64_t n, float *out) {
  for (uint64_t i = 0; i < n; i++) {
    const FF r{rh[i], rl[i]}, E{Eh[i], El[i]};
    const FF a = ff_axpy(x[i], r, E), b = ff_axpy_ord(x[i], r, E);
    const F2 X{x[i], x[i]}, RH{rh[i], rh[i]}, NRH{-rh[i], -rh[i]}, RL{rl[i], rl[i]};
    const FF2 E2{F2{Eh[i], Eh[i]}, F2{El[i], El[i]}};
    const FF2 c = ff2_axpy_nonneg(X, RH, NRH, RL, E2), d = ff2_axpy_fast(X, RH, NRH, RL, E2);
    float *o = out + i * 8u;
    o[0] = a.h; o[1] = a.l; o[2] = b.h; o[3] = b.l;
    o[4] = c.h.x; o[5] = c.l.x; o[6] = d.h.x; o[7] = d.l.x;
  }
}

void hc_fastdiv(uint32_t d, const uint32_t *x, uint64_t n, uint32_t *q) {
  FastDiv f = make_fastdiv(d);
  for (uint64_t i = 0; i < n; i++) q[i] = fdiv(x[i], f);
}

void hc_exp_window(uint32_t n, uint32_t TAtom, uint32_t t0_data, const uint32_t *t0s,
                   const uint32_t *taus, uint64_t ncells, int32_t *lohi) {
  Geom g = make_geom(n, TAtom, t0_data);
  for (uint64_t k = 0; k < ncells; k++) {
    uint32_t lo, hi;
    if (exp_window(t0s[k], taus[k], g, lo, hi)) {
      lohi[2 * k] = (int32_t)lo;
      lohi[2 * k + 1] = (int32_t)hi;
    } else {
      lohi[2 * k] = 1;
      lohi[2 * k + 1] = 0;
    }
  }
}


// The rect map kernel's walk (rect_tile) restated on the host: 32-row groups,
// columns ascending in 32-column chunks; a column whose window end equals
// the previous column's takes the previous F, and a chunk inside every
// row's clamped run (the kernel's test over the group's rows) repeats it
// for all its columns.  Gives the F map only (comp = 1 arithmetic).
int hc_rect_walk_map(const float *atoms, uint32_t n, uint32_t TAtom, uint32_t t0_data,
                     const uint32_t *t0s, uint32_t N_t0, const uint32_t *taus, uint32_t N_tau,
                     float *F) {
  Geom g = make_geom(n, TAtom, t0_data);
  float *P = (float *)malloc(sizeof(float) * (size_t)(n + 1) * kPrefixStride);
  if (!P) return -1;
  hc_prefix(atoms, n, 1, P);
  for (uint32_t mg = 0; mg < N_t0; mg += 32u) {
    uint32_t t0[32], j0[32], ef[32], e_cur[32], e_prev[32];
    bool wr[32], ok_row[32];
    float F_prev[32];
    for (uint32_t l = 0; l < 32u; l++) {
      const uint32_t m = mg + l;
      ok_row[l] = m < N_t0;
      if (!ok_row[l]) continue;
      t0[l] = t0s[m];
      j0[l] = idx_start(t0[l], g);
      wr[l] = rect_row_wrapped(t0[l], taus[0], g);
      ef[l] = idx_end(t0[l] + taus[0], g);
      e_cur[l] = rect_end(t0[l], taus[0], ef[l], wr[l], g);
      e_prev[l] = 0xFFFFFFFFu;
      F_prev[l] = 2.0f;
    }
    for (uint32_t cb = 0; cb < N_tau; cb += 32u) {
      const uint32_t ce = cb + 32u < N_tau ? cb + 32u : N_tau;
      bool mono = true;
      for (uint32_t k = cb; k + 1u < ce; k++) mono = mono && taus[k] <= taus[k + 1u];
      if (ce < N_tau) mono = mono && taus[ce - 1u] <= taus[ce];
      const uint32_t tmax = ce < N_tau ? taus[ce] : taus[ce - 1u];
      bool run = mono;
      for (uint32_t l = 0; l < 32u && run; l++) {
        if (!ok_row[l]) continue;
        run = g.TAtom >= 2u && e_cur[l] == g.numAtoms - 1u && e_prev[l] == g.numAtoms - 1u &&
              (uint64_t)t0[l] + taus[cb] + g.half >= (uint64_t)g.t0_data &&
              (uint64_t)t0[l] + tmax + g.half - g.t0_data <= 0xFFFFFFFFull &&
              (uint64_t)t0[l] + tmax <= 0xFFFFFFFFull;
      }
      uint32_t nc = cb;
      if (run) {
        for (; nc < ce; nc++)
          for (uint32_t l = 0; l < 32u; l++)
            if (ok_row[l]) F[(size_t)(mg + l) * N_tau + nc] = F_prev[l];
        for (uint32_t l = 0; l < 32u; l++) e_cur[l] = g.numAtoms - 1u;
      }
      for (; nc < ce; nc++) {
        for (uint32_t l = 0; l < 32u; l++) {
          if (!ok_row[l]) continue;
          const uint32_t ea = e_cur[l];
          uint32_t eb = 0;
          if (nc + 1u < N_tau) eb = rect_end(t0[l], taus[nc + 1u], ef[l], wr[l], g);
          float Fv = F_prev[l];
          if (ea != e_prev[l]) {
            bool ok;
            Fv = rect_cell<true, false>(P, P + (size_t)j0[l] * kPrefixStride, j0[l], ea, ok);
          }
          F[(size_t)(mg + l) * N_tau + nc] = Fv;
          e_prev[l] = ea;
          F_prev[l] = Fv;
          e_cur[l] = eb;
        }
      }
    }
  }
  free(P);
  return 0;
}
}  // extern "C"
