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

// comp = 1: the packed column the GPU runs (atoms in rows of 8);
// comp = 0: the uncompensated FP32 variant.
int hc_exp_map(const float *atoms, uint32_t n, uint32_t TAtom, uint32_t t0_data,
               const uint32_t *t0s, uint32_t N_t0, const uint32_t *taus, uint32_t N_tau,
               int comp, uint32_t row_chunk, float *F, uint8_t *okmap) {
  Geom g = make_geom(n, TAtom, t0_data);
  if (row_chunk == 0) row_chunk = N_t0;
  float *a8 = (float *)calloc((size_t)n * 8u, sizeof(float));
  if (!a8) return -1;
  for (uint32_t i = 0; i < n; i++)
    for (int c = 0; c < 7; c++) a8[(size_t)i * 8u + kRow8Slot[c]] = atoms[(size_t)i * 7u + c];
  for (uint32_t k = 0; k < N_tau; k++) {
    for (uint32_t mb = 0; mb < N_t0; mb += row_chunk) {
      uint32_t me = mb + row_chunk < N_t0 ? mb + row_chunk : N_t0;
      HostSink s{F + k, okmap ? okmap + k : nullptr, N_tau};
      if (comp)
        exp_column2<false>(a8, g, t0s, mb, me, taus[k], s);
      else
        exp_column<false, false>(atoms, g, t0s, mb, me, taus[k], s);
    }
  }
  free(a8);
  return 0;
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

}  // extern "C"
