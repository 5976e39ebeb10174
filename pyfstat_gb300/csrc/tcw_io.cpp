// Host-side file formats of the transient-map path: text maps in the
// lalpulsar write_transientFstatMap_to_fp layout (lines of "t0 tau 2F"),
// lalpulsar F-statistic atom text files, both written and parsed in native
// code (a year-long 8192 x 4096 map is 3.4e7 lines).
//
// Text map body line (pyfstat/tcw_fstat_map_funcs.py:314-317):
//   "  %10d %10d %- 11.8g\n" % (t0, tau, 2F)
// Map reader semantics (tcw_fstat_map_funcs.py:159-184): '#' lines are
// comments, columns are t0, tau, 2F.
// Atoms text (lalpulsar write_MultiFstatAtoms_to_fp, read back by
// pyfstat/utils/io.py:58-95 with comments "%%", columns checked by
// tests/test_core.py:811-826): '%' lines are comments, the data columns are
// tGPS a2 b2 ab Fa_re Fa_im Fb_re Fb_im.

#include <cerrno>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/tcw_b200.h"

namespace {

bool read_file(const char *path, std::vector<char> &buf) {
  FILE *f = std::fopen(path, "rb");
  if (!f) return false;
  buf.clear();
  char chunk[1 << 16];
  size_t n;
  while ((n = std::fread(chunk, 1, sizeof(chunk), f)) > 0) buf.insert(buf.end(), chunk, chunk + n);
  const bool ok = !std::ferror(f);
  std::fclose(f);
  buf.push_back('\0');
  return ok;
}

// Calls fn(line_begin, line_end) for each line that is not blank and does not
// start (after leading blanks) with the comment character.
template <class Fn>
int for_data_lines(const std::vector<char> &buf, char comment, Fn fn) {
  const char *p = buf.data();
  const char *end = p + buf.size() - 1;
  while (p < end) {
    const char *e = static_cast<const char *>(std::memchr(p, '\n', (size_t)(end - p)));
    if (!e) e = end;
    const char *q = p;
    while (q < e && (*q == ' ' || *q == '\t' || *q == '\r')) q++;
    if (q < e && *q != comment) {
      const int rc = fn(q, e);
      if (rc) return rc;
    }
    p = e + 1;
  }
  return 0;
}

// Parses `n` numbers from [p, e) into out; returns false on a short or bad line.
bool parse_numbers(const char *p, const char *e, int n, double *out) {
  for (int k = 0; k < n; k++) {
    while (p < e && (*p == ' ' || *p == '\t' || *p == '\r')) p++;
    if (p >= e) return false;
    char *next = nullptr;
    errno = 0;
    out[k] = std::strtod(p, &next);
    if (next == p || next > e) return false;
    p = next;
  }
  return true;
}

}  // namespace

extern "C" {

int tcw_write_map_text(const char *path, const float *F, uint32_t N_t0, uint32_t N_tau,
                       const uint32_t *t0s, const uint32_t *taus, int append) {
  if (!path || !F || !t0s || !taus) return TCW_ERR_INVALID_ARG;
  FILE *f = std::fopen(path, append ? "ab" : "wb");
  if (!f) return TCW_ERR_IO;
  static thread_local char line[96];
  std::vector<char> out;
  out.reserve(1 << 20);
  for (uint32_t m = 0; m < N_t0; m++) {
    for (uint32_t n = 0; n < N_tau; n++) {
      const double twoF = 2.0 * (double)F[(size_t)m * N_tau + n];
      // %10u prints a u32 as Python's %10d prints the same non-negative integer
      const int k = std::snprintf(line, sizeof(line), "  %10u %10u %- 11.8g\n", t0s[m], taus[n],
                                  twoF);
      out.insert(out.end(), line, line + k);
      if (out.size() > (1u << 20) - sizeof(line)) {
        if (std::fwrite(out.data(), 1, out.size(), f) != out.size()) {
          std::fclose(f);
          return TCW_ERR_IO;
        }
        out.clear();
      }
    }
  }
  const bool ok = std::fwrite(out.data(), 1, out.size(), f) == out.size();
  return (std::fclose(f) == 0 && ok) ? TCW_OK : TCW_ERR_IO;
}

int tcw_read_map_text(const char *path, uint64_t *n_lines, double *t0, double *tau, double *twoF,
                      uint64_t capacity) {
  if (!path || !n_lines) return TCW_ERR_INVALID_ARG;
  std::vector<char> buf;
  if (!read_file(path, buf)) return TCW_ERR_IO;
  uint64_t k = 0;
  const bool fill = t0 && tau && twoF;
  const int rc = for_data_lines(buf, '#', [&](const char *p, const char *e) {
    double v[3];
    if (!parse_numbers(p, e, 3, v)) return TCW_ERR_FORMAT;
    if (fill) {
      if (k >= capacity) return TCW_ERR_OVERFLOW;
      t0[k] = v[0];
      tau[k] = v[1];
      twoF[k] = v[2];
    }
    k++;
    return 0;
  });
  *n_lines = k;
  return rc;
}

int tcw_read_atoms_text(const char *path, uint64_t *n_rows, uint32_t *timestamps, float *atoms7,
                        uint64_t capacity) {
  if (!path || !n_rows) return TCW_ERR_INVALID_ARG;
  std::vector<char> buf;
  if (!read_file(path, buf)) return TCW_ERR_IO;
  uint64_t k = 0;
  const bool fill = timestamps && atoms7;
  const int rc = for_data_lines(buf, '%', [&](const char *p, const char *e) {
    double v[8];
    if (!parse_numbers(p, e, 8, v)) return TCW_ERR_FORMAT;
    if (fill) {
      if (k >= capacity) return TCW_ERR_OVERFLOW;
      if (!(v[0] >= 0.0 && v[0] <= 4294967295.0)) return TCW_ERR_FORMAT;
      timestamps[k] = (uint32_t)v[0];
      for (int c = 0; c < 7; c++) atoms7[k * 7u + c] = (float)v[1 + c];
    }
    k++;
    return 0;
  });
  *n_rows = k;
  return rc;
}

int tcw_write_atoms_text(const char *path, const uint32_t *timestamps, const float *atoms7,
                         uint64_t n_rows, int append) {
  if (!path || (n_rows && (!timestamps || !atoms7))) return TCW_ERR_INVALID_ARG;
  FILE *f = std::fopen(path, append ? "ab" : "wb");
  if (!f) return TCW_ERR_IO;
  bool ok = std::fputs("%% tGPS a2 b2 ab Fa_re Fa_im Fb_re Fb_im\n", f) >= 0;
  for (uint64_t k = 0; ok && k < n_rows; k++) {
    const float *x = atoms7 + k * 7u;
    ok = std::fprintf(f, "%10u %.9g %.9g %.9g %.9g %.9g %.9g %.9g\n", timestamps[k], x[0], x[1],
                      x[2], x[3], x[4], x[5], x[6]) > 0;
  }
  return (std::fclose(f) == 0 && ok) ? TCW_OK : TCW_ERR_IO;
}

}  // extern "C"
