// C-ABI layer of the GB300 transient-CW F-statistic map (include/tcw_b200.h).
//
// Host-side responsibilities: argument validation (with the reference's
// u32 time conventions), tiling of maps into work items, workspace
// management, stream ordering, CUDA-graph capture of batched runs, and
// status codes instead of exceptions.  All compute is in tcw_kernels.cu.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <thread>
#include <vector>

#include "../../include/tcw_b200.h"
#include "tcw_internal.h"

using namespace tcw;

struct tcw_handle {
  int device = 0;
  int n_sms = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  cudaStream_t side_stream = nullptr;  // second branch of batched runs
  cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
  // pipelined host-buffer runs: uploads on their own stream, ordered after
  // the previous run's prefix/repack kernels (the readers of the atoms)
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t consumed_ev = nullptr, consumed_side_ev = nullptr, copied_ev = nullptr;
  bool consumed_pending = false;
  int prio_high = 0, prio_low = 0;
  char *d_ws = nullptr;
  size_t ws_cap = 0;
  char *h_stage = nullptr;
  size_t stage_cap = 0;
  cudaEvent_t stage_ev = nullptr;
  bool stage_pending = false;
  int fail_alloc_countdown = 0;
  tcw_tile_config plain_cfg{};
  char err[512] = {0};
};

struct tcw_plan {
  int device = 0;
  int prec = kPrecFF;
  int flags = 0;
  uint32_t n_templates = 0, n_items = 0, n_rect = 0;
  uint32_t n_items_rect = 0, n_items_exp = 0, n_blocks_rect = 0, n_blocks_exp = 0;
  uint64_t n_cells = 0, n_atom_rows = 0, p_rows = 0;
  tcw_tile_config cfg{};
  char *d_buf = nullptr;  // one allocation for all plan-owned device arrays
  TemplateDev *d_T = nullptr;
  WorkItem *d_items = nullptr;
  Partial *d_parts = nullptr;
  uint32_t *d_rect_list = nullptr, *d_exp_list = nullptr, *d_t0s = nullptr, *d_taus = nullptr;
  uint32_t n_exp = 0;
  float *d_A8 = nullptr;  // exp templates' atoms in rows of 8 floats
  uint32_t *d_counter = nullptr;  // [0] rect tiles, [1] exp tiles
  float *d_P = nullptr;
  // graph state
  cudaGraphExec_t gexec = nullptr;
  const float *g_atoms = nullptr;
  tcw_result *g_results = nullptr;
  float *g_maps = nullptr;
  cudaStream_t g_stream = nullptr;
  // buffers of the host-buffer entry point
  float *d_atoms_in = nullptr;
  tcw_result *d_res_out = nullptr;
  float *d_maps_out = nullptr;  // maps of tcw_plan_run_maps_host (n_cells floats)
  // posterior plans: column chunks and the row / column sums
  uint2 *d_post_chunks = nullptr;
  uint32_t n_post_chunks = 0;
  float *d_rowpart = nullptr;
  double *d_colsum = nullptr;
};

namespace {

int set_err(tcw_handle *h, int code, const char *fmt, ...) {
  if (h) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(h->err, sizeof(h->err), fmt, ap);
    va_end(ap);
  }
  return code;
}

int cuda_err(tcw_handle *h, cudaError_t e, const char *what) {
  return set_err(h, TCW_ERR_CUDA, "%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
}

#define TCW_CUDA(h, call)                          \
  do {                                             \
    cudaError_t _e = (call);                       \
    if (_e != cudaSuccess) return cuda_err(h, _e, #call); \
  } while (0)

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

int ws_alloc(tcw_handle *h, void **p, size_t bytes) {
  if (h->fail_alloc_countdown > 0 && --h->fail_alloc_countdown == 0)
    return set_err(h, TCW_ERR_ALLOC, "workspace allocation of %zu bytes failed (test hook)",
                   bytes);
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_err(h, TCW_ERR_ALLOC, "cudaMalloc(%zu) failed: %s", bytes, cudaGetErrorString(e));
  }
  return TCW_OK;
}

// Grow-only device workspace.  Growing waits for the handle's stream so that
// no queued kernel still uses the old buffer.
int ensure_ws(tcw_handle *h, size_t bytes) {
  if (bytes <= h->ws_cap) return TCW_OK;
  TCW_CUDA(h, cudaStreamSynchronize(h->stream));
  if (h->d_ws) cudaFree(h->d_ws);
  h->d_ws = nullptr;
  h->ws_cap = 0;
  size_t cap = align_up(bytes + bytes / 4, 1 << 20);
  void *p = nullptr;
  int rc = ws_alloc(h, &p, cap);
  if (rc) return rc;
  h->d_ws = static_cast<char *>(p);
  h->ws_cap = cap;
  return TCW_OK;
}

// Pinned host staging for small control data (descriptors, tile lists).
int ensure_stage(tcw_handle *h, size_t bytes) {
  if (h->stage_pending) {
    TCW_CUDA(h, cudaEventSynchronize(h->stage_ev));
    h->stage_pending = false;
  }
  if (bytes <= h->stage_cap) return TCW_OK;
  if (h->h_stage) cudaFreeHost(h->h_stage);
  h->h_stage = nullptr;
  h->stage_cap = 0;
  size_t cap = align_up(bytes + bytes / 4, 1 << 16);
  void *p = nullptr;
  cudaError_t e = cudaMallocHost(&p, cap);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_err(h, TCW_ERR_ALLOC, "cudaMallocHost(%zu) failed", cap);
  }
  h->h_stage = static_cast<char *>(p);
  h->stage_cap = cap;
  return TCW_OK;
}

struct Layout {
  size_t total = 0;
  size_t add(size_t bytes) {
    size_t off = total;
    total = align_up(total + bytes, 256);
    return off;
  }
};

bool valid_window(int w) { return w == TCW_WINDOW_RECT || w == TCW_WINDOW_EXP; }

int check_geometry(tcw_handle *h, uint32_t numAtoms, uint32_t TAtom, uint32_t t0_data,
                   uint32_t N_t0, uint32_t N_tau) {
  if (numAtoms == 0) return set_err(h, TCW_ERR_INVALID_ARG, "numAtoms must be >= 1");
  if (TAtom == 0) return set_err(h, TCW_ERR_INVALID_ARG, "TAtom must be >= 1");
  if (N_t0 == 0 || N_tau == 0)
    return set_err(h, TCW_ERR_INVALID_ARG, "empty grid: N_t0=%u N_tau=%u", N_t0, N_tau);
  if ((uint64_t)t0_data + (uint64_t)numAtoms * TAtom > 0xFFFFFFFFull)
    return set_err(h, TCW_ERR_OVERFLOW,
                   "atom timestamps t0_data + i*TAtom exceed the u32 range (t0_data=%u, "
                   "numAtoms=%u, TAtom=%u)",
                   t0_data, numAtoms, TAtom);
  if ((uint64_t)N_t0 * (uint64_t)N_tau > (1ull << 62))
    return set_err(h, TCW_ERR_OVERFLOW, "N_t0*N_tau overflows");
  return TCW_OK;
}

// Host-side grid checks (only where the grids are host memory).
int check_grids(tcw_handle *h, int window, const uint32_t *t0s, uint32_t N_t0,
                const uint32_t *taus, uint32_t N_tau) {
  uint32_t t0max = 0, taumax = 0;
  for (uint32_t m = 0; m < N_t0; m++) t0max = std::max(t0max, t0s[m]);
  for (uint32_t n = 0; n < N_tau; n++) {
    taumax = std::max(taumax, taus[n]);
    if (taus[n] == 0 && window == TCW_WINDOW_EXP)
      return set_err(h, TCW_ERR_INVALID_ARG, "exponential window needs tau > 0 (taus[%u]=0)", n);
    if (window == TCW_WINDOW_RECT && n > 0 && taus[n] < taus[n - 1])
      return set_err(h, TCW_ERR_INVALID_ARG,
                     "rectangular window needs a non-decreasing tau grid (taus[%u] < taus[%u])",
                     n, n - 1);
  }
  uint64_t reach = (uint64_t)t0max + (uint64_t)taumax * (window == TCW_WINDOW_EXP ? 3u : 1u);
  if (reach > 0xFFFFFFFFull)
    return set_err(h, TCW_ERR_OVERFLOW, "t0 + %stau exceeds the u32 time range",
                   window == TCW_WINDOW_EXP ? "3*" : "");
  return TCW_OK;
}

int prec_of(int flags) {
  if (flags & TCW_FLAG_UNCOMPENSATED) return kPrecPlain32;
  if (flags & TCW_FLAG_FP64_DET) return kPrecFF_F64Det;
  return kPrecFF;
}

// Tiles of one template.  Rect: tn columns x tm rows per block.  Exp: tn
// columns per block, each thread one column over `rows` rows, the block's
// 128/tn thread rows covering consecutive row chunks; with `warp_tiles`
// (persistent plans, whose exp kernel schedules by warp) 32 columns over
// `rows` rows per tile.
void tile_template(uint32_t tmpl, const TemplateDev &t, const tcw_tile_config &cfg,
                   std::vector<WorkItem> &items, std::vector<double> *cost,
                   bool warp_tiles = false) {
  const uint32_t N_t0 = t.N_t0, N_tau = t.N_tau;
  if (t.window == TCW_WINDOW_RECT) {
    const uint32_t tn = cfg.rect_tn, tm = cfg.rect_tm;
    for (uint32_t n0 = 0; n0 < N_tau; n0 += tn)
      for (uint32_t m0 = 0; m0 < N_t0; m0 += tm) {
        WorkItem w{};
        w.tmpl = tmpl;
        w.m0 = m0;
        w.m1 = std::min(N_t0, m0 + tm);
        w.n0 = n0;
        w.n1 = std::min(N_tau, n0 + tn);
        w.tn = (uint16_t)(tm / 32u);  // row groups of 32 rows (one per warp)
        w.rows_per_lane = 0;
        items.push_back(w);
        if (cost) cost->push_back((double)(w.m1 - w.m0) * (w.n1 - w.n0));
      }
  } else {
    const uint32_t tn = warp_tiles ? 32u : cfg.exp_tn, lanes = warp_tiles ? 1u : kBlock / tn;
    uint32_t rows = cfg.exp_rows ? cfg.exp_rows : N_t0;
    // a lane's row chunk is a 16-bit count: longer columns become several tiles
    rows = std::min(std::min(rows, N_t0), 65535u);
    const uint32_t span = rows * lanes;  // rows per block
    for (uint32_t n0 = 0; n0 < N_tau; n0 += tn)
      for (uint32_t m0 = 0; m0 < N_t0; m0 += span) {
        WorkItem w{};
        w.tmpl = tmpl;
        w.m0 = m0;
        w.m1 = std::min(N_t0, m0 + span);
        w.n0 = n0;
        w.n1 = std::min(N_tau, n0 + tn);
        w.tn = (uint16_t)tn;
        w.rows_per_lane = (uint16_t)rows;
        items.push_back(w);
        if (cost) {
          // recurrence steps: window warm-up plus the rows' atom span, per column
          double atoms_per_row = 1.0;
          if (N_t0 > 1) atoms_per_row = std::max(1.0, (double)t.g.numAtoms / N_t0);
          double rows_here = (double)(w.m1 - w.m0);
          double warm = std::min((double)t.g.numAtoms, 3.0 * (double)N_tau) * lanes;
          cost->push_back(((rows_here * atoms_per_row * 2.0 + warm) * 2.0 + rows_here) *
                          (w.n1 - w.n0) / 1.0);
        }
      }
  }
}

void default_plain_cfg(const TemplateDev &t, tcw_tile_config &cfg, int n_sms) {
  const uint64_t target_blocks = (uint64_t)n_sms * 4u;
  if (t.window == TCW_WINDOW_RECT) {
    // 32-row tiles; columns per tile so that the grid has ~4 blocks per SM,
    // at least 4 columns per warp and at most 256
    cfg.rect_tm = 32;
    const uint64_t row_tiles = (t.N_t0 + 31u) / 32u;
    uint64_t tn = (uint64_t)t.N_tau * row_tiles / std::max<uint64_t>(1, target_blocks);
    tn = std::max<uint64_t>(16, std::min<uint64_t>(256, tn));
    cfg.rect_tn = (uint32_t)tn;
  } else {
    cfg.exp_tn = 32;
    // rows per thread: enough chunks for parallelism, long enough to amortise
    // each chunk's warm-up over the window
    uint32_t rows = std::max<uint32_t>(8, (t.N_t0 + 15) / 16);
    cfg.exp_rows = std::min(rows, t.N_t0);
  }
}

void fill_cfg_defaults(tcw_tile_config &c) {
  if (c.rect_tm != 32 && c.rect_tm != 64 && c.rect_tm != 128) c.rect_tm = 128;
  if (c.rect_tn == 0) c.rect_tn = 128;
  if (c.exp_tn != 32 && c.exp_tn != 64 && c.exp_tn != 128) c.exp_tn = 128;
  if (c.blocks_per_sm == 0) c.blocks_per_sm = 32;  // cap; occupancy decides below it
}

TemplateDev make_tdev(uint32_t numAtoms, uint32_t TAtom, uint32_t t0_data, int window,
                      uint32_t N_t0, uint32_t N_tau) {
  TemplateDev t{};
  t.g = make_geom(numAtoms, TAtom, t0_data);
  t.window = (uint32_t)window;
  t.N_t0 = N_t0;
  t.N_tau = N_tau;
  return t;
}

int set_device(tcw_handle *h) {
  TCW_CUDA(h, cudaSetDevice(h->device));
  return TCW_OK;
}

}  // namespace

// ====================================================================== ABI

extern "C" {

int tcw_abi_version(void) { return TCW_ABI_VERSION; }

const char *tcw_strerror(int status) {
  switch (status) {
    case TCW_OK: return "ok";
    case TCW_ERR_INVALID_ARG: return "invalid argument";
    case TCW_ERR_CUDA: return "CUDA error";
    case TCW_ERR_NO_DEVICE: return "no usable CUDA device";
    case TCW_ERR_ALLOC: return "allocation failed";
    case TCW_ERR_TIMEOUT: return "timed out waiting for the device";
    case TCW_ERR_UNSUPPORTED: return "unsupported";
    case TCW_ERR_OVERFLOW: return "size or time range overflow";
    case TCW_ERR_IO: return "file input/output error";
    case TCW_ERR_FORMAT: return "malformed line in a text file";
    default: return "unknown status";
  }
}

const char *tcw_last_error(const tcw_handle *h) { return h ? h->err : "null handle"; }

int tcw_device_count(int *count) {
  if (!count) return TCW_ERR_INVALID_ARG;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *count = 0;
    return TCW_ERR_NO_DEVICE;
  }
  *count = n;
  return TCW_OK;
}

int tcw_device_info(int device, char *name, size_t name_len, int *cc_major, int *cc_minor,
                    size_t *total_mem) {
  cudaDeviceProp prop;
  cudaError_t e = cudaGetDeviceProperties(&prop, device);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return TCW_ERR_NO_DEVICE;
  }
  if (name && name_len) {
    strncpy(name, prop.name, name_len - 1);
    name[name_len - 1] = 0;
  }
  if (cc_major) *cc_major = prop.major;
  if (cc_minor) *cc_minor = prop.minor;
  if (total_mem) *total_mem = prop.totalGlobalMem;
  return TCW_OK;
}

int tcw_device_memory(int device, size_t *free_bytes, size_t *total_bytes) {
  if (!free_bytes || !total_bytes) return TCW_ERR_INVALID_ARG;
  int prev = -1;
  if (cudaGetDevice(&prev) != cudaSuccess) {
    cudaGetLastError();
    return TCW_ERR_NO_DEVICE;
  }
  if (cudaSetDevice(device) != cudaSuccess) {
    cudaGetLastError();
    return TCW_ERR_NO_DEVICE;
  }
  size_t f = 0, t = 0;
  const cudaError_t e = cudaMemGetInfo(&f, &t);
  cudaSetDevice(prev);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return TCW_ERR_CUDA;
  }
  *free_bytes = f;
  *total_bytes = t;
  return TCW_OK;
}

int tcw_create(tcw_handle **out, int device) {
  if (!out) return TCW_ERR_INVALID_ARG;
  *out = nullptr;
  int n = 0;
  if (tcw_device_count(&n) != TCW_OK || n == 0) return TCW_ERR_NO_DEVICE;
  if (device < 0 || device >= n) return TCW_ERR_NO_DEVICE;
  tcw_handle *h = new (std::nothrow) tcw_handle();
  if (!h) return TCW_ERR_ALLOC;
  h->device = device;
  int rc = set_device(h);
  if (rc) {
    delete h;
    return rc;
  }
  cudaDeviceProp prop;
  // The kernels are built for sm_103a only: architecture-specific code that
  // loads on compute capability 10.3 and on no other device.
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess || prop.major != 10 ||
      prop.minor != 3) {
    cudaGetLastError();
    delete h;
    return TCW_ERR_NO_DEVICE;
  }
  h->n_sms = prop.multiProcessorCount;
  if (cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&h->stage_ev, cudaEventDisableTiming) != cudaSuccess) {
    cudaGetLastError();
    if (h->own_stream) cudaStreamDestroy(h->own_stream);
    delete h;
    return TCW_ERR_CUDA;
  }
  h->stream = h->own_stream;
  if (cudaDeviceGetStreamPriorityRange(&h->prio_low, &h->prio_high) != cudaSuccess ||
      cudaStreamCreateWithPriority(&h->side_stream, cudaStreamNonBlocking, h->prio_low) !=
          cudaSuccess ||
      cudaEventCreateWithFlags(&h->fork_ev, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&h->join_ev, cudaEventDisableTiming) != cudaSuccess ||
      cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&h->consumed_ev, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&h->consumed_side_ev, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&h->copied_ev, cudaEventDisableTiming) != cudaSuccess) {
    cudaGetLastError();
    tcw_destroy(h);
    return TCW_ERR_CUDA;
  }
  *out = h;
  return TCW_OK;
}

int tcw_destroy(tcw_handle *h) {
  if (!h) return TCW_ERR_INVALID_ARG;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  if (h->d_ws) cudaFree(h->d_ws);
  if (h->h_stage) cudaFreeHost(h->h_stage);
  if (h->stage_ev) cudaEventDestroy(h->stage_ev);
  if (h->side_stream) {
    cudaStreamSynchronize(h->side_stream);
    cudaStreamDestroy(h->side_stream);
  }
  if (h->fork_ev) cudaEventDestroy(h->fork_ev);
  if (h->join_ev) cudaEventDestroy(h->join_ev);
  if (h->copy_stream) {
    cudaStreamSynchronize(h->copy_stream);
    cudaStreamDestroy(h->copy_stream);
  }
  if (h->consumed_ev) cudaEventDestroy(h->consumed_ev);
  if (h->consumed_side_ev) cudaEventDestroy(h->consumed_side_ev);
  if (h->copied_ev) cudaEventDestroy(h->copied_ev);
  if (h->own_stream) cudaStreamDestroy(h->own_stream);
  cudaGetLastError();
  delete h;
  return TCW_OK;
}

int tcw_get_stream(tcw_handle *h, void **stream) {
  if (!h || !stream) return TCW_ERR_INVALID_ARG;
  *stream = (void *)h->stream;
  return TCW_OK;
}

int tcw_set_stream(tcw_handle *h, void *stream) {
  if (!h) return TCW_ERR_INVALID_ARG;
  h->stream = stream ? (cudaStream_t)stream : h->own_stream;
  return TCW_OK;
}

int tcw_sync(tcw_handle *h, int timeout_ms) {
  if (!h) return TCW_ERR_INVALID_ARG;
  int rc = set_device(h);
  if (rc) return rc;
  auto t0 = std::chrono::steady_clock::now();
  for (;;) {
    cudaError_t e = cudaStreamQuery(h->stream);
    if (e == cudaSuccess) return TCW_OK;
    if (e != cudaErrorNotReady) return cuda_err(h, e, "cudaStreamQuery");
    auto ms = std::chrono::duration_cast<std::chrono::milliseconds>(
                  std::chrono::steady_clock::now() - t0)
                  .count();
    if (timeout_ms >= 0 && ms >= timeout_ms)
      return set_err(h, TCW_ERR_TIMEOUT, "stream not done after %d ms", timeout_ms);
    std::this_thread::sleep_for(std::chrono::microseconds(50));
  }
}

int tcw_pinned_alloc(void **ptr, size_t bytes) {
  if (!ptr) return TCW_ERR_INVALID_ARG;
  *ptr = nullptr;
  if (cudaHostAlloc(ptr, std::max<size_t>(bytes, 16), cudaHostAllocDefault) != cudaSuccess) {
    cudaGetLastError();
    *ptr = nullptr;
    return TCW_ERR_ALLOC;
  }
  return TCW_OK;
}

int tcw_pinned_free(void *ptr) {
  if (!ptr) return TCW_OK;
  if (cudaFreeHost(ptr) != cudaSuccess) {
    cudaGetLastError();
    return TCW_ERR_CUDA;
  }
  return TCW_OK;
}

int tcw_debug_fail_alloc(tcw_handle *h, int n) {
  if (!h || n < 0) return TCW_ERR_INVALID_ARG;
  h->fail_alloc_countdown = n;
  return TCW_OK;
}

// ---------------------------------------------------------------- plain map

static int plain_enqueue(tcw_handle *h, const float *d_atoms, uint32_t numAtoms, uint32_t TAtom,
                         uint32_t t0_data, int window, const uint32_t *d_t0s, uint32_t N_t0,
                         const uint32_t *d_taus, uint32_t N_tau, float *d_Fmn,
                         tcw_result *d_result, int flags, char *ws, size_t ws_off) {
  TemplateDev t = make_tdev(numAtoms, TAtom, t0_data, window, N_t0, N_tau);
  tcw_tile_config cfg = h->plain_cfg;
  default_plain_cfg(t, cfg, h->n_sms);
  if (h->plain_cfg.rect_tn) cfg.rect_tn = h->plain_cfg.rect_tn;
  if (h->plain_cfg.rect_tm) cfg.rect_tm = h->plain_cfg.rect_tm;
  if (h->plain_cfg.exp_tn) cfg.exp_tn = h->plain_cfg.exp_tn;
  if (h->plain_cfg.exp_rows) cfg.exp_rows = h->plain_cfg.exp_rows;
  fill_cfg_defaults(cfg);
  std::vector<WorkItem> items;
  try {
    tile_template(0, t, cfg, items, nullptr);
  } catch (const std::bad_alloc &) {
    return set_err(h, TCW_ERR_ALLOC, "host allocation of the tile list failed");
  }
  const uint32_t n_items = (uint32_t)items.size();
  for (uint32_t k = 0; k < n_items; k++) items[k].part = k;
  t.part_off = 0;
  t.n_parts = n_items;
  t.p_off = 0;
  t.map_off = 0;

  const bool post = (flags & TCW_FLAG_POSTERIORS) != 0;
  const uint32_t n_chunks = (N_t0 + 63u) / 64u;
  Layout L;
  L.total = ws_off;
  const size_t o_T = L.add(sizeof(TemplateDev));
  const size_t o_list = L.add(sizeof(uint32_t));  // {0}: the one template
  const size_t o_items = L.add(sizeof(WorkItem) * n_items);
  const size_t o_parts = L.add(sizeof(Partial) * n_items);
  const size_t o_P = window == TCW_WINDOW_RECT
                         ? L.add(sizeof(float) * kPrefixStride * ((size_t)numAtoms + 1))
                         : 0;
  const size_t o_A8 = window == TCW_WINDOW_EXP
                          ? L.add(sizeof(float) * 8u * (size_t)numAtoms)
                          : 0;
  const size_t o_row = post ? L.add(sizeof(double) * N_t0) : 0;
  const size_t o_col = post ? L.add(sizeof(double) * (size_t)n_chunks * N_tau) : 0;
  int rc = ensure_ws(h, L.total);
  if (rc) return rc;
  ws = h->d_ws;  // the workspace may have moved
  const size_t ctl_bytes = o_parts - o_T;
  rc = ensure_stage(h, ctl_bytes);
  if (rc) return rc;
  char *st = h->h_stage;
  memcpy(st, &t, sizeof(t));
  uint32_t zero = 0;
  memcpy(st + (o_list - o_T), &zero, sizeof(zero));
  memcpy(st + (o_items - o_T), items.data(), sizeof(WorkItem) * n_items);
  TCW_CUDA(h, cudaMemcpyAsync(ws + o_T, st, ctl_bytes, cudaMemcpyHostToDevice, h->stream));
  TCW_CUDA(h, cudaEventRecord(h->stage_ev, h->stream));
  h->stage_pending = true;

  const int prec = prec_of(flags);
  const TemplateDev *dT = reinterpret_cast<const TemplateDev *>(ws + o_T);
  float *dP = window == TCW_WINDOW_RECT ? reinterpret_cast<float *>(ws + o_P) : nullptr;
  Partial *dparts = reinterpret_cast<Partial *>(ws + o_parts);
  if (window == TCW_WINDOW_RECT)
    TCW_CUDA(h, launch_prefix(dT, reinterpret_cast<const uint32_t *>(ws + o_list), 1, d_atoms,
                              dP, prec, h->stream));
  float *dA8 = window == TCW_WINDOW_EXP ? reinterpret_cast<float *>(ws + o_A8) : nullptr;
  if (window == TCW_WINDOW_EXP)
    TCW_CUDA(h, launch_repack(dT, reinterpret_cast<const uint32_t *>(ws + o_list), 1, d_atoms,
                              dA8, h->stream));
  MapLaunch ml{};
  ml.T = dT;
  ml.items = reinterpret_cast<const WorkItem *>(ws + o_items);
  ml.n_items = n_items;
  ml.persistent = false;
  ml.write_map = d_Fmn != nullptr;
  ml.prec = prec;
  ml.priority = h->prio_low;
  ml.atoms = d_atoms;
  ml.atoms8 = dA8;
  ml.t0s = d_t0s;
  ml.taus = d_taus;
  ml.P = dP;
  ml.Fmn = d_Fmn;
  ml.parts = dparts;
  TCW_CUDA(h, launch_map(window, ml, h->stream));
  TCW_CUDA(h, launch_finalize(dT, 1, dparts, d_result, h->stream));
  if (post)
    TCW_CUDA(h, launch_posteriors(dT, d_Fmn, d_result, reinterpret_cast<double *>(ws + o_row),
                                  reinterpret_cast<double *>(ws + o_col), N_t0, N_tau,
                                  h->stream));
  return TCW_OK;
}

int tcw_map_plain(tcw_handle *h, const float *d_atoms, uint32_t numAtoms, uint32_t TAtom,
                  uint32_t t0_data, int window, const uint32_t *d_t0s, uint32_t N_t0,
                  const uint32_t *d_taus, uint32_t N_tau, float *d_Fmn, tcw_result *d_result,
                  int flags) {
  if (!h) return TCW_ERR_INVALID_ARG;
  if (!d_atoms || !d_t0s || !d_taus || !d_result)
    return set_err(h, TCW_ERR_INVALID_ARG, "null device pointer");
  if (!valid_window(window))
    return set_err(h, TCW_ERR_INVALID_ARG,
                   "invalid window type %d: the device entry point takes "
                   "TCW_WINDOW_RECT or TCW_WINDOW_EXP",
                   window);
  int rc = check_geometry(h, numAtoms, TAtom, t0_data, N_t0, N_tau);
  if (rc) return rc;
  if ((flags & TCW_FLAG_POSTERIORS) && !d_Fmn)
    return set_err(h, TCW_ERR_INVALID_ARG, "posteriors need a map (d_Fmn is NULL)");
  rc = set_device(h);
  if (rc) return rc;
  return plain_enqueue(h, d_atoms, numAtoms, TAtom, t0_data, window, d_t0s, N_t0, d_taus, N_tau,
                       d_Fmn, d_result, flags, h->d_ws, 0);
}

int tcw_map_plain_host(tcw_handle *h, const float *atoms, uint32_t numAtoms, uint32_t TAtom,
                       uint32_t t0_data, int window, const uint32_t *t0s, uint32_t N_t0,
                       const uint32_t *taus, uint32_t N_tau, float *Fmn, tcw_result *result,
                       int flags) {
  if (!h) return TCW_ERR_INVALID_ARG;
  if (!atoms || !result) return set_err(h, TCW_ERR_INVALID_ARG, "null host pointer");
  if (window < 0 || window > TCW_WINDOW_EXP)
    return set_err(h, TCW_ERR_INVALID_ARG, "Unknown window-type (%d) passed as input. Allowed are [0,%d].",
                   window, TCW_WINDOW_EXP);
  uint32_t none_t0 = t0_data, none_tau = 0;
  if (window == TCW_WINDOW_NONE) {
    // one rectangular cell spanning all data (tcw_fstat_map_funcs.py:742-749)
    if ((uint64_t)numAtoms * TAtom > 0xFFFFFFFFull)
      return set_err(h, TCW_ERR_OVERFLOW, "data span exceeds the u32 range");
    none_tau = numAtoms * TAtom;
    window = TCW_WINDOW_RECT;
    t0s = &none_t0;
    taus = &none_tau;
    N_t0 = N_tau = 1;
  }
  if (!t0s || !taus) return set_err(h, TCW_ERR_INVALID_ARG, "null grid pointer");
  int rc = check_geometry(h, numAtoms, TAtom, t0_data, N_t0, N_tau);
  if (rc) return rc;
  rc = check_grids(h, window, t0s, N_t0, taus, N_tau);
  if (rc) return rc;
  rc = set_device(h);
  if (rc) return rc;
  const bool want_map = Fmn != nullptr || (flags & TCW_FLAG_POSTERIORS);
  Layout L;
  const size_t o_atoms = L.add(sizeof(float) * 7u * (size_t)numAtoms);
  const size_t o_t0 = L.add(sizeof(uint32_t) * N_t0);
  const size_t o_tau = L.add(sizeof(uint32_t) * N_tau);
  const size_t o_map = want_map ? L.add(sizeof(float) * (size_t)N_t0 * N_tau) : 0;
  const size_t o_res = L.add(sizeof(tcw_result));
  rc = ensure_ws(h, L.total + (1 << 20));
  if (rc) return rc;
  char *ws = h->d_ws;
  TCW_CUDA(h, cudaMemcpyAsync(ws + o_atoms, atoms, sizeof(float) * 7u * (size_t)numAtoms,
                              cudaMemcpyHostToDevice, h->stream));
  TCW_CUDA(h, cudaMemcpyAsync(ws + o_t0, t0s, sizeof(uint32_t) * N_t0, cudaMemcpyHostToDevice,
                              h->stream));
  TCW_CUDA(h, cudaMemcpyAsync(ws + o_tau, taus, sizeof(uint32_t) * N_tau, cudaMemcpyHostToDevice,
                              h->stream));
  // the plain enqueue places its own buffers after ours; growing the
  // workspace there would move these inputs, so reserve generously first
  size_t need_after = 0;
  {
    Layout L2;
    L2.total = L.total;
    L2.add(sizeof(TemplateDev));
    L2.add(sizeof(uint32_t));
    uint64_t items_est = (uint64_t)N_t0 * ((N_tau + 31u) / 32u) + 16u;
    L2.add(sizeof(WorkItem) * items_est);
    L2.add(sizeof(Partial) * items_est);
    if (window == TCW_WINDOW_RECT) L2.add(sizeof(float) * kPrefixStride * ((size_t)numAtoms + 1));
    if (window == TCW_WINDOW_EXP) L2.add(sizeof(float) * 8u * (size_t)numAtoms);
    L2.add(sizeof(double) * N_t0);
    L2.add(sizeof(double) * ((N_t0 + 63u) / 64u) * (size_t)N_tau);
    need_after = L2.total;
  }
  if (need_after > h->ws_cap) {
    // grow now (synchronises) and redo the input copies into the new buffer
    rc = ensure_ws(h, need_after);
    if (rc) return rc;
    ws = h->d_ws;
    TCW_CUDA(h, cudaMemcpyAsync(ws + o_atoms, atoms, sizeof(float) * 7u * (size_t)numAtoms,
                                cudaMemcpyHostToDevice, h->stream));
    TCW_CUDA(h, cudaMemcpyAsync(ws + o_t0, t0s, sizeof(uint32_t) * N_t0, cudaMemcpyHostToDevice,
                                h->stream));
    TCW_CUDA(h, cudaMemcpyAsync(ws + o_tau, taus, sizeof(uint32_t) * N_tau,
                                cudaMemcpyHostToDevice, h->stream));
  }
  float *dmap = want_map ? reinterpret_cast<float *>(ws + o_map) : nullptr;
  tcw_result *dres = reinterpret_cast<tcw_result *>(ws + o_res);
  rc = plain_enqueue(h, reinterpret_cast<const float *>(ws + o_atoms), numAtoms, TAtom, t0_data,
                     window, reinterpret_cast<const uint32_t *>(ws + o_t0), N_t0,
                     reinterpret_cast<const uint32_t *>(ws + o_tau), N_tau, dmap, dres, flags, ws,
                     L.total);
  if (rc) return rc;
  if (Fmn)
    TCW_CUDA(h, cudaMemcpyAsync(Fmn, dmap, sizeof(float) * (size_t)N_t0 * N_tau,
                                cudaMemcpyDeviceToHost, h->stream));
  TCW_CUDA(h, cudaMemcpyAsync(result, dres, sizeof(tcw_result), cudaMemcpyDeviceToHost,
                              h->stream));
  TCW_CUDA(h, cudaStreamSynchronize(h->stream));
  return TCW_OK;
}

// ---------------------------------------------------------------- batched plans

int tcw_plan_create(tcw_handle *h, const tcw_template_desc *desc, uint32_t n_templates,
                    const uint32_t *t0s, uint64_t n_t0s, const uint32_t *taus, uint64_t n_taus,
                    const tcw_tile_config *cfg_in, int flags, tcw_plan **out) {
  if (!h || !out) return TCW_ERR_INVALID_ARG;
  *out = nullptr;
  if (!desc || n_templates == 0 || !t0s || !taus)
    return set_err(h, TCW_ERR_INVALID_ARG, "empty or null template list / grids");
  int rc = set_device(h);
  if (rc) return rc;
  tcw_tile_config cfg{};
  if (cfg_in) cfg = *cfg_in;
  fill_cfg_defaults(cfg);
  cfg.exp_tn = 32;  // plans run 32-column warp tiles (tile_template's warp_tiles)

  tcw_plan *p = new (std::nothrow) tcw_plan();
  if (!p) return TCW_ERR_ALLOC;
  p->device = h->device;
  p->prec = prec_of(flags);
  p->flags = flags;
  p->n_templates = n_templates;
  p->cfg = cfg;
  std::vector<uint2> post_chunks;
  uint64_t post_rows = 0, post_cols = 0;
  std::vector<TemplateDev> T(n_templates);
  std::vector<WorkItem> items;
  std::vector<double> cost;
  std::vector<uint32_t> rect_list, exp_list;
  uint64_t p_rows = 0, a8_rows = 0, atom_rows = 0, cells = 0;
  try {
    for (uint32_t k = 0; k < n_templates; k++) {
      const tcw_template_desc &d = desc[k];
      if (!valid_window(d.window)) {
        delete p;
        return set_err(h, TCW_ERR_INVALID_ARG, "template %u: invalid window type %d", k,
                       d.window);
      }
      rc = check_geometry(h, d.numAtoms, d.TAtom, d.t0_data, d.N_t0, d.N_tau);
      if (rc) {
        delete p;
        return rc;
      }
      if (d.t0_offset + d.N_t0 > n_t0s || d.tau_offset + d.N_tau > n_taus) {
        delete p;
        return set_err(h, TCW_ERR_INVALID_ARG, "template %u: grid range outside the arrays", k);
      }
      rc = check_grids(h, d.window, t0s + d.t0_offset, d.N_t0, taus + d.tau_offset, d.N_tau);
      if (rc) {
        delete p;
        return rc;
      }
      TemplateDev t = make_tdev(d.numAtoms, d.TAtom, d.t0_data, d.window, d.N_t0, d.N_tau);
      t.atom_off = d.atom_offset;
      t.t0_off = d.t0_offset;
      t.tau_off = d.tau_offset;
      t.map_off = cells;  // maps of tcw_plan_run_maps: templates in descriptor order
      t.row_off = post_rows;  // row partials: N_t0 per column chunk
      t.col_off = post_cols;
      post_rows += (uint64_t)d.N_t0 * ((d.N_tau + kPostCols - 1u) / kPostCols);
      post_cols += d.N_tau;
      if (flags & TCW_FLAG_POSTERIORS)
        for (uint32_t n0 = 0; n0 < d.N_tau; n0 += kPostCols) post_chunks.push_back(make_uint2(k, n0));
      if (d.window == TCW_WINDOW_RECT) {
        t.p_off = p_rows;
        p_rows += (uint64_t)d.numAtoms + 1u;
        rect_list.push_back(k);
      } else {
        t.a8_off = a8_rows;
        a8_rows += d.numAtoms;
        exp_list.push_back(k);
      }
      atom_rows = std::max<uint64_t>(atom_rows, d.atom_offset + d.numAtoms);
      cells += (uint64_t)d.N_t0 * d.N_tau;
      const size_t first = items.size();
      tile_template(k, t, cfg, items, &cost, true);
      t.part_off = (uint32_t)first;
      t.n_parts = (uint32_t)(items.size() - first);
      for (size_t i = first; i < items.size(); i++) items[i].part = (uint32_t)i;
      T[k] = t;
    }
    // two queues (rect tiles, then exp tiles), each in longest-processing-time
    // order: most expensive tiles first
    std::vector<uint32_t> order(items.size());
    for (size_t i = 0; i < order.size(); i++) order[i] = (uint32_t)i;
    auto is_rect = [&](uint32_t i) { return T[items[i].tmpl].window == TCW_WINDOW_RECT; };
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) {
      if (is_rect(a) != is_rect(b)) return is_rect(a);
      return cost[a] > cost[b];
    });
    std::vector<WorkItem> sorted(items.size());
    uint32_t nr = 0;
    for (size_t i = 0; i < order.size(); i++) {
      sorted[i] = items[order[i]];
      if (is_rect(order[i])) nr++;
    }
    items.swap(sorted);
    p->n_items_rect = nr;
    p->n_items_exp = (uint32_t)items.size() - nr;
  } catch (const std::bad_alloc &) {
    delete p;
    return set_err(h, TCW_ERR_ALLOC, "host allocation failed while planning");
  }
  if (items.size() > 0xFFFFFFF0ull) {
    delete p;
    return set_err(h, TCW_ERR_OVERFLOW, "too many tiles");
  }
  p->n_items = (uint32_t)items.size();
  p->n_rect = (uint32_t)rect_list.size();
  p->n_exp = (uint32_t)exp_list.size();
  p->n_cells = cells;
  p->n_atom_rows = atom_rows;
  p->p_rows = p_rows;
  {
    const uint32_t br = (uint32_t)std::min<int>(map_blocks_per_sm(TCW_WINDOW_RECT, p->prec),
                                                (int)cfg.blocks_per_sm);
    const uint32_t be = (uint32_t)std::min<int>(map_blocks_per_sm(TCW_WINDOW_EXP, p->prec),
                                                (int)cfg.blocks_per_sm);
    p->n_blocks_rect = (uint32_t)std::max<uint64_t>(
        1, std::min<uint64_t>(p->n_items_rect, (uint64_t)br * h->n_sms));
    p->n_blocks_exp = (uint32_t)std::max<uint64_t>(
        1, std::min<uint64_t>(p->n_items_exp, (uint64_t)be * h->n_sms));
  }

  Layout L;
  const size_t o_T = L.add(sizeof(TemplateDev) * n_templates);
  const size_t o_items = L.add(sizeof(WorkItem) * p->n_items);
  const size_t o_list = L.add(sizeof(uint32_t) * std::max<size_t>(1, rect_list.size()));
  const size_t o_elist = L.add(sizeof(uint32_t) * std::max<size_t>(1, exp_list.size()));
  const size_t o_t0 = L.add(sizeof(uint32_t) * n_t0s);
  const size_t o_tau = L.add(sizeof(uint32_t) * n_taus);
  const size_t ctl_end = L.total;
  const size_t o_parts = L.add(sizeof(Partial) * p->n_items);
  const size_t o_P = L.add(sizeof(float) * kPrefixStride * std::max<uint64_t>(1, p_rows));
  const size_t o_A8 = L.add(sizeof(float) * 8u * std::max<uint64_t>(1, a8_rows));
  const size_t o_cnt = L.add(2 * sizeof(uint32_t));
  const bool post = (flags & TCW_FLAG_POSTERIORS) != 0;
  const size_t o_chunks = post ? L.add(sizeof(uint2) * std::max<size_t>(1, post_chunks.size())) : 0;
  const size_t o_rowsum = post ? L.add(sizeof(float) * std::max<uint64_t>(1, post_rows)) : 0;
  const size_t o_colsum = post ? L.add(sizeof(double) * std::max<uint64_t>(1, post_cols)) : 0;
  void *buf = nullptr;
  rc = ws_alloc(h, &buf, L.total);
  if (rc) {
    delete p;
    return rc;
  }
  p->d_buf = static_cast<char *>(buf);
  p->d_T = reinterpret_cast<TemplateDev *>(p->d_buf + o_T);
  p->d_items = reinterpret_cast<WorkItem *>(p->d_buf + o_items);
  p->d_rect_list = reinterpret_cast<uint32_t *>(p->d_buf + o_list);
  p->d_exp_list = reinterpret_cast<uint32_t *>(p->d_buf + o_elist);
  p->d_A8 = reinterpret_cast<float *>(p->d_buf + o_A8);
  p->d_t0s = reinterpret_cast<uint32_t *>(p->d_buf + o_t0);
  p->d_taus = reinterpret_cast<uint32_t *>(p->d_buf + o_tau);
  p->d_parts = reinterpret_cast<Partial *>(p->d_buf + o_parts);
  p->d_P = reinterpret_cast<float *>(p->d_buf + o_P);
  p->d_counter = reinterpret_cast<uint32_t *>(p->d_buf + o_cnt);
  if (post) {
    p->d_post_chunks = reinterpret_cast<uint2 *>(p->d_buf + o_chunks);
    p->n_post_chunks = (uint32_t)post_chunks.size();
    p->d_rowpart = reinterpret_cast<float *>(p->d_buf + o_rowsum);
    p->d_colsum = reinterpret_cast<double *>(p->d_buf + o_colsum);
  }
  // control data: a synchronous copy (plans are built once)
  std::vector<char> host(ctl_end, 0);
  memcpy(host.data() + o_T, T.data(), sizeof(TemplateDev) * n_templates);
  memcpy(host.data() + o_items, items.data(), sizeof(WorkItem) * p->n_items);
  if (!rect_list.empty())
    memcpy(host.data() + o_list, rect_list.data(), sizeof(uint32_t) * rect_list.size());
  if (!exp_list.empty())
    memcpy(host.data() + o_elist, exp_list.data(), sizeof(uint32_t) * exp_list.size());
  memcpy(host.data() + o_t0, t0s, sizeof(uint32_t) * n_t0s);
  memcpy(host.data() + o_tau, taus, sizeof(uint32_t) * n_taus);
  cudaError_t e = cudaMemcpy(p->d_buf, host.data(), ctl_end, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && post && !post_chunks.empty())
    e = cudaMemcpy(p->d_post_chunks, post_chunks.data(), sizeof(uint2) * post_chunks.size(),
                   cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(p->d_buf);
    delete p;
    return cuda_err(h, e, "plan upload");
  }
  *out = p;
  return TCW_OK;
}

int tcw_plan_destroy(tcw_plan *p) {
  if (!p) return TCW_ERR_INVALID_ARG;
  cudaSetDevice(p->device);
  cudaDeviceSynchronize();
  if (p->gexec) cudaGraphExecDestroy(p->gexec);
  if (p->d_buf) cudaFree(p->d_buf);
  if (p->d_atoms_in) cudaFree(p->d_atoms_in);
  if (p->d_res_out) cudaFree(p->d_res_out);
  if (p->d_maps_out) cudaFree(p->d_maps_out);
  cudaGetLastError();
  delete p;
  return TCW_OK;
}

int tcw_plan_info(const tcw_plan *p, uint64_t *n_cells, uint32_t *n_items,
                  uint64_t *n_atom_rows, tcw_tile_config *cfg) {
  if (!p) return TCW_ERR_INVALID_ARG;
  if (n_cells) *n_cells = p->n_cells;
  if (n_items) *n_items = p->n_items;
  if (n_atom_rows) *n_atom_rows = p->n_atom_rows;
  if (cfg) *cfg = p->cfg;
  return TCW_OK;
}

static MapLaunch plan_launch(const tcw_handle *h, const tcw_plan *p, int window,
                             const float *d_atoms, float *d_maps) {
  MapLaunch ml{};
  const bool rect = window == TCW_WINDOW_RECT;
  ml.T = p->d_T;
  ml.items = p->d_items + (rect ? 0 : p->n_items_rect);
  ml.n_items = rect ? p->n_items_rect : p->n_items_exp;
  ml.counter = p->d_counter + (rect ? 0 : 1);
  ml.n_blocks = rect ? p->n_blocks_rect : p->n_blocks_exp;
  ml.persistent = true;
  ml.write_map = d_maps != nullptr;
  ml.prec = p->prec;
  ml.priority = rect ? h->prio_low : h->prio_high;
  ml.atoms = d_atoms;
  ml.atoms8 = p->d_A8;
  ml.t0s = p->d_t0s;
  ml.taus = p->d_taus;
  ml.P = p->d_P;
  ml.Fmn = d_maps;
  ml.parts = p->d_parts;
  return ml;
}

// (repack -> exp tiles on the main stream at high priority) || (prefix ->
// rect tiles on the side stream) -> finalize.  The exp tiles are the long
// ones; the rect kernel's blocks fill SMs as exp blocks retire.
// `inputs_read` / `inputs_read_side`, if set, are recorded once the atoms
// have been read (after the repack kernel on the main stream and the prefix
// kernel on the side stream; the map kernels read only their outputs).
static int plan_enqueue(tcw_handle *h, tcw_plan *p, const float *d_atoms, tcw_result *d_results,
                        float *d_maps, cudaEvent_t inputs_read = nullptr,
                        cudaEvent_t inputs_read_side = nullptr) {
  TCW_CUDA(h, cudaMemsetAsync(p->d_counter, 0, 2 * sizeof(uint32_t), h->stream));
  // Two branches from the start: repack -> exp tiles (main stream, high
  // priority) || prefix -> rect tiles (side stream, low priority), so the
  // exp kernel does not wait for the rect templates' prefix scans; the
  // persistent rect blocks take the SMs that exp blocks leave as the exp
  // tile queue runs dry (its tail).
  TCW_CUDA(h, cudaEventRecord(h->fork_ev, h->stream));
  TCW_CUDA(h, cudaStreamWaitEvent(h->side_stream, h->fork_ev, 0));
  TCW_CUDA(h, launch_repack(p->d_T, p->d_exp_list, p->n_exp, d_atoms, p->d_A8, h->stream));
  if (inputs_read) TCW_CUDA(h, cudaEventRecord(inputs_read, h->stream));
  TCW_CUDA(h, launch_prefix(p->d_T, p->d_rect_list, p->n_rect, d_atoms, p->d_P, p->prec,
                            h->side_stream));
  if (inputs_read_side) TCW_CUDA(h, cudaEventRecord(inputs_read_side, h->side_stream));
  TCW_CUDA(h, launch_map(TCW_WINDOW_EXP, plan_launch(h, p, TCW_WINDOW_EXP, d_atoms, d_maps),
                         h->stream));
  TCW_CUDA(h, launch_map(TCW_WINDOW_RECT, plan_launch(h, p, TCW_WINDOW_RECT, d_atoms, d_maps),
                         h->side_stream));
  TCW_CUDA(h, cudaEventRecord(h->join_ev, h->side_stream));
  TCW_CUDA(h, cudaStreamWaitEvent(h->stream, h->join_ev, 0));
  TCW_CUDA(h, launch_finalize(p->d_T, p->n_templates, p->d_parts, d_results, h->stream));
  if (d_maps && (p->flags & TCW_FLAG_POSTERIORS))
    TCW_CUDA(h, launch_plan_posteriors(p->d_T, p->n_templates, p->d_post_chunks, p->n_post_chunks,
                                       d_maps, d_results, p->d_rowpart, p->d_colsum, h->stream));
  return TCW_OK;
}

}  // extern "C"

static int plan_run(tcw_handle *h, tcw_plan *p, const float *d_atoms, tcw_result *d_results,
                    float *d_maps, int use_graph) {
  if (!h || !p) return TCW_ERR_INVALID_ARG;
  if (!d_atoms || !d_results) return set_err(h, TCW_ERR_INVALID_ARG, "null device pointer");
  if ((p->flags & TCW_FLAG_POSTERIORS) && !d_maps)
    return set_err(h, TCW_ERR_INVALID_ARG,
                   "posteriors need the maps: run the plan with tcw_plan_run_maps");
  if (p->device != h->device)
    return set_err(h, TCW_ERR_INVALID_ARG, "plan and handle are on different devices");
  int rc = set_device(h);
  if (rc) return rc;
  // stream capture is not allowed on the legacy default stream: run directly
  if (!use_graph || h->stream == nullptr || h->stream == cudaStreamLegacy)
    return plan_enqueue(h, p, d_atoms, d_results, d_maps);
  if (!p->gexec || p->g_atoms != d_atoms || p->g_results != d_results || p->g_maps != d_maps ||
      p->g_stream != h->stream) {
    if (p->gexec) {
      cudaGraphExecDestroy(p->gexec);
      p->gexec = nullptr;
    }
    TCW_CUDA(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    rc = plan_enqueue(h, p, d_atoms, d_results, d_maps);
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(h->stream, &graph);
    if (rc) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    if (e != cudaSuccess) return cuda_err(h, e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&p->gexec, graph, cudaGraphInstantiateFlagUseNodePriority);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
      p->gexec = nullptr;
      return cuda_err(h, e, "cudaGraphInstantiate");
    }
    p->g_atoms = d_atoms;
    p->g_results = d_results;
    p->g_maps = d_maps;
    p->g_stream = h->stream;
  }
  TCW_CUDA(h, cudaGraphLaunch(p->gexec, h->stream));
  return TCW_OK;
}

extern "C" {

int tcw_plan_run(tcw_handle *h, tcw_plan *p, const float *d_atoms, tcw_result *d_results,
                 int use_graph) {
  return plan_run(h, p, d_atoms, d_results, nullptr, use_graph);
}

int tcw_plan_run_maps(tcw_handle *h, tcw_plan *p, const float *d_atoms, tcw_result *d_results,
                      float *d_maps, int use_graph) {
  if (h && !d_maps) return set_err(h, TCW_ERR_INVALID_ARG, "null map buffer");
  return plan_run(h, p, d_atoms, d_results, d_maps, use_graph);
}

int tcw_plan_run_timed(tcw_handle *h, tcw_plan *p, const float *d_atoms, tcw_result *d_results,
                       float *ms) {
  if (!h || !p || !ms) return TCW_ERR_INVALID_ARG;
  if (!d_atoms || !d_results) return set_err(h, TCW_ERR_INVALID_ARG, "null device pointer");
  int rc = set_device(h);
  if (rc) return rc;
  cudaEvent_t ev[5];
  for (int i = 0; i < 5; i++) TCW_CUDA(h, cudaEventCreate(&ev[i]));
  TCW_CUDA(h, cudaMemsetAsync(p->d_counter, 0, 2 * sizeof(uint32_t), h->stream));
  TCW_CUDA(h, cudaEventRecord(ev[0], h->stream));
  TCW_CUDA(h, launch_prefix(p->d_T, p->d_rect_list, p->n_rect, d_atoms, p->d_P, p->prec,
                            h->stream));
  TCW_CUDA(h, launch_repack(p->d_T, p->d_exp_list, p->n_exp, d_atoms, p->d_A8, h->stream));
  TCW_CUDA(h, cudaEventRecord(ev[1], h->stream));
  TCW_CUDA(h, launch_map(TCW_WINDOW_RECT, plan_launch(h, p, TCW_WINDOW_RECT, d_atoms, nullptr),
                         h->stream));
  TCW_CUDA(h, cudaEventRecord(ev[2], h->stream));
  TCW_CUDA(h, launch_map(TCW_WINDOW_EXP, plan_launch(h, p, TCW_WINDOW_EXP, d_atoms, nullptr),
                         h->stream));
  TCW_CUDA(h, cudaEventRecord(ev[3], h->stream));
  TCW_CUDA(h, launch_finalize(p->d_T, p->n_templates, p->d_parts, d_results, h->stream));
  TCW_CUDA(h, cudaEventRecord(ev[4], h->stream));
  TCW_CUDA(h, cudaEventSynchronize(ev[4]));
  for (int i = 0; i < 4; i++) TCW_CUDA(h, cudaEventElapsedTime(&ms[i], ev[i], ev[i + 1]));
  for (int i = 0; i < 5; i++) cudaEventDestroy(ev[i]);
  return TCW_OK;
}

// ---------------------------------------------------------------- differentiable path

// Validates descriptors, uploads descriptors, tiles and grids into the
// handle's workspace; returns the layout of what follows them.
struct DiffSetup {
  size_t o_T, o_items, o_parts, o_t0, o_cnt, o_scratch, o_rlist, o_D64, o_elist, o_A8, total;
  uint32_t n_items, n_blocks, max_rows;
  uint32_t n_rect_items, n_rect_blocks, n_rect, n_exp;
  uint64_t p_rows;
};

static int diff_prepare(tcw_handle *h, const tcw_diff_desc *desc, uint32_t n,
                        const uint32_t *t0s, uint64_t n_t0s, int pass, DiffSetup &S) {
  if (!desc || n == 0 || !t0s) return set_err(h, TCW_ERR_INVALID_ARG, "empty template list");
  std::vector<DiffTemplate> T(n);
  std::vector<DiffItem> items, ritems;
  std::vector<uint32_t> rlist, elist;
  uint32_t max_rows = 0;
  uint64_t p_rows = 0, atom_rows = 0;
  try {
    for (uint32_t k = 0; k < n; k++) {
      const tcw_diff_desc &d = desc[k];
      int rc = check_geometry(h, d.numAtoms, d.TAtom, d.t0_data, d.N_t0, d.N_tau);
      if (rc) return rc;
      if (d.t0_offset + d.N_t0 > n_t0s)
        return set_err(h, TCW_ERR_INVALID_ARG, "template %u: t0 grid outside the array", k);
      if (!(d.tau_min > 0.0) || !(d.tau_max >= d.tau_min))
        return set_err(h, TCW_ERR_INVALID_ARG, "template %u: need 0 < tau_min <= tau_max", k);
      const uint32_t *g = t0s + d.t0_offset;
      if ((uint64_t)g[0] + d.TAtom / 2u < d.t0_data)
        return set_err(h, TCW_ERR_INVALID_ARG, "template %u: t0 grid starts before the data", k);
      for (uint32_t m = 1; m < d.N_t0; m++)
        if (g[m] < g[m - 1])
          return set_err(h, TCW_ERR_INVALID_ARG, "template %u: t0 grid must be non-decreasing", k);
      if (d.window != 0 && d.window != TCW_WINDOW_EXP && d.window != TCW_WINDOW_RECT)
        return set_err(h, TCW_ERR_INVALID_ARG, "template %u: invalid window type %u", k,
                       d.window);
      const bool rect = d.window == TCW_WINDOW_RECT;
      if ((double)g[d.N_t0 - 1] + (rect ? 1.0 : 3.0) * d.tau_max >= 4294967295.0)
        return set_err(h, TCW_ERR_OVERFLOW, "template %u: window end exceeds the u32 range", k);
      DiffTemplate t{};
      t.atom_off = d.atom_offset;
      t.t0_off = d.t0_offset;
      t.g = make_geom(d.numAtoms, d.TAtom, d.t0_data);
      t.N_t0 = d.N_t0;
      t.N_tau = d.N_tau;
      t.tau_min = d.tau_min;
      t.tau_max = d.tau_max;
      t.window = rect ? (uint32_t)TCW_WINDOW_RECT : (uint32_t)TCW_WINDOW_EXP;
      std::vector<DiffItem> &dst = rect ? ritems : items;
      t.part_off = (uint32_t)dst.size();  // rect parts are shifted past the exp ones below
      // exp tiles: 128 tau columns, all rows; rect tiles: 128 t0 rows, all columns
      const uint32_t extent = rect ? d.N_t0 : d.N_tau;
      for (uint32_t n0 = 0; n0 < extent; n0 += 128u)
        dst.push_back(DiffItem{k, (uint32_t)dst.size(), n0, std::min(extent, n0 + 128u)});
      t.n_parts = (uint32_t)dst.size() - t.part_off;
      if (rect) {
        t.p_off = p_rows;
        p_rows += (uint64_t)d.numAtoms + 1u;
        rlist.push_back(k);
      } else {
        max_rows = std::max(max_rows, d.N_t0);
        elist.push_back(k);
        atom_rows = std::max<uint64_t>(atom_rows, d.atom_offset + d.numAtoms);
      }
      T[k] = t;
    }
    const uint32_t n_exp_items = (uint32_t)items.size();
    for (DiffItem &it : ritems) it.part += n_exp_items;
    for (uint32_t k : rlist) T[k].part_off += n_exp_items;
    items.insert(items.end(), ritems.begin(), ritems.end());
    S.n_rect_items = (uint32_t)ritems.size();
    S.n_items = n_exp_items;
  } catch (const std::bad_alloc &) {
    return set_err(h, TCW_ERR_ALLOC, "host allocation failed");
  }
  S.max_rows = max_rows;
  S.n_rect = (uint32_t)rlist.size();
  S.n_exp = (uint32_t)elist.size();
  S.p_rows = p_rows;
  S.n_blocks = (uint32_t)std::max<uint64_t>(
      1, std::min<uint64_t>(S.n_items, (uint64_t)diff_blocks_per_sm(pass) * h->n_sms));
  S.n_rect_blocks = (uint32_t)std::max<uint64_t>(
      1, std::min<uint64_t>(S.n_rect_items, (uint64_t)rect_diff_blocks_per_sm(pass) * h->n_sms));
  const size_t n_all_items = (size_t)S.n_items + S.n_rect_items;
  Layout L;
  S.o_T = L.add(sizeof(DiffTemplate) * n);
  S.o_items = L.add(sizeof(DiffItem) * n_all_items);
  S.o_t0 = L.add(sizeof(uint32_t) * n_t0s);
  S.o_cnt = L.add(2 * sizeof(uint32_t));
  S.o_rlist = L.add(sizeof(uint32_t) * std::max<size_t>(1, rlist.size()));
  S.o_elist = L.add(sizeof(uint32_t) * std::max<size_t>(1, elist.size()));
  const size_t ctl = L.total;
  S.o_parts = L.add(sizeof(DiffPartial) * n_all_items);
  S.o_scratch = (pass == 1 && S.n_items)
                    ? L.add(sizeof(float) * TCW_DIFF_SLOTS * 128u * (size_t)max_rows * S.n_blocks)
                    : 0;
  S.o_D64 = pass == 1 ? L.add(sizeof(double) * 8u * std::max<uint64_t>(1, p_rows)) : 0;
  // the exponential templates' atoms in 32-byte rows, at their own row index
  S.o_A8 = S.n_items ? L.add(sizeof(float) * 8u * std::max<uint64_t>(1, atom_rows)) : 0;
  S.total = L.total;
  int rc = ensure_ws(h, S.total);
  if (rc) return rc;
  rc = ensure_stage(h, ctl);
  if (rc) return rc;
  memcpy(h->h_stage + S.o_T, T.data(), sizeof(DiffTemplate) * n);
  memcpy(h->h_stage + S.o_items, items.data(), sizeof(DiffItem) * n_all_items);
  memcpy(h->h_stage + S.o_t0, t0s, sizeof(uint32_t) * n_t0s);
  memset(h->h_stage + S.o_cnt, 0, 2 * sizeof(uint32_t));
  if (!rlist.empty()) memcpy(h->h_stage + S.o_rlist, rlist.data(), sizeof(uint32_t) * rlist.size());
  if (!elist.empty()) memcpy(h->h_stage + S.o_elist, elist.data(), sizeof(uint32_t) * elist.size());
  TCW_CUDA(h, cudaMemcpyAsync(h->d_ws, h->h_stage, ctl, cudaMemcpyHostToDevice, h->stream));
  TCW_CUDA(h, cudaEventRecord(h->stage_ev, h->stream));
  h->stage_pending = true;
  return TCW_OK;
}

static DiffLaunch diff_launch(tcw_handle *h, const DiffSetup &S, const float *d_atoms,
                              double temperature) {
  DiffLaunch L{};
  L.T = reinterpret_cast<const DiffTemplate *>(h->d_ws + S.o_T);
  L.items = reinterpret_cast<const DiffItem *>(h->d_ws + S.o_items);
  L.n_items = S.n_items;
  L.n_blocks = S.n_blocks;
  L.counter = reinterpret_cast<uint32_t *>(h->d_ws + S.o_cnt);
  L.atoms = d_atoms;
  L.t0s = reinterpret_cast<const uint32_t *>(h->d_ws + S.o_t0);
  L.temp = temperature;
  L.parts = reinterpret_cast<DiffPartial *>(h->d_ws + S.o_parts);
  L.rect_items = L.items + S.n_items;
  L.n_rect_items = S.n_rect_items;
  L.n_rect_blocks = S.n_rect_blocks;
  L.rect_counter = L.counter + 1;
  L.rect_list = reinterpret_cast<const uint32_t *>(h->d_ws + S.o_rlist);
  L.n_rect = S.n_rect;
  L.D64 = S.o_D64 ? reinterpret_cast<double *>(h->d_ws + S.o_D64) : nullptr;
  L.atoms8 = S.o_A8 ? reinterpret_cast<float *>(h->d_ws + S.o_A8) : nullptr;
  L.exp_list = reinterpret_cast<const uint32_t *>(h->d_ws + S.o_elist);
  L.n_exp = S.n_exp;
  return L;
}

int tcw_map_forward(tcw_handle *h, const tcw_diff_desc *desc, uint32_t n_templates,
                    const float *d_atoms, const uint32_t *t0s, uint64_t n_t0s,
                    double temperature, double *d_lnBtSG, double *d_softmax2F) {
  if (!h) return TCW_ERR_INVALID_ARG;
  if (!d_atoms || !d_lnBtSG || !d_softmax2F)
    return set_err(h, TCW_ERR_INVALID_ARG, "null device pointer");
  if (!(temperature > 0.0)) return set_err(h, TCW_ERR_INVALID_ARG, "temperature must be > 0");
  int rc = set_device(h);
  if (rc) return rc;
  DiffSetup S;
  rc = diff_prepare(h, desc, n_templates, t0s, n_t0s, 0, S);
  if (rc) return rc;
  DiffLaunch L = diff_launch(h, S, d_atoms, temperature);
  TCW_CUDA(h, launch_diff(0, L, h->stream));
  TCW_CUDA(h, launch_diff_finalize(L.T, n_templates, L.parts, temperature, d_lnBtSG, d_softmax2F,
                                   h->stream));
  return TCW_OK;
}

int tcw_map_backward(tcw_handle *h, const tcw_diff_desc *desc, uint32_t n_templates,
                     const float *d_atoms, const uint32_t *t0s, uint64_t n_t0s,
                     double temperature, const double *d_lnBtSG, const double *d_softmax2F,
                     const double *d_grad_lnBtSG, const double *d_grad_softmax2F,
                     double *d_grad_atoms, uint64_t n_atom_rows, double *d_grad_tau) {
  if (!h) return TCW_ERR_INVALID_ARG;
  if (!d_atoms || !d_lnBtSG || !d_softmax2F || !d_grad_lnBtSG || !d_grad_softmax2F ||
      !d_grad_atoms || !d_grad_tau)
    return set_err(h, TCW_ERR_INVALID_ARG, "null device pointer");
  if (!(temperature > 0.0)) return set_err(h, TCW_ERR_INVALID_ARG, "temperature must be > 0");
  for (uint32_t k = 0; desc && k < n_templates; k++)
    if (desc[k].atom_offset + desc[k].numAtoms > n_atom_rows)
      return set_err(h, TCW_ERR_INVALID_ARG, "template %u: atoms outside the gradient array", k);
  int rc = set_device(h);
  if (rc) return rc;
  DiffSetup S;
  rc = diff_prepare(h, desc, n_templates, t0s, n_t0s, 1, S);
  if (rc) return rc;
  DiffLaunch L = diff_launch(h, S, d_atoms, temperature);
  L.lnZ1 = d_lnBtSG;
  L.lnZ2 = d_softmax2F;
  L.gB = d_grad_lnBtSG;
  L.gS = d_grad_softmax2F;
  L.scratch = reinterpret_cast<float *>(h->d_ws + S.o_scratch);
  L.scratch_rows = S.max_rows;
  L.grad_atoms = d_grad_atoms;
  L.grad_tau = d_grad_tau;
  TCW_CUDA(h, cudaMemsetAsync(d_grad_atoms, 0, sizeof(double) * 7u * n_atom_rows, h->stream));
  TCW_CUDA(h, cudaMemsetAsync(d_grad_tau, 0, sizeof(double) * 2u * n_templates, h->stream));
  if (S.n_rect)
    TCW_CUDA(h, cudaMemsetAsync(L.D64, 0, sizeof(double) * 8u * S.p_rows, h->stream));
  TCW_CUDA(h, launch_diff(1, L, h->stream));
  return TCW_OK;
}

int tcw_plan_run_host(tcw_handle *h, tcw_plan *p, const float *atoms, tcw_result *results) {
  if (!h || !p) return TCW_ERR_INVALID_ARG;
  if (!atoms || !results) return set_err(h, TCW_ERR_INVALID_ARG, "null host pointer");
  int rc = set_device(h);
  if (rc) return rc;
  const size_t abytes = sizeof(float) * 7u * (size_t)p->n_atom_rows;
  if (!p->d_atoms_in) {
    void *a = nullptr, *r = nullptr;
    rc = ws_alloc(h, &a, std::max<size_t>(abytes, 16));
    if (rc) return rc;
    rc = ws_alloc(h, &r, sizeof(tcw_result) * p->n_templates);
    if (rc) {
      cudaFree(a);
      return rc;
    }
    p->d_atoms_in = static_cast<float *>(a);
    p->d_res_out = static_cast<tcw_result *>(r);
  }
  TCW_CUDA(h, cudaMemcpyAsync(p->d_atoms_in, atoms, abytes, cudaMemcpyHostToDevice, h->stream));
  rc = tcw_plan_run(h, p, p->d_atoms_in, p->d_res_out, 1);
  if (rc) return rc;
  TCW_CUDA(h, cudaMemcpyAsync(results, p->d_res_out, sizeof(tcw_result) * p->n_templates,
                              cudaMemcpyDeviceToHost, h->stream));
  TCW_CUDA(h, cudaStreamSynchronize(h->stream));
  return TCW_OK;
}

int tcw_plan_run_host_async(tcw_handle *h, tcw_plan *p, const float *atoms,
                            tcw_result *results) {
  if (!h || !p) return TCW_ERR_INVALID_ARG;
  if (!atoms || !results) return set_err(h, TCW_ERR_INVALID_ARG, "null host pointer");
  if (p->flags & TCW_FLAG_POSTERIORS)
    return set_err(h, TCW_ERR_INVALID_ARG,
                   "posteriors need the maps: run the plan with tcw_plan_run_maps");
  if (p->device != h->device)
    return set_err(h, TCW_ERR_INVALID_ARG, "plan and handle are on different devices");
  int rc = set_device(h);
  if (rc) return rc;
  const size_t abytes = sizeof(float) * 7u * (size_t)p->n_atom_rows;
  if (!p->d_atoms_in) {
    void *a = nullptr, *r = nullptr;
    rc = ws_alloc(h, &a, std::max<size_t>(abytes, 16));
    if (rc) return rc;
    rc = ws_alloc(h, &r, sizeof(tcw_result) * p->n_templates);
    if (rc) {
      cudaFree(a);
      return rc;
    }
    p->d_atoms_in = static_cast<float *>(a);
    p->d_res_out = static_cast<tcw_result *>(r);
  }
  // the upload may start as soon as the previous run has read its atoms, so
  // it overlaps that run's map kernels
  if (h->consumed_pending) {
    TCW_CUDA(h, cudaStreamWaitEvent(h->copy_stream, h->consumed_ev, 0));
    TCW_CUDA(h, cudaStreamWaitEvent(h->copy_stream, h->consumed_side_ev, 0));
  }
  TCW_CUDA(h, cudaMemcpyAsync(p->d_atoms_in, atoms, abytes, cudaMemcpyHostToDevice,
                              h->copy_stream));
  TCW_CUDA(h, cudaEventRecord(h->copied_ev, h->copy_stream));
  TCW_CUDA(h, cudaStreamWaitEvent(h->stream, h->copied_ev, 0));
  // the compensated map kernels read only the prefix and repacked rows; the
  // uncompensated exp kernel reads the atoms themselves
  const bool maps_read_atoms = p->prec == kPrecPlain32;
  rc = plan_enqueue(h, p, p->d_atoms_in, p->d_res_out, nullptr,
                    maps_read_atoms ? nullptr : h->consumed_ev,
                    maps_read_atoms ? nullptr : h->consumed_side_ev);
  if (rc) return rc;
  if (maps_read_atoms) {
    TCW_CUDA(h, cudaEventRecord(h->consumed_ev, h->stream));
    TCW_CUDA(h, cudaEventRecord(h->consumed_side_ev, h->stream));
  }
  h->consumed_pending = true;
  TCW_CUDA(h, cudaMemcpyAsync(results, p->d_res_out, sizeof(tcw_result) * p->n_templates,
                              cudaMemcpyDeviceToHost, h->stream));
  return TCW_OK;
}

int tcw_plan_run_maps_host(tcw_handle *h, tcw_plan *p, const float *atoms, tcw_result *results,
                           float *maps) {
  if (!h || !p) return TCW_ERR_INVALID_ARG;
  if (!atoms || !results || !maps) return set_err(h, TCW_ERR_INVALID_ARG, "null host pointer");
  int rc = set_device(h);
  if (rc) return rc;
  const size_t abytes = sizeof(float) * 7u * (size_t)p->n_atom_rows;
  const size_t mbytes = sizeof(float) * (size_t)p->n_cells;
  if (!p->d_atoms_in) {
    void *a = nullptr, *r = nullptr;
    rc = ws_alloc(h, &a, std::max<size_t>(abytes, 16));
    if (rc) return rc;
    rc = ws_alloc(h, &r, sizeof(tcw_result) * p->n_templates);
    if (rc) {
      cudaFree(a);
      return rc;
    }
    p->d_atoms_in = static_cast<float *>(a);
    p->d_res_out = static_cast<tcw_result *>(r);
  }
  if (!p->d_maps_out) {
    void *m = nullptr;
    rc = ws_alloc(h, &m, std::max<size_t>(mbytes, 16));
    if (rc) return rc;
    p->d_maps_out = static_cast<float *>(m);
  }
  TCW_CUDA(h, cudaMemcpyAsync(p->d_atoms_in, atoms, abytes, cudaMemcpyHostToDevice, h->stream));
  rc = plan_run(h, p, p->d_atoms_in, p->d_res_out, p->d_maps_out, 1);
  if (rc) return rc;
  TCW_CUDA(h, cudaMemcpyAsync(results, p->d_res_out, sizeof(tcw_result) * p->n_templates,
                              cudaMemcpyDeviceToHost, h->stream));
  TCW_CUDA(h, cudaMemcpyAsync(maps, p->d_maps_out, mbytes, cudaMemcpyDeviceToHost, h->stream));
  TCW_CUDA(h, cudaStreamSynchronize(h->stream));
  return TCW_OK;
}

int tcw_map_batched(tcw_handle *h, const tcw_template_desc *desc, uint32_t n_templates,
                    const uint32_t *t0s, uint64_t n_t0s, const uint32_t *taus, uint64_t n_taus,
                    const float *atoms_concat, const tcw_tile_config *cfg, float *max2F,
                    int64_t *argmax, double *lnBtSG) {
  if (!h) return TCW_ERR_INVALID_ARG;
  if (!atoms_concat || !max2F || !argmax || !lnBtSG)
    return set_err(h, TCW_ERR_INVALID_ARG, "null host pointer");
  tcw_plan *p = nullptr;
  int rc = tcw_plan_create(h, desc, n_templates, t0s, n_t0s, taus, n_taus, cfg, TCW_FLAG_LNBTSG,
                           &p);
  if (rc) return rc;
  std::vector<tcw_result> res;
  try {
    res.resize(n_templates);
  } catch (const std::bad_alloc &) {
    tcw_plan_destroy(p);
    return set_err(h, TCW_ERR_ALLOC, "host allocation failed");
  }
  rc = tcw_plan_run_host(h, p, atoms_concat, res.data());
  tcw_plan_destroy(p);
  if (rc) return rc;
  for (uint32_t k = 0; k < n_templates; k++) {
    max2F[k] = 2.0f * res[k].maxF;
    argmax[k] = res[k].argmax;
    lnBtSG[k] = res[k].lnBtSG;
  }
  return TCW_OK;
}

int tcw_debug_check_failures(uint32_t *count) {
  if (!count) return TCW_ERR_INVALID_ARG;
  uint64_t n = (uint64_t)dcheck_failures_kernels() + dcheck_failures_diff() +
               dcheck_failures_f64() + dcheck_failures_noalloc();
  *count = (uint32_t)std::min<uint64_t>(n, 0xFFFFFFFFull);
#if defined(TCW_DEBUG_CHECKS)
  return TCW_OK;
#else
  return TCW_ERR_UNSUPPORTED;
#endif
}

int tcw_map_f64(tcw_handle *h, const float *d_atoms, uint32_t numAtoms, uint32_t TAtom,
                uint32_t t0_data, int window, const uint32_t *d_t0s, uint32_t N_t0,
                const uint32_t *d_taus, uint32_t N_tau, const uint32_t *rows, uint32_t n_rows,
                double *d_F, double *d_cond) {
  if (!h) return TCW_ERR_INVALID_ARG;
  if (!d_atoms || !d_t0s || !d_taus || !d_F)
    return set_err(h, TCW_ERR_INVALID_ARG, "null device pointer");
  if (!valid_window(window))
    return set_err(h, TCW_ERR_INVALID_ARG,
                   "invalid window type %d: TCW_WINDOW_RECT or TCW_WINDOW_EXP", window);
  int rc = check_geometry(h, numAtoms, TAtom, t0_data, N_t0, N_tau);
  if (rc) return rc;
  if (!rows && n_rows != N_t0)
    return set_err(h, TCW_ERR_INVALID_ARG, "without a row list n_rows must equal N_t0");
  if (n_rows == 0) return set_err(h, TCW_ERR_INVALID_ARG, "no rows requested");
  if (rows)
    for (uint32_t k = 0; k < n_rows; k++)
      if (rows[k] >= N_t0)
        return set_err(h, TCW_ERR_INVALID_ARG, "row %u (entry %u) outside the t0 grid of %u",
                       rows[k], k, N_t0);
  rc = set_device(h);
  if (rc) return rc;
  const uint32_t *d_rows = nullptr;
  if (rows) {
    const size_t bytes = sizeof(uint32_t) * (size_t)n_rows;
    rc = ensure_ws(h, bytes);
    if (rc) return rc;
    rc = ensure_stage(h, bytes);
    if (rc) return rc;
    memcpy(h->h_stage, rows, bytes);
    TCW_CUDA(h, cudaMemcpyAsync(h->d_ws, h->h_stage, bytes, cudaMemcpyHostToDevice, h->stream));
    TCW_CUDA(h, cudaEventRecord(h->stage_ev, h->stream));
    h->stage_pending = true;
    d_rows = reinterpret_cast<const uint32_t *>(h->d_ws);
  }
  const Geom g = make_geom(numAtoms, TAtom, t0_data);
  TCW_CUDA(h, launch_map_f64(window, d_atoms, g, d_t0s, d_taus, N_tau, d_rows, n_rows, d_F,
                             d_cond, h->stream));
  return TCW_OK;
}

}  // extern "C"
