// Plain per-template map for callers that cannot allocate device memory.
//
// Some host programs may not call cudaMalloc at all: code running inside a
// memory-pool-managed framework that forbids raw device allocations, code
// that must not synchronise the device (cudaMalloc/cudaFree can), or
// real-time loops that pre-budget every byte at start-up.  They still need
// scratch memory for the map: the compensated prefix rows (rectangular
// window) or the 32-byte atom rows (exponential window), the tile list, the
// per-tile partial reductions and the posterior sums.  This file gives them
// tcw_map_plain_noalloc(): the caller passes inputs and outputs as device
// pointers and a stream; the scratch lives in one file-scope device array
// of kNoallocScratchBytes that every GPU loading the library holds until the
// process exits.  The entry point makes no cudaMalloc / cudaFree call and
// uses no allocating library routine.
//
// Set-up: the first call on a device looks up the device address of the
// array (cudaGetSymbolAddress, with that device current) and caches it per
// device ordinal; make that first call before any stream capture.  The
// cached address belongs to the runtime's primary context of that device:
// after cudaDeviceReset of the device, or with another context made current
// on it through the driver API, the array may live elsewhere and the cached
// address is stale -- this entry point is for processes that keep the
// primary context for their lifetime.  All calls on a
// device share the array and it keeps the last call's contents, so calls
// whose work overlaps on the GPU (different streams, or threads racing to the
// same stream) corrupt each other's scratch: serialise them.  Everything a
// call reads from the array it has written earlier in the same call (tile
// list and descriptor by a set-up kernel, prefix or atom rows, partials), so
// no clearing is needed between calls.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/tcw_b200.h"
#include "tcw_internal.h"

using namespace tcw;

namespace {

constexpr size_t kNoallocScratchBytes = TCW_NOALLOC_SCRATCH_BYTES;
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

std::mutex g_scratch_mu;
void *g_scratch_ptr[kMaxDevices] = {nullptr};

// Device address of the scratch array on the current device (cached).
int scratch_address(int device, unsigned char **out) {
  if (device < 0 || device >= kMaxDevices) return TCW_ERR_NO_DEVICE;
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_ptr[device]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      return TCW_ERR_CUDA;
    }
    g_scratch_ptr[device] = p;
  }
  *out = static_cast<unsigned char *>(g_scratch_ptr[device]);
  return TCW_OK;
}

size_t align256(size_t x) { return (x + 255u) / 256u * 256u; }

// Writes the template descriptor, the one-entry template list and the tile
// list into the scratch array (so nothing is copied from the host).  Tiles
// are enumerated column tile outer, row tile inner, as the handle-based
// entry point does.
__global__ void noalloc_setup_kernel(TemplateDev t, uint32_t window, uint32_t tn,
                                     uint32_t rows_per_tile, uint32_t rows_per_lane,
                                     uint32_t n_mtiles, uint32_t n_items, TemplateDev *T,
                                     uint32_t *list, WorkItem *items) {
  const uint32_t i0 = blockIdx.x * blockDim.x + threadIdx.x;
  if (i0 == 0) {
    T[0] = t;
    list[0] = 0;
  }
  for (uint32_t k = i0; k < n_items; k += gridDim.x * blockDim.x) {
    const uint32_t nt = k / n_mtiles, mt = k % n_mtiles;
    WorkItem w{};
    w.tmpl = 0;
    w.part = k;
    w.m0 = mt * rows_per_tile;
    w.m1 = min(t.N_t0, w.m0 + rows_per_tile);
    w.n0 = nt * tn;
    w.n1 = min(t.N_tau, w.n0 + tn);
    if (window == TCW_WINDOW_RECT) {
      w.tn = (uint16_t)(rows_per_tile / 32u);
      w.rows_per_lane = 0;
    } else {
      w.tn = (uint16_t)tn;
      w.rows_per_lane = (uint16_t)rows_per_lane;
    }
    items[k] = w;
  }
}

}  // namespace

extern "C" int tcw_map_plain_noalloc(void *stream, const float *d_atoms, uint32_t numAtoms,
                                     uint32_t TAtom, uint32_t t0_data, int window,
                                     const uint32_t *d_t0s, uint32_t N_t0,
                                     const uint32_t *d_taus, uint32_t N_tau, float *d_Fmn,
                                     tcw_result *d_result, int flags) {
  if (!d_atoms || !d_t0s || !d_taus || !d_result) return TCW_ERR_INVALID_ARG;
  if (window != TCW_WINDOW_RECT && window != TCW_WINDOW_EXP) return TCW_ERR_INVALID_ARG;
  if (numAtoms == 0 || TAtom == 0 || N_t0 == 0 || N_tau == 0) return TCW_ERR_INVALID_ARG;
  if ((uint64_t)t0_data + (uint64_t)numAtoms * TAtom > 0xFFFFFFFFull) return TCW_ERR_OVERFLOW;
  const bool post = (flags & TCW_FLAG_POSTERIORS) != 0;
  if (post && !d_Fmn) return TCW_ERR_INVALID_ARG;
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess) {
    cudaGetLastError();
    return TCW_ERR_NO_DEVICE;
  }
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) {
    cudaGetLastError();
    return TCW_ERR_NO_DEVICE;
  }

  // tile shapes: the same rules as the handle-based plain entry point
  uint32_t tn, rows_per_tile, rows_per_lane = 0;
  const uint64_t target_blocks = (uint64_t)sms * 4u;
  if (window == TCW_WINDOW_RECT) {
    rows_per_tile = 32;
    const uint64_t row_tiles = (N_t0 + 31u) / 32u;
    uint64_t c = (uint64_t)N_tau * row_tiles / (target_blocks ? target_blocks : 1);
    tn = (uint32_t)(c < 16 ? 16 : (c > 256 ? 256 : c));
  } else {
    tn = 32;
    uint32_t rows = (N_t0 + 15u) / 16u;
    rows = rows < 8u ? 8u : rows;
    rows_per_lane = rows < N_t0 ? rows : N_t0;
    // a lane's row chunk is a 16-bit count: longer columns become more row
    // tiles, as in the handle-based entry point
    if (rows_per_lane > 65535u) rows_per_lane = 65535u;
    rows_per_tile = rows_per_lane * (kBlock / tn);
  }
  const uint64_t n_mtiles = (N_t0 + rows_per_tile - 1u) / rows_per_tile;
  const uint64_t n_ntiles = (N_tau + tn - 1u) / tn;
  const uint64_t n_items64 = n_mtiles * n_ntiles;
  if (n_items64 > 0x7FFFFFFFull) return TCW_ERR_OVERFLOW;
  const uint32_t n_items = (uint32_t)n_items64;
  const uint32_t n_chunks = (N_t0 + 63u) / 64u;

  // scratch layout
  size_t off = 0;
  const size_t o_T = off;
  off = align256(off + sizeof(TemplateDev));
  const size_t o_list = off;
  off = align256(off + sizeof(uint32_t));
  const size_t o_items = off;
  off = align256(off + sizeof(WorkItem) * (size_t)n_items);
  const size_t o_parts = off;
  off = align256(off + sizeof(Partial) * (size_t)n_items);
  const size_t o_rows = off;
  off = align256(off + (window == TCW_WINDOW_RECT
                            ? sizeof(float) * kPrefixStride * ((size_t)numAtoms + 1u)
                            : sizeof(float) * 8u * (size_t)numAtoms));
  const size_t o_row = off;
  if (post) off = align256(off + sizeof(double) * N_t0);
  const size_t o_col = off;
  if (post) off = align256(off + sizeof(double) * (size_t)n_chunks * N_tau);
  if (off > kNoallocScratchBytes) return TCW_ERR_OVERFLOW;

  unsigned char *base = nullptr;
  int rc = scratch_address(device, &base);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);

  TemplateDev t{};
  t.g = make_geom(numAtoms, TAtom, t0_data);
  t.window = (uint32_t)window;
  t.N_t0 = N_t0;
  t.N_tau = N_tau;
  t.part_off = 0;
  t.n_parts = n_items;
  TemplateDev *dT = reinterpret_cast<TemplateDev *>(base + o_T);
  uint32_t *dlist = reinterpret_cast<uint32_t *>(base + o_list);
  WorkItem *ditems = reinterpret_cast<WorkItem *>(base + o_items);
  Partial *dparts = reinterpret_cast<Partial *>(base + o_parts);
  float *drows = reinterpret_cast<float *>(base + o_rows);

  const uint32_t setup_blocks = n_items / 256u + 1u < 1024u ? n_items / 256u + 1u : 1024u;
  noalloc_setup_kernel<<<setup_blocks, 256, 0, s>>>(t, (uint32_t)window, tn, rows_per_tile,
                                                    rows_per_lane, (uint32_t)n_mtiles, n_items,
                                                    dT, dlist, ditems);
  if (cudaGetLastError() != cudaSuccess) return TCW_ERR_CUDA;
  const int prec = (flags & TCW_FLAG_UNCOMPENSATED) ? kPrecPlain32
                   : (flags & TCW_FLAG_FP64_DET)    ? kPrecFF_F64Det
                                                    : kPrecFF;
  cudaError_t e = window == TCW_WINDOW_RECT
                      ? launch_prefix(dT, dlist, 1, d_atoms, drows, prec, s)
                      : launch_repack(dT, dlist, 1, d_atoms, drows, s);
  if (e != cudaSuccess) return TCW_ERR_CUDA;
  MapLaunch ml{};
  ml.T = dT;
  ml.items = ditems;
  ml.n_items = n_items;
  ml.persistent = false;
  ml.write_map = d_Fmn != nullptr;
  ml.prec = prec;
  ml.priority = 0;
  ml.atoms = d_atoms;
  ml.atoms8 = window == TCW_WINDOW_EXP ? drows : nullptr;
  ml.t0s = d_t0s;
  ml.taus = d_taus;
  ml.P = window == TCW_WINDOW_RECT ? drows : nullptr;
  ml.Fmn = d_Fmn;
  ml.parts = dparts;
  if (launch_map(window, ml, s) != cudaSuccess) return TCW_ERR_CUDA;
  if (launch_finalize(dT, 1, dparts, d_result, s) != cudaSuccess) return TCW_ERR_CUDA;
  if (post && launch_posteriors(dT, d_Fmn, d_result, reinterpret_cast<double *>(base + o_row),
                                reinterpret_cast<double *>(base + o_col), N_t0, N_tau,
                                s) != cudaSuccess)
    return TCW_ERR_CUDA;
  return TCW_OK;
}

namespace tcw {
// Failed debug checks of this file's kernels (0 unless built with TCW_DEBUG_CHECKS).
unsigned int dcheck_failures_noalloc() {
#if defined(TCW_DEBUG_CHECKS)
  return tcw_dcheck_read();
#else
  return 0;
#endif
}
}  // namespace tcw
