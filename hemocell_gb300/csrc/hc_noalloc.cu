// Tile binning without any device allocation: hc_bin_tiles_noalloc.
//
// The handle-based path (HC_STAGE_BIN, hc_read_bins) keeps its per-tile
// counters in memory the handle allocates.  Some callers cannot let a library
// allocate: a host program whose device memory is already carved up by its
// own pool allocator (a cudaMalloc would fail or fragment it), or a coupling
// code on a latency-critical thread that must not pay for cudaMalloc/cudaFree,
// which can synchronise the whole device.  For them this entry point keeps
// its scratch in one fixed array in device global memory, defined below, and
// writes only into the buffers the caller passes in.
//
// The scratch is shared by every call in the process on a given device, so two
// calls whose launches may overlap (two host threads, or two streams with no
// ordering between them) race on it and give wrong lists.  Calls issued one
// after another on one stream, or otherwise ordered, are safe.
#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "hc_dev.h"
#include "hemocell_gb300.h"

namespace hcd {

// Largest tile count the fixed scratch serves: three int counters per tile
// (vertices per tile, fill cursor, cells per tile), 1.5 MiB in all.
constexpr int kNoAllocMaxTiles = 131072;

// The scratch itself.  It is part of the library's device image, so it is
// created when the library's code is loaded on a device, not by any call here.
static __device__ __align__(256) int g_tile_scratch[3 * kNoAllocMaxTiles];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
// Per device: the id of the CUDA context the address was looked up in, and
// the address.  Context ids are never reused within a process, so after a
// cudaDeviceReset (which ends the context and unloads the library's device
// image) the next call sees a new id and looks the address up again.
unsigned long long g_scratch_ctx[kMaxDevices] = {};
int* g_scratch_ptr[kMaxDevices] = {};

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

// The current context's id through the driver entry points the runtime
// hands out (no link against libcuda); 0 when it cannot be had.
unsigned long long current_context_id() {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  static bool looked_up = false;
  if (!looked_up) {
    looked_up = true;
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<CtxGetCurrentFn>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<CtxGetIdFn>(f);
  }
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS)
    return 0;
  return id;
}

// Vertices whose tile lies outside [0, ntiles) are treated as unbinned (the
// handle path marks those with -1), so no counter outside the scratch is hit.
__global__ void k_count_checked(const int* vtile, int nvert, int ntiles, int* counts) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nvert) return;
  const int t = vtile[i];
  if (t >= 0 && t < ntiles) atomicAdd(counts + t, 1);
}

__global__ void k_fill_checked(const int* vtile, int nvert, int ntiles, const int* offsets, int* cursor,
                               int* tile_vertices) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nvert) return;
  const int t = vtile[i];
  if (t < 0 || t >= ntiles) return;
  tile_vertices[offsets[t] + atomicAdd(cursor + t, 1)] = i;
}

// Set-up: the device address of g_tile_scratch for the current device.  In
// host code the array's name stands for a host-side shadow, not for device
// memory, so the address must come from cudaGetSymbolAddress, called with
// the device current.  It is looked up on the first call on each device (that
// call also loads the library's device image there if it is not loaded yet)
// and cached per device and context; a call in a new context of the device
// looks it up again.
int scratch_for_current_device(int** out, std::string& err) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    err = std::string("cudaGetDevice: ") + cudaGetErrorString(e);
    return HC_ERR_CUDA;
  }
  if (dev < 0 || dev >= kMaxDevices) {
    err = "device ordinal beyond the supported range";
    return HC_ERR_INVALID;
  }
  // a thread whose context the runtime has not made current yet reads 0 and
  // takes the lookup, which makes it current
  unsigned long long ctx = current_context_id();
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_ptr[dev] || ctx == 0 || g_scratch_ctx[dev] != ctx) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_tile_scratch);
    if (e != cudaSuccess) {
      err = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
      return HC_ERR_CUDA;
    }
    g_scratch_ptr[dev] = static_cast<int*>(p);
    g_scratch_ctx[dev] = current_context_id();
  }
  *out = g_scratch_ptr[dev];
  return HC_OK;
}

int fail_noalloc(int code, const std::string& msg) {
  set_handleless_error("hc_bin_tiles_noalloc: " + msg);
  return code;
}

}  // namespace
}  // namespace hcd

extern "C" int hc_bin_tiles_noalloc(const int* vertex_tile, const int* vertex_cell, int nvert, int ntiles,
                                    int* tile_offsets, int* tile_vertices, int* tile_cell_offsets,
                                    int* tile_cells, int max_tile_cells, void* stream) {
  using namespace hcd;
  if (ntiles < 1) return fail_noalloc(HC_ERR_INVALID, "ntiles must be at least 1");
  if (ntiles > kNoAllocMaxTiles)
    return fail_noalloc(HC_ERR_INVALID, "ntiles " + std::to_string(ntiles) + " exceeds the fixed maximum of " +
                                            std::to_string(kNoAllocMaxTiles) + " tiles");
  if (nvert < 0 || max_tile_cells < 0) return fail_noalloc(HC_ERR_INVALID, "negative size");
  if (!tile_offsets || !tile_cell_offsets) return fail_noalloc(HC_ERR_INVALID, "null offsets buffer");
  if (nvert > 0 && (!vertex_tile || !vertex_cell || !tile_vertices))
    return fail_noalloc(HC_ERR_INVALID, "null vertex buffer");
  if (max_tile_cells > 0 && !tile_cells) return fail_noalloc(HC_ERR_INVALID, "null tile_cells buffer");

  std::string err;
  int* scratch = nullptr;
  int rc = scratch_for_current_device(&scratch, err);
  if (rc != HC_OK) return fail_noalloc(rc, err);
  int* counts = scratch;
  int* cursor = scratch + kNoAllocMaxTiles;
  int* tile_cell_counts = scratch + 2 * kNoAllocMaxTiles;

  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e;
  // the counters carry the previous call's values: clear the ones this call uses
  if ((e = cudaMemsetAsync(counts, 0, sizeof(int) * ntiles, s)) != cudaSuccess ||
      (e = cudaMemsetAsync(cursor, 0, sizeof(int) * ntiles, s)) != cudaSuccess)
    return fail_noalloc(HC_ERR_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
  const int blocks = (nvert + 255) / 256;
  if (nvert > 0) k_count_checked<<<blocks, 256, 0, s>>>(vertex_tile, nvert, ntiles, counts);
  if ((e = launch_exclusive_scan(counts, ntiles, tile_offsets, s)) != cudaSuccess)
    return fail_noalloc(HC_ERR_CUDA, cudaGetErrorString(e));
  if (nvert > 0) k_fill_checked<<<blocks, 256, 0, s>>>(vertex_tile, nvert, ntiles, tile_offsets, cursor, tile_vertices);
  // tile_cell_counts is written for every tile here, so it needs no clearing
  if ((e = launch_tile_sort(tile_offsets, tile_vertices, vertex_cell, ntiles, tile_cell_counts, s)) != cudaSuccess)
    return fail_noalloc(HC_ERR_CUDA, cudaGetErrorString(e));
  if ((e = launch_tile_cells(tile_offsets, tile_vertices, vertex_cell, ntiles, tile_cell_counts, tile_cell_offsets,
                             tile_cells, max_tile_cells, s)) != cudaSuccess)
    return fail_noalloc(HC_ERR_CUDA, cudaGetErrorString(e));
  return HC_OK;
}
