// Device-side views shared by the kernels (hc_lattice.cu, hc_cells.cu) and
// the C ABI (hc_api.cu).  Arrays in HBM:
//   populations f[19][N]: post-collision values f*_i - w_i of the last
//   collision (T = double or float); readers pull the post-stream values
//   force field, double-buffered (the force of the collision in flight and
//   the next step's force = body force + spreading): float4 per node in
//   FP32, [3][N] in FP64
//   vertex x[3][V] (always double), v[3][V] and force[3][V] (T)
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

namespace hcd {

constexpr uint32_t NB_SOLID = 1u << 23;     // node itself is a wall node
constexpr uint32_t NB_INTERIOR = 1u << 22;  // fluid, no bounce-back link, on no periodic face
constexpr int NB_CLASS_SHIFT = 24;        // wall class of the bounce-back neighbours
constexpr uint32_t NB_CLASS_MIXED = 255;  // neighbours of differing wall class
constexpr int MAX_WALL_CLASSES = 16;
constexpr int MAX_TYPES = 8;

template <typename T>
struct LbmView {
  int nx, ny, nz;
  int per[3];
  long long N;
  const T* __restrict__ fsrc;
  T* __restrict__ fdst;
  const T* __restrict__ Fcur;
  T* __restrict__ Fnext;
  const uint32_t* __restrict__ nbmask;
  const uint8_t* __restrict__ flag;
  const T* __restrict__ bodyz;  // [3][nz]
  uint32_t* ntag;                // per node: stamp of the last step whose stencils touch it; null
                                 // when the node-velocity form in use evaluates every fluid node
                                 // (the spreads then write no tags)
  T* unode;                      // [3][N] velocity of tagged nodes
  uint32_t* stamp;               // device step stamp (advanced by interp_advance)
  int reverse;                   // sweep the lattice from the last z-plane down
  T omega;
  T uw[MAX_WALL_CLASSES][3];
  // 32-bit pull offsets, valid when 19 N < 2^31 (fast != 0): population j of
  // an interior node n (no wrap, no bounce-back link) is fsrc[n + off[j]]
  int fast;
  int off[19];
  unsigned int* status;  // device status word (bit 2: a pipeline wait timed out)
  // the fluid nodes in lattice order, packed x | y << 10 | z << 20 (null when
  // the lattice exceeds 1024 x 1024 x 4096 or 19 N >= 2^31)
  const uint32_t* fluid;
  int nfluid;
  int pdl;  // launch the step's kernels with programmatic dependent launch
  // collide-stream advances the node-tag stamp by one (its first thread): the
  // spread before it was fused into the force assembly, which tags with
  // stamp + 1 so that no CTA of that kernel writes the stamp
  int bump_stamp;
  // variant of the direct collide-stream: bit 0 interior nodes (NB_INTERIOR)
  // pull through the plain offsets, skipping the bounce-back and wrap
  // selects; bit 1 the populations it writes carry an L2 evict-last policy
  int k1var;
  int moving_walls;  // some wall class moves (else the moving-wall term is compiled out)
};

// status bits shared by the kernels and hc_device_status
constexpr unsigned int STATUS_NONFINITE = 1u;
constexpr unsigned int STATUS_CELL_DELETED = 2u;
constexpr unsigned int STATUS_WAIT_TIMEOUT = 4u;
// bounds-checked build only: an index outside its array was caught, and the
// access was skipped (a load reads zero)
constexpr unsigned int STATUS_INDEX_CHECK = 16u;

// The bounds-checked build (-DHC_CHECKED, libhcgpu_checked.so): HC_IN(status,
// i, n) compares index i with its array's length n before the access it
// guards; out of bounds it sets STATUS_INDEX_CHECK and yields false, and the
// caller skips the access, so nothing traps and the host reads the status.
// In the product build HC_IN is the constant true and guards compile away.
__device__ __forceinline__ bool index_ok(unsigned int* status, long long i, long long n) {
  if (i >= 0 && i < n) return true;
  atomicOr(status, STATUS_INDEX_CHECK);
  return false;
}
#ifdef HC_CHECKED
#define HC_IN(status, i, n) (::hcd::index_ok((status), (long long)(i), (long long)(n)))
#else
#define HC_IN(status, i, n) true
#endif

// Launch plan of the bulk-copy collide-stream kernel (k_collide_stream_bulk):
// each CTA owns a slab of R whole x-rows and sweeps a chunk of zlen planes,
// staging the 19 source rows of every plane in shared memory, `stages` planes ahead.
struct BulkPlan {
  int R, nslab, zlen, zchunks, stages;
  int stage_bytes;  // bytes of one stage in shared memory
  int tx_bytes;     // bytes the copies of one stage deliver
  long long spin_limit;
};

// Per-cell-type rest state and lattice-unit constants (device pointers).
struct TypeDev {
  int model, nv, nf, ne, ni;
  const int* tris;        // nf*3
  const int* edges;       // ne*2
  const int* bend_tris;   // ne*2
  const int* bend_outer;  // ne*2
  const int* ring;        // nv*6
  const int* ring_n;      // nv
  const int* inner;       // ni*2
  const int* vface;       // nv*6 per-vertex adjacency (see hc_host.h)
  const int* vedge;       // nv*6
  const int* vopp;        // nv*6
  const int* vinner_off;  // nv+1
  const int* vinner;
  const int* slot_rot;    // nv*6
  const double* slot_a0;  // nv*6
  const double* slot_l0;  // nv*6
  const float* slot_a0f;
  const float* slot_l0f;
  const double* tri_a0;
  const double* edge_l0;
  const double* edge_angle0;
  const double* patch_d0;
  const double* inner_l0;
  const float* tri_a0f;  // FP32 copies for the mixed form
  const float* edge_l0f;
  const float* edge_angle0f;
  const float* patch_d0f;
  const float* inner_l0f;
  double volume_eq, area_mean_eq, edge_mean_eq;
  double k_link, k_bend, k_volume, k_area, eta_m, k_inner_rigid, k_cyto, core_radius, radius;
};

template <typename T>
struct VertexView {
  long long V;        // vertex capacity stride of the SoA arrays
  int nvert;          // vertices in use
  double* x;          // [3][V]
  T* v;               // [3][V]
  T* f;               // [3][V]
  const int* vcell;   // vertex -> cell
  int* alive;         // per cell
  int* vnode;         // per vertex nearest node (or -1)
  int* vtile;         // per vertex tile (or -1)
  unsigned int* status;
  const T* frep_cell;  // [3][V] repulsion added to the spread force (may be null)
  const T* frep_wall;  // [3][V]
};

// Repulsion (applyRepulsionForce / applyBoundaryRepulsionForce,
// core/hemoCellParticleField.cpp:677-743, 891-918): vertices binned per node
// into REP_SLOTS slots (the reference's per-node hemo::Array<unsigned,10>,
// core/hemoCellParticleField.cpp:140); a node holding more sets
// STATUS_REP_OVERFLOW.
constexpr int REP_SLOTS = 10;
constexpr unsigned int STATUS_REP_OVERFLOW = 8u;

template <typename T>
struct RepView {
  int* cnt;              // [N] vertices binned per node (null: no inter-cell term)
  int* slot;             // [N][REP_SLOTS]
  int* vq;               // [V] node of each vertex, -1 when not binned
  T* xr;                 // [3][V] position relative to that node
  const uint8_t* bnode;  // [N] 1 on boundary nodes (wall term)
  T* fcell;              // [3][V] inter-cell term to recompute (null: keep)
  T* fwall;              // [3][V] wall term to recompute (null: keep)
  T kc, rc, kw, rw;      // constants and cutoffs (lattice units)
};

struct TileGrid {
  int tx, ty, tz;     // tile dims
  int ntx, nty, ntz;  // tiles per axis
};

template <typename T>
struct MechView {
  const int* cells;   // cells to process
  int ncells;
  const int* cell_type;
  const int* cell_voff;
  const TypeDev* types;
  VertexView<T> vv;
  int dyn_smem;       // bytes available per CTA
  // fused spread of the next step: the vertex-centric kernel spreads each
  // new vertex force (FORCE_LIMIT-clamped) into L.Fcur and tags the stencil
  // nodes, so the next step needs no spread pass
  int fuse_spread;
  // interpolation and advance fused in front of the force assembly: each CTA
  // interpolates and advances its cell's vertices first (with fuse_spread,
  // which then tags with stamp + 1)
  int fuse_advance;
  TileGrid tg;
  LbmView<T> L;
  T f_limit;
};


// Kernel launch with or without programmatic dependent launch (the kernel
// then starts with pdl_wait, see hc_async.cuh).
template <typename... KArgs, typename... Args>
cudaError_t launch_kernel(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, bool pdl,
                          Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr;
  attr.id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr.val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = &attr;
  cfg.numAttrs = pdl ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, k, args...);
}

// Launch wrappers; each enqueues on `s` and returns the launch error code.
// hc_lattice.cu
template <typename T>
cudaError_t launch_collide_stream(const LbmView<T>& L, int bx, int by, cudaStream_t s);
// bulk-copy variant: false when the lattice does not allow it (nx * sizeof
// row not a multiple of 16 bytes, no row count dividing ny, shared memory)
template <typename T>
bool make_bulk_plan(int nx, int ny, int nz, int stages, int ctas_target, BulkPlan* P);
template <typename T>
size_t bulk_smem_bytes(const BulkPlan& P);
template <typename T>
cudaError_t prepare_collide_bulk(const BulkPlan& P);
template <typename T>
cudaError_t launch_collide_stream_bulk(const LbmView<T>& L, const BulkPlan& P, cudaStream_t s);
template <typename T>
cudaError_t launch_node_velocity(const LbmView<T>& L, cudaStream_t s);
// one increment of the node-tag stamp, in stream order
cudaError_t launch_bump_stamp(uint32_t* stamp, cudaStream_t s);
// the same two kernels with one thread per fluid node (L.fluid)
template <typename T>
cudaError_t launch_collide_stream_fluid(const LbmView<T>& L, int bs, cudaStream_t s);
template <typename T>
cudaError_t launch_node_velocity_fluid(const LbmView<T>& L, cudaStream_t s);
// tagged nodes packed into whole warps (needs L.fast)
template <typename T>
cudaError_t launch_node_velocity_dense(const LbmView<T>& L, cudaStream_t s);
template <typename T>
cudaError_t launch_node_velocity_packed(const LbmView<T>& L, cudaStream_t s);
template <typename T>
cudaError_t launch_moments(const LbmView<T>& L, double* rho, double* u, cudaStream_t s);
template <typename T>
cudaError_t launch_stream_out(const LbmView<T>& L, double* out, cudaStream_t s);
template <typename T>
cudaError_t launch_stream_in(const LbmView<T>& L, const double* in, double rho, const double* u3, cudaStream_t s);
template <typename T>
cudaError_t launch_field_out(const T* F, double* out, long long N, cudaStream_t s);
template <typename T>
cudaError_t launch_field_in(const double* in, T* F, long long N, cudaStream_t s);
template <typename T>
cudaError_t launch_fill_body(T* F, const T* bodyz, long long plane, int nz, long long N, cudaStream_t s);
template <typename T>
cudaError_t launch_add_body(T* F, const T* dz, long long plane, int nz, long long N, cudaStream_t s);
cudaError_t launch_copy_words(void* dst, const void* src, size_t bytes, cudaStream_t s);
template <typename T>
size_t field_bytes(long long N);
template <typename T>
cudaError_t launch_convert_in(const double* src, T* dst, long long n, cudaStream_t s);
// hc_cells.cu
template <typename T>
cudaError_t launch_spread(const LbmView<T>& L, const VertexView<T>& vv, double f_limit, int bs, cudaStream_t s);
template <typename T>
cudaError_t launch_mark_nodes(const LbmView<T>& L, const VertexView<T>& vv, cudaStream_t s);
template <typename T>
cudaError_t launch_add_vertex_forces(const VertexView<T>& vv, const int* ids, const double* fext, int n,
                                     cudaStream_t s);
template <typename T>
cudaError_t launch_interp_advance(const LbmView<T>& L, const VertexView<T>& vv, const TileGrid& tg,
                                  int do_interp, int do_advance, int bs, cudaStream_t s);
// shared memory the staged force assembly (variant 2) needs for one cell type
size_t mechanics_staged_bytes(int model, int nv, int nf, int ne, bool f64);
template <typename T>
cudaError_t launch_mechanics(const MechView<T>& M, int bs, int grid, int variant, cudaStream_t s);
template <typename T>
size_t mechanics_smem_bytes(int nv);
template <typename T>
cudaError_t prepare_mechanics(int smem_bytes);
template <typename T>
cudaError_t launch_soa_to_aos(const T* src, double* dst, long long V, int n, cudaStream_t s);
template <typename T>
cudaError_t launch_bin_vertices(const LbmView<T>& L, const VertexView<T>& vv, const TileGrid& tg, cudaStream_t s);
template <typename T>
cudaError_t launch_cell_info(const VertexView<T>& vv, const int* cell_type, const int* cell_voff, const TypeDev* types,
                             int ncells, double* out, cudaStream_t s);
template <typename T>
cudaError_t launch_repulsion(const LbmView<T>& L, const VertexView<T>& vv, const RepView<T>& R, cudaStream_t s);
// binning: tile CSR sorted by (tile, cell, vertex)
cudaError_t launch_bin_csr(const int* vtile, int nvert, int ntiles, int* counts, int* offsets, int* cursor,
                           int* tile_vertices, const int* vcell, int* tile_cell_counts, cudaStream_t s);
cudaError_t launch_tile_cells(const int* offsets, const int* tile_vertices, const int* vcell, int ntiles,
                              int* tile_cell_counts, int* tile_cell_offsets, int* tile_cells, int max_cells,
                              cudaStream_t s);
// the two middle steps of the tile CSR on their own: out[0..n] = exclusive
// scan of in[0..n-1]; per-tile sort of tile_vertices and distinct cells per tile
cudaError_t launch_exclusive_scan(const int* in, int n, int* out, cudaStream_t s);
// per tile, the ascending distinct cells of the tile and its 26 neighbours:
// counts (offsets null) or the cells at offsets (counts unused)
cudaError_t launch_tile_neighbours(const TileGrid& tg, const int per[3], const int* tile_cell_offsets,
                                   const int* tile_cells, int ntiles, int* counts, const int* offsets, int* cells,
                                   cudaStream_t s);
cudaError_t launch_tile_sort(const int* offsets, int* tile_vertices, const int* vcell, int ntiles,
                             int* tile_cell_counts, cudaStream_t s);

// message returned by hc_last_error(NULL) for calls that take no handle
void set_handleless_error(const std::string& msg);

}  // namespace hcd

struct hc_handle;
namespace hcd {
// what the serving batch needs to know of a handle
cudaStream_t handle_stream(const hc_handle* h);
int handle_device(const hc_handle* h);
long long handle_bytes(const hc_handle* h);

}  // namespace hcd
