/*
 * hemocell_gb300 — C ABI of the GB300-native HemoCell IB-LBM time step.
 *
 * One handle (hc_handle) is one HemoCell instance: a D3Q19 lattice, its
 * cell types and cells, all resident on one GPU.  Device memory is owned by
 * the handle; host pointers passed in are borrowed for the call only.  No C++
 * exception crosses this boundary: every call returns HC_OK (0) or a negative
 * HC_ERR_* code, and hc_last_error(h) describes the last failure (like the
 * reference's hlog message + exit(1), minus the exit).  A handle is
 * thread-compatible: do not use one handle from two host threads at once.
 *
 * Each entry point names the reference interface it replaces (paths relative
 * to the HemoCell source tree).
 */
#ifndef HEMOCELL_GB300_H
#define HEMOCELL_GB300_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HC_OK 0
#define HC_ERR_INVALID (-1)   /* bad argument (config/config.cpp:80-87 throws here) */
#define HC_ERR_CUDA (-2)      /* CUDA runtime failure */
#define HC_ERR_MEMORY (-3)    /* device memory exhausted / admission refused */
#define HC_ERR_STATE (-4)     /* call not valid in the current state */
#define HC_ERR_NUMERIC (-5)   /* NaN / non-finite state detected */

/* precision forms */
#define HC_FORM_PLAIN_F64 0   /* everything FP64 */
#define HC_FORM_MIXED_F32 1   /* FP32 f_i - w_i populations, FP32 forces; FP64 positions,
                                 per-cell volume sums and area/volume constraint terms */
/* launch modes */
#define HC_LAUNCH_PER_STAGE 0 /* one kernel per stage and per cell type */
#define HC_LAUNCH_BATCHED 1   /* one launch per stage across cell types; step captured
                                 as a CUDA graph */

/* constitutive models (the Mechanics template argument of addCellType) */
#define HC_MODEL_RBC_HIGH_ORDER 0 /* mechanics/rbcHighOrderModel.cpp */
#define HC_MODEL_PLT_SIMPLE 1     /* mechanics/pltSimpleModel.cpp */
#define HC_MODEL_WBC_HIGH_ORDER 2 /* mechanics/wbcHighOrderModel.cpp */

/* body-force modes (the driver's setExternalVector after iterate()) */
#define HC_BODY_NONE 0
#define HC_BODY_UNIFORM 1     /* p[0..2] */
#define HC_BODY_KOLMOGOROV 2  /* F_x = p[0] * sin(2 pi z / nz) */

/* stages of HemoCell::iterate (core/hemoCell.cpp:299-376) */
#define HC_STAGE_SPREAD 0         /* spreadParticleForce */
#define HC_STAGE_COLLIDE_STREAM 1 /* lattice->collideAndStream + force reset */
#define HC_STAGE_INTERPOLATE 2    /* interpolateFluidVelocity */
#define HC_STAGE_ADVANCE 3        /* advanceParticles (+ binning of each vertex) */
#define HC_STAGE_MECHANICS 4      /* applyConstitutiveModel (due types) */
#define HC_STAGE_MECHANICS_FORCED 5 /* applyConstitutiveModel(forced=true) */
#define HC_STAGE_BIN 6            /* tile CSR + per-tile cell lists */
#define HC_STAGE_REPULSION 7      /* applyRepulsionForce + applyBoundaryRepulsionForce */

typedef struct hc_handle hc_handle;

/* Simulation parameters: the <domain> block of config.xml plus the lattice
 * the case program builds (examples/oneCellShear/oneCellShear.cpp:50-67). */
typedef struct hc_params {
  int nx, ny, nz;
  int periodic[3];
  double dx, dt;        /* [m], [s] */
  double nu_p, rho_p;   /* [m^2/s], [kg/m^3] */
  double kBT_p;         /* [J] */
  double tau;           /* > 0: fixes tau; <= 0: tau = 3 nu_p dt / dx^2 + 1/2 */
  int form;             /* HC_FORM_* */
  int launch;           /* HC_LAUNCH_* */
  int device;           /* CUDA device ordinal */
  int tile[3];          /* binning tile (0 => 8) */
} hc_params;

/* MaterialModel block of <celltype>.xml, SI units
 * (examples/oneCellShear/RBC.xml, examples/cell_shapes/WBC_HO.xml). */
typedef struct hc_material {
  double kLink, kBend, kVolume, kArea, eta_m;
  double kInnerRigid, kCytoskeleton, coreRadius, radius;
} hc_material;

typedef struct hc_stats {
  long long nodes;
  int vertices, cells, cells_alive, types;
  int iter;
  double tau, omega;
  long long device_bytes;
} hc_stats;

/* --- lifecycle: HemoCell::HemoCell / ~HemoCell (core/hemoCell.cpp:69-127) */
hc_handle* hc_create(const hc_params* p);
int hc_destroy(hc_handle* h);
const char* hc_last_error(const hc_handle* h); /* h may be NULL: last failure of a call
                                                  without a handle (hc_create,
                                                  hc_bin_tiles_noalloc,
                                                  hc_stl_voxelize) */
/* Parameters::lbm_base_parameters (mechanics/constantConversion.cpp:36-59):
 * out = {tau, nu_lbm, dm, df, kBT_lbm, f_limit} */
int hc_derived_units(const hc_handle* h, double* out6);

/* --- lattice set-up (boundary flags helper/genericFunctions.cpp:138-159,
 * shear walls helper/hemocellInit.hh:58-92, body force
 * examples/pipeflow/pipeflow.cpp:141-146, lattice.initialize()) */
int hc_set_flags(hc_handle* h, const uint8_t* flags); /* per node: 0 fluid, k>0 wall class k */
int hc_set_wall_velocity(hc_handle* h, int cls, const double* u3);
/* setExternalVector: the per-plane profile (3 x nz values of the form's
 * type) is copied to the device from a pinned staging buffer on every call;
 * the same force again changes nothing else, a changed one is added to the
 * next step's force field (which keeps a spread already fused into it) */
int hc_set_body_force(hc_handle* h, int mode, const double* p);
int hc_init_equilibrium(hc_handle* h, double rho, const double* u3);

/* --- cell types: HemoCell::addCellType<Mechanics>(name, shape)
 * (hemocell.h:122-127; CommonCellConstants mechanics/commonCellConstants.cpp:70-409).
 * template_xyz: nv*3 lattice-unit vertices of the rest shape; tris nf*3
 * outward-oriented; inner nI*2 (InnerEdges).  Returns the type id (>= 0). */
int hc_add_cell_type(hc_handle* h, const char* name, int model, const hc_material* m,
                     const double* template_xyz, int nv, const int* tris, int nf,
                     const int* inner_edges, int ni);
/* HemoCell::loadParticles (io/readPositionsBloodCells.cpp:290-361): place n
 * cells of a type, centred on their bounding box, rotated by
 * rotateTriangularMeshXYZ(angles in rad) and translated to centres (lattice
 * units).  Returns the first new cell id. */
int hc_add_cells(hc_handle* h, int type, int n, const double* centres, const double* angles);
/* HemoCell::loadParticles with its admission of cells
 * (io/readPositionsBloodCells.cpp:120-170, 354): places n cells as
 * hc_add_cells does, but adds only the cells all of whose vertices the
 * reference adds -- inside the lattice's box on every axis (periodic axes are
 * not wrapped at loading) and with a nearest node int(x + 0.5) that is not a
 * wall node; the other cells are left out, as deleteIncompleteCells removes
 * them.
 * loaded[n] (may be NULL) receives 1 for each cell added.  Returns the number
 * of cells added (>= 0) or an HC_ERR_* code. */
int hc_load_cells(hc_handle* h, int type, int n, const double* centres, const double* angles, int* loaded);
/* place n cells from explicit vertex positions (n*nv*3, lattice units) */
int hc_add_cells_xyz(hc_handle* h, int type, int n, const double* xyz);
/* setMaterialTimeScaleSeparation / setParticleVelocityUpdateTimeScaleSeparation
 * (hemocell.h:150,159; checked as in core/hemoCell.cpp:620-627) */
int hc_set_timescales(hc_handle* h, const int* material_every, int ntypes, int velocity_every);

/* HemoCellStretch::applyForce (helper/hemoCellStretch.cpp:63-78): a constant
 * external force added to the listed vertices' force before every spread
 * (ids are global vertex indices, forces n*3 in lattice units); n = 0 clears */
int hc_set_vertex_forces(hc_handle* h, int n, const int* ids, const double* forces);

/* HemoCell::setRepulsion (core/hemoCell.cpp:420-426): vertices of different
 * cells closer than `cutoff` (lattice units; the reference takes micrometres
 * and multiplies by 1e-6/dx) repel with k * cutoff / d, recomputed every
 * `every` steps (0 disables); applied with the spread like the reference's
 * force_repulsion (core/hemoCellParticleField.cpp:677-743, :857-859) */
int hc_set_repulsion(hc_handle* h, double k, double cutoff, int every);
/* HemoCell::enableBoundaryParticles (core/hemoCell.cpp:428-436): the same
 * push from wall nodes next to fluid (core/hemoCellParticleField.cpp:865-918) */
int hc_set_boundary_repulsion(hc_handle* h, double k, double cutoff, int every);
/* force_repulsion of every vertex, [V][3] */
int hc_read_repulsion(hc_handle* h, double* f);

/* --- the hot path: HemoCell::iterate() (core/hemoCell.cpp:299-376) */
int hc_step(hc_handle* h, int nsteps);
int hc_stage(hc_handle* h, int stage); /* one stage, for stage-wise parity */
int hc_sync(hc_handle* h);

/* timing with CUDA events recorded on the handle's stream (the stream every
 * kernel of the step is launched on): hc_time_steps runs nsteps exactly as
 * hc_step and returns the elapsed device time; hc_profile_stages runs nsteps
 * with an event between stages (no graph) and returns the mean per step of
 * {spread, collide_stream, interpolate+advance, mechanics, whole step} in ms */
int hc_time_steps(hc_handle* h, int nsteps, double* ms);
int hc_profile_stages(hc_handle* h, int nsteps, double* ms5);
/* per-kernel device time inside the step as hc_step runs it in the batched
 * launch (same kernels and fusions as its CUDA graph, launched without the
 * graph and queued ahead so that no launch gap is timed): 3 unprofiled steps,
 * then nsteps (1..100000) profiled; ms4 = mean per step of {collide-stream,
 * node velocity (interpolation + advance when they are not fused),
 * force assembly, whole step} */
int hc_profile_kernels(hc_handle* h, int nsteps, double* ms4);

/* --- readback (io/FluidHdf5IO.hh velocity/density, io/ParticleHdf5IO.cpp) */
int hc_read_fluid(hc_handle* h, double* rho, double* u);        /* rho[N], u[3][N] */
int hc_read_populations(hc_handle* h, double* f);              /* f[19][N], unshifted */
int hc_write_populations(hc_handle* h, const double* f);
int hc_read_force_field(hc_handle* h, double* F, int which);   /* 0 next, 1 last collision */
int hc_write_force_field(hc_handle* h, const double* F);       /* sets the next force field */
int hc_read_vertices(hc_handle* h, double* x, double* v, double* f); /* [V][3] each, may be NULL */
int hc_write_vertices(hc_handle* h, const double* x, const double* v, const double* f);
/* positions [V][3] copied to the host after the work queued so far, without
 * waiting: a kernel gathers them into device staging buffer `slot` (0 or 1)
 * on the handle's stream and a copy stream moves them into x (pinned host
 * memory, untouched until hc_wait_positions(slot) returns), so the next
 * steps run during the copy; a slot is reused only after its last copy */
int hc_read_positions_async(hc_handle* h, double* x, int slot);
int hc_wait_positions(hc_handle* h, int slot);
int hc_read_cells(hc_handle* h, int* alive, double* volume);
/* update_pg / ownership / neighbour lists (core/hemoCellParticleField.cpp:137-168):
 * vertex_node[V], vertex_tile[V], tile_offsets[ntiles+1], tile_vertices[V],
 * tile_cell_offsets[ntiles+1], tile_cells[max_tile_cells].  Returns ntiles. */
int hc_read_bins(hc_handle* h, int* vertex_node, int* vertex_tile, int* tile_offsets,
                 int* tile_vertices, int* tile_cell_offsets, int* tile_cells, int max_tile_cells);
/* Neighbour lists (block neighbours, core/hemoCellFields.cpp:230-236, on one
 * lattice: the tiles within the kernel halo): for every tile, the ascending
 * distinct cell ids with vertices in the tile or in one of its 26 neighbouring
 * tiles, wrapped on periodic axes.  nb_offsets[ntiles+1] (CSR), nb_cells
 * [max_cells].  Bins the current positions first.  Returns ntiles. */
int hc_read_neighbours(hc_handle* h, int* nb_offsets, int* nb_cells, int max_cells);
/* Tile binning that allocates no device memory.  No counterpart in the
 * reference: it exists for callers that must not have a library allocate on
 * their behalf -- a program whose device memory is already carved up by its
 * own pool allocator, or host code on a latency-critical thread that cannot
 * pay for cudaMalloc/cudaFree, which may synchronise the device.  It builds
 * the same lists as hc_read_bins from device-resident inputs, without a handle.
 *
 * All pointers are DEVICE pointers on the current device; work is enqueued on
 * `stream` (a cudaStream_t, NULL for the default stream) and the call returns
 * without waiting for it.  Inputs: vertex_tile[nvert] (tile of each vertex,
 * -1 or any value outside [0, ntiles) = not binned), vertex_cell[nvert].
 * Outputs: tile_offsets[ntiles+1], tile_vertices[nvert] (ascending within a
 * tile), tile_cell_offsets[ntiles+1], tile_cells[max_tile_cells] (cells per
 * tile in ascending order; if tile_cell_offsets[ntiles] > max_tile_cells the
 * list is cut at max_tile_cells).
 *
 * Limit: ntiles <= 131072; larger requests return HC_ERR_INVALID with the
 * reason in hc_last_error(NULL).  The per-tile counters live in one fixed
 * 1.5 MiB array in the library's device memory, shared by every call on a
 * device: calls that may run concurrently (two host threads, or unordered
 * streams) race on it and give wrong lists; calls ordered on one stream are
 * safe.  The first call on each device looks up that array's address (with
 * the device current), which may make the CUDA runtime load the library's
 * device code; make that first call before capturing any stream.  The
 * address is kept per device and CUDA context: after a cudaDeviceReset the
 * next call looks it up again, so a reset leaves no stale address behind.
 * A tile of any size is sorted (up to 2048 vertices in shared memory, beyond
 * that in place by a block-wide sorting network). */
int hc_bin_tiles_noalloc(const int* vertex_tile, const int* vertex_cell, int nvert, int ntiles,
                         int* tile_offsets, int* tile_vertices, int* tile_cell_offsets, int* tile_cells,
                         int max_tile_cells, void* stream);
/* CellInformationFunctionals::calculateCellInformation (helper/cellInfo.cpp:170-266):
 * 16 doubles per cell: centroid (inside the lattice on periodic axes), mean
 * velocity, membrane area, volume, largest distance between two of its
 * vertices (stretch), bounding box (xmin, xmax, ymin, ymax, zmin, zmax) and
 * its type (-1 once deleted); lattice units */
int hc_cell_info(hc_handle* h, double* out);
/* writeCellInfo_CSV (io/writeCellInfoCSV.cpp:30-74): <dir>/<type name>.<iteration
 * as 12 digits>.csv for every cell type with the reference's columns
 * X,Y,Z,area,volume,atomic_block,cellId,baseCellId,velocity_x,velocity_y,velocity_z;
 * si = 1 converts to SI units with dx and dt (outputInSiUnits) */
int hc_write_cell_info_csv(hc_handle* h, const char* dir, int si);
/* HemoCell::writeOutput (core/hemoCell.cpp:221-280) with the content of
 * io/FluidHdf5IO.hh and io/ParticleHdf5IO.cpp, as XDMF descriptors over raw
 * little-endian arrays (HDF5 is not used): <dir>/hdf5/Fluid.<iteration>.xmf
 * with Velocity, Density and Force on the nodes, and <dir>/hdf5/<type>.<iteration>.xmf
 * per cell type with the live cells' Position, Triangles, Velocity,
 * Total force (membrane + repulsion) and Cell Id; si = 1 writes SI units */
int hc_write_output(hc_handle* h, const char* dir, int si);
/* HemoCell::saveCheckPoint (core/hemoCell.cpp:210-219, core/hemoCellFields.cpp:276-319):
 * <dir>/checkpoint.xml (iteration), <dir>/lattice.dat (flags, wall velocities,
 * body force, post-collision populations, force fields) and
 * <dir>/particleField.dat (cells, positions, velocities, forces, repulsion);
 * an existing set is renamed to *.old first */
int hc_save_checkpoint(hc_handle* h, const char* dir);
/* HemoCell::loadCheckPoint (core/hemoCell.cpp:199-208): restores into a handle
 * created with the same lattice size, form and cell types; a handle without
 * cells receives the checkpoint's cells, one with cells must hold the same */
int hc_load_checkpoint(hc_handle* h, const char* dir);
int hc_get_stats(hc_handle* h, hc_stats* out);  /* waits for the handle's stream (alive cells) */
int hc_vertex_count(const hc_handle* h);         /* vertices in use; does not wait */
/* device status word, sticky: bit0 non-finite vertex velocity, bit1 cell
 * deleted at a wall, bit2 a shared-memory pipeline wait of the bulk-copy
 * collide-stream timed out (the step's results are then invalid and the
 * handle must be destroyed: copies may still have been in flight), bit3 a
 * lattice node held more repulsion candidates than its slots (pairs were
 * dropped), bit4 (bounds-checked build libhcgpu_checked.so only) an index
 * outside its array was caught and the access skipped */
int hc_device_status(hc_handle* h, unsigned int* status);

/* --- launch tuning (project autotuner; results cached on disk) */
int hc_autotune(hc_handle* h, const char* cache_path);
int hc_get_tuning(hc_handle* h, int* out8);
/* in8: collide-stream block (bx, by; bx = 0 whole rows, else 8 or 16, whose
 * warps are 8 x 4 or 16 x 2 tiles, or a multiple of 32; whole warps, at most
 * 256 threads), spread block,
 * interpolation block, mechanics block, mechanics grid (0 = one CTA per cell),
 * mechanics variant (0 vertex gather, 1 face/edge scatter, 2 staged face/edge
 * terms gathered per vertex), and in8[7]: bits 0-7 the collide-stream kind
 * (0 (x,y)-blocks or rows, 1 one thread per fluid node, else bulk copies:
 * stages | CTAs per SM << 4), bits 8-9 the node velocity (0 every tagged node,
 * 1 per fluid node, 2 over warp-packed tagged nodes, 3 every fluid node in
 * whole coalesced warps), bit 10 programmatic dependent launch
 * of the step's kernels, bit 11 keeps interpolation + advance a kernel of
 * their own in the batched step (by default the force assembly does them),
 * and variants of the direct (x,y)-block and fluid-node collide-stream:
 * bit 12 interior nodes (no bounce-back link, on no periodic face) pull
 * through plain offsets, bit 13 the populations it writes carry an L2
 * evict-last policy */
int hc_set_tuning(hc_handle* h, const int* in8);

/* --- mesh helpers (helper/meshGeneratingFunctions.hh:31-271).  Buffers are
 * caller-owned; sizes are checked against max_nv / max_nf. */
/* getFlagMatrixFromSTL (helper/voxelizeDomain.cpp:74-152): reads a binary or
 * ASCII STL surface, scales it to span ref_length lattice units along axis
 * ref_dir (0 x, 1 y, 2 z), places it `margin` nodes into the lattice and marks
 * nodes inside the closed surface fluid (0), the rest wall (1); open_ends
 * opens both x ends of a closed tube by copying the slices next to them.
 * dims3 receives the lattice size; flags (x fastest, may be NULL to query
 * the size) must hold max_nodes >= dims3[0]*dims3[1]*dims3[2] bytes.  Errors
 * are described by hc_last_error(NULL). */
int hc_stl_voxelize(const char* path, int ref_dir, double ref_length, int margin, int open_ends, int* dims3,
                    uint8_t* flags, long long max_nodes);
/* icosphere refined until nf >= min_triangles (constructSphereIcosahedron) */
int hc_mesh_icosphere(int min_triangles, double radius, double* xyz, int max_nv, int* tris,
                      int max_nf, int* nv, int* nf);
/* RBC_FROM_SPHERE: Evans-Fung biconcave map of the icosphere, radius in lattice units */
int hc_mesh_rbc(int min_triangles, double radius, double* xyz, int max_nv, int* tris, int max_nf,
                int* nv, int* nf);
/* ELLIPSOID_FROM_SPHERE: x,y scaled by radius, z by aspect*radius */
int hc_mesh_ellipsoid(int min_triangles, double radius, double aspect, double* xyz, int max_nv,
                      int* tris, int max_nf, int* nv, int* nf);
/* antipodal vertex pairs of a centrally symmetric mesh (inner edges) */
int hc_mesh_antipodal_pairs(const double* xyz, int nv, int* pairs, int max_pairs);
/* host-only placement used by hc_add_cells: n cells of one rest shape,
 * centred on the bounding box, rotated (rotateTriangularMeshXYZ, angles in
 * rad) and translated; out_xyz holds n*nv*3 doubles */
int hc_place_cells(const double* template_xyz, int nv, int n, const double* centres, const double* angles,
                   double* out_xyz);
/* seeded non-overlapping packing of cells (stands in for the reference's packCells tool):
 * type_xyz/type_nv/type_tris/type_nf describe ntypes rest shapes, counts[t]
 * cells per type; solid[N] marks forbidden nodes (may be NULL); margin in
 * lattice units.  Writes centres[total*3], angles[total*3], types[total];
 * returns the number of cells placed. */
int hc_pack_cells(int nx, int ny, int nz, const int* periodic, const uint8_t* solid, int ntypes,
                  const double* const* type_xyz, const int* type_nv, const int* const* type_tris,
                  const int* type_nf, const int* counts, double margin, unsigned long long seed,
                  int max_attempts, double* centres, double* angles, int* types);

/* --- serving: continuous batching of independent solves on one device.
 * No counterpart in the reference (one simulation per MPI job).  A batch owns
 * the handles admitted to it and steps them together: each solve keeps its own
 * lattice, meshes and stream, and hc_batch_pump keeps every stream fed with
 * chunks of `chunk_steps` steps (hc_step, graph replays in the batched launch
 * mode), so the work of all resident solves overlaps on the device.  A batch is
 * thread-compatible like a handle. */
typedef struct hc_batch hc_batch;
typedef struct hc_batch_stats {
  int active, finished, popped, max_slots;
  long long budget_bytes, bytes_in_use;
  long long admitted, completed, refused, steps_enqueued;
} hc_batch_stats;

/* upper bound of the device bytes a handle with these parameters, vertices
 * and cells holds, including the staging of hc_read_fluid, hc_read_vertices
 * and hc_read_bins (not hc_read_populations); no device call */
long long hc_estimate_device_bytes(const hc_params* p, int nvertices, int ncells);
/* budget_bytes: device bytes the resident solves may hold (their handles'
 * hc_stats.device_bytes); max_slots: resident solves at most */
hc_batch* hc_batch_create(int device, long long budget_bytes, int max_slots, int chunk_steps);
int hc_batch_destroy(hc_batch* b);              /* destroys every handle it still holds */
const char* hc_batch_last_error(const hc_batch* b);
/* 1 if a solve of `bytes` would be admitted now, else 0 */
int hc_batch_fits(const hc_batch* b, long long bytes);
/* admit a set-up handle for nsteps more steps; on HC_OK the batch owns it,
 * on HC_ERR_MEMORY (over budget or no slot) the caller keeps it */
int hc_batch_admit(hc_batch* b, hc_handle* h, int nsteps, long long tag);
/* enqueue work and collect finished solves; waits up to wait_ms for at least
 * one to finish.  Returns how many finished in this call (>= 0). */
int hc_batch_pump(hc_batch* b, double wait_ms);
/* take one finished solve: returns 1 and its tag, handle and status (HC_OK or
 * the failure of its steps), or 0 if none is waiting.  Its steps are complete
 * on the device; read it through the hc_read_* calls. */
int hc_batch_pop(hc_batch* b, long long* tag, hc_handle** h, int* status);
/* end the batch's hold of a popped solve and free its budget; destroy = 1
 * destroys the handle, 0 hands it back to the caller */
int hc_batch_release(hc_batch* b, hc_handle* h, int destroy);
int hc_batch_get_stats(const hc_batch* b, hc_batch_stats* out);

#ifdef __cplusplus
}
#endif
#endif
