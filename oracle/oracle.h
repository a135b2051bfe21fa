/*
 * FP64 CPU oracle for the HemoCell IB-LBM time step (test infrastructure).
 *
 * This library is the checker, never the product: only the test suite, the
 * smoke check and the CPU-baseline leg of the benchmark load it.  It restates,
 * in plain sequential-order C++, the per-step path of HemoCell's
 * HemoCell::iterate() (core/hemoCell.cpp:299-376):
 *
 *   spreadParticleForce      core/hemoCellParticleField.cpp:841-863
 *   collideAndStream         Palabos GuoExternalForceBGKdynamics (not in the
 *                            reference tree; restated from Guo, Zheng & Shi,
 *                            PRE 65 046308 (2002), D3Q19 BGK)
 *   interpolateFluidVelocity core/hemoCellParticleField.cpp:819-839
 *   advanceParticles         core/hemoCellParticleField.cpp:566-588,
 *                            core/hemoCellParticle.h:188-203
 *   applyConstitutiveModel   core/hemoCellParticleField.cpp:633-675 with
 *                            mechanics/rbcHighOrderModel.cpp:38-207,
 *                            mechanics/pltSimpleModel.cpp:44-208,
 *                            mechanics/wbcHighOrderModel.cpp:42-225
 *   setExternalVector reset  core/hemoCell.cpp:367-372 (+ driver body force)
 *
 * plus the one-off precompute of mechanics/commonCellConstants.cpp:70-409 and
 * the unit conversions of mechanics/constantConversion.cpp:36-59 and
 * mechanics/cellMechanics.h:50-78.
 *
 * Parity status: the reference cannot be built here (Palabos v2.3.0, MPI and
 * HDF5 are absent), so value-level parity with HemoCell itself is UNPINNED;
 * the oracle is pinned by the reference's own physical validation bounds and
 * by committed golden vectors generated from this oracle.
 */
#ifndef HC_ORACLE_H
#define HC_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_sim orc_sim;

/* Lattice and units ------------------------------------------------------ */
orc_sim* orc_create(int nx, int ny, int nz, int px, int py, int pz,
                    double tau, double f_limit);
void orc_destroy(orc_sim* s);
void orc_set_threads(int n);
/* per-node wall class: 0 fluid, k>0 bounce-back node whose wall velocity is
 * the k-th entry set by orc_set_wall_velocity */
void orc_set_flags(orc_sim* s, const uint8_t* flags);
void orc_set_wall_velocity(orc_sim* s, int cls, const double* u3);
/* mode 0: none, 1: uniform (p[0..2]), 2: Kolmogorov F_x=A sin(2 pi z / nz)
 * (p[0]=A) */
void orc_set_body_force(orc_sim* s, int mode, const double* p);
void orc_init_equilibrium(orc_sim* s, double rho, const double* u3);

/* Cell types and cells --------------------------------------------------- */
/* model 0 RBC high order, 1 PLT simple, 2 WBC high order.
 * k[] = {k_link, k_bend, k_volume, k_area, eta_m, k_inner_rigid,
 *        k_cytoskeleton, core_radius, radius}, already in lattice units */
int orc_add_cell_type(orc_sim* s, int model, int nv, const double* xyz,
                      int nf, const int* tris, int ni, const int* inner,
                      const double* k);
int orc_add_cell(orc_sim* s, int type, const double* xyz);
void orc_set_timescales(orc_sim* s, const int* material_every, int velocity_every);
/* constant external vertex forces added before each spread
 * (HemoCellStretch::applyForce, helper/hemoCellStretch.cpp:63-78) */
void orc_set_vertex_forces(orc_sim* s, int n, const int* ids, const double* forces);

/* Stepping --------------------------------------------------------------- */
void orc_step(orc_sim* s, int nsteps);
void orc_set_repulsion(orc_sim* s, double k, double cutoff, int every);
void orc_set_boundary_repulsion(orc_sim* s, double k, double cutoff, int every);
void orc_stage_repulsion(orc_sim* s);
void orc_read_repulsion(orc_sim* s, double* f); /* [V][3] */
void orc_stage_spread(orc_sim* s);
void orc_stage_collide_stream(orc_sim* s); /* + force reset, keeping the old field */
void orc_stage_interpolate(orc_sim* s);
void orc_stage_advance(orc_sim* s);
void orc_stage_mechanics(orc_sim* s, int forced);

/* Read / write state ------------------------------------------------------ */
long orc_num_nodes(orc_sim* s);
int orc_num_vertices(orc_sim* s);
int orc_num_cells(orc_sim* s);
int orc_iter(orc_sim* s);
void orc_read_fluid(orc_sim* s, double* rho, double* u);
void orc_read_populations(orc_sim* s, double* f);
void orc_write_populations(orc_sim* s, const double* f);
void orc_read_force_field(orc_sim* s, double* F, int which);
void orc_write_force_field(orc_sim* s, const double* F);
void orc_read_vertices(orc_sim* s, double* x, double* v, double* f);
void orc_write_vertices(orc_sim* s, const double* x, const double* v, const double* f);
void orc_read_cells(orc_sim* s, int* alive, double* volume);

/* Binning (a9): per vertex bin node and tile; tile CSR sorted by
 * (tile, cell, vertex); per-tile unique cell list.  Returns the number of
 * tiles, or -1 when a buffer is too small. */
int orc_bins(orc_sim* s, int tx, int ty, int tz, const double* x,
             int* vertex_node, int* vertex_tile, int* tile_offsets,
             int* tile_vertices, int* tile_cell_offsets, int* tile_cells,
             int max_tile_cells);
/* neighbour lists from the tile cell lists of orc_bins: per tile, sorted
 * distinct cells of the tile and its 26 neighbours (periodic axes wrapped) */
int orc_neighbours(int ntx, int nty, int ntz, int px, int py, int pz, const int* tile_cell_offsets,
                   const int* tile_cells, int* nb_offsets, int* nb_cells, int max_cells);

/* CommonCellConstants export for tests: sizes (nE, nI) and arrays */
int orc_type_sizes(orc_sim* s, int type, int* out4);
void orc_type_constants(orc_sim* s, int type, int* edges, double* edge_l0,
                        double* edge_angle0, int* ring, int* ring_n,
                        double* patch_d0, double* tri_a0, int* bend_outer,
                        double* scalars);

/* Units (mechanics/constantConversion.cpp:36-59, cellMechanics.h:50-78) */
void orc_units(double dx, double dt, double nu_p, double rho_p, double kBT_p,
               double tau_override, double* out /* tau, nu_lbm, dm, df,
               kBT_lbm, f_limit */);
void orc_material_scale(int model, int nfaces, const double* units,
                        double dx, double dt, const double* mat /* kLink,
                        kBend, kVolume, kArea, eta_m, kInnerRigid,
                        kCytoskeleton, coreRadius, radius (SI) */,
                        double* k_out /* 9 */);

/* Cell geometry (geometry.cpp) ------------------------------------------- */
/* constructSphereIcosahedron / constructRBCFromSphere /
 * constructEllipsoidFromSphere (helper/meshGeneratingFunctions.hh:31-271):
 * vertices xyz[nv][3] (lattice units) and outward faces tris[nf][3]; returns
 * -1 when the buffers are too small (nv, nf still set) */
int orc_mesh_icosphere(int min_triangles, double radius, double* xyz, int max_nv, int* tris, int max_nf, int* nv,
                       int* nf);
int orc_mesh_rbc(int min_triangles, double radius, double* xyz, int max_nv, int* tris, int max_nf, int* nv,
                 int* nf);
int orc_mesh_ellipsoid(int min_triangles, double radius, double aspect, double* xyz, int max_nv, int* tris,
                       int max_nf, int* nv, int* nf);
int orc_mesh_antipodal_pairs(const double* xyz, int nv, int* pairs, int max_pairs);
/* loadParticles' placement (io/readPositionsBloodCells.cpp:39-124, 290-361):
 * n cells of a template, centres in lattice units, angles in radians as the
 * reference stores them (negated .pos angles); out[n][nv][3] */
void orc_place_cells(const double* rest, int nv, int n, const double* centres, const double* angles, double* out);
/* .pos lines (micrometres, degrees) to lattice-unit centres and the
 * reference's radians (io/readPositionsBloodCells.cpp:218-224, 327-351) */
void orc_pos_to_lattice(int n, const double* pos_um, const double* angles_deg, double dx, double* centres,
                        double* angles);
/* the project's seeded packer (no reference counterpart); returns the number
 * of cells placed without overlap */
int orc_pack_cells(int nx, int ny, int nz, const int* periodic, const uint8_t* solid, int ntypes,
                   const double* const* rest, const int* nvs, const int* const* tris, const int* nfs,
                   const int* counts, double margin, unsigned long long seed, int max_attempts, double* centres,
                   double* angles, int* types);

#ifdef __cplusplus
}
#endif
#endif
