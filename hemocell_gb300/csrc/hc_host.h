// Host-side precompute of the GB300 HemoCell step: mesh generation, the
// per-cell-type rest-state constants, unit conversion, placement and packing.
// Plain C++17; no CUDA types.
#pragma once
#include <array>
#include <cstdint>
#include <string>
#include <vector>

namespace hcg {

struct Vec3 {
  double x, y, z;
};

struct Mesh {
  std::vector<Vec3> v;
  std::vector<std::array<int, 3>> t;
};

// Rest-state constants of one cell type (mechanics/commonCellConstants.cpp:70-409).
struct TypeConstants {
  int model = 0, nv = 0, nf = 0, ne = 0, ni = 0;
  std::vector<int> tris;        // nf*3
  std::vector<int> edges;       // ne*2, i<j, in triangle order
  std::vector<int> bend_tris;   // ne*2 adjacent triangles: [0] edge runs j->i, [1] i->j
  std::vector<int> bend_outer;  // ne*2 opposite vertices of those triangles
  std::vector<int> ring;        // nv*6 sorted 1-ring (-1 padded)
  std::vector<int> ring_n;      // nv
  std::vector<int> inner;       // ni*2
  // per-vertex adjacency for the vertex-centric force assembly, slot j of
  // vertex i refers to its ring neighbour ring[i][j]:
  std::vector<int> vface;       // nv*6 triangle (i, ring[j], ring[j+1])
  std::vector<int> vedge;       // nv*6 edge (i, ring[j])
  std::vector<int> vopp;        // nv*6 edge (ring[j], ring[j+1]) opposite to i
  std::vector<int> vinner_off;  // nv+1 CSR of the inner links touching i
  std::vector<int> vinner;      // inner link ids
  std::vector<int> slot_rot;       // nv*6 position of i in tris[vface] (0..2)
  std::vector<double> slot_a0;     // nv*6 rest area of vface
  std::vector<double> slot_l0;     // nv*6 rest length of vedge
  std::vector<double> tri_a0, edge_l0, edge_angle0, patch_d0, inner_l0;
  double volume_eq = 0, area_mean_eq = 0, edge_mean_eq = 0, angle_mean_eq = 0;
  std::vector<Vec3> rest;       // template vertices (lattice units)
};

// Parameters::lbm_base_parameters (mechanics/constantConversion.cpp:36-59).
struct Units {
  double tau, nu_lbm, dm, df, kBT_lbm, f_limit;
};
Units derive_units(double dx, double dt, double nu_p, double rho_p, double kBT_p, double tau_override);

// Lattice-unit model constants (mechanics/cellMechanics.h:50-78,
// mechanics/wbcHighOrderModel.cpp:243-262).
struct ModelK {
  double k_link, k_bend, k_volume, k_area, eta_m, k_inner_rigid, k_cyto, core_radius, radius;
};
ModelK scale_material(int model, int nfaces, const Units& u, double dx, double dt, const double* mat9);

// helper/meshGeneratingFunctions.hh:31-151 with vertices merged in order of
// first appearance (project-defined numbering).
Mesh icosphere(int min_triangles, double radius);
Mesh rbc_from_sphere(int min_triangles, double radius);          // :153-168, :213-241
Mesh ellipsoid_from_sphere(int min_triangles, double radius, double aspect);  // :170-183, :244-271
std::vector<std::array<int, 2>> antipodal_pairs(const std::vector<Vec3>& v);

// Returns an empty string on success, else the reason.
std::string build_constants(TypeConstants& tc, int model, const std::vector<Vec3>& rest,
                            const std::vector<std::array<int, 3>>& tris,
                            const std::vector<std::array<int, 2>>& inner);

// Placement: centre on bbox, rotateTriangularMeshXYZ (io/readPositionsBloodCells.cpp:39-118),
// translate.  Appends nv*3 positions to out.
void place_cell(const std::vector<Vec3>& rest, const double centre[3], const double angles[3],
                std::vector<double>& out);

// Seeded random sequential packing on an occupancy grid.
int pack_cells(int nx, int ny, int nz, const int* periodic, const uint8_t* solid, int ntypes,
               const std::vector<Mesh>& shapes, const int* counts, double margin, unsigned long long seed,
               int max_attempts, double* centres, double* angles, int* types);

// STL surfaces (binary or ASCII) and their voxelisation
// (helper/voxelizeDomain.cpp:74-152): the mesh is scaled to span ref_length
// lattice units along axis ref_dir and placed `margin` nodes in; nodes inside
// the closed surface are fluid (0), the rest wall (1); open_ends copies the
// slices next to both x ends onto them, opening a closed tube.
std::string read_stl(const std::string& path, std::vector<std::array<Vec3, 3>>& tris);
std::string voxelize(const std::vector<std::array<Vec3, 3>>& tris, int ref_dir, double ref_length, int margin,
                     bool open_ends, int dims[3], std::vector<uint8_t>& flags);

}  // namespace hcg
