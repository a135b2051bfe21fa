// C++ mirror of HemoCell's case-program API over the GB300 C ABI.
//
// A case program written against the reference façade (hemocell.h,
// core/hemoCell.cpp) keeps its shape:
//
//   hemo::HemoCell hemocell(argv[1], argc, argv);
//   hemo::param::lbm_shear_parameters(*hemocell.cfg, ny);
//   hemocell.lattice = new hemo::Lattice(nx, ny, nz);      // was MultiBlockLattice3D
//   hemo::iniLatticeSquareCouette(*hemocell.lattice, nx, ny, nz, param::shearrate_lbm);
//   hemocell.initializeCellfield();
//   hemocell.addCellType<hemo::RbcHighOrderModel>("RBC", RBC_FROM_SPHERE);
//   hemocell.loadParticles();
//   while (hemocell.iter < tmax) hemocell.iterate();
//
// Differences: the Palabos lattice and its boundary-condition objects become
// hemo::Lattice (node flags, wall velocities, periodicity); everything runs
// on one GPU, so there is no MPI and no envelope.  Errors print through
// std::cerr and exit(1) as the reference's hlog + exit(1) do.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/hemocell_gb300.h"
#include "config.h"

#ifndef RBC_FROM_SPHERE
#define RBC_FROM_SPHERE 1      // config/constant_defaults.h:80-84
#define ELLIPSOID_FROM_SPHERE 6
#define WBC_SPHERE 0
#endif

namespace hemo {

// Parameters (mechanics/constantConversion.h:32-55): process-global unit
// conversions computed from the <domain> block, as in the reference.
struct Parameters {
  static inline double dt = 0, dx = 0, dm = 0, df = 0, nu_p = 0, rho_p = 0, kBT_p = 0, tau = 0, re = 0;
  static inline double nu_lbm = 0, u_lbm_max = 0, kBT_lbm = 0, shearrate_lbm = 0, f_limit = 0, ef_lbm = 0;
  // mechanics/constantConversion.cpp:36-59
  static void lbm_base_parameters(Config& cfg) {
    dt = cfg["domain"]["dt"].read<double>();
    dx = cfg["domain"]["dx"].read<double>();
    nu_p = cfg["domain"]["nuP"].read<double>();
    rho_p = cfg["domain"]["rhoP"].read<double>();
    kBT_p = cfg["domain"]["kBT"].read<double>();
    if (dt < 0.0) {
      tau = 1.0;
      nu_lbm = 1.0 / 3.0 * (tau - 0.5);
      dt = nu_lbm / nu_p * (dx * dx);
    } else {
      nu_lbm = nu_p * dt / (dx * dx);
      tau = 3.0 * nu_lbm + 0.5;
    }
    dm = rho_p * (dx * dx * dx);
    df = dm * dx / (dt * dt);
    f_limit = 50.0 / 1.0e12 / df;
    kBT_lbm = kBT_p / (df * dx);
  }
  // mechanics/constantConversion.cpp:84-90
  static void lbm_shear_parameters(Config& cfg, double nx) {
    lbm_base_parameters(cfg);
    const double shearrate_p = cfg["domain"]["shearrate"].read<double>();
    re = (nx * (shearrate_p * (nx * 0.5))) / nu_p;
    shearrate_lbm = shearrate_p * dt;
    u_lbm_max = shearrate_lbm;
  }
  // mechanics/constantConversion.cpp:75-82
  static void lbm_pipe_parameters(Config& cfg, int radius) {
    lbm_base_parameters(cfg);
    re = cfg["domain"]["Re"].read<double>();
    u_lbm_max = re * nu_lbm / (radius * 2);
  }
  static void printParameters() {
    std::cout << "(HemoCell) System parameters:\n\t dx: \t" << dx << "\n\t dt: \t" << dt << "\n\t dm: \t" << dm
              << "\n\t dN: \t" << df << "\n\t tau: \t" << tau << "\n\t nu_lbm: \t" << nu_lbm
              << "\n\t u_lb_max: \t" << u_lbm_max << "\n\t f_limit: \t" << f_limit << std::endl;
  }
};
using param = Parameters;

// The lattice the case program describes: size, periodicity, wall nodes
// with their wall velocities, and the external (body) force.
struct Lattice {
  int nx, ny, nz;
  bool periodic[3] = {true, true, true};
  std::vector<uint8_t> flags;  // 0 fluid, k>0 wall class k
  std::map<int, std::array<double, 3>> wall_velocity;
  int body_mode = HC_BODY_NONE;
  double body[3] = {0, 0, 0};
  Lattice(int nx_, int ny_, int nz_) : nx(nx_), ny(ny_), nz(nz_), flags((size_t)nx_ * ny_ * nz_, 0) {}
  size_t index(int x, int y, int z) const { return x + (size_t)nx * (y + (size_t)ny * z); }
  void togglePeriodicity(int axis, bool p) { periodic[axis] = p; }
  // bounce-back nodes (helper/genericFunctions.cpp:138-159 defineDynamics BounceBack)
  void setWall(int x0, int x1, int y0, int y1, int z0, int z1, int cls) {
    for (int z = z0; z <= z1; ++z)
      for (int y = y0; y <= y1; ++y)
        for (int x = x0; x <= x1; ++x) flags[index(x, y, z)] = (uint8_t)cls;
  }
};

// helper/hemocellInit.hh:58-92: x,y periodic, walls at z=0 and z=nz-1
// moving with +-vHalf along x, vHalf = (nz-1) * shearRate / 2.  The walls
// are moving bounce-back nodes here.
inline void iniLatticeSquareCouette(Lattice& L, int nx, int ny, int nz, double shearRate) {
  L.togglePeriodicity(0, true);
  L.togglePeriodicity(1, true);
  L.togglePeriodicity(2, false);
  L.setWall(0, nx - 1, 0, ny - 1, nz - 1, nz - 1, 2);
  L.setWall(0, nx - 1, 0, ny - 1, 0, 0, 1);
  const double vHalf = (nz - 1) * shearRate * 0.5;
  L.wall_velocity[2] = {-vHalf, 0.0, 0.0};
  L.wall_velocity[1] = {vHalf, 0.0, 0.0};
}

// Mechanics models: the template argument of addCellType.
struct CellMechanics {};
struct RbcHighOrderModel : CellMechanics { static constexpr int model = HC_MODEL_RBC_HIGH_ORDER; };
struct PltSimpleModel : CellMechanics { static constexpr int model = HC_MODEL_PLT_SIMPLE; };
struct WbcHighOrderModel : CellMechanics { static constexpr int model = HC_MODEL_WBC_HIGH_ORDER; };

[[noreturn]] inline void die(const std::string& msg) {
  std::cerr << msg << std::endl;
  std::exit(1);
}

// One cell type (core/hemoCellField.h:42-84).
struct HemoCellField {
  std::string name;
  int ctype = 0;
  int model = 0;
  int numVertex = 0;
  unsigned int timescale = 1;
  std::vector<double> xyz;
  std::vector<int> tris, inner;
  std::unique_ptr<Config> materialCfg;
};

struct HemoCellFields {
  std::vector<std::unique_ptr<HemoCellField>> fields;
  unsigned int particleVelocityUpdateTimescale = 1;
  HemoCellField* operator[](const std::string& name) {
    for (auto& f : fields)
      if (f->name == name) return f.get();
    die("(HemoCell) (CellFields) no cell type named " + name);
  }
  HemoCellField* operator[](size_t i) { return fields.at(i).get(); }
  size_t size() const { return fields.size(); }
};

class HemoCell {
 public:
  enum class MPIHandle { Internal, External };
  Config* cfg = nullptr;
  Lattice* lattice = nullptr;
  HemoCellFields* cellfields = nullptr;
  unsigned int iter = 0;
  int form = HC_FORM_PLAIN_F64;
  int launch = HC_LAUNCH_PER_STAGE;
  int device = 0;

  HemoCell(const char* configFileName, int, char**, MPIHandle = MPIHandle::Internal) {
    try {
      cfg = new Config(configFileName);
    } catch (std::exception& e) {
      die(std::string("(HemoCell) cannot read config: ") + e.what());
    }
  }
  ~HemoCell() {
    if (h_) hc_destroy(h_);
    delete cellfields;
    delete lattice;
    delete cfg;
  }
  hc_handle* handle() { return h_; }

  // core/hemoCell.cpp:135-147: creates the device state of the lattice
  void initializeCellfield() {
    if (!lattice) die("(HemoCell) please create a lattice before initializing the cell field");
    if (Parameters::dx <= 0) Parameters::lbm_base_parameters(*cfg);
    hc_params p = {};
    p.nx = lattice->nx;
    p.ny = lattice->ny;
    p.nz = lattice->nz;
    for (int a = 0; a < 3; ++a) p.periodic[a] = lattice->periodic[a] ? 1 : 0;
    p.dx = Parameters::dx;
    p.dt = Parameters::dt;
    p.nu_p = Parameters::nu_p;
    p.rho_p = Parameters::rho_p;
    p.kBT_p = Parameters::kBT_p;
    p.tau = Parameters::tau;
    p.form = form;
    p.launch = launch;
    p.device = device;
    h_ = hc_create(&p);
    if (!h_) die(std::string("(HemoCell) ") + hc_last_error(nullptr));
    check(hc_set_flags(h_, lattice->flags.data()));
    for (auto& w : lattice->wall_velocity) check(hc_set_wall_velocity(h_, w.first, w.second.data()));
    check(hc_init_equilibrium(h_, 1.0, nullptr));
    check(hc_set_body_force(h_, lattice->body_mode, lattice->body));
    cellfields = new HemoCellFields();
  }

  // hemocell.h:122-127 + core/hemoCellField.cpp:38-118: reads <name>.xml and
  // builds the rest mesh of the requested shape
  template <class Mechanics>
  void addCellType(const std::string& name, int constructType) {
    auto f = std::make_unique<HemoCellField>();
    f->name = name;
    f->ctype = (int)cellfields->size();
    f->model = Mechanics::model;
    try {
      f->materialCfg = std::make_unique<Config>((name + ".xml").c_str());
    } catch (std::exception& e) {
      die("(HemoCell) (AddCellType) cannot read " + name + ".xml: " + e.what());
    }
    Config& m = *f->materialCfg;
    hc_material mat = {};
    mat.kLink = m["MaterialModel"]["kLink"].read<double>();
    mat.kBend = m["MaterialModel"]["kBend"].read<double>();
    mat.kVolume = m["MaterialModel"]["kVolume"].read<double>();
    mat.kArea = m["MaterialModel"]["kArea"].read<double>();
    mat.eta_m = m["MaterialModel"]["eta_m"].read<double>();
    mat.radius = m["MaterialModel"]["radius"].read<double>();
    if (f->model == HC_MODEL_WBC_HIGH_ORDER) {
      mat.kInnerRigid = m["MaterialModel"]["kInnerRigid"].read<double>();
      mat.kCytoskeleton = m["MaterialModel"]["kCytoskeleton"].read<double>();
      mat.coreRadius = m["MaterialModel"]["coreRadius"].read<double>();
    }
    const int minTri = (int)m["MaterialModel"]["minNumTriangles"].read<double>();
    const double R = mat.radius / Parameters::dx;
    int nf = 20;
    while (nf < minTri) nf *= 4;
    const int nvmax = nf / 2 + 2;
    f->xyz.resize(3 * nvmax);
    f->tris.resize(3 * nf);
    int nv = 0, nff = 0, rc;
    if (constructType == RBC_FROM_SPHERE) {
      rc = hc_mesh_rbc(minTri, R, f->xyz.data(), nvmax, f->tris.data(), nf, &nv, &nff);
    } else if (constructType == ELLIPSOID_FROM_SPHERE) {
      const double ar = m["MaterialModel"]["aspectRatio"].read<double>();
      rc = hc_mesh_ellipsoid(minTri, R, ar, f->xyz.data(), nvmax, f->tris.data(), nf, &nv, &nff);
    } else if (constructType == WBC_SPHERE) {
      rc = hc_mesh_icosphere(minTri, R, f->xyz.data(), nvmax, f->tris.data(), nf, &nv, &nff);
    } else {
      die("(HemoCell) (AddCellType) unsupported construct type");
    }
    if (rc != HC_OK) die("(HemoCell) (AddCellType) mesh generation failed");
    f->xyz.resize(3 * nv);
    f->tris.resize(3 * nff);
    f->numVertex = nv;
    // InnerEdges (mechanics/commonCellConstants.cpp:143-161): explicit list if
    // present, antipodal pairs for the shapes that need inner links otherwise
    try {
      f->inner = m["MaterialModel"]["InnerEdges"].readPairs();
    } catch (std::invalid_argument&) {
      if (f->model != HC_MODEL_RBC_HIGH_ORDER) {
        f->inner.resize(nv);
        const int np = hc_mesh_antipodal_pairs(f->xyz.data(), nv, f->inner.data(), nv / 2);
        f->inner.resize(2 * std::max(np, 0));
      }
    }
    const int t = hc_add_cell_type(h_, name.c_str(), f->model, &mat, f->xyz.data(), nv, f->tris.data(), nff,
                                   f->inner.empty() ? nullptr : f->inner.data(), (int)f->inner.size() / 2);
    check(t);
    cellfields->fields.push_back(std::move(f));
  }

  // core/hemoCell.cpp:191-197 + io/readPositionsBloodCells.cpp:186-361:
  // <name>.pos holds the count, then x y z [um] and three angles [deg] per
  // cell; angles are negated and converted to radians.
  void loadParticles() {
    for (auto& f : cellfields->fields) {
      std::ifstream in(f->name + ".pos");
      if (!in) {
        std::cout << "*** WARNING! particle positions input file " << f->name << ".pos does not exist!" << std::endl;
        continue;
      }
      long n = 0;
      in >> n;
      std::vector<double> c(3 * n), a(3 * n);
      for (long i = 0; i < n; ++i) {
        in >> c[3 * i] >> c[3 * i + 1] >> c[3 * i + 2] >> a[3 * i] >> a[3 * i + 1] >> a[3 * i + 2];
        for (int k = 0; k < 3; ++k) {
          c[3 * i + k] = c[3 * i + k] * (1e-6 / Parameters::dx) + 0.0;
          a[3 * i + k] = (a[3 * i + k] * (M_PI / 180.0)) * -1.0;
        }
      }
      if (!in) die("(readPositionsBloodCells) malformed " + f->name + ".pos");
      if (n > 0) {
        // cells with a vertex on a wall node or off a closed axis are left
        // out, as positionCellInParticleField + deleteIncompleteCells do
        const int added = hc_load_cells(h_, f->ctype, (int)n, c.data(), a.data(), nullptr);
        check(added);
        std::cout << "(readPositionsBloodCells) " << f->name << ": " << added << " of " << n
                  << " cells inside the fluid" << std::endl;
      }
    }
    pushTimescales();
  }

  void setMaterialTimeScaleSeparation(const std::string& name, unsigned int separation) {
    (*cellfields)[name]->timescale = separation;
    if (h_ && cellfields->size()) pushTimescales();
  }
  void setParticleVelocityUpdateTimeScaleSeparation(unsigned int separation) {
    cellfields->particleVelocityUpdateTimescale = separation;
    if (h_ && cellfields->size()) pushTimescales();
  }
  // core/hemoCell.cpp:420-426: cutoff in micrometres; the constant is used as
  // given (lattice force units), every step unless a timescale is set
  void setRepulsion(double repulsionConstant, double repulsionCutoff) {
    repulsionConstant_ = repulsionConstant;
    repulsionCutoff_ = repulsionCutoff * (1e-6 / Parameters::dx);
    check(hc_set_repulsion(h_, repulsionConstant_, repulsionCutoff_, repulsionTimescale_));
  }
  void setRepulsionTimeScaleSeperation(unsigned int separation) {
    repulsionTimescale_ = (int)separation;
    if (repulsionCutoff_ > 0) check(hc_set_repulsion(h_, repulsionConstant_, repulsionCutoff_, repulsionTimescale_));
  }
  // core/hemoCell.cpp:428-436
  void enableBoundaryParticles(double constant, double cutoff, unsigned int timestep = 1) {
    check(hc_set_boundary_repulsion(h_, constant, cutoff * (1e-6 / Parameters::dx), (int)timestep));
  }

  // setExternalVector(lattice, box, force) of the driver: a uniform body force
  void setExternalVector(double fx, double fy, double fz) {
    const double p[3] = {fx, fy, fz};
    check(hc_set_body_force(h_, HC_BODY_UNIFORM, p));
  }

  // <outputDirectory>/<checkpointDirectory>/ as config/config.cpp:168-173 sets it
  std::string outputDirectory() const {
    std::string out = "./tmp";
    try {
      out = (*cfg)["parameters"]["outputDirectory"].read<std::string>();
    } catch (std::invalid_argument&) {
    }
    return out;
  }
  std::string checkpointDirectory() const {
    std::string sub = "checkpoint";
    try {
      sub = (*cfg)["parameters"]["checkpointDirectory"].read<std::string>();
    } catch (std::invalid_argument&) {
    }
    return outputDirectory() + "/" + sub + "/";
  }
  // core/hemoCell.cpp:210-219 and :199-208
  void saveCheckPoint() { check(hc_save_checkpoint(h_, checkpointDirectory().c_str())); }
  void loadCheckPoint() {
    check(hc_load_checkpoint(h_, checkpointDirectory().c_str()));
    hc_stats st;
    check(hc_get_stats(h_, &st));
    iter = (unsigned int)st.iter;
  }
  bool outputInSiUnits = false;
  // core/hemoCell.cpp:221-280: fluid and particle fields in <outputDirectory>/hdf5/
  void writeOutput() {
    check(hc_write_output(h_, outputDirectory().c_str(), outputInSiUnits ? 1 : 0));
  }

  // core/hemoCell.cpp:299-376
  void iterate() {
    check(hc_step(h_, 1));
    iter++;
  }
  void iterate(int n) {
    check(hc_step(h_, n));
    iter += n;
  }

  // per-cell volume (helper/cellInfo.cpp calculateCellVolume), lattice units
  std::vector<double> cellVolumes() {
    hc_stats st;
    check(hc_get_stats(h_, &st));
    std::vector<double> v(st.cells);
    if (st.cells) check(hc_read_cells(h_, nullptr, v.data()));
    return v;
  }
  std::vector<double> positions() {
    hc_stats st;
    check(hc_get_stats(h_, &st));
    std::vector<double> x(3 * (size_t)st.vertices);
    if (st.vertices) check(hc_read_vertices(h_, x.data(), nullptr, nullptr));
    return x;
  }

 private:
  hc_handle* h_ = nullptr;
  double repulsionConstant_ = 0, repulsionCutoff_ = 0;
  int repulsionTimescale_ = 1;
  int check(int rc) {
    if (rc < 0) die(std::string("(HemoCell) ") + hc_last_error(h_));
    return rc;
  }
  void pushTimescales() {
    std::vector<int> every;
    for (auto& f : cellfields->fields) every.push_back((int)f->timescale);
    // core/hemoCell.cpp:620-627
    check(hc_set_timescales(h_, every.data(), (int)every.size(), (int)cellfields->particleVelocityUpdateTimescale));
  }
};

// io/writeCellInfoCSV.cpp:30-74: <outputDirectory>/csv/<type>.<iteration>.csv
inline void writeCellInfo_CSV(HemoCell& hemocell) {
  const std::string dir = hemocell.outputDirectory() + "/csv";
  if (hc_write_cell_info_csv(hemocell.handle(), dir.c_str(), hemocell.outputInSiUnits ? 1 : 0) != HC_OK)
    die(std::string("(writeCellInfo_CSV) ") + hc_last_error(hemocell.handle()));
}

}  // namespace hemo
