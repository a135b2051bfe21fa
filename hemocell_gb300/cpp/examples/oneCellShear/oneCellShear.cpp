// Single RBC in Couette shear, written against the HemoCell case API
// (the shape of examples/oneCellShear/oneCellShear.cpp of the reference),
// running on the GB300 library.
// Usage: oneCellShear <config.xml> [steps] [resume]
// <sim><tcsv> and <sim><tcheckpoint> (optional) write the cell CSV and a
// checkpoint at those intervals; "resume" continues from the checkpoint
// instead of loading RBC.pos.
#include <cmath>
#include <iostream>
#include <string>

#include "../../hemocell.h"

using namespace hemo;

int main(int argc, char* argv[]) {
  if (argc < 2) {
    std::cout << "Usage: " << argv[0] << " <configuration.xml> [steps]" << std::endl;
    return -1;
  }
  HemoCell hemocell(argv[1], argc, argv);
  Config* cfg = hemocell.cfg;

  const int nz = (int)(10.0 * (1e-6 / (*cfg)["domain"]["dx"].read<double>()));
  const int nx = 2 * nz, ny = 2 * nz;
  param::lbm_shear_parameters(*cfg, ny);
  param::printParameters();

  hemocell.lattice = new Lattice(nx, ny, nz);
  iniLatticeSquareCouette(*hemocell.lattice, nx, ny, nz, param::shearrate_lbm);

  hemocell.initializeCellfield();
  hemocell.addCellType<RbcHighOrderModel>("RBC", RBC_FROM_SPHERE);
  const bool resume = argc > 3 && std::string(argv[3]) == "resume";
  if (resume) {
    hemocell.loadCheckPoint();
    std::cout << "(OneCellShear) CHECKPOINT found at iteration " << hemocell.iter << std::endl;
  } else {
    hemocell.loadParticles();
  }

  unsigned tcsv = 0, tcheckpoint = 0;
  try {
    tcsv = (*cfg)["sim"]["tcsv"].read<unsigned>();
  } catch (std::invalid_argument&) {
  }
  try {
    tcheckpoint = (*cfg)["sim"]["tcheckpoint"].read<unsigned>();
  } catch (std::invalid_argument&) {
  }
  const unsigned tmax = argc > 2 ? (unsigned)std::atoi(argv[2]) : (*cfg)["sim"]["tmax"].read<unsigned>();
  const double v0 = hemocell.cellVolumes().at(0);
  while (hemocell.iter < tmax) {
    hemocell.iterate();
    if (tcsv && hemocell.iter % tcsv == 0) writeCellInfo_CSV(hemocell);
    if (tcheckpoint && hemocell.iter % tcheckpoint == 0) hemocell.saveCheckPoint();
  }

  std::vector<double> x = hemocell.positions();
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (size_t i = 0; i < x.size() / 3; ++i)
    for (int a = 0; a < 3; ++a) {
      lo[a] = std::min(lo[a], x[3 * i + a]);
      hi[a] = std::max(hi[a], x[3 * i + a]);
    }
  const double um = param::dx * 1e6;
  std::cout.precision(15);
  std::cout << "iter " << hemocell.iter << " volume_ratio " << hemocell.cellVolumes().at(0) / v0 << " bbox_um "
            << (hi[0] - lo[0]) * um << " " << (hi[1] - lo[1]) * um << " " << (hi[2] - lo[2]) * um << std::endl;
  return 0;
}
