// A driver written against the reference's C++ API, as its users write
// them (the scene of examples/3d_pec_sphere_bistatic_rcs.cpp: a PEC sphere
// of radius 0.1 m in an 80-cell cube of 7.5 mm cells, 12-cell CPML on every
// face, an x-polarised +z Gaussian plane wave from a TFSF box 27 cells in,
// the bistatic far field at 1 GHz from an NF-FF box 17 cells in, theta
// over [0, pi) in 180 steps, phi = 0), compiled against
// xfdtd_gb300/host/include/xfdtd/xfdtd.h and run on the GPU engine.
//
//   pec_sphere_bistatic_rcs <output dir> <steps> [fp32]
//
// Simulation::run lowers the scene, steps it on cuda:0 and writes the
// NffftFd outputs (e_theta.npy ... power_phi.npy) into the output dir.
#include <cmath>
#include <cstdlib>
#include <iostream>
#include <memory>
#include <string>
#include <vector>

#include <xfdtd/xfdtd.h>

int main(int argc, char **argv) {
  if (argc < 3) {
    std::cerr << "usage: " << argv[0] << " <output dir> <steps> [fp32]\n";
    return 2;
  }
  const std::string out_dir = argv[1];
  const size_t steps = static_cast<size_t>(std::atol(argv[2]));
  const bool fp32 = argc > 3 && std::string(argv[3]) == "fp32";
  using namespace xfdtd;

  const double dl = 7.5e-3;
  const double corner = -40 * dl, extent = 80 * dl;
  std::vector<std::shared_ptr<Object>> objects;
  objects.push_back(std::make_shared<Object>(
      "domain", std::make_unique<Cube>(PointVector{corner, corner, corner}, PointVector{extent, extent, extent}),
      Material{"air", 1, 1, 0, 0}));
  objects.push_back(std::make_shared<Object>("scatter", std::make_unique<Sphere>(PointVector{0, 0, 0}, 0.1),
                                             Material{"pec", 1, 1, 1e10, 0}));

  std::vector<std::shared_ptr<Boundary>> boundaries;
  for (Orientation o : {Orientation::XN, Orientation::XP, Orientation::YN, Orientation::YP, Orientation::ZN,
                        Orientation::ZP})
    boundaries.push_back(std::make_shared<PML>(o, 12));

  const double lambda_min = 20 * dl;
  const double tau = lambda_min / 6e8, t0 = 4.5 * tau;
  auto tfsf = std::make_unique<TFSF3D>(27, 27, 27, 1.0, 0.0, 0.0, 0.0, std::make_unique<GaussianWaveform>(1, tau, t0));
  auto nffft = std::make_unique<NffftFd>(17, 17, 17, 1e9, linspace(0.0, M_PI, 180, false), std::vector<double>{0},
                                         out_dir);

  Simulation simulation(dl, objects, boundaries, std::move(tfsf), std::move(nffft), 1);
  if (fp32) simulation.setPrecision(Precision::FP32);
  simulation.run(steps);
  std::cout << "ran " << steps << " steps into " << out_dir << "\n";
  return 0;
}
