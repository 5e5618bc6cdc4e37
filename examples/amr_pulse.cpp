// amr_pulse.cpp -- the pulse example of LAMBReX (examples/amr_pulse.cpp of
// the reference) on the GPU library: a 10x10x50 periodic box with a density
// pulse of +0.01 on the plane k = 24, renormalised by the mean of one
// z-column, tau = 0.5; density and velocity are printed at steps 0, 100 and
// 200 with 6 significant digits, in the reference's text format.
//
// build (from the repository root):
//   g++ -std=c++17 -Iinclude examples/amr_pulse.cpp -Llambrex_gb300 -llbx_cuda
//       -Wl,-rpath,<repository>/lambrex_gb300 -o amr_pulse
#include <iostream>
#include <vector>

#include "lambrex.h"

namespace {

void print_density(const AmrSim& sim) {
  const auto dims = sim.GetDims();
  const int numel = dims[0] * dims[1] * dims[2];
  std::cout.precision(6);
  std::cout << "Time: " << sim.GetTime(0) << std::endl;
  std::cout << "Density:\n{ ";
  int idx = 0;
  for (int k = 0; k < dims[2]; ++k)
    for (int j = 0; j < dims[1]; ++j)
      for (int i = 0; i < dims[0]; ++i, ++idx)
        std::cout << sim.GetDensity(i, j, k, 0) << (idx < numel - 1 ? ", " : " };");
  std::cout << std::endl;
}

void print_velocity(const AmrSim& sim) {
  const auto dims = sim.GetDims();
  const int ncell = dims[0] * dims[1] * dims[2];
  std::cout.precision(6);
  std::cout << "Time step: " << sim.GetTimeStep(0) << std::endl;
  std::cout << "Velocity:\n{ ";
  for (int k = 0; k < dims[2]; ++k)
    for (int j = 0; j < dims[1]; ++j)
      for (int i = 0; i < dims[0]; ++i)
        for (int n = 0; n < NDIMS; ++n) {
          // the reference closes the list on the last x-component entry
          const int flat = n * ncell + (k * dims[1] + j) * dims[0] + i;
          std::cout << sim.GetVelocity(i, j, k, n, 0) << (flat < 3 * ncell - 1 ? ", " : " };");
        }
  std::cout << std::endl;
}

}  // namespace

int main() {
  const int nx = 10, ny = 10, nz = 50;
  const double tau = 0.5, amplitude = 0.01;
  const int numel = nx * ny * nz;

  std::vector<double> rho_0(numel, 1.0);
  const int kp = nz / 2;
  for (int i = 0; i < nx; ++i)
    for (int j = 0; j < ny; ++j) rho_0[i * ny * nz + j * nz + kp - 1] += amplitude;
  double z_mean = 0.0;
  for (int k = 0; k < nz; ++k) z_mean += rho_0[(numel + ny * nz) / 2 + k];
  z_mean /= nz;
  for (double& r : rho_0) r /= z_mean;

  lambrexInit();
  {
    AmrSim sim(nx, ny, nz, 0, {1, 1, 1}, tau, tau);
    sim.SetInitialDensity(rho_0);
    sim.SetInitialVelocity(0.0);
    sim.InitFromScratch(0.0);
    print_density(sim);
    print_velocity(sim);
    for (int rep = 0; rep < 2; ++rep) {
      sim.Iterate(100);
      sim.CalcHydroVars(0);
      print_density(sim);
      print_velocity(sim);
    }
  }
  lambrexFinalise();
  return 0;
}
