// Host build of the paired-FP32 collision (csrc/df32.cuh, scalar form) for
// tests/test_paired_host.py: collides n seeded cells near equilibrium (rho
// and u random, a random non-equilibrium part added) and writes each cell's
// 15 input and 15 output populations (FP64, native byte order) to a file.
//
// usage: paired_host_check n omega_s omega_b out.bin
#include <cstdio>
#include <cstdlib>
#include <random>

#include "df32.cuh"

int main(int argc, char** argv) {
  if (argc != 5) return 2;
  const int n = std::atoi(argv[1]);
  const double om_s = std::atof(argv[2]), om_b = std::atof(argv[3]);
  FILE* out = std::fopen(argv[4], "wb");
  if (!out) return 3;
  std::mt19937_64 gen(12345);
  std::uniform_real_distribution<double> U(-1.0, 1.0);
  const lbx::DfRates r = lbx::df_rates(om_s, om_b);
  for (int c = 0; c < n; ++c) {
    double f[lbx::NV];
    lbx::equilibrium(1.0 + 0.05 * U(gen), 0.05 * U(gen), 0.05 * U(gen), 0.05 * U(gen), f);
    for (int q = 0; q < lbx::NV; ++q) f[q] += 1e-3 * lbx::W(q) * U(gen);
    std::fwrite(f, sizeof(double), lbx::NV, out);
    lbx::collide_f64_via_df(f, r);
    std::fwrite(f, sizeof(double), lbx::NV, out);
  }
  return std::fclose(out) == 0 ? 0 : 4;
}
