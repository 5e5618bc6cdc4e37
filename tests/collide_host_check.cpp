// Host build of the device collision (csrc/d3q15.cuh, csrc/df32.cuh) for
// tests/test_collide_host.py: collides n seeded cells near equilibrium (rho
// and u random, a random non-equilibrium part added) in one of the forms
// below and writes each cell's 15 input and 15 output populations
// (FP64, native byte order) to a file.
//
//   f64     restructured moment-space collision in FP64 (LBX_F64)
//   paired  FP64 values, collision in paired FP32, scalar form
//   packed  the same with twin operations on FP32x2 (the form LBX_F64_PAIRED runs)
//   f32     FP32 populations shifted by w_q rho0, rho0 = 1 (LBX_F32_SHIFTED);
//           the output is unshifted in FP64
//   eq      the FP64 equilibrium of the cell's rho, u (written as the input,
//           padded with zeros)
//   eq32    the FP32 shifted equilibrium around rho0 = 1, unshifted in FP64
//
// usage: collide_host_check f64|paired|packed|f32|eq|eq32 n omega_s omega_b out.bin
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>

#include "df32.cuh"

int main(int argc, char** argv) {
  if (argc != 6) return 2;
  const char* form = argv[1];
  const bool f64 = !std::strcmp(form, "f64"), paired = !std::strcmp(form, "paired"),
             packed = !std::strcmp(form, "packed"), f32 = !std::strcmp(form, "f32"),
             eq = !std::strcmp(form, "eq"), eq32 = !std::strcmp(form, "eq32");
  if (!f64 && !paired && !packed && !f32 && !eq && !eq32) return 2;
  const int n = std::atoi(argv[2]);
  const double om_s = std::atof(argv[3]), om_b = std::atof(argv[4]);
  FILE* out = std::fopen(argv[5], "wb");
  if (!out) return 3;
  std::mt19937_64 gen(12345);
  std::uniform_real_distribution<double> U(-1.0, 1.0);
  const lbx::DfRates r = lbx::df_rates(om_s, om_b);
  for (int c = 0; c < n; ++c) {
    double f[lbx::NV];
    const double rho = 1.0 + 0.05 * U(gen), ux = 0.05 * U(gen), uy = 0.05 * U(gen),
                 uz = 0.05 * U(gen);
    if (eq || eq32) {
      double in[lbx::NV] = {rho, ux, uy, uz};
      std::fwrite(in, sizeof(double), lbx::NV, out);
      if (eq) {
        lbx::equilibrium(rho, ux, uy, uz, f);
      } else {
        float g[lbx::NV];
        lbx::equilibrium_shifted(rho, ux, uy, uz, 1.0, g);
        for (int q = 0; q < lbx::NV; ++q) f[q] = (double)g[q] + lbx::W(q);
      }
      std::fwrite(f, sizeof(double), lbx::NV, out);
      continue;
    }
    lbx::equilibrium(rho, ux, uy, uz, f);
    for (int q = 0; q < lbx::NV; ++q) f[q] += 1e-3 * lbx::W(q) * U(gen);
    if (f32) {  // the stored FP32 values are the input the collision sees
      float g[lbx::NV];
      for (int q = 0; q < lbx::NV; ++q) {
        g[q] = (float)(f[q] - lbx::W(q));
        f[q] = (double)g[q] + lbx::W(q);
      }
      std::fwrite(f, sizeof(double), lbx::NV, out);
      lbx::collide<float>(g, (float)om_s, (float)om_b, 1.0f);
      for (int q = 0; q < lbx::NV; ++q) f[q] = (double)g[q] + lbx::W(q);
    } else {
      std::fwrite(f, sizeof(double), lbx::NV, out);
      if (paired)
        lbx::collide_f64_via_df(f, r);
      else if (packed)
        lbx::collide_f64_via_df_w(f, r);
      else
        lbx::collide<double>(f, om_s, om_b, 0.0);
    }
    std::fwrite(f, sizeof(double), lbx::NV, out);
  }
  return std::fclose(out) == 0 ? 0 : 4;
}
