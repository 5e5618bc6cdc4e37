// Host build of the per-cell step code of the periodic kernels (csrc/cells.cuh)
// for tests/test_step_host.py: advances a fully periodic box cell by cell on
// the CPU with the same functions the kernels call per thread, in one of two
// forms:
//
//   push  cell_step_periodic: load R_n at the cell, collide, push to x + c_q
//         with wrap (AMR base level, the batch engine's periodic boxes)
//   pull  cell_step_pull: the store holds Q_n = C(R_{n-1}); enter the form by
//         the inverse shift, step by gather + collide + aligned store, read
//         out R_n by the forward gather (the single periodic level)
//
// in one of three precisions (f64, paired: FP64 store with the packed paired
// collision, f32: FP32 store shifted by w_q rho0 with rho0 the mean density).
// push32 and pull32 are the same forms with the 32-bit element indices of the
// batch engine's boxes.
//
// After the steps the cell hydro body reads rho and u from the store as the
// hydro kernel does (gathering through the pull form).
//
// usage: step_host_check push|pull|push32|pull32 f64|paired|f32 nx ny nz steps tau_s tau_b in.bin out.bin
// in.bin: f[q][z][y][x] in FP64 (FAB order, no ghosts); out.bin: f, then
// rho[z][y][x] and u[a][z][y][x]
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <utility>
#include <vector>

#include "cells.cuh"

namespace {

template <typename T, bool PAIRED, typename I>
void run(bool pull, int nx, int ny, int nz, int steps, double tau_s, double tau_b,
         std::vector<double>& f, std::vector<double>& rho, std::vector<double>& u) {
  using lbx::NV;
  const lbx::Box3 b = lbx::make_box(nx, ny, nz, 0);
  const size_t n = (size_t)nx * ny * nz;
  const double om_s = 1.0 / (tau_s + 0.5), om_b = 1.0 / (tau_b + 0.5);  // src/AmrSim.cpp:125-126
  const lbx::DfRates r = lbx::df_rates(om_s, om_b);
  double rho0 = 0.0;
  if (sizeof(T) == sizeof(float)) {
    for (double v : f) rho0 += v;
    rho0 /= (double)n;
  }
  std::vector<T> A(NV * n), B(NV * n);
  for (int q = 0; q < NV; ++q)
    for (size_t c = 0; c < n; ++c) A[q * n + c] = (T)(f[q * n + c] - lbx::W(q) * rho0);
  const T ts = (T)om_s, tb = (T)om_b, t0 = (T)rho0;
  auto each = [&](auto&& body) {
    for (int z = 0; z < nz; ++z)
      for (int y = 0; y < ny; ++y)
        for (int x = 0; x < nx; ++x) body(x, y, z);
  };
  if (pull) {
    auto shift = [&](auto sign) {  // B(x, q) = A(x - sign c_q, q)
      each([&](int x, int y, int z) {
        T g[NV];
        lbx::gather_periodic<T, decltype(sign)::value, I>(A.data(), b, x, y, z, g);
        for (int q = 0; q < NV; ++q) B[q * n + b.at(x, y, z)] = g[q];
      });
      std::swap(A, B);
    };
    shift(std::integral_constant<int, -1>{});  // Q(x, q) = R(x + c_q, q)
    for (int s = 0; s < steps; ++s) {
      each([&](int x, int y, int z) {
        lbx::cell_step_pull<T, PAIRED, I>(A.data(), B.data(), b, x, y, z, ts, tb, t0, r);
      });
      std::swap(A, B);
    }
    each([&](int x, int y, int z) {
      lbx::cell_hydro<T, true>(A.data(), b, rho0, rho.data(), u.data(), x, y, z);
    });
    shift(std::integral_constant<int, 1>{});  // R_n(x, q) = Q_n(x - c_q, q)
  } else {
    const lbx::IBox none = lbx::empty_ibox();
    for (int s = 0; s < steps; ++s) {
      each([&](int x, int y, int z) {
        lbx::cell_step_periodic<T, false, PAIRED, I>(A.data(), B.data(), b, none, x, y, z, ts, tb,
                                                     t0, r);
      });
      std::swap(A, B);
    }
    each([&](int x, int y, int z) {
      lbx::cell_hydro<T, false>(A.data(), b, rho0, rho.data(), u.data(), x, y, z);
    });
  }
  for (int q = 0; q < NV; ++q)
    for (size_t c = 0; c < n; ++c) f[q * n + c] = (double)A[q * n + c] + lbx::W(q) * rho0;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 11) return 2;
  const char* form = argv[1];
  const bool pull = !std::strcmp(form, "pull") || !std::strcmp(form, "pull32");
  const bool i32 = !std::strcmp(form, "push32") || !std::strcmp(form, "pull32");
  if (!pull && !i32 && std::strcmp(form, "push")) return 2;
  const char* prec = argv[2];
  const int nx = std::atoi(argv[3]), ny = std::atoi(argv[4]), nz = std::atoi(argv[5]);
  const int steps = std::atoi(argv[6]);
  const double tau_s = std::atof(argv[7]), tau_b = std::atof(argv[8]);
  if (nx <= 0 || ny <= 0 || nz <= 0 || steps < 0) return 2;
  std::vector<double> f((size_t)lbx::NV * nx * ny * nz);
  FILE* in = std::fopen(argv[9], "rb");
  if (!in) return 3;
  const size_t got = std::fread(f.data(), sizeof(double), f.size(), in);
  std::fclose(in);
  if (got != f.size()) return 3;
  std::vector<double> rho((size_t)nx * ny * nz), u(3 * rho.size());
  auto go = [&](auto idx) {
    using I = decltype(idx);
    if (!std::strcmp(prec, "f64"))
      run<double, false, I>(pull, nx, ny, nz, steps, tau_s, tau_b, f, rho, u);
    else if (!std::strcmp(prec, "paired"))
      run<double, true, I>(pull, nx, ny, nz, steps, tau_s, tau_b, f, rho, u);
    else if (!std::strcmp(prec, "f32"))
      run<float, false, I>(pull, nx, ny, nz, steps, tau_s, tau_b, f, rho, u);
    else
      return false;
    return true;
  };
  if (!(i32 ? go(0) : go(0LL))) return 2;
  FILE* out = std::fopen(argv[10], "wb");
  if (!out) return 4;
  const bool ok = std::fwrite(f.data(), sizeof(double), f.size(), out) == f.size() &&
                  std::fwrite(rho.data(), sizeof(double), rho.size(), out) == rho.size() &&
                  std::fwrite(u.data(), sizeof(double), u.size(), out) == u.size();
  return std::fclose(out) == 0 && ok ? 0 : 4;
}
