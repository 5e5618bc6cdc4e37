// Host build of the batch engine's step walk (csrc/batch.cuh,
// csrc/batch_kernels.cu) for tests/test_step_host.py: an ensemble of periodic
// boxes of uneven sizes advances in the pull form the way the persistent
// kernel walks it -- iteration spaces and fast-division magics from
// set_iteration_space, the tile list from make_tiles, each tile's cells
// decoded with fdiv and stepped by cell_step_pull with 32-bit element
// indices, the boxes' stores selected by par ^ flip.
//
// usage: batch_host_check f64|f32 steps tile_cells nbox nx ny nz tau [...] in.bin out.bin
// in.bin, out.bin: every box's f[q][z][y][x] in FP64, box after box
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "batch.cuh"
#include "cells.cuh"

namespace {

using lbx::BBox;
using lbx::BTile;
using lbx::NV;

template <typename T>
int run(int steps, int tile_cells, int nbox, const int* dims, const double* tau,
        std::vector<double>& f) {
  std::vector<BBox> boxes(nbox);
  std::vector<std::vector<T>> store(2 * nbox);
  std::vector<size_t> off(nbox + 1, 0);
  for (int k = 0; k < nbox; ++k) {
    BBox& B = boxes[k];
    std::memset(&B, 0, sizeof(B));
    B.b = lbx::make_box(dims[3 * k], dims[3 * k + 1], dims[3 * k + 2], 0);
    B.cov = lbx::empty_ibox();
    B.periodic = 1;
    B.pull = 1;
    B.par = 0;
    B.om_s = B.om_b = 1.0 / (tau[k] + 0.5);  // src/AmrSim.cpp:125-126
    if (!lbx::set_iteration_space(B)) return 5;
    const size_t n = (size_t)B.b.sq;
    off[k + 1] = off[k] + NV * n;
    if (sizeof(T) == sizeof(float)) {  // shift: the box's mean density
      double m = 0.0;
      for (size_t i = off[k]; i < off[k + 1]; ++i) m += f[i];
      B.rho0 = m / (double)n;
    }
    for (int s = 0; s < 2; ++s) store[2 * k + s].assign(NV * n, T(0));
    for (int q = 0; q < NV; ++q)
      for (size_t c = 0; c < n; ++c)
        store[2 * k][q * n + c] = (T)(f[off[k] + q * n + c] - lbx::W(q) * B.rho0);
    B.buf[0] = store[2 * k].data();
    B.buf[1] = store[2 * k + 1].data();
  }
  // enter the pull form box by box: Q(x, q) = R(x + c_q, q)
  for (int k = 0; k < nbox; ++k) {
    const lbx::Box3& b = boxes[k].b;
    T* A = store[2 * k].data();
    T* Bq = store[2 * k + 1].data();
    for (int z = 0; z < b.n[2]; ++z)
      for (int y = 0; y < b.n[1]; ++y)
        for (int x = 0; x < b.n[0]; ++x) {
          T g[NV];
          lbx::gather_periodic<T, -1, int>(A, b, x, y, z, g);
          for (int q = 0; q < NV; ++q) Bq[q * b.sq + b.at(x, y, z)] = g[q];
        }
    boxes[k].par = 1;
  }
  std::vector<int> ids(nbox);
  for (int k = 0; k < nbox; ++k) ids[k] = k;
  const std::vector<BTile> tiles = lbx::make_tiles(boxes, ids, tile_cells);
  int flip = 0;
  for (int s = 0; s < steps; ++s) {
    for (const BTile& tl : tiles) {  // the persistent kernel's walk, one tile at a time
      const BBox& B = boxes[tl.box];
      const int par = B.par ^ flip;
      const T* fin = static_cast<const T*>(B.buf[par]);
      T* fout = static_cast<T*>(B.buf[par ^ 1]);
      for (int i = 0; i < tl.count; ++i) {
        const unsigned c = (unsigned)(tl.start + i);
        const int z = lbx::fdiv(c, B.mxy);
        const unsigned r = c - (unsigned)z * (unsigned)B.dxy;
        const int y = lbx::fdiv(r, B.mx);
        const int x = (int)(r - (unsigned)y * (unsigned)B.dx);
        lbx::cell_step_pull<T, false, int>(fin, fout, B.b, x, y, z, (T)B.om_s, (T)B.om_b,
                                           (T)B.rho0, lbx::DfRates{});
      }
    }
    flip ^= 1;
  }
  // read out R_n(x, q) = Q_n(x - c_q, q)
  for (int k = 0; k < nbox; ++k) {
    const BBox& B = boxes[k];
    const lbx::Box3& b = B.b;
    const T* Q = static_cast<const T*>(B.buf[B.par ^ flip]);
    const size_t n = (size_t)b.sq;
    for (int z = 0; z < b.n[2]; ++z)
      for (int y = 0; y < b.n[1]; ++y)
        for (int x = 0; x < b.n[0]; ++x) {
          T g[NV];
          lbx::gather_periodic<T, 1, int>(Q, b, x, y, z, g);
          for (int q = 0; q < NV; ++q)
            f[off[k] + q * n + b.at(x, y, z)] = (double)g[q] + lbx::W(q) * B.rho0;
        }
  }
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 6) return 2;
  const char* prec = argv[1];
  const int steps = std::atoi(argv[2]), tile_cells = std::atoi(argv[3]), nbox = std::atoi(argv[4]);
  if (steps < 0 || tile_cells <= 0 || nbox <= 0 || argc != 7 + 4 * nbox) return 2;
  std::vector<int> dims(3 * nbox);
  std::vector<double> tau(nbox);
  size_t total = 0;
  for (int k = 0; k < nbox; ++k) {
    for (int d = 0; d < 3; ++d) dims[3 * k + d] = std::atoi(argv[5 + 4 * k + d]);
    tau[k] = std::atof(argv[8 + 4 * k]);
    if (dims[3 * k] <= 0 || dims[3 * k + 1] <= 0 || dims[3 * k + 2] <= 0) return 2;
    total += (size_t)NV * dims[3 * k] * dims[3 * k + 1] * dims[3 * k + 2];
  }
  std::vector<double> f(total);
  FILE* in = std::fopen(argv[5 + 4 * nbox], "rb");
  if (!in) return 3;
  const size_t got = std::fread(f.data(), sizeof(double), f.size(), in);
  std::fclose(in);
  if (got != f.size()) return 3;
  int rc;
  if (!std::strcmp(prec, "f64"))
    rc = run<double>(steps, tile_cells, nbox, dims.data(), tau.data(), f);
  else if (!std::strcmp(prec, "f32"))
    rc = run<float>(steps, tile_cells, nbox, dims.data(), tau.data(), f);
  else
    return 2;
  if (rc) return rc;
  FILE* out = std::fopen(argv[6 + 4 * nbox], "wb");
  if (!out) return 4;
  const bool ok = std::fwrite(f.data(), sizeof(double), f.size(), out) == f.size();
  return std::fclose(out) == 0 && ok ? 0 : 4;
}
