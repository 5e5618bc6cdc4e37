// Host build of the reference-faithful Rohde cycle (csrc/faithful.cuh) for
// tests/test_step_host.py: the per-cell functions the faithful kernels call,
// run cell by cell on the CPU in the order the library's faithful driver
// launches them (src/AmrSim.cpp:430-631):
//
//   cycle(L):  fill L's post-collision buffer (level 0: single-level periodic
//              fill; above: fine now, else the parent coarse cell; outer ghost
//              layer of component 0 zeroed); masked collide of L;
//              if L+1 is the finest: fill, collide, stream, collide, stream,
//              zero invalid ghost components of it; otherwise cycle(L+1)
//              twice; then stream L, add the fine-to-coarse sum, zero invalid
//              ghost components, periodic ghost refresh on level 0.
//
// usage: faithful_host_check f64|paired nx ny nz tau steps nref
//            lo0x lo0y lo0z hi0x hi0y hi0z [lo1... hi1...] in.bin out.bin
// nref (1 or 2) tag boxes follow, each in the cells of the level it refines;
// in.bin: level-0 f[q][z][y][x] in FP64; out.bin: every level's valid f in
// FP64, level 0 first (FAB order).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <utility>
#include <vector>

#include "faithful.cuh"

namespace {

using lbx::Box3;
using lbx::Coupling;
using lbx::IBox;
using lbx::NV;

struct Lev {
  int lo[3], hi[3];  // valid box, global level coordinates
  Box3 b;
  std::vector<double> buf[3];
  int now = 0, next = 1, tmp = 2;
  double tau = 0.0;
  double* P(int k) { return buf[k].data(); }
};

int crs(int x) { return x >= 0 ? x / 2 : -((-x + 1) / 2); }

template <bool PAIRED>
struct Run {
  std::vector<Lev> lev;
  int N[3];

  Coupling coupling(int L) {  // levels (L-1, L)
    Coupling c;
    c.cb = lev[L - 1].b;
    c.fb = lev[L].b;
    for (int d = 0; d < 3; ++d) {
      c.clo[d] = lev[L - 1].lo[d];
      c.flo[d] = lev[L].lo[d];
      c.cdom[d] = N[d] << (L - 1);
    }
    c.cper = L - 1 == 0 ? 1 : 0;
    return c;
  }
  // the faithful mask: coarsen(own box) (src/AmrSim.cpp:421-425), valid-relative
  IBox covered(int L) {
    IBox c;
    for (int d = 0; d < 3; ++d) {
      c.lo[d] = crs(lev[L].lo[d]) - lev[L].lo[d];
      c.hi[d] = crs(lev[L].hi[d]) - lev[L].lo[d];
    }
    return c;
  }
  template <typename F>
  static void grown(const Box3& b, F&& body) {
    for (int z = 0; z < b.n[2] + 2 * b.g; ++z)
      for (int y = 0; y < b.n[1] + 2 * b.g; ++y)
        for (int x = 0; x < b.n[0] + 2 * b.g; ++x) body(x, y, z);
  }
  template <typename F>
  static void valid(const Box3& b, F&& body) {
    for (int z = 0; z < b.n[2]; ++z)
      for (int y = 0; y < b.n[1]; ++y)
        for (int x = 0; x < b.n[0]; ++x) body(x, y, z);
  }

  void refine(const int* tlo, const int* thi) {
    const Lev& p = lev.back();
    Lev f;
    for (int d = 0; d < 3; ++d) {
      f.lo[d] = 2 * tlo[d];
      f.hi[d] = 2 * thi[d] + 1;
    }
    f.b = lbx::make_box(f.hi[0] - f.lo[0] + 1, f.hi[1] - f.lo[1] + 1, f.hi[2] - f.lo[2] + 1, 2);
    for (auto& v : f.buf) v.assign(NV * f.b.sq, 0.0);
    f.tau = 2.0 * (p.tau - 0.5) + 0.5;  // src/AmrSim.cpp:313-314
    lev.push_back(std::move(f));
    const int L = (int)lev.size() - 1;
    const Coupling c = coupling(L);
    grown(c.fb, [&](int x, int y, int z) {
      lbx::cell_fill_from_coarse<double>(lev[L - 1].P(lev[L - 1].now), lev[L].P(lev[L].now), c, x,
                                         y, z);
    });
  }

  void init_post_collision(int L) {  // src/AmrSim.cpp:471-485
    Lev& l = lev[L];
    if (L == 0) {
      grown(l.b, [&](int x, int y, int z) {
        lbx::f_cell_fill_single(l.P(l.now), l.P(l.next), l.b, x, y, z);
      });
    } else {
      Lev& c = lev[L - 1];
      const Coupling cp = coupling(L);
      const int fd[3] = {N[0] << L, N[1] << L, N[2] << L};
      grown(l.b, [&](int x, int y, int z) {
        lbx::f_cell_fill_two(l.P(l.now), l.P(l.next), c.P(c.now), cp, fd[0], fd[1], fd[2], x, y, z);
      });
      grown(l.b, [&](int x, int y, int z) { lbx::f_cell_zero_ring0(l.P(l.next), l.b, x, y, z); });
    }
  }
  void collide(int L, bool masked) {
    Lev& l = lev[L];
    const IBox cov = masked ? covered(L) : lbx::empty_ibox();
    const double om_s = 1.0 / (l.tau + 0.5), om_b = om_s;  // src/AmrSim.cpp:125-126
    const lbx::DfRates r = PAIRED ? lbx::df_rates(om_s, om_b) : lbx::DfRates{};
    valid(l.b, [&](int x, int y, int z) {
      lbx::f_cell_collide<PAIRED>(l.P(l.next), l.b, cov, x, y, z, om_s, om_b, r);
    });
  }
  void stream(int L) {  // into a fresh (zeroed) buffer
    Lev& l = lev[L];
    l.buf[l.tmp].assign(l.buf[l.tmp].size(), 0.0);
    grown(l.b, [&](int x, int y, int z) { lbx::f_cell_stream(l.P(l.next), l.P(l.tmp), l.b, x, y, z); });
    std::swap(l.next, l.tmp);
  }
  void zero_invalid(int L) {
    Lev& l = lev[L];
    grown(l.b, [&](int x, int y, int z) { lbx::f_cell_zero_invalid(l.P(l.next), l.b, x, y, z); });
  }

  void cycle(int L) {  // src/AmrSim.cpp:430-469
    init_post_collision(L);
    collide(L, true);
    const int F = (int)lev.size() - 1;
    if (L + 1 == F) {
      init_post_collision(F);
      collide(F, false);
      stream(F);
      collide(F, false);
      stream(F);
      zero_invalid(F);
      std::swap(lev[F].now, lev[F].next);
    } else {
      cycle(L + 1);
      cycle(L + 1);
    }
    Lev& l = lev[L];
    stream(L);
    {
      Lev& f = lev[L + 1];
      const Coupling c = coupling(L + 1);
      for (int z = 0; z < c.fb.n[2] / 2 + 2; ++z)
        for (int y = 0; y < c.fb.n[1] / 2 + 2; ++y)
          for (int x = 0; x < c.fb.n[0] / 2 + 2; ++x)
            lbx::f_cell_sum_from_fine(f.P(f.now), l.P(l.next), c, x, y, z);
    }
    zero_invalid(L);
    if (L == 0)
      grown(l.b, [&](int x, int y, int z) { lbx::f_cell_fill_boundary(l.P(l.next), l.b, x, y, z); });
    std::swap(l.now, l.next);
  }
};

template <bool PAIRED>
std::vector<double> run(const int* N, double tau, int steps, int nref, const int* tags,
                        const std::vector<double>& f0) {
  Run<PAIRED> R;
  for (int d = 0; d < 3; ++d) R.N[d] = N[d];
  Lev l0;
  for (int d = 0; d < 3; ++d) {
    l0.lo[d] = 0;
    l0.hi[d] = N[d] - 1;
  }
  l0.b = lbx::make_box(N[0], N[1], N[2], 2);  // ghosts on every level of a multi-level run
  l0.tau = tau;
  for (auto& v : l0.buf) v.assign(NV * l0.b.sq, 0.0);
  const size_t n = (size_t)N[0] * N[1] * N[2];
  Run<PAIRED>::valid(l0.b, [&](int x, int y, int z) {
    const size_t c = ((size_t)z * N[1] + y) * N[0] + x;
    for (int q = 0; q < NV; ++q) l0.buf[l0.now][q * l0.b.sq + l0.b.at(x, y, z)] = f0[q * n + c];
  });
  R.lev.push_back(std::move(l0));
  for (int k = 0; k < nref; ++k) R.refine(tags + 6 * k, tags + 6 * k + 3);
  for (int s = 0; s < steps; ++s) R.cycle(0);
  std::vector<double> out;
  for (Lev& l : R.lev) {
    const double* A = l.P(l.now);
    for (int q = 0; q < NV; ++q)
      Run<PAIRED>::valid(l.b, [&](int x, int y, int z) { out.push_back(A[q * l.b.sq + l.b.at(x, y, z)]); });
  }
  return out;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 8) return 2;
  const char* prec = argv[1];
  const int N[3] = {std::atoi(argv[2]), std::atoi(argv[3]), std::atoi(argv[4])};
  const double tau = std::atof(argv[5]);
  const int steps = std::atoi(argv[6]), nref = std::atoi(argv[7]);
  if (nref < 1 || nref > 2 || argc != 10 + 6 * nref) return 2;
  if (N[0] <= 0 || N[1] <= 0 || N[2] <= 0 || steps < 0) return 2;
  int tags[12];
  for (int i = 0; i < 6 * nref; ++i) tags[i] = std::atoi(argv[8 + i]);
  std::vector<double> f0((size_t)NV * N[0] * N[1] * N[2]);
  FILE* in = std::fopen(argv[8 + 6 * nref], "rb");
  if (!in) return 3;
  const size_t got = std::fread(f0.data(), sizeof(double), f0.size(), in);
  std::fclose(in);
  if (got != f0.size()) return 3;
  std::vector<double> out;
  if (!std::strcmp(prec, "f64"))
    out = run<false>(N, tau, steps, nref, tags, f0);
  else if (!std::strcmp(prec, "paired"))
    out = run<true>(N, tau, steps, nref, tags, f0);
  else
    return 2;
  FILE* fo = std::fopen(argv[9 + 6 * nref], "wb");
  if (!fo) return 4;
  const bool ok = std::fwrite(out.data(), sizeof(double), out.size(), fo) == out.size();
  return std::fclose(fo) == 0 && ok ? 0 : 4;
}
