// Host build of the conservative multi-level step (csrc/cells.cuh) for
// tests/test_step_host.py: the per-cell functions the AMR kernels call --
// fill from coarse (new level), explode, the periodic and patch steps,
// coalesce, restrict -- run cell by cell on the CPU in the order the
// library's conservative driver launches them:
//
//   advance(L): explode coarse L onto the ghost shell of L+1 (if refined);
//               step L (level 0: periodic push, covered cells skipped; above:
//               patch push over the grown box); then, if refined, advance(L+1)
//               twice and coalesce what left L+1 into the ring of L.
//   readout:    covered coarse cells <- mean of their children, finest first.
//
// A precision with the suffix -i32 (f64-i32, f32-i32) uses the 32-bit element
// indices of the batch engine, which runs this scheme for served requests.
// With the suffix +r (f64+r, paired+r, f32+r) the rescaled coupling runs
// instead, in the order of the library's rescaled driver:
//
//   advance(L): step L with every cell active; then, if refined, twice:
//               refill the ghost shell of L+1 from the parents collided at
//               the explosion rates (sub-step 0: the state before the step;
//               sub-step 1: the mean of the states before and after it) and
//               advance(L+1); then every covered cell of L <- the mean of
//               its children collided at the restriction rates.
//
// With the suffix +p (f64+p, f32+p) the conservative coupling runs in the
// pull form of the server (csrc/server.cu), with 32-bit element indices:
//
//   admission:  every level into the pull form (cell_to_qform).
//   advance(L): if refined, explode the coarse post-collision store onto
//               the ghost shell of L+1, advance(L+1) twice and coalesce into
//               the entries the coarse ring cells gather; then step L
//               (cell_step_periodic_pull / cell_step_patch_pull).
//   readout:    every level back to streamed states (cell_to_rform), then
//               the restriction as above.
//
// usage: amr_host_check f64|paired|f32[-i32|+r|+p] nx ny nz tau steps nref
//            lo0x lo0y lo0z hi0x hi0y hi0z [lo1... hi1...] in.bin out.bin
// nref (1 or 2) tag boxes follow, each in the cells of the level it refines;
// in.bin: level-0 f[q][z][y][x] in FP64; out.bin: every level's valid f in
// FP64, level 0 first (FAB order).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <utility>
#include <vector>

#include "cells.cuh"

namespace {

using lbx::Box3;
using lbx::Coupling;
using lbx::IBox;
using lbx::NV;

template <typename T>
struct Lev {
  int lo[3], hi[3];  // valid box, global level coordinates
  Box3 b;
  std::vector<T> buf[2];
  int now = 0;
  double tau = 0.0;
};

template <typename T, bool PAIRED, typename I>
struct Run {
  std::vector<Lev<T>> lev;
  double rho0 = 0.0;

  int dom(int L, int d, const int* N) const { return N[d] << L; }

  Coupling coupling(int L, const int* N) const {  // levels (L-1, L)
    Coupling c;
    c.cb = lev[L - 1].b;
    c.fb = lev[L].b;
    for (int d = 0; d < 3; ++d) {
      c.clo[d] = lev[L - 1].lo[d];
      c.flo[d] = lev[L].lo[d];
      c.cdom[d] = dom(L - 1, d, N);
    }
    c.cper = L - 1 == 0 ? 1 : 0;
    return c;
  }
  IBox covered(int L) const {  // valid-relative coarsen(level L+1), empty on the finest
    if (L + 1 >= (int)lev.size()) return lbx::empty_ibox();
    IBox c;
    for (int d = 0; d < 3; ++d) {
      c.lo[d] = lev[L + 1].lo[d] / 2 - lev[L].lo[d];
      c.hi[d] = lev[L + 1].hi[d] / 2 - lev[L].lo[d];
    }
    return c;
  }
  template <typename F>
  static void grown(const Box3& b, int g, F&& body) {
    for (int z = 0; z < b.n[2] + 2 * g; ++z)
      for (int y = 0; y < b.n[1] + 2 * g; ++y)
        for (int x = 0; x < b.n[0] + 2 * g; ++x) body(x, y, z);
  }

  void refine(const int* tlo, const int* thi, const int* N) {
    const Lev<T>& p = lev.back();
    Lev<T> f;
    for (int d = 0; d < 3; ++d) {
      f.lo[d] = 2 * tlo[d];
      f.hi[d] = 2 * thi[d] + 1;
    }
    f.b = lbx::make_box(f.hi[0] - f.lo[0] + 1, f.hi[1] - f.lo[1] + 1, f.hi[2] - f.lo[2] + 1, 2);
    f.buf[0].assign(NV * f.b.sq, T(0));
    f.buf[1].assign(NV * f.b.sq, T(0));
    f.tau = 2.0 * p.tau;  // conservative scheme: tau_{l+1} = 2 tau_l
    lev.push_back(std::move(f));
    const int L = (int)lev.size() - 1;
    const Coupling c = coupling(L, N);
    grown(c.fb, c.fb.g, [&](int x, int y, int z) {
      lbx::cell_fill_from_coarse<T>(lev[L - 1].buf[lev[L - 1].now].data(),
                                    lev[L].buf[lev[L].now].data(), c, x, y, z);
    });
  }

  void advance(int L, const int* N) {
    Lev<T>& l = lev[L];
    const double om_s = 1.0 / (l.tau + 0.5), om_b = om_s;  // src/AmrSim.cpp:125-126
    const lbx::DfRates r = PAIRED ? lbx::df_rates(om_s, om_b) : lbx::DfRates{};
    const T ts = (T)om_s, tb = (T)om_b, t0 = (T)rho0;
    const bool refined = L + 1 < (int)lev.size();
    if (refined) {
      Lev<T>& f = lev[L + 1];
      const Coupling c = coupling(L + 1, N);
      for (long long t = 0; t < lbx::ghost_cells_of(c.fb); ++t) {
        int s[3];
        if (lbx::ghost_coords(c.fb, (int)t, s))
          lbx::cell_explode<T, PAIRED, I>(l.buf[l.now].data(), f.buf[f.now].data(), c, s[0], s[1],
                                       s[2], ts, tb, t0, r);
      }
    }
    const IBox cov = covered(L);
    const T* in = l.buf[l.now].data();
    T* out = l.buf[1 - l.now].data();
    if (L == 0) {
      grown(l.b, 0, [&](int x, int y, int z) {
        if (refined)
          lbx::cell_step_periodic<T, true, PAIRED, I>(in, out, l.b, cov, x, y, z, ts, tb, t0, r);
        else
          lbx::cell_step_periodic<T, false, PAIRED, I>(in, out, l.b, cov, x, y, z, ts, tb, t0, r);
      });
    } else {
      grown(l.b, l.b.g, [&](int x, int y, int z) {
        if (refined)
          lbx::cell_step_patch<T, true, PAIRED, I>(in, out, l.b, cov, x, y, z, ts, tb, t0, r);
        else
          lbx::cell_step_patch<T, false, PAIRED, I>(in, out, l.b, cov, x, y, z, ts, tb, t0, r);
      });
    }
    l.now = 1 - l.now;
    if (refined) {
      advance(L + 1, N);
      advance(L + 1, N);
      Lev<T>& f = lev[L + 1];
      const Coupling c = coupling(L + 1, N);
      for (long long t = 0; t < lbx::ring_cells_of(c); ++t) {
        int rc[3];
        if (!lbx::ring_coords(c, (int)t, rc)) continue;
        for (int q = 0; q < NV; ++q)
          lbx::cell_coalesce_q<T, I>(f.buf[f.now].data(), l.buf[l.now].data(), c, rc[0], rc[1],
                                  rc[2], q, t0);
      }
    }
  }

  // rescaled coupling: rates of the transfers between L-1 and L
  static void resc_rates(double tc, double tf, double* es, double* rs) {
    const double wc = 1.0 / (tc + 0.5), wf = 1.0 / (tf + 0.5);
    const double a = wc / (2.0 * wf);
    *es = 1.0 - (1.0 - wf) * a;
    *rs = 1.0 - 1.0 / a;
  }

  void advance_resc(int L, const int* N) {
    Lev<T>& l = lev[L];
    const double om = 1.0 / (l.tau + 0.5);
    const lbx::DfRates r = PAIRED ? lbx::df_rates(om, om) : lbx::DfRates{};
    const T ts = (T)om, t0 = (T)rho0;
    const IBox none = lbx::empty_ibox();
    const T* in = l.buf[l.now].data();
    T* out = l.buf[1 - l.now].data();
    if (L == 0)
      grown(l.b, 0, [&](int x, int y, int z) {
        lbx::cell_step_periodic<T, false, PAIRED, I>(in, out, l.b, none, x, y, z, ts, ts, t0, r);
      });
    else
      grown(l.b, l.b.g, [&](int x, int y, int z) {
        lbx::cell_step_patch<T, false, PAIRED, I>(in, out, l.b, none, x, y, z, ts, ts, t0, r);
      });
    l.now = 1 - l.now;
    if (L + 1 >= (int)lev.size()) return;
    Lev<T>& f = lev[L + 1];
    const Coupling c = coupling(L + 1, N);
    double es, rs;
    resc_rates(l.tau, f.tau, &es, &rs);
    const lbx::DfRates re = PAIRED ? lbx::df_rates(es, es) : lbx::DfRates{};
    const lbx::DfRates rr = PAIRED ? lbx::df_rates(rs, rs) : lbx::DfRates{};
    for (int k = 0; k < 2; ++k) {
      for (long long t = 0; t < lbx::ghost_cells_of(c.fb); ++t) {
        int sc[3];
        if (lbx::ghost_coords(c.fb, (int)t, sc))
          lbx::cell_explode_resc<T, PAIRED, I>(l.buf[1 - l.now].data(), l.buf[l.now].data(),
                                               f.buf[f.now].data(), c, sc[0], sc[1], sc[2],
                                               (T)es, (T)es, t0, (T)(1.0 - 0.5 * k),
                                               (T)(0.5 * k), re);
      }
      advance_resc(L + 1, N);
    }
    for (int z = 0; z < c.fb.n[2] / 2; ++z)
      for (int y = 0; y < c.fb.n[1] / 2; ++y)
        for (int x = 0; x < c.fb.n[0] / 2; ++x)
          lbx::cell_restrict_resc<T, PAIRED, I>(f.buf[f.now].data(), l.buf[l.now].data(), c, x, y,
                                                z, (T)rs, (T)rs, t0, rr);
  }

  // the server's pull form (every store holds post-collision populations)
  void to_qform() {
    for (int L = 0; L < (int)lev.size(); ++L) {
      Lev<T>& l = lev[L];
      const T om = (T)(1.0 / (l.tau + 0.5));
      const IBox cov = covered(L);
      grown(l.b, 0, [&](int x, int y, int z) {
        lbx::cell_to_qform<T, I>(l.buf[l.now].data(), l.b, cov, x, y, z, om, om, (T)rho0);
      });
    }
  }

  void advance_pull(int L, const int* N) {
    Lev<T>& l = lev[L];
    const T om = (T)(1.0 / (l.tau + 0.5)), t0 = (T)rho0;
    if (L + 1 < (int)lev.size()) {
      Lev<T>& f = lev[L + 1];
      const Coupling c = coupling(L + 1, N);
      for (long long t = 0; t < lbx::ghost_cells_of(c.fb); ++t) {
        int s[3];
        if (lbx::ghost_coords(c.fb, (int)t, s))
          lbx::cell_explode<T, false, I, true>(l.buf[l.now].data(), f.buf[f.now].data(), c, s[0],
                                              s[1], s[2], T(0), T(0), t0);
      }
      advance_pull(L + 1, N);
      advance_pull(L + 1, N);
      for (long long t = 0; t < lbx::ring_cells_of(c); ++t) {
        int rc[3];
        if (!lbx::ring_coords(c, (int)t, rc)) continue;
        for (int q = 0; q < NV; ++q)
          lbx::cell_coalesce_q<T, I, true>(f.buf[f.now].data(), l.buf[l.now].data(), c, rc[0],
                                          rc[1], rc[2], q, t0);
      }
    }
    const IBox cov = covered(L);
    const T* in = l.buf[l.now].data();
    T* out = l.buf[1 - l.now].data();
    if (L == 0)
      grown(l.b, 0, [&](int x, int y, int z) {
        lbx::cell_step_periodic_pull<T, I>(in, out, l.b, cov, x, y, z, om, om, t0);
      });
    else
      grown(l.b, l.b.g, [&](int x, int y, int z) {
        lbx::cell_step_patch_pull<T, I>(in, out, l.b, cov, x, y, z, om, om, t0);
      });
    l.now = 1 - l.now;
  }

  void to_rform() {
    for (Lev<T>& l : lev)
      grown(l.b, 0, [&](int x, int y, int z) {
        lbx::cell_to_rform<T, I>(l.buf[1 - l.now].data(), l.buf[l.now].data(), l.b, x, y, z);
      });
  }

  void restrict_all(const int* N) {
    for (int L = (int)lev.size() - 1; L >= 1; --L) {
      const Coupling c = coupling(L, N);
      for (int z = 0; z < c.fb.n[2] / 2; ++z)
        for (int y = 0; y < c.fb.n[1] / 2; ++y)
          for (int x = 0; x < c.fb.n[0] / 2; ++x)
            lbx::cell_restrict<T, I>(lev[L].buf[lev[L].now].data(),
                                  lev[L - 1].buf[lev[L - 1].now].data(), c, x, y, z);
    }
  }
};

template <typename T, bool PAIRED, typename I>
std::vector<double> run(const int* N, double tau, int steps, int nref, const int* tags,
                        const std::vector<double>& f0, bool rescaled, bool pull = false) {
  Run<T, PAIRED, I> R;
  const size_t n = (size_t)N[0] * N[1] * N[2];
  if (sizeof(T) == sizeof(float)) {
    for (double v : f0) R.rho0 += v;
    R.rho0 /= (double)n;
  }
  Lev<T> l0;
  for (int d = 0; d < 3; ++d) {
    l0.lo[d] = 0;
    l0.hi[d] = N[d] - 1;
  }
  l0.b = lbx::make_box(N[0], N[1], N[2], 0);
  l0.tau = tau;
  l0.buf[0].resize(NV * n);
  l0.buf[1].assign(NV * n, T(0));
  for (int q = 0; q < NV; ++q)
    for (size_t c = 0; c < n; ++c) l0.buf[0][q * n + c] = (T)(f0[q * n + c] - lbx::W(q) * R.rho0);
  R.lev.push_back(std::move(l0));
  for (int k = 0; k < nref; ++k) R.refine(tags + 6 * k, tags + 6 * k + 3, N);
  if (pull && steps > 0) R.to_qform();
  for (int s = 0; s < steps; ++s) {
    if (rescaled)
      R.advance_resc(0, N);
    else if (pull)
      R.advance_pull(0, N);
    else
      R.advance(0, N);
  }
  if (pull && steps > 0) R.to_rform();
  if (!rescaled) R.restrict_all(N);  // the rescaled coupling restricts as it steps
  std::vector<double> out;
  for (const Lev<T>& l : R.lev) {
    const T* A = l.buf[l.now].data();
    for (int q = 0; q < NV; ++q)
      for (int z = 0; z < l.b.n[2]; ++z)
        for (int y = 0; y < l.b.n[1]; ++y)
          for (int x = 0; x < l.b.n[0]; ++x)
            out.push_back((double)A[q * l.b.sq + l.b.at(x, y, z)] + lbx::W(q) * R.rho0);
  }
  return out;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 8) return 2;
  char prec[32];
  std::snprintf(prec, sizeof prec, "%s", argv[1]);
  const size_t plen = std::strlen(prec);
  const bool rescaled = plen > 2 && !std::strcmp(prec + plen - 2, "+r");
  const bool pull = plen > 2 && !std::strcmp(prec + plen - 2, "+p");
  if (rescaled || pull) prec[plen - 2] = 0;
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
  if (pull && !std::strcmp(prec, "f64"))
    out = run<double, false, int>(N, tau, steps, nref, tags, f0, false, true);
  else if (pull && !std::strcmp(prec, "f32"))
    out = run<float, false, int>(N, tau, steps, nref, tags, f0, false, true);
  else if (pull)
    return 2;
  else if (!std::strcmp(prec, "f64"))
    out = run<double, false, long long>(N, tau, steps, nref, tags, f0, rescaled);
  else if (!std::strcmp(prec, "paired"))
    out = run<double, true, long long>(N, tau, steps, nref, tags, f0, rescaled);
  else if (!std::strcmp(prec, "f32"))
    out = run<float, false, long long>(N, tau, steps, nref, tags, f0, rescaled);
  else if (!std::strcmp(prec, "f64-i32"))
    out = run<double, false, int>(N, tau, steps, nref, tags, f0, rescaled);
  else if (!std::strcmp(prec, "f32-i32"))
    out = run<float, false, int>(N, tau, steps, nref, tags, f0, rescaled);
  else
    return 2;
  FILE* fo = std::fopen(argv[9 + 6 * nref], "wb");
  if (!fo) return 4;
  const bool ok = std::fwrite(out.data(), sizeof(double), out.size(), fo) == out.size();
  return std::fclose(fo) == 0 && ok ? 0 : 4;
}
