/*
 * lbx_oracle.cpp -- CPU restatement of LAMBReX's D3Q15 time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity checker for the CUDA
 * library and the timed CPU baseline; the shipped library never links it.
 * Compile with -ffp-contract=off so that the reference operation order is
 * kept on every host (aarch64 GCC contracts a*b+c into FMA by default).
 *
 * Every function cites the reference file:line it restates.  The AMReX
 * behaviour the reference relies on (FillPatchSingleLevel,
 * FillPatchTwoLevels + PCInterp, InterpFromCoarseLevel, sum_fine_to_coarse,
 * makeFineMask, FillBoundary) is restated from AMReX's public semantics;
 * AMReX itself is not available here.
 */
#include "lbx_oracle.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <limits>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr int NV = 15;
constexpr int ND = 3;

/* D3Q15 velocity ordering, include/d3q15_bgk.h:14-22 (rest, +-x, +-y, +-z,
 * then the eight diagonals).  The ordering is part of the data format. */
constexpr int CX[NV] = {0, 1, -1, 0, 0, 0, 0, 1, 1, 1, 1, -1, -1, -1, -1};
constexpr int CY[NV] = {0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1};
constexpr int CZ[NV] = {0, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 1, -1};

/* weights W (include/d3q15_bgk.h:24-28) as exact fractions */
constexpr long WNUM[NV] = {2, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1};
constexpr long WDEN[NV] = {9, 9, 9, 9, 9, 9, 9, 72, 72, 72, 72, 72, 72, 72, 72};

constexpr double CS2 = 1.0 / 3.0;            // include/AmrSim.h:34
constexpr double NL_DENSITY = -1.0;           // include/AmrSim.h:35
constexpr double NL_VELOCITY = -3E8;          // include/AmrSim.h:36

/* ---- exact rationals, used only to build the mode tables -------------- */
struct Rat {
  long long n, d;
};
long long gcdll(long long a, long long b) {
  a = a < 0 ? -a : a;
  b = b < 0 ? -b : b;
  while (b) {
    long long t = a % b;
    a = b;
    b = t;
  }
  return a ? a : 1;
}
Rat mk(long long n, long long d) {
  if (d < 0) {
    n = -n;
    d = -d;
  }
  long long g = gcdll(n, d);
  return Rat{n / g, d / g};
}
Rat add(Rat a, Rat b) { return mk(a.n * b.d + b.n * a.d, a.d * b.d); }
Rat mul(Rat a, Rat b) { return mk(a.n * b.n, a.d * b.d); }
Rat dvd(Rat a, Rat b) { return mk(a.n * b.d, a.d * b.n); }

/* Mode polynomials of the D3Q15 basis (rows of src/AmrSim.cpp:1037-1054):
 * 0: 1; 1-3: c_a; 4,7,9: c_a^2 - 1/3; 5,6,8: c_a c_b; 10: the scalar ghost
 * (-2 on rest and diagonals, 1 on axes); 11-13: c_a times (1 on axes, -2 on
 * diagonals); 14: c_x c_y c_z. */
Rat mode_poly(int a, int i) {
  const long long x = CX[i], y = CY[i], z = CZ[i];
  const long long c2 = x * x + y * y + z * z;
  const long long h = (c2 == 1) ? 1 : -2;
  switch (a) {
    case 0: return mk(1, 1);
    case 1: return mk(x, 1);
    case 2: return mk(y, 1);
    case 3: return mk(z, 1);
    case 4: return mk(3 * x * x - 1, 3);
    case 5: return mk(x * y, 1);
    case 6: return mk(x * z, 1);
    case 7: return mk(3 * y * y - 1, 3);
    case 8: return mk(y * z, 1);
    case 9: return mk(3 * z * z - 1, 3);
    case 10: return mk(c2 == 1 ? 1 : -2, 1);
    case 11: return mk(x * h, 1);
    case 12: return mk(y * h, 1);
    case 13: return mk(z * h, 1);
    default: return mk(x * y * z, 1);
  }
}

struct Tables {
  double M[NV][NV];     // M[m][p]
  double MI[NV][NV];    // MI[p][m]
  Tables() {
    Rat R[NV][NV];
    for (int a = 0; a < NV; ++a)
      for (int i = 0; i < NV; ++i) R[a][i] = mode_poly(a, i);
    /* The basis is orthogonal under the lattice weights, so the inverse is
     * Minv[i][a] = w_i M[a][i] / sum_j w_j M[a][j]^2 (exact fractions; the
     * doubles below are then correctly rounded like 1./9. literals). */
    for (int a = 0; a < NV; ++a) {
      Rat norm = mk(0, 1);
      for (int i = 0; i < NV; ++i)
        norm = add(norm, mul(mk(WNUM[i], WDEN[i]), mul(R[a][i], R[a][i])));
      for (int i = 0; i < NV; ++i) {
        Rat inv = dvd(mul(mk(WNUM[i], WDEN[i]), R[a][i]), norm);
        MI[i][a] = (double)inv.n / (double)inv.d;
        M[a][i] = (double)R[a][i].n / (double)R[a][i].d;
      }
    }
    /* self-check: Minv * M == identity exactly in rationals */
    for (int i = 0; i < NV; ++i)
      for (int j = 0; j < NV; ++j) {
        Rat s = mk(0, 1);
        for (int a = 0; a < NV; ++a) {
          Rat norm = mk(0, 1);
          for (int k = 0; k < NV; ++k)
            norm = add(norm, mul(mk(WNUM[k], WDEN[k]), mul(R[a][k], R[a][k])));
          s = add(s, mul(dvd(mul(mk(WNUM[i], WDEN[i]), R[a][i]), norm), R[a][j]));
        }
        if (s.n != (i == j ? 1 : 0)) std::abort();
      }
  }
};
const Tables& T() {
  static const Tables t;
  return t;
}

/* DELTA = diag(1/NMODES) (src/AmrSim.cpp:1033-1035) -- not a Kronecker
 * delta; the reference's golden data depends on it. */
constexpr double DELTA_DIAG = 1.0 / NV;

/* Collision of one cell in the reference's operation order
 * (src/AmrSim.cpp:28-103).  f is read through `get`, written through `put`. */
template <class Get, class Put>
inline void collide_ref(Get get, Put put, double OMEGA_S, double OMEGA_B) {
  const Tables& t = T();
  double mode[NV] = {};
  for (int m = 0; m < NV; ++m)
    for (int p = 0; p < NV; ++p) mode[m] += get(p) * t.M[m][p];

  const double density = mode[0];
  double velocity[ND];
  double usq = 0.0;
  for (int a = 0; a < ND; ++a) {
    velocity[a] = mode[a + 1] / density;
    usq += velocity[a] * velocity[a];
  }
  double stress[ND][ND] = {{mode[4], mode[5], mode[6]},
                           {mode[5], mode[7], mode[8]},
                           {mode[6], mode[8], mode[9]}};
  double TrS = 0.0;
  for (int a = 0; a < ND; ++a) TrS += stress[a][a];
  for (int a = 0; a < ND; ++a) stress[a][a] -= (TrS / ND);
  TrS -= OMEGA_B * (TrS - density * usq);
  for (int a = 0; a < ND; ++a) {
    for (int b = 0; b < ND; ++b) {
      const double delta = (a == b) ? DELTA_DIAG : 0.0;
      stress[a][b] -= OMEGA_S * (stress[a][b] -
                                 density * (velocity[a] * velocity[b] - usq * delta));
    }
    stress[a][a] += (TrS / ND);
  }
  mode[4] = stress[0][0];
  mode[5] = stress[0][1];
  mode[6] = stress[0][2];
  mode[7] = stress[1][1];
  mode[8] = stress[1][2];
  mode[9] = stress[2][2];
  for (int m = 10; m < NV; ++m) mode[m] = 0.0;
  for (int p = 0; p < NV; ++p) {
    double fp = 0;
    for (int m = 0; m < NV; ++m) fp += mode[m] * t.MI[p][m];
    put(p, fp);
  }
}

/* Equilibrium of one cell (src/AmrSim.cpp:873-927). */
inline void equilibrium_cell(double rho, const double u[3], double out[NV]) {
  double rho_w[3], u2[3], u_cs2[3], u2_2cs4[3];
  rho_w[0] = rho * 2.0 / 9.0;
  rho_w[1] = rho / 9.0;
  rho_w[2] = rho / 72.0;
  for (int a = 0; a < 3; ++a) {
    u2[a] = u[a] * u[a];
    u_cs2[a] = u[a] / CS2;
    u2_2cs4[a] = u2[a] / (2.0 * CS2 * CS2);
  }
  const double uv_cs4 = u_cs2[0] * u_cs2[1];
  const double vw_cs4 = u_cs2[1] * u_cs2[2];
  const double uw_cs4 = u_cs2[0] * u_cs2[2];
  const double mod_sq = (u2[0] + u2[1] + u2[2]) / (2.0 * CS2);
  const double mod_sq_2 = (u2[0] + u2[1] + u2[2]) * (1 - CS2) / (2.0 * CS2 * CS2);
  out[0] = rho_w[0] * (1.0 - mod_sq);
  out[1] = rho_w[1] * (1.0 - mod_sq + u_cs2[0] + u2_2cs4[0]);
  out[2] = rho_w[1] * (1.0 - mod_sq - u_cs2[0] + u2_2cs4[0]);
  out[3] = rho_w[1] * (1.0 - mod_sq + u_cs2[1] + u2_2cs4[1]);
  out[4] = rho_w[1] * (1.0 - mod_sq - u_cs2[1] + u2_2cs4[1]);
  out[5] = rho_w[1] * (1.0 - mod_sq + u_cs2[2] + u2_2cs4[2]);
  out[6] = rho_w[1] * (1.0 - mod_sq - u_cs2[2] + u2_2cs4[2]);
  out[7] = rho_w[2] * (1.0 + u_cs2[0] + u_cs2[1] + u_cs2[2] + uv_cs4 + vw_cs4 + uw_cs4 + mod_sq_2);
  out[8] = rho_w[2] * (1.0 + u_cs2[0] + u_cs2[1] - u_cs2[2] + uv_cs4 - vw_cs4 - uw_cs4 + mod_sq_2);
  out[9] = rho_w[2] * (1.0 + u_cs2[0] - u_cs2[1] + u_cs2[2] - uv_cs4 - vw_cs4 + uw_cs4 + mod_sq_2);
  out[10] = rho_w[2] * (1.0 + u_cs2[0] - u_cs2[1] - u_cs2[2] - uv_cs4 + vw_cs4 - uw_cs4 + mod_sq_2);
  out[11] = rho_w[2] * (1.0 - u_cs2[0] + u_cs2[1] + u_cs2[2] - uv_cs4 + vw_cs4 - uw_cs4 + mod_sq_2);
  out[12] = rho_w[2] * (1.0 - u_cs2[0] + u_cs2[1] - u_cs2[2] - uv_cs4 - vw_cs4 + uw_cs4 + mod_sq_2);
  out[13] = rho_w[2] * (1.0 - u_cs2[0] - u_cs2[1] + u_cs2[2] + uv_cs4 - vw_cs4 - uw_cs4 + mod_sq_2);
  out[14] = rho_w[2] * (1.0 - u_cs2[0] - u_cs2[1] - u_cs2[2] + uv_cs4 + vw_cs4 + uw_cs4 + mod_sq_2);
}

/* Hydrodynamic moments of one cell (src/AmrSim.cpp:957-971): every mode is
 * accumulated from 0.0 in p order; only modes 0..3 are kept. */
template <class Get>
inline void hydro_cell(Get get, double* rho, double u[3]) {
  const Tables& t = T();
  double mode[4];
  for (int m = 0; m < 4; ++m) {
    mode[m] = 0.0;
    for (int p = 0; p < NV; ++p) mode[m] += get(p) * t.M[m][p];
  }
  *rho = mode[0];
  for (int a = 0; a < 3; ++a) u[a] = mode[a + 1] / mode[0];
}

inline int wrap(int x, int n) {
  int r = x % n;
  return r < 0 ? r + n : r;
}
/* AMReX IntVect::coarsen for ratio 2 (floor division) */
inline int crs(int x) { return x >= 0 ? x / 2 : -((-x + 1) / 2); }

/* ---- boxes and fabs --------------------------------------------------- */
struct Box {
  int lo[3] = {0, 0, 0}, hi[3] = {-1, -1, -1};
  bool ok() const { return hi[0] >= lo[0] && hi[1] >= lo[1] && hi[2] >= lo[2]; }
  bool contains(int i, int j, int k) const {
    return i >= lo[0] && i <= hi[0] && j >= lo[1] && j <= hi[1] && k >= lo[2] && k <= hi[2];
  }
  int len(int d) const { return hi[d] - lo[d] + 1; }
  size_t npts() const { return ok() ? (size_t)len(0) * len(1) * len(2) : 0; }
  Box grow(int g) const {
    Box b = *this;
    for (int d = 0; d < 3; ++d) {
      b.lo[d] -= g;
      b.hi[d] += g;
    }
    return b;
  }
  Box coarsen() const {
    Box b;
    for (int d = 0; d < 3; ++d) {
      b.lo[d] = crs(lo[d]);
      b.hi[d] = crs(hi[d]);
    }
    return b;
  }
  Box refine() const {
    Box b;
    for (int d = 0; d < 3; ++d) {
      b.lo[d] = 2 * lo[d];
      b.hi[d] = 2 * hi[d] + 1;
    }
    return b;
  }
  bool operator==(const Box& o) const {
    for (int d = 0; d < 3; ++d)
      if (lo[d] != o.lo[d] || hi[d] != o.hi[d]) return false;
    return true;
  }
};

/* When set, fresh FAB storage is filled with NaN instead of zero: a step
 * that reads memory it never wrote then carries NaN into its results (the
 * reference's own fresh buffers are uninitialised; this restatement defines
 * them as zero). */
static bool g_poison = false;

/* FArrayBox with ncomp components over valid box grown by ng, i fastest. */
struct Fab {
  Box vbox, gbox;
  int ng = 0, nc = 0;
  size_t ncell = 0;
  std::vector<double> d;
  void define(const Box& v, int ngrow, int ncomp) {
    vbox = v;
    ng = ngrow;
    nc = ncomp;
    gbox = v.grow(ngrow);
    ncell = gbox.npts();
    /* fresh storage is zero (defines quirk d), or NaN when poisoning */
    d.assign(ncell * nc, g_poison ? std::numeric_limits<double>::quiet_NaN() : 0.0);
  }
  void clear() {
    d.clear();
    d.shrink_to_fit();
    ncell = 0;
    vbox = Box();
    gbox = Box();
  }
  bool empty() const { return d.empty(); }
  size_t idx(int i, int j, int k) const {
    return ((size_t)(k - gbox.lo[2]) * gbox.len(1) + (j - gbox.lo[1])) * gbox.len(0) +
           (i - gbox.lo[0]);
  }
  double& operator()(int i, int j, int k, int c) { return d[c * ncell + idx(i, j, k)]; }
  double operator()(int i, int j, int k, int c) const { return d[c * ncell + idx(i, j, k)]; }
};

template <class F>
void for_box(const Box& b, F&& f) {
  for (int k = b.lo[2]; k <= b.hi[2]; ++k)
    for (int j = b.lo[1]; j <= b.hi[1]; ++j)
      for (int i = b.lo[0]; i <= b.hi[0]; ++i) f(i, j, k);
}
/* cells of b that are not in inner */
template <class F>
void for_shell(const Box& b, const Box& inner, F&& f) {
  for_box(b, [&](int i, int j, int k) {
    if (!inner.contains(i, j, k)) f(i, j, k);
  });
}
/* the same loops over planes on OpenMP threads, for passes in which every
 * call writes only its own cell (results do not depend on the thread count) */
template <class F>
void for_box_par(const Box& b, F&& f) {
#pragma omp parallel for schedule(static)
  for (int k = b.lo[2]; k <= b.hi[2]; ++k)
    for (int j = b.lo[1]; j <= b.hi[1]; ++j)
      for (int i = b.lo[0]; i <= b.hi[0]; ++i) f(i, j, k);
}
template <class F>
void for_shell_par(const Box& b, const Box& inner, F&& f) {
  for_box_par(b, [&](int i, int j, int k) {
    if (!inner.contains(i, j, k)) f(i, j, k);
  });
}

/* ---- single-level periodic stepping ----------------------------------- */

/* reference-style step on ghost-cell FABs (style 0) */
void step_refstyle(int nx, int ny, int nz, double* f, double OMEGA_S, double OMEGA_B,
                   int nsteps) {
  Box dom;
  dom.hi[0] = nx - 1;
  dom.hi[1] = ny - 1;
  dom.hi[2] = nz - 1;
  const size_t N = dom.npts();
  Fab now, next;
  now.define(dom, 2, NV);
  next.define(dom, 2, NV);
  for (int q = 0; q < NV; ++q)
    for_box(dom, [&](int i, int j, int k) {
      now(i, j, k, q) = f[q * N + ((size_t)k * ny + j) * nx + i];
    });
  auto fill_periodic = [&](Fab& dst, const Fab& src) {
    for (int q = 0; q < NV; ++q)
      for_box(dst.gbox, [&](int i, int j, int k) {
        dst(i, j, k, q) = src(wrap(i, nx), wrap(j, ny), wrap(k, nz), q);
      });
  };
  for (int s = 0; s < nsteps; ++s) {
    /* CollideLevel: DistFnFillPatch(now -> next) (src/AmrSim.cpp:129,359-372) */
    fill_periodic(next, now);
    /* Collide over valid cells, for_point_in loop order i, j, k
     * (include/amr_help.h:87-92) */
    for (int i = 0; i < nx; ++i)
      for (int j = 0; j < ny; ++j)
        for (int k = 0; k < nz; ++k)
          collide_ref([&](int p) { return next(i, j, k, p); },
                      [&](int p, double v) { next(i, j, k, p) = v; }, OMEGA_S, OMEGA_B);
    /* next.FillBoundary(periodicity) (src/AmrSim.cpp:132): ghosts from valid */
    for (int q = 0; q < NV; ++q)
      for_shell(next.gbox, dom, [&](int i, int j, int k) {
        next(i, j, k, q) = next(wrap(i, nx), wrap(j, ny), wrap(k, nz), q);
      });
    /* Stream (src/AmrSim.cpp:109-122): fresh buffer, pull over valid + 1 */
    Fab prop;
    prop.define(dom, 2, NV);
    for (int i = -1; i <= nx; ++i)
      for (int j = -1; j <= ny; ++j)
        for (int k = -1; k <= nz; ++k)
          for (int q = 0; q < NV; ++q)
            prop(i, j, k, q) = next(i - CX[q], j - CY[q], k - CZ[q], q);
    std::swap(next, prop);
    /* UpdateNow (include/multilevel.h:75-80) */
    std::swap(now, next);
  }
  for (int q = 0; q < NV; ++q)
    for_box(dom, [&](int i, int j, int k) {
      f[q * N + ((size_t)k * ny + j) * nx + i] = now(i, j, k, q);
    });
}

/* same arithmetic, ghost-free arrays, OpenMP over planes (style 1) */
void step_fast(int nx, int ny, int nz, double* f, double OMEGA_S, double OMEGA_B, int nsteps,
               int nthreads) {
  const size_t N = (size_t)nx * ny * nz;
  std::vector<double> tmp(N * NV);
  double* a = f;
  double* b = tmp.data();
  for (int s = 0; s < nsteps; ++s) {
#pragma omp parallel for num_threads(nthreads) schedule(static)
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
          const size_t c = ((size_t)k * ny + j) * nx + i;
          collide_ref([&](int p) { return a[p * N + c]; }, [&](int p, double v) { a[p * N + c] = v; },
                      OMEGA_S, OMEGA_B);
        }
#pragma omp parallel for num_threads(nthreads) schedule(static)
    for (int k = 0; k < nz; ++k)
      for (int q = 0; q < NV; ++q) {
        const int ks = wrap(k - CZ[q], nz);
        for (int j = 0; j < ny; ++j) {
          const int js = wrap(j - CY[q], ny);
          const double* src = a + q * N + ((size_t)ks * ny + js) * nx;
          double* dst = b + q * N + ((size_t)k * ny + j) * nx;
          for (int i = 0; i < nx; ++i) dst[i] = src[wrap(i - CX[q], nx)];
        }
      }
    std::swap(a, b);
  }
  if (a != f) std::memcpy(f, a, N * NV * sizeof(double));
}

/* ---- multi-level ------------------------------------------------------ */

struct Level {
  bool defined = false;
  Box box;                    /* valid box (one box per level) */
  Fab now, next;              /* 15 components, 2 ghost layers */
  std::vector<double> rho;    /* valid cells */
  std::vector<double> vel;    /* 3 x valid cells */
  double time = 0.0, dt = 0.0;
  int step = 0;
  double tau_s = 0.0, tau_b = 0.0, mass = 0.0;
  std::vector<int> mask;      /* valid cells; 1 = FINE_VAL (AmrSim.h:69-71) */
  Box tag;                    /* static refinement tag box (may be empty) */
  Fab freed;                  /* buffer the last Stream released (stale reading) */
};

}  // namespace

struct orc_amr {
  int N[3];
  int max_level;
  int mode; /* 0 faithful, 1 conservative */
  /* faithful mode: which reading of each AMReX behaviour (ORC_READ_* bits;
   * 0 = the default readings) */
  int readings = 0;
  int finest = 0;
  std::vector<Level> lev;
  std::vector<double> init_rho, init_u;

  Box domain(int L) const {
    Box b;
    for (int d = 0; d < 3; ++d) {
      b.lo[d] = 0;
      b.hi[d] = (N[d] << L) - 1;
    }
    return b;
  }
  int dn(int L, int d) const { return N[d] << L; }

  /* ComputeDt (src/AmrSim.cpp:297-322).  Faithful mode keeps the reference's
   * tau_l = r(tau_{l-1} - 1/2) + 1/2; the conservative mode uses tau_l =
   * r tau_{l-1}, which keeps the viscosity of omega = 1/(tau + 1/2). */
  void compute_dt(int L) {
    Level& l = lev[L];
    if (L) {
      const Level& c = lev[L - 1];
      const int r = 2;
      l.dt = c.dt / r;
      l.mass = c.mass / r;
      if (mode == 0) {
        l.tau_s = r * (c.tau_s - 0.5) + 0.5;
        l.tau_b = r * (c.tau_b - 0.5) + 0.5;
      } else {
        l.tau_s = r * c.tau_s;
        l.tau_b = r * c.tau_b;
      }
    } else {
      l.dt = 1.0;
      l.mass = 1.0;
    }
  }

  void define_level(int L, const Box& b) {
    Level& l = lev[L];
    l.defined = true;
    l.box = b;
    l.now.define(b, 2, NV);
    l.next.define(b, 2, NV);
    l.rho.assign(b.npts(), 0.0);
    l.vel.assign(3 * b.npts(), 0.0);
  }

  size_t vidx(const Level& l, int i, int j, int k) const {
    return ((size_t)(k - l.box.lo[2]) * l.box.len(1) + (j - l.box.lo[1])) * l.box.len(0) +
           (i - l.box.lo[0]);
  }

  /* CalcHydroVars (src/AmrSim.cpp:938-979) */
  void calc_hydro(int L) {
    Level& l = lev[L];
    const size_t n = l.box.npts();
    for_box(l.box, [&](int i, int j, int k) {
      double r, u[3];
      hydro_cell([&](int p) { return l.now(i, j, k, p); }, &r, u);
      const size_t v = vidx(l, i, j, k);
      l.rho[v] = r;
      for (int a = 0; a < 3; ++a) l.vel[a * n + v] = u[a];
    });
  }

  /* FillPatchSingleLevel: periodic copy from valid "now" into every cell of
   * dst's grown box whose periodic image is valid (src/AmrSim.cpp:364-372) */
  void fill_single(int L, Fab& dst) {
    const Level& l = lev[L];
    for (int q = 0; q < NV; ++q)
      for_box_par(dst.gbox, [&](int i, int j, int k) {
        const int a = wrap(i, dn(L, 0)), b = wrap(j, dn(L, 1)), c = wrap(k, dn(L, 2));
        if (l.box.contains(a, b, c)) dst(i, j, k, q) = l.now(a, b, c, q);
      });
  }

  /* FillPatchTwoLevels with PCInterp and a single time level
   * (src/AmrSim.cpp:373-388): fine "now" (and its periodic images) where it
   * exists, otherwise the parent coarse cell of coarse "now". */
  void fill_two(int L, Fab& dst) {
    const Level& f = lev[L];
    const Level& c = lev[L - 1];
    for (int q = 0; q < NV; ++q)
      for_box_par(dst.gbox, [&](int i, int j, int k) {
        const int a = wrap(i, dn(L, 0)), b = wrap(j, dn(L, 1)), e = wrap(k, dn(L, 2));
        if (f.box.contains(a, b, e)) {
          dst(i, j, k, q) = f.now(a, b, e, q);
        } else {
          const int ci = wrap(crs(i), dn(L - 1, 0)), cj = wrap(crs(j), dn(L - 1, 1)),
                    ck = wrap(crs(k), dn(L - 1, 2));
          if (c.box.contains(ci, cj, ck)) dst(i, j, k, q) = c.now(ci, cj, ck, q);
        }
      });
  }

  /* InterpFromCoarseLevel with PCInterp over the grown box (AmrSim.cpp:393-411) */
  void fill_from_coarse(int L, Fab& dst) {
    const Level& c = lev[L - 1];
    for (int q = 0; q < NV; ++q)
      for_box_par(dst.gbox, [&](int i, int j, int k) {
        const int ci = wrap(crs(i), dn(L - 1, 0)), cj = wrap(crs(j), dn(L - 1, 1)),
                  ck = wrap(crs(k), dn(L - 1, 2));
        if (c.box.contains(ci, cj, ck)) dst(i, j, k, q) = c.now(ci, cj, ck, q);
      });
  }

  /* MakeFineMask (src/AmrSim.cpp:419-428).  Faithful mode passes the coarse
   * level's own BoxArray as the "fine" one, so the marked region is
   * coarsen(coarse box); the conservative mode marks coarsen(fine box). */
  void make_fine_mask(int L) {
    Level& l = lev[L];
    l.mask.assign(l.box.npts(), 0);
    Box cf;
    if (mode == 0 && !(readings & ORC_READ_MASK_FINE)) {
      cf = l.box.coarsen();
    } else {
      if (L + 1 > finest || !lev[L + 1].defined) return;
      cf = lev[L + 1].box.coarsen();
    }
    for_box(l.box, [&](int i, int j, int k) {
      if (cf.contains(i, j, k)) l.mask[vidx(l, i, j, k)] = 1;
    });
  }

  /* ---- reference-faithful Rohde cycle ---- */
  void collide_level(int L, bool masked) {
    Level& l = lev[L];
    const double OS = 1.0 / (l.tau_s + 0.5), OB = 1.0 / (l.tau_b + 0.5);
#pragma omp parallel for schedule(static)
    for (int i = l.box.lo[0]; i <= l.box.hi[0]; ++i)
      for (int j = l.box.lo[1]; j <= l.box.hi[1]; ++j)
        for (int k = l.box.lo[2]; k <= l.box.hi[2]; ++k) {
          if (masked && l.mask[vidx(l, i, j, k)] == 1) {
            for (int m = 0; m < NV; ++m) l.next(i, j, k, m) = 0.0;
          } else {
            collide_ref([&](int p) { return l.next(i, j, k, p); },
                        [&](int p, double v) { l.next(i, j, k, p) = v; }, OS, OB);
          }
        }
  }
  void stream_level(int L) { /* src/AmrSim.cpp:109-122 */
    Level& l = lev[L];
    Fab prop;
    if ((readings & ORC_READ_RING2_STALE) && l.freed.gbox == l.next.gbox && !l.freed.empty())
      prop = l.freed; /* the allocator hands back the block the last Stream released */
    else
      prop.define(l.box, 2, NV);
    for_box_par(l.box.grow(1), [&](int i, int j, int k) {
      for (int q = 0; q < NV; ++q) prop(i, j, k, q) = l.next(i - CX[q], j - CY[q], k - CZ[q], q);
    });
    std::swap(l.next, prop);
    if (readings & ORC_READ_RING2_STALE) l.freed = std::move(prop);
  }
  void fill_boundary(int L) { /* next.FillBoundary(periodicity) */
    Level& l = lev[L];
    for (int q = 0; q < NV; ++q)
      for_shell(l.next.gbox, l.box, [&](int i, int j, int k) {
        const int a = wrap(i, dn(L, 0)), b = wrap(j, dn(L, 1)), c = wrap(k, dn(L, 2));
        if (l.box.contains(a, b, c)) l.next(i, j, k, q) = l.next(a, b, c, q);
      });
  }
  void init_post_collision(int L) { /* src/AmrSim.cpp:471-485 */
    Level& l = lev[L];
    if (L == 0) {
      fill_single(0, l.next);
    } else {
      fill_two(L, l.next);
      /* outermost ghost layer, component 0 only */
      for_shell(l.next.gbox, l.next.gbox.grow(-1), [&](int i, int j, int k) { l.next(i, j, k, 0) = 0.0; });
    }
  }
  void zero_invalid(int L) { /* src/AmrSim.cpp:604-617 */
    Level& l = lev[L];
    for_shell(l.next.gbox, l.box, [&](int i, int j, int k) {
      for (int m = 0; m < NV; ++m)
        if (!l.box.contains(i - 2 * CX[m], j - 2 * CY[m], k - 2 * CZ[m])) l.next(i, j, k, m) = 0.0;
    });
  }
  /* sum_fine_to_coarse: average each 2^3 block of fine "now" over the
   * coarsened fine box grown by one, then ADD into the coarse valid cells
   * through every periodic image (src/AmrSim.cpp:592-602).  The other
   * readings: the x8 block sum instead of the average (ORC_READ_SUM8), the
   * coarsened fine box without its ghost ring (ORC_READ_GROW0). */
  void sum_from_fine(int L) {
    Level& c = lev[L];
    const Level& f = lev[L + 1];
    const Box cb = f.box.coarsen().grow((readings & ORC_READ_GROW0) ? 0 : 1);
    const double wgt = (readings & ORC_READ_SUM8) ? 1.0 : 0.125;
    for (int q = 0; q < NV; ++q)
      for_box(cb, [&](int i, int j, int k) {
        double s = 0.0;
        for (int kr = 0; kr < 2; ++kr)
          for (int jr = 0; jr < 2; ++jr)
            for (int ir = 0; ir < 2; ++ir) s += f.now(2 * i + ir, 2 * j + jr, 2 * k + kr, q);
        const double avg = wgt * s;
        for (int sz = -1; sz <= 1; ++sz)
          for (int sy = -1; sy <= 1; ++sy)
            for (int sx = -1; sx <= 1; ++sx) {
              const int a = i + sx * dn(L, 0), b = j + sy * dn(L, 1), e = k + sz * dn(L, 2);
              if (c.box.contains(a, b, e)) c.next(a, b, e, q) += avg;
            }
      });
  }
  void update_distribution(int L) { /* src/AmrSim.cpp:619-631 */
    Level& l = lev[L];
    if (L && L == finest) {
      l.time += 2 * l.dt;
      l.step += 2;
    } else {
      l.time += l.dt;
      ++l.step;
    }
    std::swap(l.now, l.next);
  }
  void rohde_cycle(int L) { /* src/AmrSim.cpp:430-469 */
    init_post_collision(L);
    collide_level(L, true);
    if (L + 1 == finest) {
      const int F = finest;
      init_post_collision(F);
      collide_level(F, false);
      stream_level(F);
      collide_level(F, false);
      stream_level(F);
      zero_invalid(F);
      update_distribution(F);
    } else {
      for (int it = 0; it < 2; ++it) rohde_cycle(L + 1);
    }
    stream_level(L);
    sum_from_fine(L);
    zero_invalid(L);
    if (L == 0) fill_boundary(0);
    update_distribution(L);
  }
  void iterate_level0() { /* IterateLevel(0), src/AmrSim.cpp:124-135,324-333 */
    Level& l = lev[0];
    fill_single(0, l.next);
    collide_level(0, false);
    fill_boundary(0);
    stream_level(0);
    std::swap(l.now, l.next);
    l.time += l.dt;
    ++l.step;
  }

  /* ---- conservative volumetric scheme ----
   * State of level L > 0 lives on the grown box; its ghost shell carries the
   * populations exchanged with level L-1.  Level 0 is periodic. */
  static void collide_fast(double* f, double OS, double OB) {
    collide_ref([&](int p) { return f[p]; }, [&](int p, double v) { f[p] = v; }, OS, OB);
  }
  bool covered(int L, int i, int j, int k) const {
    return L < finest && lev[L + 1].box.coarsen().contains(i, j, k);
  }
  /* parent coarse cell of fine (i,j,k) on level L, wrapped periodically */
  void parent(int L, int i, int j, int k, int* p) const {
    p[0] = wrap(crs(i), dn(L - 1, 0));
    p[1] = wrap(crs(j), dn(L - 1, 1));
    p[2] = wrap(crs(k), dn(L - 1, 2));
  }
  void explode(int L) { /* coarse L-1 post-collision -> ghost shell of L */
    Level& f = lev[L];
    const Level& c = lev[L - 1];
    const double OS = 1.0 / (c.tau_s + 0.5), OB = 1.0 / (c.tau_b + 0.5);
    for_shell_par(f.now.gbox, f.box, [&](int i, int j, int k) {
      int p[3];
      parent(L, i, j, k, p);
      double post[NV];
      for (int q = 0; q < NV; ++q) post[q] = c.now(p[0], p[1], p[2], q);
      collide_fast(post, OS, OB);
      for (int q = 0; q < NV; ++q)
        f.now(i, j, k, q) = f.box.contains(i + 2 * CX[q], j + 2 * CY[q], k + 2 * CZ[q]) ? post[q] : 0.0;
    });
  }
  /* collide active cells, zero covered ones (unless covered cells are
   * active, as in the rescaled coupling), stream */
  void step_cons(int L, bool covered_active = false) {
    Level& l = lev[L];
    const double OS = 1.0 / (l.tau_s + 0.5), OB = 1.0 / (l.tau_b + 0.5);
    const Box& sb = (L == 0) ? l.box : l.now.gbox;
    Fab post;
    post.define(l.box, 2, NV);
    for_box_par(sb, [&](int i, int j, int k) {
      double v[NV];
      for (int q = 0; q < NV; ++q) v[q] = l.now(i, j, k, q);
      if (l.box.contains(i, j, k)) {
        if (!covered_active && covered(L, i, j, k)) {
          for (int q = 0; q < NV; ++q) v[q] = 0.0;
        } else {
          collide_fast(v, OS, OB);
        }
      }
      for (int q = 0; q < NV; ++q) post(i, j, k, q) = v[q];
    });
    for_box_par(sb, [&](int i, int j, int k) {
      for (int q = 0; q < NV; ++q) {
        int a = i - CX[q], b = j - CY[q], e = k - CZ[q];
        if (L == 0) {
          a = wrap(a, dn(0, 0));
          b = wrap(b, dn(0, 1));
          e = wrap(e, dn(0, 2));
        }
        l.next(i, j, k, q) = sb.contains(a, b, e) ? post(a, b, e, q) : 0.0;
      }
    });
    std::swap(l.now, l.next);
  }
  void coalesce(int L) { /* ghost shell of L -> coarse L-1 ring, volume 1/8 */
    const Level& f = lev[L];
    Level& c = lev[L - 1];
    const Box cf = f.box.coarsen();
    for_shell(cf.grow(1), cf, [&](int i, int j, int k) {
      const int a = wrap(i, dn(L - 1, 0)), b = wrap(j, dn(L - 1, 1)), e = wrap(k, dn(L - 1, 2));
      for (int q = 0; q < NV; ++q) {
        double s = 0.0;
        for (int kr = 0; kr < 2; ++kr)
          for (int jr = 0; jr < 2; ++jr)
            for (int ir = 0; ir < 2; ++ir) s += f.now(2 * i + ir, 2 * j + jr, 2 * k + kr, q);
        c.now(a, b, e, q) += 0.125 * s;
      }
    });
  }
  void restrict_covered(int L) { /* covered coarse cells <- mean of children */
    const Level& f = lev[L];
    Level& c = lev[L - 1];
    for_box(f.box.coarsen(), [&](int i, int j, int k) {
      for (int q = 0; q < NV; ++q) {
        double s = 0.0;
        for (int kr = 0; kr < 2; ++kr)
          for (int jr = 0; jr < 2; ++jr)
            for (int ir = 0; ir < 2; ++ir) s += f.now(2 * i + ir, 2 * j + jr, 2 * k + kr, q);
        c.now(i, j, k, q) = 0.125 * s;
      }
    });
  }
  void advance_cons(int L) {
    if (L < finest) explode(L + 1);
    step_cons(L);
    if (L < finest) {
      advance_cons(L + 1);
      advance_cons(L + 1);
      coalesce(L + 1);
      restrict_covered(L + 1);
    }
    lev[L].time += lev[L].dt;
    ++lev[L].step;
  }

  /* ---- rescaled coupling (mode 2) ----
   * Dupuis & Chopard (2003) style transfer in the conservative layout:
   * covered coarse cells stay active and hold the restricted fine state; the
   * fine ghost shell is refilled before each fine sub-step from its parent
   * coarse cells, linearly interpolated in time between the coarse states
   * at the start and the end of the coarse step, with the non-equilibrium
   * part rescaled to the fine level; after the two sub-steps every covered
   * coarse cell takes the mean of its children with the inverse rescaling.
   * Rescaling by s of the non-equilibrium moments is the collision with
   * rate 1 - s: the explosion collides the parent at 1 - (1 - w_f) a (its
   * post-collision state as seen by the fine level), the restriction
   * collides the children's mean at 1 - 1/a, a = w_c / (2 w_f) per rate
   * (trace and traceless stress); the ghost modes come out zero.  tau_l =
   * 2 tau_{l-1}.  Mass is not conserved exactly (the ghost shell and the
   * restriction replace populations instead of exchanging them). */
  struct ResRates {
    double es, eb;  /* explosion */
    double rs, rb;  /* restriction */
  };
  ResRates resc_rates(int L) const {
    const Level& c = lev[L - 1];
    const Level& f = lev[L];
    const double wcs = 1.0 / (c.tau_s + 0.5), wcb = 1.0 / (c.tau_b + 0.5);
    const double wfs = 1.0 / (f.tau_s + 0.5), wfb = 1.0 / (f.tau_b + 0.5);
    const double as = wcs / (2.0 * wfs), ab = wcb / (2.0 * wfb);
    return ResRates{1.0 - (1.0 - wfs) * as, 1.0 - (1.0 - wfb) * ab, 1.0 - 1.0 / as, 1.0 - 1.0 / ab};
  }
  /* fine ghost shell of level L before its sub-step k (0 or 1) of the
   * coarse step: the coarse level has stepped, "next" holds its state at
   * the start of the step and "now" at the end */
  void explode_resc(int L, int k) {
    Level& f = lev[L];
    const Level& c = lev[L - 1];
    const ResRates R = resc_rates(L);
    const double wn = 0.5 * k, wp = 1.0 - wn;
    for_shell_par(f.now.gbox, f.box, [&](int i, int j, int kk) {
      int p[3];
      parent(L, i, j, kk, p);
      double a[NV], b[NV];
      for (int q = 0; q < NV; ++q) a[q] = c.next(p[0], p[1], p[2], q);
      collide_fast(a, R.es, R.eb);
      if (k) {
        for (int q = 0; q < NV; ++q) b[q] = c.now(p[0], p[1], p[2], q);
        collide_fast(b, R.es, R.eb);
        for (int q = 0; q < NV; ++q) a[q] = wp * a[q] + wn * b[q];
      }
      for (int q = 0; q < NV; ++q) f.now(i, j, kk, q) = a[q];
    });
  }
  void restrict_resc(int L) { /* covered coarse cells <- rescaled mean of children */
    const Level& f = lev[L];
    Level& c = lev[L - 1];
    const ResRates R = resc_rates(L);
    for_box_par(f.box.coarsen(), [&](int i, int j, int k) {
      double v[NV];
      for (int q = 0; q < NV; ++q) {
        double s8 = 0.0;
        for (int kr = 0; kr < 2; ++kr)
          for (int jr = 0; jr < 2; ++jr)
            for (int ir = 0; ir < 2; ++ir) s8 += f.now(2 * i + ir, 2 * j + jr, 2 * k + kr, q);
        v[q] = 0.125 * s8;
      }
      collide_fast(v, R.rs, R.rb);
      for (int q = 0; q < NV; ++q) c.now(i, j, k, q) = v[q];
    });
  }
  void advance_resc(int L) {
    step_cons(L, true);
    if (L < finest) {
      for (int k = 0; k < 2; ++k) {
        explode_resc(L + 1, k);
        advance_resc(L + 1);
      }
      restrict_resc(L + 1);
    }
    lev[L].time += lev[L].dt;
    ++lev[L].step;
  }
};

extern "C" {

void orc_set_poison(int on) { g_poison = on != 0; }

void orc_mode_tables(double* M, double* Minv) {
  const Tables& t = T();
  for (int a = 0; a < NV; ++a)
    for (int b = 0; b < NV; ++b) {
      M[a * NV + b] = t.M[a][b];
      Minv[a * NV + b] = t.MI[a][b];
    }
}

void orc_collide_cell(double* f15, double omega_s, double omega_b) {
  collide_ref([&](int p) { return f15[p]; }, [&](int p, double v) { f15[p] = v; }, omega_s, omega_b);
}

int orc_c_to_fab(int nx, int ny, int nz, const double* rho_c, size_t nrho, const double* u_c,
                 size_t nu, double* rho, double* u) {
  const size_t N = (size_t)nx * ny * nz;
  if (nrho < N || nu < 3 * N) return -1;
#pragma omp parallel for schedule(static)
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const size_t c = ((size_t)k * ny + j) * nx + i;
        const size_t l = ((size_t)i * ny + j) * nz + k; /* CLindex */
        rho[c] = rho_c[l];
        for (int n = 0; n < 3; ++n) u[n * N + c] = u_c[l * 3 + n];
      }
  return 0;
}

void orc_equilibrium(int nx, int ny, int nz, const double* rho, const double* u, double* f) {
  const size_t N = (size_t)nx * ny * nz;
#pragma omp parallel for schedule(static)
  for (size_t c = 0; c < N; ++c) {
    const double uu[3] = {u[c], u[N + c], u[2 * N + c]};
    double out[NV];
    equilibrium_cell(rho[c], uu, out);
    for (int q = 0; q < NV; ++q) f[q * N + c] = out[q];
  }
}

int orc_step(int nx, int ny, int nz, double* f, double tau_s, double tau_b, int nsteps,
             int nthreads, int style) {
  if (nx <= 0 || ny <= 0 || nz <= 0 || nsteps < 0) return -1;
  const double OS = 1.0 / (tau_s + 0.5), OB = 1.0 / (tau_b + 0.5); /* AmrSim.cpp:125-126 */
  if (style == 0)
    step_refstyle(nx, ny, nz, f, OS, OB, nsteps);
  else
    step_fast(nx, ny, nz, f, OS, OB, nsteps, nthreads > 0 ? nthreads : 1);
  return 0;
}

void orc_hydro(int nx, int ny, int nz, const double* f, double* rho, double* u) {
  const size_t N = (size_t)nx * ny * nz;
  for (size_t c = 0; c < N; ++c) {
    double r, uu[3];
    hydro_cell([&](int p) { return f[p * N + c]; }, &r, uu);
    rho[c] = r;
    for (int a = 0; a < 3; ++a) u[a * N + c] = uu[a];
  }
}

void orc_mass_momentum(int nx, int ny, int nz, const double* f, double* out) {
  const size_t N = (size_t)nx * ny * nz;
  long double m = 0, j[3] = {0, 0, 0};
  for (int q = 0; q < NV; ++q)
    for (size_t c = 0; c < N; ++c) {
      const long double v = f[q * N + c];
      m += v;
      j[0] += CX[q] * v;
      j[1] += CY[q] * v;
      j[2] += CZ[q] * v;
    }
  out[0] = (double)m;
  for (int a = 0; a < 3; ++a) out[a + 1] = (double)j[a];
}

orc_amr* orc_amr_create(int nx, int ny, int nz, int max_level, double tau_s, double tau_b,
                        int mode) {
  if (nx <= 0 || ny <= 0 || nz <= 0 || max_level < 0 || mode < 0 || mode > 2) return nullptr;
  orc_amr* s = new orc_amr();
  s->N[0] = nx;
  s->N[1] = ny;
  s->N[2] = nz;
  s->max_level = max_level;
  s->mode = mode;
  s->lev.resize(max_level + 1);
  s->lev[0].tau_s = tau_s;
  s->lev[0].tau_b = tau_b;
  return s;
}

void orc_amr_destroy(orc_amr* s) { delete s; }

int orc_amr_set_readings(orc_amr* s, int readings) {
  if (readings & ~(ORC_READ_SUM8 | ORC_READ_GROW0 | ORC_READ_MASK_FINE | ORC_READ_RING2_STALE))
    return -1;
  s->readings = readings;
  for (int L = 0; L <= s->finest; ++L)
    if (s->lev[L].defined) s->make_fine_mask(L);
  return 0;
}

int orc_amr_init(orc_amr* s, const double* rho_c, size_t nrho, const double* u_c, size_t nu,
                 double time) {
  /* MakeNewLevelFromScratch(0) (src/AmrSim.cpp:665-687) */
  const Box dom = s->domain(0);
  const size_t N = dom.npts();
  std::vector<double> rho(N), u(3 * N);
  if (orc_c_to_fab(s->N[0], s->N[1], s->N[2], rho_c, nrho, u_c, nu, rho.data(), u.data()))
    return -1;
  s->define_level(0, dom);
  Level& l = s->lev[0];
  l.time = time;
  s->compute_dt(0);
  l.step = 0;
  l.rho = rho;
  l.vel = u;
  for_box(dom, [&](int i, int j, int k) {
    const size_t c = s->vidx(l, i, j, k);
    const double uu[3] = {u[c], u[N + c], u[2 * N + c]};
    double out[NV];
    equilibrium_cell(rho[c], uu, out);
    for (int q = 0; q < NV; ++q) l.now(i, j, k, q) = out[q];
  });
  s->finest = 0;
  return 0;
}

int orc_amr_refine(orc_amr* s, int level, const int* lo, const int* hi) {
  if (level < 0 || level >= s->max_level || level > s->finest) return -1;
  Box tag;
  for (int d = 0; d < 3; ++d) {
    tag.lo[d] = std::max(lo[d], 0);
    tag.hi[d] = std::min(hi[d], s->dn(level, d) - 1);
  }
  if (!tag.ok()) return -1;
  Level& c = s->lev[level];
  if (!tag.contains(tag.lo[0], tag.lo[1], tag.lo[2])) return -1;
  /* the tag must nest inside the parent's valid box */
  for (int d = 0; d < 3; ++d)
    if (tag.lo[d] < c.box.lo[d] || tag.hi[d] > c.box.hi[d]) return -1;
  c.tag = tag;
  const int L = level + 1;
  const Box fb = tag.refine();
  if (s->lev[L].defined && s->lev[L].box == fb) {
    s->make_fine_mask(level);
    return 0;
  }
  if (s->lev[L].defined) {
    /* RemakeLevel (src/AmrSim.cpp:715-744): refill from old fine + coarse */
    Level& f = s->lev[L];
    Fab nf;
    nf.define(fb, 2, NV);
    s->fill_two(L, nf);
    f.box = fb;
    std::swap(f.now, nf);
    f.next.define(fb, 2, NV);
    f.rho.assign(fb.npts(), 0.0);
    f.vel.assign(3 * fb.npts(), 0.0);
    f.time = c.time;
    s->calc_hydro(L);
  } else {
    /* MakeNewLevelFromCoarse (src/AmrSim.cpp:689-713) */
    s->define_level(L, fb);
    Level& f = s->lev[L];
    f.time = c.time;
    s->compute_dt(L);
    f.step = 0;
    s->fill_from_coarse(L, f.now);
    s->calc_hydro(L);
    s->finest = std::max(s->finest, L);
    s->make_fine_mask(L - 1);
  }
  s->make_fine_mask(level);
  return 0;
}

int orc_amr_unrefine(orc_amr* s, int level) {
  if (level < 0 || level > s->max_level) return -1;
  s->lev[level].tag = Box();
  for (int L = level + 1; L <= s->max_level; ++L) {
    Level& f = s->lev[L];
    f.now.clear();
    f.next.clear();
    f.rho.clear();
    f.vel.clear();
    f.defined = false;
    f.time = 0.0;
    f.dt = 0.0;
    f.step = 0;
  }
  s->finest = std::min(s->finest, level);
  s->make_fine_mask(level);
  return 0;
}

int orc_amr_iterate(orc_amr* s, int nsteps) {
  if (nsteps < 0) return -1;
  for (int t = 0; t < nsteps; ++t) {
    if (s->mode == 0) {
      if (s->finest == 0)
        s->iterate_level0();
      else
        s->rohde_cycle(0);
    } else if (s->mode == 1) {
      s->advance_cons(0);
    } else {
      s->advance_resc(0);
    }
  }
  return 0;
}

int orc_amr_finest(const orc_amr* s) { return s->finest; }

int orc_amr_extent(const orc_amr* s, int level, int* lo, int* hi) {
  if (level < 0 || level > s->finest) return -1;
  for (int d = 0; d < 3; ++d) {
    lo[d] = s->lev[level].box.lo[d];
    hi[d] = s->lev[level].box.hi[d];
  }
  return 0;
}

int orc_amr_copy_f(const orc_amr* s, int level, double* out) {
  if (level < 0 || level > s->finest) return -1;
  const Level& l = s->lev[level];
  const size_t n = l.box.npts();
  for (int q = 0; q < NV; ++q)
    for_box(l.box, [&](int i, int j, int k) { out[q * n + s->vidx(l, i, j, k)] = l.now(i, j, k, q); });
  return 0;
}

int orc_amr_copy_f_grown(const orc_amr* s, int level, double* out) {
  if (level < 0 || level > s->finest) return -1;
  const Level& l = s->lev[level];
  std::memcpy(out, l.now.d.data(), l.now.d.size() * sizeof(double));
  return 0;
}

int orc_amr_calc_hydro(orc_amr* s, int level) {
  if (level < 0 || level > s->finest) return -1;
  s->calc_hydro(level);
  return 0;
}

int orc_amr_get_hydro(const orc_amr* s, int level, double* rho, double* u) {
  if (level < 0 || level > s->finest) return -1;
  const Level& l = s->lev[level];
  std::copy(l.rho.begin(), l.rho.end(), rho);
  std::copy(l.vel.begin(), l.vel.end(), u);
  return 0;
}

int orc_amr_time(const orc_amr* s, int level, double* time, double* dt, int* step,
                 double* tau_s, double* tau_b) {
  if (level < 0 || level > s->max_level) return -1;
  const Level& l = s->lev[level];
  *time = l.time;
  *dt = l.dt;
  *step = l.step;
  *tau_s = l.tau_s;
  *tau_b = l.tau_b;
  return 0;
}

double orc_amr_mass(const orc_amr* s) {
  long double m = 0;
  long double vol = 1;
  for (int L = 0; L <= s->finest; ++L) {
    const Level& l = s->lev[L];
    for_box(l.box, [&](int i, int j, int k) {
      if (s->covered(L, i, j, k)) return;
      for (int q = 0; q < NV; ++q) m += vol * (long double)l.now(i, j, k, q);
    });
    vol /= 8;
  }
  return (double)m;
}

}  // extern "C"
