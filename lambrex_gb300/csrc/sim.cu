// sim.cu -- host runtime behind the C ABI of include/lbx.h: the simulation
// handle (one per AmrSim), its levels in HBM, the time-step drivers and the
// device-pointer entry points.
//
// Reference call stacks restated here:
//   Iterate -> IterateLevel -> CollideAndStream       src/AmrSim.cpp:981-993, 324-333
//   RohdeCycle (faithful two-level step)              src/AmrSim.cpp:430-631
//   SetStaticRefinement -> MakeNewLevelFromCoarse     src/AmrSim.cpp:995-1009, 689-713
//   ComputeDt                                         src/AmrSim.cpp:297-322
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "checked.cuh"
#include "kernels.cuh"
#include "lbx.h"
#include "sim_internal.h"

using lbx::Box3;
using lbx::Coupling;
using lbx::IBox;

namespace lbx {

int status_from_cuda(cudaError_t e) {
  if (e == cudaSuccess) return LBX_OK;
  if (e == cudaErrorMemoryAllocation) return LBX_ERR_OOM;
  return LBX_ERR_CUDA;
}

thread_local char g_last_error[256] = {0};
void note_error(const char* where, cudaError_t e) {
  std::snprintf(g_last_error, sizeof(g_last_error), "%s: %s", where, cudaGetErrorString(e));
}

}  // namespace lbx

#define CK(call)                                              \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) {                                  \
      lbx::note_error(#call, e_);                             \
      return lbx::status_from_cuda(e_);                       \
    }                                                         \
  } while (0)

#define RET(call)                  \
  do {                             \
    int r_ = (call);               \
    if (r_ != LBX_OK) return r_;   \
  } while (0)

namespace {

constexpr double kNL_DENSITY = -1.0;   // include/AmrSim.h:35
constexpr double kNL_VELOCITY = -3E8;  // include/AmrSim.h:36

struct Level {
  bool defined = false;
  int lo[3] = {0, 0, 0}, hi[3] = {-1, -1, -1};  // valid box, global level coordinates
  Box3 box{};
  void* buf[3] = {nullptr, nullptr, nullptr};
  int now = 0, next = 1, tmp = 2;
  // pull form: "now" holds Q_n = C(R_{n-1}), the previous step's
  // post-collision populations of a periodic single level, instead of R_n
  // (see cells.cuh); readouts gather R_n = S(Q_n) through it
  bool pform = false;
  // buf[next] already holds the step after "now": CalcHydroVars ran that step
  // with the hydrodynamic fields as its epilogue, and the next Iterate takes it
  bool spec_next = false;
  double* d_rho = nullptr;
  double* d_u = nullptr;
  // host copy of the level's Density / velocity fields for the getters;
  // refreshed from d_rho / d_u on first use after the device fields change
  mutable std::vector<double> h_rho, h_u;
  mutable bool host_stale = false;
  double time = 0.0, dt = 0.0;
  int step = 0;
  double tau_s = 0.0, tau_b = 0.0, mass = 0.0;
  size_t cells() const { return (size_t)box.n[0] * box.n[1] * box.n[2]; }
  bool contains(int i, int j, int k) const {
    return i >= lo[0] && i <= hi[0] && j >= lo[1] && j <= hi[1] && k >= lo[2] && k <= hi[2];
  }
};

}  // namespace

namespace {
// What a captured step graph depends on, per level: geometry, the buffers and
// which of them plays which role, the form of the store and the rates.
struct LevelSig {
  bool defined = false;
  int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
  void* buf[3] = {nullptr, nullptr, nullptr};
  int now = 0, next = 0, tmp = 0;
  bool pform = false;
  double tau_s = 0.0, tau_b = 0.0;
  bool operator==(const LevelSig& o) const {
    for (int d = 0; d < 3; ++d)
      if (lo[d] != o.lo[d] || hi[d] != o.hi[d] || buf[d] != o.buf[d]) return false;
    return defined == o.defined && now == o.now && next == o.next && tmp == o.tmp &&
           pform == o.pform && tau_s == o.tau_s && tau_b == o.tau_b;
  }
};

// A CUDA graph of `period` whole macro steps, captured from the simulation's
// own launches.  After `period` steps every level's buffers are back in their
// roles, so the graph can be replayed as long as the state matches `sig`.
struct StepGraph {
  cudaGraphExec_t exec = nullptr;
  int period = 0;
  long long launches = 0;       // kernels per replay
  std::vector<LevelSig> sig;    // state before (and after) one replay
  int finest = -1;
  double rho0 = 0.0;
  std::vector<double> dtime;    // per-level bookkeeping of one replay
  std::vector<int> dstep;
};
}  // namespace

struct lbx_sim {
  int N[3] = {0, 0, 0};
  int max_level = 0;
  int precision = LBX_F64;
  int amr_mode = LBX_AMR_FAITHFUL;
  int finest = 0;
  bool initialised = false;
  bool restrict_pending = false;  // conservative mode: covered cells not yet restricted
  double tau_s0 = 0.0, tau_b0 = 0.0;
  double rho0 = 0.0;  // population shift of the FP32 store
  std::vector<Level> lev;
  // Initial vectors (C order).  The library keeps its own copy, as the
  // reference does (src/AmrSim.cpp:804-822), but on the device: each Set call
  // uploads the caller's vector at once, a scalar is kept as a value.
  double* d_init[2] = {nullptr, nullptr};  // rho, u
  size_t n_init[2] = {0, 0};               // elements given (a scalar counts as a full field)
  bool init_scalar[2] = {false, false};
  double init_value[2] = {0.0, 0.0};
  cudaStream_t stream = nullptr;
  double* d_partials = nullptr;
  double* d_out4 = nullptr;
  double* h_out4 = nullptr;
  long long launches = 0;  // kernels issued by lbx_iterate (counted per launch)
  // replayable macro steps (lbx_iterate): the two most recent captures, since
  // a step taken ahead by CalcHydroVars swaps the store roles between calls
  StepGraph graphs[2];
  int gcur = 0;            // the slot that matched or was captured last
  // CalcHydroVars on a single pull-form level runs the next step with the
  // fields as its epilogue once the program has shown that it steps on after
  // reading fields (an Iterate after a CalcHydroVars); until then it runs the
  // hydro pass alone, so that a final readout costs no extra step
  bool fuse_hydro = false;
  bool hydro_since_iterate = false;
  int nbuf() const { return amr_mode == LBX_AMR_FAITHFUL ? 3 : 2; }
  // FP64 store (LBX_F64 and LBX_F64_PAIRED) or FP32 shifted store
  bool f64() const { return precision != LBX_F32_SHIFTED; }
  size_t esize() const { return f64() ? sizeof(double) : sizeof(float); }
  int dn(int L, int d) const { return N[d] << L; }
};

namespace {

void free_level(Level& l) {
  for (auto& p : l.buf)
    if (p) {
      cudaFree(p);
      p = nullptr;
    }
  if (l.d_rho) cudaFree(l.d_rho);
  if (l.d_u) cudaFree(l.d_u);
  l.d_rho = l.d_u = nullptr;
  l.h_rho.clear();
  l.h_u.clear();
  l.h_rho.shrink_to_fit();
  l.h_u.shrink_to_fit();
  l.defined = false;
  l.now = 0;
  l.next = 1;
  l.tmp = 2;
  l.pform = false;
  l.spec_next = false;
}

int define_level(lbx_sim* s, int L, const int* lo, const int* hi, int ghost) {
  Level& l = s->lev[L];
  free_level(l);
  for (int d = 0; d < 3; ++d) {
    l.lo[d] = lo[d];
    l.hi[d] = hi[d];
  }
  l.box = lbx::make_box(hi[0] - lo[0] + 1, hi[1] - lo[1] + 1, hi[2] - lo[2] + 1, ghost);
  const size_t bytes = (size_t)lbx::NV * (size_t)l.box.sq * s->esize();
  // a single periodic level (no ghost, no covered cell) has every entry of
  // its stores written before it is read: by the initialisation or an
  // import, then by each step; other levels start from zeros
  const bool every_entry_written = L == 0 && ghost == 0 && s->max_level == 0 && s->nbuf() == 2;
  for (int b = 0; b < s->nbuf(); ++b) {
    CK(cudaMalloc(&l.buf[b], bytes));
    if (!every_entry_written) CK(cudaMemsetAsync(l.buf[b], 0, bytes, s->stream));
  }
  CK(cudaMalloc(&l.d_rho, l.cells() * sizeof(double)));
  CK(cudaMalloc(&l.d_u, 3 * l.cells() * sizeof(double)));
  l.defined = true;
  return LBX_OK;
}

IBox rel_box(const Level& l, const int* glo, const int* ghi) {
  IBox b;
  for (int d = 0; d < 3; ++d) {
    b.lo[d] = glo[d] - l.lo[d];
    b.hi[d] = ghi[d] - l.lo[d];
  }
  return b;
}

int crs(int x) { return x >= 0 ? x / 2 : -((-x + 1) / 2); }

// cells of level L whose dynamics are replaced by level L+1
IBox covered_box(const lbx_sim* s, int L) {
  const Level& l = s->lev[L];
  int glo[3], ghi[3];
  if (s->amr_mode == LBX_AMR_FAITHFUL) {
    // MakeFineMask passes the coarse BoxArray as the fine one
    // (src/AmrSim.cpp:421-425): the mask is coarsen(own box).
    for (int d = 0; d < 3; ++d) {
      glo[d] = crs(l.lo[d]);
      ghi[d] = crs(l.hi[d]);
    }
  } else {
    if (L >= s->finest) return lbx::empty_ibox();
    const Level& f = s->lev[L + 1];
    for (int d = 0; d < 3; ++d) {
      glo[d] = f.lo[d] / 2;
      ghi[d] = f.hi[d] / 2;
    }
  }
  return rel_box(l, glo, ghi);
}

// cells of level L covered by level L+1 (composite-mass bookkeeping)
IBox true_cover(const lbx_sim* s, int L) {
  if (L >= s->finest) return lbx::empty_ibox();
  const Level& f = s->lev[L + 1];
  int glo[3], ghi[3];
  for (int d = 0; d < 3; ++d) {
    glo[d] = f.lo[d] / 2;
    ghi[d] = f.hi[d] / 2;
  }
  return rel_box(s->lev[L], glo, ghi);
}

Coupling coupling(const lbx_sim* s, int L) {  // levels (L-1, L)
  Coupling c;
  const Level& cl = s->lev[L - 1];
  const Level& fl = s->lev[L];
  c.cb = cl.box;
  c.fb = fl.box;
  for (int d = 0; d < 3; ++d) {
    c.clo[d] = cl.lo[d];
    c.flo[d] = fl.lo[d];
    c.cdom[d] = s->dn(L - 1, d);
  }
  c.cper = (L - 1 == 0) ? 1 : 0;
  return c;
}

double omega(double tau) { return 1.0 / (tau + 0.5); }  // src/AmrSim.cpp:125-126

template <typename T>
T* P(void* p) {
  return static_cast<T*>(p);
}

// ComputeDt (src/AmrSim.cpp:297-322).  Faithful: tau_l = r(tau_{l-1} - 1/2)
// + 1/2 as the reference; conservative and rescaled: tau_l = r tau_{l-1},
// the rule that keeps the viscosity of omega = 1/(tau + 1/2) across levels.
void compute_dt(lbx_sim* s, int L) {
  Level& l = s->lev[L];
  if (L) {
    const Level& c = s->lev[L - 1];
    const int r = 2;
    l.dt = c.dt / r;
    l.mass = c.mass / r;
    if (s->amr_mode == LBX_AMR_FAITHFUL) {
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

// Host copy of a level's density and velocity for the point getters, made
// on first use after the device fields change (allocated on first use too).
int refresh_host(const lbx_sim* s, const Level& l) {
  if (!l.host_stale && l.h_rho.size() == l.cells()) return LBX_OK;
  if (l.h_rho.size() != l.cells()) {
    l.h_rho.resize(l.cells());
    l.h_u.resize(3 * l.cells());
  }
  CK(lbx::download_host(l.h_rho.data(), l.d_rho, l.cells() * sizeof(double), s->stream));
  CK(lbx::download_host(l.h_u.data(), l.d_u, 3 * l.cells() * sizeof(double), s->stream));
  l.host_stale = false;
  return LBX_OK;
}

template <typename T>
int calc_hydro_T(lbx_sim* s, int L) {
  Level& l = s->lev[L];
  if (L == 0 && s->finest == 0 && l.pform && s->fuse_hydro) {
    // the next step with the fields of the current state as its epilogue:
    // the same rho and u as the hydro pass, and the next state ready in
    // buf[next] for the next Iterate (which then skips that step)
    CK(lbx::launch_step_pull_hydro<T>(P<T>(l.buf[l.now]), P<T>(l.buf[l.next]), l.box,
                                      omega(l.tau_s), omega(l.tau_b), s->rho0,
                                      s->precision == LBX_F64_PAIRED, l.d_rho, l.d_u, s->stream));
    l.spec_next = true;
  } else {
    CK(lbx::launch_hydro<T>(P<T>(l.buf[l.now]), l.box, s->rho0, l.d_rho, l.d_u, s->stream,
                            l.pform));
  }
  s->hydro_since_iterate = true;
  l.host_stale = true;  // the getters copy to the host on first use
  CK(cudaStreamSynchronize(s->stream));
  return LBX_OK;
}
int calc_hydro(lbx_sim* s, int L) {
  return s->f64() ? calc_hydro_T<double>(s, L) : calc_hydro_T<float>(s, L);
}

// ---- single level -------------------------------------------------------
// One step of the periodic single level in the pull form: the store holds
// Q_n = C(R_{n-1}) (so that R_n = S(Q_n)) and the kernel maps it to
// Q_{n+1} = C(S(Q_n)); entering the form shifts the stored R back once.
template <typename T>
int step_single(lbx_sim* s) {
  Level& l = s->lev[0];
  const bool paired = s->precision == LBX_F64_PAIRED;
  if (!l.pform) {
    CK(lbx::launch_unstream<T>(P<T>(l.buf[l.now]), P<T>(l.buf[l.next]), l.box, s->stream));
    std::swap(l.now, l.next);
    ++s->launches;
    l.pform = true;
  }
  CK(lbx::launch_step_pull<T>(P<T>(l.buf[l.now]), P<T>(l.buf[l.next]), l.box, omega(l.tau_s),
                              omega(l.tau_b), s->rho0, paired, s->stream));
  ++s->launches;
  std::swap(l.now, l.next);
  l.time += l.dt;  // IterateLevel (src/AmrSim.cpp:324-333)
  ++l.step;
  return LBX_OK;
}

// Leave the pull form: now <- S(now) = R.
template <typename T>
int to_rform_T(lbx_sim* s, Level& l) {
  l.spec_next = false;
  CK(lbx::launch_stream_gather<T>(P<T>(l.buf[l.now]), P<T>(l.buf[l.next]), l.box, s->stream));
  std::swap(l.now, l.next);
  l.pform = false;
  return LBX_OK;
}
int ensure_rform(lbx_sim* s, int L) {
  Level& l = s->lev[L];
  if (!l.defined || !l.pform) return LBX_OK;
  return s->f64() ? to_rform_T<double>(s, l) : to_rform_T<float>(s, l);
}

// ---- reference-faithful Rohde cycle (FP64) ------------------------------
double* DB(Level& l, int which) { return static_cast<double*>(l.buf[which]); }

int f_init_post_collision(lbx_sim* s, int L) {  // src/AmrSim.cpp:471-485
  Level& l = s->lev[L];
  s->launches += (L == 0) ? 1 : 2;
  if (L == 0) {
    CK(lbx::launch_f_fill_single(DB(l, l.now), DB(l, l.next), l.box, s->stream));
  } else {
    Level& c = s->lev[L - 1];
    const Coupling cp = coupling(s, L);
    const int fdom[3] = {s->dn(L, 0), s->dn(L, 1), s->dn(L, 2)};
    CK(lbx::launch_f_fill_two(DB(l, l.now), DB(l, l.next), DB(c, c.now), cp, fdom, s->stream));
    CK(lbx::launch_f_zero_ring0(DB(l, l.next), l.box, s->stream));
  }
  return LBX_OK;
}
int f_collide(lbx_sim* s, int L, bool masked) {
  Level& l = s->lev[L];
  const IBox cov = masked ? covered_box(s, L) : lbx::empty_ibox();
  ++s->launches;
  CK(lbx::launch_f_collide(DB(l, l.next), l.box, cov, omega(l.tau_s), omega(l.tau_b), s->stream,
                           s->precision == LBX_F64_PAIRED));
  return LBX_OK;
}
int f_stream(lbx_sim* s, int L) {  // src/AmrSim.cpp:109-122 (fresh, zeroed buffer)
  Level& l = s->lev[L];
  CK(cudaMemsetAsync(l.buf[l.tmp], 0, (size_t)lbx::NV * l.box.sq * sizeof(double), s->stream));
  CK(lbx::launch_f_stream(DB(l, l.next), DB(l, l.tmp), l.box, s->stream));
  ++s->launches;
  std::swap(l.next, l.tmp);
  return LBX_OK;
}
void f_update_distribution(lbx_sim* s, int L) {  // src/AmrSim.cpp:619-631
  Level& l = s->lev[L];
  if (L && L == s->finest) {
    l.time += 2 * l.dt;
    l.step += 2;
  } else {
    l.time += l.dt;
    ++l.step;
  }
  std::swap(l.now, l.next);
}
int f_rohde_cycle(lbx_sim* s, int L) {  // src/AmrSim.cpp:430-469
  RET(f_init_post_collision(s, L));
  RET(f_collide(s, L, true));
  if (L + 1 == s->finest) {
    const int F = s->finest;
    RET(f_init_post_collision(s, F));
    RET(f_collide(s, F, false));
    RET(f_stream(s, F));
    RET(f_collide(s, F, false));
    RET(f_stream(s, F));
    CK(lbx::launch_f_zero_invalid(DB(s->lev[F], s->lev[F].next), s->lev[F].box, s->stream));
    ++s->launches;
    f_update_distribution(s, F);
  } else {
    for (int it = 0; it < 2; ++it) RET(f_rohde_cycle(s, L + 1));
  }
  Level& l = s->lev[L];
  RET(f_stream(s, L));
  {
    Level& f = s->lev[L + 1];
    CK(lbx::launch_f_sum_from_fine(DB(f, f.now), DB(l, l.next), coupling(s, L + 1), s->stream));
  }
  CK(lbx::launch_f_zero_invalid(DB(l, l.next), l.box, s->stream));
  if (L == 0) CK(lbx::launch_f_fill_boundary(DB(l, l.next), l.box, s->stream));
  s->launches += (L == 0) ? 3 : 2;
  f_update_distribution(s, L);
  return LBX_OK;
}

// ---- conservative volumetric scheme ------------------------------------
template <typename T>
int c_advance(lbx_sim* s, int L) {
  Level& l = s->lev[L];
  const bool paired = s->precision == LBX_F64_PAIRED;
  if (L < s->finest) {
    Level& f = s->lev[L + 1];
    CK(lbx::launch_explode<T>(P<T>(l.buf[l.now]), P<T>(f.buf[f.now]), coupling(s, L + 1),
                              omega(l.tau_s), omega(l.tau_b), s->rho0, s->stream, paired));
  }
  const IBox cov = covered_box(s, L);
  s->launches += (L < s->finest) ? 3 : 1;  // explode, step, coalesce
  if (L == 0)
    CK(lbx::launch_step_periodic<T>(P<T>(l.buf[l.now]), P<T>(l.buf[l.next]), l.box, cov,
                                    omega(l.tau_s), omega(l.tau_b), s->rho0, s->stream, 128,
                                    paired));
  else
    CK(lbx::launch_step_patch<T>(P<T>(l.buf[l.now]), P<T>(l.buf[l.next]), l.box, cov,
                                 omega(l.tau_s), omega(l.tau_b), s->rho0, s->stream, paired));
  std::swap(l.now, l.next);
  if (L < s->finest) {
    RET(c_advance<T>(s, L + 1));
    RET(c_advance<T>(s, L + 1));
    Level& f = s->lev[L + 1];
    const Coupling cp = coupling(s, L + 1);
    CK(lbx::launch_coalesce<T>(P<T>(f.buf[f.now]), P<T>(l.buf[l.now]), cp, s->rho0, s->stream));
    // covered coarse cells do not take part in the dynamics: their restricted
    // values are produced on demand by ensure_restricted
    s->restrict_pending = true;
  }
  l.time += l.dt;
  ++l.step;
  return LBX_OK;
}

// ---- rescaled coupling ---------------------------------------------------
// Rates of the transfers between levels L-1 and L.  The fine level sees the
// coarse non-equilibrium moments scaled by a = w_c / (2 w_f) (w = 1/(tau +
// 1/2) per rate: the non-equilibrium stress goes as 1/w times the time step;
// Dupuis & Chopard 2003); a post-collision fine state is then the coarse
// pre-collision state collided at 1 - (1 - w_f) a, and a coarse state is
// the fine mean collided at 1 - 1/a.
struct ResRates {
  double es, eb;  // explosion
  double rs, rb;  // restriction
};
ResRates resc_rates(const lbx_sim* s, int L) {
  const Level& c = s->lev[L - 1];
  const Level& f = s->lev[L];
  const double wcs = omega(c.tau_s), wcb = omega(c.tau_b);
  const double wfs = omega(f.tau_s), wfb = omega(f.tau_b);
  const double as = wcs / (2.0 * wfs), ab = wcb / (2.0 * wfb);
  return ResRates{1.0 - (1.0 - wfs) * as, 1.0 - (1.0 - wfb) * ab, 1.0 - 1.0 / as, 1.0 - 1.0 / ab};
}

// One step of level L and, inside it, two sub-steps of every finer level:
// the level steps first (covered cells collide like the others), then
// before each fine sub-step k the fine ghost shell is refilled from the
// parents at time t + k/2 (linear between the level's state before the step,
// now in "next", and after it), and after the two sub-steps the covered
// cells take the restricted fine state.
template <typename T>
int r_advance(lbx_sim* s, int L) {
  Level& l = s->lev[L];
  const bool paired = s->precision == LBX_F64_PAIRED;
  ++s->launches;
  if (L == 0)
    CK(lbx::launch_step_periodic<T>(P<T>(l.buf[l.now]), P<T>(l.buf[l.next]), l.box,
                                    lbx::empty_ibox(), omega(l.tau_s), omega(l.tau_b), s->rho0,
                                    s->stream, 128, paired));
  else
    CK(lbx::launch_step_patch<T>(P<T>(l.buf[l.now]), P<T>(l.buf[l.next]), l.box,
                                 lbx::empty_ibox(), omega(l.tau_s), omega(l.tau_b), s->rho0,
                                 s->stream, paired));
  std::swap(l.now, l.next);
  if (L < s->finest) {
    Level& f = s->lev[L + 1];
    const Coupling cp = coupling(s, L + 1);
    const ResRates R = resc_rates(s, L + 1);
    for (int k = 0; k < 2; ++k) {
      CK(lbx::launch_explode_resc<T>(P<T>(l.buf[l.next]), P<T>(l.buf[l.now]), P<T>(f.buf[f.now]),
                                     cp, R.es, R.eb, s->rho0, 1.0 - 0.5 * k, 0.5 * k, s->stream,
                                     paired));
      ++s->launches;
      RET(r_advance<T>(s, L + 1));
    }
    CK(lbx::launch_restrict_resc<T>(P<T>(f.buf[f.now]), P<T>(l.buf[l.now]), cp, R.rs, R.rb,
                                    s->rho0, s->stream, paired));
    ++s->launches;
  }
  l.time += l.dt;
  ++l.step;
  return LBX_OK;
}

// Covered coarse cells <- mean of their children, finest pair first (the
// conservative scheme's output view of the coarse levels).
template <typename T>
int restrict_all_T(lbx_sim* s) {
  for (int L = s->finest; L >= 1; --L) {
    Level& f = s->lev[L];
    Level& c = s->lev[L - 1];
    CK(lbx::launch_restrict<T>(P<T>(f.buf[f.now]), P<T>(c.buf[c.now]), coupling(s, L), s->stream));
  }
  return LBX_OK;
}
int ensure_restricted(lbx_sim* s) {
  if (!s->restrict_pending) return LBX_OK;
  s->restrict_pending = false;
  return s->f64() ? restrict_all_T<double>(s) : restrict_all_T<float>(s);
}

template <typename T>
int fill_from_coarse_T(lbx_sim* s, int L) {
  Level& f = s->lev[L];
  Level& c = s->lev[L - 1];
  CK(lbx::launch_fill_from_coarse<T>(P<T>(c.buf[c.now]), P<T>(f.buf[f.now]), coupling(s, L),
                                     s->stream));
  return LBX_OK;
}

int check_level(const lbx_sim* s, int level) {
  if (!s) return LBX_ERR_ARG;
  if (level < 0 || level > s->max_level) return LBX_ERR_ARG;
  if (!s->lev[level].defined) return LBX_ERR_STATE;
  return LBX_OK;
}

std::mutex g_scratch_mu;
std::map<int, double*> g_scratch;  // device -> partial-sum scratch of the device-pointer reduce

}  // namespace

namespace {
// ---- one macro step and its CUDA-graph replay -----------------------------
// One step of the coarsest level, with every finer level sub-cycled inside it.
int macro_step(lbx_sim* s) {
  if (s->finest == 0) return s->f64() ? step_single<double>(s) : step_single<float>(s);
  if (s->amr_mode == LBX_AMR_FAITHFUL) return f_rohde_cycle(s, 0);
  if (s->amr_mode == LBX_AMR_RESCALED)
    return s->f64() ? r_advance<double>(s, 0) : r_advance<float>(s, 0);
  return s->f64() ? c_advance<double>(s, 0) : c_advance<float>(s, 0);
}

constexpr int kGraphMinSteps = 4;   // shorter runs launch directly
constexpr int kGraphMaxPeriod = 12; // buffer roles cycle with a period dividing 6 or 2

std::vector<LevelSig> signature(const lbx_sim* s) {
  std::vector<LevelSig> v(s->lev.size());
  for (size_t L = 0; L < s->lev.size(); ++L) {
    const Level& l = s->lev[L];
    LevelSig& g = v[L];
    g.defined = l.defined && (int)L <= s->finest;
    if (!g.defined) continue;
    for (int d = 0; d < 3; ++d) {
      g.lo[d] = l.lo[d];
      g.hi[d] = l.hi[d];
      g.buf[d] = l.buf[d];
    }
    g.now = l.now;
    g.next = l.next;
    g.tmp = l.tmp;
    g.pform = l.pform;
    g.tau_s = l.tau_s;
    g.tau_b = l.tau_b;
  }
  return v;
}

bool graph_matches(lbx_sim* s) {
  const std::vector<LevelSig> sig = signature(s);
  for (int i = 0; i < 2; ++i) {
    const StepGraph& G = s->graphs[i];
    if (G.exec && G.finest == s->finest && G.rho0 == s->rho0 && sig == G.sig) {
      s->gcur = i;
      return true;
    }
  }
  return false;
}

// Capture macro steps from the simulation's own launches until every level's
// buffers are back in their roles, then run the captured steps once (the
// host-side bookkeeping already advanced while capturing).  Keeps the graph
// for replay when the roles did return.
int capture_graph(lbx_sim* s, int* left) {
  s->gcur ^= 1;  // replaces the older of the two captures
  StepGraph& G = s->graphs[s->gcur];
  if (G.exec) {
    CK(cudaStreamSynchronize(s->stream));
    cudaGraphExecDestroy(G.exec);
    G.exec = nullptr;
  }
  const std::vector<LevelSig> sig0 = signature(s);
  std::vector<double> t0(s->lev.size());
  std::vector<int> n0(s->lev.size());
  for (size_t L = 0; L < s->lev.size(); ++L) {
    t0[L] = s->lev[L].time;
    n0[L] = s->lev[L].step;
  }
  const long long launches0 = s->launches;
  CK(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
  int m = 0, rc = LBX_OK;
  do {
    rc = macro_step(s);
    ++m;
  } while (rc == LBX_OK && m < std::min(kGraphMaxPeriod, *left) && !(signature(s) == sig0));
  cudaGraph_t g = nullptr;
  const cudaError_t e = cudaStreamEndCapture(s->stream, &g);
  if (rc != LBX_OK || e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    if (rc != LBX_OK) return rc;
    CK(e);
  }
  cudaGraphExec_t exec = nullptr;
  const cudaError_t ei = cudaGraphInstantiate(&exec, g, 0);
  cudaGraphDestroy(g);
  CK(ei);
  CK(cudaGraphLaunch(exec, s->stream));  // the m steps just captured
  *left -= m;
  if (!(signature(s) == sig0)) {  // not replayable: run once, drop
    CK(cudaStreamSynchronize(s->stream));
    cudaGraphExecDestroy(exec);
    return LBX_OK;
  }
  G.exec = exec;
  G.period = m;
  G.launches = s->launches - launches0;
  G.sig = sig0;
  G.finest = s->finest;
  G.rho0 = s->rho0;
  G.dtime.assign(s->lev.size(), 0.0);
  G.dstep.assign(s->lev.size(), 0);
  for (size_t L = 0; L < s->lev.size(); ++L) {
    G.dtime[L] = s->lev[L].time - t0[L];  // exact: dt is a power of two
    G.dstep[L] = s->lev[L].step - n0[L];
  }
  return LBX_OK;
}

int replay_graph(lbx_sim* s) {
  StepGraph& G = s->graphs[s->gcur];
  CK(cudaGraphLaunch(G.exec, s->stream));
  for (size_t L = 0; L < s->lev.size() && L < G.dtime.size(); ++L) {
    s->lev[L].time += G.dtime[L];
    s->lev[L].step += G.dstep[L];
  }
  s->launches += G.launches;
  if (s->amr_mode == LBX_AMR_CONSERVATIVE && s->finest > 0) s->restrict_pending = true;
  return LBX_OK;
}

// ---- checkpoint file -------------------------------------------------------
constexpr char kCkptMagic[8] = {'L', 'B', 'X', 'C', 'K', 'P', 'T', '1'};
struct CkptHeader {
  char magic[8];
  int32_t version, precision, amr_mode, n[3], max_level, finest;
  double tau_s0, tau_b0, rho0;
};
struct CkptLevel {
  int32_t lo[3], hi[3];
  double time, dt, tau_s, tau_b, mass;
  int64_t step;
};

// the valid cells of level L's current store, packed (storage type)
int pack_level(lbx_sim* s, int L, std::vector<char>& out) {
  Level& l = s->lev[L];
  const size_t bytes = (size_t)lbx::NV * l.cells() * s->esize();
  out.resize(bytes);
  void* d = nullptr;
  CK(cudaMalloc(&d, bytes));
  cudaError_t e = s->f64() ? lbx::launch_pack<double>(P<double>(l.buf[l.now]), l.box, P<double>(d), s->stream)
                           : lbx::launch_pack<float>(P<float>(l.buf[l.now]), l.box, P<float>(d), s->stream);
  if (e == cudaSuccess) e = lbx::download_host(out.data(), d, bytes, s->stream);
  cudaFree(d);
  CK(e);
  return LBX_OK;
}
int unpack_level(lbx_sim* s, int L, const std::vector<char>& in) {
  Level& l = s->lev[L];
  void* d = nullptr;
  CK(cudaMalloc(&d, in.size()));
  cudaError_t e = lbx::upload_host(d, in.data(), in.size(), s->stream);
  if (e == cudaSuccess)
    e = s->f64() ? lbx::launch_unpack<double>(P<double>(d), P<double>(l.buf[l.now]), l.box, s->stream)
                 : lbx::launch_unpack<float>(P<float>(d), P<float>(l.buf[l.now]), l.box, s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  cudaFree(d);
  CK(e);
  return LBX_OK;
}

// Keep initial vector k (0 = density, 1 = velocity; `per_cell` values per
// cell): a scalar broadcasts to the whole field (src/AmrSim.cpp:804-807,
// 814-817), a vector is copied (:809-812, 819-822) -- here straight to the
// device, before the call returns, so the caller may reuse its buffer.
int keep_initial(lbx_sim* s, int k, const double* v, size_t n, size_t per_cell) {
  if (s->d_init[k]) {
    CK(cudaStreamSynchronize(s->stream));
    CK(cudaFree(s->d_init[k]));
    s->d_init[k] = nullptr;
  }
  const size_t numel = (size_t)s->N[0] * s->N[1] * s->N[2];
  s->init_scalar[k] = (n == 1);
  if (n == 1) {
    s->init_value[k] = v[0];
    s->n_init[k] = per_cell * numel;
    return LBX_OK;
  }
  s->n_init[k] = n;
  if (n == 0) return LBX_OK;
  // a plain allocation: growing the stream-ordered pool by gigabytes after
  // it was trimmed costs more than the copy itself
  CK(cudaMalloc(&s->d_init[k], n * sizeof(double)));
  CK(lbx::upload_host(s->d_init[k], v, n * sizeof(double), s->stream));
  return LBX_OK;
}
void drop_initial(lbx_sim* s) {
  for (int k = 0; k < 2; ++k)
    if (s->d_init[k]) {
      cudaFree(s->d_init[k]);
      s->d_init[k] = nullptr;
    }
}
}  // namespace

namespace {
// whole field of a level into the caller's buffer: from the host copy when
// it is current, else from the device (no host cache is made)
int field_out(const lbx_sim* s, const Level& l, const double* dev,
              const std::vector<double>& host, size_t count, double* out) {
  if (!l.host_stale && host.size() == count) {
    std::memcpy(out, host.data(), count * sizeof(double));
    return LBX_OK;
  }
  CK(lbx::download_host(out, dev, count * sizeof(double), s->stream));
  return LBX_OK;
}

// Whether the tag box tlo..thi (inclusive, level-`level` cells, inside the
// domain) may become level level+1 under the parent box plo..phi: it nests in
// the parent, with one parent cell of margin above level 0; in the
// conservative and rescaled modes the exchange ring around a level-1 patch does not wrap
// onto the patch; and the new level's cells fit 32-bit indices.
int check_tag_box(int amr_mode, const int* N, int level, const int* plo, const int* phi,
                  const int* tlo, const int* thi) {
  for (int d = 0; d < 3; ++d) {
    if (thi[d] < tlo[d]) return LBX_ERR_ARG;
    if (tlo[d] < plo[d] || thi[d] > phi[d]) return LBX_ERR_ARG;
    if (level > 0 && (tlo[d] - 1 < plo[d] || thi[d] + 1 > phi[d])) return LBX_ERR_ARG;
    if (amr_mode != LBX_AMR_FAITHFUL && level == 0 && thi[d] - tlo[d] + 1 > N[d] - 2)
      return LBX_ERR_UNSUPPORTED;
  }
  if (8ll * (thi[0] - tlo[0] + 1) * (thi[1] - tlo[1] + 1) * (thi[2] - tlo[2] + 1) >= (1ll << 31))
    return LBX_ERR_UNSUPPORTED;
  return LBX_OK;
}
}  // namespace

#ifdef LBX_CHECKED
namespace lbx {
// readers of the per-unit bounds counters, registered while the library loads
static std::vector<OobReader>& oob_readers() {
  static std::vector<OobReader> v;
  return v;
}
int register_oob_reader(OobReader r) {
  oob_readers().push_back(r);
  return 1;
}
}  // namespace lbx
#endif

extern "C" {

const char* lbx_status_string(int st) {
  switch (st) {
    case LBX_OK: return "ok";
    case LBX_ERR_ARG: return "invalid argument";
    case LBX_ERR_STATE: return "invalid state for this call";
    case LBX_ERR_CUDA: return lbx::g_last_error[0] ? lbx::g_last_error : "CUDA error";
    case LBX_ERR_OOM: return "out of device memory";
    case LBX_ERR_UNSUPPORTED: return "unsupported configuration";
    case LBX_ERR_RANGE: return "initial vector shorter than the domain";
    case LBX_ERR_TIMEOUT: return "bounded device wait timed out";
    case LBX_ERR_NOT_FOUND: return "point not on this level";
    case LBX_ERR_IO: return "checkpoint file unreadable or unwritable";
    default: return "unknown status";
  }
}

double lbx_nl_density(void) { return kNL_DENSITY; }
double lbx_nl_velocity(void) { return kNL_VELOCITY; }

int lbx_debug_bounds(long long* count, long long* first_bad_index, int reset) {
  if (!count || !first_bad_index) return LBX_ERR_ARG;
#ifdef LBX_CHECKED
  CK(cudaDeviceSynchronize());  // counters are final once every kernel is done
  unsigned long long total = 0;
  long long first = -1;
  for (lbx::OobReader r : lbx::oob_readers()) {
    unsigned long long n = 0;
    long long f = 0;
    if (r(&n, &f, reset != 0) != 0) return LBX_ERR_CUDA;
    if (n && first < 0) first = f;
    total += n;
  }
  *count = (long long)total;
  *first_bad_index = first;
  return LBX_OK;
#else
  *count = 0;
  *first_bad_index = -1;
  (void)reset;
  return LBX_ERR_UNSUPPORTED;
#endif
}

int lbx_init(void) {
  int n = 0;
  CK(cudaGetDeviceCount(&n));
  if (n <= 0) return LBX_ERR_CUDA;
  CK(cudaFree(nullptr));
  return LBX_OK;
}

int lbx_set_device(int device) {
  int n = 0;
  CK(cudaGetDeviceCount(&n));
  if (device < 0 || device >= n) return LBX_ERR_ARG;
  CK(cudaSetDevice(device));
  return LBX_OK;
}

int lbx_finalize(void) {
  std::lock_guard<std::mutex> g(g_scratch_mu);
  int cur = 0;
  cudaGetDevice(&cur);
  for (auto& kv : g_scratch) {
    cudaSetDevice(kv.first);
    cudaFree(kv.second);
  }
  g_scratch.clear();
  cudaSetDevice(cur);
  return LBX_OK;
}

int lbx_create(int nx, int ny, int nz, int max_level, const int* periodicity, double tau_s,
               double tau_b, int precision, int amr_mode, lbx_sim** out) {
  if (!out) return LBX_ERR_ARG;
  *out = nullptr;
  if (nx <= 0 || ny <= 0 || nz <= 0 || max_level < 0 || max_level > 8) return LBX_ERR_ARG;
  if ((long long)nx * ny * nz >= (1ll << 31)) return LBX_ERR_UNSUPPORTED;  // 32-bit cell indices
  if (precision != LBX_F64 && precision != LBX_F32_SHIFTED && precision != LBX_F64_PAIRED)
    return LBX_ERR_ARG;
  if (amr_mode != LBX_AMR_FAITHFUL && amr_mode != LBX_AMR_CONSERVATIVE &&
      amr_mode != LBX_AMR_RESCALED)
    return LBX_ERR_ARG;
  // only periodic boundaries (src/AmrSim.cpp:788-797)
  if (!periodicity || !periodicity[0] || !periodicity[1] || !periodicity[2])
    return LBX_ERR_UNSUPPORTED;
  if (precision == LBX_F32_SHIFTED && amr_mode == LBX_AMR_FAITHFUL && max_level > 0)
    return LBX_ERR_UNSUPPORTED;  // the faithful cycle zeroes raw f; FP64 only
  int ndev = 0;
  CK(cudaGetDeviceCount(&ndev));
  if (ndev <= 0) return LBX_ERR_CUDA;
  lbx_sim* s = new lbx_sim();
  s->N[0] = nx;
  s->N[1] = ny;
  s->N[2] = nz;
  s->max_level = max_level;
  s->precision = precision;
  s->amr_mode = amr_mode;
  s->tau_s0 = tau_s;
  s->tau_b0 = tau_b;
  s->lev.resize(max_level + 1);
  s->lev[0].tau_s = tau_s;  // src/AmrSim.cpp:800-801
  s->lev[0].tau_b = tau_b;
  cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&s->d_partials, lbx::reduce_partials_doubles() * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&s->d_out4, 4 * sizeof(double));
  if (e == cudaSuccess) e = cudaMallocHost(&s->h_out4, 4 * sizeof(double));
  if (e != cudaSuccess) {
    lbx::note_error("lbx_create", e);
    lbx_destroy(s);
    return lbx::status_from_cuda(e);
  }
  *out = s;
  return LBX_OK;
}

int lbx_destroy(lbx_sim* s) {
  if (!s) return LBX_OK;
  if (s->stream) cudaStreamSynchronize(s->stream);
  for (auto& G : s->graphs)
    if (G.exec) cudaGraphExecDestroy(G.exec);
  for (auto& l : s->lev) free_level(l);
  drop_initial(s);
  if (s->stream) cudaStreamSynchronize(s->stream);
  if (s->d_partials) cudaFree(s->d_partials);
  if (s->d_out4) cudaFree(s->d_out4);
  if (s->h_out4) cudaFreeHost(s->h_out4);
  if (s->stream) cudaStreamDestroy(s->stream);
  delete s;
  return LBX_OK;
}

int lbx_set_initial_density(lbx_sim* s, const double* rho, size_t n) {
  if (!s || (!rho && n)) return LBX_ERR_ARG;
  lbx::Range range("lbx_set_initial_density");
  return keep_initial(s, 0, rho, n, 1);
}

int lbx_set_initial_velocity(lbx_sim* s, const double* u, size_t n) {
  if (!s || (!u && n)) return LBX_ERR_ARG;
  lbx::Range range("lbx_set_initial_velocity");
  return keep_initial(s, 1, u, n, 3);
}

int lbx_init_from_scratch(lbx_sim* s, double time) {
  if (!s) return LBX_ERR_ARG;
  lbx::Range range("lbx_init_from_scratch");
  const int nx = s->N[0], ny = s->N[1], nz = s->N[2];
  const size_t N = (size_t)nx * ny * nz;
  // InitDensity / InitVelocity read the C-order vectors with .at()
  // (src/AmrSim.cpp:138-295): a short vector is an error.
  if (s->n_init[0] < N || s->n_init[1] < 3 * N) return LBX_ERR_RANGE;
  for (int L = 1; L <= s->max_level; ++L) free_level(s->lev[L]);
  s->finest = 0;
  const int lo[3] = {0, 0, 0}, hi[3] = {nx - 1, ny - 1, nz - 1};
  const int ghost = (s->amr_mode == LBX_AMR_FAITHFUL && s->max_level > 0) ? 2 : 0;
  RET(define_level(s, 0, lo, hi, ghost));
  Level& l = s->lev[0];
  l.time = time;
  l.tau_s = s->tau_s0;
  l.tau_b = s->tau_b0;
  compute_dt(s, 0);
  l.step = 0;
  // C-order vectors (already on the device) transposed to FAB order
  // (InitDensity / InitVelocity, CLindex include/AmrSim.h:79-83); a scalar
  // fills the whole field
  if (s->init_scalar[0])
    CK(lbx::launch_fill(l.d_rho, N, s->init_value[0], s->stream));
  if (s->init_scalar[1])
    CK(lbx::launch_fill(l.d_u, 3 * N, s->init_value[1], s->stream));
  if (!s->init_scalar[0] || !s->init_scalar[1])
    CK(lbx::launch_c_to_fab(s->init_scalar[0] ? nullptr : s->d_init[0],
                            s->init_scalar[1] ? nullptr : s->d_init[1], l.d_rho, l.d_u, nx, ny, nz,
                            s->stream));
  l.host_stale = true;
  if (s->precision == LBX_F32_SHIFTED) {
    // shift by the mean initial density: the stored g = f - w rho0 are then
    // the small fluctuations (compensated sum on the device)
    CK(lbx::launch_sum(l.d_rho, N, s->d_partials, s->d_out4, s->stream));
    CK(cudaMemcpyAsync(s->h_out4, s->d_out4, 4 * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    s->rho0 = s->h_out4[0] / (double)N;
  } else {
    s->rho0 = 0.0;
  }
  if (s->f64())
    CK(lbx::launch_equilibrium<double>(l.d_rho, l.d_u, P<double>(l.buf[l.now]), l.box, 0.0, s->stream));
  else
    CK(lbx::launch_equilibrium<float>(l.d_rho, l.d_u, P<float>(l.buf[l.now]), l.box, s->rho0, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  s->initialised = true;
  return LBX_OK;
}

int lbx_set_static_refinement(lbx_sim* s, int level, const int* lo, const int* hi) {
  if (!s || !lo || !hi) return LBX_ERR_ARG;
  lbx::Range range("lbx_set_static_refinement");
  if (!s->initialised) return LBX_ERR_STATE;
  if (level < 0 || level >= s->max_level || level > s->finest) return LBX_ERR_ARG;
  RET(ensure_rform(s, level));  // the coupling works on streamed populations
  RET(ensure_restricted(s));    // new fine cells may take covered parents' values
  Level& c = s->lev[level];
  int tlo[3], thi[3];
  for (int d = 0; d < 3; ++d) {
    tlo[d] = std::max(lo[d], 0);
    thi[d] = std::min(hi[d], s->dn(level, d) - 1);
  }
  RET(check_tag_box(s->amr_mode, s->N, level, c.lo, c.hi, tlo, thi));
  if (level + 1 < s->finest) return LBX_ERR_UNSUPPORTED;  // regrid of an inner level
  const int L = level + 1;
  int flo[3], fhi[3];
  for (int d = 0; d < 3; ++d) {
    flo[d] = 2 * tlo[d];
    fhi[d] = 2 * thi[d] + 1;
  }
  Level& f = s->lev[L];
  if (f.defined && std::equal(flo, flo + 3, f.lo) && std::equal(fhi, fhi + 3, f.hi)) return LBX_OK;
  if (f.defined) {
    // RemakeLevel (src/AmrSim.cpp:715-744): new box filled from the old fine
    // data where it exists, else from the coarse level.
    Level old = f;  // takes ownership of the old buffers
    for (auto& p : f.buf) p = nullptr;
    f.d_rho = f.d_u = nullptr;
    f.defined = false;
    // fill_two reads "fine now" through the old box: do it in two passes,
    // coarse parents first, then a copy of the overlap of the old and new
    // valid boxes
    // (the stored values as they are: the FP32 store's shift is the same)
    auto copy_overlap = [&](auto zero) -> int {
      using T = decltype(zero);
      const Box3& ob = old.box;
      std::vector<T> h((size_t)lbx::NV * ob.sq);
      std::vector<T> hn((size_t)lbx::NV * f.box.sq);
      CK(cudaMemcpyAsync(h.data(), old.buf[old.now], h.size() * sizeof(T),
                         cudaMemcpyDeviceToHost, s->stream));
      CK(cudaMemcpyAsync(hn.data(), f.buf[f.now], hn.size() * sizeof(T),
                         cudaMemcpyDeviceToHost, s->stream));
      CK(cudaStreamSynchronize(s->stream));
      for (int z = std::max(old.lo[2], flo[2]); z <= std::min(old.hi[2], fhi[2]); ++z)
        for (int y = std::max(old.lo[1], flo[1]); y <= std::min(old.hi[1], fhi[1]); ++y)
          for (int x = std::max(old.lo[0], flo[0]); x <= std::min(old.hi[0], fhi[0]); ++x)
            for (int q = 0; q < lbx::NV; ++q)
              hn[q * f.box.sq + f.box.at(x - flo[0], y - flo[1], z - flo[2])] =
                  h[q * ob.sq + ob.at(x - old.lo[0], y - old.lo[1], z - old.lo[2])];
      CK(cudaMemcpyAsync(f.buf[f.now], hn.data(), hn.size() * sizeof(T),
                         cudaMemcpyHostToDevice, s->stream));
      CK(cudaStreamSynchronize(s->stream));
      return LBX_OK;
    };
    int rc = define_level(s, L, flo, fhi, 2);
    if (rc == LBX_OK)
      rc = s->f64() ? fill_from_coarse_T<double>(s, L) : fill_from_coarse_T<float>(s, L);
    if (rc == LBX_OK) rc = s->f64() ? copy_overlap(0.0) : copy_overlap(0.0f);
    f.dt = old.dt;
    f.step = old.step;
    f.tau_s = old.tau_s;
    f.tau_b = old.tau_b;
    f.mass = old.mass;
    f.time = c.time;
    free_level(old);
    if (rc != LBX_OK) {  // neither box is left: the parent is the finest level
      free_level(f);
      s->finest = level;
      return rc;
    }
    return calc_hydro(s, L);
  }
  // MakeNewLevelFromCoarse (src/AmrSim.cpp:689-713)
  int rc = define_level(s, L, flo, fhi, 2);
  if (rc == LBX_OK) {
    f.time = c.time;
    compute_dt(s, L);
    f.step = 0;
    rc = s->f64() ? fill_from_coarse_T<double>(s, L) : fill_from_coarse_T<float>(s, L);
  }
  if (rc != LBX_OK) {
    free_level(f);
    return rc;
  }
  s->finest = std::max(s->finest, L);
  return calc_hydro(s, L);
}

int lbx_unset_static_refinement(lbx_sim* s, int level) {
  if (!s || level < 0 || level > s->max_level) return LBX_ERR_ARG;
  lbx::Range range("lbx_unset_static_refinement");
  RET(ensure_restricted(s));  // uncovered cells take over their restricted values
  CK(cudaStreamSynchronize(s->stream));
  for (int L = level + 1; L <= s->max_level; ++L) {
    free_level(s->lev[L]);
    s->lev[L].time = 0.0;  // ClearLevel (src/AmrSim.cpp:746-751)
    s->lev[L].dt = 0.0;
    s->lev[L].step = 0;
  }
  s->finest = std::min(s->finest, level);
  return LBX_OK;
}

int lbx_iterate(lbx_sim* s, int nsteps) {
  if (!s || nsteps < 0) return LBX_ERR_ARG;
  if (!s->initialised) return LBX_ERR_STATE;
  lbx::Range range("lbx_iterate");
  int left = nsteps;
  if (s->hydro_since_iterate) s->fuse_hydro = true;  // the program steps on after readouts
  s->hydro_since_iterate = false;
  Level& l0 = s->lev[0];
  if (left > 0 && l0.spec_next && s->finest == 0 && l0.pform) {
    // the step CalcHydroVars already ran (its launch was counted there)
    std::swap(l0.now, l0.next);
    l0.time += l0.dt;
    ++l0.step;
    --left;
  }
  l0.spec_next = false;
  // entering the pull form is a one-off extra launch: take it directly
  while (left > 0 && s->finest == 0 && !s->lev[0].pform) {
    RET(macro_step(s));
    --left;
  }
  if (left >= kGraphMinSteps) {
    if (!graph_matches(s)) RET(capture_graph(s, &left));
    const StepGraph& G = s->graphs[s->gcur];
    while (G.exec && left >= G.period) {
      RET(replay_graph(s));
      left -= G.period;
    }
  }
  for (; left > 0; --left) RET(macro_step(s));
  return LBX_OK;
}

int lbx_iterate_timed(lbx_sim* s, int nsteps, double* ms) {
  if (!s || nsteps < 0 || !ms) return LBX_ERR_ARG;
  if (!s->initialised) return LBX_ERR_STATE;
  // the timed region runs every step it reports: a step CalcHydroVars ran
  // ahead is recomputed instead of taken
  s->lev[0].spec_next = false;
  cudaEvent_t a, b;
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&b));
  CK(cudaEventRecord(a, s->stream));
  int rc = lbx_iterate(s, nsteps);
  CK(cudaEventRecord(b, s->stream));
  CK(cudaEventSynchronize(b));
  float t = 0.f;
  CK(cudaEventElapsedTime(&t, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  *ms = t;
  return rc;
}

int lbx_launch_count(const lbx_sim* s, long long* out) {
  if (!s || !out) return LBX_ERR_ARG;
  *out = s->launches;
  return LBX_OK;
}

int lbx_calc_hydro(lbx_sim* s, int level) {
  RET(check_level(s, level));
  lbx::Range range("lbx_calc_hydro");
  RET(ensure_restricted(s));
  return calc_hydro(s, level);
}

int lbx_calc_equilibrium(lbx_sim* s, int level) {
  RET(check_level(s, level));
  Level& l = s->lev[level];
  if (s->f64())
    CK(lbx::launch_equilibrium<double>(l.d_rho, l.d_u, P<double>(l.buf[l.now]), l.box, 0.0, s->stream));
  else
    CK(lbx::launch_equilibrium<float>(l.d_rho, l.d_u, P<float>(l.buf[l.now]), l.box, s->rho0, s->stream));
  l.pform = false;  // the store holds R again
  l.spec_next = false;
  CK(cudaStreamSynchronize(s->stream));
  return LBX_OK;
}

int lbx_get_density(const lbx_sim* s, int i, int j, int k, int level, double* out) {
  if (!s || !out) return LBX_ERR_ARG;
  *out = kNL_DENSITY;
  if (level < 0 || level > s->max_level) return LBX_ERR_ARG;
  const Level& l = s->lev[level];
  if (!l.defined || !l.contains(i, j, k)) return LBX_ERR_NOT_FOUND;
  RET(refresh_host(s, l));
  const size_t v = ((size_t)(k - l.lo[2]) * l.box.n[1] + (j - l.lo[1])) * l.box.n[0] + (i - l.lo[0]);
  *out = l.h_rho[v];
  return LBX_OK;
}

int lbx_get_velocity(const lbx_sim* s, int i, int j, int k, int n, int level, double* out) {
  if (!s || !out) return LBX_ERR_ARG;
  *out = kNL_VELOCITY;
  if (level < 0 || level > s->max_level || n < 0 || n > 2) return LBX_ERR_ARG;
  const Level& l = s->lev[level];
  if (!l.defined || !l.contains(i, j, k)) return LBX_ERR_NOT_FOUND;
  RET(refresh_host(s, l));
  const size_t v = ((size_t)(k - l.lo[2]) * l.box.n[1] + (j - l.lo[1])) * l.box.n[0] + (i - l.lo[0]);
  *out = l.h_u[n * l.cells() + v];
  return LBX_OK;
}

int lbx_get_density_field(const lbx_sim* s, int level, double* out, size_t n) {
  RET(check_level(s, level));
  const Level& l = s->lev[level];
  if (!out || n < l.cells()) return LBX_ERR_ARG;
  return field_out(s, l, l.d_rho, l.h_rho, l.cells(), out);
}

int lbx_get_velocity_field(const lbx_sim* s, int level, double* out, size_t n) {
  RET(check_level(s, level));
  const Level& l = s->lev[level];
  if (!out || n < 3 * l.cells()) return LBX_ERR_ARG;
  return field_out(s, l, l.d_u, l.h_u, 3 * l.cells(), out);
}

int lbx_get_time(const lbx_sim* s, int level, double* t) {
  if (!s || !t || level < 0 || level > s->max_level) return LBX_ERR_ARG;
  *t = s->lev[level].time;
  return LBX_OK;
}
int lbx_get_time_step(const lbx_sim* s, int level, int* st) {
  if (!s || !st || level < 0 || level > s->max_level) return LBX_ERR_ARG;
  *st = s->lev[level].step;
  return LBX_OK;
}
int lbx_get_dt(const lbx_sim* s, int level, double* dt) {
  if (!s || !dt || level < 0 || level > s->max_level) return LBX_ERR_ARG;
  *dt = s->lev[level].dt;
  return LBX_OK;
}
int lbx_get_tau(const lbx_sim* s, int level, double* ts, double* tb) {
  if (!s || !ts || !tb || level < 0 || level > s->max_level) return LBX_ERR_ARG;
  *ts = s->lev[level].tau_s;
  *tb = s->lev[level].tau_b;
  return LBX_OK;
}
int lbx_get_dims(const lbx_sim* s, int* d) {
  if (!s || !d) return LBX_ERR_ARG;
  for (int i = 0; i < 3; ++i) d[i] = s->N[i];
  return LBX_OK;
}
int lbx_max_level(const lbx_sim* s, int* out) {
  if (!s || !out) return LBX_ERR_ARG;
  *out = s->max_level;
  return LBX_OK;
}
int lbx_finest_level(const lbx_sim* s, int* out) {
  if (!s || !out) return LBX_ERR_ARG;
  *out = s->finest;
  return LBX_OK;
}
int lbx_ref_ratio(const lbx_sim* s, int level, int* r) {
  if (!s || !r || level < 0 || level > s->max_level) return LBX_ERR_ARG;
  r[0] = r[1] = r[2] = 2;  // src/AmrSim.cpp:766
  return LBX_OK;
}
int lbx_get_extent(const lbx_sim* s, int level, int* lo, int* hi) {
  RET(check_level(s, level));
  for (int d = 0; d < 3; ++d) {
    lo[d] = s->lev[level].lo[d];
    hi[d] = s->lev[level].hi[d];
  }
  return LBX_OK;
}

static int reduce_level(lbx_sim* s, int level, IBox skip, double* out4);

int lbx_error_est(const lbx_sim* s, int level, unsigned char* tags, size_t n) {
  RET(check_level(s, level));
  const Level& l = s->lev[level];
  if (!tags || n < (size_t)l.cells()) return LBX_ERR_ARG;
  // the static tag box of `level` is the one its refinement was made from
  int tlo[3] = {0, 0, 0}, thi[3] = {-1, -1, -1};
  if (level < s->finest)
    for (int d = 0; d < 3; ++d) {
      tlo[d] = s->lev[level + 1].lo[d] / 2;
      thi[d] = s->lev[level + 1].hi[d] / 2;
    }
  size_t v = 0;
  for (int z = l.lo[2]; z <= l.hi[2]; ++z)
    for (int y = l.lo[1]; y <= l.hi[1]; ++y)
      for (int x = l.lo[0]; x <= l.hi[0]; ++x)
        tags[v++] = (x >= tlo[0] && x <= thi[0] && y >= tlo[1] && y <= thi[1] && z >= tlo[2] &&
                     z <= thi[2])
                        ? 1
                        : 0;
  return LBX_OK;
}

int lbx_tag_density(lbx_sim* s, int level, double threshold, int* lo, int* hi,
                    long long* ntagged) {
  RET(check_level(s, level));
  if (!lo || !hi || !ntagged || !(threshold >= 0.0)) return LBX_ERR_ARG;
  lbx::Range range("lbx_tag_density");
  RET(ensure_restricted(s));
  RET(calc_hydro(s, level));
  double m[4];
  RET(reduce_level(s, level, lbx::empty_ibox(), m));
  Level& l = s->lev[level];
  const double ref = m[0] / (double)l.cells();
  struct Tags {
    int box[6];
    unsigned long long count;
  };
  Tags h{{l.box.n[0], l.box.n[1], l.box.n[2], -1, -1, -1}, 0ull};
  Tags* d = nullptr;
  CK(cudaMallocAsync(&d, sizeof(Tags), s->stream));
  cudaError_t e = cudaMemcpyAsync(d, &h, sizeof(Tags), cudaMemcpyHostToDevice, s->stream);
  if (e == cudaSuccess)
    e = lbx::launch_tag_density(l.d_rho, l.box.n, ref, threshold, d->box, &d->count, s->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, d, sizeof(Tags), cudaMemcpyDeviceToHost, s->stream);
  cudaFreeAsync(d, s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  CK(e);
  *ntagged = (long long)h.count;
  if (h.count)
    for (int d3 = 0; d3 < 3; ++d3) {
      lo[d3] = l.lo[d3] + h.box[d3];
      hi[d3] = l.lo[d3] + h.box[3 + d3];
    }
  return LBX_OK;
}

int lbx_copy_f(lbx_sim* s, int level, double* out, size_t n) {
  RET(check_level(s, level));
  lbx::Range range("lbx_copy_f");
  RET(ensure_restricted(s));
  Level& l = s->lev[level];
  const size_t need = (size_t)lbx::NV * l.cells();
  if (!out || n < need) return LBX_ERR_ARG;
  double* d = nullptr;
  CK(cudaMallocAsync(&d, need * sizeof(double), s->stream));
  cudaError_t e = s->f64()
                      ? lbx::launch_copy_out<double>(P<double>(l.buf[l.now]), l.box, 0.0, d, s->stream, l.pform)
                      : lbx::launch_copy_out<float>(P<float>(l.buf[l.now]), l.box, s->rho0, d, s->stream, l.pform);
  if (e == cudaSuccess) e = lbx::download_host(out, d, need * sizeof(double), s->stream);
  cudaFreeAsync(d, s->stream);
  CK(e);
  return LBX_OK;
}

int lbx_set_f(lbx_sim* s, int level, const double* in, size_t n) {
  RET(check_level(s, level));
  lbx::Range range("lbx_set_f");
  Level& l = s->lev[level];
  const size_t need = (size_t)lbx::NV * l.cells();
  if (!in || n < need) return LBX_ERR_ARG;
  double* d = nullptr;
  CK(cudaMallocAsync(&d, need * sizeof(double), s->stream));
  cudaError_t e = lbx::upload_host(d, in, need * sizeof(double), s->stream);
  if (e == cudaSuccess)
    e = s->f64()
            ? lbx::launch_copy_in<double>(d, P<double>(l.buf[l.now]), l.box, 0.0, s->stream)
            : lbx::launch_copy_in<float>(d, P<float>(l.buf[l.now]), l.box, s->rho0, s->stream);
  l.pform = false;  // the store holds the imported R
  l.spec_next = false;
  cudaFreeAsync(d, s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  CK(e);
  return LBX_OK;
}

static int reduce_level(lbx_sim* s, int level, IBox skip, double* out4) {
  Level& l = s->lev[level];
  if (s->f64())
    CK(lbx::launch_reduce<double>(P<double>(l.buf[l.now]), l.box, skip, 0.0, s->d_partials,
                                  s->d_out4, s->stream));
  else
    CK(lbx::launch_reduce<float>(P<float>(l.buf[l.now]), l.box, skip, s->rho0, s->d_partials,
                                 s->d_out4, s->stream));
  CK(cudaMemcpyAsync(s->h_out4, s->d_out4, 4 * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  for (int i = 0; i < 4; ++i) out4[i] = s->h_out4[i];
  return LBX_OK;
}

int lbx_reduce_mass_momentum(lbx_sim* s, int level, double* out4) {
  RET(check_level(s, level));
  if (!out4) return LBX_ERR_ARG;
  lbx::Range range("lbx_reduce_mass_momentum");
  RET(ensure_restricted(s));
  return reduce_level(s, level, lbx::empty_ibox(), out4);
}

int lbx_total_mass(lbx_sim* s, double* out) {
  if (!s || !out) return LBX_ERR_ARG;
  if (!s->initialised) return LBX_ERR_STATE;
  long double m = 0, vol = 1;
  for (int L = 0; L <= s->finest; ++L) {
    double r[4];
    RET(reduce_level(s, L, true_cover(s, L), r));
    m += vol * (long double)r[0];
    vol /= 8;
  }
  *out = (double)m;
  return LBX_OK;
}

int lbx_synchronize(lbx_sim* s) {
  if (!s) return LBX_ERR_ARG;
  CK(cudaStreamSynchronize(s->stream));
  return LBX_OK;
}

int lbx_get_stream(const lbx_sim* s, void** st) {
  if (!s || !st) return LBX_ERR_ARG;
  *st = (void*)s->stream;
  return LBX_OK;
}

int lbx_get_device_f(lbx_sim* s, int level, void** ptr, int* dims3, int* ghost, int* prec) {
  RET(check_level(s, level));
  RET(ensure_restricted(s));
  RET(ensure_rform(s, level));  // hand out the streamed populations f
  const Level& l = s->lev[level];
  if (ptr) *ptr = l.buf[l.now];
  if (dims3)
    for (int d = 0; d < 3; ++d) dims3[d] = l.box.n[d];
  if (ghost) *ghost = l.box.g;
  if (prec) *prec = s->precision;
  return LBX_OK;
}

// ---- device-pointer entry points ----------------------------------------
int lbx_step_periodic_f64(const double* fin, double* fout, int nx, int ny, int nz, double tau_s,
                          double tau_b, void* stream) {
  if (!fin || !fout || fin == fout || nx <= 0 || ny <= 0 || nz <= 0) return LBX_ERR_ARG;
  CK(lbx::launch_step_periodic<double>(fin, fout, lbx::make_box(nx, ny, nz, 0), lbx::empty_ibox(),
                                       omega(tau_s), omega(tau_b), 0.0, (cudaStream_t)stream));
  return LBX_OK;
}

int lbx_step_periodic_f64p(const double* fin, double* fout, int nx, int ny, int nz, double tau_s,
                           double tau_b, void* stream) {
  if (!fin || !fout || fin == fout || nx <= 0 || ny <= 0 || nz <= 0) return LBX_ERR_ARG;
  CK(lbx::launch_step_periodic_pairs_scalar(fin, fout, lbx::make_box(nx, ny, nz, 0), omega(tau_s),
                                             omega(tau_b), (cudaStream_t)stream));
  return LBX_OK;
}

int lbx_step_periodic_f32s(const float* gin, float* gout, int nx, int ny, int nz, double tau_s,
                           double tau_b, double rho0, void* stream) {
  if (!gin || !gout || gin == gout || nx <= 0 || ny <= 0 || nz <= 0) return LBX_ERR_ARG;
  CK(lbx::launch_step_periodic<float>(gin, gout, lbx::make_box(nx, ny, nz, 0), lbx::empty_ibox(),
                                      omega(tau_s), omega(tau_b), rho0, (cudaStream_t)stream));
  return LBX_OK;
}

int lbx_equilibrium_f64(const double* rho, const double* u, double* f, int nx, int ny, int nz,
                        void* stream) {
  if (!rho || !u || !f || nx <= 0 || ny <= 0 || nz <= 0) return LBX_ERR_ARG;
  CK(lbx::launch_equilibrium<double>(rho, u, f, lbx::make_box(nx, ny, nz, 0), 0.0, (cudaStream_t)stream));
  return LBX_OK;
}

int lbx_hydro_f64(const double* f, double* rho, double* u, int nx, int ny, int nz, void* stream) {
  if (!f || !rho || !u || nx <= 0 || ny <= 0 || nz <= 0) return LBX_ERR_ARG;
  CK(lbx::launch_hydro<double>(f, lbx::make_box(nx, ny, nz, 0), 0.0, rho, u, (cudaStream_t)stream));
  return LBX_OK;
}

int lbx_reduce_mass_momentum_f64(const double* f, size_t ncells, double* out4, void* stream) {
  if (!f || !out4 || ncells == 0 || ncells > (size_t)0x7fffffff) return LBX_ERR_ARG;
  int dev = 0;
  CK(cudaGetDevice(&dev));
  double* scratch = nullptr;
  {
    std::lock_guard<std::mutex> g(g_scratch_mu);
    auto it = g_scratch.find(dev);
    if (it == g_scratch.end()) {
      CK(cudaMalloc(&scratch, lbx::reduce_partials_doubles() * sizeof(double)));
      g_scratch[dev] = scratch;
    } else {
      scratch = it->second;
    }
  }
  // a flat run of cells: view it as an (ncells x 1 x 1) box
  const Box3 b = lbx::make_box((int)ncells, 1, 1, 0);
  CK(lbx::launch_reduce<double>(f, b, lbx::empty_ibox(), 0.0, scratch, out4, (cudaStream_t)stream));
  return LBX_OK;
}

int lbx_checkpoint_write(lbx_sim* s, const char* path) {
  if (!s || !path) return LBX_ERR_ARG;
  if (!s->initialised) return LBX_ERR_STATE;
  lbx::Range range("lbx_checkpoint_write");
  RET(ensure_restricted(s));
  for (int L = 0; L <= s->finest; ++L) RET(ensure_rform(s, L));  // the reference form
  CkptHeader h{};
  std::memcpy(h.magic, kCkptMagic, 8);
  h.version = 1;
  h.precision = s->precision;
  h.amr_mode = s->amr_mode;
  for (int d = 0; d < 3; ++d) h.n[d] = s->N[d];
  h.max_level = s->max_level;
  h.finest = s->finest;
  h.tau_s0 = s->tau_s0;
  h.tau_b0 = s->tau_b0;
  h.rho0 = s->rho0;
  std::vector<std::vector<char>> data(s->finest + 1);
  for (int L = 0; L <= s->finest; ++L) RET(pack_level(s, L, data[L]));
  FILE* fp = std::fopen(path, "wb");
  if (!fp) return LBX_ERR_IO;
  bool ok = std::fwrite(&h, sizeof h, 1, fp) == 1;
  for (int L = 0; ok && L <= s->finest; ++L) {
    const Level& l = s->lev[L];
    CkptLevel c{};
    for (int d = 0; d < 3; ++d) {
      c.lo[d] = l.lo[d];
      c.hi[d] = l.hi[d];
    }
    c.time = l.time;
    c.dt = l.dt;
    c.tau_s = l.tau_s;
    c.tau_b = l.tau_b;
    c.mass = l.mass;
    c.step = l.step;
    ok = std::fwrite(&c, sizeof c, 1, fp) == 1;
  }
  for (int L = 0; ok && L <= s->finest; ++L)
    ok = std::fwrite(data[L].data(), 1, data[L].size(), fp) == data[L].size();
  ok = (std::fclose(fp) == 0) && ok;
  return ok ? LBX_OK : LBX_ERR_IO;
}

int lbx_checkpoint_read(const char* path, lbx_sim** out) {
  if (!path || !out) return LBX_ERR_ARG;
  *out = nullptr;
  lbx::Range range("lbx_checkpoint_read");
  FILE* fp = std::fopen(path, "rb");
  if (!fp) return LBX_ERR_IO;
  CkptHeader h{};
  bool ok = std::fread(&h, sizeof h, 1, fp) == 1 && std::memcmp(h.magic, kCkptMagic, 8) == 0 &&
            h.version == 1 && h.finest >= 0 && h.finest <= h.max_level && h.max_level <= 8;
  std::vector<CkptLevel> lv;
  if (ok) {
    lv.resize(h.finest + 1);
    ok = std::fread(lv.data(), sizeof(CkptLevel), lv.size(), fp) == lv.size();
  }
  for (int L = 0; ok && L <= h.finest; ++L)
    for (int d = 0; d < 3; ++d) {
      const long long ext = (long long)h.n[d] << L;
      const CkptLevel& c = lv[L];
      if (c.lo[d] < 0 || c.hi[d] >= ext || c.hi[d] < c.lo[d]) ok = false;
      if (L == 0 && (c.lo[d] != 0 || c.hi[d] != ext - 1)) ok = false;  // level 0 is the domain
    }
  // a finer level is the refinement of a tag box that lbx_set_static_refinement
  // would accept under its parent
  for (int L = 1; ok && L <= h.finest; ++L) {
    int tlo[3], thi[3];
    for (int d = 0; d < 3; ++d) {
      if (lv[L].lo[d] % 2 != 0 || lv[L].hi[d] % 2 != 1) ok = false;
      tlo[d] = lv[L].lo[d] / 2;
      thi[d] = lv[L].hi[d] / 2;
    }
    if (ok && check_tag_box(h.amr_mode, h.n, L - 1, lv[L - 1].lo, lv[L - 1].hi, tlo, thi) != LBX_OK)
      ok = false;
  }
  if (!ok) {
    std::fclose(fp);
    return LBX_ERR_IO;
  }
  const int per[3] = {1, 1, 1};
  lbx_sim* s = nullptr;
  int rc = lbx_create(h.n[0], h.n[1], h.n[2], h.max_level, per, h.tau_s0, h.tau_b0, h.precision,
                      h.amr_mode, &s);
  if (rc != LBX_OK) {
    std::fclose(fp);
    return rc == LBX_ERR_ARG ? LBX_ERR_IO : rc;
  }
  s->rho0 = h.rho0;
  for (int L = 0; rc == LBX_OK && L <= h.finest; ++L) {
    const CkptLevel& c = lv[L];
    const int ghost = L ? 2 : ((h.amr_mode == LBX_AMR_FAITHFUL && h.max_level > 0) ? 2 : 0);
    rc = define_level(s, L, c.lo, c.hi, ghost);
    if (rc != LBX_OK) break;
    Level& l = s->lev[L];
    l.time = c.time;
    l.dt = c.dt;
    l.tau_s = c.tau_s;
    l.tau_b = c.tau_b;
    l.mass = c.mass;
    l.step = (int)c.step;
    l.host_stale = true;
    std::vector<char> data((size_t)lbx::NV * l.cells() * s->esize());
    if (std::fread(data.data(), 1, data.size(), fp) != data.size()) {
      rc = LBX_ERR_IO;
      break;
    }
    rc = unpack_level(s, L, data);
  }
  std::fclose(fp);
  if (rc != LBX_OK) {
    lbx_destroy(s);
    return rc;
  }
  s->finest = h.finest;
  s->initialised = true;
  *out = s;
  return LBX_OK;
}

}  // extern "C"
