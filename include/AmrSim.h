// -*- mode: c++; -*-
// AmrSim.h -- header-only C++ drop-in for LAMBReX's AmrSim
// (include/AmrSim.h:23-155 of the reference) over the C ABI of
// liblbx_cuda.so (lbx.h).  Public methods keep the reference's names,
// argument meaning and semantics:
//   * SetInitialDensity/Velocity take a scalar or a C-order vector by value;
//   * Iterate does not refresh density/velocity (call CalcHydroVars);
//   * GetDensity/GetVelocity return -1 / -3e8 for points not on the level;
//   * where the reference calls amrex::Abort, this throws lbx::Error (an
//     uncaught exception terminates the program like the abort does).
// AMReX types are not exposed; InitFromScratch, maxLevel, finestLevel and
// refRatio stand in for the AmrCore members the reference's users call.
#ifndef LBX_AMRSIM_H
#define LBX_AMRSIM_H

#include <array>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "lbx.h"

#ifndef NDIMS
#define NDIMS 3
#endif
#ifndef NMODES
#define NMODES 15
#endif

namespace lbx {

struct Error : std::runtime_error {
  int status;
  Error(int st, const std::string& where)
      : std::runtime_error(where + ": " + lbx_status_string(st)), status(st) {}
};

inline void check(int st, const char* where) {
  if (st != LBX_OK) throw Error(st, where);
}

// F64: FP64 store and arithmetic.  F32Shifted: FP32 store of f - w rho0.
// F64Paired: FP64 store, every collision in pairs of FP32 values (4.8x the
// FP64 rate on GB300 for one level, same 1e-12 agreement).
enum class Precision { F64 = LBX_F64, F32Shifted = LBX_F32_SHIFTED, F64Paired = LBX_F64_PAIRED };
// Faithful: the reference's Rohde cycle with its quirks (the default, so that
// a LAMBReX program gets the reference's algorithm).  It does not conserve
// mass and diverges once a level is refined: the reference's covered-cell
// mask marks coarsen(coarse box) rather than the refined region, so coarse
// cells under the patch both collide and receive the fine average (a 64^3
// level refined over [16,47]^3 gains a factor 7.6e34 of mass in 50 coarse
// steps).  Conservative: the volumetric coupling, mass conserved to
// round-off.  Rescaled: covered coarse cells stay active, the fine ghost
// shell is refilled before every fine sub-step from the parents interpolated
// in time with the non-equilibrium part rescaled between the levels; the
// most accurate at the interface, with a small mass drift.
enum class AmrMode {
  Faithful = LBX_AMR_FAITHFUL,
  Conservative = LBX_AMR_CONSERVATIVE,
  Rescaled = LBX_AMR_RESCALED
};

}  // namespace lbx

class AmrSim {
 public:
  AmrSim(int const nx, int const ny, int const nz, int const max_ref_level,
         const std::array<int, NDIMS>& periodicity, double const tau_s, double const tau_b,
         lbx::Precision precision = lbx::Precision::F64,
         lbx::AmrMode mode = lbx::AmrMode::Faithful)
      : NX(nx), NY(ny), NZ(nz) {
    lbx::check(lbx_create(nx, ny, nz, max_ref_level, periodicity.data(), tau_s, tau_b,
                          static_cast<int>(precision), static_cast<int>(mode), &sim_),
               "AmrSim");
  }
  AmrSim(const AmrSim&) = delete;
  AmrSim& operator=(const AmrSim&) = delete;
  AmrSim(AmrSim&& o) noexcept : NX(o.NX), NY(o.NY), NZ(o.NZ), sim_(o.sim_) { o.sim_ = nullptr; }
  virtual ~AmrSim() { lbx_destroy(sim_); }

  // ---- public interface of the reference (include/AmrSim.h:128-154) ----
  double GetTime(int const level) const {
    double t = 0;
    lbx::check(lbx_get_time(sim_, level, &t), "GetTime");
    return t;
  }
  int GetTimeStep(int const level) const {
    int s = 0;
    lbx::check(lbx_get_time_step(sim_, level, &s), "GetTimeStep");
    return s;
  }
  std::array<int, NDIMS> GetDims() const { return std::array<int, NDIMS>{NX, NY, NZ}; }
  bool OnProcessDensity(double const rho) const { return rho != lbx_nl_density(); }
  bool OnProcessVelocity(double const u) const { return u != lbx_nl_velocity(); }
  void SetInitialDensity(double const rho) {
    lbx::check(lbx_set_initial_density(sim_, &rho, 1), "SetInitialDensity");
  }
  void SetInitialDensity(std::vector<double> const rho) {
    lbx::check(lbx_set_initial_density(sim_, rho.data(), rho.size()), "SetInitialDensity");
  }
  void SetInitialVelocity(double const u) {
    lbx::check(lbx_set_initial_velocity(sim_, &u, 1), "SetInitialVelocity");
  }
  void SetInitialVelocity(std::vector<double> const u) {
    lbx::check(lbx_set_initial_velocity(sim_, u.data(), u.size()), "SetInitialVelocity");
  }
  double GetDensity(int const i, int const j, int const k, int const level) const {
    double v = lbx_nl_density();
    lbx_get_density(sim_, i, j, k, level, &v);
    return v;
  }
  double GetVelocity(int const i, int const j, int const k, int const n, int const level) const {
    double v = lbx_nl_velocity();
    lbx_get_velocity(sim_, i, j, k, n, level, &v);
    return v;
  }
  void CalcEquilibriumDist(int const level) {
    lbx::check(lbx_calc_equilibrium(sim_, level), "CalcEquilibriumDist");
  }
  void CalcHydroVars(int const level) { lbx::check(lbx_calc_hydro(sim_, level), "CalcHydroVars"); }
  void Iterate(int const nsteps) { lbx::check(lbx_iterate(sim_, nsteps), "Iterate"); }
  void SetStaticRefinement(int const level, const std::array<int, NDIMS>& lo,
                           const std::array<int, NDIMS>& hi) {
    lbx::check(lbx_set_static_refinement(sim_, level, lo.data(), hi.data()), "SetStaticRefinement");
  }
  void UnsetStaticRefinement(int const level) {
    lbx::check(lbx_unset_static_refinement(sim_, level), "UnsetStaticRefinement");
  }
  std::pair<std::array<int, NDIMS>, std::array<int, NDIMS>> GetExtent(int const level) const {
    std::array<int, NDIMS> lo{}, hi{};
    lbx::check(lbx_get_extent(sim_, level, lo.data(), hi.data()), "GetExtent");
    return std::make_pair(lo, hi);
  }
  // ErrorEst (src/AmrSim.cpp:633-663): the level's tags in FAB order, 1 (SET)
  // inside its static tag box, 0 (CLEAR) elsewhere
  std::vector<unsigned char> ErrorEst(int const level) const {
    const auto ext = GetExtent(level);
    size_t n = 1;
    for (int d = 0; d < NDIMS; ++d) n *= (size_t)(ext.second[d] - ext.first[d] + 1);
    std::vector<unsigned char> tags(n);
    lbx::check(lbx_error_est(sim_, level, tags.data(), tags.size()), "ErrorEst");
    return tags;
  }

  // ---- AmrCore members used by the reference's callers ----
  void InitFromScratch(double const time) {
    lbx::check(lbx_init_from_scratch(sim_, time), "InitFromScratch");
  }
  int maxLevel() const {
    int v = 0;
    lbx::check(lbx_max_level(sim_, &v), "maxLevel");
    return v;
  }
  int finestLevel() const {
    int v = 0;
    lbx::check(lbx_finest_level(sim_, &v), "finestLevel");
    return v;
  }
  std::array<int, NDIMS> refRatio(int const level) const {
    std::array<int, NDIMS> r{};
    lbx::check(lbx_ref_ratio(sim_, level, r.data()), "refRatio");
    return r;
  }

  // ---- additions of this library ----
  lbx_sim* handle() const { return sim_; }
  // solution-driven tagging: the bounding box of the level's cells whose
  // density differs from the level's mean by more than threshold (false if
  // none); SetStaticRefinement(level, lo, hi) then regrids to it
  bool TagDensity(int const level, double const threshold, std::array<int, NDIMS>& lo,
                  std::array<int, NDIMS>& hi, long long* ntagged = nullptr) {
    long long n = 0;
    lbx::check(lbx_tag_density(sim_, level, threshold, lo.data(), hi.data(), &n), "TagDensity");
    if (ntagged) *ntagged = n;
    return n > 0;
  }
  std::vector<double> CopyDistribution(int const level) {
    const auto ext = GetExtent(level);
    size_t n = NMODES;
    for (int d = 0; d < NDIMS; ++d) n *= (size_t)(ext.second[d] - ext.first[d] + 1);
    std::vector<double> f(n);
    lbx::check(lbx_copy_f(sim_, level, f.data(), f.size()), "CopyDistribution");
    return f;
  }
  double TotalMass() {
    double m = 0;
    lbx::check(lbx_total_mass(sim_, &m), "TotalMass");
    return m;
  }
  // checkpoint / restart (no counterpart in the reference): a restored
  // simulation continues bit for bit
  void WriteCheckpoint(const std::string& path) {
    lbx::check(lbx_checkpoint_write(sim_, path.c_str()), "WriteCheckpoint");
  }
  static AmrSim ReadCheckpoint(const std::string& path) {
    lbx_sim* s = nullptr;
    lbx::check(lbx_checkpoint_read(path.c_str(), &s), "ReadCheckpoint");
    int d[NDIMS] = {0, 0, 0};
    const int st = lbx_get_dims(s, d);
    if (st != LBX_OK) {
      lbx_destroy(s);
      throw lbx::Error(st, "ReadCheckpoint");
    }
    return AmrSim(s, d[0], d[1], d[2]);
  }

 protected:
  const int NX, NY, NZ;

 private:
  AmrSim(lbx_sim* s, int nx, int ny, int nz) : NX(nx), NY(ny), NZ(nz), sim_(s) {}
  lbx_sim* sim_ = nullptr;
};

#endif  // LBX_AMRSIM_H
