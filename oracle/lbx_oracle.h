/*
 * lbx_oracle.h -- CPU restatement of LAMBReX's D3Q15 lattice Boltzmann time
 * step.  TEST INFRASTRUCTURE ONLY: this library is the parity checker for the
 * CUDA implementation in lambrex_gb300/csrc and the timed CPU baseline of
 * bench.py.  Nothing in the shipped library links, loads or calls it.
 *
 * Pinning: the single-level path is checked against the reference's own
 * known-answer data (tests/pulseRegression.h, driven by
 * tests/catch2RegressionTests.cpp:6-93) by tests/test_oracle.py.  The
 * two-level path follows src/AmrSim.cpp:359-631 plus stated AMReX semantics
 * (AMReX is a third-party dependency that is not available here); beyond the
 * reference's ml_pulse expectation it is parity-unpinned.
 *
 * Layouts (all arrays double precision):
 *   f    : [q][k][j][i]   15 populations, i fastest (AMReX FAB order,
 *                         include/field.h:124-126 without ghost cells)
 *   rho  : [k][j][i]
 *   u    : [n][k][j][i]   n = 0..2
 *   C-order user input (src/AmrSim.cpp:138-295, include/AmrSim.h:79-83):
 *          rho_c[(i*ny + j)*nz + k],  u_c[((i*ny + j)*nz + k)*3 + n]
 */
#ifndef LBX_ORACLE_H
#define LBX_ORACLE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Fill fresh ghost-cell storage with NaN (on != 0) instead of zero, so that
 * reads of memory a step never wrote show up as NaN in its results. */
void orc_set_poison(int on);

/* 15x15 mode matrix M[m][p] and inverse Minv[p][m], row-major
 * (src/AmrSim.cpp:1037-1073), derived from the velocity set. */
void orc_mode_tables(double* M, double* Minv);

/* One reference-order collision of a single cell (src/AmrSim.cpp:25-107). */
void orc_collide_cell(double* f15, double omega_s, double omega_b);

/* C-order user vectors -> FAB-order fields (InitDensity/InitVelocity).
 * nrho / nu are the lengths of the user vectors; returns 0, or -1 if a
 * vector is too short (the reference's std::vector::at throws). */
int orc_c_to_fab(int nx, int ny, int nz, const double* rho_c, size_t nrho,
                 const double* u_c, size_t nu, double* rho, double* u);

/* Second-order D3Q15 equilibrium from FAB-order rho, u
 * (src/AmrSim.cpp:845-936). */
void orc_equilibrium(int nx, int ny, int nz, const double* rho,
                     const double* u, double* f);

/* nsteps single-level periodic steps now <- S(C(now)) (src/AmrSim.cpp:
 * 109-135, 297-333).  style 0: reference-style (ghost-cell FABs, separate
 * fill / collide / fill-boundary / stream passes, a fresh stream buffer per
 * step, i-j-k loop order with k innermost, one thread).  style 1: the same
 * per-cell arithmetic with cache-friendly loops on nthreads OpenMP threads.
 * Both styles give bit-identical results. */
int orc_step(int nx, int ny, int nz, double* f, double tau_s, double tau_b,
             int nsteps, int nthreads, int style);

/* CalcHydroVars (src/AmrSim.cpp:938-979). */
void orc_hydro(int nx, int ny, int nz, const double* f, double* rho,
               double* u);

/* sum f, sum c_a f in long double accumulation: out[0]=mass, out[1..3]=j */
void orc_mass_momentum(int nx, int ny, int nz, const double* f, double* out);

/* ---- multi-level (static AMR) ------------------------------------------ */
typedef struct orc_amr orc_amr;

/* mode 0: reference-faithful Rohde cycle (src/AmrSim.cpp:430-631);
 * mode 1: the conservative volumetric scheme of the CUDA library;
 * mode 2: the rescaled coupling of the CUDA library (non-equilibrium
 *         rescaling, ghost data interpolated in time across the sub-steps). */
orc_amr* orc_amr_create(int nx, int ny, int nz, int max_level, double tau_s,
                        double tau_b, int mode);
void orc_amr_destroy(orc_amr* s);

/* Readings of the AMReX behaviour the faithful cycle relies on (AMReX is not
 * available here, so each is a reading of its public semantics).  0 selects
 * the default readings:
 *   sum_fine_to_coarse (src/AmrSim.cpp:592-602) averages each 2^3 fine block
 *     over the coarsened fine box grown by one ghost cell and ADDs it;
 *   makeFineMask (src/AmrSim.cpp:419-428) is handed the coarse level's own
 *     BoxArray, so it marks coarsen(coarse box);
 *   the fresh buffer of Stream (src/AmrSim.cpp:111-112) is zero beyond the
 *     valid box + 1 ring that the stream writes.
 * Each bit flips one of them. */
#define ORC_READ_SUM8 1        /* x8 block sum instead of the average          */
#define ORC_READ_GROW0 2       /* restrict the coarsened fine box, no ghost ring */
#define ORC_READ_MASK_FINE 4   /* mask = coarsen(fine box), the intended mask   */
#define ORC_READ_RING2_STALE 8 /* Stream's fresh buffer reuses the block the
                                  level's previous Stream released            */
int orc_amr_set_readings(orc_amr* s, int readings);
int orc_amr_init(orc_amr* s, const double* rho_c, size_t nrho,
                 const double* u_c, size_t nu, double time);
int orc_amr_refine(orc_amr* s, int level, const int* lo, const int* hi);
int orc_amr_unrefine(orc_amr* s, int level);
int orc_amr_iterate(orc_amr* s, int nsteps);
int orc_amr_finest(const orc_amr* s);
int orc_amr_extent(const orc_amr* s, int level, int* lo, int* hi);
/* valid-region f of level `level` (state "now") in FAB order */
int orc_amr_copy_f(const orc_amr* s, int level, double* out);
/* whole grown box (valid + 2 ghosts) of state "now", FAB order */
int orc_amr_copy_f_grown(const orc_amr* s, int level, double* out);
int orc_amr_calc_hydro(orc_amr* s, int level);
int orc_amr_get_hydro(const orc_amr* s, int level, double* rho, double* u);
int orc_amr_time(const orc_amr* s, int level, double* time, double* dt,
                 int* step, double* tau_s, double* tau_b);
/* mass of the composite solution: active cells of every level weighted by
 * their volume 8^-level (long double accumulation) */
double orc_amr_mass(const orc_amr* s);

#ifdef __cplusplus
}
#endif
#endif
