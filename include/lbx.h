/*
 * lbx.h -- C ABI of liblbx_cuda.so, the GB300 (sm_103a) implementation of
 * LAMBReX's D3Q15 lattice Boltzmann time step.
 *
 * Every function returns an int status (LBX_OK == 0).  Plain pointers and
 * sizes only.  One simulation per handle; each handle owns one CUDA stream.
 * The ABI is thread-compatible (different handles may be used from different
 * threads), not thread-safe per handle.  Stepping is asynchronous on the
 * handle's stream; errors of queued work surface at the next call that
 * synchronises (hydro, copies, reductions, lbx_synchronize).
 *
 * Layouts
 *   user vectors (C order, src/AmrSim.cpp:138-295, include/AmrSim.h:79-83):
 *       rho[(i*NY + j)*NZ + k],  u[((i*NY + j)*NZ + k)*3 + n]
 *   field exports (AMReX FAB order, include/field.h:124-126):
 *       f[q][k][j][i], rho[k][j][i], u[n][k][j][i]   (i fastest)
 *   velocity ordering q = 0..14 as include/d3q15_bgk.h:14-22.
 */
#ifndef LBX_H
#define LBX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define LBX_OK 0
#define LBX_ERR_ARG 1          /* bad argument (the reference aborts)       */
#define LBX_ERR_STATE 2        /* call not valid in the current state       */
#define LBX_ERR_CUDA 3         /* CUDA runtime error / no device            */
#define LBX_ERR_OOM 4          /* device memory or HBM budget exhausted     */
#define LBX_ERR_UNSUPPORTED 5  /* combination not implemented              */
#define LBX_ERR_RANGE 6        /* initial vector shorter than the domain    */
#define LBX_ERR_TIMEOUT 7      /* a bounded device wait gave up             */
#define LBX_ERR_NOT_FOUND 8    /* point not on the level (getter miss)      */
#define LBX_ERR_IO 9           /* checkpoint file unreadable or unwritable  */

/* precision of the distribution store */
#define LBX_F64 0              /* FP64 drop-in                              */
#define LBX_F32_SHIFTED 1      /* FP32 populations f_i - w_i rho0           */
#define LBX_F64_PAIRED 2       /* FP64 store; every collision is carried in
                                  pairs of FP32 values (48-bit significand)
                                  on the FP32 pipe, within the same 1e-12 of
                                  the reference order as LBX_F64             */

/* multi-level coupling */
#define LBX_AMR_FAITHFUL 0     /* the reference's Rohde cycle, quirks kept;
                                  not mass-conserving: its covered-cell mask
                                  (src/AmrSim.cpp:419-428) lets a refined run
                                  gain mass without bound                    */
#define LBX_AMR_CONSERVATIVE 1 /* volumetric scheme, mass conserved exactly */
#define LBX_AMR_RESCALED 2     /* covered coarse cells active; the fine ghost
                                  shell refilled before each fine sub-step
                                  from the parents interpolated in time, the
                                  non-equilibrium part rescaled between the
                                  levels both ways (Dupuis & Chopard 2003);
                                  the most accurate at the interface, mass
                                  not exactly conserved                      */

typedef struct lbx_sim lbx_sim;

const char* lbx_status_string(int status);
/* sentinels returned by the getters on a miss (include/AmrSim.h:35-36) */
double lbx_nl_density(void);
double lbx_nl_velocity(void);

/* lambrexInit / lambrexFinalise (include/lambrex.h:6-7, src/lambrex.cpp:4-14):
 * select and warm up the CUDA device; release library-wide resources. */
int lbx_init(void);
int lbx_finalize(void);
/* make `device` current for the calling host thread (one GPU per process
 * or thread; handles created afterwards live on it) */
int lbx_set_device(int device);

/* AmrSim::AmrSim (include/AmrSim.h:128-129, src/AmrSim.cpp:753-802).
 * periodicity must be {1,1,1} (the reference aborts otherwise, :795).
 * amr_mode is LBX_AMR_FAITHFUL, LBX_AMR_CONSERVATIVE or LBX_AMR_RESCALED. */
int lbx_create(int nx, int ny, int nz, int max_level, const int* periodicity, double tau_s,
               double tau_b, int precision, int amr_mode, lbx_sim** out);
int lbx_destroy(lbx_sim* sim);

/* SetInitialDensity / SetInitialVelocity (src/AmrSim.cpp:804-822).  n == 1
 * broadcasts a scalar; otherwise the vector (length n) is copied. */
int lbx_set_initial_density(lbx_sim* sim, const double* rho, size_t n);
int lbx_set_initial_velocity(lbx_sim* sim, const double* u, size_t n);

/* AmrCore::InitFromScratch -> MakeNewLevelFromScratch(0)
 * (src/AmrSim.cpp:665-687): fields from the initial vectors, equilibrium f. */
int lbx_init_from_scratch(lbx_sim* sim, double time);

/* SetStaticRefinement / UnsetStaticRefinement (src/AmrSim.cpp:995-1017).
 * lo/hi are inclusive corners in level-`level` cells; the new level is
 * exactly refine(lo..hi) (one box, no error buffer). */
int lbx_set_static_refinement(lbx_sim* sim, int level, const int* lo, const int* hi);
int lbx_unset_static_refinement(lbx_sim* sim, int level);

/* Iterate (src/AmrSim.cpp:981-993); asynchronous on the sim's stream. */
int lbx_iterate(lbx_sim* sim, int nsteps);

/* lbx_iterate bracketed by CUDA events on the sim's stream; waits for the
 * steps to finish and returns their device time in *ms. */
int lbx_iterate_timed(lbx_sim* sim, int nsteps, double* ms);
/* number of kernel launches lbx_iterate has issued on this handle */
int lbx_launch_count(const lbx_sim* sim, long long* out);

/* CalcHydroVars (src/AmrSim.cpp:938-979): rho,u of the level on the device;
 * the point getters copy them to the host on their first call after it. */
int lbx_calc_hydro(lbx_sim* sim, int level);
/* CalcEquilibriumDist (src/AmrSim.cpp:845-936) from the level's rho,u. */
int lbx_calc_equilibrium(lbx_sim* sim, int level);

/* GetDensity / GetVelocity (src/AmrSim.cpp:824-843).  On a miss *out is the
 * sentinel and the status is LBX_ERR_NOT_FOUND. */
int lbx_get_density(const lbx_sim* sim, int i, int j, int k, int level, double* out);
int lbx_get_velocity(const lbx_sim* sim, int i, int j, int k, int n, int level, double* out);
/* whole fields of a level, FAB order over its valid box, copied from the
 * device into `out` */
int lbx_get_density_field(const lbx_sim* sim, int level, double* out, size_t n);
int lbx_get_velocity_field(const lbx_sim* sim, int level, double* out, size_t n);

/* GetTime / GetTimeStep / GetDims (include/AmrSim.h:130-137), the per-level
 * dt and tau (AmrSim.cpp:297-322), maxLevel/finestLevel/refRatio of AmrCore */
int lbx_get_time(const lbx_sim* sim, int level, double* time);
int lbx_get_time_step(const lbx_sim* sim, int level, int* step);
int lbx_get_dt(const lbx_sim* sim, int level, double* dt);
int lbx_get_tau(const lbx_sim* sim, int level, double* tau_s, double* tau_b);
int lbx_get_dims(const lbx_sim* sim, int* dims3);
int lbx_max_level(const lbx_sim* sim, int* out);
int lbx_finest_level(const lbx_sim* sim, int* out);
int lbx_ref_ratio(const lbx_sim* sim, int level, int* ratio3);
/* GetExtent (src/AmrSim.cpp:1019-1030) */
int lbx_get_extent(const lbx_sim* sim, int level, int* lo, int* hi);
/* ErrorEst (src/AmrSim.cpp:633-663) with TagCell (:413-417): the tags of the
 * level's valid cells, FAB order (x fastest), 1 (TagBox::SET) inside the
 * level's static tag box, 0 (CLEAR) elsewhere and on a level without one;
 * n >= the level's cell count. */
int lbx_error_est(const lbx_sim* sim, int level, unsigned char* tags, size_t n);
/* Solution-driven tagging (the reference tags static boxes only): computes
 * the level's hydrodynamic fields (as lbx_calc_hydro) and, in the level's
 * cells, the bounding box lo..hi of the cells whose density differs from
 * the level's mean by more than threshold; *ntagged = their number, lo and
 * hi are left as they are when it is 0.  A refinement box for
 * lbx_set_static_refinement, which regrids (RemakeLevel). */
int lbx_tag_density(lbx_sim* sim, int level, double threshold, int* lo, int* hi,
                    long long* ntagged);

/* distribution export / import, FAB order over the level's valid box, f
 * in FP64 whatever the storage precision (n = 15 * cells) */
int lbx_copy_f(lbx_sim* sim, int level, double* out, size_t n);
int lbx_set_f(lbx_sim* sim, int level, const double* in, size_t n);

/* compensated FP64 sums over the level's valid box:
 * out[0] = sum f, out[1..3] = sum c_a f */
int lbx_reduce_mass_momentum(lbx_sim* sim, int level, double* out4);
/* composite mass: uncovered cells of every level weighted by 8^-level */
int lbx_total_mass(lbx_sim* sim, double* out);

int lbx_synchronize(lbx_sim* sim);
/* the handle's cudaStream_t, for callers that order their own work */
int lbx_get_stream(const lbx_sim* sim, void** stream);
/* device pointer and layout of the level's current f store (read-only use;
 * valid until the next call that steps or changes the level) */
int lbx_get_device_f(lbx_sim* sim, int level, void** ptr, int* storage_dims3, int* ghost,
                     int* precision);

/* ---- device-pointer kernels (no handle; caller owns memory) ------------
 * One fused collide+stream step of a fully periodic box, f_in -> f_out, FAB
 * order without ghosts, on `stream` (a cudaStream_t, NULL = default).
 * Replaces Collide + FillBoundary + Stream + UpdateNow of one level
 * (src/AmrSim.cpp:25-135, include/component.h:22-29). */
int lbx_step_periodic_f64(const double* f_in, double* f_out, int nx, int ny, int nz,
                          double tau_s, double tau_b, void* stream);
/* FP64 store, collision in paired FP32 arithmetic (LBX_F64_PAIRED) in its
 * one-cell scalar form, which the simulation's packed form reproduces bit
 * for bit */
int lbx_step_periodic_f64p(const double* f_in, double* f_out, int nx, int ny, int nz,
                           double tau_s, double tau_b, void* stream);
/* FP32 shifted populations g = f - w rho0 */
int lbx_step_periodic_f32s(const float* g_in, float* g_out, int nx, int ny, int nz,
                           double tau_s, double tau_b, double rho0, void* stream);
/* Equilibrium (src/AmrSim.cpp:845-936) from device rho[k][j][i], u[n][k][j][i] */
int lbx_equilibrium_f64(const double* rho, const double* u, double* f, int nx, int ny, int nz,
                        void* stream);
/* CalcHydroVars (src/AmrSim.cpp:938-979) on device arrays */
int lbx_hydro_f64(const double* f, double* rho, double* u, int nx, int ny, int nz,
                  void* stream);
/* Compensated FP64 mass/momentum sums of f (n cells, 15 components of
 * stride n) into out4 (device or host-pinned pointer).  The library
 * allocates its scratch partial sums with cudaMalloc on first use per
 * device and keeps them until lbx_finalize. */
int lbx_reduce_mass_momentum_f64(const double* f, size_t ncells, double* out4, void* stream);
/* The same reduction for callers that cannot let the library allocate device
 * memory (an application that gives all of HBM to its own pool at start-up,
 * or a latency-bound loop that must not take the allocator's locks).  No
 * counterpart in the reference.  It calls no allocator: its partial sums
 * live in a fixed 32 KiB device array that every GPU loading the library
 * holds until exit.  The first call on a device looks up that array's
 * address (make it before any stream capture); the address is kept per
 * device context, so the first call after a context is re-created
 * (cudaDeviceReset) looks it up again and belongs before any capture too.
 * Calls share the array, so calls that overlap on the GPU race.  At most 2^31 - 1 cells; larger inputs
 * return LBX_ERR_ARG without GPU work. */
int lbx_reduce_mass_momentum_f64_noalloc(const double* f, size_t ncells, double* out4,
                                         void* stream);

/* ---- checkpoint / restart ---------------------------------------------
 * No counterpart in the reference (it writes no plotfile or checkpoint).
 * lbx_checkpoint_write saves the simulation's state: sizes, precision,
 * coupling mode, every level's box, time, step and rates, the FP32 shift, and
 * each level's stored populations over its valid cells in FAB order
 * (component-major, x fastest) in the storage type itself, so that a restart
 * continues bit for bit.  lbx_checkpoint_read creates a new simulation from
 * such a file (the caller destroys it).  Format: little-endian, magic
 * "LBXCKPT1"; a wrong or truncated file, or one whose fine levels
 * lbx_set_static_refinement could not have made, returns LBX_ERR_IO. */
int lbx_checkpoint_write(lbx_sim* sim, const char* path);
int lbx_checkpoint_read(const char* path, lbx_sim** out);

/* ---- debug build --------------------------------------------------------
 * liblbx_cuda_checked.so is the same library compiled with bounds checks on
 * every global load and store of its kernels: an out-of-range element index
 * is counted, the access is skipped (a load yields 0) and nothing traps.
 * This call returns the number of such accesses on the current device since
 * the last reset and the first bad index; reset != 0 clears the counters.
 * The release library returns LBX_ERR_UNSUPPORTED.  No counterpart in the
 * reference (its loops run on the host under AMReX's own array checks). */
int lbx_debug_bounds(long long* count, long long* first_bad_index, int reset);

/* ---- batched ensemble --------------------------------------------------
 * Many independent periodic boxes of uneven sizes advance together: one
 * persistent launch per step over a device tile work-list, steps replayed
 * from a captured CUDA graph.  Each box behaves as an AmrSim single-level
 * run (src/AmrSim.cpp:981-985) with tau_s = tau_b = tau[b]. */
typedef struct lbx_ensemble lbx_ensemble;
/* dims: 3 extents per box; tau: one value per box; precision LBX_F64 or
 * LBX_F32_SHIFTED (shift rho0 = mean initial density of the box) */
int lbx_ensemble_create(int nbox, const int* dims, const double* tau, int precision,
                        lbx_ensemble** out);
int lbx_ensemble_destroy(lbx_ensemble* e);
/* equilibrium state of box b from C-order rho / u vectors (as
 * lbx_set_initial_* + lbx_init_from_scratch) */
int lbx_ensemble_init_box(lbx_ensemble* e, int b, const double* rho, size_t nrho,
                          const double* u, size_t nu);
/* time every (tile cells, block, cells per thread) candidate for trial_steps
 * steps on the current state (which is saved and restored), keep the
 * fastest; chosen3 (optional) receives it */
int lbx_ensemble_autotune(lbx_ensemble* e, int trial_steps, int* chosen3);
int lbx_ensemble_set_config(lbx_ensemble* e, int tile_cells, int block, int cells_per_thread);
/* advance every box by nsteps (asynchronous on the ensemble's stream) */
int lbx_ensemble_iterate(lbx_ensemble* e, int nsteps);
/* lbx_ensemble_iterate bracketed by CUDA events on the ensemble's stream;
 * waits and returns the device time in *ms */
int lbx_ensemble_iterate_timed(lbx_ensemble* e, int nsteps, double* ms);
/* f of box b in FP64, FAB order (n >= 15 * cells of the box) */
int lbx_ensemble_copy_f(lbx_ensemble* e, int b, double* out, size_t n);
/* rho[k][j][i], u[n][k][j][i] of box b */
int lbx_ensemble_hydro(lbx_ensemble* e, int b, double* rho, double* u, size_t ncells);
int lbx_ensemble_synchronize(lbx_ensemble* e);
int lbx_ensemble_get_stream(const lbx_ensemble* e, void** stream);
/* kernel launches issued by the last lbx_ensemble_iterate */
int lbx_ensemble_launches(const lbx_ensemble* e, long long* out);

/* ---- serving loop (continuous batching of simulation requests) --------
 * A request is a periodic simulation of 1..3 levels (refinement ratio 2,
 * each refined box the centred half of its parent, conservative coupling,
 * tau_{l+1} = 2 tau_l), starting from rho = 1 + amplitude on one plane and
 * u = 0.  Requests are admitted first-come first-served while a slot is free
 * and their stores fit the HBM budget, stay resident until done, and advance
 * together: each phase of a coarse step is one persistent launch over the
 * tiles of every resident request, and pairs of coarse steps replay a
 * captured CUDA graph.  Requests join and leave at coarse-step boundaries. */
typedef struct lbx_server lbx_server;
typedef struct lbx_request {
  int levels;       /* 1..3 */
  int nx, ny, nz;   /* coarse extents (multiples of 2^(levels+1) when refined, >= 8) */
  int steps;        /* coarse steps to run */
  double tau;       /* tau_s = tau_b on the coarse level */
  int pulse_axis;   /* 0..2 */
  int pulse_index;  /* plane index on the coarse level */
  double amplitude; /* rho = 1 + amplitude on that plane */
  int keep_field;   /* 1: keep the level-0 density for lbx_server_take */
} lbx_request;
/* precision is LBX_F32_SHIFTED or LBX_F64 for every request of the server */
int lbx_server_create(size_t hbm_budget_bytes, int max_active, int precision, lbx_server** out);
int lbx_server_destroy(lbx_server* s);
/* queue a request; *id receives its ticket (LBX_ERR_OOM if it can never fit
 * the budget, LBX_ERR_UNSUPPORTED if a level's box has 2^23 or more cells or
 * a plane of 2^17 or more, ghost layers included) */
int lbx_server_submit(lbx_server* s, const lbx_request* req, long long* id);
/* admit what fits, advance every resident request by min(quantum, fewest
 * remaining steps) coarse steps, retire finished ones; waits for the GPU */
int lbx_server_pump(lbx_server* s, int quantum, int* active, int* queued);
/* *done = 1 once finished; then *mass (composite mass) and *probe (level-0
 * density at the pulse plane, centre of the other axes) are set */
int lbx_server_poll(lbx_server* s, long long id, int* done, double* mass, double* probe);
/* level-0 density of a finished request (FAB order; only when submitted
 * with keep_field, rho may be NULL), then forget it */
int lbx_server_take(lbx_server* s, long long id, double* rho, size_t n);
int lbx_server_stats(const lbx_server* s, long long* cell_updates, size_t* bytes_in_use,
                     long long* launches);
/* host wall seconds spent admitting, retiring, rebuilding the batch tables
 * and stepping (the last includes waiting for the GPU) */
int lbx_server_timing(const lbx_server* s, double* seconds4);
/* launch shape of the server's step kernels: cells per tile, threads per
 * block (32..512, a multiple of 32) and cells per thread (1 or 2); takes
 * effect at the next pump (tables and graph are rebuilt) */
int lbx_server_set_config(lbx_server* s, int tile_cells, int block, int cells_per_thread);

#ifdef __cplusplus
}
#endif
#endif /* LBX_H */
