// kernels.cuh -- launchers of the device kernels of liblbx_cuda.so.
// All launchers are asynchronous on `st` and return cudaGetLastError().
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "d3q15.cuh"

namespace lbx {

// An axis-aligned box of cells in storage-valid coordinates (0..n-1 of the
// valid region); empty when hi < lo in any direction.
struct IBox {
  int lo[3], hi[3];
  __host__ __device__ bool contains(int x, int y, int z) const {
    return x >= lo[0] && x <= hi[0] && y >= lo[1] && y <= hi[1] && z >= lo[2] && z <= hi[2];
  }
};
inline IBox empty_ibox() { return IBox{{0, 0, 0}, {-1, -1, -1}}; }

// Launch shape of a kernel over rows of x: blocks of `threads` threads laid
// out as bx x by, bx = the row length rounded up to a warp (at most
// `threads`) and by = threads / bx rows, so that short rows (AMR patches,
// small boxes) do not leave most of a block idle.
struct RowLaunch {
  dim3 grid, block;
};
inline RowLaunch row_launch(int nx, int ny, int nz, int threads) {
  int bx = (nx + 31) / 32 * 32;
  if (bx > threads) bx = threads;
  const int by = threads / bx;
  return RowLaunch{dim3((unsigned)((nx + bx - 1) / bx), (unsigned)((ny + by - 1) / by), (unsigned)nz),
                   dim3((unsigned)bx, (unsigned)by, 1)};
}
#ifdef __CUDACC__
// (x, y, z) of this thread under row_launch
__device__ __forceinline__ void row_xyz(int& x, int& y, int& z) {
  x = blockIdx.x * blockDim.x + threadIdx.x;
  y = blockIdx.y * blockDim.y + threadIdx.y;
  z = blockIdx.z;
}
#endif

// ---- single box, fully periodic over its valid region -------------------
// One fused collide + push-stream step (now <- S(C(now))).  Cells inside
// `covered` are inactive: they emit zero populations (f = 0).
// paired: FP64 store with the collision carried in pairs of FP32 values
// (df32.cuh); ignored for the FP32 store.
template <typename T>
cudaError_t launch_step_periodic(const T* fin, T* fout, const Box3& b, IBox covered, double om_s,
                                 double om_b, double rho0, cudaStream_t st, int block = 128,
                                 bool paired = false);

// FP64 store, periodic push step with the paired collision in its one-cell
// scalar form (the device-pointer entry lbx_step_periodic_f64p)
cudaError_t launch_step_periodic_pairs_scalar(const double* fin, double* fout, const Box3& b,
                                              double om_s, double om_b, cudaStream_t st);

// compensated sum of x[0..n) into out4[0] (out4[1..3] = 0); partials holds
// kReduceBlocks x 8 doubles
cudaError_t launch_sum(const double* x, size_t n, double* partials, double* out4, cudaStream_t st);
// p[0..n) = v
cudaError_t launch_fill(double* p, size_t n, double v, cudaStream_t st);

// C-order user vectors (rho_c, u_c) -> FAB-order rho, u (nz <= 65535*128,
// ny and nx <= 65535).
cudaError_t launch_c_to_fab(const double* rho_c, const double* u_c, double* rho, double* u,
                            int nx, int ny, int nz, cudaStream_t st);

// Equilibrium of rho = 1 + amplitude on the plane coord[axis] == index and
// u = 0 (a request of the serving loop), shifted by rho0.
template <typename T>
cudaError_t launch_init_pulse(T* f, const Box3& b, int axis, int index, double amplitude,
                              double rho0, cudaStream_t st);

// Equilibrium of the valid region from double rho[k][j][i], u[n][k][j][i].
template <typename T>
cudaError_t launch_equilibrium(const double* rho, const double* u, T* f, const Box3& b,
                               double rho0, cudaStream_t st);
// rho, u (double, FAB order) of the valid region; gather = the store holds
// post-collision populations of a periodic box (pull form) and the
// streamed state is read through the neighbours.
template <typename T>
cudaError_t launch_hydro(const T* f, const Box3& b, double rho0, double* rho, double* u,
                         cudaStream_t st, bool gather = false);
// Cells to refine by density (solution-driven tagging): over an FP64
// density field in FAB order of extents n[3], the cells with
// |rho - ref| > threshold; box6 (device, int[6]) receives the bounding box
// (lo x,y,z then hi x,y,z; to be initialised to n / -1) and count (device)
// how many.  Blocks of 256 threads over rows of x.
cudaError_t launch_tag_density(const double* rho, const int* n, double ref, double threshold,
                               int* box6, unsigned long long* count, cudaStream_t st);
// valid region <-> packed FAB order in the storage type (raw values)
template <typename T>
cudaError_t launch_pack(const T* f, const Box3& b, T* out, cudaStream_t st);
template <typename T>
cudaError_t launch_unpack(const T* in, T* f, const Box3& b, cudaStream_t st);
// valid region <-> FP64 FAB order
template <typename T>
cudaError_t launch_copy_out(const T* f, const Box3& b, double rho0, double* out, cudaStream_t st,
                            bool gather = false);

// ---- pull form of a periodic box: the store holds Q_n = C(R_{n-1}) -----
// one step Q -> C(S(Q)); paired selects the paired-FP32 collision (FP64 store)
template <typename T>
cudaError_t launch_step_pull(const T* fin, T* fout, const Box3& b, double om_s, double om_b,
                             double rho0, bool paired, cudaStream_t st, int block = 256);
// the same step with CalcHydroVars fused in: rho, u of the state the step
// gathers (what launch_hydro with gather gives) are written on the way
template <typename T>
cudaError_t launch_step_pull_hydro(const T* fin, T* fout, const Box3& b, double om_s, double om_b,
                                   double rho0, bool paired, double* rho, double* u,
                                   cudaStream_t st);
// R -> Q = S^-1(R) into fout (entering the form)
template <typename T>
cudaError_t launch_unstream(const T* fin, T* fout, const Box3& b, cudaStream_t st);
// Q -> S(Q) = R into fout (leaving the form)
template <typename T>
cudaError_t launch_stream_gather(const T* fin, T* fout, const Box3& b, cudaStream_t st);
template <typename T>
cudaError_t launch_copy_in(const double* in, T* f, const Box3& b, double rho0, cudaStream_t st);

// Compensated FP64 sums over the valid region minus `skip`:
// out4 = {sum f, sum cx f, sum cy f, sum cz f}.  `partials` must hold
// reduce_partials_doubles() doubles; the kernels write every entry they read.
constexpr int kReduceBlocks = 512;
constexpr int kReduceThreads = 256;
inline size_t reduce_partials_doubles() { return (size_t)kReduceBlocks * 8; }
template <typename T>
cudaError_t launch_reduce(const T* f, const Box3& b, IBox skip, double rho0, double* partials,
                          double* out4, cudaStream_t st);

// ---- conservative two-level coupling ------------------------------------
// Geometry of a fine patch relative to its parent.  Global coordinates of
// level L are 0..N_L-1; storage-valid coordinate s maps to global lo + s.
struct Coupling {
  Box3 cb;        // coarse storage
  int clo[3];     // global coordinates of the coarse valid origin
  int cdom[3];    // coarse domain extents (periodic wrap of parent indices)
  int cper;       // 1 if the coarse level is the periodic level 0
  Box3 fb;        // fine storage (ghost width 2)
  int flo[3];     // global coordinates of the fine valid origin
};
// fine ghost shell <- coarse post-collision populations heading into the patch
// (paired: FP64 store, collision in paired FP32 as in launch_step_periodic)
template <typename T>
cudaError_t launch_explode(const T* coarse, T* fine, const Coupling& c, double om_s,
                           double om_b, double rho0, cudaStream_t st, bool paired = false);
// fused step of a patch level: valid cells collide (covered ones emit zero),
// ghost cells stream raw, populations leaving the storage are dropped.
template <typename T>
cudaError_t launch_step_patch(const T* fin, T* fout, const Box3& b, IBox covered, double om_s,
                              double om_b, double rho0, cudaStream_t st, bool paired = false);
// coarse ring cells += volume-weighted populations that left the patch
template <typename T>
cudaError_t launch_coalesce(const T* fine, T* coarse, const Coupling& c, double rho0,
                            cudaStream_t st);
// covered coarse cells <- mean of their eight children
template <typename T>
cudaError_t launch_restrict(const T* fine, T* coarse, const Coupling& c, cudaStream_t st);
// ---- rescaled coupling ------------------------------------------------------
// fine ghost shell <- parents collided at the explosion rates (om_s, om_b),
// wp x (coarse at the start of the coarse step) + wn x (coarse at its end)
template <typename T>
cudaError_t launch_explode_resc(const T* cprev, const T* cnow, T* fine, const Coupling& c,
                                double om_s, double om_b, double rho0, double wp, double wn,
                                cudaStream_t st, bool paired = false);
// covered coarse cells <- mean of their children collided at the restriction rates
template <typename T>
cudaError_t launch_restrict_resc(const T* fine, T* coarse, const Coupling& c, double om_s,
                                 double om_b, double rho0, cudaStream_t st, bool paired = false);
// level creation: fine grown box <- parent coarse cell (piecewise constant)
template <typename T>
cudaError_t launch_fill_from_coarse(const T* coarse, T* fine, const Coupling& c,
                                    cudaStream_t st);

// ---- reference-faithful Rohde cycle (FP64, ghost width 2 everywhere) ------
// FillPatchSingleLevel of the periodic level 0: every storage cell of dst
// <- the periodic image in src's valid region.
cudaError_t launch_f_fill_single(const double* src, double* dst, const Box3& b,
                                 cudaStream_t st);
// FillPatchTwoLevels + PCInterp: fine now where it (or a periodic image)
// exists, otherwise the parent cell of coarse now.  fdom = fine domain.
cudaError_t launch_f_fill_two(const double* fine_now, double* dst, const double* coarse_now,
                              const Coupling& c, const int* fdom, cudaStream_t st);
cudaError_t launch_f_zero_ring0(double* f, const Box3& b, cudaStream_t st);
cudaError_t launch_f_collide(double* f, const Box3& b, IBox covered, double om_s, double om_b,
                             cudaStream_t st, bool paired = false);
// pull stream over valid + 1 ring into a zeroed buffer
cudaError_t launch_f_stream(const double* src, double* dst, const Box3& b, cudaStream_t st);
cudaError_t launch_f_fill_boundary(double* f, const Box3& b, cudaStream_t st);
cudaError_t launch_f_zero_invalid(double* f, const Box3& b, cudaStream_t st);
// coarse next += mean of 2^3 fine blocks over the coarsened fine box grown by
// one, through every periodic image (sum_fine_to_coarse, FabArrayBase::ADD)
cudaError_t launch_f_sum_from_fine(const double* fine_now, double* coarse_next,
                                   const Coupling& c, cudaStream_t st);

}  // namespace lbx
