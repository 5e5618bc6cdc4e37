// batch_kernels.cu -- persistent kernels of the batch engine.  Every launch
// walks a tile work-list (box, first cell, cell count) with a grid sized to
// the SM count; tiles of all boxes of a phase (independent simulations,
// AMR levels of several requests) share the launch.
#include "batch.cuh"
#include "cells.cuh"

namespace lbx {

namespace {

// One kernel per box kind (every launch covers boxes of one kind), so each
// instantiation carries only its own cell body.  The tile's box descriptor
// is staged in shared memory: the cell code reads its geometry from there
// instead of holding it in registers, which keeps occupancy high.
template <typename T, int KIND, int CPT>
__global__ void __launch_bounds__(512) k_b_step(const BBox* __restrict__ boxes,
                                                const BTile* __restrict__ tiles, int ntiles,
                                                int flip) {
  __shared__ BBox sbox;
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const BTile tl = tiles[t];
    __syncthreads();  // the previous tile is done with sbox
    if (threadIdx.x == 0) sbox = boxes[tl.box];
    __syncthreads();
    const BBox& B = sbox;
    const int par = B.par ^ flip;
    const T* __restrict__ fin = static_cast<const T*>(B.buf[par]);
    T* __restrict__ fout = static_cast<T*>(B.buf[par ^ 1]);
    const Box3& b = B.b;
    const IBox& cov = B.cov;
    const T om_s = (T)B.om_s, om_b = (T)B.om_b, rho0 = (T)B.rho0;
    const unsigned long long mx = B.mx, mxy = B.mxy;
    const int dx = B.dx, dxy = B.dxy;
    for (int i0 = threadIdx.x; i0 < tl.count; i0 += blockDim.x * CPT) {
#pragma unroll
      for (int u = 0; u < CPT; ++u) {
        const int i = i0 + u * blockDim.x;
        if (i >= tl.count) break;
        const unsigned c = (unsigned)(tl.start + i);
        const int z = fdiv(c, mxy);
        const unsigned r = c - (unsigned)z * (unsigned)dxy;
        const int y = fdiv(r, mx);
        const int x = (int)(r - (unsigned)y * (unsigned)dx);
        // boxes of the batch engine are below 2^23 cells: 32-bit indices
        if constexpr (KIND == kBoxPull)
          cell_step_pull<T, false, int>(fin, fout, b, x, y, z, om_s, om_b, rho0, DfRates{});
        else if constexpr (KIND == kBoxPeriodic)
          cell_step_periodic_pull<T, int>(fin, fout, b, cov, x, y, z, om_s, om_b, rho0);
        else
          cell_step_patch_pull<T, int>(fin, fout, b, cov, x, y, z, om_s, om_b, rho0);
      }
    }
  }
}

template <typename T, int KIND>
int occupancy(int block, int cpt) {
  int n = 0;
  if (cpt >= 2)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_b_step<T, KIND, 2>, block, 0);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_b_step<T, KIND, 1>, block, 0);
  return n;
}

template <typename T, int KIND>
void launch_kind(const BBox* boxes, const BTile* tiles, int ntiles, int flip, int grid, int block,
                 int cpt, cudaStream_t st) {
  if (cpt >= 2)
    k_b_step<T, KIND, 2><<<grid, block, 0, st>>>(boxes, tiles, ntiles, flip);
  else
    k_b_step<T, KIND, 1><<<grid, block, 0, st>>>(boxes, tiles, ntiles, flip);
}

template <typename T>
__global__ void k_b_explode(const BBox* __restrict__ boxes, const BCoupling* __restrict__ cps,
                            const BTile* __restrict__ tiles, int ntiles, int flip_c, int flip_f) {
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const BTile tl = tiles[t];
    const BCoupling& cp = cps[tl.box];
    const BBox& C = boxes[cp.cbox];
    const BBox& F = boxes[cp.fbox];
    const T* coarse = static_cast<const T*>(C.buf[C.par ^ flip_c]);
    T* fine = static_cast<T*>(F.buf[F.par ^ flip_f]);
    for (int i = threadIdx.x; i < tl.count; i += blockDim.x) {
      int s[3];
      if (ghost_coords(cp.c.fb, tl.start + i, s))  // the ghost shell only
        cell_explode<T, false, int, true>(coarse, fine, cp.c, s[0], s[1], s[2], (T)C.om_s,
                                          (T)C.om_b, (T)C.rho0);
    }
  }
}

template <typename T>
__global__ void k_b_coalesce(const BBox* __restrict__ boxes, const BCoupling* __restrict__ cps,
                             const BTile* __restrict__ tiles, int ntiles, int flip_c, int flip_f) {
  // ring-cell coordinates are decoded once per cell into shared memory, then
  // the block's threads take the (ring cell, population) items
  constexpr int kChunk = 256;
  __shared__ int sr[kChunk][3];
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const BTile tl = tiles[t];
    const BCoupling& cp = cps[tl.box];
    const BBox& C = boxes[cp.cbox];
    const BBox& F = boxes[cp.fbox];
    T* coarse = static_cast<T*>(C.buf[C.par ^ flip_c]);
    const T* fine = static_cast<const T*>(F.buf[F.par ^ flip_f]);
    for (int c0 = 0; c0 < tl.count; c0 += kChunk) {
      const int nc = min(kChunk, tl.count - c0);
      __syncthreads();  // the previous chunk is done with sr
      for (int i = threadIdx.x; i < nc; i += blockDim.x) {
        int r[3];
        if (!ring_coords(cp.c, tl.start + c0 + i, r)) r[0] = -1;
        sr[i][0] = r[0];
        sr[i][1] = r[1];
        sr[i][2] = r[2];
      }
      __syncthreads();
      // ring cells fastest: a warp's items are neighbouring ring cells of one
      // population, whose fine children and coarse entries lie side by side
      for (int i = threadIdx.x; i < nc * NV; i += blockDim.x) {
        const int q = i / nc, cell = i - q * nc;
        if (sr[cell][0] >= 0)
          cell_coalesce_q<T, int, true>(fine, coarse, cp.c, sr[cell][0], sr[cell][1], sr[cell][2],
                                        q, (T)C.rho0);
      }
    }
  }
}

template <typename T>
__global__ void k_b_to_qform(T* f, Box3 b, IBox cov, T om_s, T om_b, T rho0) {
  const int n = b.n[0] * b.n[1] * b.n[2];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int x = i % b.n[0], y = (i / b.n[0]) % b.n[1], z = i / (b.n[0] * b.n[1]);
    cell_to_qform<T, int>(f, b, cov, x, y, z, om_s, om_b, rho0);
  }
}

template <typename T>
__global__ void k_b_to_rform(const T* __restrict__ qprev, T* __restrict__ r, Box3 b) {
  const int n = b.n[0] * b.n[1] * b.n[2];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int x = i % b.n[0], y = (i / b.n[0]) % b.n[1], z = i / (b.n[0] * b.n[1]);
    cell_to_rform<T, int>(qprev, r, b, x, y, z);
  }
}

int conversion_blocks(const Box3& b) {
  const long long n = (long long)b.n[0] * b.n[1] * b.n[2];
  return (int)std::min<long long>((n + 255) / 256, 4096);
}

}  // namespace

template <typename T>
cudaError_t launch_b_to_qform(T* f, const Box3& b, const IBox& cov, double om_s, double om_b,
                              double rho0, cudaStream_t st) {
  k_b_to_qform<T><<<conversion_blocks(b), 256, 0, st>>>(f, b, cov, (T)om_s, (T)om_b, (T)rho0);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_b_to_rform(const T* qprev, T* r, const Box3& b, cudaStream_t st) {
  k_b_to_rform<T><<<conversion_blocks(b), 256, 0, st>>>(qprev, r, b);
  return cudaGetLastError();
}

template <typename T>
int b_step_blocks_per_sm(int block, int cpt, int kind) {
  const int n = kind == kBoxPull ? occupancy<T, kBoxPull>(block, cpt)
                : kind == kBoxPeriodic ? occupancy<T, kBoxPeriodic>(block, cpt)
                                       : occupancy<T, kBoxPatch>(block, cpt);
  return n > 0 ? n : 1;
}
template int b_step_blocks_per_sm<float>(int, int, int);
template int b_step_blocks_per_sm<double>(int, int, int);

template <typename T>
cudaError_t launch_b_step(const BBox* boxes, const BTile* tiles, int ntiles, int flip, int grid,
                          int block, int cpt, int kind, cudaStream_t st) {
  if (ntiles <= 0) return cudaSuccess;
  grid = grid < ntiles ? grid : ntiles;
  if (kind == kBoxPull)
    launch_kind<T, kBoxPull>(boxes, tiles, ntiles, flip, grid, block, cpt, st);
  else if (kind == kBoxPeriodic)
    launch_kind<T, kBoxPeriodic>(boxes, tiles, ntiles, flip, grid, block, cpt, st);

  else
    launch_kind<T, kBoxPatch>(boxes, tiles, ntiles, flip, grid, block, cpt, st);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_b_explode(const BBox* boxes, const BCoupling* cps, const BTile* tiles,
                             int ntiles, int flip_c, int flip_f, cudaStream_t st) {
  if (ntiles <= 0) return cudaSuccess;
  k_b_explode<T><<<ntiles, 128, 0, st>>>(boxes, cps, tiles, ntiles, flip_c, flip_f);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_b_coalesce(const BBox* boxes, const BCoupling* cps, const BTile* tiles,
                              int ntiles, int flip_c, int flip_f, cudaStream_t st) {
  if (ntiles <= 0) return cudaSuccess;
  k_b_coalesce<T><<<ntiles, 128, 0, st>>>(boxes, cps, tiles, ntiles, flip_c, flip_f);
  return cudaGetLastError();
}

#define LBX_INST(T)                                                                             \
  template cudaError_t launch_b_step<T>(const BBox*, const BTile*, int, int, int, int, int, int,\
                                        cudaStream_t);                                          \
  template cudaError_t launch_b_explode<T>(const BBox*, const BCoupling*, const BTile*, int,    \
                                           int, int, cudaStream_t);                             \
  template cudaError_t launch_b_coalesce<T>(const BBox*, const BCoupling*, const BTile*, int,   \
                                            int, int, cudaStream_t);                            \
  template cudaError_t launch_b_to_qform<T>(T*, const Box3&, const IBox&, double, double, double,\
                                            cudaStream_t);                                      \
  template cudaError_t launch_b_to_rform<T>(const T*, T*, const Box3&, cudaStream_t);
LBX_INST(double)
LBX_INST(float)
#undef LBX_INST

}  // namespace lbx
