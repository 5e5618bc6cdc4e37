// batch.cuh -- device side of the batch engine: many boxes (independent
// simulations, AMR levels of several requests) advance in one persistent
// launch driven by a device tile work-list.
//
// Each box has two stores; which one is "now" is par ^ flip, with par kept
// per box in the table and flip passed to the launch.  A captured sequence
// whose every box steps an even number of times leaves all parities where
// they started, so the same CUDA graph can be replayed without host
// bookkeeping between replays.
#pragma once
#include <algorithm>
#include <vector>

#include "kernels.cuh"

namespace lbx {

struct BBox {
  void* buf[2];      // the two stores (T*)
  Box3 b;            // geometry: valid extents, ghost width, strides
  IBox cov;          // inactive (covered) cells, valid-relative; empty if none
  int periodic;      // 1: wrap over the valid region (level 0); 0: AMR patch
  int pull;          // periodic boxes only: the store holds Q_n = C(R_{n-1})
                     // and steps gather (cells.cuh, pull form)
  int par;           // store index of "now" when flip == 0
  unsigned long long mx, mxy;  // fast-division magics (2^40 / d + 1) of the iteration space
  int dx, dxy;       // divisors: row length and plane size of the iteration space
  double om_s, om_b, rho0;
};

struct BTile {
  int box;    // index into the box (or coupling) table
  int start;  // first cell of the tile in the iteration space
  int count;  // cells in the tile
};

// coarse/fine pair of boxes inside the batch (AMR coupling of one request)
struct BCoupling {
  Coupling c;
  int cbox, fbox;  // box-table indices of the coarse and the fine level
  int nring;       // coarse ring cells (grown coarsened patch minus interior)
};

// Division by an iteration-space extent d: q = (x * m) >> 40 with
// m = floor(2^40 / d) + 1 equals x / d whenever x * d < 2^40, and x * m
// stays below 2^64 for x < 2^23.  The batch engine therefore limits a box's
// iteration space to fewer than 2^23 cells and its plane to fewer than 2^17.
constexpr long long kMaxBatchCells = 1ll << 23;
constexpr long long kMaxBatchPlane = 1ll << 17;
inline unsigned long long fastdiv_magic(unsigned d) {
  return (1ull << 40) / d + 1ull;
}

// box kinds of a batch launch (every launch steps boxes of one kind); all
// in the pull form (cells.cuh): the stores hold post-collision populations
constexpr int kBoxPull = 0;      // periodic box (ensemble)
constexpr int kBoxPeriodic = 1;  // periodic box that may have covered cells (AMR level 0)
constexpr int kBoxPatch = 2;     // AMR patch with a ghost shell, may have covered cells

// resident blocks per SM of the batch step kernel (occupancy calculator)
template <typename T>
int b_step_blocks_per_sm(int block, int cpt, int kind);

// x / d for x < 2^23 and d < 2^17 with magic = fastdiv_magic(d)
__host__ __device__ __forceinline__ int fdiv(unsigned x, unsigned long long magic) {
  return (int)(((unsigned long long)x * magic) >> 40);
}

// fill the iteration-space fields of a box (periodic: valid cells; patch:
// storage cells); returns false if the box is too large for the 2^40 magic
inline bool set_iteration_space(BBox& b) {
  long long dx, dxy, cells;
  if (b.periodic) {
    dx = b.b.n[0];
    dxy = (long long)b.b.n[0] * b.b.n[1];
    cells = dxy * b.b.n[2];
  } else {
    dx = b.b.sx;
    dxy = b.b.sxy;
    cells = b.b.sq;
  }
  if (cells >= kMaxBatchCells || dxy >= kMaxBatchPlane) return false;
  b.dx = (int)dx;
  b.dxy = (int)dxy;
  b.mx = fastdiv_magic((unsigned)dx);
  b.mxy = fastdiv_magic((unsigned)dxy);
  return true;
}

// cells of a box's iteration space
inline long long box_cells(const BBox& b) {
  return b.periodic ? (long long)b.dxy * b.b.n[2] : b.b.sq;
}

// split the iteration space of each listed box into tiles of tile_cells
inline std::vector<BTile> make_tiles(const std::vector<BBox>& boxes, const std::vector<int>& ids,
                                     int tile_cells) {
  std::vector<BTile> t;
  for (int id : ids) {
    const long long n = box_cells(boxes[id]);
    for (long long s = 0; s < n; s += tile_cells)
      t.push_back(BTile{id, (int)s, (int)std::min<long long>(tile_cells, n - s)});
  }
  return t;
}

template <typename T>
cudaError_t launch_b_step(const BBox* boxes, const BTile* tiles, int ntiles, int flip, int grid,
                          int block, int cpt, int kind, cudaStream_t st);
// AMR levels of the batch engine in the pull form: a box's store `f` into
// it in place (after initialisation in the streamed state), and back (the
// streamed state gathered from the store before the last step into the
// latest one)
template <typename T>
cudaError_t launch_b_to_qform(T* f, const Box3& b, const IBox& cov, double om_s, double om_b,
                              double rho0, cudaStream_t st);
template <typename T>
cudaError_t launch_b_to_rform(const T* qprev, T* r, const Box3& b, cudaStream_t st);
// explode / coalesce over coupling tiles; flip_c / flip_f select
// the coarse and fine "now" stores at the time of the call (explosion and
// coalescence in the pull form)
template <typename T>
cudaError_t launch_b_explode(const BBox* boxes, const BCoupling* cps, const BTile* tiles,
                             int ntiles, int flip_c, int flip_f, cudaStream_t st);
template <typename T>
cudaError_t launch_b_coalesce(const BBox* boxes, const BCoupling* cps, const BTile* tiles,
                              int ntiles, int flip_c, int flip_f, cudaStream_t st);

}  // namespace lbx
