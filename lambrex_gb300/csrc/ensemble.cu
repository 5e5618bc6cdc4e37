// ensemble.cu -- batched ensemble of independent periodic simulations
// (lbx_ensemble_* in lbx.h).  All boxes advance in one persistent launch per
// step over a device tile work-list; steps are replayed from a captured CUDA
// graph of two launches; tile size, block size and cells per thread come
// from a timing autotuner.  The reference has no batching: each box here is
// an independent AmrSim single-level run (src/AmrSim.cpp:981-985).
#include <algorithm>
#include <cstring>
#include <vector>

#include "batch.cuh"
#include "ensemble_internal.h"
#include "lbx.h"
#include "sim_internal.h"

#define CK(call)                            \
  do {                                      \
    cudaError_t e_ = (call);                \
    if (e_ != cudaSuccess) {                \
      lbx::note_error(#call, e_);           \
      return lbx::status_from_cuda(e_);     \
    }                                       \
  } while (0)
#define RET(call)                \
  do {                           \
    int r_ = (call);             \
    if (r_ != LBX_OK) return r_; \
  } while (0)

namespace lbx {

int init_box_state(const BBox& b, int precision, int now, const double* rho_c, const double* u_c,
                   cudaStream_t st) {
  const int nx = b.b.n[0], ny = b.b.n[1], nz = b.b.n[2];
  const size_t N = (size_t)nx * ny * nz;
  double* d = nullptr;
  CK(cudaMallocAsync(&d, 8 * N * sizeof(double), st));
  cudaError_t e = cudaMemcpyAsync(d, rho_c, N * sizeof(double), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d + N, u_c, 3 * N * sizeof(double), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = launch_c_to_fab(d, d + N, d + 4 * N, d + 5 * N, nx, ny, nz, st);
  if (e == cudaSuccess) {
    const size_t bytes = (size_t)NV * b.b.sq * (precision == LBX_F64 ? 8 : 4);
    e = cudaMemsetAsync(b.buf[now], 0, bytes, st);
  }
  if (e == cudaSuccess)
    e = precision == LBX_F64
            ? launch_equilibrium<double>(d + 4 * N, d + 5 * N, static_cast<double*>(b.buf[now]),
                                         b.b, 0.0, st)
            : launch_equilibrium<float>(d + 4 * N, d + 5 * N, static_cast<float*>(b.buf[now]),
                                        b.b, b.rho0, st);
  cudaFreeAsync(d, st);
  CK(e);
  return LBX_OK;
}

}  // namespace lbx

using lbx::BBox;
using lbx::BTile;
using lbx::Range;

struct lbx_ensemble {
  int nbox = 0;
  int precision = LBX_F32_SHIFTED;
  std::vector<BBox> hb;
  BBox* d_boxes = nullptr;
  std::vector<BTile> ht;
  BTile* d_tiles = nullptr;
  int tile_cells = 8192, block = 256, cpt = 1, grid = 0;
  int flip = 0;  // all boxes step together: store "now" is par ^ flip
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  cudaGraphExec_t gexec = nullptr;
  long long launches = 0, last_launches = 0;
  size_t esize() const { return precision == LBX_F64 ? 8 : 4; }
};

namespace {

int upload_tiles(lbx_ensemble* e) {
  std::vector<int> ids(e->nbox);
  for (int i = 0; i < e->nbox; ++i) ids[i] = i;
  e->ht = lbx::make_tiles(e->hb, ids, e->tile_cells);
  if (e->d_tiles) cudaFree(e->d_tiles);
  e->d_tiles = nullptr;
  CK(cudaMalloc(&e->d_tiles, e->ht.size() * sizeof(BTile)));
  CK(cudaMemcpyAsync(e->d_tiles, e->ht.data(), e->ht.size() * sizeof(BTile), cudaMemcpyHostToDevice,
                     e->stream));
  const int per_sm = e->precision == LBX_F64
                         ? lbx::b_step_blocks_per_sm<double>(e->block, e->cpt, lbx::kBoxPull)
                         : lbx::b_step_blocks_per_sm<float>(e->block, e->cpt, lbx::kBoxPull);
  e->grid = e->num_sms * per_sm;
  if (e->gexec) {
    cudaGraphExecDestroy(e->gexec);
    e->gexec = nullptr;
  }
  return LBX_OK;
}

cudaError_t step_launch(lbx_ensemble* e, int flip) {
  const int n = (int)e->ht.size();
  return e->precision == LBX_F64
             ? lbx::launch_b_step<double>(e->d_boxes, e->d_tiles, n, flip, e->grid, e->block, e->cpt,
                                          lbx::kBoxPull, e->stream)
             : lbx::launch_b_step<float>(e->d_boxes, e->d_tiles, n, flip, e->grid, e->block, e->cpt,
                                         lbx::kBoxPull, e->stream);
}

int build_graph(lbx_ensemble* e) {
  if (e->gexec) return LBX_OK;
  cudaGraph_t g = nullptr;
  CK(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
  cudaError_t a = step_launch(e, 0);
  cudaError_t b = step_launch(e, 1);
  cudaError_t c = cudaStreamEndCapture(e->stream, &g);
  CK(a);
  CK(b);
  CK(c);
  cudaError_t d = cudaGraphInstantiate(&e->gexec, g, 0);
  cudaGraphDestroy(g);
  CK(d);
  return LBX_OK;
}

int advance(lbx_ensemble* e, int nsteps) {
  if (nsteps <= 0) return LBX_OK;
  if (e->flip == 1) {  // realign so that graph replays start at flip 0
    CK(step_launch(e, 1));
    e->flip = 0;
    --nsteps;
    ++e->launches;
  }
  if (nsteps >= 2) RET(build_graph(e));
  for (int i = 0; i + 1 < nsteps; i += 2) {
    CK(cudaGraphLaunch(e->gexec, e->stream));
    e->launches += 2;
  }
  if (nsteps & 1) {
    CK(step_launch(e, 0));
    e->flip = 1;
    ++e->launches;
  }
  return LBX_OK;
}

int box_now(const lbx_ensemble* e, int b) { return e->hb[b].par ^ e->flip; }

}  // namespace

extern "C" {

int lbx_ensemble_create(int nbox, const int* dims, const double* tau, int precision,
                        lbx_ensemble** out) {
  if (!out || nbox <= 0 || !dims || !tau) return LBX_ERR_ARG;
  if (precision != LBX_F64 && precision != LBX_F32_SHIFTED) return LBX_ERR_ARG;
  *out = nullptr;
  for (int b = 0; b < nbox; ++b)
    for (int d = 0; d < 3; ++d)
      if (dims[3 * b + d] <= 0) return LBX_ERR_ARG;
  lbx_ensemble* e = new lbx_ensemble();
  e->nbox = nbox;
  e->precision = precision;
  int dev = 0;
  cudaError_t err = cudaGetDevice(&dev);
  if (err == cudaSuccess) err = cudaDeviceGetAttribute(&e->num_sms, cudaDevAttrMultiProcessorCount, dev);
  if (err == cudaSuccess) err = cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking);
  e->hb.resize(nbox);
  for (int b = 0; b < nbox && err == cudaSuccess; ++b) {
    BBox& B = e->hb[b];
    std::memset(&B, 0, sizeof(B));
    B.b = lbx::make_box(dims[3 * b], dims[3 * b + 1], dims[3 * b + 2], 0);
    B.cov = lbx::empty_ibox();
    B.periodic = 1;
    B.pull = 1;
    B.par = 0;
    B.om_s = B.om_b = 1.0 / (tau[b] + 0.5);  // src/AmrSim.cpp:125-126
    B.rho0 = precision == LBX_F64 ? 0.0 : 1.0;
    if (!lbx::set_iteration_space(B)) {
      lbx_ensemble_destroy(e);
      return LBX_ERR_UNSUPPORTED;
    }
    const size_t bytes = (size_t)lbx::NV * B.b.sq * e->esize();
    for (int k = 0; k < 2 && err == cudaSuccess; ++k) err = cudaMalloc(&B.buf[k], bytes);
    for (int k = 0; k < 2 && err == cudaSuccess; ++k) err = cudaMemsetAsync(B.buf[k], 0, bytes, e->stream);
  }
  if (err == cudaSuccess) err = cudaMalloc(&e->d_boxes, nbox * sizeof(BBox));
  if (err == cudaSuccess)
    err = cudaMemcpyAsync(e->d_boxes, e->hb.data(), nbox * sizeof(BBox), cudaMemcpyHostToDevice, e->stream);
  if (err != cudaSuccess) {
    lbx::note_error("lbx_ensemble_create", err);
    lbx_ensemble_destroy(e);
    return lbx::status_from_cuda(err);
  }
  int rc = upload_tiles(e);
  if (rc != LBX_OK) {
    lbx_ensemble_destroy(e);
    return rc;
  }
  *out = e;
  return LBX_OK;
}

int lbx_ensemble_destroy(lbx_ensemble* e) {
  if (!e) return LBX_OK;
  if (e->stream) cudaStreamSynchronize(e->stream);
  if (e->gexec) cudaGraphExecDestroy(e->gexec);
  for (auto& B : e->hb)
    for (auto& p : B.buf)
      if (p) cudaFree(p);
  if (e->d_boxes) cudaFree(e->d_boxes);
  if (e->d_tiles) cudaFree(e->d_tiles);
  if (e->stream) cudaStreamDestroy(e->stream);
  delete e;
  return LBX_OK;
}

int lbx_ensemble_init_box(lbx_ensemble* e, int b, const double* rho, size_t nrho, const double* u,
                          size_t nu) {
  if (!e || b < 0 || b >= e->nbox || !rho || !u) return LBX_ERR_ARG;
  Range range("lbx_ensemble_init_box");
  BBox& B = e->hb[b];
  const size_t N = (size_t)B.b.n[0] * B.b.n[1] * B.b.n[2];
  if (nrho < N || nu < 3 * N) return LBX_ERR_RANGE;
  if (e->precision == LBX_F32_SHIFTED) {
    double part[4] = {0, 0, 0, 0};
    for (size_t c = 0; c < N; ++c) part[c & 3] += rho[c];
    B.rho0 = ((part[0] + part[1]) + (part[2] + part[3])) / (double)N;
  }
  const int now = box_now(e, b);
  RET(lbx::init_box_state(B, e->precision, now, rho, u, e->stream));
  // enter the pull form: the other store receives Q = S^-1(R) and becomes "now"
  CK(e->precision == LBX_F64
         ? lbx::launch_unstream<double>(static_cast<double*>(B.buf[now]), static_cast<double*>(B.buf[now ^ 1]), B.b, e->stream)
         : lbx::launch_unstream<float>(static_cast<float*>(B.buf[now]), static_cast<float*>(B.buf[now ^ 1]), B.b, e->stream));
  B.par ^= 1;
  CK(cudaMemcpyAsync(e->d_boxes + b, &B, sizeof(BBox), cudaMemcpyHostToDevice, e->stream));
  CK(cudaStreamSynchronize(e->stream));
  return LBX_OK;
}

int lbx_ensemble_set_config(lbx_ensemble* e, int tile_cells, int block, int cpt) {
  if (!e || tile_cells < 32 || (block != 128 && block != 256 && block != 512) || cpt < 1 || cpt > 2)
    return LBX_ERR_ARG;
  e->tile_cells = tile_cells;
  e->block = block;
  e->cpt = cpt;
  return upload_tiles(e);
}

int lbx_ensemble_autotune(lbx_ensemble* e, int trial_steps, int* chosen3) {
  if (!e || trial_steps < 2) return LBX_ERR_ARG;
  Range range("lbx_ensemble_autotune");
  // keep the state: save every box's "now" store, time the candidates,
  // then restore stores, flip and launch counters
  std::vector<void*> saved(e->nbox, nullptr);
  const int flip0 = e->flip;
  const long long launches0 = e->launches;
  for (int b = 0; b < e->nbox; ++b) {
    const size_t bytes = (size_t)lbx::NV * e->hb[b].b.sq * e->esize();
    CK(cudaMallocAsync(&saved[b], bytes, e->stream));
    CK(cudaMemcpyAsync(saved[b], e->hb[b].buf[box_now(e, b)], bytes, cudaMemcpyDeviceToDevice, e->stream));
  }
  const int tiles[] = {2048, 8192, 32768};
  const int blocks[] = {128, 256, 512};
  const int cpts[] = {1, 2};
  float best = 1e30f;
  int bt = e->tile_cells, bb = e->block, bc = e->cpt;
  cudaEvent_t a, z;
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&z));
  int rc = LBX_OK;
  for (int t : tiles)
    for (int bl : blocks)
      for (int c : cpts) {
        if ((rc = lbx_ensemble_set_config(e, t, bl, c)) != LBX_OK) break;
        if ((rc = advance(e, 2)) != LBX_OK) break;  // warm-up, builds the graph
        cudaEventRecord(a, e->stream);
        if ((rc = advance(e, trial_steps)) != LBX_OK) break;
        cudaEventRecord(z, e->stream);
        cudaEventSynchronize(z);
        float ms = 0;
        cudaEventElapsedTime(&ms, a, z);
        if (ms < best) {
          best = ms;
          bt = t;
          bb = bl;
          bc = c;
        }
      }
  cudaEventDestroy(a);
  cudaEventDestroy(z);
  e->flip = flip0;
  for (int b = 0; b < e->nbox; ++b) {
    const size_t bytes = (size_t)lbx::NV * e->hb[b].b.sq * e->esize();
    cudaMemcpyAsync(e->hb[b].buf[box_now(e, b)], saved[b], bytes, cudaMemcpyDeviceToDevice, e->stream);
    cudaFreeAsync(saved[b], e->stream);
  }
  e->launches = launches0;
  RET(rc);
  RET(lbx_ensemble_set_config(e, bt, bb, bc));
  CK(cudaStreamSynchronize(e->stream));
  if (chosen3) {
    chosen3[0] = bt;
    chosen3[1] = bb;
    chosen3[2] = bc;
  }
  return LBX_OK;
}

int lbx_ensemble_iterate(lbx_ensemble* e, int nsteps) {
  if (!e || nsteps < 0) return LBX_ERR_ARG;
  Range range("lbx_ensemble_iterate");
  const long long l0 = e->launches;
  RET(advance(e, nsteps));
  e->last_launches = e->launches - l0;
  return LBX_OK;
}

int lbx_ensemble_iterate_timed(lbx_ensemble* e, int nsteps, double* ms) {
  if (!e || nsteps < 0 || !ms) return LBX_ERR_ARG;
  cudaEvent_t a, z;
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&z));
  CK(cudaEventRecord(a, e->stream));
  const int rc = lbx_ensemble_iterate(e, nsteps);
  CK(cudaEventRecord(z, e->stream));
  CK(cudaEventSynchronize(z));
  float t = 0.f;
  CK(cudaEventElapsedTime(&t, a, z));
  cudaEventDestroy(a);
  cudaEventDestroy(z);
  *ms = t;
  return rc;
}

int lbx_ensemble_copy_f(lbx_ensemble* e, int b, double* out, size_t n) {
  if (!e || b < 0 || b >= e->nbox || !out) return LBX_ERR_ARG;
  const BBox& B = e->hb[b];
  const size_t need = (size_t)lbx::NV * B.b.n[0] * B.b.n[1] * B.b.n[2];
  if (n < need) return LBX_ERR_ARG;
  double* d = nullptr;
  CK(cudaMallocAsync(&d, need * sizeof(double), e->stream));
  const int now = box_now(e, b);
  cudaError_t err = e->precision == LBX_F64
                        ? lbx::launch_copy_out<double>(static_cast<double*>(B.buf[now]), B.b, 0.0, d, e->stream, B.pull != 0)
                        : lbx::launch_copy_out<float>(static_cast<float*>(B.buf[now]), B.b, B.rho0, d, e->stream, B.pull != 0);
  if (err == cudaSuccess) err = cudaMemcpyAsync(out, d, need * sizeof(double), cudaMemcpyDeviceToHost, e->stream);
  cudaFreeAsync(d, e->stream);
  if (err == cudaSuccess) err = cudaStreamSynchronize(e->stream);
  CK(err);
  return LBX_OK;
}

int lbx_ensemble_hydro(lbx_ensemble* e, int b, double* rho, double* u, size_t ncells) {
  if (!e || b < 0 || b >= e->nbox || !rho || !u) return LBX_ERR_ARG;
  const BBox& B = e->hb[b];
  const size_t N = (size_t)B.b.n[0] * B.b.n[1] * B.b.n[2];
  if (ncells < N) return LBX_ERR_ARG;
  double* d = nullptr;
  CK(cudaMallocAsync(&d, 4 * N * sizeof(double), e->stream));
  const int now = box_now(e, b);
  cudaError_t err = e->precision == LBX_F64
                        ? lbx::launch_hydro<double>(static_cast<double*>(B.buf[now]), B.b, 0.0, d, d + N, e->stream, B.pull != 0)
                        : lbx::launch_hydro<float>(static_cast<float*>(B.buf[now]), B.b, B.rho0, d, d + N, e->stream, B.pull != 0);
  if (err == cudaSuccess) err = cudaMemcpyAsync(rho, d, N * sizeof(double), cudaMemcpyDeviceToHost, e->stream);
  if (err == cudaSuccess) err = cudaMemcpyAsync(u, d + N, 3 * N * sizeof(double), cudaMemcpyDeviceToHost, e->stream);
  cudaFreeAsync(d, e->stream);
  if (err == cudaSuccess) err = cudaStreamSynchronize(e->stream);
  CK(err);
  return LBX_OK;
}

int lbx_ensemble_synchronize(lbx_ensemble* e) {
  if (!e) return LBX_ERR_ARG;
  CK(cudaStreamSynchronize(e->stream));
  return LBX_OK;
}

int lbx_ensemble_get_stream(const lbx_ensemble* e, void** stream) {
  if (!e || !stream) return LBX_ERR_ARG;
  *stream = (void*)e->stream;
  return LBX_OK;
}

int lbx_ensemble_launches(const lbx_ensemble* e, long long* out) {
  if (!e || !out) return LBX_ERR_ARG;
  *out = e->last_launches;
  return LBX_OK;
}

}  // extern "C"
