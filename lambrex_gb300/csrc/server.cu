// server.cu -- continuous-batching serving loop (lbx_server_* in lbx.h).
//
// Requests are simulations of 1..3 levels (ratio 2, each refined box half the
// parent extent, centred) run with the conservative volumetric coupling.  A
// request is admitted when its stores fit the HBM budget and a slot is free;
// it then stays resident.  Every pump advances all resident requests together
// in coarse steps: each phase (explode 0->1, explode 1->2, steps of level 2,
// coalesce 2->1, step level 1, ..., coalesce 1->0, step level 0) is one
// persistent launch over the tiles of every request that has that level, and
// pairs of coarse steps are replayed from a captured CUDA graph.  The levels
// are stepped in the pull form (their stores hold post-collision
// populations; the results are the push form's, bit for bit): a request is
// converted at admission and back to streamed states when it finishes.
// Finished requests leave at coarse-step boundaries and free their memory
// for the queue.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <map>
#include <vector>

#include "batch.cuh"
#include "cells.cuh"
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

using lbx::BBox;
using lbx::BCoupling;
using lbx::BTile;
using lbx::IBox;
using lbx::Range;

namespace {

constexpr int kMaxLevels = 3;
// cells per tile of the coupling kernels (128-thread blocks).  Explosion:
// one ghost cell per thread.  Coalescence: each ring cell is fifteen
// (cell, population) items of eight loads; 32 ring cells per block spread a
// launch over enough blocks to fill the GPU (256 per block left a launch of
// a few requests at 0.1 waves and 6 % of the warp slots, latency-bound).
constexpr int kExplodeTile = 128;
constexpr int kCoalesceTile = 32;

struct ReqLevel {
  int lo[3], hi[3];  // valid box in level coordinates
  BBox box;          // batch descriptor (buf, geometry, rates)
};

struct Req {
  long long id = 0;
  lbx_request r{};
  int state = 0;  // 0 queued, 1 active, 2 done
  int remaining = 0;
  int nlev = 1;
  ReqLevel lev[kMaxLevels];
  size_t bytes = 0;
  double mass = 0.0, probe = 0.0;
  std::vector<double> rho;  // level-0 density at completion (if kept)
};

size_t level_bytes(const int* n, int ghost, int esize) {
  return 2ull * lbx::NV * (size_t)(n[0] + 2 * ghost) * (n[1] + 2 * ghost) * (n[2] + 2 * ghost) * esize;
}

}  // namespace

struct lbx_server {
  size_t budget = 0, in_use = 0;
  int max_active = 0;
  int precision = LBX_F32_SHIFTED;
  std::deque<long long> queue;
  std::map<long long, Req> reqs;
  std::vector<long long> active;
  long long next_id = 1;
  // batch tables
  std::vector<BBox> hb;
  BBox* d_boxes = nullptr;
  std::vector<BCoupling> hc;
  BCoupling* d_cps = nullptr;
  std::vector<BTile> tiles_step[kMaxLevels], tiles_ex[2], tiles_co[2];
  BTile* d_tiles = nullptr;  // all tile lists back to back
  size_t off_step[kMaxLevels], off_ex[2], off_co[2];
  // the three tables back to back in one device buffer, filled from one
  // page-locked staging buffer; both grow only when a rebuild needs more
  char* d_tables = nullptr;
  char* h_tables = nullptr;
  size_t tables_cap = 0;
  int F[kMaxLevels] = {0, 0, 0};  // store "now" of a level-L box is par ^ F[L]
  bool dirty = true;
  cudaGraphExec_t gexec = nullptr;
  int graph_F0 = -1;
  long long graph_launches = 0;
  cudaStream_t stream = nullptr;
  cudaMemPool_t pool = nullptr;  // request stores (release threshold = budget)
  int num_sms = 0, block = 128, cpt = 1, tile_cells = 1024;  // measured best on GB300
  int grid[3] = {0, 0, 0};  // persistent grid per box kind (SMs x resident blocks)
  long long cell_updates = 0, launches = 0;
  long long updates_per_macro = 0;
  // host wall time spent admitting, retiring, rebuilding tables, and stepping
  // (stepping includes waiting for the GPU)
  double t_admit = 0, t_finish = 0, t_tables = 0, t_step = 0;
  size_t esize() const { return precision == LBX_F64 ? 8 : 4; }
};

namespace {

int free_request(lbx_server* s, Req& q) {
  for (int L = 0; L < q.nlev; ++L)
    for (auto& p : q.lev[L].box.buf)
      if (p) {
        cudaFreeAsync(p, s->stream);  // back to the pool, ordered after queued work
        p = nullptr;
      }
  s->in_use -= q.bytes;
  q.bytes = 0;
  return LBX_OK;
}

// geometry of a request: level 0 = the periodic coarse box; level L+1 =
// refine(centred half of level L)
void plan_levels(Req& q) {
  const lbx_request& r = q.r;
  int n[3] = {r.nx, r.ny, r.nz};
  q.nlev = r.levels;
  for (int d = 0; d < 3; ++d) {
    q.lev[0].lo[d] = 0;
    q.lev[0].hi[d] = n[d] - 1;
  }
  for (int L = 1; L < q.nlev; ++L)
    for (int d = 0; d < 3; ++d) {
      const int plo = q.lev[L - 1].lo[d], len = q.lev[L - 1].hi[d] - plo + 1;
      const int tlo = plo + len / 4, thi = plo + len / 4 + len / 2 - 1;
      q.lev[L].lo[d] = 2 * tlo;
      q.lev[L].hi[d] = 2 * thi + 1;
    }
}

size_t request_bytes(const Req& q, int esize) {
  size_t b = 0;
  for (int L = 0; L < q.nlev; ++L) {
    int n[3];
    for (int d = 0; d < 3; ++d) n[d] = q.lev[L].hi[d] - q.lev[L].lo[d] + 1;
    b += level_bytes(n, L ? 2 : 0, esize);
  }
  return b;
}

lbx::Coupling coupling_of(const Req& q, int L) {  // levels (L-1, L)
  lbx::Coupling c;
  c.cb = q.lev[L - 1].box.b;
  c.fb = q.lev[L].box.b;
  for (int d = 0; d < 3; ++d) {
    c.clo[d] = q.lev[L - 1].lo[d];
    c.flo[d] = q.lev[L].lo[d];
    c.cdom[d] = (d == 0 ? q.r.nx : d == 1 ? q.r.ny : q.r.nz) << (L - 1);
  }
  c.cper = (L - 1 == 0) ? 1 : 0;
  return c;
}

int admit(lbx_server* s, Req& q) {
  const int es = (int)s->esize();
  // level 0 starts from rho = 1 + amplitude on one plane, u = 0; the FP32
  // store is shifted by the mean density 1 + amplitude / extent
  const int n0[3] = {q.r.nx, q.r.ny, q.r.nz};
  const double rho0 =
      s->precision == LBX_F32_SHIFTED ? 1.0 + q.r.amplitude / n0[q.r.pulse_axis] : 0.0;
  double tau = q.r.tau;
  for (int L = 0; L < q.nlev; ++L) {
    ReqLevel& lv = q.lev[L];
    std::memset(&lv.box, 0, sizeof(BBox));
    int n[3];
    for (int d = 0; d < 3; ++d) n[d] = lv.hi[d] - lv.lo[d] + 1;
    lv.box.b = lbx::make_box(n[0], n[1], n[2], L ? 2 : 0);
    lv.box.periodic = L == 0 ? 1 : 0;
    lv.box.par = s->F[L];  // "now" is store 0 at admission
    lv.box.om_s = lv.box.om_b = 1.0 / (tau + 0.5);
    lv.box.rho0 = rho0;
    tau *= 2.0;  // conservative scheme: viscosity-preserving tau_{l+1} = 2 tau_l
    lv.box.cov = lbx::empty_ibox();
    if (!lbx::set_iteration_space(lv.box)) return LBX_ERR_UNSUPPORTED;
    const size_t bytes = (size_t)lbx::NV * lv.box.b.sq * es;
    for (int k = 0; k < 2; ++k) {
      // stream-ordered allocation from the server's pool: freed stores stay
      // in the pool for the next admission
      CK(cudaMallocFromPoolAsync(&lv.box.buf[k], bytes, s->pool, s->stream));
      CK(cudaMemsetAsync(lv.box.buf[k], 0, bytes, s->stream));
    }
  }
  for (int L = 0; L + 1 < q.nlev; ++L) {  // covered region of each coarse level
    IBox cov;
    for (int d = 0; d < 3; ++d) {
      cov.lo[d] = q.lev[L + 1].lo[d] / 2 - q.lev[L].lo[d];
      cov.hi[d] = q.lev[L + 1].hi[d] / 2 - q.lev[L].lo[d];
    }
    q.lev[L].box.cov = cov;
  }
  q.bytes = request_bytes(q, es);
  s->in_use += q.bytes;
  {
    const BBox& B0 = q.lev[0].box;
    cudaError_t e = s->precision == LBX_F64
                        ? lbx::launch_init_pulse<double>(static_cast<double*>(B0.buf[0]), B0.b, q.r.pulse_axis,
                                                         q.r.pulse_index, q.r.amplitude, 0.0, s->stream)
                        : lbx::launch_init_pulse<float>(static_cast<float*>(B0.buf[0]), B0.b, q.r.pulse_axis,
                                                        q.r.pulse_index, q.r.amplitude, rho0, s->stream);
    CK(e);
  }
  for (int L = 1; L < q.nlev; ++L) {  // new levels from their parent (piecewise constant)
    const lbx::Coupling c = coupling_of(q, L);
    cudaError_t e = s->precision == LBX_F64
                        ? lbx::launch_fill_from_coarse<double>(static_cast<double*>(q.lev[L - 1].box.buf[0]),
                                                               static_cast<double*>(q.lev[L].box.buf[0]), c, s->stream)
                        : lbx::launch_fill_from_coarse<float>(static_cast<float*>(q.lev[L - 1].box.buf[0]),
                                                              static_cast<float*>(q.lev[L].box.buf[0]), c, s->stream);
    CK(e);
  }
  for (int L = 0; L < q.nlev && q.r.steps > 0; ++L) {  // into the pull form
    const BBox& B = q.lev[L].box;
    cudaError_t e = s->precision == LBX_F64
                        ? lbx::launch_b_to_qform<double>(static_cast<double*>(B.buf[0]), B.b, B.cov, B.om_s,
                                                         B.om_b, B.rho0, s->stream)
                        : lbx::launch_b_to_qform<float>(static_cast<float*>(B.buf[0]), B.b, B.cov, B.om_s,
                                                        B.om_b, B.rho0, s->stream);
    CK(e);
  }
  q.state = 1;
  q.remaining = q.r.steps;
  return LBX_OK;
}

void append(std::vector<BTile>& all, size_t& off, const std::vector<BTile>& t) {
  off = all.size();
  all.insert(all.end(), t.begin(), t.end());
}

int rebuild_tables(lbx_server* s) {
  s->hb.clear();
  s->hc.clear();
  std::vector<int> ids[kMaxLevels];
  std::vector<int> cids[2];
  s->updates_per_macro = 0;
  for (long long id : s->active) {
    Req& q = s->reqs[id];
    int bidx[kMaxLevels];
    for (int L = 0; L < q.nlev; ++L) {
      bidx[L] = (int)s->hb.size();
      s->hb.push_back(q.lev[L].box);
      ids[L].push_back(bidx[L]);
      const long long valid = (long long)q.lev[L].box.b.n[0] * q.lev[L].box.b.n[1] * q.lev[L].box.b.n[2];
      s->updates_per_macro += valid << L;  // level L sub-cycles 2^L times
    }
    for (int L = 1; L < q.nlev; ++L) {
      BCoupling c;
      c.c = coupling_of(q, L);
      c.cbox = bidx[L - 1];
      c.fbox = bidx[L];
      c.nring = 0;
      cids[L - 1].push_back((int)s->hc.size());
      s->hc.push_back(c);
    }
  }
  std::vector<BTile> all;
  for (int L = 0; L < kMaxLevels; ++L) {
    s->tiles_step[L] = lbx::make_tiles(s->hb, ids[L], s->tile_cells);
    append(all, s->off_step[L], s->tiles_step[L]);
  }
  for (int k = 0; k < 2; ++k) {
    std::vector<BTile> ex, co;
    for (int ci : cids[k]) {
      const lbx::Coupling& c = s->hc[ci].c;
      // ghost shell (explode), ring (coalesce);
      // small tiles so that even one patch fills the GPU
      const int nexp = (int)lbx::ghost_cells_of(c.fb);
      const int nring = (int)lbx::ring_cells_of(c);
      for (int st = 0; st < nexp; st += kExplodeTile)
        ex.push_back(BTile{ci, st, std::min(kExplodeTile, nexp - st)});
      for (int st = 0; st < nring; st += kCoalesceTile)
        co.push_back(BTile{ci, st, std::min(kCoalesceTile, nring - st)});
    }
    s->tiles_ex[k] = ex;
    s->tiles_co[k] = co;
    append(all, s->off_ex[k], ex);
    append(all, s->off_co[k], co);
  }
  auto align = [](size_t n) { return (n + 255) & ~size_t(255); };
  const size_t nb = s->hb.size() * sizeof(BBox), nc = s->hc.size() * sizeof(BCoupling),
               nt = all.size() * sizeof(BTile);
  const size_t oc = align(nb), ot = oc + align(nc), total = ot + nt;
  CK(cudaStreamSynchronize(s->stream));  // the staging buffer's last copy is done
  if (total > s->tables_cap) {
    if (s->d_tables) cudaFree(s->d_tables);
    if (s->h_tables) cudaFreeHost(s->h_tables);
    s->d_tables = s->h_tables = nullptr;
    s->tables_cap = 0;
    const size_t cap = align(total + total / 2);
    CK(cudaMalloc(&s->d_tables, cap));
    CK(cudaHostAlloc(&s->h_tables, cap, cudaHostAllocDefault));
    s->tables_cap = cap;
  }
  if (total) {
    std::memcpy(s->h_tables, s->hb.data(), nb);
    std::memcpy(s->h_tables + oc, s->hc.data(), nc);
    std::memcpy(s->h_tables + ot, all.data(), nt);
    CK(cudaMemcpyAsync(s->d_tables, s->h_tables, total, cudaMemcpyHostToDevice, s->stream));
  }
  s->d_boxes = reinterpret_cast<BBox*>(s->d_tables);
  s->d_cps = reinterpret_cast<BCoupling*>(s->d_tables + oc);
  s->d_tiles = reinterpret_cast<BTile*>(s->d_tables + ot);
  if (s->gexec) {
    cudaGraphExecDestroy(s->gexec);
    s->gexec = nullptr;
  }
  s->graph_F0 = -1;
  s->dirty = false;
  return LBX_OK;
}

template <typename T>
cudaError_t phase_step(lbx_server* s, int L) {
  const int n = (int)s->tiles_step[L].size();
  if (!n) return cudaSuccess;
  ++s->launches;
  // level 0 boxes are periodic (covered cells), finer ones patches
  const int kind = L == 0 ? lbx::kBoxPeriodic : lbx::kBoxPatch;
  return lbx::launch_b_step<T>(s->d_boxes, s->d_tiles + s->off_step[L], n, s->F[L], s->grid[kind],
                               s->block, s->cpt, kind, s->stream);
}

// one step of level L (and, recursively, its finer levels): the
// conservative cycle of the single-simulation driver, batched over requests,
// in the pull form.  The push form's order (explode, step L, two steps of
// L+1, coalesce into the streamed coarse state) becomes: explode from the
// coarse post-collision store, two steps of L+1, coalesce into the entries
// the coarse cells will gather, step L.
template <typename T>
cudaError_t advance_level(lbx_server* s, int L) {
  cudaError_t e = cudaSuccess;
  const bool has_fine = L + 1 < kMaxLevels && !s->tiles_step[L + 1].empty();
  if (has_fine) {
    if (!s->tiles_ex[L].empty()) {
      ++s->launches;
      e = lbx::launch_b_explode<T>(s->d_boxes, s->d_cps, s->d_tiles + s->off_ex[L],
                                   (int)s->tiles_ex[L].size(), s->F[L], s->F[L + 1], s->stream);
      if (e != cudaSuccess) return e;
    }
    for (int k = 0; k < 2; ++k) {
      e = advance_level<T>(s, L + 1);
      if (e != cudaSuccess) return e;
    }
    if (!s->tiles_co[L].empty()) {
      // covered coarse cells are restricted only when a request finishes
      ++s->launches;
      e = lbx::launch_b_coalesce<T>(s->d_boxes, s->d_cps, s->d_tiles + s->off_co[L],
                                    (int)s->tiles_co[L].size(), s->F[L], s->F[L + 1], s->stream);
      if (e != cudaSuccess) return e;
    }
  }
  e = phase_step<T>(s, L);
  s->F[L] ^= 1;
  return e;
}

cudaError_t macro_step(lbx_server* s) {
  return s->precision == LBX_F64 ? advance_level<double>(s, 0) : advance_level<float>(s, 0);
}

int run_macro_steps(lbx_server* s, int n) {
  // pairs of coarse steps leave every flip where it was: replay a graph
  int done = 0;
  if (n >= 2) {
    if (!s->gexec || s->graph_F0 != s->F[0]) {
      if (s->gexec) cudaGraphExecDestroy(s->gexec);
      s->gexec = nullptr;
      const long long l0 = s->launches;
      cudaGraph_t g = nullptr;
      CK(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
      cudaError_t a = macro_step(s);
      cudaError_t b = a == cudaSuccess ? macro_step(s) : a;
      cudaError_t c = cudaStreamEndCapture(s->stream, &g);
      CK(a);
      CK(b);
      CK(c);
      cudaError_t d = cudaGraphInstantiate(&s->gexec, g, 0);
      cudaGraphDestroy(g);
      CK(d);
      s->graph_F0 = s->F[0];
      s->graph_launches = s->launches - l0;  // kernels recorded in the graph
      s->launches = l0;                      // capture itself ran nothing
    }
    for (; done + 1 < n; done += 2) {
      CK(cudaGraphLaunch(s->gexec, s->stream));
      s->launches += s->graph_launches;
      s->cell_updates += 2 * s->updates_per_macro;
    }
  }
  if (done < n) {
    CK(macro_step(s));
    s->cell_updates += s->updates_per_macro;
  }
  return LBX_OK;
}

template <typename T>
int finish_request(lbx_server* s, Req& q) {
  // every level back to its streamed state, gathered from the store each
  // level's last step read (its coarse cells' entries hold the coalescence);
  // a request of zero steps never left it
  for (int L = 0; L < q.nlev && q.r.steps > 0; ++L) {
    const BBox& B = q.lev[L].box;
    const int now = B.par ^ s->F[L];
    CK(lbx::launch_b_to_rform<T>(static_cast<const T*>(B.buf[now ^ 1]), static_cast<T*>(B.buf[now]),
                                 B.b, s->stream));
  }
  // composite mass: uncovered cells of each level weighted by 8^-L
  double* d = nullptr;
  CK(cudaMallocAsync(&d, (lbx::reduce_partials_doubles() + 8) * sizeof(double), s->stream));
  long double mass = 0, vol = 1;
  double h[4];
  for (int L = 0; L < q.nlev; ++L) {
    const BBox& B = q.lev[L].box;
    const IBox skip = (L + 1 < q.nlev) ? B.cov : lbx::empty_ibox();
    cudaError_t e = lbx::launch_reduce<T>(static_cast<const T*>(B.buf[B.par ^ s->F[L]]), B.b, skip, B.rho0, d + 8,
                                          d, s->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h, d, 4 * sizeof(double), cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) {
      cudaFreeAsync(d, s->stream);
      CK(e);
    }
    mass += vol * (long double)h[0];
    vol /= 8;
  }
  cudaFreeAsync(d, s->stream);
  q.mass = (double)mass;
  // covered cells of each level <- mean of their children (finest pair first)
  for (int L = q.nlev - 1; L >= 1; --L) {
    const BBox& F = q.lev[L].box;
    const BBox& C = q.lev[L - 1].box;
    CK(lbx::launch_restrict<T>(static_cast<const T*>(F.buf[F.par ^ s->F[L]]),
                               static_cast<T*>(C.buf[C.par ^ s->F[L - 1]]), coupling_of(q, L), s->stream));
  }
  // level-0 density (FAB order) when kept, and a probe value on the pulse plane
  const BBox& B0 = q.lev[0].box;
  const size_t N = (size_t)q.r.nx * q.r.ny * q.r.nz;
  double* dr = nullptr;
  CK(cudaMallocAsync(&dr, 4 * N * sizeof(double), s->stream));
  cudaError_t e = lbx::launch_hydro<T>(static_cast<const T*>(B0.buf[B0.par ^ s->F[0]]), B0.b, B0.rho0, dr, dr + N,
                                       s->stream);
  int pc[3] = {q.r.nx / 2, q.r.ny / 2, q.r.nz / 2};
  pc[q.r.pulse_axis] = q.r.pulse_index;
  const size_t probe_at = ((size_t)pc[2] * q.r.ny + pc[1]) * q.r.nx + pc[0];
  std::vector<double> rho(q.r.keep_field ? N : 0);
  if (e == cudaSuccess)
    e = q.r.keep_field
            ? cudaMemcpyAsync(rho.data(), dr, N * sizeof(double), cudaMemcpyDeviceToHost, s->stream)
            : cudaMemcpyAsync(&q.probe, dr + probe_at, sizeof(double), cudaMemcpyDeviceToHost, s->stream);
  cudaFreeAsync(dr, s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  CK(e);
  if (q.r.keep_field) q.probe = rho[probe_at];
  q.rho = std::move(rho);
  return LBX_OK;
}

}  // namespace

extern "C" {

int lbx_server_create(size_t hbm_budget_bytes, int max_active, int precision, lbx_server** out) {
  if (!out || hbm_budget_bytes == 0 || max_active <= 0) return LBX_ERR_ARG;
  if (precision != LBX_F64 && precision != LBX_F32_SHIFTED) return LBX_ERR_ARG;
  *out = nullptr;
  lbx_server* s = new lbx_server();
  s->budget = hbm_budget_bytes;
  s->max_active = max_active;
  s->precision = precision;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&s->num_sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    e = cudaMemPoolCreate(&s->pool, &props);
    if (e == cudaSuccess) {
      uint64_t keep = (uint64_t)hbm_budget_bytes;  // keep freed stores for reuse up to the budget
      e = cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
  }
  if (e != cudaSuccess) {
    lbx::note_error("lbx_server_create", e);
    if (s->pool) cudaMemPoolDestroy(s->pool);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return lbx::status_from_cuda(e);
  }
  for (int kind = 0; kind < 3; ++kind) {
    const int per_sm = precision == LBX_F64 ? lbx::b_step_blocks_per_sm<double>(s->block, s->cpt, kind)
                                            : lbx::b_step_blocks_per_sm<float>(s->block, s->cpt, kind);
    s->grid[kind] = s->num_sms * per_sm;
  }
  *out = s;
  return LBX_OK;
}

int lbx_server_set_config(lbx_server* s, int tile_cells, int block, int cells_per_thread) {
  if (!s || block < 32 || block > 512 || block % 32 || cells_per_thread < 1 ||
      cells_per_thread > 2 || tile_cells < block)
    return LBX_ERR_ARG;
  s->tile_cells = tile_cells;
  s->block = block;
  s->cpt = cells_per_thread;
  for (int kind = 0; kind < 3; ++kind) {
    const int per_sm = s->precision == LBX_F64
                           ? lbx::b_step_blocks_per_sm<double>(s->block, s->cpt, kind)
                           : lbx::b_step_blocks_per_sm<float>(s->block, s->cpt, kind);
    s->grid[kind] = s->num_sms * per_sm;
  }
  s->dirty = true;  // new tiles and a new graph at the next pump
  return LBX_OK;
}

int lbx_server_destroy(lbx_server* s) {
  if (!s) return LBX_OK;
  if (s->stream) cudaStreamSynchronize(s->stream);
  for (auto& kv : s->reqs)
    if (kv.second.state == 1) free_request(s, kv.second);
  if (s->gexec) cudaGraphExecDestroy(s->gexec);
  if (s->d_tables) cudaFree(s->d_tables);
  if (s->h_tables) cudaFreeHost(s->h_tables);
  if (s->stream) {
    cudaStreamSynchronize(s->stream);  // pool frees are stream-ordered
    cudaStreamDestroy(s->stream);
  }
  if (s->pool) cudaMemPoolDestroy(s->pool);
  delete s;
  return LBX_OK;
}

int lbx_server_timing(const lbx_server* s, double* seconds4) {
  if (!s || !seconds4) return LBX_ERR_ARG;
  seconds4[0] = s->t_admit;
  seconds4[1] = s->t_finish;
  seconds4[2] = s->t_tables;
  seconds4[3] = s->t_step;
  return LBX_OK;
}

int lbx_server_submit(lbx_server* s, const lbx_request* r, long long* id) {
  if (!s || !r || !id) return LBX_ERR_ARG;
  if (r->levels < 1 || r->levels > kMaxLevels || r->steps < 0 || r->tau <= 0.0) return LBX_ERR_ARG;
  if (r->pulse_axis < 0 || r->pulse_axis > 2) return LBX_ERR_ARG;
  const int n[3] = {r->nx, r->ny, r->nz};
  for (int d = 0; d < 3; ++d) {
    // refined boxes are half the parent, centred: extents must split evenly
    const int need = r->levels > 1 ? (1 << (r->levels + 1)) : 1;
    if (n[d] < 8 || n[d] % need) return LBX_ERR_ARG;
  }
  if (r->pulse_index < 0 || r->pulse_index >= n[r->pulse_axis]) return LBX_ERR_ARG;
  Req q;
  q.r = *r;
  plan_levels(q);
  for (int L = 0; L < q.nlev; ++L) {  // each box within the batch engine's index limits
    BBox b{};
    int m[3];
    for (int d = 0; d < 3; ++d) m[d] = q.lev[L].hi[d] - q.lev[L].lo[d] + 1;
    b.b = lbx::make_box(m[0], m[1], m[2], L ? 2 : 0);
    b.periodic = L == 0 ? 1 : 0;
    if (!lbx::set_iteration_space(b)) return LBX_ERR_UNSUPPORTED;
  }
  if (request_bytes(q, (int)s->esize()) > s->budget) return LBX_ERR_OOM;
  q.id = s->next_id++;
  s->reqs[q.id] = q;
  s->queue.push_back(q.id);
  *id = q.id;
  return LBX_OK;
}

int lbx_server_pump(lbx_server* s, int quantum, int* active, int* queued) {
  if (!s || quantum <= 0) return LBX_ERR_ARG;
  using clk = std::chrono::steady_clock;
  auto secs = [](clk::time_point a, clk::time_point b) {
    return std::chrono::duration<double>(b - a).count();
  };
  Range range("lbx_server_pump");
  // admission: FIFO while a slot is free and the stores fit the budget
  auto t0 = clk::now();
  nvtxRangePushA("admit");
  while (!s->queue.empty() && (int)s->active.size() < s->max_active) {
    Req& q = s->reqs[s->queue.front()];
    const size_t need = request_bytes(q, (int)s->esize());
    if (s->in_use + need > s->budget) break;
    int rc = admit(s, q);
    if (rc != LBX_OK) {
      nvtxRangePop();
      free_request(s, q);
      return rc;
    }
    s->active.push_back(q.id);
    s->queue.pop_front();
    s->dirty = true;
  }
  nvtxRangePop();
  auto t1 = clk::now();
  s->t_admit += secs(t0, t1);
  if (s->dirty) {
    Range r("rebuild_tables");
    RET(rebuild_tables(s));
  }
  auto t2 = clk::now();
  s->t_tables += secs(t1, t2);
  if (!s->active.empty()) {
    int n = quantum;
    for (long long id : s->active) n = std::min(n, std::max(s->reqs[id].remaining, 0));
    {
      Range r("run_macro_steps");
      if (n > 0) RET(run_macro_steps(s, n));
      CK(cudaStreamSynchronize(s->stream));
    }
    Range r("finish");
    auto t3 = clk::now();
    s->t_step += secs(t2, t3);
    std::vector<long long> still;
    for (long long id : s->active) {
      Req& q = s->reqs[id];
      q.remaining -= n;
      if (q.remaining <= 0) {
        RET(s->precision == LBX_F64 ? finish_request<double>(s, q) : finish_request<float>(s, q));
        free_request(s, q);
        q.state = 2;
        s->dirty = true;
      } else {
        still.push_back(id);
      }
    }
    s->active.swap(still);
    s->t_finish += secs(t3, clk::now());
  }
  if (active) *active = (int)s->active.size();
  if (queued) *queued = (int)s->queue.size();
  return LBX_OK;
}

int lbx_server_poll(lbx_server* s, long long id, int* done, double* mass, double* probe) {
  if (!s || !done) return LBX_ERR_ARG;
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return LBX_ERR_NOT_FOUND;
  *done = it->second.state == 2 ? 1 : 0;
  if (*done) {
    if (mass) *mass = it->second.mass;
    if (probe) *probe = it->second.probe;
  }
  return LBX_OK;
}

int lbx_server_take(lbx_server* s, long long id, double* rho, size_t n) {
  if (!s) return LBX_ERR_ARG;
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return LBX_ERR_NOT_FOUND;
  if (it->second.state != 2) return LBX_ERR_STATE;
  if (rho) {
    if (n < it->second.rho.size()) return LBX_ERR_ARG;
    std::copy(it->second.rho.begin(), it->second.rho.end(), rho);
  }
  s->reqs.erase(it);
  return LBX_OK;
}

int lbx_server_stats(const lbx_server* s, long long* cell_updates, size_t* bytes_in_use,
                     long long* launches) {
  if (!s) return LBX_ERR_ARG;
  if (cell_updates) *cell_updates = s->cell_updates;
  if (bytes_in_use) *bytes_in_use = s->in_use;
  if (launches) *launches = s->launches;
  return LBX_OK;
}

}  // extern "C"
