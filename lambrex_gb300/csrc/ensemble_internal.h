// ensemble_internal.h -- box helpers shared by the ensemble and the server.
#pragma once
#include <cuda_runtime.h>

#include "batch.cuh"

namespace lbx {
// cells of a box's iteration space
long long box_cells(const BBox& b);
// equilibrium state of a periodic box from C-order rho/u host vectors into
// store `now` (rho0 of the box must already be set)
int init_box_state(const BBox& b, int precision, int now, const double* rho_c, const double* u_c,
                   cudaStream_t st);
}  // namespace lbx
